/* Stand-in for the psrfits_utils subint struct: only the members the
 * reference's vmSendSToFits() copies into. Oracle harness use only. */
#ifndef VGB_STUB_PSRFITS_H
#define VGB_STUB_PSRFITS_H
struct subint {
    int bytes_per_subint;
    float *dat_offsets;
    float *dat_scales;
    unsigned char *data;
    double offs;
    double lst;
    double tsubint;
};
struct psrfits {
    struct subint sub;
    long long tot_rows;
};
#endif
