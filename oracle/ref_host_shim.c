/*
 * Plain-signature entry points into the reference's own host C (jones.c,
 * filter.c, geometry.c), compiled against the configured reference header by
 * oracle/build_ref.sh. Test infrastructure only: the CPU tests call these to
 * pin the oracle's table builders against the reference implementation.
 *
 * Each function fills just the vcsbeam_context / MetafitsMetadata members
 * the reference routine reads, then calls it.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "vcsbeam.h"

/* jones.c:97 vmCalcJ. D is [nant][nchan][2][2] complex, B is
 * [npointing][nant][2][2] complex, J (out) is [npointing][nant][nchan][2][2]. */
void refhost_calc_j(int npointing, int nant, int nchan,
                    cuDoubleComplex *D, cuDoubleComplex *B, cuDoubleComplex *J)
{
    vcsbeam_context vm;
    MetafitsMetadata md;
    memset(&vm, 0, sizeof(vm));
    memset(&md, 0, sizeof(md));
    md.num_ants = nant;
    md.num_ant_pols = 2;
    vm.obs_metadata = &md;
    vm.nfine_chan = nchan;
    vm.npointing = npointing;
    vm.D = D;
    vm.pb.B = B;
    vm.J = J;
    vmCalcJ(&vm);
}

/* geometry.c:40 calc_geometric_delays for one pointing and frequency.
 * Antenna a has inputs 2a ('X') and 2a+1 ('Y'); phi (out) is [nant]. */
void refhost_calc_geometric_delays(double unit_E, double unit_N, double unit_H,
                                   uint32_t freq_hz, int nant,
                                   const double *east, const double *north,
                                   const double *height, const double *cable,
                                   cuDoubleComplex *phi)
{
    MetafitsMetadata md;
    memset(&md, 0, sizeof(md));
    Rfinput *rf = (Rfinput *)calloc(2 * nant, sizeof(Rfinput));
    static char X[] = "X", Y[] = "Y";
    for (int a = 0; a < nant; a++) {
        for (int p = 0; p < 2; p++) {
            Rfinput *r = &rf[2 * a + p];
            r->ant = a;
            r->pol = p ? Y : X;
            r->east_m = east[a];
            r->north_m = north[a];
            r->height_m = height[a];
            r->electrical_length_m = cable[a];
        }
    }
    md.rf_inputs = rf;
    md.num_rf_inputs = 2 * nant;
    md.num_ants = nant;
    beam_geom bg;
    memset(&bg, 0, sizeof(bg));
    bg.unit_E = unit_E;
    bg.unit_N = unit_N;
    bg.unit_H = unit_H;
    calc_geometric_delays(&bg, freq_hz, &md, phi);
    free(rf);
}

/* filter.c:64 vmLoadFilter + filter.c:160 vmScaleFilterCoeffs. Copies up to
 * maxn coefficients into coeffs; returns ncoeffs (ntaps via *ntaps). */
int refhost_load_filter(char *name, int synthesis, int nchans, double scale,
                        double *coeffs, int maxn, int *ntaps)
{
    vcsbeam_context vm;
    memset(&vm, 0, sizeof(vm));
    filter_type type = synthesis ? SYNTHESIS_FILTER : ANALYSIS_FILTER;
    vmLoadFilter(&vm, name, type, nchans);
    vmScaleFilterCoeffs(&vm, type, scale);
    pfb_filter *f = synthesis ? vm.synth_filter : vm.analysis_filter;
    int n = f->ncoeffs < maxn ? f->ncoeffs : maxn;
    memcpy(coeffs, f->coeffs, n * sizeof(double));
    *ntaps = f->ntaps;
    int nc = f->ncoeffs;
    free(f->twiddles);
    free_pfb_filter(f);
    return nc;
}

/* The reference host code names these; the harness never reaches them. */
static void refhost_unreachable(const char *what)
{
    fprintf(stderr, "ref_host_shim: %s is not available in the harness\n", what);
    abort();
}
void logger_start_stopwatch(logger *log, const char *n, bool p) { (void)log; (void)n; (void)p; }
void logger_stop_stopwatch(logger *log, const char *n) { (void)log; (void)n; }
void vmCalcB(vcsbeam_context *vm, beam_geom *bg) { (void)vm; (void)bg; refhost_unreachable("vmCalcB"); }
void palMap(double rm, double dm, double pr, double pd, double px, double rv,
            double eq, double date, double *ra, double *da)
{ (void)rm; (void)dm; (void)pr; (void)pd; (void)px; (void)rv; (void)eq; (void)date; (void)ra; (void)da; refhost_unreachable("palMap"); }
void palDe2h(double ha, double dec, double phi, double *az, double *el)
{ (void)ha; (void)dec; (void)phi; (void)az; (void)el; refhost_unreachable("palDe2h"); }
double palRanorm(double a) { (void)a; refhost_unreachable("palRanorm"); return 0; }
double palGmst(double u) { (void)u; refhost_unreachable("palGmst"); return 0; }
void palDtf2r(int h, int m, double s, double *r, int *j)
{ (void)h; (void)m; (void)s; (void)r; (void)j; refhost_unreachable("palDtf2r"); }
void palDaf2r(int d, int m, double s, double *r, int *j)
{ (void)d; (void)m; (void)s; (void)r; (void)j; refhost_unreachable("palDaf2r"); }
void palCaldj(int y, int m, int d, double *r, int *j)
{ (void)y; (void)m; (void)d; (void)r; (void)j; refhost_unreachable("palCaldj"); }
