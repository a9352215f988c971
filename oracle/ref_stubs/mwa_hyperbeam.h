/* Stand-in for mwa_hyperbeam's opaque beam handle. Oracle harness use only. */
#ifndef VGB_STUB_HYPERBEAM_H
#define VGB_STUB_HYPERBEAM_H
typedef struct FEEBeam FEEBeam;
#include <stdint.h>
int32_t new_fee_beam(const char *hdf5_file, FEEBeam **fee_beam);
void free_fee_beam(FEEBeam *fee_beam);
int32_t calc_jones(FEEBeam *fee_beam, double az_rad, double za_rad, uint32_t freq_hz, const uint32_t *delays,
                   const double *amps, uint32_t num_amps, uint8_t norm_to_zenith, const double *latitude_rad,
                   uint8_t iau_order, double *jones);
int hb_last_error_length(void);
int hb_last_error_message(char *buffer, int length);
#endif
