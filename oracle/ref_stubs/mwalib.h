/*
 * Stand-in declarations for the parts of mwalib (v1.x, a Rust crate with a C
 * API; not installed in this environment) that the VCSBeam hot-path sources
 * name. Only the field names the reference code reads are declared; the
 * layout is this harness's own and is not mwalib's.
 *
 * Test infrastructure: used only to compile the reference sources for the
 * oracle harness (oracle/build_ref.sh).
 */
#ifndef VGB_STUB_MWALIB_H
#define VGB_STUB_MWALIB_H

#include <stdint.h>
#include <stddef.h>
#include <stdbool.h>
#include <time.h>

#define MWALIB_SUCCESS 0
#define MWALIB_SPEED_OF_LIGHT_IN_VACUUM_M_PER_S 299792458.0
#define MWALIB_MWA_LATITUDE_RADIANS (-0.4660608448386394)
#define MWALIB_MWA_LONGITUDE_RADIANS (2.0362898668561042)
#define MWALIB_MWA_ALTITUDE_METRES 377.827

typedef enum MWAVersion {
    CorrOldLegacy = 1,
    CorrLegacy = 2,
    CorrMWAXv2 = 3,
    VCSLegacyRecombined = 4,
    VCSMWAXv2 = 5
} MWAVersion;

typedef struct Rfinput {
    uint32_t input;
    uint32_t ant;
    uint32_t tile_id;
    char *tile_name;
    char *pol;
    double electrical_length_m;
    double north_m;
    double east_m;
    double height_m;
    uint32_t vcs_order;
    uint32_t subfile_order;
    bool flagged;
    uint32_t *digital_gains;
    size_t num_digital_gains;
    double *dipole_gains;
    size_t num_dipole_gains;
    uint32_t *dipole_delays;
    size_t num_dipole_delays;
    uint32_t rec_number;
    uint32_t rec_slot_number;
} Rfinput;

typedef struct Antenna {
    uint32_t ant;
    uint32_t tile_id;
    char *tile_name;
    size_t rfinput_x;
    size_t rfinput_y;
    double electrical_length_m;
    double north_m;
    double east_m;
    double height_m;
} Antenna;

typedef struct CoarseChannel {
    size_t corr_chan_number;
    size_t rec_chan_number;
    size_t gpubox_number;
    uint32_t chan_width_hz;
    uint32_t chan_start_hz;
    uint32_t chan_centre_hz;
    uint32_t chan_end_hz;
} CoarseChannel;

typedef struct MetafitsMetadata {
    MWAVersion mwa_version;
    uint32_t obs_id;
    uint64_t sched_start_gps_time_ms;
    time_t sched_start_utc;
    double sched_start_mjd;
    char *project_id;
    Antenna *antennas;
    size_t num_ants;
    Rfinput *rf_inputs;
    size_t num_rf_inputs;
    size_t num_ant_pols;
    size_t num_visibility_pols;
    CoarseChannel *metafits_coarse_chans;
    size_t num_metafits_coarse_chans;
    uint32_t coarse_chan_width_hz;
    uint32_t num_delays;
    uint32_t *delays;
    size_t num_corr_fine_chans_per_coarse;
    uint32_t corr_fine_chan_width_hz;
    size_t num_volt_fine_chans_per_coarse;
    double ra_tile_pointing_deg;
    double dec_tile_pointing_deg;
} MetafitsMetadata;

typedef struct VoltageMetadata {
    MWAVersion mwa_version;
    uint64_t num_samples_per_voltage_block;
    uint64_t num_voltage_blocks_per_second;
    uint64_t voltage_block_size_bytes;
} VoltageMetadata;

typedef struct MetafitsContext MetafitsContext;
typedef struct VoltageContext VoltageContext;

#endif
