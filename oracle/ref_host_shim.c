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

/* geometry.c:440-467 calc_array_factor between a look direction and each of
 * npix test directions (Eq. A4 of Meyers et al. 2017). */
void refhost_array_factor(const double *look, const double *dirs, int npix, uint32_t freq_hz, int nant,
                          const double *east, const double *north, const double *height, const double *cable,
                          double *af)
{
    MetafitsMetadata md;
    memset(&md, 0, sizeof(md));
    Rfinput *rf = (Rfinput *)calloc(2 * nant, sizeof(Rfinput));
    static char X[] = "X", Y[] = "Y";
    for (int a = 0; a < nant; a++)
        for (int p = 0; p < 2; p++) {
            Rfinput *r = &rf[2 * a + p];
            r->ant = a;
            r->pol = p ? Y : X;
            r->east_m = east[a];
            r->north_m = north[a];
            r->height_m = height[a];
            r->electrical_length_m = cable[a];
        }
    md.rf_inputs = rf;
    md.num_rf_inputs = 2 * nant;
    md.num_ants = nant;
    beam_geom b1, b2;
    memset(&b1, 0, sizeof(b1));
    b1.unit_E = look[0];
    b1.unit_N = look[1];
    b1.unit_H = look[2];
    for (int i = 0; i < npix; i++) {
        memset(&b2, 0, sizeof(b2));
        b2.unit_E = dirs[3 * i];
        b2.unit_N = dirs[3 * i + 1];
        b2.unit_H = dirs[3 * i + 2];
        af[i] = calc_array_factor(&md, freq_hz, &b1, &b2);
    }
    free(rf);
}

/* ---- calibration.c (vmLoadOffringaSolution, vmLoadRTSSolution,
 * vmApplyCalibrationCorrections, parse_calibration_correction_file) driven
 * through a vcsbeam_context populated with the fields those routines read:
 * antenna a's RF inputs are 2a ('X') and 2a+1 ('Y'), tile ids 1000 + a in the
 * calibration metadata and 1000 + cal_ant[a] in the target observation. ---- */
typedef struct {
    MetafitsMetadata meta;
    Rfinput *inputs;
    Antenna *ants;
    char **names;
    CoarseChannel cc[32];
} refh_meta;

static void refh_meta_init(refh_meta *m, int nant, int nchan_cal, int chan_width_hz, const int *tile_of_ant)
{
    memset(m, 0, sizeof(*m));
    m->inputs = (Rfinput *)calloc(2 * nant, sizeof(Rfinput));
    m->ants = (Antenna *)calloc(nant, sizeof(Antenna));
    m->names = (char **)calloc(nant, sizeof(char *));
    for (int a = 0; a < nant; a++) {
        m->names[a] = (char *)malloc(16);
        snprintf(m->names[a], 16, "Tile%03d", tile_of_ant ? tile_of_ant[a] : a);
        m->ants[a].ant = a;
        m->ants[a].tile_name = m->names[a];
        m->ants[a].tile_id = 1000 + (tile_of_ant ? tile_of_ant[a] : a);
        for (int p = 0; p < 2; p++) {
            Rfinput *r = &m->inputs[2 * a + p];
            r->input = 2 * a + p;
            r->ant = a;
            r->tile_id = m->ants[a].tile_id;
            r->tile_name = m->names[a];
            r->pol = p ? "Y" : "X";
        }
    }
    m->meta.num_ants = nant;
    m->meta.antennas = m->ants;
    m->meta.rf_inputs = m->inputs;
    m->meta.num_rf_inputs = 2 * nant;
    m->meta.num_ant_pols = 2;
    m->meta.num_visibility_pols = 4;
    m->meta.num_metafits_coarse_chans = 24;
    m->meta.metafits_coarse_chans = m->cc;
    m->meta.coarse_chan_width_hz = 1280000;
    m->meta.num_corr_fine_chans_per_coarse = nchan_cal;
    m->meta.corr_fine_chan_width_hz = chan_width_hz;
    m->meta.num_volt_fine_chans_per_coarse = 128;
}

static void refh_meta_free(refh_meta *m, int nant)
{
    for (int a = 0; a < nant; a++) free(m->names[a]);
    free(m->names);
    free(m->ants);
    free(m->inputs);
}

void refhost_load_offringa(char *path, int coarse_chan_idx, int mpi_size, int nant, int nchan_cal, int nfine,
                           double *D)
{
    refh_meta cal;
    refh_meta_init(&cal, nant, nchan_cal, 1280000 / nchan_cal, NULL);
    vcsbeam_context vm;
    memset(&vm, 0, sizeof(vm));
    vm.cal.caldir = path;
    vm.cal_coarse_chan_idxs_to_process = &coarse_chan_idx;
    vm.cal_metadata = &cal.meta;
    vm.mpi_size = mpi_size;
    vm.nfine_chan = nfine;
    vm.D = (gpuDoubleComplex *)D;
    vmLoadOffringaSolution(&vm);
    refh_meta_free(&cal, nant);
}

void refhost_load_rts(char *caldir, int use_bandpass, int corr_chan_number, int nant, int nchan_cal,
                      int chan_width_hz, const int *cal_ant, int nfine, double *D)
{
    refh_meta cal, obs;
    refh_meta_init(&cal, nant, nchan_cal, chan_width_hz, NULL);
    refh_meta_init(&obs, nant, nchan_cal, chan_width_hz, cal_ant);
    cal.cc[0].corr_chan_number = corr_chan_number;
    vcsbeam_context vm;
    memset(&vm, 0, sizeof(vm));
    vm.cal.caldir = caldir;
    vm.cal.use_bandpass = use_bandpass;
    vm.coarse_chan_idx = 0;
    vm.cal_metadata = &cal.meta;
    vm.obs_metadata = &obs.meta;
    vm.nfine_chan = nfine;
    vm.D = (gpuDoubleComplex *)D;
    vmLoadRTSSolution(&vm);
    refh_meta_free(&cal, nant);
    refh_meta_free(&obs, nant);
}

void refhost_apply_corrections(double *D, int nant, int nfine, int ref_ant, int keep_cross_terms, double slope,
                               double offset, unsigned chan_start_hz)
{
    refh_meta obs;
    refh_meta_init(&obs, nant, 128, 10000, NULL);
    obs.cc[0].chan_start_hz = chan_start_hz;
    char name[16] = "NONE";
    if (ref_ant >= 0) snprintf(name, sizeof(name), "Tile%03d", ref_ant);
    vcsbeam_context vm;
    memset(&vm, 0, sizeof(vm));
    vm.cal.ref_ant = name;
    vm.cal.keep_cross_terms = keep_cross_terms;
    vm.cal.phase_slope = slope;
    vm.cal.phase_offset = offset;
    vm.coarse_chan_idx = 0;
    vm.obs_metadata = &obs.meta;
    vm.nfine_chan = nfine;
    vm.D = (gpuDoubleComplex *)D;
    vmApplyCalibrationCorrections(&vm);
    refh_meta_free(&obs, nant);
}

/* RUNTIME_DIR/pq_phase_correction.txt for one GPS second; found = the
 * returned reference tile is not "NONE". */
int refhost_pq_correction(unsigned gpstime, double *slope, double *offset, char *ref_tile, int len)
{
    calibration cal;
    memset(&cal, 0, sizeof(cal));
    parse_calibration_correction_file(gpstime, &cal);
    *slope = cal.phase_slope;
    *offset = cal.phase_offset;
    snprintf(ref_tile, len, "%s", cal.ref_ant);
    int found = strcmp(cal.ref_ant, "NONE") != 0;
    free(cal.ref_ant);
    return found;
}

/* metadata.c helpers calibration.c calls (same matching rules). */
Rfinput *find_matching_rf_input(MetafitsMetadata *metadata, Rfinput *rfinput)
{
    for (uintptr_t i = 0; i < metadata->num_rf_inputs; i++)
        if (rfinput->tile_id == metadata->rf_inputs[i].tile_id && *(rfinput->pol) == *(metadata->rf_inputs[i].pol))
            return &(metadata->rf_inputs[i]);
    return NULL;
}
Antenna *find_antenna_by_name(MetafitsMetadata *obs_metadata, char *tile_name)
{
    for (int i = 0; i < (int)obs_metadata->num_ants; i++)
        if (strcmp(tile_name, obs_metadata->antennas[i].tile_name) == 0) return &(obs_metadata->antennas[i]);
    return NULL;
}
void logger_timed_message(logger *log, const char *message) { (void)log; (void)message; }
void logger_message(logger *log, const char *message) { (void)log; (void)message; }
void vmSetNumNotFlaggedRFInputs(vcsbeam_context *vm) { (void)vm; }

/* The reference host code names these; the harness never reaches them. */
static void refhost_unreachable(const char *what)
{
    fprintf(stderr, "ref_host_shim: %s is not available in the harness\n", what);
    abort();
}
void logger_start_stopwatch(logger *log, const char *n, bool p) { (void)log; (void)n; (void)p; }
void logger_stop_stopwatch(logger *log, const char *n) { (void)log; (void)n; }
int32_t new_fee_beam(const char *f, FEEBeam **b) { (void)f; (void)b; refhost_unreachable("new_fee_beam"); return 1; }
void free_fee_beam(FEEBeam *b) { (void)b; }
int32_t calc_jones(FEEBeam *b, double az, double za, uint32_t f, const uint32_t *d, const double *a, uint32_t n,
                   uint8_t z, const double *lat, uint8_t iau, double *j)
{ (void)b; (void)az; (void)za; (void)f; (void)d; (void)a; (void)n; (void)z; (void)lat; (void)iau; (void)j;
  refhost_unreachable("calc_jones"); return 1; }
int hb_last_error_length(void) { return 1; }
int hb_last_error_message(char *buffer, int length) { if (length > 0) buffer[0] = 0; return 0; }
void palDh2e(double az, double el, double phi, double *ha, double *dec)
{ (void)az; (void)el; (void)phi; (void)ha; (void)dec; refhost_unreachable("palDh2e"); }
double palPa(double ha, double dec, double phi) { (void)ha; (void)dec; (void)phi; refhost_unreachable("palPa"); return 0.0; }

/* primary_beam.c's dead-dipole hash, for parity of vgb_hash_dipole_config */
int refhost_hash_dipole_config(double *amps) { return hash_dipole_config(amps); }
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
