// Host-side table inputs of the beamformer: calibration solutions (the D of
// J = D B), their corrections and tile flags (calibration.c), and PFB filter
// coefficient files (filter.c). One-off per observation or per second; they
// run on the host and hand D / filter taps to the device kernels.
//
// Layouts follow the reference: D [ant][fine channel][2][2] complex double
// (D_IDX, vcsbeam.h.in:242-251); Offringa solutions as described by its
// reader (calibration.c:426-582, header of 48 bytes, 64-byte Jones matrices);
// RTS DIJones / Bandpass text files (calibration.c:227-412).
#include <cuComplex.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "vcsbeam_gb300.h"

namespace vgb {
int set_error(int code, const char *fmt, ...);
}
using vgb::set_error;

namespace {

constexpr long kOffringaHeaderBytes = 48;
constexpr long kJonesBytes = 64;
constexpr int kBandpassRowsPerAnt = 8;

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) : f(path ? std::fopen(path, mode) : nullptr) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

// 2x2 complex helpers with the reference's operation order (jones.c).
void mult2x2(const cuDoubleComplex *a, const cuDoubleComplex *b, cuDoubleComplex *out)
{
    cuDoubleComplex m[4];
    m[0] = cuCadd(cuCmul(a[0], b[0]), cuCmul(a[1], b[2]));
    m[1] = cuCadd(cuCmul(a[0], b[1]), cuCmul(a[1], b[3]));
    m[2] = cuCadd(cuCmul(a[2], b[0]), cuCmul(a[3], b[2]));
    m[3] = cuCadd(cuCmul(a[2], b[1]), cuCmul(a[3], b[3]));
    std::memcpy(out, m, sizeof(m));
}

// inverse via the determinant and its reciprocal (jones.c:212-260)
void inv2x2(const cuDoubleComplex *m, cuDoubleComplex *out)
{
    const cuDoubleComplex det = cuCsub(cuCmul(m[0], m[3]), cuCmul(m[1], m[2]));
    const double scale = 1.0 / (det.x * det.x + det.y * det.y);
    const cuDoubleComplex inv_det = make_cuDoubleComplex(scale * det.x, -scale * det.y);
    const cuDoubleComplex neg_inv = make_cuDoubleComplex(-inv_det.x, -inv_det.y);
    cuDoubleComplex r[4];
    r[0] = cuCmul(inv_det, m[3]);
    r[1] = cuCmul(neg_inv, m[1]);
    r[2] = cuCmul(neg_inv, m[2]);
    r[3] = cuCmul(inv_det, m[0]);
    std::memcpy(out, r, sizeof(r));
}

// element order reversal (jones.c:439-449): [a b; c d] -> [d c; b a]
void reverse2x2(const cuDoubleComplex *m, cuDoubleComplex *out)
{
    cuDoubleComplex r[4] = {m[3], m[2], m[1], m[0]};
    std::memcpy(out, r, sizeof(r));
}

// Reads the next number of a comma/whitespace separated text stream the way
// fscanf("%lf,") does: leading white space skipped, one optional comma eaten.
bool read_num(FILE *f, double *v)
{
    if (std::fscanf(f, "%lf", v) != 1) return false;
    int c = std::fgetc(f);
    if (c != ',' && c != EOF) std::ungetc(c, f);
    return true;
}

} // namespace

extern "C" int vgb_cal_load_offringa(const char *path, int coarse_chan_idx, int ncc, int nant, int nchan_cal,
                                     int nfine, double *D, uint32_t *counts)
{
    if (!path || !D) return set_error(VGB_ERR_INVALID, "cal_load_offringa: NULL argument");
    if (nant <= 0 || nchan_cal <= 0 || nfine <= 0 || ncc <= 0 || coarse_chan_idx < 0)
        return set_error(VGB_ERR_INVALID, "cal_load_offringa: sizes must be positive");
    File fp(path, "rb");
    if (!fp.f) return set_error(VGB_ERR_INVALID, "cal_load_offringa: cannot open %s", path);
    uint32_t hdr[4];
    if (std::fseek(fp.f, 16, SEEK_SET) || std::fread(hdr, sizeof(uint32_t), 4, fp.f) != 4)
        return set_error(VGB_ERR_INVALID, "cal_load_offringa: %s is too short for the header", path);
    if (counts) std::memcpy(counts, hdr, sizeof(hdr));
    const uint32_t antennaCount = hdr[1], channelCount = hdr[2];
    if ((int)antennaCount != nant)
        return set_error(VGB_ERR_INVALID, "cal_load_offringa: %s holds %u antennas, %d requested", path,
                         antennaCount, nant);
    // the solution's channel count wins when it differs from the request
    uint32_t nChan = (uint32_t)nchan_cal * (uint32_t)ncc;
    uint32_t nchan = (uint32_t)nchan_cal;
    if (channelCount != nChan) {
        nChan = channelCount;
        nchan = nChan / (uint32_t)ncc;
    }
    if (nchan == 0) return set_error(VGB_ERR_INVALID, "cal_load_offringa: no channels per coarse channel");
    const uint32_t interp = (uint32_t)nfine / nchan;
    double J[8];
    for (int ant = 0; ant < nant; ant++) {
        for (uint32_t ch = 0; ch < nchan; ch++) {
            const uint32_t Ch = ch + (uint32_t)coarse_chan_idx * nchan;
            const long pos = kOffringaHeaderBytes + (long)ant * ((long)nChan * kJonesBytes) + (long)Ch * kJonesBytes;
            if (std::fseek(fp.f, pos, SEEK_SET) || std::fread(J, 1, kJonesBytes, fp.f) != (size_t)kJonesBytes)
                return set_error(VGB_ERR_INVALID, "cal_load_offringa: %s ends before antenna %d channel %u", path,
                                 ant, Ch);
            if (std::isnan(J[0])) std::memset(J, 0, sizeof(J)); // a NaN matrix is a flagged one
            for (uint32_t v = ch * interp; v < (ch + 1) * interp; v++)
                std::memcpy(D + 8 * ((size_t)ant * nfine + v), J, sizeof(J));
        }
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_cal_load_rts(const char *dijones_path, const char *bandpass_path, int nant_cal, int nchan_cal,
                                int chan_width_hz, const int *cal_ant, int nant, int nfine, double *D)
{
    if (!dijones_path || !cal_ant || !D) return set_error(VGB_ERR_INVALID, "cal_load_rts: NULL argument");
    if (nant_cal <= 0 || nchan_cal <= 0 || nant <= 0 || nfine <= 0 || chan_width_hz <= 0)
        return set_error(VGB_ERR_INVALID, "cal_load_rts: sizes must be positive");
    for (int a = 0; a < nant; a++)
        if (cal_ant[a] < 0 || cal_ant[a] >= nant_cal)
            return set_error(VGB_ERR_INVALID, "cal_load_rts: cal_ant[%d] = %d out of range", a, cal_ant[a]);

    // DIJones: amplitude, alignment matrix A, then one Jones matrix per antenna
    std::vector<cuDoubleComplex> Dd((size_t)nant_cal * 4);
    cuDoubleComplex A[4];
    {
        File fp(dijones_path, "r");
        if (!fp.f) return set_error(VGB_ERR_INVALID, "cal_load_rts: cannot open %s", dijones_path);
        double amp;
        if (std::fscanf(fp.f, "%lf", &amp) != 1)
            return set_error(VGB_ERR_INVALID, "cal_load_rts: %s has no amplitude", dijones_path);
        double *Ad = reinterpret_cast<double *>(A);
        for (int i = 0; i < 8; i++)
            if (!read_num(fp.f, &Ad[i]))
                return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: alignment matrix is short", dijones_path);
        double *Jd = reinterpret_cast<double *>(Dd.data());
        for (int i = 0; i < 8 * nant_cal; i++)
            if (!read_num(fp.f, &Jd[i]))
                return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: fewer than %d Jones matrices", dijones_path,
                                 nant_cal);
    }
    cuDoubleComplex Ainv[4];
    inv2x2(A, Ainv);

    // Bandpass: fitted matrices (odd rows); channels and antennas absent from
    // the file stay zero, i.e. flagged
    std::vector<cuDoubleComplex> Db;
    if (bandpass_path) {
        Db.assign((size_t)nant_cal * nchan_cal * 4, make_cuDoubleComplex(0.0, 0.0));
        File fp(bandpass_path, "r");
        if (!fp.f) return set_error(VGB_ERR_INVALID, "cal_load_rts: cannot open %s", bandpass_path);
        std::vector<char> line(4096);
        if (!std::fgets(line.data(), (int)line.size(), fp.f))
            return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: no frequency row", bandpass_path);
        std::vector<int> chan_idx;
        const char *p = line.data();
        double mhz;
        int pos;
        while (std::sscanf(p, "%lf,%n", &mhz, &pos) == 1) {
            if ((int)chan_idx.size() >= nchan_cal)
                return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: more than %d channel columns", bandpass_path,
                                 nchan_cal);
            // the reference rounds in single precision (roundf of the double quotient)
            chan_idx.push_back((int)std::roundf((float)(mhz * 1e6 / (double)chan_width_hz)));
            p += pos;
        }
        for (int ci : chan_idx)
            if (ci < 0 || ci >= nchan_cal)
                return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: channel %d out of range", bandpass_path, ci);
        for (int ant = 0; ant < nant_cal; ant++) {
            int cur;
            if (std::fscanf(fp.f, "%d,", &cur) == EOF) break;
            cur--;
            if (cur < ant) return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: antennas out of order", bandpass_path);
            if (cur >= nant_cal)
                return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: antenna %d out of range", bandpass_path, cur + 1);
            ant = cur;
            for (int row = 0; row < kBandpassRowsPerAnt; row++) {
                if (row > 0) {
                    if (std::fscanf(fp.f, "%d,", &cur) != 1 || cur - 1 != ant)
                        return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: fewer than 8 rows for antenna %d",
                                         bandpass_path, ant + 1);
                }
                if (row % 2 == 0) { // measured values: not used
                    if (!std::fgets(line.data(), (int)line.size(), fp.f)) break;
                    continue;
                }
                const int pol = row / 2;
                for (int ci : chan_idx) {
                    double a, ph;
                    if (std::fscanf(fp.f, "%lf,%lf,", &a, &ph) != 2)
                        return set_error(VGB_ERR_INVALID, "cal_load_rts: %s: short row", bandpass_path);
                    Db[((size_t)ant * nchan_cal + ci) * 4 + pol] = make_cuDoubleComplex(a * std::cos(ph), a * std::sin(ph));
                }
            }
        }
    }

    // D = Dd Db Ainv, then reversed into the (q, p) basis
    const int interp = nfine / nchan_cal;
    if (interp <= 0) return set_error(VGB_ERR_INVALID, "cal_load_rts: fewer fine channels than calibration channels");
    for (int a = 0; a < nant; a++) {
        const cuDoubleComplex *dd = &Dd[(size_t)cal_ant[a] * 4];
        for (int ch = 0; ch < nfine; ch++) {
            cuDoubleComplex *d = reinterpret_cast<cuDoubleComplex *>(D + 8 * ((size_t)a * nfine + ch));
            const int cal_ch = ch / interp;
            if (bandpass_path)
                mult2x2(dd, &Db[((size_t)cal_ant[a] * nchan_cal + cal_ch) * 4], d);
            else
                std::memcpy(d, dd, 4 * sizeof(cuDoubleComplex));
            mult2x2(d, Ainv, d);
            reverse2x2(d, d);
        }
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_cal_apply_corrections(double *D, int nant, int nfine, int ref_ant, int keep_cross_terms,
                                         double phase_slope, double phase_offset, long long chan_start_hz,
                                         int coarse_chan_width_hz)
{
    if (!D) return set_error(VGB_ERR_INVALID, "cal_apply_corrections: NULL D");
    if (nant <= 0 || nfine <= 0 || ref_ant >= nant)
        return set_error(VGB_ERR_INVALID, "cal_apply_corrections: bad sizes or reference antenna");
    const bool do_ref = ref_ant >= 0, do_zero = !keep_cross_terms;
    const bool do_slope = phase_offset != 0.0 || phase_slope != 0.0;
    if (!do_ref && !do_zero && !do_slope) return VGB_SUCCESS;
    const int chan_width = coarse_chan_width_hz / nfine;
    cuDoubleComplex *Dc = reinterpret_cast<cuDoubleComplex *>(D);
    for (int ch = 0; ch < nfine; ch++) {
        cuDoubleComplex ref[4], unit[4];
        bool finite[4] = {false, false, false, false};
        if (do_ref) {
            std::memcpy(ref, Dc + 4 * ((size_t)ref_ant * nfine + ch), sizeof(ref));
            // each element of the reference matrix normalised to unit magnitude
            // (remove_reference_phase, calibration.c:617-638)
            for (int i = 0; i < 4; i++) {
                const double s = 1.0 / cuCabs(ref[i]);
                unit[i] = make_cuDoubleComplex(s * cuCreal(ref[i]), s * cuCimag(ref[i]));
                finite[i] = std::isfinite(s);
            }
        }
        cuDoubleComplex z = make_cuDoubleComplex(1.0, 0.0);
        if (do_slope) {
            const long long f = chan_start_hz + (long long)ch * chan_width;
            const double phi = phase_slope * (double)f + phase_offset;
            z = make_cuDoubleComplex(std::cos(phi), std::sin(phi));
        }
        for (int a = 0; a < nant; a++) {
            cuDoubleComplex *d = Dc + 4 * ((size_t)a * nfine + ch);
            if (do_ref)
                for (int i = 0; i < 4; i++)
                    if (finite[i]) d[i] = cuCdiv(d[i], unit[i]);
            if (do_zero) d[1] = d[2] = make_cuDoubleComplex(0.0, 0.0);
            if (do_slope) {
                d[0] = cuCmul(d[0], z);
                d[2] = cuCmul(d[2], z);
            }
        }
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_cal_pq_correction(const char *path, uint32_t gpstime, double *slope, double *offset,
                                     char *ref_tile, int ref_tile_len, int *found)
{
    if (!path || !slope || !offset || !found) return set_error(VGB_ERR_INVALID, "cal_pq_correction: NULL argument");
    File fp(path, "r");
    if (!fp.f) return set_error(VGB_ERR_INVALID, "cal_pq_correction: cannot open %s", path);
    char buf[4096], name[32];
    *found = 0;
    while (std::fgets(buf, sizeof(buf), fp.f)) {
        if (!(buf[0] >= '0' && buf[0] <= '9')) continue;
        unsigned from, to;
        double s, o;
        if (std::sscanf(buf, "%u %u %lf %lf %31s", &from, &to, &s, &o, name) != 5)
            return set_error(VGB_ERR_INVALID, "cal_pq_correction: cannot parse line \"%s\"", buf);
        if (from <= gpstime && gpstime <= to) {
            *slope = s;
            *offset = o;
            *found = 1;
            if (ref_tile && ref_tile_len > 0) {
                std::strncpy(ref_tile, name, (size_t)ref_tile_len - 1);
                ref_tile[ref_tile_len - 1] = '\0';
            }
            return VGB_SUCCESS;
        }
    }
    if (ref_tile && ref_tile_len > 0) {
        std::strncpy(ref_tile, "NONE", (size_t)ref_tile_len - 1);
        ref_tile[ref_tile_len - 1] = '\0';
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_cal_flag_tiles(double *D, int nant, int nfine, const int *ants, int nflags)
{
    if (!D || (nflags > 0 && !ants)) return set_error(VGB_ERR_INVALID, "cal_flag_tiles: NULL argument");
    for (int i = 0; i < nflags; i++) {
        if (ants[i] < 0 || ants[i] >= nant)
            return set_error(VGB_ERR_INVALID, "cal_flag_tiles: antenna %d out of range", ants[i]);
        std::memset(D + 8 * (size_t)ants[i] * nfine, 0, sizeof(double) * 8 * (size_t)nfine);
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_load_filter(const char *path, int nchans, double scale, double *coeffs, int max_coeffs,
                               int *ncoeffs, int *ntaps)
{
    if (!path || !ncoeffs) return set_error(VGB_ERR_INVALID, "load_filter: NULL argument");
    if (nchans <= 0) return set_error(VGB_ERR_INVALID, "load_filter: nchans must be positive");
    File fp(path, "r");
    if (!fp.f) return set_error(VGB_ERR_INVALID, "load_filter: could not find filter '%s'", path);
    // ASCII floating-point numbers separated by white space (filter.c:103-133)
    int n = 0;
    double v;
    while (std::fscanf(fp.f, "%lf", &v) == 1) {
        if (coeffs && n < max_coeffs) coeffs[n] = v * scale;
        n++;
    }
    if (n == 0) return set_error(VGB_ERR_INVALID, "load_filter: no coefficients found in '%s'", path);
    *ncoeffs = n;
    if (ntaps) *ntaps = n / nchans;
    if (coeffs && n > max_coeffs)
        return set_error(VGB_ERR_INVALID, "load_filter: '%s' holds %d coefficients, room for %d", path, n, max_coeffs);
    return VGB_SUCCESS;
}
