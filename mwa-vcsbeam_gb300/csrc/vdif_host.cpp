// VDIF frame headers on the host: the header template of a second's first
// frame, as VCSBeam builds it through vdifio (beam_vdif.c:154-246:
// createVDIFHeader, setVDIFEpochMJD, setVDIFFrameMJDSec, setVDIFFrameNumber)
// and advances it frame by frame (nextVDIFHeader, beam_vdif.c:80).
//
// The words follow the VDIF 1.0 specification (and vdifio's vdif_header bit
// fields, least significant bit first):
//   w0: seconds from the reference epoch [0, 30), legacy [30], invalid [31]
//   w1: frame number within the second [0, 24), reference epoch [24, 30)
//       (half-years since 2000-01-01 00:00 UT)
//   w2: frame length in units of 8 bytes [0, 24), log2(channels) [24, 29),
//       version [29, 32)
//   w3: station id [0, 16), thread id [16, 26), bits per sample - 1 [26, 31),
//       complex [31]
//   w4..w7: extended user data (zero)
#include <cmath>
#include <cstdint>
#include <cstring>

#include "vcsbeam_gb300.h"

namespace vgb {
int set_error(int code, const char *fmt, ...);
}

namespace {

constexpr int kVdifHeaderBytes = 32;
constexpr long long kMjdUnixEpoch = 40587; // MJD of 1970-01-01

// Days since 1970-01-01 of a proleptic Gregorian date, and back (the
// era-based civil-calendar conversion: 400-year eras of 146097 days).
long long days_from_civil(long long y, int m, int d)
{
    y -= m <= 2;
    const long long era = (y >= 0 ? y : y - 399) / 400;
    const long long yoe = y - era * 400;
    const long long doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
    const long long doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
    return era * 146097 + doe - 719468;
}

void civil_from_days(long long z, long long &y, int &m, int &d)
{
    z += 719468;
    const long long era = (z >= 0 ? z : z - 146096) / 146097;
    const long long doe = z - era * 146097;
    const long long yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
    const long long doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
    const long long mp = (5 * doy + 2) / 153;
    d = (int)(doy - (153 * mp + 2) / 5 + 1);
    m = (int)(mp < 10 ? mp + 3 : mp - 9);
    y = yoe + era * 400 + (m <= 2);
}

// MJD of the first day of reference epoch `e` (January or July of 2000 + e/2).
long long epoch_mjd(int e) { return days_from_civil(2000 + e / 2, 1 + 6 * (e % 2), 1) + kMjdUnixEpoch; }

} // namespace

extern "C" {

int vgb_vdif_header_create(uint32_t *hdr, int dataarraylength, int threadid, int bits, int nchan, int iscomplex,
                           const char *stationid)
{
    if (!hdr || !stationid) return vgb::set_error(VGB_ERR_INVALID, "vdif header: NULL argument");
    if (bits < 1 || bits > 32) return vgb::set_error(VGB_ERR_INVALID, "vdif header: bits must be 1..32");
    if (dataarraylength <= 0 || dataarraylength % 8)
        return vgb::set_error(VGB_ERR_INVALID, "vdif header: data array length must be a positive multiple of 8");
    if ((dataarraylength + kVdifHeaderBytes) / 8 >= (1 << 24))
        return vgb::set_error(VGB_ERR_INVALID, "vdif header: frame too long");
    if (threadid < 0 || threadid >= 1024) return vgb::set_error(VGB_ERR_INVALID, "vdif header: thread id must be 0..1023");
    int lognchan = 0;
    while ((1 << lognchan) < nchan && lognchan < 31) lognchan++;
    if (nchan <= 0 || (1 << lognchan) != nchan || lognchan > 31)
        return vgb::set_error(VGB_ERR_INVALID, "vdif header: channels must be a power of two");
    std::memset(hdr, 0, kVdifHeaderBytes);
    const uint32_t station = ((uint32_t)(unsigned char)stationid[0] << 8) |
                             (stationid[0] ? (uint32_t)(unsigned char)stationid[1] : 0u);
    hdr[2] = (uint32_t)((dataarraylength + kVdifHeaderBytes) / 8) | ((uint32_t)lognchan << 24);
    hdr[3] = (station & 0xFFFFu) | ((uint32_t)threadid << 16) | ((uint32_t)(bits - 1) << 26) |
             ((iscomplex ? 1u : 0u) << 31);
    return VGB_SUCCESS;
}

int vgb_vdif_header_set_epoch_mjd(uint32_t *hdr, int mjd)
{
    if (!hdr) return vgb::set_error(VGB_ERR_INVALID, "vdif header: NULL argument");
    long long y;
    int m, d;
    civil_from_days((long long)mjd - kMjdUnixEpoch, y, m, d);
    const long long e = 2 * (y - 2000) + (m >= 7 ? 1 : 0);
    if (e < 0 || e >= 64) return vgb::set_error(VGB_ERR_INVALID, "vdif header: MJD %d outside epochs 2000-2031", mjd);
    hdr[1] = (hdr[1] & ~(0x3Fu << 24)) | ((uint32_t)e << 24);
    return VGB_SUCCESS;
}

int vgb_vdif_header_epoch_mjd(const uint32_t *hdr, int *mjd)
{
    if (!hdr || !mjd) return vgb::set_error(VGB_ERR_INVALID, "vdif header: NULL argument");
    *mjd = (int)epoch_mjd((int)((hdr[1] >> 24) & 0x3Fu));
    return VGB_SUCCESS;
}

int vgb_vdif_header_set_mjdsec(uint32_t *hdr, long long mjdsec)
{
    if (!hdr) return vgb::set_error(VGB_ERR_INVALID, "vdif header: NULL argument");
    const long long s = mjdsec - epoch_mjd((int)((hdr[1] >> 24) & 0x3Fu)) * 86400LL;
    if (s < 0 || s >= (1LL << 30))
        return vgb::set_error(VGB_ERR_INVALID, "vdif header: %lld s outside the header's reference epoch", mjdsec);
    hdr[0] = (hdr[0] & 0xC0000000u) | (uint32_t)s;
    return VGB_SUCCESS;
}

int vgb_vdif_header_set_frame(uint32_t *hdr, int frame)
{
    if (!hdr) return vgb::set_error(VGB_ERR_INVALID, "vdif header: NULL argument");
    if (frame < 0 || frame >= (1 << 24)) return vgb::set_error(VGB_ERR_INVALID, "vdif header: bad frame number");
    hdr[1] = (hdr[1] & 0xFF000000u) | (uint32_t)frame;
    return VGB_SUCCESS;
}

int vgb_vdif_header_next(uint32_t *hdr, int frames_per_second)
{
    if (!hdr || frames_per_second <= 0) return vgb::set_error(VGB_ERR_INVALID, "vdif header: bad argument");
    uint32_t frame = (hdr[1] & 0xFFFFFFu) + 1;
    if (frame >= (uint32_t)frames_per_second) {
        frame = 0;
        hdr[0] = (hdr[0] & 0xC0000000u) | ((hdr[0] + 1) & 0x3FFFFFFFu);
    }
    hdr[1] = (hdr[1] & 0xFF000000u) | frame;
    return VGB_SUCCESS;
}

int vgb_vdif_populate_header(uint32_t *hdr, int intmjd, double fracmjd, int threadid, const char *stationid)
{
    // beam_vdif.c:178-209: 8-bit complex samples, 2 channels (one per pol),
    // 128 samples per frame (512 data bytes); epoch from the day, seconds from
    // the day plus the fraction rounded to a whole second, frame 0.
    int rc = vgb_vdif_header_create(hdr, 2 * 2 * 128, threadid, 8, 2, 1, stationid ? stationid : "mw");
    if (rc) return rc;
    if ((rc = vgb_vdif_header_set_epoch_mjd(hdr, intmjd))) return rc;
    const long long mjdsec = (long long)intmjd * 86400LL + (long long)roundf((float)(fracmjd * 86400.0));
    if ((rc = vgb_vdif_header_set_mjdsec(hdr, mjdsec))) return rc;
    return vgb_vdif_header_set_frame(hdr, 0);
}

} // extern "C"
