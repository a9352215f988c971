// Voltage file readers on the host: one second of one coarse channel into a
// caller's (pinned) buffer, in the layout the pipeline and vgb_voltages take.
// They stand in for mwalib_voltage_context_read_second (metadata.c:973-985,
// app/make_mwa_incoh_beam.c:333-345) and mwalib's expected file names
// (metadata.c:1214-1226), which VCSBeam gets from the mwalib library.
//
// MWAX voltage subfiles (<obsid>_<gps>_<receiver channel>.sub, 8 s each): an
// ASCII "KEY value" header of HDR_SIZE bytes, one block of per-input delay
// metadata, then 20 blocks per second of [input][64000 samples] char2 (the
// reference's vMWAX_IDX layout, vcsbeam.h.in:238-240). Legacy recombined
// files (<obsid>_<gps>_ch<receiver channel>.dat, 1 s each, no header) hold
// [10000 samples][128 channels][256 inputs] 4+4-bit bytes (v_IDX).
//
// A second is read with several positioned reads in parallel (one contiguous
// range per thread), straight into the destination.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "vcsbeam_gb300.h"

namespace vgb {
int set_error(int code, const char *fmt, ...);
}
using vgb::set_error;

namespace {

constexpr int kBlocksPerSecond = 20;       // 1.28 MHz / 64000 samples
constexpr long long kDefaultHeaderBytes = 4096;

struct Fd {
    int fd = -1;
    ~Fd()
    {
        if (fd >= 0) close(fd);
    }
};

// Read [offset, offset + bytes) of `fd` into dst with `nthreads` positioned
// reads in parallel; returns VGB_SUCCESS or an error for a short or failed read.
int pread_parallel(int fd, const char *path, long long offset, char *dst, long long bytes, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 64) nthreads = 64;
    const long long chunk = ((bytes + nthreads - 1) / nthreads + 4095) / 4096 * 4096;
    std::vector<int> err(nthreads, 0);
    std::vector<long long> got(nthreads, 0);
    auto work = [&](int t) {
        long long lo = t * chunk, hi = lo + chunk < bytes ? lo + chunk : bytes;
        while (lo < hi) {
            const ssize_t r = pread(fd, dst + lo, (size_t)(hi - lo), (off_t)(offset + lo));
            if (r < 0) {
                if (errno == EINTR) continue;
                err[t] = errno;
                return;
            }
            if (r == 0) return; // end of file
            lo += r;
            got[t] += r;
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; t++)
        if ((long long)t * chunk < bytes) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    long long total = 0;
    for (int t = 0; t < nthreads; t++) {
        if (err[t]) return set_error(VGB_ERR_INVALID, "%s: read failed: %s", path, strerror(err[t]));
        total += got[t];
    }
    if (total != bytes)
        return set_error(VGB_ERR_INVALID, "%s: file ends %lld bytes early", path, bytes - total);
    return VGB_SUCCESS;
}

// Value of `key` in a "KEY value" header (lines separated by '\n'), or false.
bool header_value(const std::string &hdr, const char *key, long long &out)
{
    const size_t klen = strlen(key);
    size_t pos = 0;
    while (pos < hdr.size()) {
        size_t end = hdr.find('\n', pos);
        if (end == std::string::npos) end = hdr.size();
        if (end - pos > klen && hdr.compare(pos, klen, key) == 0 && (hdr[pos + klen] == ' ' || hdr[pos + klen] == '\t')) {
            const std::string v = hdr.substr(pos + klen, end - pos - klen);
            char *stop = nullptr;
            out = strtoll(v.c_str(), &stop, 10);
            return stop != v.c_str();
        }
        pos = end + 1;
    }
    return false;
}

} // namespace

extern "C" {

int vgb_subfile_info_read(const char *path, vgb_subfile_info *info)
{
    if (!path || !info) return set_error(VGB_ERR_INVALID, "subfile_info_read: NULL argument");
    Fd f;
    f.fd = open(path, O_RDONLY);
    if (f.fd < 0) return set_error(VGB_ERR_INVALID, "%s: cannot open: %s", path, strerror(errno));
    std::string hdr(kDefaultHeaderBytes, '\0');
    const ssize_t r = pread(f.fd, &hdr[0], hdr.size(), 0);
    if (r < 0) return set_error(VGB_ERR_INVALID, "%s: cannot read the header: %s", path, strerror(errno));
    hdr.resize((size_t)r);
    const size_t nul = hdr.find('\0');
    if (nul != std::string::npos) hdr.resize(nul);
    long long v;
    vgb_subfile_info in{};
    in.header_bytes = header_value(hdr, "HDR_SIZE", v) ? v : kDefaultHeaderBytes;
    if (!header_value(hdr, "NINPUTS", v) || v <= 0 || v > 65536)
        return set_error(VGB_ERR_INVALID, "%s: header has no valid NINPUTS", path);
    in.ninputs = (int)v;
    if (header_value(hdr, "NBIT", v) && v != 8)
        return set_error(VGB_ERR_UNSUPPORTED, "%s: NBIT %lld (8-bit samples expected)", path, v);
    in.secs_per_subobs = header_value(hdr, "SECS_PER_SUBOBS", v) ? (int)v : 8;
    if (in.secs_per_subobs <= 0) return set_error(VGB_ERR_INVALID, "%s: bad SECS_PER_SUBOBS", path);
    in.obs_id = header_value(hdr, "OBS_ID", v) ? v : 0;
    in.subobs_id = header_value(hdr, "SUBOBS_ID", v) ? v : 0;
    in.coarse_channel = header_value(hdr, "COARSE_CHANNEL", v) ? (int)v : -1;
    in.samples_per_block = VGB_SAMPLES_PER_BLOCK;
    in.metadata_blocks = 1;
    in.block_bytes = (long long)in.ninputs * in.samples_per_block * 2;
    if (in.header_bytes < 0) return set_error(VGB_ERR_INVALID, "%s: bad HDR_SIZE", path);
    struct stat st;
    if (fstat(f.fd, &st) != 0) return set_error(VGB_ERR_INVALID, "%s: cannot stat", path);
    const long long need = in.header_bytes + (in.metadata_blocks + (long long)kBlocksPerSecond * in.secs_per_subobs) *
                                                 in.block_bytes;
    in.file_bytes = (long long)st.st_size;
    in.complete = in.file_bytes >= need ? 1 : 0;
    *info = in;
    return VGB_SUCCESS;
}

int vgb_subfile_read_second(const char *path, long long gps_second, void *dst, long long dst_bytes, int nthreads)
{
    if (!path || !dst) return set_error(VGB_ERR_INVALID, "subfile_read_second: NULL argument");
    vgb_subfile_info in;
    int rc = vgb_subfile_info_read(path, &in);
    if (rc) return rc;
    const long long k = gps_second - in.subobs_id;
    if (k < 0 || k >= in.secs_per_subobs)
        return set_error(VGB_ERR_INVALID, "%s: GPS second %lld is outside the file (%lld + %d s)", path, gps_second,
                         in.subobs_id, in.secs_per_subobs);
    const long long bytes = kBlocksPerSecond * in.block_bytes;
    if (dst_bytes < bytes)
        return set_error(VGB_ERR_INVALID, "subfile_read_second: destination holds %lld bytes, a second is %lld",
                         dst_bytes, bytes);
    Fd f;
    f.fd = open(path, O_RDONLY);
    if (f.fd < 0) return set_error(VGB_ERR_INVALID, "%s: cannot open: %s", path, strerror(errno));
    const long long offset = in.header_bytes + (in.metadata_blocks + k * kBlocksPerSecond) * in.block_bytes;
    return pread_parallel(f.fd, path, offset, static_cast<char *>(dst), bytes, nthreads);
}

int vgb_legacy_read_second(const char *path, void *dst, long long dst_bytes, int nthreads)
{
    if (!path || !dst) return set_error(VGB_ERR_INVALID, "legacy_read_second: NULL argument");
    if (dst_bytes <= 0) return set_error(VGB_ERR_INVALID, "legacy_read_second: empty destination");
    Fd f;
    f.fd = open(path, O_RDONLY);
    if (f.fd < 0) return set_error(VGB_ERR_INVALID, "%s: cannot open: %s", path, strerror(errno));
    return pread_parallel(f.fd, path, 0, static_cast<char *>(dst), dst_bytes, nthreads);
}

int vgb_volt_filename(char *out, int out_len, long long obs_id, long long gps_second, int rec_chan, int mwax)
{
    if (!out || out_len <= 0) return set_error(VGB_ERR_INVALID, "volt_filename: NULL argument");
    int n;
    if (mwax) {
        // 8-second subfiles named by the GPS second they start at, a multiple
        // of 8 (metadata.c:1152)
        const long long start = gps_second - gps_second % 8;
        n = snprintf(out, (size_t)out_len, "%lld_%lld_%03d.sub", obs_id, start, rec_chan);
    } else {
        n = snprintf(out, (size_t)out_len, "%lld_%lld_ch%03d.dat", obs_id, gps_second, rec_chan);
    }
    if (n < 0 || n >= out_len) return set_error(VGB_ERR_INVALID, "volt_filename: buffer too short");
    return VGB_SUCCESS;
}

} // extern "C"
