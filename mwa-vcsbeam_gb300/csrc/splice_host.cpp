// Host side of the PSRFITS channel splice when coarse channels are spread
// over processes: the reference gathers every rank's 8-bit sub-integration,
// offsets and scales to the writer rank and interleaves the channels
// (MPI_Igather of the coarse-channel blocks into the spliced types,
// beam_psrfits.c:608-628). With all channels on one GPU the renormalise
// kernel writes the spliced rows directly; with channels on several GPUs each
// process's pipeline writes spliced rows of its own channels and the writer
// places them with this call after a host-staged gather.
#include <cstring>

#include "vcsbeam_gb300.h"

namespace vgb {
int set_error(int code, const char *fmt, ...);
}

extern "C" int vgb_splice_psrfits(const uint8_t *part, int nspectra, int nstokes, int nchan, int ncc_part,
                                  int cc_offset, int ncc_total, uint8_t *out)
{
    if (!part || !out) return vgb::set_error(VGB_ERR_INVALID, "splice_psrfits: NULL buffer");
    if (nspectra < 0 || nstokes <= 0 || nchan <= 0 || ncc_part < 0 || cc_offset < 0 ||
        cc_offset + ncc_part > ncc_total)
        return vgb::set_error(VGB_ERR_INVALID,
                              "splice_psrfits: channels [%d, %d) outside the %d of the spliced rows", cc_offset,
                              cc_offset + ncc_part, ncc_total);
    const size_t w_part = (size_t)ncc_part * nchan, w_all = (size_t)ncc_total * nchan;
    for (long long r = 0; r < (long long)nspectra * nstokes; r++)
        std::memcpy(out + r * w_all + (size_t)cc_offset * nchan, part + r * w_part, w_part);
    return VGB_SUCCESS;
}
