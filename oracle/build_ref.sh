#!/usr/bin/env bash
# Build recipe for the reference-side checker (test infrastructure only).
#
# Compiles the UNMODIFIED VCSBeam sources where they lie (default
# /root/reference, override with VGB_REFERENCE_DIR) against the stand-in
# headers in oracle/ref_stubs/, writing only into oracle/_ref/:
#
#   oracle/_ref/include/vcsbeam.h   configured from include/vcsbeam.h.in, with
#                                   src/gpu_includes.h, gpu_macros.h and
#                                   gpu_fft.hpp beside it
#   oracle/_ref/ref_pfb.cubin       device code of src/pfb.cpp       (sm_103a)
#   oracle/_ref/ref_form_beam.cubin device code of src/form_beam.cpp (sm_103a)
#   oracle/_ref/libref_host.so      src/jones.c, src/filter.c, src/geometry.c,
#                                   src/calibration.c, src/primary_beam.c
#                                   + oracle/ref_host_shim.c (host, this machine)
#   oracle/_ref/runtime/            RUNTIME_DIR: links to the reference's
#                                   pfb_filter/*.dat and pq_phase_correction.txt
#   oracle/_ref/source_dir          the VCSBeam source tree's path (text)
#
# The cubins travel to a GPU machine with the repository; there
# oracle/ref_harness.cu (built by __graft_entry__.build()) loads them with the
# CUDA driver API and launches the reference kernels with the reference's own
# launch shapes. Nothing here is part of the shipped library.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${VGB_REFERENCE_DIR:-/root/reference}"
OUT="$HERE/_ref"
CUDA_HOME="${CUDA_HOME:-/usr/local/cuda}"
NVCC="${NVCC:-$CUDA_HOME/bin/nvcc}"

if [ ! -f "$REF/src/pfb.cpp" ]; then
    echo "build_ref.sh: reference sources not found at $REF; nothing to build"
    exit 0
fi
mkdir -p "$OUT/include" "$OUT/runtime"
# where the source tree is, for CPU tests that compile the reference's own
# programs against the configured header (a path, not a link, so that no
# copy of the tree follows the build output anywhere)
rm -f "$OUT/source"
printf '%s\n' "$REF" > "$OUT/source_dir"
for f in "$REF"/pfb_filter/*.dat "$REF/pq_phase_correction.txt"; do
    [ -f "$f" ] && ln -sf "$f" "$OUT/runtime/$(basename "$f")"
done

# the reference's GPU portability headers that vcsbeam.h includes, beside it,
# so that code compiled against the configured header needs only _ref/include
for f in gpu_includes.h gpu_macros.h gpu_fft.hpp; do
    cp -f "$REF/src/$f" "$OUT/include/$f"
done

# include/vcsbeam.h.in -> vcsbeam.h (the three #cmakedefine lines only)
sed -e "s|^#cmakedefine VCSBEAM_VERSION.*|#define VCSBEAM_VERSION \"reference\"|" \
    -e "s|^#cmakedefine RUNTIME_DIR.*|#define RUNTIME_DIR \"$OUT/runtime\"|" \
    -e "s|^#cmakedefine HYPERBEAM_HDF5.*|#define HYPERBEAM_HDF5 \"\"|" \
    "$REF/include/vcsbeam.h.in" > "$OUT/include/vcsbeam.h"

INC=(-I"$HERE/ref_stubs" -I"$OUT/include" -I"$REF/src" -I"$CUDA_HOME/include")

# Device code of the two kernel sources, exactly as the reference's CMake
# treats them (.cpp compiled as CUDA with -D__NVCC__).
for f in pfb form_beam; do
    "$NVCC" -cubin -x cu -D__NVCC__ -O3 -gencode arch=compute_103a,code=sm_103a \
        "${INC[@]}" "$REF/src/$f.cpp" -o "$OUT/ref_$f.cubin" &
done

# Host C (table builders) for CPU-side pinning of the oracle.
gcc -O2 -fPIC -shared -D__NVCC__ -w "${INC[@]}" \
    "$REF/src/jones.c" "$REF/src/filter.c" "$REF/src/geometry.c" "$REF/src/calibration.c" \
    "$REF/src/primary_beam.c" \
    "$HERE/ref_host_shim.c" \
    -o "$OUT/libref_host.so" -L"$CUDA_HOME/lib64" -lcudart -lm &
wait
echo "build_ref.sh: built $(ls "$OUT" | tr '\n' ' ')"
