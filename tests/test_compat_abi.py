"""VCSBeam's own library API (libvcsbeam_compat.so) without a GPU: the
library exports every function the reference's GPU translation units define,
a VCSBeam program's loop compiles and links against the reference's
configured vcsbeam.h and this library, and, where the VCSBeam sources are
present, the reference's own app/ programs compile against that header and
every symbol they take from pfb.cpp / form_beam.cpp is exported here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "mwa-vcsbeam_gb300", "lib", "libvcsbeam_compat.so")
LIBDIR = os.path.dirname(LIB)
REF_INC = os.path.join(ROOT, "oracle", "_ref", "include")
STUBS = os.path.join(ROOT, "oracle", "ref_stubs")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

# Every function src/pfb.cpp and src/form_beam.cpp define (pfb.cpp:378-1102,
# form_beam.cpp:463-805): this library replaces both files.
GPU_TU_FUNCTIONS = [
    "vmInitForwardPFB", "vmFreeForwardPFB", "vmUploadForwardPFBChunk", "vmWOLAChunk", "vmFPGARoundingChunk",
    "vmFFTChunk", "vmPackChunk", "vmDownloadForwardPFBChunk", "vmExecuteForwardPFB", "vmWritePFBOutputToFile",
    "cu_invert_pfb", "cu_load_ipfb_filter", "malloc_ipfb", "free_ipfb",
    "cu_form_incoh_beam", "vmApplyJChunk", "vmBeamformChunk", "vmBeamformSecond", "vmPullE", "vmPullS",
    "vmSendSToFits", "vmPushPolIdxLists", "create_pinned_data_buffer", "create_detected_beam",
    "create_data_buffer_fine", "prepare_data_buffer_fine", "allocate_input_output_arrays",
    "free_input_output_arrays",
]
# The helpers of metadata.c / geometry.c / buffer.c the loop calls, exported
# weak (a build that keeps those files uses theirs).
WEAK_HELPERS = [
    "vmInitReadBuffer", "vmFreeReadBuffer", "vmReadBufferCopyMargin", "vmMallocVHost", "vmFreeVHost",
    "vmMallocVDevice", "vmFreeVDevice", "vmMallocJVHost", "vmFreeJVHost", "vmMallocJVDevice", "vmFreeJVDevice",
    "vmMallocEHost", "vmFreeEHost", "vmMallocEDevice", "vmFreeEDevice", "vmMallocSHost", "vmFreeSHost",
    "vmMallocSDevice", "vmFreeSDevice", "vmMallocJHost", "vmFreeJHost", "vmMallocJDevice", "vmFreeJDevice",
    "vmMallocDHost", "vmFreeDHost", "vmMallocDDevice", "vmFreeDDevice", "vmMallocPQIdxsHost", "vmFreePQIdxsHost",
    "vmMallocPQIdxsDevice", "vmFreePQIdxsDevice", "vmSetMaxGPUMem", "vmPushChunk", "vmPushJ", "vmPushPhi",
    "vmCreateCudaStreams", "vmDestroyCudaStreams", "vmCreateStatistics", "vmDestroyStatistics",
]


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    syms = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) == 3:
            syms[parts[2]] = parts[1]
    return syms


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(os.path.join(REF_INC, "vcsbeam.h")):
        pytest.skip("no configured vcsbeam.h (oracle/build_ref.sh needs the VCSBeam sources)")
    if not os.path.exists(LIB):
        import __graft_entry__ as G

        G.build()
    return exported(LIB)


def test_exports_the_gpu_translation_units(lib):
    missing = [f for f in GPU_TU_FUNCTIONS if f not in lib]
    assert not missing, missing
    assert all(lib[f] == "T" for f in GPU_TU_FUNCTIONS)


def test_exports_the_loop_helpers_weak(lib):
    missing = [f for f in WEAK_HELPERS if f not in lib]
    assert not missing, missing
    assert all(lib[f] == "W" for f in WEAK_HELPERS)


@pytest.mark.parametrize("prog", ["app_loop", "legacy_loop"])
def test_program_loop_compiles_and_links(lib, tmp_path, prog):
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    exe = tmp_path / prog
    subprocess.run(["gcc", "-O2", "-D__NVCC__", "-Wall", "-Werror", "-Wno-unused-function",
                    "-I", REF_INC, "-I", STUBS, "-I", os.path.join(CUDA, "include"),
                    os.path.join(ROOT, "tests", "compat", f"{prog}.c"), "-o", str(exe), "-L", LIBDIR,
                    "-lvcsbeam_compat", "-lvcsbeam_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
                    f"-Wl,-rpath,{LIBDIR}"], check=True)
    assert exe.exists()


@pytest.mark.parametrize("prog", ["make_mwa_tied_array_beam", "fine_pfb_offline", "make_mwa_incoh_beam"])
def test_reference_programs_take_their_gpu_symbols_from_here(lib, prog, tmp_path):
    ref_root = os.environ.get("VGB_REFERENCE_DIR", "")
    marker = os.path.join(ROOT, "oracle", "_ref", "source_dir")
    if not ref_root and os.path.exists(marker):
        ref_root = open(marker).read().strip()
    src = os.path.join(ref_root, "app", f"{prog}.c")
    if not os.path.exists(src):
        pytest.skip("VCSBeam app sources not available (oracle/build_ref.sh links them)")
    obj = tmp_path / f"{prog}.o"
    subprocess.run(["gcc", "-O2", "-D__NVCC__", "-w", "-c", "-I", REF_INC, "-I", STUBS,
                    "-I", os.path.join(ref_root, "src"), "-I", os.path.join(CUDA, "include"), src, "-o", str(obj)],
                   check=True)
    und = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True, check=True).stdout.split()
    wanted = [s for s in und if s in GPU_TU_FUNCTIONS]
    assert wanted, "the program calls none of the GPU entry points"
    assert all(s in lib for s in wanted), [s for s in wanted if s not in lib]
