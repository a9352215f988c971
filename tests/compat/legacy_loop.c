/*
 * The tied-array beam program's per-second loop on legacy recombined input
 * (already fine-channelised 4+4-bit voltages, v_IDX [sample][chan][input]),
 * several pointings, compiled against VCSBeam's configured vcsbeam.h and
 * linked to libvcsbeam_compat.so. On legacy data vmBeamformSecond pushes each
 * chunk of the read buffer (vmPushChunk) and forms every pointing's beam
 * (vmApplyJChunk + vmBeamformChunk, form_beam.cpp:587-627); vmSendSToFits
 * renormalises every pointing into its own PSRFITS sub-integration.
 *
 * usage: legacy_loop NANT NPOINTING NSECONDS NCHUNKS INDIR OUTDIR
 *   INDIR: volt.bin  uint8 [NSECONDS][10000][128][2*NANT] (4+4-bit)
 *          i_idx.bin 2*NANT int32: VCS order of antenna a's X (2a) / Y (2a+1)
 *          J.bin     [NSECONDS][NPOINTING][NANT][128][2][2] complex double
 *          phi.bin   [NSECONDS][NPOINTING][NANT][128] complex double
 *   OUTDIR/<name>_<pointing>_<second>.bin: psrfits (uint8 [s][4][128]),
 *          offsets, scales (float [4][128]); S_<second>.bin (float
 *          [pointing][s][4][128]) and e_<second>.bin (complex double
 *          [pointing][s][128][2]).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vcsbeam.h"

static void *read_file(const char *dir, const char *name, size_t bytes)
{
    char path[1024];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "legacy_loop: cannot open %s\n", path); exit(2); }
    void *buf = malloc(bytes);
    if (fread(buf, 1, bytes, f) != bytes) { fprintf(stderr, "legacy_loop: short read %s\n", path); exit(2); }
    fclose(f);
    return buf;
}

static void write_file(const char *dir, const char *name, const void *buf, size_t bytes)
{
    char path[1024];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f || fwrite(buf, 1, bytes, f) != bytes) { fprintf(stderr, "legacy_loop: cannot write %s\n", path); exit(2); }
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc != 7) {
        fprintf(stderr, "usage: legacy_loop NANT NPOINTING NSECONDS NCHUNKS INDIR OUTDIR\n");
        return 2;
    }
    const int nant = atoi(argv[1]), npnt = atoi(argv[2]), nsec = atoi(argv[3]), nchunks = atoi(argv[4]);
    const char *in = argv[5], *out = argv[6];
    const int ninputs = 2 * nant, K = 128, nstokes = 4, ns = 10000;
    const size_t second_bytes = (size_t)ns * K * ninputs;

    MetafitsMetadata obs;
    memset(&obs, 0, sizeof obs);
    int32_t *i_idx = read_file(in, "i_idx.bin", sizeof(int32_t) * ninputs);
    obs.mwa_version = VCSLegacyRecombined;
    obs.num_ants = nant;
    obs.num_rf_inputs = ninputs;
    obs.num_ant_pols = 2;
    obs.num_visibility_pols = 4;

    vcsbeam_context *vm = calloc(1, sizeof(vcsbeam_context));
    vm->obs_metadata = &obs;
    vm->sample_rate = ns;
    vm->fine_sample_rate = ns;
    vm->nfine_chan = K;
    vm->bytes_per_second = (int)second_bytes;
    vm->npointing = npnt;
    vm->num_not_flagged = ninputs;
    vm->out_nstokes = nstokes;
    vm->output_fine_channels = true;
    vm->datatype = VM_INT4;

    vmSetMaxGPUMem(vm, nchunks);
    vmMallocVHost(vm);
    vmMallocVDevice(vm);
    vmMallocJVDevice(vm);
    vmMallocEHost(vm);
    vmMallocEDevice(vm);
    vmMallocSHost(vm);
    vmMallocSDevice(vm);
    vmMallocJHost(vm);
    vmMallocJDevice(vm);
    vmMallocPQIdxsHost(vm);
    vmMallocPQIdxsDevice(vm);
    for (int a = 0; a < nant; a++) {
        vm->polQ_idxs[a] = (uint32_t)i_idx[2 * a];
        vm->polP_idxs[a] = (uint32_t)i_idx[2 * a + 1];
    }
    vmPushPolIdxLists(vm);
    mpi_psrfits *mpfs = calloc(npnt, sizeof(mpi_psrfits));
    for (int p = 0; p < npnt; p++) {
        mpfs[p].coarse_chan_pf.sub.bytes_per_subint = ns * K * nstokes;
        mpfs[p].coarse_chan_pf.sub.data = malloc((size_t)ns * K * nstokes);
        mpfs[p].coarse_chan_pf.sub.dat_offsets = malloc(sizeof(float) * K * nstokes);
        mpfs[p].coarse_chan_pf.sub.dat_scales = malloc(sizeof(float) * K * nstokes);
    }
    vmCreateStatistics(vm, mpfs);
    vmCreateCudaStreams(vm);
    vm->gdelays.npointings = npnt;
    vm->gdelays.nant = nant;
    vm->gdelays.nchan = K;
    const size_t phi_bytes = (size_t)npnt * nant * K * sizeof(gpuDoubleComplex);
    cudaMallocHost((void **)&vm->gdelays.phi, phi_bytes);
    cudaMalloc((void **)&vm->gdelays.d_phi, phi_bytes);

    char *volt = read_file(in, "volt.bin", (size_t)nsec * second_bytes);
    char *J_all = read_file(in, "J.bin", (size_t)nsec * vm->J_size_bytes);
    char *phi_all = read_file(in, "phi.bin", (size_t)nsec * phi_bytes);
    char name[256];
    for (int t = 0; t < nsec; t++) {
        vm->v->locked = true;
        memcpy(vm->v->read_ptr, volt + (size_t)t * second_bytes, vm->v->read_size);
        memcpy(vm->J, J_all + (size_t)t * vm->J_size_bytes, vm->J_size_bytes);
        memcpy(vm->gdelays.phi, phi_all + (size_t)t * phi_bytes, phi_bytes);
        vmPushPhi(vm);
        vmPushJ(vm);
        vmBeamformSecond(vm);
        vmPullE(vm);
        vmPullS(vm);
        vmSendSToFits(vm, mpfs);
        for (int p = 0; p < npnt; p++) {
            snprintf(name, sizeof name, "psrfits_%d_%d.bin", p, t);
            write_file(out, name, mpfs[p].coarse_chan_pf.sub.data, (size_t)ns * K * nstokes);
            snprintf(name, sizeof name, "offsets_%d_%d.bin", p, t);
            write_file(out, name, mpfs[p].coarse_chan_pf.sub.dat_offsets, sizeof(float) * K * nstokes);
            snprintf(name, sizeof name, "scales_%d_%d.bin", p, t);
            write_file(out, name, mpfs[p].coarse_chan_pf.sub.dat_scales, sizeof(float) * K * nstokes);
        }
        snprintf(name, sizeof name, "S_%d.bin", t);
        write_file(out, name, vm->S, vm->S_size_bytes);
        snprintf(name, sizeof name, "e_%d.bin", t);
        write_file(out, name, vm->e, vm->e_size_bytes);
    }
    vmDestroyStatistics(vm);
    vmDestroyCudaStreams(vm);
    vmFreeVDevice(vm);
    vmFreeJVDevice(vm);
    vmFreeEHost(vm);
    vmFreeEDevice(vm);
    vmFreeSHost(vm);
    vmFreeSDevice(vm);
    vmFreeJHost(vm);
    vmFreeJDevice(vm);
    vmFreePQIdxsHost(vm);
    vmFreePQIdxsDevice(vm);
    vmFreeVHost(vm);
    cudaFreeHost(vm->gdelays.phi);
    cudaFree(vm->gdelays.d_phi);
    printf("legacy_loop: %d seconds, %d pointings done\n", nsec, npnt);
    return 0;
}
