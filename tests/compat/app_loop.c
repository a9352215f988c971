/*
 * A VCSBeam program's per-second loop, written against VCSBeam's own
 * configured vcsbeam.h and linked to libvcsbeam_compat.so (the vm* / cu_*
 * entry points on the GB300 kernels) instead of the reference's pfb.cpp and
 * form_beam.cpp. The calls and their order follow the tied-array beam
 * program (app/make_mwa_tied_array_beam.c:105-308): vmInitForwardPFB,
 * create_data_buffer_fine, vmSetMaxGPUMem, the vmMalloc* calls,
 * vmPushPolIdxLists, create_pinned_data_buffer, malloc_ipfb,
 * cu_load_ipfb_filter, vmCreateStatistics, then per second vmPushPhi,
 * vmPushJ, vmBeamformSecond, vmPullE, prepare_data_buffer_fine,
 * cu_invert_pfb, vmPullS, vmSendSToFits.
 *
 * What comes from mwalib / PAL / hyperbeam in the real program comes from
 * files here: the metadata (antennas, RF inputs and their VCS order) is
 * filled in directly, each second's voltages are read from a file into the
 * read buffer where mwalib_voltage_context_read_second would put them
 * (after vmReadBufferCopyMargin, as vmReadNextSecond does), and each
 * second's J^-1 and phi (vmCalcJonesAndDelays) are read from files.
 *
 * usage: app_loop NANT NSECONDS NCHUNKS INDIR OUTDIR
 *   INDIR: volt.bin  int8 [(1 + 20*NSECONDS) blocks][2*NANT][64000][2]
 *                    (block 0 is the read buffer's first margin)
 *          ana.bin   1536 doubles (analysis filter)
 *          syn.bin   1536 doubles (synthesis filter, already scaled)
 *          i_idx.bin 2*NANT int32: VCS order of MWAX input 2a + pol
 *          J.bin     [NSECONDS][NANT][128][2][2] complex double
 *          phi.bin   [NSECONDS][NANT][128] complex double
 *   OUTDIR/<name>_<second>.bin: psrfits (uint8 [s][4][128]), offsets,
 *          scales (float [4][128]), vdif (float [s*128][2][2]), S (float
 *          [s][4][128]), e (complex double [s][128][2]).
 * Exit status 0 on success; the library ends the process on an error.
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
    if (!f) { fprintf(stderr, "app_loop: cannot open %s\n", path); exit(2); }
    void *buf = malloc(bytes);
    if (fread(buf, 1, bytes, f) != bytes) { fprintf(stderr, "app_loop: short read %s\n", path); exit(2); }
    fclose(f);
    return buf;
}

static void write_file(const char *dir, const char *name, int t, const void *buf, size_t bytes)
{
    char path[1024];
    snprintf(path, sizeof path, "%s/%s_%d.bin", dir, name, t);
    FILE *f = fopen(path, "wb");
    if (!f || fwrite(buf, 1, bytes, f) != bytes) { fprintf(stderr, "app_loop: cannot write %s\n", path); exit(2); }
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc != 6) { fprintf(stderr, "usage: app_loop NANT NSECONDS NCHUNKS INDIR OUTDIR\n"); return 2; }
    const int nant = atoi(argv[1]), nsec = atoi(argv[2]), nchunks = atoi(argv[3]);
    const char *in = argv[4], *out = argv[5];
    const int ninputs = 2 * nant, K = 128, nstokes = 4;
    const size_t block_bytes = (size_t)ninputs * 64000 * 2;

    /* metadata mwalib would supply */
    MetafitsMetadata obs;
    VoltageMetadata vcs;
    memset(&obs, 0, sizeof obs);
    memset(&vcs, 0, sizeof vcs);
    int32_t *i_idx = read_file(in, "i_idx.bin", sizeof(int32_t) * ninputs);
    Rfinput *rf = calloc(ninputs, sizeof(Rfinput));
    for (int i = 0; i < ninputs; i++) {
        rf[i].input = i;
        rf[i].ant = i / 2;
        rf[i].pol = (i % 2) ? "Y" : "X";
        rf[i].vcs_order = (uint32_t)i_idx[i];
    }
    obs.mwa_version = VCSMWAXv2;
    obs.num_ants = nant;
    obs.rf_inputs = rf;
    obs.num_rf_inputs = ninputs;
    obs.num_ant_pols = 2;
    obs.num_visibility_pols = 4;
    vcs.mwa_version = VCSMWAXv2;
    vcs.num_samples_per_voltage_block = 64000;
    vcs.num_voltage_blocks_per_second = 20;
    vcs.voltage_block_size_bytes = block_bytes;

    vcsbeam_context *vm = calloc(1, sizeof(vcsbeam_context));
    vm->obs_metadata = &obs;
    vm->vcs_metadata = &vcs;
    vm->sample_rate = 1280000;
    vm->bytes_per_second = (int)(20 * block_bytes);
    vm->npointing = 1;
    vm->num_not_flagged = ninputs;
    vm->do_forward_pfb = true;
    vm->do_inverse_pfb = true;
    vm->output_fine_channels = true;
    vm->out_nstokes = nstokes;
    vm->chunks_per_second = nchunks;

    pfb_filter ana = {read_file(in, "ana.bin", 1536 * sizeof(double)), 1536, 12, 128, NULL, ANALYSIS_FILTER};
    pfb_filter syn = {read_file(in, "syn.bin", 1536 * sizeof(double)), 1536, 12, 128, NULL, SYNTHESIS_FILTER};
    vm->analysis_filter = &ana;
    vm->synth_filter = &syn;

    /* set-up, in the tied-array beam program's order */
    vmInitForwardPFB(vm, K, PFB_FULL_PRECISION);
    const int nchans = vm->nfine_chan, npols = 2;
    const int nsamples = vm->fine_sample_rate;
    gpuDoubleComplex *data_buffer_fine = create_data_buffer_fine(vm->npointing, 2 * nsamples, nchans, npols);
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
    vmMallocDHost(vm);
    vmMallocDDevice(vm);
    vmMallocPQIdxsHost(vm);
    vmMallocPQIdxsDevice(vm);
    for (int a = 0; a < nant; a++) { /* vmSetPolIdxLists: the VCS order of each antenna's X and Y input */
        vm->polQ_idxs[a] = (uint32_t)i_idx[2 * a];
        vm->polP_idxs[a] = (uint32_t)i_idx[2 * a + 1];
    }
    vmPushPolIdxLists(vm);
    struct gpu_ipfb_arrays gi;
    float *data_buffer_vdif = create_pinned_data_buffer((size_t)nsamples * nchans * npols * vm->npointing * 2 *
                                                        sizeof(float));
    malloc_ipfb(&gi, vm->synth_filter, nsamples, npols, vm->npointing);
    cu_load_ipfb_filter(vm->synth_filter, &gi);
    mpi_psrfits mpfs[1];
    memset(mpfs, 0, sizeof mpfs);
    mpfs[0].coarse_chan_pf.sub.bytes_per_subint = nsamples * nchans * nstokes;
    mpfs[0].coarse_chan_pf.sub.data = malloc((size_t)nsamples * nchans * nstokes);
    mpfs[0].coarse_chan_pf.sub.dat_offsets = malloc(sizeof(float) * nchans * nstokes);
    mpfs[0].coarse_chan_pf.sub.dat_scales = malloc(sizeof(float) * nchans * nstokes);
    vmCreateStatistics(vm, mpfs);
    vmCreateCudaStreams(vm);
    /* vmCreateGeometricDelays' buffers */
    vm->gdelays.npointings = vm->npointing;
    vm->gdelays.nant = nant;
    vm->gdelays.nchan = nchans;
    const size_t phi_bytes = (size_t)nant * nchans * sizeof(gpuDoubleComplex);
    cudaMallocHost((void **)&vm->gdelays.phi, phi_bytes);
    cudaMalloc((void **)&vm->gdelays.d_phi, phi_bytes);

    const size_t J_bytes = (size_t)nant * nchans * 4 * sizeof(gpuDoubleComplex);
    char *J_all = read_file(in, "J.bin", nsec * J_bytes);
    char *phi_all = read_file(in, "phi.bin", nsec * phi_bytes);
    char *volt = read_file(in, "volt.bin", (1 + 20 * (size_t)nsec) * block_bytes);
    memcpy(vm->v->buffer, volt, block_bytes); /* the first second's margin */

    for (int t = 0; t < nsec; t++) {
        /* vmReadNextSecond: lock, copy the margin, read the second */
        vm->v->locked = true;
        if (t > 0) vmReadBufferCopyMargin(vm->v);
        memcpy(vm->v->read_ptr, volt + (1 + 20 * (size_t)t) * block_bytes, vm->v->read_size);
        /* vmCalcJonesAndDelays */
        memcpy(vm->J, J_all + t * J_bytes, J_bytes);
        memcpy(vm->gdelays.phi, phi_all + t * phi_bytes, phi_bytes);
        vmPushPhi(vm);
        vmPushJ(vm);
        vmBeamformSecond(vm);
        vmPullE(vm);
        prepare_data_buffer_fine(data_buffer_fine, vm, t);
        cu_invert_pfb(data_buffer_fine, t, vm->npointing, nsamples, nchans, npols, 0, &gi, data_buffer_vdif);
        vmPullS(vm);
        vmSendSToFits(vm, mpfs);
        write_file(out, "psrfits", t, mpfs[0].coarse_chan_pf.sub.data, (size_t)nsamples * nchans * nstokes);
        write_file(out, "offsets", t, mpfs[0].coarse_chan_pf.sub.dat_offsets, sizeof(float) * nchans * nstokes);
        write_file(out, "scales", t, mpfs[0].coarse_chan_pf.sub.dat_scales, sizeof(float) * nchans * nstokes);
        write_file(out, "vdif", t, data_buffer_vdif, (size_t)nsamples * nchans * npols * 2 * sizeof(float));
        write_file(out, "S", t, vm->S, vm->S_size_bytes);
        write_file(out, "e", t, vm->e, vm->e_size_bytes);
    }

    free_ipfb(&gi);
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
    vmFreeDHost(vm);
    vmFreeDDevice(vm);
    vmFreePQIdxsHost(vm);
    vmFreePQIdxsDevice(vm);
    vmFreeVHost(vm);
    vmFreeForwardPFB(vm->fpfb);
    cudaFreeHost(vm->gdelays.phi);
    cudaFree(vm->gdelays.d_phi);
    cudaFreeHost(data_buffer_vdif);
    free(data_buffer_fine);
    printf("app_loop: %d seconds done\n", nsec);
    return 0;
}
