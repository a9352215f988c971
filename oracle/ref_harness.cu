/*
 * ref_harness.cu -- runs the reference's OWN CUDA kernels on a GPU.
 *
 * TEST INFRASTRUCTURE. oracle/build_ref.sh compiles the unmodified
 * src/pfb.cpp and src/form_beam.cpp device code into oracle/_ref/*.cubin;
 * this file (built on the GPU machine by __graft_entry__.build()) loads those
 * cubins through the CUDA driver API and drives them with the launch shapes,
 * memsets and cuFFT calls of the reference's host code, cited per function.
 * It produces the golden vectors the oracle is pinned against
 * (tests/golden/make_golden.py) and times the reference CUDA build.
 *
 * Every entry point returns 0 on success or a nonzero error code; the last
 * error text is available from refh_last_error().
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;
CUmodule g_mod_pfb = nullptr, g_mod_beam = nullptr;
CUfunction g_wola, g_round, g_i2f, g_pack, g_ipfb;
CUfunction g_incoh, g_applyj, g_beamform, g_renorm;

int fail(const std::string &what)
{
    g_err = what;
    return 1;
}

#define RT(x)                                                                  \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess)                                                 \
            return fail(std::string(#x) + ": " + cudaGetErrorString(e_));     \
    } while (0)
#define DRV(x)                                                                 \
    do {                                                                       \
        CUresult e_ = (x);                                                     \
        if (e_ != CUDA_SUCCESS) {                                              \
            const char *s_ = nullptr;                                          \
            cuGetErrorString(e_, &s_);                                         \
            return fail(std::string(#x) + ": " + (s_ ? s_ : "?"));            \
        }                                                                      \
    } while (0)

/* Find a kernel whose (mangled) name contains `key` (length-prefixed, so
 * "13vmWOLA_kernel" cannot match anything else). */
int find_fn(CUmodule mod, const char *key, CUfunction *out)
{
    unsigned n = 0;
    DRV(cuModuleGetFunctionCount(&n, mod));
    std::vector<CUfunction> fs(n);
    DRV(cuModuleEnumerateFunctions(fs.data(), n, mod));
    for (unsigned i = 0; i < n; i++) {
        const char *nm = nullptr;
        DRV(cuFuncGetName(&nm, fs[i]));
        if (nm && strstr(nm, key)) {
            *out = fs[i];
            return 0;
        }
    }
    return fail(std::string("kernel not found: ") + key);
}

int launch(CUfunction f, dim3 g, dim3 b, unsigned smem, void **args)
{
    DRV(cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, smem, 0, args, nullptr));
    return 0;
}

template <class T> struct DevBuf {
    T *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    int alloc(size_t n)
    {
        RT(cudaMalloc((void **)&p, n * sizeof(T) + 16));
        return 0;
    }
};

} // namespace

extern "C" const char *refh_last_error(void) { return g_err.c_str(); }

extern "C" int refh_init(const char *dir)
{
    if (g_mod_pfb) return 0;
    RT(cudaFree(0));
    std::string d(dir);
    DRV(cuModuleLoad(&g_mod_pfb, (d + "/ref_pfb.cubin").c_str()));
    DRV(cuModuleLoad(&g_mod_beam, (d + "/ref_form_beam.cubin").c_str()));
    int r = 0;
    r |= find_fn(g_mod_pfb, "13vmWOLA_kernel", &g_wola);
    r |= find_fn(g_mod_pfb, "26fpga_rounding_and_demotion", &g_round);
    r |= find_fn(g_mod_pfb, "9int2float", &g_i2f);
    r |= find_fn(g_mod_pfb, "27pack_into_recombined_format", &g_pack);
    r |= find_fn(g_mod_pfb, "11ipfb_kernel", &g_ipfb);
    r |= find_fn(g_mod_beam, "10incoh_beam", &g_incoh);
    r |= find_fn(g_mod_beam, "15vmApplyJ_kernel", &g_applyj);
    r |= find_fn(g_mod_beam, "17vmBeamform_kernel", &g_beamform);
    r |= find_fn(g_mod_beam, "27renormalise_channels_kernel", &g_renorm);
    return r;
}

/*
 * Forward PFB of one chunk, as vmExecuteForwardPFB (pfb.cpp:730-773) drives
 * it: memset of the WOLA buffer (pfb.cpp:580), vmWOLA_kernel
 * <<<(nspectra, I, P), K>>> (pfb.cpp:574-582), rounding or int2float
 * (pfb.cpp:602-616), cufftPlanMany + I/32 cufftExecC2C calls
 * (pfb.cpp:478-488, 637-644), pack <<<(nspectra, K), I>>> (pfb.cpp:662-668).
 * htr: MWAX bytes [nblocks][I][64000][2] on the host; out: host, int4 bytes
 * or complex doubles [nspectra][K][I]; wola_out (nullable): int32 b after
 * the WOLA kernel. Requires I % 32 == 0 (the reference's cuFFT batching).
 */
extern "C" int refh_fpfb(const void *htr, size_t htr_bytes, int I, int nspectra,
                         const int *filter, int K, int P, const int *i_idx,
                         int flags, int32_t *wola_out, void *out,
                         float *elapsed_ms)
{
    if (I % 32 != 0) return fail("refh_fpfb: I must be a multiple of 32");
    const bool int4 = (flags & 0x10) != 0;
    const size_t nb = (size_t)nspectra * I * K; // complex elements
    DevBuf<char> d_htr;
    DevBuf<int> d_filt, d_idx;
    DevBuf<float> d_wola;
    DevBuf<char> d_out;
    if (d_htr.alloc(htr_bytes) || d_filt.alloc((size_t)K * P) || d_idx.alloc(I) ||
        d_wola.alloc(2 * nb) || d_out.alloc(nb * (int4 ? 1 : 16)))
        return 1;
    RT(cudaMemcpy(d_htr.p, htr, htr_bytes, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_filt.p, filter, sizeof(int) * K * P, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_idx.p, i_idx, sizeof(int) * I, cudaMemcpyHostToDevice));

    cufftHandle plan;
    int n = K;
    int batch32 = nspectra * 32;
    if (cufftPlanMany(&plan, 1, &n, NULL, 0, 0, NULL, 0, 0, CUFFT_C2C, batch32) != CUFFT_SUCCESS)
        return fail("cufftPlanMany failed");

    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0));
    RT(cudaMemset(d_wola.p, 0, sizeof(float) * 2 * nb));
    {
        void *a0 = d_htr.p, *a1 = d_filt.p, *a2 = d_wola.p;
        void *args[] = {&a0, &a1, &a2};
        if (launch(g_wola, dim3(nspectra, I, P), dim3(K), 0, args)) return 1;
    }
    if (wola_out) {
        RT(cudaDeviceSynchronize());
        RT(cudaMemcpy(wola_out, d_wola.p, sizeof(int32_t) * 2 * nb, cudaMemcpyDeviceToHost));
    }
    if (flags & 0x200) {
        void *a0 = d_wola.p;
        void *args[] = {&a0};
        if (launch(g_round, dim3(nspectra, I), dim3(K), 0, args)) return 1;
    } else {
        if ((2 * nb) % 1024 != 0) return fail("int2float grid must divide by 1024");
        void *a0 = d_wola.p;
        double scale = 1.0 / 16384.0;
        void *args[] = {&a0, &scale};
        if (launch(g_i2f, dim3((unsigned)(2 * nb / 1024)), dim3(1024), 0, args)) return 1;
    }
    for (int b = 0; b < I / 32; b++) {
        cufftComplex *p = (cufftComplex *)d_wola.p + (size_t)b * batch32 * K;
        if (cufftExecC2C(plan, p, p, CUFFT_FORWARD) != CUFFT_SUCCESS)
            return fail("cufftExecC2C failed");
    }
    {
        void *a0 = d_wola.p, *a1 = d_out.p, *a2 = d_idx.p;
        int fl = flags;
        void *args[] = {&a0, &a1, &a2, &fl};
        if (launch(g_pack, dim3(nspectra, K), dim3(I), 0, args)) return 1;
    }
    RT(cudaEventRecord(e1));
    RT(cudaEventSynchronize(e1));
    if (elapsed_ms) RT(cudaEventElapsedTime(elapsed_ms, e0, e1));
    RT(cudaMemcpy(out, d_out.p, nb * (int4 ? 1 : 16), cudaMemcpyDeviceToHost));
    cufftDestroy(plan);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

/*
 * vmApplyJChunk + vmBeamformChunk for one chunk (form_beam.cpp:510-582):
 * per pointing, vmApplyJ_kernel <<<(nchan, ns), nant>>> then
 * vmBeamform_kernel <<<(nchan, ns), nant, 11*nant*8>>>.
 * v: host int4 bytes (datatype 0) or complex doubles (1), [ns][nchan][2*nant].
 * J: [npointing][nant][nchan][2][2] complex; phi: [npointing][nant][nchan].
 * S: [npointing][ns][nstokes][nchan] float; e: [npointing][ns][nchan][2].
 */
extern "C" int refh_beamform(const void *v, int datatype, int ns, int nchan, int nant,
                             const double *J, const double *phi,
                             const uint32_t *polQ, const uint32_t *polP,
                             int npointing, double invw, int nstokes,
                             float *S, double *e, float *elapsed_ms)
{
    const size_t nv = (size_t)ns * nchan * 2 * nant;
    const size_t vbytes = nv * (datatype == 0 ? 1 : 16);
    const size_t njv = (size_t)npointing * ns * nchan * nant;
    DevBuf<char> d_v;
    DevBuf<double> d_J, d_phi, d_JvQ, d_JvP, d_e;
    DevBuf<uint32_t> d_Q, d_P;
    DevBuf<float> d_S;
    if (d_v.alloc(vbytes) || d_J.alloc((size_t)npointing * nant * nchan * 8) ||
        d_phi.alloc((size_t)npointing * nant * nchan * 2) || d_JvQ.alloc(2 * njv) ||
        d_JvP.alloc(2 * njv) || d_e.alloc((size_t)npointing * ns * nchan * 4) ||
        d_Q.alloc(nant) || d_P.alloc(nant) || d_S.alloc((size_t)npointing * ns * nstokes * nchan))
        return 1;
    RT(cudaMemcpy(d_v.p, v, vbytes, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_J.p, J, sizeof(double) * npointing * nant * nchan * 8, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_phi.p, phi, sizeof(double) * npointing * nant * nchan * 2, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_Q.p, polQ, sizeof(uint32_t) * nant, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_P.p, polP, sizeof(uint32_t) * nant, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0));
    for (int p = 0; p < npointing; p++) {
        void *a0 = d_v.p, *a1 = d_J.p, *a2 = d_JvQ.p, *a3 = d_JvP.p, *a4 = d_Q.p, *a5 = d_P.p;
        int npol = 2, pp = p, dt = datatype;
        void *args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &npol, &pp, &dt};
        if (launch(g_applyj, dim3(nchan, ns), dim3(nant), 0, args)) return 1;
    }
    for (int p = 0; p < npointing; p++) {
        void *a0 = d_JvQ.p, *a1 = d_JvP.p, *a2 = d_phi.p, *a7 = d_e.p, *a8 = d_S.p;
        double w = invw;
        int pp = p, soff = 0, nchunk = 1, npol = 2, nst = nstokes;
        void *args[] = {&a0, &a1, &a2, &w, &pp, &soff, &nchunk, &a7, &a8, &npol, &nst};
        if (launch(g_beamform, dim3(nchan, ns), dim3(nant), 11 * nant * sizeof(double), args))
            return 1;
    }
    RT(cudaEventRecord(e1));
    RT(cudaEventSynchronize(e1));
    if (elapsed_ms) RT(cudaEventElapsedTime(elapsed_ms, e0, e1));
    RT(cudaMemcpy(S, d_S.p, sizeof(float) * npointing * ns * nstokes * nchan, cudaMemcpyDeviceToHost));
    if (e) RT(cudaMemcpy(e, d_e.p, sizeof(double) * npointing * ns * nchan * 4, cudaMemcpyDeviceToHost));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

/* vmSendSToFits's kernel (form_beam.cpp:653-663):
 * renormalise_channels_kernel <<<npointing, (nchan, nstokes)>>>. */
extern "C" int refh_renormalise(const float *S, int npointing, int nstep, int nstokes,
                                int nchan, float *offsets, float *scales, uint8_t *out)
{
    const size_t n = (size_t)npointing * nstep * nstokes * nchan;
    DevBuf<float> d_S, d_off, d_sc;
    DevBuf<uint8_t> d_out;
    if (d_S.alloc(n) || d_off.alloc((size_t)npointing * nstokes * nchan) ||
        d_sc.alloc((size_t)npointing * nstokes * nchan) || d_out.alloc(n))
        return 1;
    RT(cudaMemcpy(d_S.p, S, sizeof(float) * n, cudaMemcpyHostToDevice));
    void *a0 = d_S.p, *a2 = d_off.p, *a3 = d_sc.p, *a4 = d_out.p;
    int ns = nstep;
    void *args[] = {&a0, &ns, &a2, &a3, &a4};
    if (launch(g_renorm, dim3(npointing), dim3(nchan, nstokes), 0, args)) return 1;
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(offsets, d_off.p, sizeof(float) * npointing * nstokes * nchan, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(scales, d_sc.p, sizeof(float) * npointing * nstokes * nchan, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(out, d_out.p, n, cudaMemcpyDeviceToHost));
    return 0;
}

/* refh_renormalise with the kernel's device time (CUDA events around the
 * launch) in *elapsed_ms. */
extern "C" int refh_renormalise_timed(const float *S, int npointing, int nstep, int nstokes, int nchan,
                                      float *offsets, float *scales, uint8_t *out, float *elapsed_ms)
{
    const size_t n = (size_t)npointing * nstep * nstokes * nchan;
    DevBuf<float> d_S, d_off, d_sc;
    DevBuf<uint8_t> d_out;
    if (d_S.alloc(n) || d_off.alloc((size_t)npointing * nstokes * nchan) ||
        d_sc.alloc((size_t)npointing * nstokes * nchan) || d_out.alloc(n))
        return 1;
    RT(cudaMemcpy(d_S.p, S, sizeof(float) * n, cudaMemcpyHostToDevice));
    void *a0 = d_S.p, *a2 = d_off.p, *a3 = d_sc.p, *a4 = d_out.p;
    int ns = nstep;
    void *args[] = {&a0, &ns, &a2, &a3, &a4};
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0));
    if (launch(g_renorm, dim3(npointing), dim3(nchan, nstokes), 0, args)) return 1;
    RT(cudaEventRecord(e1));
    RT(cudaEventSynchronize(e1));
    if (elapsed_ms) RT(cudaEventElapsedTime(elapsed_ms, e0, e1));
    RT(cudaMemcpy(offsets, d_off.p, sizeof(float) * npointing * nstokes * nchan, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(scales, d_sc.p, sizeof(float) * npointing * nstokes * nchan, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(out, d_out.p, n, cudaMemcpyDeviceToHost));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

/* cu_form_incoh_beam's first kernel (form_beam.cpp:487-490):
 * incoh_beam <<<(nchan, nsample), ninput>>>. */
extern "C" int refh_incoh(const uint8_t *data, int nsample, int nchan, int ninput, float *incoh)
{
    const size_t n = (size_t)nsample * nchan * ninput;
    DevBuf<uint8_t> d_data;
    DevBuf<float> d_inc;
    if (d_data.alloc(n) || d_inc.alloc((size_t)nsample * nchan)) return 1;
    RT(cudaMemcpy(d_data.p, data, n, cudaMemcpyHostToDevice));
    void *a0 = d_data.p, *a1 = d_inc.p;
    void *args[] = {&a0, &a1};
    if (launch(g_incoh, dim3(nchan, nsample), dim3(ninput), 0, args)) return 1;
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(incoh, d_inc.p, sizeof(float) * nsample * nchan, cudaMemcpyDeviceToHost));
    return 0;
}

/*
 * cu_invert_pfb's kernel (pfb.cpp:996-998): ipfb_kernel
 * <<<nsamples, nchan*npol>>>. in_real/in_imag: [(nsamples+ntaps)][nchan][npol]
 * as cu_invert_pfb packs them (pfb.cpp:953-984); ft_real/ft_imag:
 * [nchan][ntaps*nchan] as cu_load_ipfb_filter builds them (pfb.cpp:1032-1041).
 *
 * The reference kernel reads up to 127 floats BEFORE ft_real/ft_imag for the
 * first 1536 output samples (its tap range truncates toward zero,
 * pfb.cpp:863). So that every read stays inside memory this harness owns, the
 * tables are placed 1024 floats into their allocations, after zeros.
 */
extern "C" int refh_ipfb(const float *in_real, const float *in_imag, const float *ft_real,
                         const float *ft_imag, int ntaps, int nsamples, int nchan, int npol,
                         float *out, float *elapsed_ms)
{
    const size_t nin = (size_t)(nsamples + ntaps) * nchan * npol;
    const size_t nft = (size_t)ntaps * nchan * nchan;
    const size_t nout = (size_t)nsamples * nchan * npol * 2;
    const size_t guard = 1024;
    DevBuf<float> d_ir, d_ii, d_fr, d_fi, d_out;
    if (d_ir.alloc(nin) || d_ii.alloc(nin) || d_fr.alloc(nft + guard) ||
        d_fi.alloc(nft + guard) || d_out.alloc(nout))
        return 1;
    RT(cudaMemset(d_fr.p, 0, sizeof(float) * (nft + guard)));
    RT(cudaMemset(d_fi.p, 0, sizeof(float) * (nft + guard)));
    RT(cudaMemcpy(d_ir.p, in_real, sizeof(float) * nin, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_ii.p, in_imag, sizeof(float) * nin, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_fr.p + guard, ft_real, sizeof(float) * nft, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d_fi.p + guard, ft_imag, sizeof(float) * nft, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    void *a0 = d_ir.p, *a1 = d_ii.p, *a6 = d_out.p;
    void *a2 = d_fr.p + guard, *a3 = d_fi.p + guard;
    int nt = ntaps, np = npol;
    void *args[] = {&a0, &a1, &a2, &a3, &nt, &np, &a6};
    RT(cudaEventRecord(e0));
    if (launch(g_ipfb, dim3(nsamples), dim3(nchan * npol), 0, args)) return 1;
    RT(cudaEventRecord(e1));
    RT(cudaEventSynchronize(e1));
    if (elapsed_ms) RT(cudaEventElapsedTime(elapsed_ms, e0, e1));
    RT(cudaMemcpy(out, d_out.p, sizeof(float) * nout, cudaMemcpyDeviceToHost));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}
