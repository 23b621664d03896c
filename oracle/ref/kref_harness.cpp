// kref_harness.cpp — TEST INFRASTRUCTURE: runs the reference's own CUDA
// kernels (compiled from the reference sources into oracle/_ref/*.cubin) in
// the exact order of KaminoSolver::stepForward (KaminoGPU/kernel/
// KaminoSolver.cu:197-221), with cuFFT for the two FFTs as the reference does
// (KaminoCore.cu:763-764, 812-813; plan KaminoSolver.cu:61-66).
//
// Differences from the reference program, all outside its kernels:
//  * buffers are harness-owned with nTheta+2 rows, the rows past the data
//    zeroed: the reference's u_theta sampler reads two rows past its
//    allocation for departure points in (pi, pi+2h) (KaminoCore.cu:103);
//    here those reads see zeros instead of whatever memory follows;
//  * the particle kernel is skipped when there are no particles (the
//    reference launches it with a zero block size and aborts, N6), and the
//    particle count must be <= 1024 or a multiple of 1024 (the kernel has no
//    bounds check, KaminoCore.cu:323);
//  * the __constant__ parameters are written once at create time, like
//    Kamino::run does (KaminoCore.cu:868-872).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {
thread_local char g_err[1024] = "";
int fail(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return 1;
}
#define KD(call)                                                                        \
    do {                                                                                \
        CUresult r_ = (call);                                                           \
        if (r_ != CUDA_SUCCESS) {                                                       \
            const char* s_ = nullptr;                                                   \
            cuGetErrorString(r_, &s_);                                                  \
            return fail("%s: %s (line %d)", #call, s_ ? s_ : "?", __LINE__);            \
        }                                                                               \
    } while (0)
#define KR(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return fail("%s: %s", #call, cudaGetErrorString(e_));    \
    } while (0)
} // namespace

struct kref {
    int nt, np;
    float R, dt, h;
    long long npart;
    size_t pitch;  // elements
    CUmodule core = nullptr, tdm = nullptr, solver = nullptr;
    CUfunction advPhi, advTheta, advCentered, advParticles, geoFill, assignPhi, assignTheta, fillDiv, shiftF,
        copy2U, cacheZero, shiftU, applyTheta, applyPhi, cr, precompute, probeIndex, probeWrap;
    // pitched double buffers [this, next]
    float *velPhi[2], *velTheta[2], *pressure[2], *density[2], *part[2];
    int cu = 0, ct = 0, cp = 0, cd = 0, cpart = 0;
    float2 *UFourier, *FFourier;
    float *UReal, *UImag, *FReal, *FImag, *FZero, *A, *B, *C;
    cufftHandle plan = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
};

extern "C" const char* kref_last_error(void) { return g_err; }

static int load_fn(CUmodule m, CUfunction* f, const char* name)
{
    CUresult r = cuModuleGetFunction(f, m, name);
    if (r != CUDA_SUCCESS) return fail("reference cubin has no kernel %s", name);
    return 0;
}

template <typename T>
static int set_const(CUmodule m, const char* name, T v)
{
    CUdeviceptr p;
    size_t sz;
    CUresult r = cuModuleGetGlobal(&p, &sz, m, name);
    if (r != CUDA_SUCCESS) return fail("reference cubin has no symbol %s", name);
    if (sz != sizeof(T)) return fail("symbol %s has size %zu, expected %zu", name, sz, sizeof(T));
    KD(cuMemcpyHtoD(p, &v, sizeof(T)));
    return 0;
}

// determineLayout (KaminoSolver.cu:165-180) with maxThreadsDim[0] = 1024
static void layout(unsigned rows, unsigned cols, unsigned* grid, unsigned* block)
{
    if (cols <= 1024) {
        *grid = rows;
        *block = cols;
    } else {
        unsigned split = (cols + 1023) / 1024;
        *grid = rows * split;
        *block = 1024;
    }
}

static int launch(kref* k, CUfunction f, unsigned grid, unsigned block, void** args, unsigned smem = 0)
{
    KD(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, (CUstream)k->stream, args, nullptr));
    return 0;
}

extern "C" void kref_destroy(kref* k)
{
    if (!k) return;
    if (k->stream) cudaStreamSynchronize(k->stream);
    if (k->plan) cufftDestroy(k->plan);
    for (void* p : k->allocs) cudaFree(p);
    if (k->core) cuModuleUnload(k->core);
    if (k->tdm) cuModuleUnload(k->tdm);
    if (k->solver) cuModuleUnload(k->solver);
    if (k->stream) cudaStreamDestroy(k->stream);
    delete k;
}

extern "C" int kref_create(const char* cubin_dir, int nt, float radius, float dt, long long npart, kref** out)
{
    *out = nullptr;
    if (nt < 4 || nt > 2048 || (nt & (nt - 1))) return fail("nTheta %d unsupported", nt);
    if (npart < 0 || (npart > 1024 && npart % 1024)) return fail("particle count %lld unsupported", npart);
    KR(cudaSetDevice(0));
    KR(cudaFree(0));  // primary context current for the driver API
    kref* k = new kref();
    k->nt = nt;
    k->np = 2 * nt;
    k->R = radius;
    k->dt = dt;
    k->h = (float)(M_PI / nt);  // Kamino::gridLen (KaminoCore.cu:849)
    k->npart = npart;
    k->pitch = k->np;
    int rc = 0;
    auto cleanup = [&]() {
        kref_destroy(k);
        return 1;
    };
    std::string d(cubin_dir);
    if (cuModuleLoad(&k->core, (d + "/ref_core.cubin").c_str()) != CUDA_SUCCESS ||
        cuModuleLoad(&k->tdm, (d + "/ref_tdm.cubin").c_str()) != CUDA_SUCCESS ||
        cuModuleLoad(&k->solver, (d + "/ref_solver.cubin").c_str()) != CUDA_SUCCESS) {
        fail("cannot load reference cubins from %s", cubin_dir);
        return cleanup();
    }
    struct {
        CUmodule m;
        CUfunction* f;
        const char* n;
    } fns[] = {{k->core, &k->advPhi, "_Z19advectionVPhiKernelPfS_S_m"},
               {k->core, &k->advTheta, "_Z21advectionVThetaKernelPfS_S_m"},
               {k->core, &k->advCentered, "_Z17advectionCenteredPfS_S_S_m"},
               {k->core, &k->advParticles, "_Z18advectionParticlesPfS_S_S_m"},
               {k->core, &k->geoFill, "_Z19geometricFillKernelPfS_S_S_m"},
               {k->core, &k->assignPhi, "_Z15assignPhiKernelPfS_m"},
               {k->core, &k->assignTheta, "_Z17assignThetaKernelPfS_m"},
               {k->core, &k->fillDiv, "_Z20fillDivergenceKernelP6float2PfS1_mm"},
               {k->core, &k->shiftF, "_Z12shiftFKernelP6float2PfS1_"},
               {k->core, &k->copy2U, "_Z13copy2UFourierP6float2PfS1_"},
               {k->core, &k->cacheZero, "_Z19cacheZeroComponentsPfP6float2"},
               {k->core, &k->shiftU, "_Z12shiftUKernelP6float2PfS1_m"},
               {k->core, &k->applyTheta, "_Z18applyPressureThetaPfS_S_mm"},
               {k->core, &k->applyPhi, "_Z16applyPressurePhiPfS_S_mm"},
               {k->core, &k->probeIndex, "kref_probe_index"},
               {k->core, &k->probeWrap, "kref_probe_wrap"},
               {k->tdm, &k->cr, "_Z8crKernelPfS_S_S_S_"},
               {k->solver, &k->precompute, "_Z19precomputeABCKernelPfS_S_"}};
    for (auto& f : fns)
        if (load_fn(f.m, f.f, f.n)) return cleanup();
    // Kamino::run (KaminoCore.cu:868-872) and precomputeABCCoef (KaminoSolver.cu:184-186)
    size_t snp = k->np, snt = k->nt;
    float gl_solver = (float)(6.28318530717958647692 / k->np);  // KaminoSolver gridLen
    if (set_const(k->core, "nPhiGlobal", snp) || set_const(k->core, "nThetaGlobal", snt) ||
        set_const(k->core, "radiusGlobal", radius) || set_const(k->core, "timeStepGlobal", dt) ||
        set_const(k->core, "gridLenGlobal", k->h) || set_const(k->solver, "nPhiGlobal", snp) ||
        set_const(k->solver, "nThetaGlobal", snt) || set_const(k->solver, "gridLenGlobal", gl_solver))
        return cleanup();
    if (cudaStreamCreateWithFlags(&k->stream, cudaStreamNonBlocking) != cudaSuccess) {
        fail("stream");
        return cleanup();
    }
    auto alloc = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, bytes);
        k->allocs.push_back(p);
        return p;
    };
    const size_t field = sizeof(float) * (size_t)(nt + 2) * k->np;
    for (int s = 0; s < 2; s++) {
        k->velPhi[s] = (float*)alloc(field);
        k->velTheta[s] = (float*)alloc(field);
        k->pressure[s] = (float*)alloc(field);
        k->density[s] = (float*)alloc(field);
        k->part[s] = (float*)alloc(sizeof(float) * 2 * (size_t)(npart > 0 ? npart : 1));
    }
    const size_t C = (size_t)nt * k->np;
    k->UFourier = (float2*)alloc(sizeof(float2) * C);
    k->FFourier = (float2*)alloc(sizeof(float2) * C);
    k->UReal = (float*)alloc(4 * C);
    k->UImag = (float*)alloc(4 * C);
    k->FReal = (float*)alloc(4 * C);
    k->FImag = (float*)alloc(4 * C);
    k->FZero = (float*)alloc(4 * (size_t)nt);
    k->A = (float*)alloc(4 * C);
    k->B = (float*)alloc(4 * C);
    k->C = (float*)alloc(4 * C);
    for (void* p : k->allocs)
        if (!p) {
            fail("allocation failed");
            return cleanup();
        }
    int sig[1] = {k->np};
    if (cufftPlanMany(&k->plan, 1, sig, nullptr, 1, k->np, nullptr, 1, k->np, CUFFT_C2C, nt) != CUFFT_SUCCESS ||
        cufftSetStream(k->plan, k->stream) != CUFFT_SUCCESS) {
        fail("cufftPlanMany failed");
        return cleanup();
    }
    unsigned g, b;
    layout(k->np, k->nt, &g, &b);  // precomputeABCCoef, KaminoSolver.cu:190
    void* a[] = {&k->A, &k->B, &k->C};
    rc = launch(k, k->precompute, g, b, a);
    if (rc || cudaStreamSynchronize(k->stream) != cudaSuccess) {
        if (!rc) fail("precomputeABCKernel failed");
        return cleanup();
    }
    *out = k;
    return 0;
}

static float* field_ptr(kref* k, int field, size_t* rows)
{
    switch (field) {
    case 0: *rows = k->nt; return k->velPhi[k->cu];
    case 1: *rows = k->nt - 1; return k->velTheta[k->ct];
    case 2: *rows = k->nt; return k->density[k->cd];
    case 3: *rows = k->nt; return k->pressure[k->cp];
    case 4: *rows = 0; return k->part[k->cpart];
    }
    return nullptr;
}

extern "C" int kref_set_state(kref* k, int field, const float* host)
{
    size_t rows;
    float* d = field_ptr(k, field, &rows);
    if (!d) return fail("bad field %d", field);
    size_t n = field == 4 ? 2 * (size_t)k->npart : rows * k->np;
    if (n) KR(cudaMemcpy(d, host, 4 * n, cudaMemcpyHostToDevice));
    return 0;
}

extern "C" int kref_get_state(kref* k, int field, float* host)
{
    size_t rows;
    float* d = field_ptr(k, field, &rows);
    if (!d) return fail("bad field %d", field);
    size_t n = field == 4 ? 2 * (size_t)k->npart : rows * k->np;
    KR(cudaStreamSynchronize(k->stream));
    if (n) KR(cudaMemcpy(host, d, 4 * n, cudaMemcpyDeviceToHost));
    return 0;
}

// KaminoSolver::advection (KaminoCore.cu:344-384)
extern "C" int kref_advection(kref* k)
{
    unsigned g, b;
    size_t pitch = k->pitch;
    float *un = k->velPhi[1 - k->cu], *u = k->velPhi[k->cu];
    float *vn = k->velTheta[1 - k->ct], *v = k->velTheta[k->ct];
    float *dn = k->density[1 - k->cd], *d = k->density[k->cd];
    layout(k->nt, k->np, &g, &b);
    void* a1[] = {&un, &u, &v, &pitch};
    if (launch(k, k->advPhi, g, b, a1)) return 1;
    layout(k->nt - 1, k->np, &g, &b);
    void* a2[] = {&vn, &u, &v, &pitch};
    if (launch(k, k->advTheta, g, b, a2)) return 1;
    layout(k->nt, k->np, &g, &b);
    void* a3[] = {&dn, &u, &v, &d, &pitch};
    if (launch(k, k->advCentered, g, b, a3)) return 1;
    k->cd ^= 1;
    if (k->npart > 0) {
        float *pn = k->part[1 - k->cpart], *p = k->part[k->cpart];
        layout(1, (unsigned)k->npart, &g, &b);
        void* a4[] = {&pn, &u, &v, &p, &pitch};
        if (launch(k, k->advParticles, g, b, a4)) return 1;
        k->cpart ^= 1;
    }
    k->cu ^= 1;
    k->ct ^= 1;
    return 0;
}

// KaminoSolver::geometric (KaminoCore.cu:551-583)
extern "C" int kref_geometric(kref* k)
{
    unsigned g, b;
    size_t pitch = k->pitch;
    float *pt = k->pressure[k->cp], *pn = k->pressure[1 - k->cp];
    float *u = k->velPhi[k->cu], *v = k->velTheta[k->ct];
    float *un = k->velPhi[1 - k->cu], *vn = k->velTheta[1 - k->ct];
    layout(k->nt, k->np, &g, &b);
    void* a1[] = {&pt, &pn, &u, &v, &pitch};
    if (launch(k, k->geoFill, g, b, a1)) return 1;
    void* a2[] = {&un, &pt, &pitch};
    if (launch(k, k->assignPhi, g, b, a2)) return 1;
    layout(k->nt - 1, k->np, &g, &b);
    void* a3[] = {&vn, &pn, &pitch};
    if (launch(k, k->assignTheta, g, b, a3)) return 1;
    k->cu ^= 1;
    k->ct ^= 1;
    return 0;
}

// KaminoSolver::projection (KaminoCore.cu:749-842)
extern "C" int kref_projection(kref* k)
{
    unsigned g, b;
    size_t pitch = k->pitch;
    float *u = k->velPhi[k->cu], *v = k->velTheta[k->ct];
    float *un = k->velPhi[1 - k->cu], *vn = k->velTheta[1 - k->ct];
    float* p = k->pressure[k->cp];
    layout(k->nt, k->np, &g, &b);
    void* a1[] = {&k->FFourier, &u, &v, &pitch, &pitch};
    if (launch(k, k->fillDiv, g, b, a1)) return 1;
    if (cufftExecC2C(k->plan, k->FFourier, k->FFourier, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return fail("cufftExecC2C inverse");
    void* a2[] = {&k->FFourier, &k->FReal, &k->FImag};
    if (launch(k, k->shiftF, g, b, a2)) return 1;
    unsigned smem = (unsigned)(k->nt * 5 * sizeof(float));
    void* a3[] = {&k->A, &k->B, &k->C, &k->FReal, &k->UReal};
    if (launch(k, k->cr, k->np, k->nt / 2, a3, smem)) return 1;
    void* a4[] = {&k->A, &k->B, &k->C, &k->FImag, &k->UImag};
    if (launch(k, k->cr, k->np, k->nt / 2, a4, smem)) return 1;
    void* a5[] = {&k->UFourier, &k->UReal, &k->UImag};
    if (launch(k, k->copy2U, g, b, a5)) return 1;
    unsigned g1, b1;
    layout(1, k->nt, &g1, &b1);
    void* a6[] = {&k->FZero, &k->UFourier};
    if (launch(k, k->cacheZero, g1, b1, a6)) return 1;
    if (cufftExecC2C(k->plan, k->UFourier, k->UFourier, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return fail("cufftExecC2C forward");
    void* a7[] = {&k->UFourier, &p, &k->FZero, &pitch};
    if (launch(k, k->shiftU, g, b, a7)) return 1;
    layout(k->nt - 1, k->np, &g, &b);
    void* a8[] = {&vn, &v, &p, &pitch, &pitch};
    if (launch(k, k->applyTheta, g, b, a8)) return 1;
    layout(k->nt, k->np, &g, &b);
    void* a9[] = {&un, &u, &p, &pitch, &pitch};
    if (launch(k, k->applyPhi, g, b, a9)) return 1;
    k->cu ^= 1;
    k->ct ^= 1;
    return 0;
}

extern "C" int kref_step(kref* k, int n)
{
    for (int s = 0; s < n; s++)
        if (kref_advection(k) || kref_geometric(k) || kref_projection(k)) return 1;
    return 0;
}

extern "C" int kref_synchronize(kref* k)
{
    KR(cudaStreamSynchronize(k->stream));
    return 0;
}

// Device time of n steps, CUDA events on the harness stream.  *stage_ms gets
// the advection / geometric / projection split (summed over the n steps).
extern "C" int kref_time_steps(kref* k, int n, double* ms_total, double* stage_ms)
{
    cudaEvent_t e[4];
    for (auto& x : e) KR(cudaEventCreate(&x));
    double tot = 0, st[3] = {0, 0, 0};
    int rc = 0;
    for (int s = 0; s < n && !rc; s++) {
        cudaEventRecord(e[0], k->stream);
        rc |= kref_advection(k);
        cudaEventRecord(e[1], k->stream);
        rc |= kref_geometric(k);
        cudaEventRecord(e[2], k->stream);
        rc |= kref_projection(k);
        cudaEventRecord(e[3], k->stream);
        // the reference synchronises after almost every kernel; one sync per
        // step here is strictly kinder to it
        cudaStreamSynchronize(k->stream);
        float a, b, c;
        cudaEventElapsedTime(&a, e[0], e[1]);
        cudaEventElapsedTime(&b, e[1], e[2]);
        cudaEventElapsedTime(&c, e[2], e[3]);
        st[0] += a;
        st[1] += b;
        st[2] += c;
        tot += a + b + c;
    }
    for (auto& x : e) cudaEventDestroy(x);
    if (rc) return rc;
    *ms_total = tot;
    if (stage_ms)
        for (int i = 0; i < 3; i++) stage_ms[i] = st[i];
    return 0;
}

extern "C" int kref_probe_index(kref* k, int kind, const float* phi, const float* theta, long long n, int* out,
                                float* alpha)
{
    if (n <= 0) return 0;
    float *dp, *dt, *da;
    int* di;
    KR(cudaMalloc(&dp, 4 * n));
    KR(cudaMalloc(&dt, 4 * n));
    KR(cudaMalloc(&da, 8 * n));
    KR(cudaMalloc(&di, 16 * n));
    KR(cudaMemcpy(dp, phi, 4 * n, cudaMemcpyHostToDevice));
    KR(cudaMemcpy(dt, theta, 4 * n, cudaMemcpyHostToDevice));
    void* a[] = {&kind, &dp, &dt, &n, &di, &da};
    int rc = launch(k, k->probeIndex, (unsigned)((n + 255) / 256), 256, a);
    if (!rc) {
        KR(cudaStreamSynchronize(k->stream));
        KR(cudaMemcpy(out, di, 16 * n, cudaMemcpyDeviceToHost));
        KR(cudaMemcpy(alpha, da, 8 * n, cudaMemcpyDeviceToHost));
    }
    cudaFree(dp);
    cudaFree(dt);
    cudaFree(da);
    cudaFree(di);
    return rc;
}

extern "C" int kref_probe_wrap(kref* k, float* phi, float* theta, long long n, int* cells)
{
    if (n <= 0) return 0;
    float *dp, *dt;
    int* dc;
    KR(cudaMalloc(&dp, 4 * n));
    KR(cudaMalloc(&dt, 4 * n));
    KR(cudaMalloc(&dc, 8 * n));
    KR(cudaMemcpy(dp, phi, 4 * n, cudaMemcpyHostToDevice));
    KR(cudaMemcpy(dt, theta, 4 * n, cudaMemcpyHostToDevice));
    void* a[] = {&dp, &dt, &n, &dc};
    int rc = launch(k, k->probeWrap, (unsigned)((n + 255) / 256), 256, a);
    if (!rc) {
        KR(cudaStreamSynchronize(k->stream));
        KR(cudaMemcpy(phi, dp, 4 * n, cudaMemcpyDeviceToHost));
        KR(cudaMemcpy(theta, dt, 4 * n, cudaMemcpyDeviceToHost));
        KR(cudaMemcpy(cells, dc, 8 * n, cudaMemcpyDeviceToHost));
    }
    cudaFree(dp);
    cudaFree(dt);
    cudaFree(dc);
    return rc;
}
