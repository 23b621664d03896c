// kamino_noalloc.cu — a pressure projection that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool, code that must not change the process's device
// allocation footprint after start-up, or code whose only device memory is
// the buffers its host hands it.  kamino_projection_noalloc() serves them: the
// caller passes device pointers for the input and output fields, and every
// temporary of the projection (spectrum, per-mode solutions, tables) lives in
// one fixed array compiled into this library.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds its KAMINO_NOALLOC_SCRATCH_BYTES until the process exits.  In
// host code its name is only a host-side stand-in; the device address is
// looked up with cudaGetSymbolAddress once per device (on that device's first
// call, with the device current) and passed to the kernels.  All calls share
// the array and it keeps whatever the last call left: calls whose work
// overlaps on the GPU (different streams, or a second call before the first
// has finished) race on it.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "kamino_common.h"
#include "kamino_kernels.cuh"

namespace {

constexpr int NOALLOC_MAX_NT = 256;
constexpr int NOALLOC_FP64_MODES = 4;
constexpr size_t NOALLOC_BYTES = (size_t)1280 << 10;  // 1.25 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

struct DeviceSlot {
    void* base = nullptr;  // device address of g_noalloc_scratch on this device
    int nt_loaded = 0;     // n_theta whose tables the array currently holds
};
constexpr int MAX_DEVICES = 64;
DeviceSlot g_slots[MAX_DEVICES];
std::mutex g_mu;

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

// Carve the array for n_theta = nt; returns the bytes used.
size_t carve(char* base, int nt, KBufs* b)
{
    char* p = base;
    auto take = [&p](size_t n) {
        char* r = p;
        p += up256(n);
        return r;
    };
    b->spec = (float2*)take(sizeof(float2) * (size_t)nt * nt);
    b->sol = (float2*)take(sizeof(float2) * (size_t)nt * nt);
    b->s64 = (double*)take(sizeof(double) * kk::s64_stride(nt) * NOALLOC_FP64_MODES);
    float** rowf[] = {&b->cof_c, &b->cof_v, &b->cell_c, &b->cell_v, &b->gfac, &b->negHs, &b->divf,
                      &b->sinN,  &b->sinS,  &b->lapA,   &b->lapC,   &b->lapB0, &b->lapS};
    for (float** f : rowf) *f = (float*)take(sizeof(float) * nt);
    b->lapA64 = (double*)take(sizeof(double) * nt);
    b->lapC64 = (double*)take(sizeof(double) * nt);
    b->lapB064 = (double*)take(sizeof(double) * nt);
    b->lapS64 = (double*)take(sizeof(double) * nt);
    b->tw = (float2*)take(sizeof(float2) * nt);
    b->rt = (float2*)take(sizeof(float2) * (nt + 1));
    return (size_t)(p - base);
}

KGeo make_geo(int nt)
{
    KGeo g = {};
    g.nt = nt;
    g.np = 2 * nt;
    g.mask = g.np - 1;
    g.half = nt;
    while ((1 << g.log2nt) < nt) g.log2nt++;
    g.h = (float)(KAMINO_PI_D / nt);
    g.halfh = 0.5f * g.h;
    g.invh = (float)(1.0 / (double)g.h);
    g.R = 1.0f;   // the projection uses neither radius nor dt
    g.dt = 1.0f;
    g.cofTheta = 1.0f;
    g.pitch = g.np;
    g.rows = nt;
    return g;
}

// Fill the tables for nt into the array (ordered on `stream`).  Host
// vectors only; the copies come from pageable memory, so they are staged
// before cudaMemcpyAsync returns.
int load_tables(int nt, const KGeo& g, const KBufs& b, cudaStream_t stream)
{
    std::vector<double> A, C, B0, S, t64;
    laplacian_rows(nt, A, C, B0, S);
    fp64_tables(nt, NOALLOC_FP64_MODES, A, C, S, t64);
    std::vector<float> Af(A.begin(), A.end()), Cf(C.begin(), C.end()), B0f(B0.begin(), B0.end()),
        Sf(S.begin(), S.end());
    std::vector<float2> tw(nt), rt(nt + 1);
    for (int k = 0; k < nt; k++) {
        double a = -2.0 * KAMINO_PI_D * k / nt;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    for (int m = 0; m <= nt; m++) {
        double a = -KAMINO_PI_D * m / nt;
        rt[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    struct {
        void* d;
        const void* s;
        size_t n;
    } ups[] = {{b.lapA, Af.data(), 4 * (size_t)nt},    {b.lapC, Cf.data(), 4 * (size_t)nt},
               {b.lapB0, B0f.data(), 4 * (size_t)nt},  {b.lapS, Sf.data(), 4 * (size_t)nt},
               {b.lapA64, A.data(), 8 * (size_t)nt},   {b.lapC64, C.data(), 8 * (size_t)nt},
               {b.lapB064, B0.data(), 8 * (size_t)nt}, {b.lapS64, S.data(), 8 * (size_t)nt},
               {b.tw, tw.data(), 8 * (size_t)nt},      {b.rt, rt.data(), 8 * (size_t)(nt + 1)},
               {b.s64, t64.data(), 8 * t64.size()}};
    for (auto& u : ups) {
        cudaError_t e = cudaMemcpyAsync(u.d, u.s, u.n, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess)
            return kamino_fail(KAMINO_ERR_CUDA, "kamino_projection_noalloc: table upload: %s", cudaGetErrorString(e));
    }
    kk::k_tables<<<(nt + 127) / 128, 128, 0, stream>>>(g, b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return kamino_fail(KAMINO_ERR_CUDA, "kamino_projection_noalloc: tables: %s", cudaGetErrorString(e));
    return KAMINO_OK;
}

} // namespace

extern "C" int kamino_projection_noalloc(int n_theta, const float* u_phi, const float* u_theta, float* u_phi_out,
                                         float* u_theta_out, float* pressure_out, void* stream_ptr)
{
    const int nt = n_theta;
    if (nt < 32 || nt > NOALLOC_MAX_NT || (nt & (nt - 1)))
        return kamino_fail(KAMINO_ERR_INVALID,
                           "kamino_projection_noalloc: n_theta=%d; it must be a power of two in [32, %d] (the "
                           "fixed scratch array holds %zu bytes)",
                           nt, NOALLOC_MAX_NT, NOALLOC_BYTES);
    if (!u_phi || !u_theta || !u_phi_out || !u_theta_out || !pressure_out)
        return kamino_fail(KAMINO_ERR_INVALID, "kamino_projection_noalloc: null field pointer");
    for (const void* ptr : {(const void*)u_phi, (const void*)u_theta, (const void*)u_phi_out,
                            (const void*)u_theta_out, (const void*)pressure_out})
        if (reinterpret_cast<uintptr_t>(ptr) % 16 != 0)
            return kamino_fail(KAMINO_ERR_INVALID, "kamino_projection_noalloc: field pointers must be 16-byte aligned");
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return kamino_fail(KAMINO_ERR_CUDA, "kamino_projection_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return kamino_fail(KAMINO_ERR_INVALID, "device %d out of range", dev);
    const KGeo g = make_geo(nt);
    KBufs b = {};
    {
        std::lock_guard<std::mutex> lock(g_mu);
        DeviceSlot& slot = g_slots[dev];
        if (!slot.base) {  // once per device, with that device current
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return kamino_fail(KAMINO_ERR_CUDA, "kamino_projection_noalloc: cudaGetSymbolAddress: %s",
                                   cudaGetErrorString(e));
            slot.base = ptr;
        }
        if (carve((char*)slot.base, nt, &b) > NOALLOC_BYTES)
            return kamino_fail(KAMINO_ERR_INVALID, "kamino_projection_noalloc: scratch too small for n_theta=%d", nt);
        if (slot.nt_loaded != nt) {
            // A table upload copies from host vectors that are freed when
            // this call returns, so it must run now, not be recorded.
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            e = cudaStreamIsCapturing(stream, &cs);
            if (e != cudaSuccess)
                return kamino_fail(KAMINO_ERR_CUDA, "kamino_projection_noalloc: cudaStreamIsCapturing: %s",
                                   cudaGetErrorString(e));
            if (cs != cudaStreamCaptureStatusNone)
                return kamino_fail(KAMINO_ERR_INVALID,
                                   "kamino_projection_noalloc: the tables of n_theta=%d are not loaded and cannot "
                                   "be loaded while the stream is capturing; call once with this n_theta outside "
                                   "the capture first",
                                   nt);
            // the array holds no complete set of tables until the upload has
            // been queued in full: a failure part-way leaves nothing to reuse
            slot.nt_loaded = 0;
            int rc = load_tables(nt, g, b, stream);
            if (rc) return rc;
            slot.nt_loaded = nt;
        }
    }
    b.u[0] = const_cast<float*>(u_phi);
    b.v[0] = const_cast<float*>(u_theta);
    b.u[1] = u_phi_out;
    b.v[1] = u_theta_out;
    b.p = pressure_out;
    const int rpc = kk::fft_rows_per_cta(nt);
    const int fft_threads = kk::fft_threads(nt);
    const size_t fft_smem = kk::fft_smem(nt);
    const size_t solve_smem = kk::solve_smem(nt);
    // same launches as kamino_projection (the divergence from face
    // velocities, the mode solves, the inverse FFT and both gradients)
    kk::div_fft_kernel<2>(nt)<<<nt / rpc, fft_threads, fft_smem, stream>>>(g, b, 0, 1);
    kk::solve_kernel(nt)<<<kk::solve_tiles(nt, NOALLOC_FP64_MODES), kk::SOLVE_THREADS, solve_smem, stream>>>(
        g, b, NOALLOC_FP64_MODES);
    kk::ifft_kernel(nt)<<<nt / rpc, fft_threads, fft_smem, stream>>>(g, b, 0, 1);
    const int nv = kk::elem_groups((nt - 1) * g.np);
    kk::k_vgrad<<<(nv + 2 * kk::ELEM_THREADS - 1) / (2 * kk::ELEM_THREADS), kk::ELEM_THREADS, 0, stream>>>(g, b, 0, 1);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return kamino_fail(KAMINO_ERR_CUDA, "kamino_projection_noalloc: launch: %s", cudaGetErrorString(e));
    return KAMINO_OK;
}
