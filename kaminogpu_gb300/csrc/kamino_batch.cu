// kamino_batch.cu — many spheres per launch, and a continuous-batching server.
//
// Batched form.  Spheres of uneven nTheta (each a kamino_handle with its own
// arena) advance together: every stage of the step is ONE persistent launch
// whose CTAs drain a work queue of (sphere, tile) items — a tile is a block
// of grid points (advection, elementwise stages), a group of latitude rows
// (FFT stages) or one Fourier mode (solve).  Items are ordered largest
// sphere first, so the tail of a stage is made of small items.  The device
// code of a tile is the same function the one-sphere kernels run, so a sphere
// gives bit-identical fields alone and in a batch.  A step is one CUDA graph
// (counter reset + six persistent launches) per buffer parity.  The
// autotuner times candidate launch shapes (CTAs per SM for the three kernel
// families, advection tiles per work item) on the live batch.
//
// Served form.  Requests (one sphere each) are queued on submit, admitted
// while their device state fits the HBM budget (and the slot limit), advanced
// in rounds together with everything already resident, and retired when
// their steps are done; retired device memory returns to a per-size pool so
// later requests of that size do not call cudaMalloc.  Latency is measured
// from the request's arrival to the end of the round that finished it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

#include "kamino_common.h"
#include "kamino_kernels.cuh"

namespace {

// Per-sphere descriptor for the persistent kernels.
struct KSphere {
    KGeo g;
    KBufs b;
    int nb_u, nb_v, nb_r, nb_adv;  // advection tiles (u_phi, u_theta, thickness, all incl. particles)
    int nb_elem;                   // tiles of ELEM_THREADS four-cell groups of nt * nPhi
    int nb_fft;                    // row groups of the FFT kernels
    int nfp64;
    int ref;                       // reference-rounding sampler
};

enum { ST_ADV = 0, ST_GEO, ST_DIV, ST_SOLVE, ST_IFFT, ST_VGRAD, ST_COUNT };

// Fetch the next work item for the whole CTA (and copy its sphere's
// descriptor into shared memory).  Returns false when the queue is empty.
__device__ __forceinline__ bool next_item(int* counter, int n, const int2* __restrict__ items,
                                          const KSphere* __restrict__ sph, int per_item, KSphere* s, int* s_item,
                                          int2* w)
{
    __syncthreads();  // everyone is done with the previous item
    if (threadIdx.x == 0) *s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = *s_item;
    if (it >= n) return false;
    *w = items[it];
    // cooperative copy of the descriptor
    const int words = sizeof(KSphere) / 4;
    const unsigned* src = reinterpret_cast<const unsigned*>(sph + w->x);
    unsigned* dst = reinterpret_cast<unsigned*>(s);
    for (int k = threadIdx.x; k < words; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    (void)per_item;
    return true;
}

// CELLS: every sphere of the batch has the cell-exact sampler and no
// particles, so a work item is cell tiles only and the kernel holds none of
// the reference-rounding or particle code (which would otherwise set its
// register budget: the general instance spills).
template <bool CELLS>
__global__ void __launch_bounds__(kk::ADV_THREADS, 8) kb_advect(const KSphere* __restrict__ sph,
                                                              const int2* __restrict__ items, int n, int* counter,
                                                              int cu, int cr, int tiles_per_item)
{
    __shared__ KSphere s;
    __shared__ int s_item;
    int2 w;
    kk::pdl_wait();
    while (next_item(counter, n, items, sph, tiles_per_item, &s, &s_item, &w)) {
        const int t0 = w.y * tiles_per_item, t1 = min(t0 + tiles_per_item, s.nb_adv);
        if constexpr (CELLS) {
            // the item's sphere constants and pointers in registers
            const KGeo g = s.g;
            const float *u = s.b.u[cu], *v = s.b.v[cu], *rho = s.b.rho[cr], *cc = s.b.cell_c, *cv = s.b.cell_v;
            float *uo = s.b.u[1 - cu], *vo = s.b.v[1 - cu], *ro = s.b.rho[1 - cr];
            for (int t = t0; t < t1; t++) kk::advect_cells_tile(g, u, v, rho, uo, vo, ro, cc, cv, t, threadIdx.x);
        } else {
            for (int t = t0; t < t1; t++) {
                if (s.ref)
                    kk::advect_tile<true>(s.g, s.b, cu, 1 - cu, cr, 1 - cr, s.nb_u, s.nb_v, s.nb_r, t, threadIdx.x);
                else
                    kk::advect_tile<false>(s.g, s.b, cu, 1 - cu, cr, 1 - cr, s.nb_u, s.nb_v, s.nb_r, t, threadIdx.x);
            }
        }
    }
}

__global__ void __launch_bounds__(kk::ELEM_THREADS, 8) kb_geo(const KSphere* __restrict__ sph,
                                                            const int2* __restrict__ items, int n, int* counter,
                                                            int src, int tiles_per_item)
{
    __shared__ KSphere s;
    __shared__ int s_item;
    int2 w;
    kk::pdl_wait();
    while (next_item(counter, n, items, sph, tiles_per_item, &s, &s_item, &w)) {
        const int t0 = w.y * tiles_per_item, t1 = min(t0 + tiles_per_item, s.nb_elem);
        for (int t = t0; t < t1; t++) kk::geo_tile(s.g, s.b, src, t * kk::ELEM_THREADS + threadIdx.x);
    }
}

// kb_geo and the 256 class of kb_solve are compiled for eight resident CTAs
// per SM (32 and 64 registers, a few bytes spilled): a persistent stage
// drains its queue faster with more CTAs in flight than with the registers
// that would avoid the spills (0.458 -> 0.442 ms per step on the 256-sphere
// mix, against 60 and 94 registers).
//
// The FFT and solve stages come in two instances by the batch's largest
// nTheta (MAXN = 256, 1024; batched spheres have nTheta <= 1024): a batch of
// small spheres does not run code sized, in registers, for the 1024-row
// tiles.  The 256 class of the FFT stages runs tiles of at most 64 threads
// and is compiled for sixteen of them per SM (64 registers, 740 and 812
// bytes spilled): 32 warps per SM instead of 16 at 128 registers, and
// 0.442 -> 0.421 ms per batched step; 48 registers spill twice as much and
// lose (0.474).
constexpr int fft_stage_threads(int maxn) { return maxn <= 256 ? 64 : kk::FFT_MAX_THREADS; }
constexpr int fft_stage_min_ctas(int maxn) { return maxn <= 256 ? 16 : 1; }
template <int MAXN>
__global__ void __launch_bounds__(fft_stage_threads(MAXN), fft_stage_min_ctas(MAXN)) kb_div_fft(const KSphere* __restrict__ sph,
                                                                  const int2* __restrict__ items, int n,
                                                                  int* counter, int uv_in, int uv_out)
{
    extern __shared__ float2 sm2[];
    __shared__ KSphere s;
    __shared__ int s_item;
    int2 w;
    kk::pdl_wait();
    while (next_item(counter, n, items, sph, 1, &s, &s_item, &w))
        kk::div_fft_tile<0, MAXN>(s.g, s.b, uv_in, uv_out, w.y, threadIdx.x, sm2);
}

template <int MAXN>
__global__ void __launch_bounds__(kk::SOLVE_THREADS, MAXN <= 256 ? 8 : 1) kb_solve(const KSphere* __restrict__ sph,
                                                               const int2* __restrict__ items, int n, int* counter)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ KSphere s;
    __shared__ int s_item;
    int2 w;
    kk::pdl_wait();
    while (next_item(counter, n, items, sph, 1, &s, &s_item, &w))
        kk::solve_tile<MAXN>(s.g, s.b, s.nfp64, w.y, threadIdx.x, smraw);
}

template <int MAXN>
__global__ void __launch_bounds__(fft_stage_threads(MAXN), fft_stage_min_ctas(MAXN)) kb_ifft(const KSphere* __restrict__ sph,
                                                               const int2* __restrict__ items, int n, int* counter,
                                                               int uv_in, int uv_out)
{
    extern __shared__ float2 sm2[];
    __shared__ KSphere s;
    __shared__ int s_item;
    int2 w;
    kk::pdl_wait();
    while (next_item(counter, n, items, sph, 1, &s, &s_item, &w))
        kk::ifft_tile<MAXN>(s.g, s.b, uv_in, uv_out, w.y, threadIdx.x, sm2);
}

using FftStageKernel = void (*)(const KSphere*, const int2*, int, int*, int, int);
using SolveStageKernel = void (*)(const KSphere*, const int2*, int, int*);

// smallest size class (256, 1024) holding nTheta = nt
inline int size_class(int nt) { return nt <= 256 ? 256 : 1024; }
inline FftStageKernel div_stage(int cls) { return cls == 256 ? kb_div_fft<256> : kb_div_fft<1024>; }
inline FftStageKernel ifft_stage(int cls) { return cls == 256 ? kb_ifft<256> : kb_ifft<1024>; }
inline SolveStageKernel solve_stage(int cls) { return cls == 256 ? kb_solve<256> : kb_solve<1024>; }

__global__ void __launch_bounds__(kk::ELEM_THREADS) kb_vgrad(const KSphere* __restrict__ sph,
                                                              const int2* __restrict__ items, int n, int* counter,
                                                              int uv_in, int uv_out, int tiles_per_item)
{
    __shared__ KSphere s;
    __shared__ int s_item;
    int2 w;
    kk::pdl_wait();
    while (next_item(counter, n, items, sph, tiles_per_item, &s, &s_item, &w)) {
        const int t0 = w.y * tiles_per_item, t1 = min(t0 + tiles_per_item, s.nb_elem);
        for (int t = t0; t < t1; t++) kk::vgrad_tile(s.g, s.b, uv_in, uv_out, t * kk::ELEM_THREADS + threadIdx.x);
    }
}

#define BCUDA(call)                                                                                    \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return kamino_fail(KAMINO_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                               __FILE__, __LINE__);                                                    \
    } while (0)

struct Shapes {
    int adv_cta_per_sm = 8, fft_cta_per_sm = 8, solve_cta_per_sm = 8, adv_tiles_per_item = 2;
};

// A set of handles advanced together.  Owns the device descriptor array, the
// work tables and the per-stage counters; not the handles.
struct Engine {
    int device = 0, nsm = 0;
    cudaStream_t stream = nullptr;
    std::vector<kamino_handle> hs;
    std::vector<KSphere> host_desc;
    KSphere* d_desc = nullptr;
    int2* d_items = nullptr;
    int* d_counters = nullptr;
    int n_items[ST_COUNT] = {};
    size_t item_off[ST_COUNT] = {};
    size_t smem_fft = 0, smem_solve = 0;
    int fft_block = 128;  // threads of the FFT kernels: the largest sphere's fft_threads
    int fft_resident = 1; // FFT CTAs of that size resident per SM (registers, shared memory)
    int cls = 1024;       // size class of the FFT and solve kernels: the largest sphere's
    bool cells_only = true;  // no sphere has particles or the reference-rounding sampler
    Shapes shapes;
    int cu = 0, cr = 0;
    cudaGraphExec_t graph[2][2] = {};
    size_t cap_desc = 0, cap_items = 0;
    int64_t cells = 0;

    ~Engine() { release(); }
    void release()
    {
        for (auto* gph : {&graph[0][0], &graph[0][1], &graph[1][0], &graph[1][1]})
            if (*gph) {
                cudaGraphExecDestroy(*gph);
                *gph = nullptr;
            }
        if (d_desc) cudaFree(d_desc);
        if (d_items) cudaFree(d_items);
        if (d_counters) cudaFree(d_counters);
        if (stream) cudaStreamDestroy(stream);
        d_desc = nullptr;
        d_items = nullptr;
        d_counters = nullptr;
        stream = nullptr;
    }

    int init(int dev)
    {
        device = dev;
        BCUDA(cudaSetDevice(dev));
        BCUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        BCUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        BCUDA(cudaMalloc(&d_counters, sizeof(int) * ST_COUNT));
        return KAMINO_OK;
    }

    void drop_graphs()
    {
        for (auto* gph : {&graph[0][0], &graph[0][1], &graph[1][0], &graph[1][1]})
            if (*gph) {
                cudaGraphExecDestroy(*gph);
                *gph = nullptr;
            }
    }

    // Rebuild descriptors and work tables for the current handle set (all
    // handles must share one buffer parity).
    int rebuild()
    {
        drop_graphs();
        host_desc.clear();
        cells = 0;
        if (hs.empty()) return KAMINO_OK;
        int pu = -1, pr = -1;
        for (kamino_handle h : hs) {
            KSphere s;
            std::memset(&s, 0, sizeof(s));
            int cuv, crr;
            int rc = kamino_internal_desc(h, &s.g, &s.b, &s.nfp64, &cuv, &crr);
            if (rc) return rc;
            if (pu < 0) {
                pu = cuv;
                pr = crr;
            } else if (pu != cuv || pr != crr) {
                return kamino_fail(KAMINO_ERR_INVALID, "batched spheres must share one buffer parity");
            }
            if (s.g.nt > 1024) return kamino_fail(KAMINO_ERR_INVALID, "batched spheres need n_theta <= 1024");
            kk::adv_tiles(s.g, s.nb_u, s.nb_v, s.nb_r);
            s.nb_adv = s.nb_u + s.nb_v + s.nb_r + (int)((s.b.npart + kk::ADV_THREADS - 1) / kk::ADV_THREADS);
            s.nb_elem = (kk::elem_groups(s.g.nt * s.g.np) + kk::ELEM_THREADS - 1) / kk::ELEM_THREADS;
            s.nb_fft = s.g.nt / kk::fft_rows_per_cta(s.g.nt);
            s.ref = (s.g.flags & KAMINO_F_REFERENCE_ROUNDING) ? 1 : 0;
            host_desc.push_back(s);
            cells += (int64_t)s.g.nt * s.g.np;
        }
        cu = pu;
        cr = pr;
        cells_only = true;
        for (const KSphere& s : host_desc) cells_only = cells_only && !s.ref && s.b.npart == 0;
        // work tables, largest sphere first
        std::vector<int> order(hs.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b2) { return host_desc[a].g.nt > host_desc[b2].g.nt; });
        std::vector<int2> items;
        const int tpi = std::max(1, shapes.adv_tiles_per_item);
        for (int st = 0; st < ST_COUNT; st++) {
            item_off[st] = items.size();
            for (int i : order) {
                const KSphere& s = host_desc[i];
                int count = 0;
                switch (st) {
                case ST_ADV: count = (s.nb_adv + tpi - 1) / tpi; break;
                case ST_GEO:
                case ST_VGRAD: count = (s.nb_elem + tpi - 1) / tpi; break;
                case ST_DIV:
                case ST_IFFT: count = s.nb_fft; break;
                case ST_SOLVE: count = kk::solve_tiles(s.g.nt, s.nfp64); break;
                }
                for (int t = 0; t < count; t++) items.push_back(make_int2(i, t));
            }
            n_items[st] = (int)(items.size() - item_off[st]);
        }
        BCUDA(cudaSetDevice(device));
        if (host_desc.size() > cap_desc) {
            if (d_desc) cudaFree(d_desc);
            cap_desc = std::max(host_desc.size(), cap_desc * 2);
            BCUDA(cudaMalloc(&d_desc, sizeof(KSphere) * cap_desc));
        }
        if (items.size() > cap_items) {
            if (d_items) cudaFree(d_items);
            cap_items = std::max(items.size(), cap_items * 2);
            BCUDA(cudaMalloc(&d_items, sizeof(int2) * cap_items));
        }
        BCUDA(cudaMemcpyAsync(d_desc, host_desc.data(), sizeof(KSphere) * host_desc.size(), cudaMemcpyHostToDevice,
                              stream));
        BCUDA(cudaMemcpyAsync(d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, stream));
        // dynamic shared memory: largest sphere decides
        smem_fft = 0;
        smem_solve = 0;
        fft_block = 32;
        int max_nt = 32;
        for (const KSphere& s : host_desc) {
            const int nt = s.g.nt;
            smem_fft = std::max(smem_fft, kk::fft_smem(nt));
            smem_solve = std::max(smem_solve, kk::solve_smem(nt));
            fft_block = std::max(fft_block, kk::fft_threads(nt));
            max_nt = std::max(max_nt, nt);
        }
        cls = size_class(max_nt);
        for (int c : {256, 1024}) {  // attributes belong to the functions, shared by every engine
            BCUDA(cudaFuncSetAttribute(div_stage(c), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kk::fft_smem_max()));
            BCUDA(cudaFuncSetAttribute(ifft_stage(c), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kk::fft_smem_max()));
            BCUDA(cudaFuncSetAttribute(solve_stage(c), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kk::solve_smem_max()));
        }
        int occ_div = 1, occ_ifft = 1;
        BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_div, div_stage(cls), fft_block, smem_fft));
        BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_ifft, ifft_stage(cls), fft_block, smem_fft));
        fft_resident = std::max(1, std::min(occ_div, occ_ifft));
        BCUDA(cudaStreamSynchronize(stream));  // host tables go out of scope
        return KAMINO_OK;
    }

    int grid(int st) const
    {
        int per = st == ST_ADV ? shapes.adv_cta_per_sm
                               : ((st == ST_DIV || st == ST_IFFT) ? shapes.fft_cta_per_sm
                                                                   : (st == ST_SOLVE ? shapes.solve_cta_per_sm
                                                                                     : shapes.adv_cta_per_sm));
        // no more CTAs than can be resident (threads, shared memory)
        if (st == ST_DIV || st == ST_IFFT) per = std::max(1, std::min(per, fft_resident));

        return std::max(1, std::min(n_items[st], per * nsm));
    }

    int enqueue_step(int c, int r)
    {
        BCUDA(cudaMemsetAsync(d_counters, 0, sizeof(int) * ST_COUNT, stream));
        const int tpi = std::max(1, shapes.adv_tiles_per_item);
        // programmatic dependent launches: each stage's CTAs are scheduled as
        // the previous stage's finish and wait in pdl_wait for all of it
        const KSphere* D = d_desc;
        BCUDA(kk::launch_pdl(cells_only ? kb_advect<true> : kb_advect<false>, grid(ST_ADV), kk::ADV_THREADS, 0,
                             stream, D, (const int2*)(d_items + item_off[ST_ADV]), n_items[ST_ADV],
                             d_counters + ST_ADV, c, r, tpi));
        BCUDA(kk::launch_pdl(kb_geo, grid(ST_GEO), kk::ELEM_THREADS, 0, stream, D,
                             (const int2*)(d_items + item_off[ST_GEO]), n_items[ST_GEO], d_counters + ST_GEO, 1 - c,
                             tpi));
        BCUDA(kk::launch_pdl(div_stage(cls), grid(ST_DIV), fft_block, smem_fft, stream, D,
                             (const int2*)(d_items + item_off[ST_DIV]), n_items[ST_DIV], d_counters + ST_DIV, 1 - c, c));
        BCUDA(kk::launch_pdl(solve_stage(cls), grid(ST_SOLVE), kk::SOLVE_THREADS, smem_solve, stream, D,
                             (const int2*)(d_items + item_off[ST_SOLVE]), n_items[ST_SOLVE], d_counters + ST_SOLVE));
        BCUDA(kk::launch_pdl(ifft_stage(cls), grid(ST_IFFT), fft_block, smem_fft, stream, D,
                             (const int2*)(d_items + item_off[ST_IFFT]), n_items[ST_IFFT], d_counters + ST_IFFT, c,
                             1 - c));
        BCUDA(kk::launch_pdl(kb_vgrad, grid(ST_VGRAD), kk::ELEM_THREADS, 0, stream, D,
                             (const int2*)(d_items + item_off[ST_VGRAD]), n_items[ST_VGRAD], d_counters + ST_VGRAD, c,
                             1 - c, tpi));
        BCUDA(cudaGetLastError());
        return KAMINO_OK;
    }

    // n steps of every sphere (asynchronous)
    int step_n(int n)
    {
        if (hs.empty() || n <= 0) return KAMINO_OK;
        BCUDA(cudaSetDevice(device));
        // the particles' visiting orders that are due, on the spheres' own
        // streams, before the batch's launches
        for (kamino_handle h : hs) {
            int launched = 0;
            if (int rc = kamino_internal_sort_particles(h, &launched)) return rc;
            if (launched) BCUDA(cudaStreamSynchronize(kamino_internal_stream(h)));
        }
        for (int k = 0; k < n; k++) {
            cudaGraphExec_t& ge = graph[cu][cr];
            if (!ge) {
                cudaGraph_t gph = nullptr;
                BCUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                int rc = enqueue_step(cu, cr);
                cudaError_t e = cudaStreamEndCapture(stream, &gph);
                if (rc) {
                    if (gph) cudaGraphDestroy(gph);
                    return rc;
                }
                if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
                e = cudaGraphInstantiate(&ge, gph, 0);
                cudaGraphDestroy(gph);
                if (e != cudaSuccess) {
                    ge = nullptr;
                    return kamino_fail(KAMINO_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
                }
            }
            BCUDA(cudaGraphLaunch(ge, stream));
            cu ^= 1;
            cr ^= 1;
        }
        for (kamino_handle h : hs) kamino_internal_advance(h, n);
        return KAMINO_OK;
    }
};

} // namespace

// =================================================================== batch
struct kamino_batch_s {
    Engine eng;
    std::vector<kamino_handle> owned;
    void* flush = nullptr;
    size_t flush_bytes = 0;
    ~kamino_batch_s()
    {
        eng.release();
        for (kamino_handle h : owned) kamino_destroy(h);
        if (flush) cudaFree(flush);
    }
};

extern "C" int kamino_batch_create(const kamino_config* cfgs, int n_spheres, kamino_batch* out)
{
    if (!cfgs || !out || n_spheres <= 0) return kamino_fail(KAMINO_ERR_INVALID, "kamino_batch_create: bad arguments");
    *out = nullptr;
    for (int i = 0; i < n_spheres; i++)
        if (cfgs[i].device != cfgs[0].device)
            return kamino_fail(KAMINO_ERR_INVALID, "all spheres of a batch must be on one device");
    for (int i = 0; i < n_spheres; i++)
        if (cfgs[i].n_theta > 1024 || cfgs[i].n_theta < 32)
            return kamino_fail(KAMINO_ERR_INVALID, "sphere %d: batched spheres need 32 <= n_theta <= 1024", i);
    auto* b = new kamino_batch_s();
    int rc = b->eng.init(cfgs[0].device);
    for (int i = 0; i < n_spheres && !rc; i++) {
        kamino_handle h = nullptr;
        rc = kamino_create(&cfgs[i], &h);
        if (!rc) b->owned.push_back(h);
    }
    if (!rc) {
        b->eng.hs = b->owned;
        rc = b->eng.rebuild();
    }
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return KAMINO_OK;
}

extern "C" int kamino_batch_destroy(kamino_batch b)
{
    if (b) {
        cudaSetDevice(b->eng.device);
        if (b->eng.stream) cudaStreamSynchronize(b->eng.stream);
        delete b;
    }
    return KAMINO_OK;
}

static int batch_handle(kamino_batch b, int sphere, kamino_handle* h)
{
    if (!b) return kamino_fail(KAMINO_ERR_INVALID, "null batch");
    if (sphere < 0 || sphere >= (int)b->owned.size())
        return kamino_fail(KAMINO_ERR_INVALID, "sphere %d out of range [0, %zu)", sphere, b->owned.size());
    *h = b->owned[sphere];
    cudaSetDevice(b->eng.device);
    cudaError_t e = cudaStreamSynchronize(b->eng.stream);
    if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "batch stream: %s", cudaGetErrorString(e));
    return KAMINO_OK;
}

extern "C" int kamino_batch_set_state(kamino_batch b, int sphere, int field, const float* host, size_t pitch_bytes)
{
    kamino_handle h = nullptr;
    int rc = batch_handle(b, sphere, &h);
    return rc ? rc : kamino_set_state(h, field, host, pitch_bytes);
}

extern "C" int kamino_batch_get_state(kamino_batch b, int sphere, int field, float* host, size_t pitch_bytes)
{
    kamino_handle h = nullptr;
    int rc = batch_handle(b, sphere, &h);
    return rc ? rc : kamino_get_state(h, field, host, pitch_bytes);
}

extern "C" int kamino_batch_step_n(kamino_batch b, int n)
{
    if (!b) return kamino_fail(KAMINO_ERR_INVALID, "null batch");
    // the handles' own streams may still hold state copies
    for (kamino_handle h : b->owned) {
        int rc = kamino_synchronize(h);
        if (rc) return rc;
    }
    return b->eng.step_n(n);
}

extern "C" int kamino_batch_synchronize(kamino_batch b)
{
    if (!b) return kamino_fail(KAMINO_ERR_INVALID, "null batch");
    BCUDA(cudaSetDevice(b->eng.device));
    BCUDA(cudaStreamSynchronize(b->eng.stream));
    return KAMINO_OK;
}

extern "C" int64_t kamino_batch_cells(kamino_batch b) { return b ? b->eng.cells : -1; }

extern "C" int kamino_batch_time_steps(kamino_batch b, int n, int flush_l2, double* ms_total)
{
    if (!b || n <= 0 || !ms_total) return kamino_fail(KAMINO_ERR_INVALID, "bad arguments");
    int rc = kamino_batch_step_n(b, 0);
    if (rc) return rc;
    Engine& e = b->eng;
    BCUDA(cudaSetDevice(e.device));
    if (flush_l2 && !b->flush) {
        b->flush_bytes = (size_t)256 << 20;
        BCUDA(cudaMalloc(&b->flush, b->flush_bytes));
    }
    std::vector<cudaEvent_t> ev(2 * (size_t)n);
    for (auto& x : ev) BCUDA(cudaEventCreate(&x));
    for (int k = 0; k < n && !rc; k++) {
        if (flush_l2) BCUDA(kk::flush_l2(b->flush, b->flush_bytes, k & 0xff, e.stream));
        BCUDA(cudaEventRecord(ev[2 * k], e.stream));
        rc = e.step_n(1);
        BCUDA(cudaEventRecord(ev[2 * k + 1], e.stream));
    }
    cudaError_t err = cudaStreamSynchronize(e.stream);
    double tot = 0;
    for (int k = 0; k < n && err == cudaSuccess; k++) {
        float ms = 0;
        err = cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]);
        tot += ms;
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (rc) return rc;
    if (err != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "batch timing: %s", cudaGetErrorString(err));
    *ms_total = tot;
    return KAMINO_OK;
}

// Candidate launch shapes are timed on the live batch; the state of every
// sphere is copied aside first and restored afterwards.
extern "C" int kamino_batch_autotune(kamino_batch b, int reps, int* chosen, int max_chosen)
{
    if (!b || reps <= 0) return kamino_fail(KAMINO_ERR_INVALID, "bad arguments");
    Engine& e = b->eng;
    int rc = kamino_batch_step_n(b, 0);
    if (rc) return rc;
    BCUDA(cudaSetDevice(e.device));
    BCUDA(cudaStreamSynchronize(e.stream));
    // save: every handle's fields and particles, both parities' current halves
    struct Saved {
        std::vector<float> u, v, r, p;
    };
    std::vector<Saved> saved(b->owned.size());
    struct Counters {
        int cu, cr;
        int64_t steps;
        double time;
    };
    std::vector<Counters> par(b->owned.size());
    for (size_t i = 0; i < b->owned.size(); i++) {
        kamino_handle h = b->owned[i];
        KGeo g;
        KBufs bb;
        int cuv, crr;
        kamino_internal_desc(h, &g, &bb, nullptr, &cuv, &crr);
        size_t nf = (size_t)g.nt * g.np;
        saved[i].u.resize(nf);
        saved[i].v.resize(nf);
        saved[i].r.resize(nf);
        saved[i].p.resize(2 * (size_t)bb.npart);
        if ((rc = kamino_get_state(h, KAMINO_U_PHI, saved[i].u.data(), 0))) return rc;
        if ((rc = kamino_get_state(h, KAMINO_U_THETA, saved[i].v.data(), 0))) return rc;
        if ((rc = kamino_get_state(h, KAMINO_THICKNESS, saved[i].r.data(), 0))) return rc;
        if (bb.npart && (rc = kamino_get_state(h, KAMINO_PARTICLES, saved[i].p.data(), 0))) return rc;
        kamino_internal_get_counters(h, &par[i].cu, &par[i].cr, &par[i].steps, &par[i].time);
    }
    const Shapes base = e.shapes;
    Shapes best = base;
    double best_ms = 1e30;
    const int adv_opts[] = {4, 8, 16}, fft_opts[] = {4, 8, 16}, solve_opts[] = {4, 8, 16}, tpi_opts[] = {1, 2, 4};
    auto trial = [&](const Shapes& s, double* ms) {
        e.shapes = s;
        int r2 = e.rebuild();
        if (r2) return r2;
        r2 = e.step_n(2);  // warm-up (and graph build)
        if (r2) return r2;
        cudaEvent_t a, z;
        cudaEventCreate(&a);
        cudaEventCreate(&z);
        cudaEventRecord(a, e.stream);
        r2 = e.step_n(2 * reps);
        cudaEventRecord(z, e.stream);
        cudaEventSynchronize(z);
        float t = 0;
        cudaEventElapsedTime(&t, a, z);
        cudaEventDestroy(a);
        cudaEventDestroy(z);
        *ms = t;
        return r2;
    };
    // coordinate search: one parameter at a time, starting from the defaults
    for (int pass = 0; pass < 4 && !rc; pass++) {
        for (int k = 0; k < 3 && !rc; k++) {
            Shapes s = best;
            if (pass == 0) s.adv_cta_per_sm = adv_opts[k];
            if (pass == 1) s.fft_cta_per_sm = fft_opts[k];
            if (pass == 2) s.solve_cta_per_sm = solve_opts[k];
            if (pass == 3) s.adv_tiles_per_item = tpi_opts[k];
            double ms = 0;
            rc = trial(s, &ms);
            if (!rc && ms < best_ms) {
                best_ms = ms;
                best = s;
            }
        }
    }
    // restore the state and parity the batch had before the trials
    e.shapes = best;
    for (size_t i = 0; i < b->owned.size() && !rc; i++) {
        kamino_handle h = b->owned[i];
        kamino_internal_set_counters(h, par[i].cu, par[i].cr, par[i].steps, par[i].time);
        if ((rc = kamino_set_state(h, KAMINO_U_PHI, saved[i].u.data(), 0))) break;
        if ((rc = kamino_set_state(h, KAMINO_U_THETA, saved[i].v.data(), 0))) break;
        if ((rc = kamino_set_state(h, KAMINO_THICKNESS, saved[i].r.data(), 0))) break;
        if (!saved[i].p.empty() && (rc = kamino_set_state(h, KAMINO_PARTICLES, saved[i].p.data(), 0))) break;
    }
    if (!rc) rc = e.rebuild();
    if (rc) return rc;
    const int vals[4] = {best.adv_cta_per_sm, best.fft_cta_per_sm, best.solve_cta_per_sm, best.adv_tiles_per_item};
    for (int k = 0; k < max_chosen && k < 4 && chosen; k++) chosen[k] = vals[k];
    return KAMINO_OK;
}

// ================================================================= serving
namespace {

// Pooled device memory is interchangeable between requests of one n_theta
// and one number of FP64 modes (the multiplier tables depend on both).
int pool_key(const kamino_config& c) { return c.n_theta * 64 + std::min(std::max(c.fp64_modes, 0), 63); }

struct Request {
    int64_t id = 0;
    kamino_config cfg;
    int32_t steps = 0, remaining = 0;
    double arrival = 0, done_at = -1;
    std::vector<float> u, v, r;  // initial state, then the result
    kamino_handle h = nullptr;
    size_t bytes = 0;
    bool done = false;
    int status = KAMINO_OK;  // KAMINO_ERR_BUDGET for a request that can never fit
    bool solo = false;       // advanced by its own one-sphere graphs
    cudaEvent_t finished = nullptr;  // solo: recorded after its last step
    cudaEvent_t started = nullptr;   // solo: recorded before its first step
};

} // namespace

struct kamino_server_s {
    kamino_server_config cfg;
    Engine eng;
    std::chrono::steady_clock::time_point t0;
    int64_t next_id = 1;
    std::deque<std::shared_ptr<Request>> queue;
    std::vector<std::shared_ptr<Request>> resident;
    std::map<int64_t, std::shared_ptr<Request>> all;
    std::map<int, std::vector<kamino_handle>> pool;  // free handles by n_theta
    std::map<int, size_t> bytes_for;                 // device bytes of a handle by n_theta
    std::vector<double> latencies;
    int64_t cell_steps = 0, completed = 0;
    int64_t solo_cells = 0, batched_cells = 0, rounds = 0;
    double round_seconds = 0, solo_seconds = 0, poll_seconds = 0;
    cudaEvent_t round_start = nullptr;
    size_t resident_bytes = 0, peak_bytes = 0;
    size_t pooled_bytes = 0;  // free handles kept for reuse also hold HBM
    double busy = 0;
    bool dirty = true;
    // the batched step's round in flight
    cudaEvent_t round_done = nullptr;
    bool round_pending = false;
    double last_poll = 0;  // for busy_seconds
    std::vector<cudaEvent_t> free_events;
    ~kamino_server_s()
    {
        cudaDeviceSynchronize();
        eng.release();
        for (auto& r : resident) {
            if (r->h) kamino_destroy(r->h);
            if (r->finished) cudaEventDestroy(r->finished);
        }
        for (auto& kv : pool)
            for (kamino_handle h : kv.second) kamino_destroy(h);
        for (cudaEvent_t e : free_events) cudaEventDestroy(e);
        if (round_done) cudaEventDestroy(round_done);
        if (round_start) cudaEventDestroy(round_start);
    }
    int solo_n_theta() const { return cfg.solo_n_theta > 0 ? cfg.solo_n_theta : 512; }
    int solo_slots() const { return cfg.solo_slots > 0 ? cfg.solo_slots : 3; }
    int solo_running() const
    {
        int n = 0;
        for (auto& r : resident) n += r->solo ? 1 : 0;
        return n;
    }
    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

extern "C" int kamino_server_create(const kamino_server_config* cfg, kamino_server* out)
{
    if (!cfg || !out) return kamino_fail(KAMINO_ERR_INVALID, "kamino_server_create: null argument");
    if (cfg->budget_bytes == 0) return kamino_fail(KAMINO_ERR_INVALID, "budget_bytes must be > 0");
    auto* s = new kamino_server_s();
    s->cfg = *cfg;
    if (s->cfg.steps_per_round <= 0) s->cfg.steps_per_round = 10;
    s->t0 = std::chrono::steady_clock::now();
    int rc = s->eng.init(cfg->device);
    if (!rc && (cudaEventCreate(&s->round_done) != cudaSuccess || cudaEventCreate(&s->round_start) != cudaSuccess))
        rc = kamino_fail(KAMINO_ERR_CUDA, "kamino_server_create: event");
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return KAMINO_OK;
}

extern "C" int kamino_server_destroy(kamino_server s)
{
    if (s) {
        cudaSetDevice(s->eng.device);
        if (s->eng.stream) cudaStreamSynchronize(s->eng.stream);
        delete s;
    }
    return KAMINO_OK;
}

extern "C" double kamino_server_now(kamino_server s) { return s ? s->now() : -1.0; }

extern "C" int kamino_server_submit(kamino_server s, const kamino_config* cfg, const float* u_phi,
                                    const float* u_theta, const float* thickness, int32_t steps,
                                    double arrival_time_s, int64_t* request_id)
{
    if (!s || !cfg || !u_phi || !u_theta || !thickness || steps < 0)
        return kamino_fail(KAMINO_ERR_INVALID, "kamino_server_submit: bad arguments");
    const int nt = cfg->n_theta;
    if (nt < 32 || nt > 1024 || (nt & (nt - 1)))
        return kamino_fail(KAMINO_ERR_INVALID, "served spheres need n_theta a power of two in [32, 1024]");
    if (cfg->device != s->eng.device) return kamino_fail(KAMINO_ERR_INVALID, "request device != server device");
    if (kamino_particle_count(cfg) != 0) return kamino_fail(KAMINO_ERR_INVALID, "served spheres carry no particles");
    auto r = std::make_shared<Request>();
    r->id = s->next_id++;
    r->cfg = *cfg;
    r->steps = r->remaining = steps;
    r->arrival = arrival_time_s >= 0 ? arrival_time_s : s->now();
    const size_t nf = (size_t)nt * 2 * nt, nv = (size_t)(nt - 1) * 2 * nt;
    r->u.assign(u_phi, u_phi + nf);
    r->v.assign(u_theta, u_theta + nv);
    r->r.assign(thickness, thickness + nf);
    s->queue.push_back(r);
    s->all[r->id] = r;
    if (request_id) *request_id = r->id;
    return KAMINO_OK;
}

// Device bytes of one handle for this request's shape.  The first request of
// a shape creates a handle to measure it; the handle is pooled when it fits
// the budget (the request that asked takes it) and destroyed otherwise.
static int server_device_bytes(kamino_server s, const kamino_config& c, size_t* bytes)
{
    auto it = s->bytes_for.find(pool_key(c));
    if (it != s->bytes_for.end()) {
        *bytes = it->second;
        return KAMINO_OK;
    }
    kamino_handle h = nullptr;
    int rc = kamino_create(&c, &h);
    if (rc) return rc;
    size_t n = 0;
    kamino_device_bytes(h, &n);
    s->bytes_for[pool_key(c)] = n;
    if (n <= s->cfg.budget_bytes) {
        s->pool[pool_key(c)].push_back(h);
        s->pooled_bytes += n;
    } else {
        kamino_destroy(h);
    }
    *bytes = n;
    return KAMINO_OK;
}

// Frees pooled handles of other shapes until `need` more bytes fit beside
// everything the server holds.  Returns whether they fit.
static bool server_make_room(kamino_server s, int key, size_t need)
{
    for (auto& kv : s->pool) {
        if (s->resident_bytes + s->pooled_bytes + need <= s->cfg.budget_bytes) break;
        if (kv.first == key) continue;
        const size_t each = s->bytes_for[kv.first];
        while (!kv.second.empty() && s->resident_bytes + s->pooled_bytes + need > s->cfg.budget_bytes) {
            kamino_destroy(kv.second.back());
            kv.second.pop_back();
            s->pooled_bytes -= each;
        }
    }
    return s->resident_bytes + s->pooled_bytes + need <= s->cfg.budget_bytes;
}

// Moves a finished request's result to the host and its handle to the pool.
static int server_retire(kamino_server s, const std::shared_ptr<Request>& r, double t)
{
    int rc = kamino_get_state(r->h, KAMINO_U_PHI, r->u.data(), 0);
    if (!rc) rc = kamino_get_state(r->h, KAMINO_U_THETA, r->v.data(), 0);
    if (!rc) rc = kamino_get_state(r->h, KAMINO_THICKNESS, r->r.data(), 0);
    if (rc) return rc;
    r->done = true;
    r->done_at = t;
    s->latencies.push_back(t - r->arrival);
    s->completed++;
    s->resident_bytes -= r->bytes;
    s->pooled_bytes += r->bytes;
    s->pool[pool_key(r->cfg)].push_back(r->h);
    r->h = nullptr;
    if (r->started && r->finished) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, r->started, r->finished) == cudaSuccess) s->solo_seconds += ms / 1e3;
    }
    if (r->started) {
        cudaEventDestroy(r->started);
        r->started = nullptr;
    }
    if (r->finished) {
        s->free_events.push_back(r->finished);
        r->finished = nullptr;
    }
    return KAMINO_OK;
}

// One turn of the request loop; never waits for the device.
//  1. solo requests whose last step has finished, and batched ones whose
//     steps are done once the round in flight has finished, are retired;
//  2. queued requests whose arrival time has passed are admitted FIFO while
//     their state fits the budget (and the slot limit): a solo request gets
//     all its steps launched at once on its handle's stream, a batched one
//     joins the next round;
//  3. if no round is in flight, the batched spheres take a round of
//     min(steps_per_round, fewest steps left) steps.
static int server_poll(kamino_server s, int* n_completed);

extern "C" int kamino_server_poll(kamino_server s, int* n_completed)
{
    if (!s) return kamino_fail(KAMINO_ERR_INVALID, "null server");
    const double t_in = s->now();
    const int rc = server_poll(s, n_completed);
    s->poll_seconds += s->now() - t_in;
    return rc;
}

static int server_poll(kamino_server s, int* n_completed)
{
    Engine& e = s->eng;
    BCUDA(cudaSetDevice(e.device));
    const double t = s->now();
    if (!s->resident.empty()) s->busy += t - s->last_poll;
    s->last_poll = t;
    int done_now = 0;
    if (s->round_pending) {
        cudaError_t q = cudaEventQuery(s->round_done);
        if (q == cudaSuccess) {
            s->round_pending = false;
            float ms = 0;
            if (cudaEventElapsedTime(&ms, s->round_start, s->round_done) == cudaSuccess) s->round_seconds += ms / 1e3;
            s->rounds++;
        } else if (q != cudaErrorNotReady) {
            return kamino_fail(KAMINO_ERR_CUDA, "batched round: %s", cudaGetErrorString(q));
        }
    }
    for (size_t i = 0; i < s->resident.size();) {
        auto r = s->resident[i];
        bool finished = false;
        if (r->solo) {
            cudaError_t q = cudaEventQuery(r->finished);
            if (q != cudaSuccess && q != cudaErrorNotReady)
                return kamino_fail(KAMINO_ERR_CUDA, "request %lld: %s", (long long)r->id, cudaGetErrorString(q));
            finished = q == cudaSuccess;
        } else {
            finished = r->remaining == 0 && !s->round_pending;
        }
        if (!finished) {
            i++;
            continue;
        }
        int rc = server_retire(s, r, t);
        if (rc) return rc;
        done_now++;
        if (!r->solo) s->dirty = true;
        s->resident[i] = s->resident.back();
        s->resident.pop_back();
    }
    // admit queued requests (FIFO, arrival time reached) while they fit; a
    // solo request waiting for a solo slot is passed over, not waited for
    int solo_free = s->solo_slots() - s->solo_running();
    for (auto qi = s->queue.begin(); qi != s->queue.end();) {
        auto r = *qi;
        if (r->arrival > t) break;
        if (s->cfg.max_resident > 0 && (int)s->resident.size() >= s->cfg.max_resident) break;
        const bool solo = r->cfg.n_theta >= s->solo_n_theta() || r->cfg.n_theta > 1024;  // batched: <= 1024
        if (solo && solo_free <= 0) {
            ++qi;
            continue;
        }
        size_t need = 0;
        int rc = server_device_bytes(s, r->cfg, &need);
        if (rc) return rc;
        if (need > s->cfg.budget_bytes) {
            // can never fit: the request fails and leaves the queue
            r->done = true;
            r->status = KAMINO_ERR_BUDGET;
            r->done_at = t;
            s->queue.erase(qi);
            return kamino_fail(KAMINO_ERR_BUDGET, "request %lld needs %zu bytes, budget %zu", (long long)r->id, need,
                               s->cfg.budget_bytes);
        }
        if (s->resident_bytes + need > s->cfg.budget_bytes) break;
        auto& free_list = s->pool[pool_key(r->cfg)];
        kamino_handle h = nullptr;
        if (!free_list.empty()) {
            h = free_list.back();
            free_list.pop_back();
            s->pooled_bytes -= need;
            rc = kamino_internal_reset(h, &r->cfg);
        } else {
            if (!server_make_room(s, pool_key(r->cfg), need)) break;
            rc = kamino_create(&r->cfg, &h);
        }
        r->solo = solo;
        // a batched sphere joins at the batched step's buffer parity before
        // its state is written (every batched sphere advances together)
        if (!rc && !r->solo) rc = kamino_internal_set_counters(h, e.cu, e.cr, 0, 0.0);
        if (!rc) rc = kamino_set_state(h, KAMINO_U_PHI, r->u.data(), 0);
        if (!rc) rc = kamino_set_state(h, KAMINO_U_THETA, r->v.data(), 0);
        if (!rc) rc = kamino_set_state(h, KAMINO_THICKNESS, r->r.data(), 0);
        if (!rc && r->solo) {
            if (!s->free_events.empty()) {
                r->finished = s->free_events.back();
                s->free_events.pop_back();
            } else if (cudaEventCreate(&r->finished) != cudaSuccess) {
                rc = kamino_fail(KAMINO_ERR_CUDA, "request event");
            }
            if (!rc && (cudaEventCreate(&r->started) != cudaSuccess ||
                        cudaEventRecord(r->started, kamino_internal_stream(h)) != cudaSuccess))
                rc = kamino_fail(KAMINO_ERR_CUDA, "request start event");
            if (!rc) rc = kamino_step_n(h, r->remaining);
            if (!rc && cudaEventRecord(r->finished, kamino_internal_stream(h)) != cudaSuccess)
                rc = kamino_fail(KAMINO_ERR_CUDA, "request event record");
            if (!rc) {
                const int64_t cs = (int64_t)r->remaining * r->cfg.n_theta * 2 * r->cfg.n_theta;
                s->cell_steps += cs;
                s->solo_cells += cs;
                r->remaining = 0;
            }
        }
        if (rc) {
            if (h) kamino_destroy(h);
            for (cudaEvent_t* ev : {&r->finished, &r->started})
                if (*ev) {
                    cudaEventDestroy(*ev);
                    *ev = nullptr;
                }
            return rc;
        }
        r->h = h;
        r->bytes = need;
        s->resident_bytes += need;
        s->peak_bytes = std::max(s->peak_bytes, s->resident_bytes);
        s->resident.push_back(r);
        qi = s->queue.erase(qi);
        if (r->solo)
            solo_free--;
        else
            s->dirty = true;
    }
    if (!s->round_pending) {
        int steps = s->cfg.steps_per_round;
        bool any = false;
        for (auto& r : s->resident)
            if (!r->solo) {
                any = true;
                steps = std::min(steps, (int)r->remaining);
            }
        if (any && steps > 0) {
            if (s->dirty) {
                e.hs.clear();
                for (auto& r : s->resident)
                    if (!r->solo) e.hs.push_back(r->h);
                int rc = e.rebuild();
                if (rc) return rc;
                s->dirty = false;
            }
            BCUDA(cudaEventRecord(s->round_start, e.stream));
            int rc = e.step_n(steps);
            if (rc) return rc;
            BCUDA(cudaEventRecord(s->round_done, e.stream));
            s->round_pending = true;
            for (auto& r : s->resident)
                if (!r->solo) r->remaining -= steps;
            s->cell_steps += (int64_t)steps * e.cells;
            s->batched_cells += (int64_t)steps * e.cells;
        }
    }
    if (n_completed) *n_completed = done_now;
    return KAMINO_OK;
}

extern "C" int kamino_server_fetch(kamino_server s, int64_t request_id, int field, float* host)
{
    if (!s || !host) return kamino_fail(KAMINO_ERR_INVALID, "null argument");
    auto it = s->all.find(request_id);
    if (it == s->all.end()) return kamino_fail(KAMINO_ERR_NOT_FOUND, "unknown request %lld", (long long)request_id);
    auto& r = it->second;
    if (!r->done) return KAMINO_ERR_NOT_READY;
    if (r->status) return kamino_fail(r->status, "request %lld failed admission", (long long)request_id);
    const std::vector<float>* src = field == KAMINO_U_PHI ? &r->u
                                    : field == KAMINO_U_THETA ? &r->v
                                    : field == KAMINO_THICKNESS ? &r->r
                                                                : nullptr;
    if (!src) return kamino_fail(KAMINO_ERR_INVALID, "field %d is not kept for served requests", field);
    std::memcpy(host, src->data(), sizeof(float) * src->size());
    return KAMINO_OK;
}

extern "C" int kamino_server_release(kamino_server s, int64_t request_id)
{
    if (!s) return kamino_fail(KAMINO_ERR_INVALID, "null server");
    auto it = s->all.find(request_id);
    if (it == s->all.end()) return kamino_fail(KAMINO_ERR_NOT_FOUND, "unknown request %lld", (long long)request_id);
    if (!it->second->done) return KAMINO_ERR_NOT_READY;
    s->all.erase(it);
    return KAMINO_OK;
}

extern "C" int kamino_server_get_stats(kamino_server s, kamino_server_stats* st)
{
    if (!s || !st) return kamino_fail(KAMINO_ERR_INVALID, "null argument");
    std::memset(st, 0, sizeof(*st));
    st->submitted = s->next_id - 1;
    st->completed = s->completed;
    st->resident = (int64_t)s->resident.size();
    st->queued = (int64_t)s->queue.size();
    st->cell_steps = s->cell_steps;
    st->busy_seconds = s->busy;
    st->solo_cell_steps = s->solo_cells;
    st->batched_cell_steps = s->batched_cells;
    st->batched_rounds = s->rounds;
    st->batched_round_seconds = s->round_seconds;
    st->solo_seconds = s->solo_seconds;
    st->poll_seconds = s->poll_seconds;
    std::vector<double> l = s->latencies;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) { return l[std::min(l.size() - 1, (size_t)std::floor(q * (l.size() - 1) + 0.5))]; };
        st->p50_latency_s = pct(0.50);
        st->p99_latency_s = pct(0.99);
        double m = 0;
        for (double x : l) m += x;
        st->mean_latency_s = m / l.size();
    }
    st->resident_bytes = s->resident_bytes;
    st->peak_resident_bytes = s->peak_bytes;
    return KAMINO_OK;
}
