// kamino_solver.cu — one-sphere solver behind the C ABI (kamino_gb300.h).
//
// Host orchestration replacing KaminoSolver (KaminoGPU/kernel/KaminoSolver.cu
// :12-238) and the stage functions of KaminoCore.cu (:344-384, 551-583,
// 749-842).  All state lives in one device arena allocated at create time;
// a step is five kernel launches (kamino_kernels.cuh) replayed from a CUDA
// graph on the handle's own stream.  Every failure returns a status code.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "kamino_common.h"
#include "kamino_kernels.cuh"

// ------------------------------------------------------------------ errors
static thread_local char g_err[1024] = "";

int kamino_fail(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char* kamino_last_error(void) { return g_err; }

#define KCUDA(call)                                                                                  \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return kamino_fail(KAMINO_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                               __FILE__, __LINE__);                                                  \
    } while (0)

// ------------------------------------------------------------------ handle
struct kamino_solver_s {
    kamino_config cfg;
    KGeo g;
    KBufs b;
    int device = 0;
    cudaStream_t stream = nullptr;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    int cur_uv = 0, cur_r = 0;  // which buffer holds (u, v) and (thickness, particles)
    int nfp64 = 0;
    int64_t steps = 0;
    double time = 0.0;
    float last_dt = 0.0f;
    cudaGraphExec_t graph[2][2][2] = {};  // [steps-1][cur_uv][cur_r]
    void* flush = nullptr;
    size_t flush_bytes = 0;
    size_t smem_div = 0, smem_solve = 0, smem_ifft = 0;
    cudaStream_t io_stream = nullptr;  // kamino_step_host: the early thickness download
    cudaEvent_t ev_adv = nullptr;      // kamino_step_host: the advection has written its fields
    cudaEvent_t ev_uv = nullptr;       // kamino_step_host: u_phi and u_theta are on the device
    cudaEvent_t ev_rho = nullptr;      // kamino_step_host: the thickness is on the device
    cudaEvent_t ev_u = nullptr;        // kamino_step_host: u_phi of the step is final
    KFrames* frames = nullptr;         // frame output (kamino_frames.cu), made on first use
    // the particles' visiting order (KBufs::pperm): rebuilt by sort_particles
    // every kSortEvery steps, and before the first step after the particles
    // were set from outside
    int* pkeys = nullptr;
    int* pcounts = nullptr;
    int* ptmp = nullptr;  // the new visiting order, copied into KBufs::pperm
    int64_t sorted_at = -1;  // step count of the last sort; -1: due
};

// Steps between rebuilds of the particles' visiting order: particles move
// a fraction of a cell a step, so the order stays mostly block by block for
// a few dozen (nTheta = 512, dt = 0.002: the advection launch takes the same
// time with a rebuild every 8, 16 or 32 steps, and a rebuild ~25 us).
static const int kSortEvery = 16;

static const char* const kKernelNames[] = {"k_advect", "k_geo_centers", "k_div_fft",
                                           "k_solve",  "k_ifft_u",      "k_vgrad"};
static const int kNumKernels = 6;

extern "C" const char* kamino_kernel_name(int index)
{
    return (index >= 0 && index < kNumKernels) ? kKernelNames[index] : "";
}

// Smallest float x with floorf((float)((double)x / M_2PI)) >= 1, i.e. the
// first phi the reference wraps back by 2pi (KaminoCore.cu:27).
static float wrap_threshold()
{
    auto wraps = [](float x) { return (int)floorf((float)((double)x / KAMINO_2PI_D)) >= 1; };
    float x = (float)KAMINO_2PI_D;
    while (wraps(x)) x = nextafterf(x, 0.0f);
    while (!wraps(x)) x = nextafterf(x, 100.0f);
    return x;
}

static float pi_up_threshold()
{
    // smallest float strictly greater than M_PI (as a double)
    float x = (float)KAMINO_PI_D;
    while ((double)x > KAMINO_PI_D) x = nextafterf(x, 0.0f);
    while (!((double)x > KAMINO_PI_D)) x = nextafterf(x, 100.0f);
    return x;
}

static int fill_geo(const kamino_config* c, KGeo* g)
{
    const int nt = c->n_theta;
    if (nt < 32 || nt > 2048 || (nt & (nt - 1)))
        return kamino_fail(KAMINO_ERR_INVALID, "n_theta=%d: must be a power of two in [32, 2048]", nt);
    if (!(c->radius > 0) || !std::isfinite(c->radius))
        return kamino_fail(KAMINO_ERR_INVALID, "radius=%g must be positive", c->radius);
    if (!(c->dt > 0) || !std::isfinite(c->dt))
        return kamino_fail(KAMINO_ERR_INVALID, "dt=%g must be positive", c->dt);
    std::memset(g, 0, sizeof(*g));
    g->nt = nt;
    g->np = 2 * nt;
    g->mask = g->np - 1;
    g->half = nt;
    int l = 0;
    while ((1 << l) < nt) l++;
    g->log2nt = l;
    g->h = (float)(KAMINO_PI_D / nt);  // Kamino::gridLen, KaminoCore.cu:849
    g->halfh = 0.5f * g->h;
    g->invh = (float)(1.0 / (double)g->h);
    g->R = (float)c->radius;
    g->dt = (float)c->dt;
    g->cofTheta = g->dt / g->R;
    g->cellTheta = (float)(c->dt / (c->radius * (KAMINO_PI_D / nt)));
    g->pi_up = pi_up_threshold();
    g->wrap_phi_hi = wrap_threshold();
    g->pitch = g->np;
    g->rows = nt + 2;
    g->flags = c->flags;
    return KAMINO_OK;
}

static size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

static void destroy_graphs(kamino_solver_s* h)
{
    for (auto& a : h->graph)
        for (auto& b : a)
            for (auto& e : b)
                if (e) {
                    cudaGraphExecDestroy(e);
                    e = nullptr;
                }
}

extern "C" int kamino_destroy(kamino_handle h)
{
    if (!h) return KAMINO_OK;
    int dev0 = 0;
    cudaGetDevice(&dev0);
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    destroy_graphs(h);
    kamino_frames_release(h->frames);
    if (h->io_stream) cudaStreamSynchronize(h->io_stream);
    for (cudaEvent_t e : {h->ev_adv, h->ev_uv, h->ev_rho, h->ev_u})
        if (e) cudaEventDestroy(e);
    if (h->io_stream) cudaStreamDestroy(h->io_stream);
    if (h->arena) cudaFree(h->arena);
    if (h->flush) cudaFree(h->flush);
    if (h->stream) cudaStreamDestroy(h->stream);
    cudaSetDevice(dev0);
    delete h;
    return KAMINO_OK;
}

// Laplacian rows of precomputeABCKernel (KaminoSolver.cu:128-159) for n != 0,
// with h = pi/nTheta in double: B(n) = B0 - n^2 * S.
void laplacian_rows(int nt, std::vector<double>& A, std::vector<double>& C, std::vector<double>& B0,
                    std::vector<double>& S)
{
    const double h = KAMINO_PI_D / nt;
    A.resize(nt);
    C.resize(nt);
    B0.resize(nt);
    S.resize(nt);
    for (int i = 0; i < nt; i++) {
        double th = (i + 0.5) * h, c = std::cos(th), s = std::sin(th);
        double a = 1.0 / (h * h) - c / 2.0 / h / s;
        double cc = 1.0 / (h * h) + c / 2.0 / h / s;
        double b0 = -2.0 / (h * h);
        if (i == 0) {
            b0 += a;
            a = 0.0;
        }
        if (i == nt - 1) {
            b0 += cc;
            cc = 0.0;
        }
        A[i] = a;
        C[i] = cc;
        B0[i] = b0;
        S[i] = 1.0 / (s * s);
    }
}

// Multiplier tables of the FP64 mode solves (layout: kk::s64_stride).  The
// device solve of a mode repeats the dominance-form elimination of
// solve_mode32 on the right-hand side only; the matrix part is fixed per
// sphere, so it is run here once, in double.
void fp64_tables(int nt, int nmodes, const std::vector<double>& A, const std::vector<double>& C,
                 const std::vector<double>& S, std::vector<double>& out)
{
    const size_t stride = kk::s64_stride(nt);
    out.assign(stride * (size_t)nmodes, 0.0);
    const int TH = kk::s64_threads(nt), P = nt / TH;  // P >= 2
    struct R3 {
        double a, c, s;
    };
    for (int q = 0; q < nmodes; q++) {
        const double m2 = (double)(q + 1) * (q + 1);
        double* tb = out.data() + stride * q;
        double *dn = tb, *up = tb + nt, *bA = tb + 2 * nt, *bC = tb + 3 * nt, *bInv = tb + 4 * nt;
        double *rF = tb + 5 * nt, *pl = rF + kk::S64_TH, *ph = pl + kk::S64_L * kk::S64_R,
               *pinv = ph + kk::S64_L * kk::S64_R;
        std::vector<R3> red;
        {
            std::vector<double> a(A), c(C), s(nt);
            for (int i = 0; i < nt; i++) s[i] = m2 * S[i];
            for (int k = 0; k < TH; k++) {
                const int f = k * P, l = f + P - 1;
                for (int i = f + 2; i <= l; i++) {  // downward
                    double r = a[i] / (s[i - 1] + a[i - 1] + c[i - 1]);
                    dn[i] = r;
                    a[i] = r * a[i - 1];
                    s[i] += r * s[i - 1];
                }
                R3 L = {a[l], c[l], s[l]};
                if (P >= 3) {  // row l-1 starts the upward pass as it is
                    bA[l - 1] = a[l - 1];
                    bC[l - 1] = c[l - 1];
                    bInv[l - 1] = 1.0 / (s[l - 1] + a[l - 1] + c[l - 1]);
                }
                for (int i = l - 2; i >= f + 1; i--) {  // upward
                    double r = c[i] / (s[i + 1] + a[i + 1] + c[i + 1]);
                    up[i] = r;
                    a[i] += r * a[i + 1];
                    c[i] = r * c[i + 1];
                    s[i] += r * s[i + 1];
                    bA[i] = a[i];
                    bC[i] = c[i];
                    bInv[i] = 1.0 / (s[i] + a[i] + c[i]);
                }
                R3 F = {a[f], c[f], s[f]};
                if (P >= 3) {
                    double r = c[f] / (s[f + 1] + a[f + 1] + c[f + 1]);
                    rF[k] = r;
                    F.c = r * c[f + 1];
                    F.s += r * s[f + 1];
                }
                red.push_back(F);
                red.push_back(L);
            }
        }
        const int R = (int)red.size();
        int level = 0;
        for (int sft = 1; sft < R; sft <<= 1, level++) {
            std::vector<R3> nx(R);
            for (int i = 0; i < R; i++) {
                R3 lo = i - sft >= 0 ? red[i - sft] : R3{0, 0, 1};
                R3 hi = i + sft < R ? red[i + sft] : R3{0, 0, 1};
                double rl = red[i].a / (lo.s + lo.a + lo.c), rh = red[i].c / (hi.s + hi.a + hi.c);
                pl[level * kk::S64_R + i] = rl;
                ph[level * kk::S64_R + i] = rh;
                nx[i] = {rl * lo.a, rh * hi.c, red[i].s + rl * lo.s + rh * hi.s};
            }
            red = nx;
        }
        for (int i = 0; i < R; i++) pinv[i] = 1.0 / (red[i].s + red[i].a + red[i].c);
    }
}

extern "C" int kamino_create(const kamino_config* cfg, kamino_handle* out)
{
    if (!cfg || !out) return kamino_fail(KAMINO_ERR_INVALID, "kamino_create: null argument");
    *out = nullptr;
    KGeo g;
    int rc = fill_geo(cfg, &g);
    if (rc) return rc;
    int64_t npart = kamino_particle_count(cfg);
    if (npart < 0 || npart > ((int64_t)1 << 31))
        return kamino_fail(KAMINO_ERR_INVALID, "particle count %lld out of range", (long long)npart);
    if (cfg->fp64_modes < 0) return kamino_fail(KAMINO_ERR_INVALID, "fp64_modes must be >= 0");
    int ndev = 0;
    KCUDA(cudaGetDeviceCount(&ndev));
    if (cfg->device < 0 || cfg->device >= ndev)
        return kamino_fail(KAMINO_ERR_INVALID, "device %d not present (%d devices)", cfg->device, ndev);
    KCUDA(cudaSetDevice(cfg->device));

    auto* h = new kamino_solver_s();
    h->cfg = *cfg;
    h->g = g;
    h->device = cfg->device;
    h->nfp64 = std::min(cfg->fp64_modes, g.nt);
    h->last_dt = g.dt;
    const int nt = g.nt, np = g.np;
    const size_t field = align_up(sizeof(float) * (size_t)g.rows * np);
    const size_t spec = align_up(sizeof(float2) * (size_t)nt * nt);
    const size_t part = align_up(sizeof(float2) * (size_t)std::max<int64_t>(npart, 1));
    const size_t rowf = align_up(sizeof(float) * nt), rowd = align_up(sizeof(double) * nt);
    const size_t tw = align_up(sizeof(float2) * nt), rt = align_up(sizeof(float2) * (nt + 1));
    const size_t s64 = align_up(sizeof(double) * kk::s64_stride(nt) * std::max(h->nfp64, 1));
    const size_t pint = npart > 0 ? align_up(sizeof(int) * (size_t)npart) : 0;  // visiting order, keys, new order
    const size_t pcnt = npart > 0 ? align_up(sizeof(int) * (size_t)kk::pblocks(nt)) : 0;
    size_t total = 9 * field + 2 * spec + 2 * part + 13 * rowf + 4 * rowd + tw + rt + s64 + 3 * pint + pcnt;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->arena, total);
    if (e != cudaSuccess) {
        int code = e == cudaErrorMemoryAllocation ? KAMINO_ERR_ALLOC : KAMINO_ERR_CUDA;
        kamino_destroy(h);
        return kamino_fail(code, "kamino_create: %s (%zu bytes)", cudaGetErrorString(e), total);
    }
    h->arena_bytes = total;
    char* p = (char*)h->arena;
    auto take = [&p](size_t n) {
        char* r = p;
        p += n;
        return r;
    };
    KBufs& b = h->b;
    for (int s = 0; s < 2; s++) {
        b.u[s] = (float*)take(field);
        b.v[s] = (float*)take(field);
        b.rho[s] = (float*)take(field);
        b.part[s] = (float2*)take(part);
    }
    b.cu = (float*)take(field);
    b.cv = (float*)take(field);
    b.p = (float*)take(field);
    b.spec = (float2*)take(spec);
    b.sol = (float2*)take(spec);
    b.s64 = (double*)take(s64);
    b.cof_c = (float*)take(rowf);
    b.cof_v = (float*)take(rowf);
    b.cell_c = (float*)take(rowf);
    b.cell_v = (float*)take(rowf);
    b.gfac = (float*)take(rowf);
    b.negHs = (float*)take(rowf);
    b.divf = (float*)take(rowf);
    b.sinN = (float*)take(rowf);
    b.sinS = (float*)take(rowf);
    b.lapA = (float*)take(rowf);
    b.lapC = (float*)take(rowf);
    b.lapB0 = (float*)take(rowf);
    b.lapS = (float*)take(rowf);
    b.lapA64 = (double*)take(rowd);
    b.lapC64 = (double*)take(rowd);
    b.lapB064 = (double*)take(rowd);
    b.lapS64 = (double*)take(rowd);
    b.tw = (float2*)take(tw);
    b.rt = (float2*)take(rt);
    b.npart = npart;
    if (npart > 0) {
        b.pperm = (const int*)take(pint);
        h->pkeys = (int*)take(pint);
        h->ptmp = (int*)take(pint);
        h->pcounts = (int*)take(pcnt);
    } else {
        b.pperm = nullptr;
    }

    rc = KAMINO_OK;
    do {
        e = cudaMemsetAsync(h->arena, 0, total, h->stream);
        if (e != cudaSuccess) break;
        std::vector<double> A, C, B0, S;
        laplacian_rows(nt, A, C, B0, S);
        std::vector<float> Af(A.begin(), A.end()), Cf(C.begin(), C.end()), B0f(B0.begin(), B0.end()),
            Sf(S.begin(), S.end());
        std::vector<float2> twh(nt), rth(nt + 1);
        for (int k = 0; k < nt; k++) {
            double a = -2.0 * KAMINO_PI_D * k / nt;
            twh[k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        for (int m = 0; m <= nt; m++) {
            double a = -KAMINO_PI_D * m / nt;
            rth[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        // velocity -> displacement in cells, dt / (R sin(theta) h), exact h
        std::vector<float> cellc(nt), cellv(nt);
        {
            const double hd = KAMINO_PI_D / nt;
            for (int j = 0; j < nt; j++) {
                cellc[j] = (float)(cfg->dt / (cfg->radius * std::sin((j + 0.5) * hd) * hd));
                cellv[j] = (float)(cfg->dt / (cfg->radius * std::sin((j + 1.0) * hd) * hd));
            }
        }
        std::vector<double> t64;
        if (h->nfp64 > 0) fp64_tables(nt, h->nfp64, A, C, S, t64);
        struct {
            void* d;
            const void* s;
            size_t n;
        } ups[] = {{b.lapA, Af.data(), 4 * (size_t)nt},    {b.lapC, Cf.data(), 4 * (size_t)nt},
                   {b.lapB0, B0f.data(), 4 * (size_t)nt},  {b.lapS, Sf.data(), 4 * (size_t)nt},
                   {b.lapA64, A.data(), 8 * (size_t)nt},   {b.lapC64, C.data(), 8 * (size_t)nt},
                   {b.lapB064, B0.data(), 8 * (size_t)nt}, {b.lapS64, S.data(), 8 * (size_t)nt},
                   {b.tw, twh.data(), 8 * (size_t)nt},     {b.rt, rth.data(), 8 * (size_t)(nt + 1)},
                   {b.cell_c, cellc.data(), 4 * (size_t)nt}, {b.cell_v, cellv.data(), 4 * (size_t)nt},
                   {b.s64, t64.data(), 8 * t64.size()}};
        for (auto& u : ups) {
            if (!u.n) continue;
            e = cudaMemcpyAsync(u.d, u.s, u.n, cudaMemcpyHostToDevice, h->stream);
            if (e != cudaSuccess) break;
        }
        if (e != cudaSuccess) break;
        kk::k_tables<<<(nt + 127) / 128, 128, 0, h->stream>>>(h->g, h->b);
        if (npart > 0)  // a valid visiting order from the start (rebuilt before the first step)
            kk::k_piota<<<(unsigned)((npart + 255) / 256), 256, 0, h->stream>>>(const_cast<int*>(b.pperm), npart);
        e = cudaGetLastError();
        if (e != cudaSuccess) break;
        e = cudaStreamSynchronize(h->stream);  // host vectors above go out of scope
        if (e != cudaSuccess) break;
        h->smem_div = kk::fft_smem(nt);
        h->smem_ifft = h->smem_div;
        h->smem_solve = kk::solve_smem(nt);
        e = kk::set_fft_smem_limits();
    } while (0);
    if (e != cudaSuccess) {
        rc = kamino_fail(KAMINO_ERR_CUDA, "kamino_create: %s", cudaGetErrorString(e));
        kamino_destroy(h);
        return rc;
    }
    *out = h;
    return KAMINO_OK;
}

// ----------------------------------------------------------------- launches
// Status of the launch just made (its returned status, else the last
// error), naming the kernel on failure.
static int launched(const char* name, cudaError_t ret = cudaSuccess)
{
    cudaError_t e = cudaGetLastError();
    if (ret != cudaSuccess) e = ret;
    return e == cudaSuccess ? KAMINO_OK : kamino_fail(KAMINO_ERR_CUDA, "%s launch: %s", name, cudaGetErrorString(e));
}

static int launch_advect(kamino_solver_s* h, int suv, int duv, int sr, int dr)
{
    const KGeo& g = h->g;
    const int T = kk::ADV_THREADS;
    int nb_u, nb_v, nb_r;
    kk::adv_tiles(g, nb_u, nb_v, nb_r);
    int nb_p = (int)((h->b.npart + T - 1) / T);
    const dim3 grid(nb_u + nb_v + nb_r + nb_p);
    cudaError_t e = (g.flags & KAMINO_F_REFERENCE_ROUNDING)
                        ? kk::launch_pdl(kk::k_advect<true>, grid, T, 0, h->stream, g, h->b, suv, duv, sr, dr, nb_u,
                                         nb_v, nb_r)
                        : kk::launch_pdl(kk::k_advect<false>, grid, T, 0, h->stream, g, h->b, suv, duv, sr, dr, nb_u,
                                         nb_v, nb_r);
    return launched("k_advect", e);
}

static int launch_geo(kamino_solver_s* h, int src)
{
    const KGeo& g = h->g;
    int n = kk::elem_groups(g.nt * g.np);
    cudaError_t e = kk::launch_pdl(kk::k_geo_centers, (n + kk::ELEM_THREADS - 1) / kk::ELEM_THREADS,
                                   kk::ELEM_THREADS, 0, h->stream, g, h->b, src);
    return launched("k_geo_centers", e);
}

static int launch_assign(kamino_solver_s* h, int uv_out)
{
    const KGeo& g = h->g;
    int n = g.nt * g.np;
    kk::k_assign<<<(n + kk::ELEM_THREADS - 1) / kk::ELEM_THREADS, kk::ELEM_THREADS, 0, h->stream>>>(g, h->b,
                                                                                                   uv_out);
    return launched("k_assign");
}

template <int MODE>
static int launch_div(kamino_solver_s* h, int uv_in, int uv_out)
{
    const KGeo& g = h->g;
    const int rpc = kk::fft_rows_per_cta(g.nt);
    cudaError_t e = kk::launch_pdl(kk::div_fft_kernel<MODE>(g.nt), g.nt / rpc, kk::fft_threads(g.nt), h->smem_div, h->stream, g,
                                   h->b, uv_in, uv_out);
    return launched("k_div_fft", e);
}

static int launch_solve(kamino_solver_s* h)
{
    const KGeo& g = h->g;
    cudaError_t e = kk::launch_pdl(kk::solve_kernel(g.nt), kk::solve_tiles(g.nt, h->nfp64), kk::SOLVE_THREADS,
                                   h->smem_solve, h->stream, g, h->b, h->nfp64);
    return launched("k_solve", e);
}

static int launch_ifft(kamino_solver_s* h, int uv_in, int uv_out)
{
    const KGeo& g = h->g;
    const int rpc = kk::fft_rows_per_cta(g.nt);
    cudaError_t e = kk::launch_pdl(kk::ifft_kernel(g.nt), g.nt / rpc, kk::fft_threads(g.nt), h->smem_ifft, h->stream,
                                   g, h->b, uv_in, uv_out);
    if (int rc = launched("k_ifft_u", e)) return rc;
    int n = kk::elem_groups((g.nt - 1) * g.np);
    e = kk::launch_pdl(kk::k_vgrad, (n + 2 * kk::ELEM_THREADS - 1) / (2 * kk::ELEM_THREADS), kk::ELEM_THREADS, 0, h->stream, g,
                       h->b, uv_in, uv_out);
    return launched("k_vgrad", e);
}

// Events of the step with the state in host memory (kamino_step_host): the
// advection runs as two launches, u_phi and u_theta first and the thickness
// once rho_ready (its upload) has completed; u_done is recorded when u_phi is
// final.
struct HostIo {
    cudaEvent_t rho_ready, u_done;
};

// The six launches of one step from buffer parity (cu, cr).  ev: optional
// per-kernel timing events (graph capture); after_advect: optional event
// recorded once the advection has written the step's thickness; io: the
// split advection of kamino_step_host (cell-exact sampler only).
static int enqueue_step(kamino_solver_s* h, int cu, int cr, cudaEvent_t* ev, cudaEvent_t after_advect = nullptr,
                        const HostIo* io = nullptr)
{
    cudaError_t pending = cudaGetLastError();
    if (pending != cudaSuccess)
        return kamino_fail(KAMINO_ERR_CUDA, "CUDA error pending before the step: %s", cudaGetErrorString(pending));
    int rc = KAMINO_OK;
    auto mark = [&](int k) {
        if (ev) cudaEventRecordWithFlags(ev[k], h->stream, cudaEventRecordExternal);
    };
    mark(0);
    if (!rc && io) {
        const KGeo& g = h->g;
        const int T = kk::ADV_THREADS;
        const int nb_u = (kk::adv_cell_threads(g) + T - 1) / T, nb_p = (int)((h->b.npart + T - 1) / T);
        cudaError_t e = kk::launch_pdl(kk::k_advect_part<3>, nb_u + nb_p, T, 0, h->stream, g, h->b, cu, 1 - cu, cr,
                                       1 - cr, nb_u);
        rc = launched("k_advect_part<3>", e);
        if (!rc) KCUDA(cudaStreamWaitEvent(h->stream, io->rho_ready, 0));
        if (!rc) {
            e = kk::launch_pdl(kk::k_advect_part<4>, nb_u, T, 0, h->stream, g, h->b, cu, 1 - cu, cr, 1 - cr, nb_u);
            rc = launched("k_advect_part<4>", e);
        }
    } else if (!rc) {
        rc = launch_advect(h, cu, 1 - cu, cr, 1 - cr);
    }
    if (!rc && after_advect) KCUDA(cudaEventRecord(after_advect, h->stream));
    mark(1);
    if (!rc) rc = launch_geo(h, 1 - cu);
    mark(2);
    if (!rc) rc = launch_div<0>(h, 1 - cu, cu);
    mark(3);
    if (!rc) rc = launch_solve(h);
    mark(4);
    if (!rc) {
        const KGeo& g = h->g;
        const int rpc = kk::fft_rows_per_cta(g.nt);
        cudaError_t e = kk::launch_pdl(kk::ifft_kernel(g.nt), g.nt / rpc, kk::fft_threads(g.nt), h->smem_ifft,
                                       h->stream, g, h->b, cu, 1 - cu);
        rc = launched("k_ifft_u", e);
    }
    if (!rc && io) KCUDA(cudaEventRecord(io->u_done, h->stream));
    mark(5);
    if (!rc) {
        const KGeo& g = h->g;
        int n = kk::elem_groups((g.nt - 1) * g.np);
        cudaError_t e = kk::launch_pdl(kk::k_vgrad, (n + 2 * kk::ELEM_THREADS - 1) / (2 * kk::ELEM_THREADS), kk::ELEM_THREADS,
                                       0, h->stream, g, h->b, cu, 1 - cu);
        rc = launched("k_vgrad", e);
    }
    mark(6);
    return rc;
}

static int get_graph(kamino_solver_s* h, int nsteps, cudaGraphExec_t* out)
{
    cudaGraphExec_t& ge = h->graph[nsteps - 1][h->cur_uv][h->cur_r];
    if (!ge) {
        cudaGraph_t graph = nullptr;
        KCUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = KAMINO_OK;
        int cu = h->cur_uv, cr = h->cur_r;
        for (int s = 0; s < nsteps && rc == KAMINO_OK; s++) {
            rc = enqueue_step(h, cu, cr, nullptr);
            cu ^= 1;
            cr ^= 1;
        }
        cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
        if (rc != KAMINO_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&ge, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ge = nullptr;
            return kamino_fail(KAMINO_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        }
    }
    *out = ge;
    return KAMINO_OK;
}

static int check_handle(kamino_solver_s* h)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return KAMINO_OK;
}

// Rebuilds the particles' visiting order from their current positions (a
// counting sort by block of cells, on the handle's stream) when it is due.
static int sort_particles(kamino_solver_s* h)
{
    const int64_t n = h->b.npart;
    if (n == 0 || (h->sorted_at >= 0 && h->steps - h->sorted_at < kSortEvery)) return KAMINO_OK;
    const KGeo& g = h->g;
    const int nb = kk::pblocks(g.nt), T = kk::ELEM_THREADS;
    const unsigned blocks = (unsigned)((n + T - 1) / T);
    KCUDA(cudaMemsetAsync(h->pcounts, 0, sizeof(int) * (size_t)nb, h->stream));
    kk::k_pkeys<<<blocks, T, 0, h->stream>>>(g, h->b.part[h->cur_r], h->b.pperm, n, h->pkeys, h->pcounts);
    kk::k_pscan<<<1, 1024, 0, h->stream>>>(h->pcounts, nb);
    kk::k_pscatter<<<blocks, T, 0, h->stream>>>(h->pkeys, h->b.pperm, n, h->pcounts, h->ptmp);
    KCUDA(cudaGetLastError());
    // into the buffer the step graphs read
    KCUDA(cudaMemcpyAsync(const_cast<int*>(h->b.pperm), h->ptmp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice,
                          h->stream));
    h->sorted_at = h->steps;
    return KAMINO_OK;
}

// Rebuild dt-dependent tables when KAMINO_F_HONOR_STEP_DT asks for a new dt:
// every table and constant kamino_create derives from the configured dt, so
// the step equals that of a handle created with this dt.
static int apply_dt(kamino_solver_s* h, float dt)
{
    if (!(h->g.flags & KAMINO_F_HONOR_STEP_DT) || dt == h->g.dt) return KAMINO_OK;
    if (!(dt > 0) || !std::isfinite(dt)) return kamino_fail(KAMINO_ERR_INVALID, "dt=%g must be positive", dt);
    const int nt = h->g.nt;
    const double dtd = dt, R = h->cfg.radius, hd = KAMINO_PI_D / nt;
    std::vector<float> cellc(nt), cellv(nt);
    for (int j = 0; j < nt; j++) {  // as kamino_create
        cellc[j] = (float)(dtd / (R * std::sin((j + 0.5) * hd) * hd));
        cellv[j] = (float)(dtd / (R * std::sin((j + 1.0) * hd) * hd));
    }
    h->g.dt = dt;
    h->g.cofTheta = dt / h->g.R;
    h->g.cellTheta = (float)(dtd / (R * hd));
    KCUDA(cudaMemcpyAsync(h->b.cell_c, cellc.data(), 4 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
    KCUDA(cudaMemcpyAsync(h->b.cell_v, cellv.data(), 4 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
    kk::k_tables<<<(nt + 127) / 128, 128, 0, h->stream>>>(h->g, h->b);
    KCUDA(cudaGetLastError());
    KCUDA(cudaStreamSynchronize(h->stream));  // the host tables above go out of scope
    destroy_graphs(h);
    return KAMINO_OK;
}

extern "C" int kamino_step(kamino_handle h, float dt)
{
    int rc = check_handle(h);
    if (rc) return rc;
    h->last_dt = dt;  // stored, as stepForward does (KaminoSolver.cu:199)
    rc = apply_dt(h, dt);
    if (!rc) rc = sort_particles(h);
    if (rc) return rc;
    cudaGraphExec_t ge = nullptr;
    rc = get_graph(h, 1, &ge);
    if (rc) return rc;
    KCUDA(cudaGraphLaunch(ge, h->stream));
    h->cur_uv ^= 1;
    h->cur_r ^= 1;
    h->steps++;
    h->time += h->g.dt;
    return KAMINO_OK;
}

extern "C" int kamino_step_n(kamino_handle h, int n)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0) return kamino_fail(KAMINO_ERR_INVALID, "step count %d < 0", n);
    for (int k = 0; k < n;) {
        int s = (n - k >= 2) ? 2 : 1;
        if ((rc = sort_particles(h))) return rc;
        cudaGraphExec_t ge = nullptr;
        rc = get_graph(h, s, &ge);
        if (rc) return rc;
        KCUDA(cudaGraphLaunch(ge, h->stream));
        if (s == 1) {
            h->cur_uv ^= 1;
            h->cur_r ^= 1;
        }
        h->steps += s;
        h->time += (double)h->g.dt * s;
        k += s;
    }
    return KAMINO_OK;
}

extern "C" int kamino_advection(kamino_handle h)
{
    int rc = check_handle(h);
    if (rc) return rc;
    rc = sort_particles(h);
    if (!rc) rc = launch_advect(h, h->cur_uv, 1 - h->cur_uv, h->cur_r, 1 - h->cur_r);
    if (rc) return rc;
    h->cur_uv ^= 1;
    h->cur_r ^= 1;
    return KAMINO_OK;
}

extern "C" int kamino_geometric(kamino_handle h)
{
    int rc = check_handle(h);
    if (rc) return rc;
    rc = launch_geo(h, h->cur_uv);
    if (!rc) rc = launch_assign(h, 1 - h->cur_uv);
    if (rc) return rc;
    h->cur_uv ^= 1;
    return KAMINO_OK;
}

extern "C" int kamino_projection(kamino_handle h)
{
    int rc = check_handle(h);
    if (rc) return rc;
    rc = launch_div<2>(h, h->cur_uv, 1 - h->cur_uv);
    if (!rc) rc = launch_solve(h);
    if (!rc) rc = launch_ifft(h, h->cur_uv, 1 - h->cur_uv);
    if (rc) return rc;
    h->cur_uv ^= 1;
    h->steps++;  // a full advection+geometric+projection sequence is a step
    h->time += h->g.dt;
    return KAMINO_OK;
}

extern "C" int kamino_run_frames(kamino_handle h, int frames, int64_t* steps_taken)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (frames < 0) return kamino_fail(KAMINO_ERR_INVALID, "frames=%d < 0", frames);
    int64_t total = kamino_frame_steps(h->cfg.dt, h->cfg.frame_dt, frames);
    if (total < 0) return kamino_fail(KAMINO_ERR_INVALID, "frame_dt and dt must be > 0");
    if (total > 0x7fffffff) return kamino_fail(KAMINO_ERR_INVALID, "too many steps");
    rc = kamino_step_n(h, (int)total);
    if (steps_taken) *steps_taken = total;
    return rc;
}

extern "C" int kamino_synchronize(kamino_handle h)
{
    int rc = check_handle(h);
    if (rc) return rc;
    KCUDA(cudaStreamSynchronize(h->stream));
    return KAMINO_OK;
}

// ------------------------------------------------------------ internal hooks
int kamino_internal_desc(kamino_handle h, KGeo* g, KBufs* b, int* nfp64, int* cur_uv, int* cur_r)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    if (g) *g = h->g;
    if (b) *b = h->b;
    if (nfp64) *nfp64 = h->nfp64;
    if (cur_uv) *cur_uv = h->cur_uv;
    if (cur_r) *cur_r = h->cur_r;
    return KAMINO_OK;
}

int kamino_internal_advance(kamino_handle h, int nsteps)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    if (nsteps & 1) {
        h->cur_uv ^= 1;
        h->cur_r ^= 1;
    }
    h->steps += nsteps;
    h->time += (double)h->g.dt * nsteps;
    return KAMINO_OK;
}

int kamino_internal_get_counters(kamino_handle h, int* cur_uv, int* cur_r, int64_t* steps, double* time)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    if (cur_uv) *cur_uv = h->cur_uv;
    if (cur_r) *cur_r = h->cur_r;
    if (steps) *steps = h->steps;
    if (time) *time = h->time;
    return KAMINO_OK;
}

int kamino_internal_sort_particles(kamino_handle h, int* launched)
{
    int rc = check_handle(h);
    if (rc) return rc;
    const int64_t before = h->sorted_at;
    rc = sort_particles(h);
    if (launched) *launched = h->sorted_at != before;
    return rc;
}

int kamino_internal_set_counters(kamino_handle h, int cur_uv, int cur_r, int64_t steps, double time)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    h->cur_uv = cur_uv & 1;
    h->cur_r = cur_r & 1;
    if (steps != h->steps) h->sorted_at = -1;
    h->steps = steps;
    h->time = time;
    return KAMINO_OK;
}

cudaStream_t kamino_internal_stream(kamino_handle h) { return h ? h->stream : nullptr; }

int kamino_internal_frames(kamino_handle h, KFrames*** out)
{
    int rc = check_handle(h);
    if (rc) return rc;
    *out = &h->frames;
    return KAMINO_OK;
}

int kamino_internal_config(kamino_handle h, kamino_config* cfg)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    *cfg = h->cfg;
    return KAMINO_OK;
}

int kamino_internal_reset(kamino_handle h, const kamino_config* cfg)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!cfg || cfg->n_theta != h->g.nt)
        return kamino_fail(KAMINO_ERR_INVALID, "reset needs a config with the same n_theta");
    KGeo g;
    rc = fill_geo(cfg, &g);
    if (rc) return rc;
    if (kamino_particle_count(cfg) != h->b.npart)
        return kamino_fail(KAMINO_ERR_INVALID, "reset needs the same particle count");
    h->cfg = *cfg;
    h->g = g;
    h->cur_uv = h->cur_r = 0;
    h->steps = 0;
    h->time = 0.0;
    h->last_dt = g.dt;
    h->sorted_at = -1;
    destroy_graphs(h);
    const int nt = g.nt;
    std::vector<float> cellc(nt), cellv(nt);
    const double hd = KAMINO_PI_D / nt;
    for (int j = 0; j < nt; j++) {
        cellc[j] = (float)(cfg->dt / (cfg->radius * std::sin((j + 0.5) * hd) * hd));
        cellv[j] = (float)(cfg->dt / (cfg->radius * std::sin((j + 1.0) * hd) * hd));
    }
    const size_t field = sizeof(float) * (size_t)g.rows * g.np;
    for (int s = 0; s < 2; s++) {
        KCUDA(cudaMemsetAsync(h->b.u[s], 0, field, h->stream));
        KCUDA(cudaMemsetAsync(h->b.v[s], 0, field, h->stream));
        KCUDA(cudaMemsetAsync(h->b.rho[s], 0, field, h->stream));
    }
    KCUDA(cudaMemcpyAsync(h->b.cell_c, cellc.data(), 4 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
    KCUDA(cudaMemcpyAsync(h->b.cell_v, cellv.data(), 4 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
    kk::k_tables<<<(nt + 127) / 128, 128, 0, h->stream>>>(h->g, h->b);
    KCUDA(cudaGetLastError());
    KCUDA(cudaStreamSynchronize(h->stream));
    return KAMINO_OK;
}

extern "C" int kamino_time_elapsed(kamino_handle h, double* t, int64_t* steps)
{
    if (!h) return kamino_fail(KAMINO_ERR_INVALID, "null handle");
    if (t) *t = h->time;
    if (steps) *steps = h->steps;
    return KAMINO_OK;
}

extern "C" int kamino_launches_per_step(kamino_handle) { return kNumKernels; }

extern "C" int kamino_device_bytes(kamino_handle h, size_t* bytes)
{
    if (!h || !bytes) return kamino_fail(KAMINO_ERR_INVALID, "null argument");
    *bytes = h->arena_bytes;
    return KAMINO_OK;
}

// --------------------------------------------------------------- state I/O
static int field_geometry(kamino_solver_s* h, int field, int* rows)
{
    switch (field) {
    case KAMINO_U_PHI:
    case KAMINO_THICKNESS:
    case KAMINO_PRESSURE: *rows = h->g.nt; return KAMINO_OK;
    case KAMINO_U_THETA: *rows = h->g.nt - 1; return KAMINO_OK;
    case KAMINO_PARTICLES: *rows = 0; return KAMINO_OK;
    }
    return kamino_fail(KAMINO_ERR_INVALID, "unknown field %d", field);
}

static float* field_dev(kamino_solver_s* h, int field)
{
    switch (field) {
    case KAMINO_U_PHI: return h->b.u[h->cur_uv];
    case KAMINO_U_THETA: return h->b.v[h->cur_uv];
    case KAMINO_THICKNESS: return h->b.rho[h->cur_r];
    case KAMINO_PRESSURE: return h->b.p;
    case KAMINO_PARTICLES: return (float*)h->b.part[h->cur_r];
    }
    return nullptr;
}

// bytes between device memory d and host memory hp.  (Measured on GB300: the
// copy engines reach the host link's rate; an SM copy kernel over the link is
// no faster.)
static int copy_host(kamino_solver_s* h, float* d, void* hp, size_t bytes, bool to_device)
{
    if (to_device)
        KCUDA(cudaMemcpyAsync(d, hp, bytes, cudaMemcpyHostToDevice, h->stream));
    else
        KCUDA(cudaMemcpyAsync(hp, d, bytes, cudaMemcpyDeviceToHost, h->stream));
    return KAMINO_OK;
}

static int copy_field(kamino_solver_s* h, int field, void* other, size_t pitch, bool to_device,
                      cudaMemcpyKind kind, bool sync)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!other) return kamino_fail(KAMINO_ERR_INVALID, "null buffer");
    int rows = 0;
    rc = field_geometry(h, field, &rows);
    if (rc) return rc;
    float* d = field_dev(h, field);
    if (field == KAMINO_PARTICLES && to_device) h->sorted_at = -1;  // the visiting order is rebuilt before the next step
    if (field == KAMINO_PARTICLES) {
        size_t n = sizeof(float2) * (size_t)h->b.npart;
        if (n == 0) return KAMINO_OK;
        if (kind != cudaMemcpyDeviceToDevice) {
            if ((rc = copy_host(h, d, other, n, to_device))) return rc;
        } else if (to_device) {
            KCUDA(cudaMemcpyAsync(d, other, n, kind, h->stream));
        } else {
            KCUDA(cudaMemcpyAsync(other, d, n, kind, h->stream));
        }
    } else {
        const size_t w = sizeof(float) * h->g.np;
        if (pitch == 0) pitch = w;
        if (pitch < w) return kamino_fail(KAMINO_ERR_INVALID, "pitch %zu < row bytes %zu", pitch, w);
        if (pitch == w && kind != cudaMemcpyDeviceToDevice) {  // dense rows on both sides: one linear copy
            if ((rc = copy_host(h, d, other, w * rows, to_device))) return rc;
        } else if (pitch == w) {
            if (to_device)
                KCUDA(cudaMemcpyAsync(d, other, w * rows, kind, h->stream));
            else
                KCUDA(cudaMemcpyAsync(other, d, w * rows, kind, h->stream));
        } else if (to_device)
            KCUDA(cudaMemcpy2DAsync(d, w, other, pitch, w, rows, kind, h->stream));
        else
            KCUDA(cudaMemcpy2DAsync(other, pitch, d, w, w, rows, kind, h->stream));
    }
    if (sync) KCUDA(cudaStreamSynchronize(h->stream));
    return KAMINO_OK;
}

extern "C" int kamino_set_state(kamino_handle h, int field, const float* host, size_t pitch_bytes)
{
    return copy_field(h, field, (void*)host, pitch_bytes, true, cudaMemcpyHostToDevice, true);
}

extern "C" int kamino_get_state(kamino_handle h, int field, float* host, size_t pitch_bytes)
{
    return copy_field(h, field, host, pitch_bytes, false, cudaMemcpyDeviceToHost, true);
}

// One step with the state in host memory (KaminoQuantity::copyToGPU,
// KaminoSolver::stepForward, KaminoQuantity::copyBackToCPU in one call:
// KaminoQuantity.cu:3-18, KaminoSolver.cu:197-221).  The thickness is final
// once the advection has run, so its download starts then, on a second
// stream, and overlaps the projection; u_phi and u_theta follow the step.
extern "C" int kamino_step_host(kamino_handle h, float dt, const float* u_phi_in, const float* u_theta_in,
                                const float* thickness_in, float* u_phi_out, float* u_theta_out,
                                float* thickness_out, size_t pitch_bytes)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!u_phi_in || !u_theta_in || !thickness_in || !u_phi_out || !u_theta_out || !thickness_out)
        return kamino_fail(KAMINO_ERR_INVALID, "kamino_step_host: null buffer");
    const size_t w = sizeof(float) * h->g.np;
    if (pitch_bytes == 0) pitch_bytes = w;
    if (pitch_bytes < w) return kamino_fail(KAMINO_ERR_INVALID, "pitch %zu < row bytes %zu", pitch_bytes, w);
    if (!h->io_stream) {
        KCUDA(cudaStreamCreateWithFlags(&h->io_stream, cudaStreamNonBlocking));
        for (cudaEvent_t* e : {&h->ev_adv, &h->ev_uv, &h->ev_rho, &h->ev_u})
            KCUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    h->last_dt = dt;
    if ((rc = apply_dt(h, dt)) || (rc = sort_particles(h))) return rc;
    const int rows = h->g.nt;
    auto d2h = [&](float* dst, const float* src, int nrows) {
        if (pitch_bytes == w) return cudaMemcpyAsync(dst, src, w * nrows, cudaMemcpyDeviceToHost, h->io_stream);
        return cudaMemcpy2DAsync(dst, pitch_bytes, src, w, w, nrows, cudaMemcpyDeviceToHost, h->io_stream);
    };
    const int cu = h->cur_uv, cr = h->cur_r;
    if (h->g.flags & KAMINO_F_REFERENCE_ROUNDING) {
        // one advection launch: uploads, the step, and the thickness download
        // overlapping the projection
        if ((rc = copy_field(h, KAMINO_U_PHI, (void*)u_phi_in, pitch_bytes, true, cudaMemcpyHostToDevice, false)) ||
            (rc = copy_field(h, KAMINO_U_THETA, (void*)u_theta_in, pitch_bytes, true, cudaMemcpyHostToDevice, false)) ||
            (rc = copy_field(h, KAMINO_THICKNESS, (void*)thickness_in, pitch_bytes, true, cudaMemcpyHostToDevice,
                             false)))
            return rc;
        if ((rc = enqueue_step(h, cu, cr, nullptr, h->ev_adv))) return rc;
        KCUDA(cudaStreamWaitEvent(h->io_stream, h->ev_adv, 0));
        KCUDA(d2h(thickness_out, h->b.rho[1 - cr], rows));
        h->cur_uv ^= 1;
        h->cur_r ^= 1;
        if ((rc = copy_field(h, KAMINO_U_PHI, u_phi_out, pitch_bytes, false, cudaMemcpyDeviceToHost, false)) ||
            (rc = copy_field(h, KAMINO_U_THETA, u_theta_out, pitch_bytes, false, cudaMemcpyDeviceToHost, false)))
            return rc;
    } else {
        // u_phi and u_theta go up first and their advection starts while the
        // thickness is still being copied in (on the second stream); the
        // thickness comes back during the projection and u_phi during the
        // u_theta gradient
        if ((rc = copy_field(h, KAMINO_U_PHI, (void*)u_phi_in, pitch_bytes, true, cudaMemcpyHostToDevice, false)) ||
            (rc = copy_field(h, KAMINO_U_THETA, (void*)u_theta_in, pitch_bytes, true, cudaMemcpyHostToDevice, false)))
            return rc;
        KCUDA(cudaEventRecord(h->ev_uv, h->stream));
        KCUDA(cudaStreamWaitEvent(h->io_stream, h->ev_uv, 0));
        if (pitch_bytes == w)
            KCUDA(cudaMemcpyAsync(h->b.rho[cr], thickness_in, w * rows, cudaMemcpyHostToDevice, h->io_stream));
        else
            KCUDA(cudaMemcpy2DAsync(h->b.rho[cr], w, thickness_in, pitch_bytes, w, rows, cudaMemcpyHostToDevice,
                                    h->io_stream));
        KCUDA(cudaEventRecord(h->ev_rho, h->io_stream));
        const HostIo io = {h->ev_rho, h->ev_u};
        if ((rc = enqueue_step(h, cu, cr, nullptr, h->ev_adv, &io))) return rc;
        KCUDA(cudaStreamWaitEvent(h->io_stream, h->ev_adv, 0));
        KCUDA(d2h(thickness_out, h->b.rho[1 - cr], rows));
        KCUDA(cudaStreamWaitEvent(h->io_stream, h->ev_u, 0));
        KCUDA(d2h(u_phi_out, h->b.u[1 - cu], rows));
        h->cur_uv ^= 1;
        h->cur_r ^= 1;
        if ((rc = copy_field(h, KAMINO_U_THETA, u_theta_out, pitch_bytes, false, cudaMemcpyDeviceToHost, false)))
            return rc;
    }
    h->steps++;
    h->time += h->g.dt;
    KCUDA(cudaStreamSynchronize(h->io_stream));
    KCUDA(cudaStreamSynchronize(h->stream));
    return KAMINO_OK;
}

// KaminoSolver::initialize_velocity (KaminoInitializer.cu:3-85; the
// reference's constructor calls it, KaminoSolver.cu:59): u_phi and u_theta
// from its FBM curl noise, computed on the device.
extern "C" int kamino_init_fbm(kamino_handle h)
{
    int rc = check_handle(h);
    if (rc) return rc;
    const KGeo& g = h->g;
    const int n = g.nt * g.np + (g.nt - 1) * g.np;
    kk::k_init_fbm<<<(n + 255) / 256, 256, 0, h->stream>>>(g, h->b, h->cur_uv);
    KCUDA(cudaGetLastError());
    KCUDA(cudaStreamSynchronize(h->stream));
    return KAMINO_OK;
}

extern "C" int kamino_set_state_device(kamino_handle h, int field, const float* dev, size_t pitch_bytes)
{
    return copy_field(h, field, (void*)dev, pitch_bytes, true, cudaMemcpyDeviceToDevice, false);
}

extern "C" int kamino_get_state_device(kamino_handle h, int field, float* dev, size_t pitch_bytes)
{
    return copy_field(h, field, dev, pitch_bytes, false, cudaMemcpyDeviceToDevice, false);
}

// ----------------------------------------------------------------- timing
static int ensure_flush(kamino_solver_s* h)
{
    if (h->flush) return KAMINO_OK;
    // larger than the 129 MB L2 of GB300
    h->flush_bytes = (size_t)256 << 20;
    cudaError_t e = cudaMalloc(&h->flush, h->flush_bytes);
    if (e != cudaSuccess) {
        h->flush = nullptr;
        return kamino_fail(KAMINO_ERR_ALLOC, "L2 flush buffer: %s", cudaGetErrorString(e));
    }
    return KAMINO_OK;
}

int kamino_internal_flush_l2(kamino_handle h)
{
    int rc = check_handle(h);
    if (!rc) rc = ensure_flush(h);
    if (rc) return rc;
    KCUDA(kk::flush_l2(h->flush, h->flush_bytes, 0, h->stream));
    return KAMINO_OK;
}

extern "C" int kamino_time_steps(kamino_handle h, int n, int flush_l2, double* ms_total)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n <= 0 || !ms_total) return kamino_fail(KAMINO_ERR_INVALID, "bad arguments");
    if (flush_l2 && (rc = ensure_flush(h))) return rc;
    std::vector<cudaEvent_t> ev(2 * (size_t)n, nullptr);
    for (auto& e : ev) KCUDA(cudaEventCreate(&e));
    for (int k = 0; k < n && rc == KAMINO_OK; k++) {
        if (flush_l2) KCUDA(kk::flush_l2(h->flush, h->flush_bytes, k & 0xff, h->stream));
        KCUDA(cudaEventRecord(ev[2 * k], h->stream));
        rc = kamino_step(h, h->g.dt);
        KCUDA(cudaEventRecord(ev[2 * k + 1], h->stream));
    }
    cudaError_t e = cudaStreamSynchronize(h->stream);
    double tot = 0;
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        float ms = 0;
        e = cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]);
        tot += ms;
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (rc) return rc;
    if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "timing: %s", cudaGetErrorString(e));
    *ms_total = tot;
    return KAMINO_OK;
}

extern "C" int kamino_time_kernels(kamino_handle h, int reps, int flush_l2, double* ms, int max, int* count)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (reps <= 0 || !ms) return kamino_fail(KAMINO_ERR_INVALID, "bad arguments");
    if (flush_l2 && (rc = ensure_flush(h))) return rc;
    std::vector<double> acc(kNumKernels, 0.0);
    cudaEvent_t ev[2][kNumKernels + 1];
    for (auto& row : ev)
        for (auto& e : row) KCUDA(cudaEventCreate(&e));
    if ((rc = sort_particles(h))) return rc;
    // one graph per parity, each with event nodes around every kernel
    cudaGraphExec_t ge[2][2] = {};
    for (int r = 0; r < reps && rc == KAMINO_OK; r++) {
        int cu = h->cur_uv, cr = h->cur_r;
        cudaGraphExec_t& x = ge[cu][cr];
        if (!x) {
            cudaGraph_t graph = nullptr;
            KCUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_step(h, cu, cr, ev[cu ^ cr]);
            cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
            if (rc || e != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                if (!rc) rc = kamino_fail(KAMINO_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
                break;
            }
            e = cudaGraphInstantiate(&x, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                rc = kamino_fail(KAMINO_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
                break;
            }
        }
        if (flush_l2) KCUDA(kk::flush_l2(h->flush, h->flush_bytes, r & 0xff, h->stream));
        KCUDA(cudaGraphLaunch(x, h->stream));
        KCUDA(cudaStreamSynchronize(h->stream));
        for (int k = 0; k < kNumKernels; k++) {
            float t = 0;
            KCUDA(cudaEventElapsedTime(&t, ev[cu ^ cr][k], ev[cu ^ cr][k + 1]));
            acc[k] += t;
        }
        h->cur_uv ^= 1;
        h->cur_r ^= 1;
        h->steps++;
        h->time += h->g.dt;
    }
    for (auto& a : ge)
        for (auto& x : a)
            if (x) cudaGraphExecDestroy(x);
    for (auto& row : ev)
        for (auto& e : row) cudaEventDestroy(e);
    if (rc) return rc;
    int n = std::min(max, kNumKernels);
    for (int k = 0; k < n; k++) ms[k] = acc[k] / reps;
    if (count) *count = n;
    return KAMINO_OK;
}

// ----------------------------------------------------------------- probes
extern "C" int kamino_probe_index(kamino_handle h, int kind, const float* phi, const float* theta, int64_t n,
                                  int32_t* out, float* alpha)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (kind < 0 || kind > 2 || n < 0 || (n && (!phi || !theta || !out || !alpha)))
        return kamino_fail(KAMINO_ERR_INVALID, "kamino_probe_index: bad arguments");
    if (n == 0) return KAMINO_OK;
    float *dp = nullptr, *dt = nullptr, *da = nullptr;
    int* di = nullptr;
    cudaError_t e = cudaMalloc(&dp, 4 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dt, 4 * n);
    if (e == cudaSuccess) e = cudaMalloc(&da, 8 * n);
    if (e == cudaSuccess) e = cudaMalloc(&di, 16 * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp, phi, 4 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, theta, 4 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        kk::k_probe_index<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(h->g, kind, dp, dt, n, di, da);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, di, 16 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(alpha, da, 8 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dp);
    cudaFree(dt);
    cudaFree(da);
    cudaFree(di);
    if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "kamino_probe_index: %s", cudaGetErrorString(e));
    return KAMINO_OK;
}

extern "C" int kamino_probe_wrap(kamino_handle h, float* phi, float* theta, int64_t n, int32_t* cells)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 0 || (n && (!phi || !theta || !cells)))
        return kamino_fail(KAMINO_ERR_INVALID, "kamino_probe_wrap: bad arguments");
    if (n == 0) return KAMINO_OK;
    float *dp = nullptr, *dt = nullptr;
    int* dc = nullptr;
    cudaError_t e = cudaMalloc(&dp, 4 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dt, 4 * n);
    if (e == cudaSuccess) e = cudaMalloc(&dc, 8 * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp, phi, 4 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, theta, 4 * n, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        kk::k_probe_wrap<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(h->g, dp, dt, n, dc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(phi, dp, 4 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(theta, dt, 4 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cells, dc, 8 * n, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dp);
    cudaFree(dt);
    cudaFree(dc);
    if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_CUDA, "kamino_probe_wrap: %s", cudaGetErrorString(e));
    return KAMINO_OK;
}

// --------------------------------------------------------------- host memory
extern "C" int kamino_host_alloc(size_t bytes, void** out)
{
    if (!out) return kamino_fail(KAMINO_ERR_INVALID, "null out");
    KCUDA(cudaMallocHost(out, bytes ? bytes : 1));
    return KAMINO_OK;
}

extern "C" int kamino_host_free(void* p)
{
    if (p) KCUDA(cudaFreeHost(p));
    return KAMINO_OK;
}
