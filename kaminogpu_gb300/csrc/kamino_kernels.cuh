// kamino_kernels.cuh — the per-step kernels of one sphere.
//
// One step (KaminoSolver::stepForward, KaminoSolver.cu:197-221) is six
// launches on the handle's stream, replayed from a CUDA graph:
//   k_advect      RK2 semi-Lagrangian u_phi, u_theta, thickness + particles
//                 (advection(), KaminoCore.cu:344-384)
//   k_geo_centers the metric-term solve at cell centres
//                 (geometricFillKernel, KaminoCore.cu:457-514)
//   k_div_fft     re-staggering to faces (assignPhi/ThetaKernel, :517-549),
//                 divergence (fillDivergenceKernel, :587-638) and the forward
//                 real FFT of every latitude row; writes the spectrum
//                 mode-major (replaces cuFFT INVERSE + shiftFKernel, :763-775)
//   k_solve       one CTA per Fourier mode: tridiagonal solve in theta
//                 (replaces crKernel x2, tdm.cu:3-96, :779-792); modes
//                 |m| <= fp64_modes in FP64; writes the solution row-major
//   k_ifft_u      inverse real FFT per row, pressure, u_phi gradient update
//                 (copy2UFourier .. shiftUKernel, applyPressurePhi, :796-839)
//   k_vgrad       u_theta gradient update (applyPressureTheta, :705-722)
// Fields are dense [row][nPhi] float rows with nTheta+2 rows allocated; rows
// past the data stay zero, which defines the reference's out-of-range reads.
#pragma once

#include "kamino_device.cuh"

namespace kk {
// internal linkage: every translation unit that launches these kernels
// compiles its own copy
namespace {

using namespace kdev;

constexpr int ADV_THREADS = 256;
constexpr int ELEM_THREADS = 256;
constexpr int SOLVE_THREADS = 128;  // threads per Fourier mode in k_solve (nTheta >= 128)

// ----------------------------------------------------------- per-row tables
// Evaluated on the device with the reference's own float expressions
// (sinf/cosf of the same float angles), so the tables hold exactly the values
// the reference kernels compute inline.
__global__ void k_tables(KGeo g, KBufs b)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nt) return;
    float thc = __fmul_rn((float)j + 0.5f, g.h);  // (j + centeredThetaOffset) * h
    float thv = __fmul_rn((float)j + 1.0f, g.h);  // (j + vThetaThetaOffset) * h
    float sc = sinf(thc), sv = sinf(thv);
    b.cof_c[j] = __fdiv_rn(g.dt, __fmul_rn(g.R, sc));          // KaminoCore.cu:202-203
    b.cof_v[j] = __fdiv_rn(g.dt, __fmul_rn(g.R, sv));
    b.gfac[j] = __fdiv_rn(__fmul_rn(g.dt, cosf(thc)), __fmul_rn(g.R, sc));  // :494
    b.negHs[j] = __fmul_rn(-g.h, sc);                            // :744
    b.divf[j] = __fdiv_rn(__frcp_rn(sc), g.h);                   // :625, :628
    b.sinN[j] = sinf(__fsub_rn(thc, g.halfh));                   // :606, :626
    b.sinS[j] = sinf(__fadd_rn(thc, g.halfh));                   // :605, :627
}

// --------------------------------------------------------------- advection
// Particles keep the reference's radian form in both sampler modes: their
// state is (phi, theta) in radians and validateCoord is applied to it.
__device__ __forceinline__ void advect_particle(const KGeo& g, const float* __restrict__ u,
                                                const float* __restrict__ v, float2 pos, float2& out)
{
    const bool vf = (g.flags & KAMINO_F_POLE_SIGN_FLIP) != 0;
    float posPhi = pos.x, posTheta = pos.y;
    float uPhi = sample<KIND_VPHI>(u, posPhi, posTheta, g, vf);
    float uTheta = sample<KIND_VTHETA>(v, posPhi, posTheta, g, vf);
    float latRadius = __fmul_rn(g.R, sinf(posTheta));
    float cofPhi = __fdiv_rn(g.dt, latRadius);
    float updatedTheta, updatedPhi;
    if (!(g.flags & KAMINO_F_PARTICLE_RK2)) {
        // advectionParticles, KaminoCore.cu:321-342 (forward Euler)
        updatedTheta = __fadd_rn(posTheta, __fmul_rn(uTheta, g.cofTheta));
        updatedPhi = posPhi;
        if (latRadius > 1e-7f) updatedPhi = __fadd_rn(posPhi, __fmul_rn(uPhi, cofPhi));
    } else {
        // midpoint rule in (phi, theta)
        float midTheta = __fadd_rn(posTheta, __fmul_rn(0.5f * uTheta, g.cofTheta));
        float midPhi = posPhi;
        if (latRadius > 1e-7f) midPhi = __fadd_rn(posPhi, __fmul_rn(0.5f * uPhi, cofPhi));
        wrap_coord(midPhi, midTheta, g);
        float mPhi = sample<KIND_VPHI>(u, midPhi, midTheta, g, vf);
        float mTheta = sample<KIND_VTHETA>(v, midPhi, midTheta, g, vf);
        float latMid = __fmul_rn(g.R, sinf(midTheta));
        updatedTheta = __fadd_rn(posTheta, __fmul_rn(mTheta, g.cofTheta));
        updatedPhi = posPhi;
        if (latMid > 1e-7f) updatedPhi = __fadd_rn(posPhi, __fmul_rn(mPhi, __fdiv_rn(g.dt, latMid)));
    }
    wrap_coord(updatedPhi, updatedTheta, g);
    out = make_float2(updatedPhi, updatedTheta);
}

// Tile `blk` of the advection: tiles [0, nb_u) advect u_phi, then u_theta,
// then thickness, then particles, ADV_THREADS points each; thread `tid` one
// grid point or one particle.  REF selects the reference-rounding (radian)
// sampler, otherwise the cell-exact one.
template <bool REF>
__device__ __forceinline__ void advect_tile(const KGeo& g, const KBufs& b, int suv, int duv, int sr, int dr,
                                            int nb_u, int nb_v, int nb_r, int blk, int tid)
{
    const float* __restrict__ u = b.u[suv];
    const float* __restrict__ v = b.v[suv];
    const int lg = g.log2nt + 1;  // log2(nPhi)
    if (blk < nb_u + nb_v + nb_r) {
        const int which = blk < nb_u ? 0 : (blk < nb_u + nb_v ? 1 : 2);
        const int b0 = which == 0 ? 0 : (which == 1 ? nb_u : nb_u + nb_v);
        int idx = (blk - b0) * ADV_THREADS + tid;
        if (idx >= (which == 1 ? g.nt - 1 : g.nt) * g.np) return;
        int j = idx >> lg, i = idx & g.mask;
        float val;
        if (REF) {
            if (which == 0) {
                float gPhi = __fmul_rn((float)i - 0.5f, g.h), gTheta = __fmul_rn((float)j + 0.5f, g.h);
                val = advect_point<KIND_VPHI>(u, v, u, gPhi, gTheta, __ldg(b.cof_c + j), g);
            } else if (which == 1) {
                float gPhi = __fmul_rn((float)i, g.h), gTheta = __fmul_rn((float)j + 1.0f, g.h);
                val = advect_point<KIND_VTHETA>(u, v, v, gPhi, gTheta, __ldg(b.cof_v + j), g);
            } else {
                float gPhi = __fmul_rn((float)i, g.h), gTheta = __fmul_rn((float)j + 0.5f, g.h);
                val = advect_point<KIND_CENTERED>(u, v, b.rho[sr], gPhi, gTheta, __ldg(b.cof_c + j), g);
            }
        } else {
            if (which == 0)
                val = advect_cell<KIND_VPHI>(u, v, u, i, j, __ldg(b.cell_c + j), g.cellTheta, g);
            else if (which == 1)
                val = advect_cell<KIND_VTHETA>(u, v, v, i, j, __ldg(b.cell_v + j), g.cellTheta, g);
            else
                val = advect_cell<KIND_CENTERED>(u, v, b.rho[sr], i, j, __ldg(b.cell_c + j), g.cellTheta, g);
        }
        float* dst = which == 0 ? b.u[duv] : (which == 1 ? b.v[duv] : b.rho[dr]);
        dst[idx] = val;
        return;
    }
    blk -= nb_u + nb_v + nb_r;
    int64_t k = (int64_t)blk * ADV_THREADS + tid;
    if (k >= b.npart) return;
    float2 out;
    advect_particle(g, u, v, b.part[sr][k], out);
    b.part[dr][k] = out;
}

template <bool REF>
__global__ void __launch_bounds__(ADV_THREADS) k_advect(KGeo g, KBufs b, int suv, int duv, int sr, int dr,
                                                         int nb_u, int nb_v, int nb_r)
{
    advect_tile<REF>(g, b, suv, duv, sr, dr, nb_u, nb_v, nb_r, blockIdx.x, threadIdx.x);
}

// --------------------------------------------------------------- geometric
__device__ __forceinline__ void geo_tile(const KGeo& g, const KBufs& b, int src, int idx)
{
    if (idx >= g.nt * g.np) return;
    const int lg = g.log2nt + 1;
    int j = idx >> lg, i = idx & g.mask;
    const float* __restrict__ u = b.u[src];
    const float* __restrict__ v = b.v[src];
    float uPrev = 0.5f * __fadd_rn(__ldg(u + idx), __ldg(u + (idx & ~g.mask) + ((i + 1) & g.mask)));
    float vPrev;
    if (j == 0 || j == g.nt - 1) {
        const float* vr = v + (j == 0 ? 0 : g.nt - 2) * g.np;
        vPrev = __fmaf_rn(0.75f, __ldg(vr + i), 0.25f * __ldg(vr + ((i + g.half) & g.mask)));
    } else {
        vPrev = 0.5f * __fadd_rn(__ldg(v + idx - g.np), __ldg(v + idx));
    }
    float G = __ldg(b.gfac + j);
    float uNext = geo_root(G, uPrev, vPrev);
    float vNext = __fadd_rn(vPrev, __fmul_rn(__fmul_rn(G, uNext), uNext));
    b.cu[idx] = uNext;
    b.cv[idx] = vNext;
}

__global__ void __launch_bounds__(ELEM_THREADS) k_geo_centers(KGeo g, KBufs b, int src)
{
    geo_tile(g, b, src, blockIdx.x * blockDim.x + threadIdx.x);
}

// assignPhiKernel / assignThetaKernel (KaminoCore.cu:517-549) alone, for the
// geometric stage called by itself; the fused step does this in k_div_fft.
__global__ void __launch_bounds__(ELEM_THREADS) k_assign(KGeo g, KBufs b, int uv_out)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.nt * g.np) return;
    const int lg = g.log2nt + 1;
    int j = idx >> lg, i = idx & g.mask;
    const size_t row = (size_t)j * g.np;
    b.u[uv_out][idx] = 0.5f * __fadd_rn(__ldg(b.cu + row + ((i - 1) & g.mask)), __ldg(b.cu + idx));
    if (j < g.nt - 1) b.v[uv_out][idx] = 0.5f * __fadd_rn(__ldg(b.cv + idx), __ldg(b.cv + idx + g.np));
}

// ------------------------------------------------------------ FFT (Stockham)
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// 4-point DFT in place, kernel e^{-2 pi i/4} = -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ void dft4(float2& a, float2& b, float2& c, float2& d)
{
    float2 apc = f2add(a, c), amc = f2sub(a, c), bpd = f2add(b, d), bmd = f2sub(b, d);
    float2 sb = INV ? make_float2(-bmd.y, bmd.x) : make_float2(bmd.y, -bmd.x);
    a = f2add(apc, bpd);
    c = f2sub(apc, bpd);
    b = f2add(amc, sb);
    d = f2sub(amc, sb);
}

// Complex FFT of length N (power of two, >= 16) by T = N/4 threads, Stockham
// autosort: radix-4 stages, then one radix-2 stage when log2 N is odd.
// Thread t enters holding x[t + r T], r = 0..3, and the transform ends in
// natural order in the returned shared buffer.  tw[k] = e^{-2 pi i k/N}.
template <bool INV>
__device__ __forceinline__ float2* stockham(float2 v[4], float2* bufA, float2* bufB, int N, int t,
                                            const float2* __restrict__ tw)
{
    const int T = N >> 2;
    float2* out = bufA;
    int Ns = 1, ls = 0;
    while (true) {
        if (4 * Ns <= N) {
            const int k = t & (Ns - 1);
            if (Ns > 1) {
                const int step = N >> (ls + 2);
#pragma unroll
                for (int r = 1; r < 4; r++) {
                    float2 w = __ldg(tw + r * k * step);
                    if (INV) w.y = -w.y;
                    v[r] = cmul(w, v[r]);
                }
            }
            dft4<INV>(v[0], v[1], v[2], v[3]);
            const int base = ((t - k) << 2) + k;
#pragma unroll
            for (int r = 0; r < 4; r++) out[base + r * Ns] = v[r];
            Ns <<= 2;
            ls += 2;
        } else {  // radix-2, Ns = N/2: butterflies t and t + T
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int idx = t + q * T;
                float2 w = __ldg(tw + idx);
                if (INV) w.y = -w.y;
                float2 y = cmul(w, v[q + 2]);
                out[idx] = f2add(v[q], y);
                out[idx + Ns] = f2sub(v[q], y);
            }
            Ns <<= 1;
            ls += 1;
        }
        __syncthreads();
        if (Ns >= N) return out;
#pragma unroll
        for (int r = 0; r < 4; r++) v[r] = out[t + r * T];
        out = (out == bufA) ? bufB : bufA;
    }
}

// Rows per CTA for the per-row FFT kernels: N/4 threads per row, up to 256
// threads per CTA.
__host__ __device__ inline int fft_rows_per_cta(int nt) { return nt >= 1024 ? 1 : 1024 / nt; }

// Divergence and forward real FFT of latitude rows.
// MODE 0: from cell centres, also writing u**, v** (the fused step)
// MODE 2: from face velocities (projection stage called by itself)
// Writes c_m = (1/nPhi) sum_j div_j e^{-i m phi_j}, m = 1..nt, mode-major:
// spec[(m-1)*nt + row].  c_0 (the dropped m = 0 mode) is never formed.
// Tile `blk` = rows [blk*rpc, blk*rpc + rpc) with rpc*N/4 threads.
template <int MODE>
__device__ __forceinline__ void div_fft_tile(const KGeo& g, const KBufs& b, int uv_in, int uv_out, int blk,
                                             int tid, float2* sm2)
{
    const int N = g.nt, T = N >> 2, rpc = fft_rows_per_cta(N);
    const int lr = tid / T, t = tid - lr * T;
    const int j = blk * rpc + lr;
    const int np = g.np, mask = g.mask;
    float2* bufA = sm2 + (size_t)lr * 2 * N;
    float2* bufB = bufA + N;
    const float* __restrict__ cu = b.cu;
    const float* __restrict__ cv = b.cv;
    const float* __restrict__ uf = b.u[uv_in];
    const float* __restrict__ vf = b.v[uv_in];
    float* __restrict__ uo = b.u[uv_out];
    float* __restrict__ vo = b.v[uv_out];
    const float fct = __ldg(b.divf + j), sN = __ldg(b.sinN + j), sS = __ldg(b.sinS + j);
    const size_t row = (size_t)j * np;
    float2 v[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int k = t + r * T;
        float d[2];
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int i = 2 * k + e;
            float uW, uE, vN, vS;
            if (MODE == 0) {
                float cm1 = __ldg(cu + row + ((i - 1) & mask)), c0 = __ldg(cu + row + i);
                float c1 = __ldg(cu + row + ((i + 1) & mask));
                uW = 0.5f * __fadd_rn(cm1, c0);  // assignPhiKernel, KaminoCore.cu:531-533
                uE = 0.5f * __fadd_rn(c0, c1);
                float cvj = __ldg(cv + row + i);
                vN = j > 0 ? 0.5f * __fadd_rn(__ldg(cv + row - np + i), cvj) : 0.0f;  // :546-548
                vS = j < N - 1 ? 0.5f * __fadd_rn(cvj, __ldg(cv + row + np + i)) : 0.0f;
                uo[row + i] = uW;
                if (j < N - 1) vo[row + i] = vS;
            } else {
                uW = __ldg(uf + row + i);
                uE = __ldg(uf + row + ((i + 1) & mask));
                vN = j > 0 ? __ldg(vf + row - np + i) : 0.0f;
                vS = j < N - 1 ? __ldg(vf + row + i) : 0.0f;
            }
            // fillDivergenceKernel, KaminoCore.cu:625-632
            float termTheta = __fmul_rn(fct, __fsub_rn(__fmul_rn(vS, sS), __fmul_rn(vN, sN)));
            float termPhi = __fmul_rn(fct, __fsub_rn(uE, uW));
            d[e] = __fadd_rn(termTheta, termPhi);
        }
        v[r] = make_float2(d[0], d[1]);  // z_k = f_{2k} + i f_{2k+1}
    }
    const float2* Z = stockham<false>(v, bufA, bufB, N, t, b.tw);
    // c_m = (1/nPhi)[E_m + e^{-i pi m/N} O_m], E/O from Z_m and conj(Z_{N-m});
    // pairs (m, N-m) share their inputs.
    const float scale = 1.0f / (float)np;
    for (int m = t; m <= N / 2; m += T) {
        if (m == 0) {  // c_N (real): Re Z_0 - Im Z_0
            float2 z0 = Z[0];
            b.spec[(size_t)(N - 1) * N + j] = make_float2((z0.x - z0.y) * scale, 0.0f);
            continue;
        }
        const int mb = N - m;
        float2 za = Z[m], zb = Z[mb];
        float2 wa = __ldg(b.rt + m), wb = __ldg(b.rt + mb);
        float er = 0.5f * (za.x + zb.x), ei = 0.5f * (za.y - zb.y);
        float orr = 0.5f * (za.y + zb.y), oi = -0.5f * (za.x - zb.x);
        b.spec[(size_t)(m - 1) * N + j] =
            make_float2((er + wa.x * orr - wa.y * oi) * scale, (ei + wa.x * oi + wa.y * orr) * scale);
        if (mb != m)  // (Zb, Za): E' = conj(E), O' = conj(O)
            b.spec[(size_t)(mb - 1) * N + j] =
                make_float2((er + wb.x * orr + wb.y * oi) * scale, (-ei - wb.x * oi + wb.y * orr) * scale);
    }
}

template <int MODE>
__global__ void __launch_bounds__(512) k_div_fft(KGeo g, KBufs b, int uv_in, int uv_out)
{
    extern __shared__ float2 sm2[];
    div_fft_tile<MODE>(g, b, uv_in, uv_out, blockIdx.x, threadIdx.x, sm2);
}

// ------------------------------------------------------------- mode solve
// Each Fourier mode m >= 1 of the pressure solves the reference's tridiagonal
// system (precomputeABCKernel, KaminoSolver.cu:128-159; crKernel, tdm.cu)
//   A_i x_{i-1} + B_i x_i + C_i x_{i+1} = c_i,  B_i = -(A_i + C_i + m^2/sin^2).
// Written as the M-matrix  -A x_{i-1} + P x_i - C x_{i+1} = -c  with
// P = A + C + s and the row dominance s = m^2/sin^2(theta_i) held
// explicitly, elimination and cyclic reduction only ever add non-negative
// terms (the new dominance is s_i + (A_i/P_{i-1}) s_{i-1}; the diagonal is
// recomputed as s + |couplings|).  Nothing cancels, so FP32 keeps high
// relative accuracy for every mode; the direct FP32 forms lose about
// cond(T) ~ nTheta^2/m^2 ulps on the low modes.
//
// FP32 modes: SOLVE_THREADS threads per mode, P = nTheta/SOLVE_THREADS rows
// per thread in registers.  Each thread eliminates inside its block so the
// interior rows couple only to the block's first and last unknowns; those
// 2*SOLVE_THREADS rows form a tridiagonal M-matrix solved by parallel cyclic
// reduction in shared memory.  FP64 modes: one warp, multipliers
// precomputed in FP64 on the host (the matrix is fixed), so the device only
// runs the right-hand-side recurrences.
template <typename T>
struct Row {
    T a, c, s, dr, di;  // couplings (>= 0), dominance (>= 0), right-hand side
};

__device__ __forceinline__ float rcpf(float x) { return __frcp_rn(x); }

// One cyclic-reduction step of row x with its neighbours lo (-s) and hi (+s).
__device__ __forceinline__ Row<float> pcr_combine(const Row<float>& x, const Row<float>& lo, const Row<float>& hi)
{
    float rl = x.a * rcpf(lo.s + lo.a + lo.c);
    float rh = x.c * rcpf(hi.s + hi.a + hi.c);
    Row<float> o;
    o.a = rl * lo.a;
    o.c = rh * hi.c;
    o.s = x.s + rl * lo.s + rh * hi.s;
    o.dr = x.dr + rl * lo.dr + rh * hi.dr;
    o.di = x.di + rl * lo.di + rh * hi.di;
    return o;
}

// Shared-memory PCR over R rows (R a power of two); thread t owns rows
// t*Q .. t*Q+Q-1.  Every thread of the CTA calls it (it synchronises);
// threads with active == false own no rows.
template <int Q>
__device__ __forceinline__ void pcr_smem(Row<float> (&r)[Q], Row<float>* rs, int R, int t, bool active)
{
    for (int s = 1; s < R; s <<= 1) {
        if (active) {
#pragma unroll
            for (int e = 0; e < Q; e++) rs[t * Q + e] = r[e];
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < Q; e++) {
            if (!active) break;
            const int i = t * Q + e;
            Row<float> lo, hi;
            if (i - s >= 0) {
                lo = rs[i - s];
            } else {
                lo.a = lo.c = lo.dr = lo.di = 0.0f;
                lo.s = 1.0f;
            }
            if (i + s < R) {
                hi = rs[i + s];
            } else {
                hi.a = hi.c = hi.dr = hi.di = 0.0f;
                hi.s = 1.0f;
            }
            r[e] = pcr_combine(r[e], lo, hi);
        }
        __syncthreads();
    }
}

// FP32 solve of mode m by one CTA: thread t owns rows [t P, t P + P).  With
// P == 1 the CTA may be wider than nt (threads t >= nt only synchronise);
// with P >= 2 it has exactly nt / P threads.
template <int P>
__device__ void solve_mode32(const KGeo& g, const KBufs& b, int m, Row<float>* rs, int t)
{
    const int n = g.nt;
    const float m2 = (float)m * (float)m;
    const float2* __restrict__ col = b.spec + (size_t)(m - 1) * n;
    float2* __restrict__ sol = b.sol + (m - 1);  // sol[row * n + m - 1]
    if (P == 1) {
        const bool active = t < n;
        Row<float> r[1];
        if (active) {
            r[0].a = __ldg(b.lapA + t);
            r[0].c = __ldg(b.lapC + t);
            r[0].s = m2 * __ldg(b.lapS + t);
            float2 d = col[t];
            r[0].dr = -d.x;
            r[0].di = -d.y;
        }
        pcr_smem<1>(r, rs, n, t, active);
        if (active) {
            float inv = rcpf(r[0].s + r[0].a + r[0].c);
            sol[(size_t)t * n] = make_float2(r[0].dr * inv, r[0].di * inv);
        }
        return;
    }
    const int f = t * P;
    float A[P], C[P], S[P], Dr[P], Di[P];
#pragma unroll
    for (int q = 0; q < P; q++) {
        A[q] = __ldg(b.lapA + f + q);
        C[q] = __ldg(b.lapC + f + q);
        S[q] = m2 * __ldg(b.lapS + f + q);
        float2 d = col[f + q];
        Dr[q] = -d.x;
        Di[q] = -d.y;
    }
    // downward: rows q >= 2 couple x_f instead of x_{q-1}
#pragma unroll
    for (int q = 2; q < P; q++) {
        float r = A[q] * rcpf(S[q - 1] + A[q - 1] + C[q - 1]);
        A[q] = r * A[q - 1];
        S[q] += r * S[q - 1];
        Dr[q] += r * Dr[q - 1];
        Di[q] += r * Di[q - 1];
    }
    Row<float> rr[2];
    rr[1].a = A[P - 1];
    rr[1].c = C[P - 1];
    rr[1].s = S[P - 1];
    rr[1].dr = Dr[P - 1];
    rr[1].di = Di[P - 1];
    // upward: rows P-3 .. 1 couple x_f and x_l
#pragma unroll
    for (int q = P - 3; q >= 1; q--) {
        float r = C[q] * rcpf(S[q + 1] + A[q + 1] + C[q + 1]);
        A[q] += r * A[q + 1];
        C[q] = r * C[q + 1];
        S[q] += r * S[q + 1];
        Dr[q] += r * Dr[q + 1];
        Di[q] += r * Di[q + 1];
    }
    rr[0].a = A[0];
    rr[0].c = C[0];
    rr[0].s = S[0];
    rr[0].dr = Dr[0];
    rr[0].di = Di[0];
    if (P >= 3) {
        float r = C[0] * rcpf(S[1] + A[1] + C[1]);
        rr[0].c = r * C[1];
        rr[0].s += r * S[1];
        rr[0].dr += r * Dr[1];
        rr[0].di += r * Di[1];
    }
    pcr_smem<2>(rr, rs, 2 * (n / P), t, true);
    float iF = rcpf(rr[0].s + rr[0].a + rr[0].c), iL = rcpf(rr[1].s + rr[1].a + rr[1].c);
    const float xfr = rr[0].dr * iF, xfi = rr[0].di * iF, xlr = rr[1].dr * iL, xli = rr[1].di * iL;
    sol[(size_t)f * n] = make_float2(xfr, xfi);
    sol[(size_t)(f + P - 1) * n] = make_float2(xlr, xli);
#pragma unroll
    for (int q = 1; q < P - 1; q++) {
        float inv = rcpf(S[q] + A[q] + C[q]);
        sol[(size_t)(f + q) * n] =
            make_float2((Dr[q] + A[q] * xfr + C[q] * xlr) * inv, (Di[q] + A[q] * xfi + C[q] * xli) * inv);
    }
}

// Layout of the FP64 multiplier tables of one mode (host-built by
// fp64_tables() in kamino_solver.cu): per row dn, up, bA, bC, bInv, then
// rF[32], pl[6][64], ph[6][64], pinv[64].
__host__ __device__ inline size_t s64_stride(int nt) { return 5 * (size_t)nt + 32 + 2 * 6 * 64 + 64; }

// FP64 solve of mode m by one warp: lane k owns rows [k P, k P + P), P =
// nt/32 (one row per lane when nt == 32).  Only the right-hand side is
// carried; every multiplier comes from the tables.
__device__ void solve_mode64(const KGeo& g, const KBufs& b, int m, double* sdr, double* sdi)
{
    const int n = g.nt, lane = threadIdx.x & 31;
    const int P = n >> 5;
    const double* tb = b.s64 + (size_t)(m - 1) * s64_stride(n);
    const double *dn = tb, *up = tb + n, *bA = tb + 2 * n, *bC = tb + 3 * n, *bInv = tb + 4 * n;
    const double *rF = tb + 5 * n, *pl = rF + 32, *ph = pl + 6 * 64, *pinv = ph + 6 * 64;
    const float2* __restrict__ col = b.spec + (size_t)(m - 1) * n;
    float2* __restrict__ sol = b.sol + (m - 1);
    auto pidx = [P](int r) { return r + r / P; };
    for (int r = lane; r < n; r += 32) {
        float2 d = col[r];
        sdr[pidx(r)] = -(double)d.x;
        sdi[pidx(r)] = -(double)d.y;
    }
    __syncwarp();
    const int R = P == 1 ? 32 : 64;
    double Fr, Fi, Lr = 0, Li = 0;
    const int f = lane * P, l = f + P - 1;
    if (P == 1) {
        Fr = sdr[pidx(f)];
        Fi = sdi[pidx(f)];
    } else {
        for (int i = f + 2; i <= l; i++) {
            double r = dn[i];
            sdr[pidx(i)] += r * sdr[pidx(i - 1)];
            sdi[pidx(i)] += r * sdi[pidx(i - 1)];
        }
        Lr = sdr[pidx(l)];
        Li = sdi[pidx(l)];
        for (int i = l - 2; i >= f + 1; i--) {
            double r = up[i];
            sdr[pidx(i)] += r * sdr[pidx(i + 1)];
            sdi[pidx(i)] += r * sdi[pidx(i + 1)];
        }
        Fr = sdr[pidx(f)];
        Fi = sdi[pidx(f)];
        if (P >= 3) {
            Fr += rF[lane] * sdr[pidx(f + 1)];
            Fi += rF[lane] * sdi[pidx(f + 1)];
        }
    }
    // cyclic reduction on the right-hand sides of the R boundary rows
    // (row 2k = F, 2k+1 = L of lane k; one row per lane when R = 32)
    int level = 0;
    for (int s = 1; s < R; s <<= 1, level++) {
        const double* L0 = pl + level * 64;
        const double* H0 = ph + level * 64;
        if (R == 32) {
            double lr = __shfl_up_sync(0xffffffffu, Fr, s), li = __shfl_up_sync(0xffffffffu, Fi, s);
            double hr = __shfl_down_sync(0xffffffffu, Fr, s), hi = __shfl_down_sync(0xffffffffu, Fi, s);
            if (lane < s) lr = li = 0.0;
            if (lane + s >= 32) hr = hi = 0.0;
            Fr += L0[lane] * lr + H0[lane] * hr;
            Fi += L0[lane] * li + H0[lane] * hi;
            continue;
        }
        double lFr, lFi, hFr, hFi, lLr, lLi, hLr, hLi;  // neighbours of F (row 2k) and L (row 2k+1)
        if (s == 1) {
            lFr = __shfl_up_sync(0xffffffffu, Lr, 1);
            lFi = __shfl_up_sync(0xffffffffu, Li, 1);
            hLr = __shfl_down_sync(0xffffffffu, Fr, 1);
            hLi = __shfl_down_sync(0xffffffffu, Fi, 1);
            if (lane == 0) lFr = lFi = 0.0;
            if (lane == 31) hLr = hLi = 0.0;
            hFr = Lr;
            hFi = Li;
            lLr = Fr;
            lLi = Fi;
        } else {
            const int t = s >> 1;
            lFr = __shfl_up_sync(0xffffffffu, Fr, t);
            lFi = __shfl_up_sync(0xffffffffu, Fi, t);
            hFr = __shfl_down_sync(0xffffffffu, Fr, t);
            hFi = __shfl_down_sync(0xffffffffu, Fi, t);
            lLr = __shfl_up_sync(0xffffffffu, Lr, t);
            lLi = __shfl_up_sync(0xffffffffu, Li, t);
            hLr = __shfl_down_sync(0xffffffffu, Lr, t);
            hLi = __shfl_down_sync(0xffffffffu, Li, t);
            if (lane < t) lFr = lFi = lLr = lLi = 0.0;
            if (lane + t >= 32) hFr = hFi = hLr = hLi = 0.0;
        }
        const int iF = 2 * lane, iL = iF + 1;
        double nFr = Fr + L0[iF] * lFr + H0[iF] * hFr, nFi = Fi + L0[iF] * lFi + H0[iF] * hFi;
        double nLr = Lr + L0[iL] * lLr + H0[iL] * hLr, nLi = Li + L0[iL] * lLi + H0[iL] * hLi;
        Fr = nFr;
        Fi = nFi;
        Lr = nLr;
        Li = nLi;
    }
    if (P == 1) {
        double iv = pinv[lane];
        sol[(size_t)f * n] = make_float2((float)(Fr * iv), (float)(Fi * iv));
        return;
    }
    const double xfr = Fr * pinv[2 * lane], xfi = Fi * pinv[2 * lane];
    const double xlr = Lr * pinv[2 * lane + 1], xli = Li * pinv[2 * lane + 1];
    sol[(size_t)f * n] = make_float2((float)xfr, (float)xfi);
    sol[(size_t)l * n] = make_float2((float)xlr, (float)xli);
    for (int i = f + 1; i <= l - 1; i++) {
        double iv = bInv[i];
        double xr = (sdr[pidx(i)] + bA[i] * xfr + bC[i] * xlr) * iv;
        double xi = (sdi[pidx(i)] + bA[i] * xfi + bC[i] * xli) * iv;
        sol[(size_t)i * n] = make_float2((float)xr, (float)xi);
    }
}

// Mode blk + 1: FP64 (warp 0) when blk < nfp64, otherwise FP32 with P rows
// per thread (P is a runtime value here; the batched kernels mix sizes).
__device__ __forceinline__ void solve_tile_p(const KGeo& g, const KBufs& b, int nfp64, int blk, int tid,
                                             unsigned char* smraw, int P)
{
    if (blk < nfp64) {  // FP64 mode, warp 0; the other threads have nothing to do
        if (tid >= 32) return;
        double* base = reinterpret_cast<double*>(smraw);
        const int stride = g.nt + 32;
        solve_mode64(g, b, blk + 1, base, base + stride);
        return;
    }
    Row<float>* rs = reinterpret_cast<Row<float>*>(smraw);
    switch (P) {
    case 1: solve_mode32<1>(g, b, blk + 1, rs, tid); break;
    case 2: solve_mode32<2>(g, b, blk + 1, rs, tid); break;
    case 4: solve_mode32<4>(g, b, blk + 1, rs, tid); break;
    case 8: solve_mode32<8>(g, b, blk + 1, rs, tid); break;
    default: solve_mode32<16>(g, b, blk + 1, rs, tid); break;
    }
}

template <int P>
__global__ void __launch_bounds__(SOLVE_THREADS) k_solve(KGeo g, KBufs b, int nfp64)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    if ((int)blockIdx.x < nfp64) {
        if (threadIdx.x >= 32) return;
        double* base = reinterpret_cast<double*>(smraw);
        const int stride = g.nt + 32;
        solve_mode64(g, b, blockIdx.x + 1, base, base + stride);
        return;
    }
    solve_mode32<P>(g, b, (int)blockIdx.x + 1, reinterpret_cast<Row<float>*>(smraw), threadIdx.x);
}

// ---------------------------------------------------- inverse FFT + u update
// p_j = sum_{m=1}^{nt-1} 2 Re(U_m e^{i m phi_j}) + U_nt (-1)^j: the m = 0
// mode is never synthesised, which is exactly the reference's subtraction of
// the cached zero component (cacheZeroComponents / shiftUKernel,
// KaminoCore.cu:672-703).  Through a length-nt complex FFT of
// Y_m = (X_m + X_{m+nt}) + i (X_m - X_{m+nt}) e^{i pi m/nt}, X the Hermitian
// spectrum, whose output is z_k = p_{2k} + i p_{2k+1}.
__device__ __forceinline__ void ifft_tile(const KGeo& g, const KBufs& b, int uv_in, int uv_out, int blk, int tid,
                                          float2* sm2)
{
    const int N = g.nt, T = N >> 2, rpc = fft_rows_per_cta(N);
    const int lr = tid / T, t = tid - lr * T;
    const int j = blk * rpc + lr;
    const int np = g.np, mask = g.mask;
    float2* bufA = sm2 + (size_t)lr * 2 * N;
    float2* bufB = bufA + N;
    const float2* __restrict__ U = b.sol + (size_t)j * N;  // U[m-1] = U_m
    float2 v[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int m = t + r * T;
        if (m == 0) {
            float un = __ldg(&U[N - 1].x);  // X_nt = U_nt, real
            v[r] = make_float2(un, -un);
            continue;
        }
        float2 ua = __ldg(U + m - 1), ub = __ldg(U + N - m - 1);  // X_m, and X_{m+nt} = conj(U_{nt-m})
        float2 ea = __ldg(b.rt + m);
        float Er = ua.x + ub.x, Ei = ua.y - ub.y, Dr = ua.x - ub.x, Di = ua.y + ub.y;
        float Or = Dr * ea.x + Di * ea.y, Oi = Di * ea.x - Dr * ea.y;  // D * e^{+i pi m/nt}
        v[r] = make_float2(Er - Oi, Ei + Or);
    }
    const float2* Z = stockham<true>(v, bufA, bufB, N, t, b.tw);
    const float* pr = reinterpret_cast<const float*>(Z);
    const float* __restrict__ uf = b.u[uv_in];
    float* __restrict__ uo = b.u[uv_out];
    const float nhs = __ldg(b.negHs + j);
    const size_t row = (size_t)j * np;
    for (int i = t; i < np; i += T) {
        float pc = pr[i], pw = pr[(i - 1) & mask];
        // applyPressurePhi, KaminoCore.cu:740-746
        uo[row + i] = __fadd_rn(__ldg(uf + row + i), __fdiv_rn(__fsub_rn(pc, pw), nhs));
        b.p[row + i] = pc;
    }
}

__global__ void __launch_bounds__(512) k_ifft_u(KGeo g, KBufs b, int uv_in, int uv_out, int write_p)
{
    extern __shared__ float2 sm2[];
    ifft_tile(g, b, uv_in, uv_out, blockIdx.x, threadIdx.x, sm2);
    (void)write_p;
}

// applyPressureTheta (KaminoCore.cu:716-721): v -= (p[j+1] - p[j]) / h
__device__ __forceinline__ void vgrad_tile(const KGeo& g, const KBufs& b, int uv_in, int uv_out, int idx)
{
    if (idx >= (g.nt - 1) * g.np) return;
    float pn = __ldg(b.p + idx), ps = __ldg(b.p + idx + g.np);
    b.v[uv_out][idx] = __fadd_rn(__ldg(b.v[uv_in] + idx), __fdiv_rn(__fsub_rn(ps, pn), -g.h));
}

__global__ void __launch_bounds__(ELEM_THREADS) k_vgrad(KGeo g, KBufs b, int uv_in, int uv_out)
{
    vgrad_tile(g, b, uv_in, uv_out, blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------------------------- probes
__global__ void k_probe_index(KGeo g, int kind, const float* phi, const float* theta, int64_t n, int* out,
                              float* alpha)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    SampleIndex s;
    if (kind == KIND_VPHI)
        s = sample_index<KIND_VPHI>(phi[k], theta[k], g);
    else if (kind == KIND_VTHETA)
        s = sample_index<KIND_VTHETA>(phi[k], theta[k], g);
    else
        s = sample_index<KIND_CENTERED>(phi[k], theta[k], g);
    out[4 * k] = s.ip;
    out[4 * k + 1] = s.it;
    out[4 * k + 2] = s.flipped ? 1 : 0;
    out[4 * k + 3] = s.pole ? 1 : 0;
    alpha[2 * k] = s.ap;
    alpha[2 * k + 1] = s.at;
}

__global__ void k_probe_wrap(KGeo g, float* phi, float* theta, int64_t n, int* cells)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float p = phi[k], t = theta[k];
    wrap_coord(p, t, g);
    phi[k] = p;
    theta[k] = t;
    // KaminoParticles.cu:56-57: std::floor(phi / gridLen) in fReal
    cells[2 * k] = (int)floorf(__fdiv_rn(p, g.h));
    cells[2 * k + 1] = (int)floorf(__fdiv_rn(t, g.h));
}

} // namespace
} // namespace kk
