// kamino_kernels.cuh — the per-step kernels of one sphere.
//
// One step (KaminoSolver::stepForward, KaminoSolver.cu:197-221) is five
// launches on the handle's stream, replayed from a CUDA graph:
//   k_advect      RK2 semi-Lagrangian u_phi, u_theta, thickness + particles
//                 (advection(), KaminoCore.cu:344-384)
//   k_geo_centers the metric-term solve at cell centres
//                 (geometricFillKernel, KaminoCore.cu:457-514)
//   k_div_fft     re-staggering to faces (assignPhi/ThetaKernel, :517-549),
//                 divergence (fillDivergenceKernel, :587-638) and the forward
//                 real FFT of every latitude row; writes the spectrum
//                 mode-major (replaces cuFFT INVERSE + shiftFKernel, :763-775)
//   k_solve       one warp per Fourier mode: partitioned tridiagonal solve
//                 in theta (replaces crKernel x2, tdm.cu:3-96, :779-792);
//                 modes |m| <= fp64_modes in FP64
//   k_ifft_grad   inverse real FFT per row and the pressure gradient
//                 (copy2UFourier .. applyPressurePhi, :796-839)
// Fields are dense [row][nPhi] float rows with nTheta+2 rows allocated; rows
// past the data stay zero, which defines the reference's out-of-range reads.
#pragma once

#include "kamino_device.cuh"

namespace kk {

using namespace kdev;

constexpr int ADV_THREADS = 256;
constexpr int FFT_ROWS = 4;      // latitude rows per CTA in k_div_fft / k_ifft_grad
constexpr int SOLVE_WARPS = 4;   // modes per CTA in k_solve

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

// Blocks [0, nb_u) advect u_phi, then u_theta, then thickness, then
// particles; each thread one grid point or one particle.
__global__ void __launch_bounds__(ADV_THREADS) k_advect(KGeo g, KBufs b, int suv, int duv, int sr, int dr,
                                                         int nb_u, int nb_v, int nb_r)
{
    const float* __restrict__ u = b.u[suv];
    const float* __restrict__ v = b.v[suv];
    int blk = blockIdx.x;
    const int lg = g.log2nt + 1;  // log2(nPhi)
    if (blk < nb_u) {
        int idx = blk * ADV_THREADS + threadIdx.x;
        if (idx >= g.nt * g.np) return;
        int j = idx >> lg, i = idx & g.mask;
        float gPhi = __fmul_rn((float)i - 0.5f, g.h), gTheta = __fmul_rn((float)j + 0.5f, g.h);
        b.u[duv][idx] = advect_point<KIND_VPHI>(u, v, u, gPhi, gTheta, __ldg(b.cof_c + j), g);
        return;
    }
    blk -= nb_u;
    if (blk < nb_v) {
        int idx = blk * ADV_THREADS + threadIdx.x;
        if (idx >= (g.nt - 1) * g.np) return;
        int j = idx >> lg, i = idx & g.mask;
        float gPhi = __fmul_rn((float)i, g.h), gTheta = __fmul_rn((float)j + 1.0f, g.h);
        b.v[duv][idx] = advect_point<KIND_VTHETA>(u, v, v, gPhi, gTheta, __ldg(b.cof_v + j), g);
        return;
    }
    blk -= nb_v;
    if (blk < nb_r) {
        int idx = blk * ADV_THREADS + threadIdx.x;
        if (idx >= g.nt * g.np) return;
        int j = idx >> lg, i = idx & g.mask;
        float gPhi = __fmul_rn((float)i, g.h), gTheta = __fmul_rn((float)j + 0.5f, g.h);
        b.rho[dr][idx] = advect_point<KIND_CENTERED>(u, v, b.rho[sr], gPhi, gTheta, __ldg(b.cof_c + j), g);
        return;
    }
    blk -= nb_r;
    int64_t k = (int64_t)blk * ADV_THREADS + threadIdx.x;
    if (k >= b.npart) return;
    float2 out;
    advect_particle(g, u, v, b.part[sr][k], out);
    b.part[dr][k] = out;
}

// --------------------------------------------------------------- geometric
__global__ void __launch_bounds__(256) k_geo_centers(KGeo g, KBufs b, int src)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.nt * g.np) return;
    const int lg = g.log2nt + 1;
    int j = idx >> lg, i = idx & g.mask;
    const float* __restrict__ u = b.u[src];
    const float* __restrict__ v = b.v[src];
    float uPrev = 0.5f * __fadd_rn(__ldg(u + idx), __ldg(u + (idx & ~g.mask) + ((i + 1) & g.mask)));
    float vPrev;
    if (j == 0 || j == g.nt - 1) {
        const float* vr = v + (size_t)(j == 0 ? 0 : g.nt - 2) * g.np;
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

// ------------------------------------------------------- divergence + FFT
// MODE 0: from centres: write u**, v** and the spectrum (fused step)
// MODE 1: from centres: write u**, v** only (geometric stage alone)
// MODE 2: from faces: spectrum of the divergence of (u, v) (projection alone)
template <int MODE>
__global__ void __launch_bounds__(32 * FFT_ROWS) k_div_fft(KGeo g, KBufs b, int uv_in, int uv_out)
{
    extern __shared__ float2 sm2[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = blockIdx.x * FFT_ROWS, j = r0 + warp;
    const int nt = g.nt, np = g.np, mask = g.mask;
    float2* buf = sm2 + warp * (nt + 1);
    const float* __restrict__ cu = b.cu;
    const float* __restrict__ cv = b.cv;
    const float* __restrict__ uf = b.u[uv_in];
    const float* __restrict__ vf = b.v[uv_in];
    float* __restrict__ uo = b.u[uv_out];
    float* __restrict__ vo = b.v[uv_out];
    const float fct = __ldg(b.divf + j), sN = __ldg(b.sinN + j), sS = __ldg(b.sinS + j);
    const size_t row = (size_t)j * np;
    for (int k = lane; k < nt; k += 32) {
        float d[2];
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int i = 2 * k + e;
            float uW, uE, vN, vS;
            if (MODE != 2) {
                float cm1 = __ldg(cu + row + ((i - 1) & mask)), c0 = __ldg(cu + row + i);
                float c1 = __ldg(cu + row + ((i + 1) & mask));
                uW = 0.5f * __fadd_rn(cm1, c0);  // assignPhiKernel, KaminoCore.cu:531-533
                uE = 0.5f * __fadd_rn(c0, c1);
                float cvj = __ldg(cv + row + i);
                vN = j > 0 ? 0.5f * __fadd_rn(__ldg(cv + row - np + i), cvj) : 0.0f;  // :546-548
                vS = j < nt - 1 ? 0.5f * __fadd_rn(cvj, __ldg(cv + row + np + i)) : 0.0f;
                uo[row + i] = uW;
                if (j < nt - 1) vo[row + i] = vS;
            } else {
                uW = __ldg(uf + row + i);
                uE = __ldg(uf + row + ((i + 1) & mask));
                vN = j > 0 ? __ldg(vf + row - np + i) : 0.0f;
                vS = j < nt - 1 ? __ldg(vf + row + i) : 0.0f;
            }
            // fillDivergenceKernel, KaminoCore.cu:625-632
            float termTheta = __fmul_rn(fct, __fsub_rn(__fmul_rn(vS, sS), __fmul_rn(vN, sN)));
            float termPhi = __fmul_rn(fct, __fsub_rn(uE, uW));
            d[e] = __fadd_rn(termTheta, termPhi);
        }
        if (MODE != 1) buf[bitrev(k, g.log2nt)] = make_float2(d[0], d[1]);
    }
    if (MODE == 1) return;
    __syncwarp();
    fft_dit_warp<false>(buf, nt, g.log2nt, b.tw, lane);
    // Real-FFT unpacking: c_m = (1/nPhi) [E_m + e^{-i pi m/nt} O_m] with
    // E, O from Z_m and conj(Z_{nt-m}).  Pairs (m, nt-m) are updated in place
    // by one lane; c_nt (real) goes to slot 0 whose c_0 is never used.
    const float scale = 1.0f / (float)np;
    for (int m = lane; m <= nt / 2; m += 32) {
        if (m == 0) {
            float2 z0 = buf[0];
            buf[0] = make_float2((z0.x - z0.y) * scale, 0.0f);
            continue;
        }
        const int mb = nt - m;
        float2 za = buf[m], zb = buf[mb];
        float2 wa = __ldg(b.rt + m), wb = __ldg(b.rt + mb);
        float er = 0.5f * (za.x + zb.x), ei = 0.5f * (za.y - zb.y);
        float orr = 0.5f * (za.y + zb.y), oi = -0.5f * (za.x - zb.x);
        buf[m] = make_float2((er + wa.x * orr - wa.y * oi) * scale, (ei + wa.x * oi + wa.y * orr) * scale);
        if (mb != m) {
            // (Zb, Za) pair: E' = conj(E), O' = conj(O)
            float er2 = er, ei2 = -ei, or2 = orr, oi2 = -oi;
            buf[mb] = make_float2((er2 + wb.x * or2 - wb.y * oi2) * scale,
                                  (ei2 + wb.x * oi2 + wb.y * or2) * scale);
        }
    }
    __syncthreads();
    // mode-major store: spec[(m-1)*nt + row], FFT_ROWS rows per 32-byte run
    for (int t = threadIdx.x; t < nt * FFT_ROWS; t += blockDim.x) {
        int mi = t / FFT_ROWS, r = t - mi * FFT_ROWS;
        b.spec[(size_t)mi * nt + r0 + r] = sm2[r * (nt + 1) + ((mi + 1) & (nt - 1))];
    }
}

// ------------------------------------------------------------- mode solve
// Normalised rows a_i x_{i-1} + x_i + c_i x_{i+1} = d_i (complex d).  A lane
// owns P = nt/32 consecutive rows.  Eliminating inside the block leaves each
// interior row coupled only to the block's first and last unknowns, and
// those first/last rows form a tridiagonal system of 64 unknowns (two per
// lane) solved by parallel cyclic reduction over warp shuffles.
template <typename T>
struct Row {
    T a, c, dr, di;
};

template <typename T>
__device__ __forceinline__ Row<T> shfl_row_up(const Row<T>& r, int s, int lane)
{
    Row<T> o;
    o.a = __shfl_up_sync(0xffffffffu, r.a, s);
    o.c = __shfl_up_sync(0xffffffffu, r.c, s);
    o.dr = __shfl_up_sync(0xffffffffu, r.dr, s);
    o.di = __shfl_up_sync(0xffffffffu, r.di, s);
    if (lane < s) o.a = o.c = o.dr = o.di = T(0);
    return o;
}

template <typename T>
__device__ __forceinline__ Row<T> shfl_row_down(const Row<T>& r, int s, int lane)
{
    Row<T> o;
    o.a = __shfl_down_sync(0xffffffffu, r.a, s);
    o.c = __shfl_down_sync(0xffffffffu, r.c, s);
    o.dr = __shfl_down_sync(0xffffffffu, r.dr, s);
    o.di = __shfl_down_sync(0xffffffffu, r.di, s);
    if (lane + s >= 32) o.a = o.c = o.dr = o.di = T(0);
    return o;
}

// One PCR reduction of row x with its neighbours at -s (lo) and +s (hi).
template <typename T>
__device__ __forceinline__ Row<T> pcr_combine(const Row<T>& x, const Row<T>& lo, const Row<T>& hi)
{
    T diag = T(1) - x.a * lo.c - x.c * hi.a;
    T inv = T(1) / diag;
    Row<T> o;
    o.a = -x.a * lo.a * inv;
    o.c = -x.c * hi.c * inv;
    o.dr = (x.dr - x.a * lo.dr - x.c * hi.dr) * inv;
    o.di = (x.di - x.a * lo.di - x.c * hi.di) * inv;
    return o;
}

template <typename T>
__device__ void solve_mode(const KGeo& g, const KBufs& b, int m, T* sa, T* sc, T* sdr, T* sdi, int lane)
{
    const int n = g.nt;
    const int P = n > 32 ? n >> 5 : 1;  // rows per lane; n <= 32: one row per lane
    auto pidx = [P](int r) { return r + r / P; };
    float2* col = b.spec + (size_t)(m - 1) * n;
    const T m2 = (T)m * (T)m;
    for (int r = lane; r < n; r += 32) {
        T A, C, B;
        if (sizeof(T) == 8) {
            A = (T)b.lapA64[r];
            C = (T)b.lapC64[r];
            B = (T)b.lapB064[r] - m2 * (T)b.lapS64[r];
        } else {
            A = (T)b.lapA[r];
            C = (T)b.lapC[r];
            B = (T)b.lapB0[r] - m2 * (T)b.lapS[r];
        }
        T inv = T(1) / B;
        float2 d = col[r];
        int q = pidx(r);
        sa[q] = A * inv;
        sc[q] = C * inv;
        sdr[q] = (T)d.x * inv;
        sdi[q] = (T)d.y * inv;
    }
    __syncwarp();
    Row<T> F, L;
    const int f = lane * P, l = f + P - 1;
    if (n <= 32) {
        // PCR over 32 rows, one per lane; lanes past n carry identity rows
        // (a = c = 0) that the last real row (c = 0) never couples to.
        int q = pidx(lane);
        const bool real = lane < n;
        F.a = real ? sa[q] : T(0);
        F.c = real ? sc[q] : T(0);
        F.dr = real ? sdr[q] : T(0);
        F.di = real ? sdi[q] : T(0);
        for (int s = 1; s < 32; s <<= 1) {
            Row<T> lo = shfl_row_up(F, s, lane), hi = shfl_row_down(F, s, lane);
            F = pcr_combine(F, lo, hi);
        }
        __syncwarp();
        if (real) {
            sdr[q] = F.dr;
            sdi[q] = F.di;
        }
    } else {
        // downward: rows f+2..l now couple x_f instead of x_{i-1}
        for (int i = f + 2; i <= l; i++) {
            int q = pidx(i), qm = pidx(i - 1);
            T ai = sa[q], ci = sc[q];
            T r = T(1) / (T(1) - ai * sc[qm]);
            sa[q] = -ai * sa[qm] * r;
            sc[q] = ci * r;
            sdr[q] = (sdr[q] - ai * sdr[qm]) * r;
            sdi[q] = (sdi[q] - ai * sdi[qm]) * r;
        }
        {
            int q = pidx(l);
            L.a = sa[q];
            L.c = sc[q];
            L.dr = sdr[q];
            L.di = sdi[q];
        }
        // upward: rows l-2..f+1 couple x_f and x_l
        for (int i = l - 2; i >= f + 1; i--) {
            int q = pidx(i), qp = pidx(i + 1);
            T ci = sc[q];
            sa[q] = sa[q] - ci * sa[qp];
            sc[q] = -ci * sc[qp];
            sdr[q] = sdr[q] - ci * sdr[qp];
            sdi[q] = sdi[q] - ci * sdi[qp];
        }
        {
            int q = pidx(f);
            T af = sa[q], cf = sc[q], dfr = sdr[q], dfi = sdi[q];
            if (P >= 3) {
                int q1 = pidx(f + 1);
                T inv = T(1) / (T(1) - cf * sa[q1]);
                F.a = af * inv;
                F.c = -cf * sc[q1] * inv;
                F.dr = (dfr - cf * sdr[q1]) * inv;
                F.di = (dfi - cf * sdi[q1]) * inv;
            } else {
                F.a = af;
                F.c = cf;
                F.dr = dfr;
                F.di = dfi;
            }
        }
        // PCR over the 64 boundary rows: row 2k = F, row 2k+1 = L of lane k
        {
            Row<T> Bm = shfl_row_up(L, 1, lane);    // row 2k-1
            Row<T> Ap = shfl_row_down(F, 1, lane);  // row 2k+2
            Row<T> nF = pcr_combine(F, Bm, L);
            Row<T> nL = pcr_combine(L, F, Ap);
            F = nF;
            L = nL;
        }
        for (int t = 1; t < 32; t <<= 1) {
            Row<T> Fm = shfl_row_up(F, t, lane), Fp = shfl_row_down(F, t, lane);
            Row<T> Lm = shfl_row_up(L, t, lane), Lp = shfl_row_down(L, t, lane);
            F = pcr_combine(F, Fm, Fp);
            L = pcr_combine(L, Lm, Lp);
        }
        const T xfr = F.dr, xfi = F.di, xlr = L.dr, xli = L.di;
        for (int i = f + 1; i <= l - 1; i++) {
            int q = pidx(i);
            T ai = sa[q], ci = sc[q];
            sdr[q] = sdr[q] - ai * xfr - ci * xlr;
            sdi[q] = sdi[q] - ai * xfi - ci * xli;
        }
        sdr[pidx(f)] = xfr;
        sdi[pidx(f)] = xfi;
        sdr[pidx(l)] = xlr;
        sdi[pidx(l)] = xli;
    }
    __syncwarp();
    for (int r = lane; r < n; r += 32) {
        int q = pidx(r);
        col[r] = make_float2((float)sdr[q], (float)sdi[q]);
    }
}

// Blocks [0, nfp64) solve modes 1..nfp64 in FP64 (warp 0 only); the rest
// solve SOLVE_WARPS FP32 modes each.
__global__ void __launch_bounds__(32 * SOLVE_WARPS) k_solve(KGeo g, KBufs b, int nfp64)
{
    extern __shared__ unsigned char smraw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = g.nt, stride = n + 32;
    if ((int)blockIdx.x < nfp64) {
        if (warp != 0) return;
        double* base = reinterpret_cast<double*>(smraw);
        solve_mode<double>(g, b, blockIdx.x + 1, base, base + stride, base + 2 * stride, base + 3 * stride,
                           lane);
        return;
    }
    const int m = nfp64 + 1 + (blockIdx.x - nfp64) * SOLVE_WARPS + warp;
    if (m > n) return;
    float* base = reinterpret_cast<float*>(smraw) + (size_t)warp * 4 * stride;
    solve_mode<float>(g, b, m, base, base + stride, base + 2 * stride, base + 3 * stride, lane);
}

// ---------------------------------------------------- inverse FFT + gradient
// Rows r0..r0+FFT_ROWS-1 are updated; row r0+FFT_ROWS (when it exists) is
// synthesised too because v at row j needs p at rows j and j+1.
__global__ void __launch_bounds__(32 * (FFT_ROWS + 1)) k_ifft_grad(KGeo g, KBufs b, int uv_in, int uv_out,
                                                                    int write_p)
{
    extern __shared__ float2 sm2[];
    const int nt = g.nt, np = g.np, mask = g.mask;
    const int r0 = blockIdx.x * FFT_ROWS;
    const int nrows = min(FFT_ROWS + 1, nt - r0);
    const int ld = nt + 1;
    float2* U = sm2;                         // staged U_m, slot m % nt
    float2* Fb = sm2 + (FFT_ROWS + 1) * ld;  // FFT rows
    for (int t = threadIdx.x; t < nt * nrows; t += blockDim.x) {
        int mi = t / nrows, r = t - mi * nrows;
        U[r * ld + ((mi + 1) & (nt - 1))] = b.spec[(size_t)mi * nt + r0 + r];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < nrows) {
        const float2* Ur = U + warp * ld;
        float2* x = Fb + warp * ld;
        // Y_m = (X_m + X_{m+nt}) + i (X_m - X_{m+nt}) e^{i pi m/nt} with
        // X_0 = 0, X_m = U_m, X_{m+nt} = conj(U_{nt-m}); X_nt = U_nt (real).
        for (int m = lane; m <= nt / 2; m += 32) {
            if (m == 0) {
                float un = Ur[0].x;
                x[0] = make_float2(un, -un);
                continue;
            }
            const int mb = nt - m;
            float2 ua = Ur[m], ub = Ur[mb];
            float2 ea = __ldg(b.rt + m), eb = __ldg(b.rt + mb);
            {
                float Er = ua.x + ub.x, Ei = ua.y - ub.y, Dr = ua.x - ub.x, Di = ua.y + ub.y;
                float Or = Dr * ea.x + Di * ea.y, Oi = Di * ea.x - Dr * ea.y;  // D * conj(rt)
                x[bitrev(m, g.log2nt)] = make_float2(Er - Oi, Ei + Or);
            }
            if (mb != m) {
                float Er = ub.x + ua.x, Ei = ub.y - ua.y, Dr = ub.x - ua.x, Di = ub.y + ua.y;
                float Or = Dr * eb.x + Di * eb.y, Oi = Di * eb.x - Dr * eb.y;
                x[bitrev(mb, g.log2nt)] = make_float2(Er - Oi, Ei + Or);
            }
        }
        __syncwarp();
        fft_dit_warp<true>(x, nt, g.log2nt, b.tw, lane);
    }
    __syncthreads();
    const float* __restrict__ uf = b.u[uv_in];
    const float* __restrict__ vf = b.v[uv_in];
    float* __restrict__ uo = b.u[uv_out];
    float* __restrict__ vo = b.v[uv_out];
    const float* pr = reinterpret_cast<const float*>(Fb);
    const int ldp = 2 * ld;
    const float neg_h = -g.h;
    for (int t = threadIdx.x; t < FFT_ROWS * np; t += blockDim.x) {
        int r = t / np, i = t - r * np;
        int j = r0 + r;
        size_t gi = (size_t)j * np + i;
        float pc = pr[r * ldp + i], pw = pr[r * ldp + ((i - 1) & mask)];
        // applyPressurePhi, KaminoCore.cu:740-746
        uo[gi] = __fadd_rn(__ldg(uf + gi), __fdiv_rn(__fsub_rn(pc, pw), __ldg(b.negHs + j)));
        if (j < nt - 1) {
            // applyPressureTheta, KaminoCore.cu:716-721
            float ps = pr[(r + 1) * ldp + i];
            vo[gi] = __fadd_rn(__ldg(vf + gi), __fdiv_rn(__fsub_rn(ps, pc), neg_h));
        }
        if (write_p) b.p[gi] = pc;
    }
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

} // namespace kk
