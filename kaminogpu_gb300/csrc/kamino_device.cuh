// kamino_device.cuh — device building blocks of the GB300 Kamino step.
//
// Index exactness.  The reference evaluates its sample positions with float
// variables and double literals (KaminoHeader.cuh:26-41), so validateCoord
// (KaminoCore.cu:11-29) and the staggering shifts run in double and round
// to float on assignment.  Doubles are 1/64-rate on GB300, so the samplers
// here run the common case in FP32 and reproduce the reference bit for bit:
//  * shift: (float)((double)a - (double)h * off) equals the FP32 a - h*off
//    because off*h is exact and one double operation followed by rounding to
//    float equals the correctly rounded float operation (53 >= 2*24 + 2,
//    the innocuous double-rounding bound for + - * /);
//  * validateCoord leaves (phi, theta) untouched exactly when
//    0 <= theta < pi_up (theta <= M_PI as a double, so no flip and the
//    2pi-wrap count is 0) and 0 <= phi < wrap_phi_hi (the first float whose
//    floorf((float)(phi / M_2PI)) is 1); -0.0 passes, as in the reference.
// Everything else (pole crossings and the phi = 0 seam) goes to
// ref_validate(), the reference's arithmetic in FP64, which only a few
// points per row reach.  kamino_probe_index() exposes this stage so the
// tests compare it with the reference restatement on arbitrary inputs.
#pragma once

#include <cuda_runtime.h>

#include "kamino_common.h"

namespace kdev {

// validateCoord with the reference's exact arithmetic (KaminoCore.cu:11-29).
__device__ __forceinline__ float ref_validate(float& phi, float& theta)
{
    float ret = 1.0f;
    {
        float q = __double2float_rn(__ddiv_rn((double)theta, KAMINO_2PI_D));
        int n = (int)floorf(q);
        theta = __double2float_rn(__dadd_rn((double)theta, -__dmul_rn((double)n, KAMINO_2PI_D)));
    }
    if ((double)theta > KAMINO_PI_D) {
        theta = __double2float_rn(__dsub_rn(KAMINO_2PI_D, (double)theta));
        phi = __double2float_rn(__dadd_rn((double)phi, KAMINO_PI_D));
        ret = -ret;
    }
    if (theta < 0) {
        theta = -theta;
        phi = __double2float_rn(__dadd_rn((double)phi, KAMINO_PI_D));
        ret = -ret;
    }
    {
        float q = __double2float_rn(__ddiv_rn((double)phi, KAMINO_2PI_D));
        int n = (int)floorf(q);
        phi = __double2float_rn(__dadd_rn((double)phi, -__dmul_rn((double)n, KAMINO_2PI_D)));
    }
    return ret;
}

// validateCoord: FP32 fast path when no wrap applies, exact path otherwise.
__device__ __forceinline__ bool wrap_coord(float& phi, float& theta, const KGeo& g)
{
    if (theta >= 0.0f && theta < g.pi_up && phi >= 0.0f && phi < g.wrap_phi_hi) return false;
    return ref_validate(phi, theta) < 0.0f;
}

// kaminoLerp (KaminoCore.cu:31-34): (1 - t) a + t b.
__device__ __forceinline__ float klerp(float a, float b, float t)
{
    return __fmaf_rn(t, b, __fmul_rn(1.0f - t, a));
}

enum { KIND_VPHI = 0, KIND_VTHETA = 1, KIND_CENTERED = 2 };

struct SampleIndex {
    int ip, it;      // phiIndex (wrapped to [0, nPhi)), thetaIndex
    float ap, at;    // alphaPhi, alphaTheta
    bool flipped;    // validateCoord returned -1
    bool pole;       // the pole branch of the sampler
};

// Index stage of sampleVPhi / sampleVTheta / sampleCentered
// (KaminoCore.cu:38-52, 88-103, 138-153).
template <int KIND>
__device__ __forceinline__ SampleIndex sample_index(float phiRaw, float thetaRaw, const KGeo& g)
{
    // staggering offsets: u_phi (-0.5, 0.5), u_theta (0, 1), centred (0, 0.5)
    float phi = (KIND == KIND_VPHI) ? __fadd_rn(phiRaw, g.halfh) : phiRaw;
    float theta = (KIND == KIND_VTHETA) ? __fsub_rn(thetaRaw, g.h) : __fsub_rn(thetaRaw, g.halfh);
    SampleIndex s;
    s.flipped = wrap_coord(phi, theta, g);
    float nphi = __fmul_rn(phi, g.invh), nth = __fmul_rn(theta, g.invh);
    float fp = floorf(nphi), ft = floorf(nth);
    // alpha = normed - (float)(int)floor(normed): adding +0 turns a -0.0
    // floor into the +0.0 that the int round trip gives
    s.ap = __fsub_rn(nphi, __fadd_rn(fp, 0.0f));
    s.at = __fsub_rn(nth, __fadd_rn(ft, 0.0f));
    s.ip = ((int)fp) & g.mask;
    // After validateCoord theta is in [0, pi], so thetaIndex is in [0, nt].
    // The clamp only matters for non-finite input, where it keeps every read
    // inside the allocation instead of faulting.
    s.it = min(max((int)ft, 0), g.nt);
    const int pole_row = (KIND == KIND_VTHETA) ? g.nt - 2 : g.nt - 1;
    s.pole = (s.it == 0 && s.flipped) || s.it == pole_row;
    return s;
}

// Bilinear sample with the reference's pole branch.  vec selects the
// optional sign flip of vector components across a pole.
template <int KIND>
__device__ __forceinline__ float sample(const float* __restrict__ f, float phiRaw, float thetaRaw,
                                        const KGeo& g, bool vec_flip)
{
    SampleIndex s = sample_index<KIND>(phiRaw, thetaRaw, g);
    const int i0 = s.ip, i1 = (s.ip + 1) & g.mask;
    const float* r0 = f + (size_t)s.it * g.pitch;
    float v00 = __ldg(r0 + i0), v01 = __ldg(r0 + i1);
    if (s.pole) {
        const int j0 = (i0 + g.half) & g.mask, j1 = (i1 + g.half) & g.mask;
        float v10 = __ldg(r0 + j0), v11 = __ldg(r0 + j1);
        float lo = klerp(v00, v01, s.ap), hi = klerp(v10, v11, s.ap);
        if (vec_flip) hi = -hi;
        float w = (KIND == KIND_VPHI) ? s.at : 0.5f * s.at;
        float r = klerp(lo, hi, w);
        return (vec_flip && s.flipped) ? -r : r;
    }
    const float* r1 = r0 + g.pitch;
    float v10 = __ldg(r1 + i0), v11 = __ldg(r1 + i1);
    float r = klerp(klerp(v00, v01, s.ap), klerp(v10, v11, s.ap), s.at);
    return (vec_flip && s.flipped) ? -r : r;
}

// RK2 back-trace of one grid point (advectionVPhiKernel /
// advectionVThetaKernel / advectionCentered, KaminoCore.cu:186-319).
// cofPhi = dt / (R sinf(gTheta)) comes from a per-row table computed with
// the same expression.
template <int KIND>
__device__ __forceinline__ float advect_point(const float* __restrict__ u, const float* __restrict__ v,
                                              const float* __restrict__ field, float gPhi, float gTheta,
                                              float cofPhi, const KGeo& g)
{
    const bool vf = (g.flags & KAMINO_F_POLE_SIGN_FLIP) != 0;
    float guPhi = sample<KIND_VPHI>(u, gPhi, gTheta, g, vf);
    float guTheta = sample<KIND_VTHETA>(v, gPhi, gTheta, g, vf);
    float deltaPhi = __fmul_rn(guPhi, cofPhi);
    float deltaTheta = __fmul_rn(guTheta, g.cofTheta);
    float midPhi = __fsub_rn(gPhi, 0.5f * deltaPhi);
    float midTheta = __fsub_rn(gTheta, 0.5f * deltaTheta);
    float muPhi = sample<KIND_VPHI>(u, midPhi, midTheta, g, vf);
    float muTheta = sample<KIND_VTHETA>(v, midPhi, midTheta, g, vf);
    float averuPhi = 0.5f * __fadd_rn(muPhi, guPhi);
    float averuTheta = 0.5f * __fadd_rn(muTheta, guTheta);
    deltaPhi = __fmul_rn(averuPhi, cofPhi);
    deltaTheta = __fmul_rn(averuTheta, g.cofTheta);
    float pPhi = __fsub_rn(gPhi, deltaPhi);
    float pTheta = __fsub_rn(gTheta, deltaTheta);
    return sample<KIND>(field, pPhi, pTheta, g, vf && KIND != KIND_CENTERED);
}

// sample() for a position that needs no wrap (validateCoord leaves it
// untouched) and is not in a pole row, with no branch: `bad` is set for any
// other position, whose value is then meaningless; the row is clamped, so
// the reads stay inside the field whatever the position.  Where `bad` stays
// clear the operations are sample()'s own, so the value is the same.
template <int KIND>
__device__ __forceinline__ float sample_ref_try(const float* __restrict__ f, float phiRaw, float thetaRaw,
                                                const KGeo& g, bool& bad)
{
    const float phi = (KIND == KIND_VPHI) ? __fadd_rn(phiRaw, g.halfh) : phiRaw;
    const float theta = (KIND == KIND_VTHETA) ? __fsub_rn(thetaRaw, g.h) : __fsub_rn(thetaRaw, g.halfh);
    bad |= !(theta >= 0.0f && theta < g.pi_up && phi >= 0.0f && phi < g.wrap_phi_hi);
    const float nphi = __fmul_rn(phi, g.invh), nth = __fmul_rn(theta, g.invh);
    const float fp = floorf(nphi), ft = floorf(nth);
    const float ap = __fsub_rn(nphi, __fadd_rn(fp, 0.0f));
    const float at = __fsub_rn(nth, __fadd_rn(ft, 0.0f));
    const int i0 = ((int)fp) & g.mask, i1 = (i0 + 1) & g.mask;
    const unsigned pole_row = (KIND == KIND_VTHETA) ? g.nt - 2 : g.nt - 1;
    const unsigned it = (unsigned)(int)ft;
    bad |= it >= pole_row;
    const float* r0 = f + (size_t)min(it, pole_row - 1) * g.pitch;
    const float* r1 = r0 + g.pitch;
    const float v00 = __ldg(r0 + i0), v01 = __ldg(r0 + i1), v10 = __ldg(r1 + i0), v11 = __ldg(r1 + i1);
    return klerp(klerp(v00, v01, ap), klerp(v10, v11, ap), at);
}

// advect_point through sample_ref_try: a point one of whose five samples
// needs a wrap or lies in a pole row is recomputed by advect_point, so the
// value is advect_point's in every case.
template <int KIND>
__device__ __forceinline__ float advect_point_fast(const float* __restrict__ u, const float* __restrict__ v,
                                                   const float* __restrict__ field, float gPhi, float gTheta,
                                                   float cofPhi, const KGeo& g)
{
    bool bad = false;
    const float guPhi = sample_ref_try<KIND_VPHI>(u, gPhi, gTheta, g, bad);
    const float guTheta = sample_ref_try<KIND_VTHETA>(v, gPhi, gTheta, g, bad);
    float deltaPhi = __fmul_rn(guPhi, cofPhi);
    float deltaTheta = __fmul_rn(guTheta, g.cofTheta);
    const float midPhi = __fsub_rn(gPhi, 0.5f * deltaPhi);
    const float midTheta = __fsub_rn(gTheta, 0.5f * deltaTheta);
    const float muPhi = sample_ref_try<KIND_VPHI>(u, midPhi, midTheta, g, bad);
    const float muTheta = sample_ref_try<KIND_VTHETA>(v, midPhi, midTheta, g, bad);
    const float averuPhi = 0.5f * __fadd_rn(muPhi, guPhi);
    const float averuTheta = 0.5f * __fadd_rn(muTheta, guTheta);
    deltaPhi = __fmul_rn(averuPhi, cofPhi);
    deltaTheta = __fmul_rn(averuTheta, g.cofTheta);
    const float pPhi = __fsub_rn(gPhi, deltaPhi);
    const float pTheta = __fsub_rn(gTheta, deltaTheta);
    const float r = sample_ref_try<KIND>(field, pPhi, pTheta, g, bad);
    return bad ? advect_point<KIND>(u, v, field, gPhi, gTheta, cofPhi, g) : r;
}

// ------------------------------------------------- cell-exact positions
// A position is a grid point (i, j) plus a small FP32 offset (fp, ft) in
// cells, so the integer part is exact and the fraction keeps full relative
// precision.  The staggering shifts of the samplers are exact small
// constants, the phi seam is an integer mask, and the pole remap of
// validateCoord (theta < 0 or theta > pi: theta -> -theta or 2pi - theta,
// phi -> phi + pi) is exact integer/fraction arithmetic with pi = nTheta
// cells.  Same branches and blends as the reference samplers.
template <int KIND>
__device__ __forceinline__ SampleIndex cell_index(int i, int j, float fp, float ft, const KGeo& g)
{
    SampleIndex s;
    float kp = floorf(fp), kt = floorf(ft);
    s.ap = fp - kp;
    s.at = ft - kt;
    int ip = i + (int)kp, it = j + (int)kt;
    s.flipped = false;
    if (it < 0) {  // theta < 0: reflect through the north pole
        s.flipped = true;
        ip += g.half;
        if (s.at == 0.0f) {
            it = -it;
        } else {
            it = -it - 1;
            s.at = 1.0f - s.at;
        }
    } else if (it >= g.nt && (it > g.nt || s.at > 0.0f)) {  // theta > pi
        s.flipped = true;
        ip += g.half;
        if (s.at == 0.0f) {
            it = 2 * g.nt - it;
        } else {
            it = 2 * g.nt - it - 1;
            s.at = 1.0f - s.at;
        }
    }
    s.ip = ip & g.mask;
    s.it = min(max(it, 0), g.nt);  // only non-finite input can need this
    const int pole_row = (KIND == KIND_VTHETA) ? g.nt - 2 : g.nt - 1;
    s.pole = (s.it == 0 && s.flipped) || s.it == pole_row;
    return s;
}

__device__ __forceinline__ float lerp2(float a, float b, float t) { return __fmaf_rn(t, b - a, a); }

template <int KIND>
__device__ __forceinline__ float sample_cell(const float* __restrict__ f, int i, int j, float fp, float ft,
                                             const KGeo& g, bool vec_flip)
{
    SampleIndex s = cell_index<KIND>(i, j, fp, ft, g);
    const int i0 = s.ip, i1 = (s.ip + 1) & g.mask;
    const float* r0 = f + s.it * g.pitch;
    float v00 = __ldg(r0 + i0), v01 = __ldg(r0 + i1);
    if (s.pole) {
        const int j0 = (i0 + g.half) & g.mask, j1 = (i1 + g.half) & g.mask;
        float v10 = __ldg(r0 + j0), v11 = __ldg(r0 + j1);
        float lo = lerp2(v00, v01, s.ap), hi = lerp2(v10, v11, s.ap);
        if (vec_flip) hi = -hi;
        float w = (KIND == KIND_VPHI) ? s.at : 0.5f * s.at;
        float r = lerp2(lo, hi, w);
        return (vec_flip && s.flipped) ? -r : r;
    }
    const float* r1 = r0 + g.pitch;
    float v10 = __ldg(r1 + i0), v11 = __ldg(r1 + i1);
    float r = lerp2(lerp2(v00, v01, s.ap), lerp2(v10, v11, s.ap), s.at);
    return (vec_flip && s.flipped) ? -r : r;
}

// Packed pairs (f32x2: one instruction for two FP32 lanes of a register
// pair, sm_100 and later) carry the two coordinates of a position and the
// two row lerps of a bilinear sample.  Each lane rounds as the scalar
// instruction would.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// RK2 back-trace in cells.  (cgp, cgt) is the grid point's staggering
// offset in cells (u_phi: -1/2, 1/2; u_theta: 0, 1; centred: 0, 1/2); the
// samplers' own offsets are u_phi (-1/2, 1/2), u_theta (0, 1), centred
// (0, 1/2), so each sample position is (i, j) + (cg - so) - d exactly.
// cP, cT convert velocity to displacement in cells (dt / (R sin(theta) h),
// dt / (R h)); cP uses the grid point's latitude as the reference does.
// The positions are formed by the same packed instructions as advect_from's,
// so for a cell of rows 1 .. nTheta-3 away from the seam the two give the
// same value wherever every sample of advect_from stays in its domain.
template <int KIND>
__device__ __forceinline__ float advect_cell(const float* __restrict__ u, const float* __restrict__ v,
                                             const float* __restrict__ field, int i, int j, float cP, float cT,
                                             const KGeo& g)
{
    constexpr float cgp = (KIND == KIND_VPHI) ? -0.5f : 0.0f;
    constexpr float cgt = (KIND == KIND_VTHETA) ? 1.0f : 0.5f;
    constexpr float ou_p = cgp + 0.5f, ou_t = cgt - 0.5f;  // offsets for the u_phi sampler
    constexpr float ov_p = cgp, ov_t = cgt - 1.0f;         // u_theta sampler
    // a field's own sampler offset equals its staggering: offset 0
    const bool vf = (g.flags & KAMINO_F_POLE_SIGN_FLIP) != 0;
    const float2 gv = f2(sample_cell<KIND_VPHI>(u, i, j, ou_p, ou_t, g, vf),
                         sample_cell<KIND_VTHETA>(v, i, j, ov_p, ov_t, g, vf));
    const float2 nhc = __fmul2_rn(f2(cP, cT), f2(-0.5f, -0.5f));
    const float2 hd = __fmul2_rn(gv, nhc);
    const float2 pu = __fadd2_rn(hd, f2(ou_p, ou_t)), pv = __fadd2_rn(hd, f2(ov_p, ov_t));
    const float mu = sample_cell<KIND_VPHI>(u, i, j, pu.x, pu.y, g, vf);
    const float mv = sample_cell<KIND_VTHETA>(v, i, j, pv.x, pv.y, g, vf);
    const float2 d = __fmul2_rn(__fadd2_rn(f2(mu, mv), gv), nhc);
    return sample_cell<KIND>(field, i, j, d.x, d.y, g, vf && KIND != KIND_CENTERED);
}


// floor of a position pair by a round-down add of 1.5 * 2^23: t - 1.5 * 2^23
// is floor(x) exactly for -2^22 <= x < 2^23, so the fraction x - floor(x) is
// exact too; the caller reads floor(x) + 0x4B400000 from t's bits.
constexpr float kFloorBias = 12582912.0f;
constexpr int kFloorBits = 0x4B400000;

// sample_cell for positions whose rows it, it + 1 both lie in [0, pole_row)
// and whose column pair does not straddle the phi seam: plain bilinear from
// one address (the phi neighbour at +1, the next row at +pitch), equal to
// sample_cell's value there for every phi offset of less than 2^22 cells (any
// displacement a stable time step can make).  Outside that domain (a pole
// row, a crossing, the seam, a non-finite position) `bad` is set and the
// value is meaningless; the reads still stay inside the field: the row is
// clamped to pole_row - 1, so they touch rows 0 .. pole_row and, from the
// last column, the first element of the row after (each field has two rows
// past its data).
// ib, jb = i, j - 0x4B400000 (mod 2^32): ib + bits(t) = i + floor(x).
template <int KIND>
__device__ __forceinline__ float sample_try(const float* __restrict__ f, unsigned ib, unsigned jb, float2 p,
                                            const KGeo& g, bool& bad)
{
    const float2 t = __fadd2_rd(p, f2(kFloorBias, kFloorBias));
    const float2 a = __fadd2_rn(p, __ffma2_rn(t, f2(-1.0f, -1.0f), f2(kFloorBias, kFloorBias)));
    const unsigned it = jb + (unsigned)__float_as_int(t.y);
    const int i0 = (int)(ib + (unsigned)__float_as_int(t.x)) & g.mask;
    const unsigned pole_row = (KIND == KIND_VTHETA) ? g.nt - 2 : g.nt - 1;
    bad |= (it >= pole_row) | (i0 == g.mask);
    const float* p0 = f + ((int)min(it, pole_row - 1) * g.pitch + i0);
    const float* p1 = p0 + g.pitch;
    const float2 lo = f2(__ldg(p0), __ldg(p1)), hi = f2(__ldg(p0 + 1), __ldg(p1 + 1));
    const float2 r = __ffma2_rn(f2(a.x, a.x), __ffma2_rn(lo, f2(-1.0f, -1.0f), hi), lo);
    return lerp2(r.x, r.y, a.y);
}

// RK2 step of one quantity from its start-point velocities gv = (u, v):
// advect_cell after its first two samples, through sample_try (`bad` set
// when a sample left its domain; the caller then takes advect_cell).
// nhc = (-cP / 2, -cT / 2).
template <int KIND>
__device__ __forceinline__ float advect_from(const float* __restrict__ u, const float* __restrict__ v,
                                             const float* __restrict__ field, unsigned ib, unsigned jb, float2 gv,
                                             float2 nhc, const KGeo& g, bool& bad)
{
    constexpr float cgp = (KIND == KIND_VPHI) ? -0.5f : 0.0f;
    constexpr float cgt = (KIND == KIND_VTHETA) ? 1.0f : 0.5f;
    constexpr float ou_p = cgp + 0.5f, ou_t = cgt - 0.5f;
    constexpr float ov_p = cgp, ov_t = cgt - 1.0f;
    // midpoint: offset - d / 2 for each sampler
    const float2 hd = __fmul2_rn(gv, nhc);
    const float mu = sample_try<KIND_VPHI>(u, ib, jb, __fadd2_rn(hd, f2(ou_p, ou_t)), g, bad);
    const float mv = sample_try<KIND_VTHETA>(v, ib, jb, __fadd2_rn(hd, f2(ov_p, ov_t)), g, bad);
    // departure point: -(mid + start) / 2 * c
    const float2 d = __fmul2_rn(__fadd2_rn(f2(mu, mv), gv), nhc);
    return sample_try<KIND>(field, ib, jb, d, g, bad);
}

// The three advected quantities of cell (i, j) in one thread: u_phi at
// (i - 1/2, j + 1/2), u_theta at (i, j + 1) when j < nTheta - 1, thickness
// at (i, j + 1/2).  In rows 1 .. nTheta-3 the start-point velocities are
// fixed stencils of the grid (the samplers' alphas there are 0 or 1/2 and
// no pole branch applies), shared between the three quantities:
//   u_phi point:    u = u[j][i],        v = bilinear of v[j-1..j][i-1..i]
//   u_theta point:  u = bilinear of u[j..j+1][i..i+1],  v = v[j][i]
//   centred point:  u = mean of u[j][i..i+1],  v = mean of v[j-1..j][i]
// The rows next to the poles and the two columns at the phi seam run
// advect_cell for each quantity, and so does a cell one of whose samples left
// sample_try's domain (its fast values are discarded), with one copy of the
// exact path in the kernel.  advect_cell forms its positions with
// advect_from's instructions and sample_cell equals sample_try inside the
// domain, so a quantity whose samples all stayed inside it gets the same
// value either way.
// MASK selects the quantities (bit 0 u_phi, bit 1 u_theta, bit 2 thickness);
// each one's value does not depend on which others are computed.
template <int MASK = 7>
__device__ __forceinline__ void advect_cell3(const float* __restrict__ u, const float* __restrict__ v,
                                             const float* __restrict__ rho, int i, int j, float cPc, float cPv,
                                             float cT, const KGeo& g, float& out_u, float& out_v, float& out_r)
{
    bool exact = true;
    if (j >= 1 && j <= g.nt - 3 && i >= 1 && i < g.mask) {
        // columns i - 1 .. i + 1 without wrapping: neighbours at +-1
        const float* uj = u + (j * g.pitch + i);
        const float* ujn = uj + g.pitch;
        const float* vj = v + (j * g.pitch + i);
        const float* vm = vj - g.pitch;
        const float u00 = __ldg(uj), u01 = __ldg(uj + 1);
        const float u10 = __ldg(ujn), u11 = __ldg(ujn + 1);
        const float vmm = __ldg(vm - 1), vm0 = __ldg(vm);
        const float v0m = __ldg(vj - 1), v00 = __ldg(vj);
        const float gu_phi = u00;
        const float gv_phi = lerp2(lerp2(vmm, vm0, 0.5f), lerp2(v0m, v00, 0.5f), 0.5f);
        const float u_mid0 = lerp2(u00, u01, 0.5f);
        const float gu_th = lerp2(u_mid0, lerp2(u10, u11, 0.5f), 0.5f);
        const float gv_th = v00;
        const float gu_c = u_mid0;
        const float gv_c = lerp2(vm0, v00, 0.5f);
        const unsigned ib = (unsigned)i - (unsigned)kFloorBits, jb = (unsigned)j - (unsigned)kFloorBits;
        const float2 nhc = __fmul2_rn(f2(cPc, cT), f2(-0.5f, -0.5f));
        const float2 nhv = f2(-0.5f * cPv, nhc.y);
        bool bad = false;
        if constexpr ((MASK & 1) != 0)
            out_u = advect_from<KIND_VPHI>(u, v, u, ib, jb, f2(gu_phi, gv_phi), nhc, g, bad);
        if constexpr ((MASK & 2) != 0)
            out_v = advect_from<KIND_VTHETA>(u, v, v, ib, jb, f2(gu_th, gv_th), nhv, g, bad);
        if constexpr ((MASK & 4) != 0)
            out_r = advect_from<KIND_CENTERED>(u, v, rho, ib, jb, f2(gu_c, gv_c), nhc, g, bad);
        exact = bad;
    }
    if (exact) {
        if constexpr ((MASK & 1) != 0) out_u = advect_cell<KIND_VPHI>(u, v, u, i, j, cPc, cT, g);
        if constexpr ((MASK & 2) != 0)
            if (j < g.nt - 1) out_v = advect_cell<KIND_VTHETA>(u, v, v, i, j, cPv, cT, g);
        if constexpr ((MASK & 4) != 0) out_r = advect_cell<KIND_CENTERED>(u, v, rho, i, j, cPc, cT, g);
    }
}

// PTX rcp.approx.ftz.f32: the hardware reciprocal, within about an ulp.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ------------------------------------------------------------ geometric
// The reference's solveCubic (KaminoCore.cu:421-454) with a = 0, in FP64,
// used only when 1 + G v <= 0 (three real roots possible).
__device__ __forceinline__ double ref_solve_cubic64(double b, double c)
{
    const double eps = (double)1e-7f;
    double q = (0.0 - 3 * b) / 9.0;
    double r = (27.0 * c) / 54.0;
    double r2 = r * r, q3 = q * q * q;
    if (r2 <= (q3 + eps)) {
        double t = r / sqrt(q3);
        if (t < -1) t = -1;
        if (t > 1) t = 1;
        t = acos(t);
        q = -2.0 * sqrt(q);
        return q * cos(t / 3.0);
    }
    double x = fabs(r) + sqrt(r2 - q3);
    double A = (x > 0 && isfinite(x)) ? -cbrt(x) : -x;
    if (r < 0) A = -A;
    double B = A == 0 ? 0 : q / A;
    return A + B;
}

// The FP64 branch of geo_roots (1 + G v <= 0).  Not inlined, so none of its
// double arithmetic is evaluated ahead of the branch for every cell (FP64 is
// 1/64 of the FP32 rate on GB300).
static __device__ __noinline__ float geo_root_fp64(float G, float uPrev, float vPrev)
{
    double G2 = (double)G * (double)G;
    return (float)ref_solve_cubic64(((double)G * vPrev + 1.0) / G2, -(double)uPrev / G2);
}

// u' of geometricFillKernel (KaminoCore.cu:494-508) for N cells of one row
// (one G): the root the reference takes of
// u^3 + ((G v + 1)/G^2) u - uPrev/G^2 = 0.  When 1 + G v > 0 that root is
// unique and g(u) = G^2 u^3 + (1 + G v) u - uPrev is increasing and
// convex/concave on either side of 0, so Newton from uPrev/(1 + G v)
// converges monotonically; FP32 keeps full relative accuracy (the
// reference's FP32 Cardano form cancels A + B catastrophically near the
// equator, where G is small).  The N Newton iterations run in lockstep (N
// independent dependency chains in flight), each cell's x frozen from the
// iteration its own test stops it, so a root does not depend on N.  For
// every cell that iterates, df >= 1 + G v > 0.
template <int N>
__device__ __forceinline__ void geo_roots(float G, const float (&uPrev)[N], const float (&vPrev)[N], float (&x)[N])
{
    if (!(fabsf(G) > 1e-7f)) {
#pragma unroll
        for (int k = 0; k < N; k++) x[k] = uPrev[k];
        return;
    }
    const float G2 = G * G;
    float a[N];
    bool live[N];
#pragma unroll
    for (int k = 0; k < N; k++) {
        a[k] = __fmaf_rn(G, vPrev[k], 1.0f);
        live[k] = a[k] > 0.0f;
        x[k] = live[k] ? uPrev[k] * rcp_approx(a[k]) : 0.0f;
    }
    for (int it = 0; it < 40; it++) {
        bool any = false;
#pragma unroll
        for (int k = 0; k < N; k++) {
            const float x2 = x[k] * x[k];
            const float f = __fmaf_rn(G2 * x2, x[k], __fmaf_rn(a[k], x[k], -uPrev[k]));
            const float df = __fmaf_rn(3.0f * G2, x2, a[k]);
            const float dx = f * rcp_approx(df);
            const float xn = x[k] - dx;
            if (live[k]) x[k] = xn;
            live[k] = live[k] && fabsf(dx) > 5e-7f * fabsf(xn);
            any |= live[k];
        }
        if (!any) break;
    }
#pragma unroll
    for (int k = 0; k < N; k++)
        if (!(a[k] > 0.0f)) x[k] = geo_root_fp64(G, uPrev[k], vPrev[k]);
}

// ------------------------------------------------------- complex product
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}



} // namespace kdev
