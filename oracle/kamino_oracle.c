/*
 * kamino_oracle.c — CPU restatement of Kamino's solver step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this
 * file; tests/, the smoke check and bench.py's CPU-baseline leg use it as
 * the checker.  It follows the reference kernels line by line:
 *   samplers / advection      KaminoGPU/kernel/KaminoCore.cu:11-342
 *   geometric step            KaminoGPU/kernel/KaminoCore.cu:386-549
 *   projection                KaminoGPU/kernel/KaminoCore.cu:587-747
 *   Laplacian coefficients    KaminoGPU/kernel/KaminoSolver.cu:117-163
 *   stage order               KaminoGPU/kernel/KaminoSolver.cu:197-221
 *
 * Two restatements live here:
 *  1. The FP64 step (oracle_*): every fReal of the reference becomes a double
 *     (h = pi/nTheta in double).  The cuFFT C2C pair and the shift kernels
 *     are replaced by the spectral identities they implement: the pressure is
 *     p = Re sum_{n != 0} U_n e^{i n phi} with U_n the solution of the
 *     per-mode tridiagonal system for c_n = (1/nPhi) sum_j div_j e^{-i n phi_j}
 *     (KaminoCore.cu:640-703).  Both signs of n share one matrix (it depends
 *     on n^2, KaminoSolver.cu:133-134), so only n = 1..nTheta are solved.
 *     The tridiagonal systems are solved by the Thomas algorithm in FP64
 *     (the reference uses FP32 cyclic reduction, tdm.cu:3-96, which has the
 *     same exact solution).
 *  2. The index stage of the samplers and validateCoord in the reference's
 *     own arithmetic (oracle_ref_*): float variables, double literals
 *     (M_PI, M_2PI, offsets) promoting the expressions they appear in, as
 *     C++ does in KaminoCore.cu:11-52.  Compiled with -ffp-contract=off so no
 *     multiply-add is fused behind our back.
 *
 * Out-of-range rows (the reference reads past the u_theta allocation for
 * departure points in (pi, pi+2h), KaminoCore.cu:103) read as zero: every
 * field here has nTheta+2 rows with the rows past the data zeroed.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_PI 3.14159265358979323846  /* M_PI, KaminoHeader.cuh:26 */
#define O_2PI 6.28318530717958647692 /* M_2PI, KaminoHeader.cuh:27 */

enum { K_VPHI = 0, K_VTHETA = 1, K_CENTERED = 2 };
enum { F_U = 0, F_V = 1, F_RHO = 2, F_P = 3, F_PART = 4 };
enum { FL_PARTICLE_RK2 = 1, FL_POLE_SIGN_FLIP = 2 };

typedef struct oracle_s {
    int nt, np, mask;
    double h, R, dt;
    unsigned flags;
    size_t rows_alloc; /* nt + 2 */
    double *u, *v, *rho, *p;
    double *un, *vn, *rhon;
    double *cu, *cv;
    int64_t npart;
    double *part, *partn;
    /* projection */
    double *lapA, *lapB0, *lapC, *lapS; /* per row, KaminoSolver.cu:128-159 */
    double *twr, *twi;                  /* e^{-2 pi i k / nt}, k < nt       */
    double *rtr, *rti;                  /* e^{-i pi m / nt},  m <= nt       */
    double *spec;                       /* [nt modes][nt rows][2]           */
    double *divbuf;
} oracle;

/* ---------------------------------------------------------------- helpers */
static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

int oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* validateCoord in FP64 (KaminoCore.cu:11-29). */
static double o_validate(double *phi, double *theta)
{
    double ret = 1.0;
    *theta = *theta - floor(*theta / O_2PI) * O_2PI;
    if (*theta > O_PI) {
        *theta = O_2PI - *theta;
        *phi += O_PI;
        ret = -ret;
    }
    if (*theta < 0) {
        *theta = -*theta;
        *phi += O_PI;
        ret = -ret;
    }
    *phi = *phi - floor(*phi / O_2PI) * O_2PI;
    return ret;
}

/* kaminoLerp (KaminoCore.cu:31-34). */
static inline double o_lerp(double a, double b, double t) { return (1.0 - t) * a + t * b; }

/* sampleVPhi / sampleVTheta / sampleCentered in FP64 (KaminoCore.cu:36-184).
 * The three differ only in the staggering offset, the row that takes the
 * pole branch, and the pole blend weight (alphaTheta vs 0.5*alphaTheta). */
static double o_sample(const oracle *o, const double *f, int kind, double phiRaw,
                       double thetaRaw, int vector_field)
{
    static const double offp[3] = {-0.5, 0.0, 0.0}; /* KaminoHeader.cuh:30-41 */
    static const double offt[3] = {0.5, 1.0, 0.5};
    double phi = phiRaw - o->h * offp[kind];
    double theta = thetaRaw - o->h * offt[kind];
    double flip = o_validate(&phi, &theta);
    double inv = 1.0 / o->h;
    double nphi = phi * inv, ntheta = theta * inv;
    int ip = (int)floor(nphi), it = (int)floor(ntheta);
    double ap = nphi - (double)ip, at = ntheta - (double)it;
    int pole_row = (kind == K_VTHETA) ? o->nt - 2 : o->nt - 1;
    size_t pitch = (size_t)o->np;
    int sgn = (vector_field && (o->flags & FL_POLE_SIGN_FLIP)) ? 1 : 0;
    if ((it == 0 && flip == -1.0) || it == pole_row) {
        int i0 = ip & o->mask, i1 = (i0 + 1) & o->mask;
        int j0 = (i0 + o->np / 2) & o->mask, j1 = (i1 + o->np / 2) & o->mask;
        const double *row = f + (size_t)it * pitch;
        double lower = o_lerp(row[i0], row[i1], ap);
        double higher = o_lerp(row[j0], row[j1], ap);
        if (sgn) higher = -higher;
        double w = (kind == K_VPHI) ? at : 0.5 * at;
        double r = o_lerp(lower, higher, w);
        return sgn ? flip * r : r;
    } else {
        int i0 = ip & o->mask, i1 = (i0 + 1) & o->mask;
        const double *r0 = f + (size_t)it * pitch, *r1 = r0 + pitch;
        double lower = o_lerp(r0[i0], r0[i1], ap);
        double higher = o_lerp(r1[i0], r1[i1], ap);
        double r = o_lerp(lower, higher, at);
        return sgn ? flip * r : r;
    }
}

/* RK2 back-trace shared by the three advection kernels
 * (KaminoCore.cu:186-229, 231-274, 276-319). */
static double o_trace(const oracle *o, const double *field, int kind, double gPhi, double gTheta)
{
    double guPhi = o_sample(o, o->u, K_VPHI, gPhi, gTheta, 1);
    double guTheta = o_sample(o, o->v, K_VTHETA, gPhi, gTheta, 1);
    double latRadius = o->R * sin(gTheta);
    double cofPhi = o->dt / latRadius, cofTheta = o->dt / o->R;
    double deltaPhi = guPhi * cofPhi, deltaTheta = guTheta * cofTheta;
    double midPhi = gPhi - 0.5 * deltaPhi, midTheta = gTheta - 0.5 * deltaTheta;
    double muPhi = o_sample(o, o->u, K_VPHI, midPhi, midTheta, 1);
    double muTheta = o_sample(o, o->v, K_VTHETA, midPhi, midTheta, 1);
    double averuPhi = 0.5 * (muPhi + guPhi), averuTheta = 0.5 * (muTheta + guTheta);
    deltaPhi = averuPhi * cofPhi;
    deltaTheta = averuTheta * cofTheta;
    return o_sample(o, field, kind, gPhi - deltaPhi, gTheta - deltaTheta, kind != K_CENTERED);
}

static void swapp(double **a, double **b)
{
    double *t = *a;
    *a = *b;
    *b = t;
}

/* ------------------------------------------------------------- lifecycle */
/* h <= 0 selects the exact spacing pi/nTheta; a positive h (e.g. the float
 * gridLenGlobal of the reference) is used as given. */
oracle *oracle_create_h(int nt, double R, double dt, unsigned flags, int64_t npart, double h_in)
{
    if (nt < 4 || (nt & (nt - 1))) return NULL;
    oracle *o = (oracle *)calloc(1, sizeof(oracle));
    o->nt = nt;
    o->np = 2 * nt;
    o->mask = o->np - 1;
    o->h = h_in > 0 ? h_in : O_PI / nt;
    o->R = R;
    o->dt = dt;
    o->flags = flags;
    o->rows_alloc = (size_t)nt + 2;
    size_t fs = o->rows_alloc * (size_t)o->np;
    o->u = zalloc(fs);
    o->v = zalloc(fs);
    o->rho = zalloc(fs);
    o->p = zalloc(fs);
    o->un = zalloc(fs);
    o->vn = zalloc(fs);
    o->rhon = zalloc(fs);
    o->cu = zalloc(fs);
    o->cv = zalloc(fs);
    o->divbuf = zalloc(fs);
    o->npart = npart > 0 ? npart : 0;
    o->part = zalloc(2 * (size_t)o->npart);
    o->partn = zalloc(2 * (size_t)o->npart);
    o->lapA = zalloc(nt);
    o->lapB0 = zalloc(nt);
    o->lapC = zalloc(nt);
    o->lapS = zalloc(nt);
    /* precomputeABCKernel (KaminoSolver.cu:117-163) for n != 0, split into
     * the n-independent parts and 1/sin^2 so B(n) = B0 - n^2 * S. */
    double h = o->h;
    for (int i = 0; i < nt; i++) {
        double th = (i + 0.5) * h;
        double c = cos(th), s = sin(th);
        double A = 1.0 / (h * h) - c / 2.0 / h / s;
        double C = 1.0 / (h * h) + c / 2.0 / h / s;
        double B0 = -2.0 / (h * h);
        if (i == 0) {
            B0 += A;
            A = 0.0;
        }
        if (i == nt - 1) {
            B0 += C;
            C = 0.0;
        }
        o->lapA[i] = A;
        o->lapC[i] = C;
        o->lapB0[i] = B0;
        o->lapS[i] = 1.0 / (s * s);
    }
    o->twr = zalloc(nt);
    o->twi = zalloc(nt);
    for (int k = 0; k < nt; k++) {
        o->twr[k] = cos(-2.0 * O_PI * k / nt);
        o->twi[k] = sin(-2.0 * O_PI * k / nt);
    }
    o->rtr = zalloc(nt + 1);
    o->rti = zalloc(nt + 1);
    for (int m = 0; m <= nt; m++) {
        o->rtr[m] = cos(-O_PI * m / nt);
        o->rti[m] = sin(-O_PI * m / nt);
    }
    o->spec = zalloc(2 * (size_t)nt * nt);
    return o;
}

oracle *oracle_create(int nt, double R, double dt, unsigned flags, int64_t npart)
{
    return oracle_create_h(nt, R, dt, flags, npart, 0.0);
}

void oracle_destroy(oracle *o)
{
    if (!o) return;
    double *ps[] = {o->u,    o->v,    o->rho,  o->p,    o->un,   o->vn,   o->rhon,
                    o->cu,   o->cv,   o->divbuf, o->part, o->partn, o->lapA, o->lapB0,
                    o->lapC, o->lapS, o->twr,  o->twi,  o->rtr,  o->rti,  o->spec};
    for (size_t i = 0; i < sizeof(ps) / sizeof(ps[0]); i++) free(ps[i]);
    free(o);
}

static int field_rows(const oracle *o, int field) { return field == F_V ? o->nt - 1 : o->nt; }

static double *field_ptr(oracle *o, int field)
{
    switch (field) {
    case F_U: return o->u;
    case F_V: return o->v;
    case F_RHO: return o->rho;
    case F_P: return o->p;
    case F_PART: return o->part;
    }
    return NULL;
}

/* Dense float input: rows x nPhi, or 2*npart for particles. */
int oracle_set_state(oracle *o, int field, const float *src)
{
    double *d = field_ptr(o, field);
    if (!d) return 1;
    if (field == F_PART) {
        for (int64_t i = 0; i < 2 * o->npart; i++) d[i] = src[i];
        return 0;
    }
    size_t n = (size_t)field_rows(o, field) * o->np;
    size_t all = o->rows_alloc * (size_t)o->np;
    for (size_t i = 0; i < all; i++) d[i] = i < n ? (double)src[i] : 0.0;
    return 0;
}

int oracle_set_state_f64(oracle *o, int field, const double *src)
{
    double *d = field_ptr(o, field);
    if (!d) return 1;
    if (field == F_PART) {
        memcpy(d, src, sizeof(double) * 2 * (size_t)o->npart);
        return 0;
    }
    size_t n = (size_t)field_rows(o, field) * o->np;
    size_t all = o->rows_alloc * (size_t)o->np;
    for (size_t i = 0; i < all; i++) d[i] = i < n ? src[i] : 0.0;
    return 0;
}

int oracle_get_state(oracle *o, int field, double *dst)
{
    double *d = field_ptr(o, field);
    if (!d) return 1;
    size_t n = field == F_PART ? 2 * (size_t)o->npart : (size_t)field_rows(o, field) * o->np;
    memcpy(dst, d, sizeof(double) * n);
    return 0;
}

/* ------------------------------------------------------------- advection */
/* KaminoSolver::advection (KaminoCore.cu:344-384): u*, v*, thickness and the
 * particles all read the pre-advection velocity; the swaps follow. */
void oracle_advection(oracle *o)
{
    const int nt = o->nt, np = o->np;
    const double h = o->h;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; j++) {
        for (int i = 0; i < np; i++) {
            /* advectionVPhiKernel, KaminoCore.cu:195-196 */
            o->un[(size_t)j * np + i] = o_trace(o, o->u, K_VPHI, (i - 0.5) * h, (j + 0.5) * h);
            /* advectionCentered, KaminoCore.cu:285-286 */
            o->rhon[(size_t)j * np + i] =
                o_trace(o, o->rho, K_CENTERED, (i + 0.0) * h, (j + 0.5) * h);
            /* advectionVThetaKernel, KaminoCore.cu:240-241 */
            if (j < nt - 1)
                o->vn[(size_t)j * np + i] =
                    o_trace(o, o->v, K_VTHETA, (i + 0.0) * h, (j + 1.0) * h);
        }
    }
    /* advectionParticles (KaminoCore.cu:321-342): forward Euler with '+'. */
    const double dt = o->dt, R = o->R;
    const int rk2 = (o->flags & FL_PARTICLE_RK2) != 0;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < o->npart; k++) {
        double posPhi = o->part[2 * k], posTheta = o->part[2 * k + 1];
        double uPhi = o_sample(o, o->u, K_VPHI, posPhi, posTheta, 1);
        double uTheta = o_sample(o, o->v, K_VTHETA, posPhi, posTheta, 1);
        double latRadius = R * sin(posTheta);
        double cofPhi = dt / latRadius, cofTheta = dt / R;
        double updatedTheta, updatedPhi;
        if (!rk2) {
            updatedTheta = posTheta + uTheta * cofTheta;
            updatedPhi = posPhi;
            if (latRadius > (double)1e-7f) updatedPhi = posPhi + uPhi * cofPhi;
        } else {
            /* midpoint rule in (phi, theta): half an Euler step, resample */
            double midTheta = posTheta + 0.5 * uTheta * cofTheta;
            double midPhi = posPhi;
            if (latRadius > (double)1e-7f) midPhi = posPhi + 0.5 * uPhi * cofPhi;
            o_validate(&midPhi, &midTheta);
            double mPhi = o_sample(o, o->u, K_VPHI, midPhi, midTheta, 1);
            double mTheta = o_sample(o, o->v, K_VTHETA, midPhi, midTheta, 1);
            double latMid = R * sin(midTheta);
            updatedTheta = posTheta + mTheta * cofTheta;
            updatedPhi = posPhi;
            if (latMid > (double)1e-7f) updatedPhi = posPhi + mPhi * (dt / latMid);
        }
        o_validate(&updatedPhi, &updatedTheta);
        o->partn[2 * k] = updatedPhi;
        o->partn[2 * k + 1] = updatedTheta;
    }
    swapp(&o->rho, &o->rhon);
    swapp(&o->part, &o->partn);
    swapp(&o->u, &o->un);
    swapp(&o->v, &o->vn);
}

/* ------------------------------------------------------------- geometric */
/* _root3 / root3 (KaminoCore.cu:386-417).  The reference loops forever on an
 * infinite argument; the oracle returns it instead. */
static double o__root3(double x)
{
    if (!isfinite(x)) return x;
    double s = 1.;
    while (x < 1.) {
        x *= 8.;
        s *= 0.5;
    }
    while (x > 8.) {
        x *= 0.125;
        s *= 2.;
    }
    double r = 1.5;
    for (int k = 0; k < 6; k++) r -= 1. / 3. * (r - x / (r * r));
    return r * s;
}

static double o_root3(double x)
{
    if (x > 0) return o__root3(x);
    if (x < 0) return -o__root3(-x);
    return 0.0;
}

/* solveCubic (KaminoCore.cu:421-454), eps = 1e-7f (:419). */
static double o_solve_cubic(double a, double b, double c)
{
    const double eps = (double)1e-7f;
    double a2 = a * a;
    double q = (a2 - 3 * b) / 9.0;
    double r = (a * (2.0 * a2 - 9.0 * b) + 27.0 * c) / 54.0;
    double r2 = r * r, q3 = q * q * q;
    if (r2 <= (q3 + eps)) {
        double t = r / sqrt(q3);
        if (t < -1) t = -1;
        if (t > 1) t = 1;
        t = acos(t);
        a /= 3.0;
        q = -2.0 * sqrt(q);
        return q * cos(t / 3.0) - a;
    }
    double A = -o_root3(fabs(r) + sqrt(r2 - q3));
    if (r < 0) A = -A;
    double B = A == 0 ? 0 : q / A;
    a /= 3.0;
    return (A + B) - a;
}

/* KaminoSolver::geometric (KaminoCore.cu:551-583): geometricFillKernel at the
 * cell centres (:457-514), then assignPhiKernel (:517-534) and
 * assignThetaKernel (:537-549). */
void oracle_geometric(oracle *o)
{
    const int nt = o->nt, np = o->np;
    const double h = o->h, dt = o->dt, R = o->R;
    const double eps = (double)1e-7f;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; j++) {
        double gTheta = (j + 0.5) * h;
        double G = dt * cos(gTheta) / (R * sin(gTheta));
        for (int i = 0; i < np; i++) {
            int ir = (i + 1) & o->mask, opp = (i + np / 2) & o->mask;
            double uPrev = 0.5 * (o->u[(size_t)j * np + i] + o->u[(size_t)j * np + ir]);
            double vPrev;
            if (j == 0)
                vPrev = 0.75 * o->v[i] + 0.25 * o->v[opp];
            else if (j == nt - 1)
                vPrev = 0.75 * o->v[(size_t)(j - 1) * np + i] +
                        0.25 * o->v[(size_t)(j - 1) * np + opp];
            else
                vPrev = 0.5 * (o->v[(size_t)(j - 1) * np + i] + o->v[(size_t)j * np + i]);
            double uNext;
            if (fabs(G) > eps) {
                double cof = G * G;
                double B = (G * vPrev + 1.0) / cof;
                double C = -uPrev / cof;
                uNext = o_solve_cubic(0.0, B, C);
            } else {
                uNext = uPrev;
            }
            o->cu[(size_t)j * np + i] = uNext;
            o->cv[(size_t)j * np + i] = vPrev + G * uNext * uNext;
        }
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; j++) {
        for (int i = 0; i < np; i++) {
            int il = i == 0 ? np - 1 : i - 1;
            o->un[(size_t)j * np + i] =
                0.5 * (o->cu[(size_t)j * np + il] + o->cu[(size_t)j * np + i]);
            if (j < nt - 1)
                o->vn[(size_t)j * np + i] =
                    0.5 * (o->cv[(size_t)j * np + i] + o->cv[(size_t)(j + 1) * np + i]);
        }
    }
    swapp(&o->u, &o->un);
    swapp(&o->v, &o->vn);
}

/* ------------------------------------------------------------ projection */
/* fillDivergenceKernel (KaminoCore.cu:587-638) in FP64, on any u, v. */
static void o_divergence_rows(const oracle *o, const double *u, const double *v, double *div)
{
    const int nt = o->nt, np = o->np;
    const double h = o->h;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; j++) {
        double th = (j + 0.5) * h, half = 0.5 * h;
        double invs = 1.0 / sin(th), sN = sin(th - half), sS = sin(th + half);
        double factor = invs / h;
        for (int i = 0; i < np; i++) {
            double uW = u[(size_t)j * np + i], uE = u[(size_t)j * np + ((i + 1) & o->mask)];
            double vN = j != 0 ? v[(size_t)(j - 1) * np + i] : 0.0;
            double vS = j != nt - 1 ? v[(size_t)j * np + i] : 0.0;
            div[(size_t)j * np + i] = factor * (vS * sS - vN * sN) + factor * (uE - uW);
        }
    }
}

/* In-place radix-2 complex FFT of length n (power of two), e^{sign*2pi i}. */
static void o_fft(double *re, double *im, int n, const double *twr, const double *twi, int tstride,
                  int inverse)
{
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i];
            re[i] = re[j];
            re[j] = t;
            t = im[i];
            im[i] = im[j];
            im[j] = t;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int step = (n / len) * tstride;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < len / 2; k++) {
                double wr = twr[k * step], wi = inverse ? -twi[k * step] : twi[k * step];
                double ar = re[i + k], ai = im[i + k];
                double br = re[i + k + len / 2], bi = im[i + k + len / 2];
                double tr = br * wr - bi * wi, ti = br * wi + bi * wr;
                re[i + k] = ar + tr;
                im[i + k] = ai + ti;
                re[i + k + len / 2] = ar - tr;
                im[i + k + len / 2] = ai - ti;
            }
        }
    }
}

/* c_m = (1/nPhi) sum_j f_j e^{-2 pi i j m / nPhi} for m = 1..nt, through a
 * length-nt complex FFT of z_k = f_{2k} + i f_{2k+1}. */
static void o_row_forward(const oracle *o, const double *f, double *cre, double *cim, double *zr,
                          double *zi)
{
    const int n = o->nt;
    for (int k = 0; k < n; k++) {
        zr[k] = f[2 * k];
        zi[k] = f[2 * k + 1];
    }
    o_fft(zr, zi, n, o->twr, o->twi, 1, 0);
    const double scale = 1.0 / o->np;
    for (int m = 1; m <= n; m++) {
        int a = m % n, b = (n - m) % n;
        double er = 0.5 * (zr[a] + zr[b]), ei = 0.5 * (zi[a] - zi[b]);
        double orr = 0.5 * (zi[a] + zi[b]), oi = -0.5 * (zr[a] - zr[b]);
        double wr = o->rtr[m], wi = o->rti[m];
        cre[m - 1] = (er + wr * orr - wi * oi) * scale;
        cim[m - 1] = (ei + wr * oi + wi * orr) * scale;
    }
}

/* p_j = sum_{m=1}^{nt-1} 2 Re(U_m e^{2 pi i j m / nPhi}) + U_nt (-1)^j. */
static void o_row_inverse(const oracle *o, const double *ure, const double *uim, double *p,
                          double *zr, double *zi)
{
    const int n = o->nt;
    /* X_m for m = 0..2n-1 is Hermitian with X_0 = 0, X_m = U_m, X_n = U_n.
     * Y_m = (X_m + X_{m+n}) + i (X_m - X_{m+n}) e^{i pi m / n}, z = IDFT_n(Y)
     * gives z_k = p_{2k} + i p_{2k+1}. */
    for (int m = 0; m < n; m++) {
        /* X_m (X_0 = 0: the m = 0 mode is dropped) and X_{m+n}: X_n = U_n is
         * the real Nyquist mode, X_{m+n} = conj(U_{n-m}) otherwise. */
        double xr = m == 0 ? 0.0 : ure[m - 1], xi = m == 0 ? 0.0 : uim[m - 1];
        double yr = m == 0 ? ure[n - 1] : ure[n - m - 1];
        double yi = m == 0 ? 0.0 : -uim[n - m - 1];
        double sr = xr + yr, si = xi + yi;
        double dr = xr - yr, di = xi - yi;
        double er = o->rtr[m], ei = -o->rti[m]; /* e^{+i pi m/n} */
        double tr = dr * er - di * ei, ti = dr * ei + di * er;
        zr[m] = sr - ti;
        zi[m] = si + tr;
    }
    o_fft(zr, zi, n, o->twr, o->twi, 1, 1);
    for (int k = 0; k < n; k++) {
        p[2 * k] = zr[k];
        p[2 * k + 1] = zi[k];
    }
}

/* KaminoSolver::projection (KaminoCore.cu:749-842). */
void oracle_projection(oracle *o)
{
    const int nt = o->nt, np = o->np;
    const double h = o->h;
    o_divergence_rows(o, o->u, o->v, o->divbuf);
    double *spec = o->spec; /* [mode m-1][row][re,im] */
#pragma omp parallel
    {
        double *zr = zalloc(nt), *zi = zalloc(nt), *cre = zalloc(nt), *cim = zalloc(nt);
#pragma omp for schedule(static)
        for (int j = 0; j < nt; j++) {
            o_row_forward(o, o->divbuf + (size_t)j * np, cre, cim, zr, zi);
            for (int m = 0; m < nt; m++) {
                spec[2 * ((size_t)m * nt + j)] = cre[m];
                spec[2 * ((size_t)m * nt + j) + 1] = cim[m];
            }
        }
        free(zr);
        free(zi);
        free(cre);
        free(cim);
    }
    /* per-mode tridiagonal solve (crKernel, tdm.cu:3-96), Thomas in FP64 */
#pragma omp parallel
    {
        double *cp = zalloc(nt), *dr = zalloc(nt), *di = zalloc(nt);
#pragma omp for schedule(static)
        for (int m = 1; m <= nt; m++) {
            double *s = spec + 2 * (size_t)(m - 1) * nt;
            double n2 = (double)m * (double)m;
            for (int i = 0; i < nt; i++) {
                double a = o->lapA[i], b = o->lapB0[i] - n2 * o->lapS[i], c = o->lapC[i];
                double den = i ? b - a * cp[i - 1] : b;
                cp[i] = c / den;
                dr[i] = (s[2 * i] - (i ? a * dr[i - 1] : 0.0)) / den;
                di[i] = (s[2 * i + 1] - (i ? a * di[i - 1] : 0.0)) / den;
            }
            for (int i = nt - 2; i >= 0; i--) {
                dr[i] -= cp[i] * dr[i + 1];
                di[i] -= cp[i] * di[i + 1];
            }
            for (int i = 0; i < nt; i++) {
                s[2 * i] = dr[i];
                s[2 * i + 1] = di[i];
            }
        }
        free(cp);
        free(dr);
        free(di);
    }
    /* synthesis without the m = 0 mode (copy2UFourier .. shiftUKernel,
     * KaminoCore.cu:658-703) */
#pragma omp parallel
    {
        double *zr = zalloc(nt), *zi = zalloc(nt), *ur = zalloc(nt), *ui = zalloc(nt);
#pragma omp for schedule(static)
        for (int j = 0; j < nt; j++) {
            for (int m = 0; m < nt; m++) {
                ur[m] = spec[2 * ((size_t)m * nt + j)];
                ui[m] = spec[2 * ((size_t)m * nt + j) + 1];
            }
            o_row_inverse(o, ur, ui, o->p + (size_t)j * np, zr, zi);
        }
        free(zr);
        free(zi);
        free(ur);
        free(ui);
    }
    /* applyPressureTheta / applyPressurePhi (KaminoCore.cu:705-747) */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; j++) {
        double thetaBelt = (j + 0.5) * h;
        double hs = -h * sin(thetaBelt);
        for (int i = 0; i < np; i++) {
            int iw = i == 0 ? np - 1 : i - 1;
            double pW = o->p[(size_t)j * np + iw], pE = o->p[(size_t)j * np + i];
            o->un[(size_t)j * np + i] = o->u[(size_t)j * np + i] + (pE - pW) / hs;
            if (j < nt - 1) {
                double pN = o->p[(size_t)j * np + i], pS = o->p[(size_t)(j + 1) * np + i];
                o->vn[(size_t)j * np + i] = o->v[(size_t)j * np + i] + (pS - pN) / (-h);
            }
        }
    }
    swapp(&o->u, &o->un);
    swapp(&o->v, &o->vn);
}

void oracle_step(oracle *o, int n)
{
    for (int k = 0; k < n; k++) {
        oracle_advection(o);
        oracle_geometric(o);
        oracle_projection(o);
    }
}

/* The reference's discrete divergence (fillDivergenceKernel) of the oracle's
 * current velocity, or of given dense float fields when u, v are non-NULL. */
void oracle_divergence(oracle *o, const float *u, const float *v, double *div)
{
    if (u && v) {
        size_t fs = o->rows_alloc * (size_t)o->np;
        double *uu = zalloc(fs), *vv = zalloc(fs);
        for (size_t i = 0; i < (size_t)o->nt * o->np; i++) uu[i] = u[i];
        for (size_t i = 0; i < (size_t)(o->nt - 1) * o->np; i++) vv[i] = v[i];
        o_divergence_rows(o, uu, vv, div);
        free(uu);
        free(vv);
    } else {
        o_divergence_rows(o, o->u, o->v, div);
    }
}

/* ================================================================ ref32
 * The index stage of the samplers in the reference's own arithmetic: fReal
 * is float (KaminoHeader.cuh:48); M_PI, M_2PI and the staggering offsets are
 * double literals (:26-41), so each expression they touch is evaluated in
 * double and rounded to float on assignment.  floorf takes a float, so a
 * double argument is first rounded to float. */
static float r_validate(float *phi, float *theta)
{
    float ret = 1.0f;
    {
        float q = (float)((double)*theta / O_2PI);
        int n = (int)floorf(q);
        *theta = (float)((double)*theta - (double)n * O_2PI);
    }
    if ((double)*theta > O_PI) {
        *theta = (float)(O_2PI - (double)*theta);
        *phi = (float)((double)*phi + O_PI);
        ret = -ret;
    }
    if (*theta < 0) {
        *theta = -*theta;
        *phi = (float)((double)*phi + O_PI);
        ret = -ret;
    }
    {
        float q = (float)((double)*phi / O_2PI);
        int n = (int)floorf(q);
        *phi = (float)((double)*phi - (double)n * O_2PI);
    }
    return ret;
}

/* (phiIndex, thetaIndex, flipped, pole branch) and (alphaPhi, alphaTheta) of
 * sampleVPhi / sampleVTheta / sampleCentered (KaminoCore.cu:38-52, 88-103,
 * 138-153) for n raw coordinates; h is gridLenGlobal (float). */
void oracle_ref_index(int kind, const float *phiRaw, const float *thetaRaw, int64_t n, float h,
                      int nt, int32_t *out, float *alpha)
{
    static const double offp[3] = {-0.5, 0.0, 0.0};
    static const double offt[3] = {0.5, 1.0, 0.5};
    for (int64_t k = 0; k < n; k++) {
        float phi = (float)((double)phiRaw[k] - (double)h * offp[kind]);
        float theta = (float)((double)thetaRaw[k] - (double)h * offt[kind]);
        float invGridLen = (float)(1.0 / (double)h);
        float flip = r_validate(&phi, &theta);
        float normedPhi = phi * invGridLen;
        float normedTheta = theta * invGridLen;
        int phiIndex = (int)floorf(normedPhi);
        int thetaIndex = (int)floorf(normedTheta);
        float alphaPhi = normedPhi - (float)phiIndex;
        float alphaTheta = normedTheta - (float)thetaIndex;
        int pole_row = kind == K_VTHETA ? nt - 2 : nt - 1;
        int pole = (thetaIndex == 0 && flip == -1.0f) || thetaIndex == pole_row;
        /* phiIndex % nPhi in size_t arithmetic; nPhi is a power of two */
        out[4 * k + 0] = (int32_t)((uint64_t)(int64_t)phiIndex % (uint64_t)(2 * nt));
        out[4 * k + 1] = thetaIndex;
        out[4 * k + 2] = flip == -1.0f;
        out[4 * k + 3] = pole;
        if (alpha) {
            alpha[2 * k] = alphaPhi;
            alpha[2 * k + 1] = alphaTheta;
        }
    }
}

/* validateCoord on n coordinate pairs in place, then the particle cell
 * index floor(phi/h), floor(theta/h) of KaminoParticles.cu:56-57. */
void oracle_ref_wrap(float *phi, float *theta, int64_t n, float h, int32_t *cells)
{
    for (int64_t k = 0; k < n; k++) {
        r_validate(&phi[k], &theta[k]);
        if (cells) {
            cells[2 * k] = (int32_t)floorf(phi[k] / h);
            cells[2 * k + 1] = (int32_t)floorf(theta[k] / h);
        }
    }
}

/* ============================================================ FBM init
 * KaminoSolver::initialize_velocity with its FBM / interpNoise2D / rand
 * (KaminoInitializer.cu:3-134) in the reference's arithmetic: fReal is
 * float; vec2 holds doubles (vectorUtil.cuh:9-24), so rand's dot product is
 * double, rounded to float on assignment; the sin argument mixes a float
 * and a double literal (double); kaminoLerpHost's (1.0 - alpha) makes its
 * first product double; std::pow(float, int) returns double (exact powers of
 * two here). */
static float r_rand(double x, double y)
{
    const float dot = (float)(x * 12.9898 + y * 4.1414);
    const float val = (float)sin((double)dot * 43758.5453);
    return val - floorf(val);
}
static float r_lerp(float from, float to, float alpha)
{
    return (float)((1.0 - (double)alpha) * (double)from + (double)(alpha * to));
}
static float r_noise2(float x, float y)
{
    const float ix = floorf(x), fx = x - ix, iy = floorf(y), fy = y - iy;
    const float v1 = r_rand(ix, iy), v2 = r_rand(ix + 1, iy), v3 = r_rand(ix, iy + 1), v4 = r_rand(ix + 1, iy + 1);
    return r_lerp(r_lerp(v1, v2, fx), r_lerp(v3, v4, fx), fy);
}
static float r_fbm(float x, float y)
{
    float total = 0.0f;
    const float resX = (float)0.15, resY = (float)0.5, pers = (float)0.5;
    for (int i = 0; i < 4; i++) {
        const float freq = (float)pow(2.0, i), amp = (float)pow((double)pers, i);
        total += amp * r_noise2(x * freq / resX, y * freq / resY);
    }
    const float a = 1 - pers;
    return a * total / 2.0f;
}

/* u_phi (nt rows) and u_theta (nt-1 rows) of nPhi = 2 nt columns; h is
 * gridLen (float) and radius the float radius. */
void oracle_ref_init_fbm(int nt, float radius, float h, float *u, float *v)
{
    const int np = 2 * nt;
    const float gain = (float)(4096.0 / np);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; j++) {
        for (int i = 0; i < np; i++) {
            float urx, ury, lrx, lry, ulx, uly, llx, lly;
            if (i > 0) {
                urx = (float)i * h + h / 2;
                ulx = (float)i * h - h / 2;
            } else {  /* the phi = 0 seam: the west points wrap to 2 pi */
                urx = h / 2;
                ulx = (float)(2 * O_PI - (double)(h / 2));
            }
            lrx = urx;
            llx = ulx;
            ury = uly = (float)(j + 1) * h;
            lry = lly = (float)j * h;
            const float nur = r_fbm(urx, ury), nlr = r_fbm(lrx, lry), nul = r_fbm(ulx, uly), nll = r_fbm(llx, lly);
            const float dl = (nur - nlr) / (radius * h), dr = (nul - nll) / (radius * h);
            const float avg = (float)((double)(dl + dr) / 2.0);
            u[(size_t)j * np + i] = avg * gain;
        }
    }
#pragma omp parallel for schedule(static)
    for (int j = 1; j < nt; j++) {
        for (int i = 0; i < np; i++) {
            /* as the reference: the lower-left point sits at + h/2, like the upper-left */
            const float urx = (float)(i + 1) * h, ury = (float)j * h + h / 2;
            const float lrx = (float)(i + 1) * h, lry = (float)j * h - h / 2;
            const float ulx = (float)i * h, uly = (float)j * h + h / 2;
            const float llx = (float)i * h, lly = (float)j * h + h / 2;
            const float nur = r_fbm(urx, ury), nlr = r_fbm(lrx, lry), nul = r_fbm(ulx, uly), nll = r_fbm(llx, lly);
            const float du = -1 * (nur - nul) / (radius * h), dd = -1 * (nlr - nll) / (radius * h);
            const float avg = (float)((double)(du + dd) / 2.0);
            v[(size_t)(j - 1) * np + i] = avg * gain;
        }
    }
}

/* ------------------------------------------------------------------------
 * 3. Frame output records (oracle_frame_*), in the reference's host float
 * arithmetic: KaminoSolver::write_data_bgeo (KaminoSolver.cu:284-357) and
 * write_particles_bgeo (:359-396) with mapPToSphere / mapVToSphere
 * (:398-423).  fReal is float; the vec3 components are double, so the
 * cell-centre coordinates are exact double products rounded to float by
 * the float locals of the map functions, and every other expression is a
 * float expression (sinf / cosf are the float overloads the reference's
 * sin / cos of a float resolve to).  Records are native-order floats:
 * grid x y z 1 vx vy vz density (rows j, then columns i); particles
 * x y z 1 0 0 0 r g b with zero colour (no colour image).
 */
void oracle_frame_grid(int nt, float radius, float h, const float *u, const float *v, const float *rho,
                       float *rec)
{
    const int np = 2 * nt;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nt; ++j) {
        for (int i = 0; i < np; ++i) {
            const int ie = (i == np - 1) ? 0 : i + 1;
            int jn, js;
            if (j == 0) {
                jn = js = 0;
            } else if (j == nt - 1) {
                jn = js = nt - 2;
            } else {
                jn = j - 1;
                js = j;
            }
            const float uWest = u[(size_t)j * np + i], uEast = u[(size_t)j * np + ie];
            const float vNorth = v[(size_t)jn * np + i], vSouth = v[(size_t)js * np + i];
            const float velocityPhi = (float)((double)(uWest + uEast) / 2.0);
            const float velocityTheta = (float)((double)(vNorth + vSouth) / 2.0);
            const float phi = (float)(((double)i + 0.0) * (double)h);
            const float theta = (float)(((double)j + 0.5) * (double)h);
            float *r = rec + 8 * ((size_t)j * np + i);
            r[4] = cosf(theta) * cosf(phi) * velocityTheta - sinf(phi) * velocityPhi;
            r[6] = cosf(theta) * sinf(phi) * velocityTheta + cosf(phi) * velocityPhi;
            r[5] = -sinf(theta) * velocityTheta;
            r[0] = radius * sinf(theta) * cosf(phi);
            r[2] = radius * sinf(theta) * sinf(phi);
            r[1] = radius * cosf(theta);
            r[3] = 1.0f;
            r[7] = rho[(size_t)j * np + i];
        }
    }
}

void oracle_frame_particles(float radius, const float *part, int64_t n, float *rec)
{
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        const float phi = part[2 * k], theta = part[2 * k + 1];
        float *r = rec + 10 * k;
        r[0] = radius * sinf(theta) * cosf(phi);
        r[2] = radius * sinf(theta) * sinf(phi);
        r[1] = radius * cosf(theta);
        r[3] = 1.0f;
        for (int c = 4; c < 10; ++c) r[c] = 0.0f;
    }
}

/* KaminoParticles::KaminoParticles (KaminoParticles.cu:20-62) without a
 * colour image: the jittered particle grid, drawn with the C library's
 * srand(seed) / rand() as the reference does (it never seeds: seed 1), in its
 * float arithmetic (fReal variables, double literals M_PI, 0.5, 2.0, 0.0).
 * out: (phi, theta) pairs, index i * numTheta + j.  Returns the count. */
int64_t oracle_ref_particles(float particleDensity, int nTheta, unsigned seed, float *out)
{
    const float linearDensity = sqrtf(particleDensity);
    const float delta = (float)(3.14159265358979323846 / (double)(size_t)nTheta / (double)linearDensity);
    const float halfDelta = (float)((double)delta / 2.0);
    const unsigned numThetaParticles = (unsigned)(linearDensity * (float)(size_t)nTheta);
    const unsigned numPhiParticles = 2 * numThetaParticles;
    srand(seed);
    for (unsigned i = 0; i < numPhiParticles; ++i) {
        for (unsigned j = 0; j < numThetaParticles; ++j) {
            float signPhi = (float)rand() / (float)RAND_MAX;
            signPhi = (double)signPhi >= 0.5 ? 1.0f : -1.0f;
            float signTheta = (float)rand() / (float)RAND_MAX;
            signTheta = (double)signTheta >= 0.5 ? 1.0f : -1.0f;
            float randPhi = signPhi * halfDelta * (float)rand() / (float)RAND_MAX;
            float randTheta = signTheta * halfDelta * (float)rand() / (float)RAND_MAX;
            float phi = (float)i * delta + randPhi;
            float theta = (float)j * delta + randTheta;
            if ((double)phi < 0.0) phi = 0.0f;
            if ((double)theta < 0.0) theta = 0.0f;
            size_t index = (size_t)i * numThetaParticles + j;
            out[2 * index] = phi;
            out[2 * index + 1] = theta;
        }
    }
    return (int64_t)numThetaParticles * numPhiParticles;
}

/* Image input (KaminoSolver::initDensityfromPic, KaminoSolver.cu:243-277;
 * KaminoParticles' colours, KaminoParticles.cu:6-17, 56-72), restated for
 * the library's resampling: the image mirrored left-right (cv::flip code 1)
 * and resampled to dw x dh pixels bilinearly at half-pixel centres with the
 * edges clamped (cv::resize INTER_LINEAR placement), columns then rows, in
 * float with -ffp-contract=off, each channel rounded to nearest (ties to
 * even) and clamped to 8 bits.  OpenCV's own 8-bit path uses fixed-point
 * weights, so its pixels can differ from these by one level.
 * out: dw * dh pixels of 3 bytes (B, G, R), rows of dw. */
static void o_axis(int src, int dst, int mirror, int *i0, int *i1, float *a)
{
    const double scale = (double)src / dst;
    for (int d = 0; d < dst; d++) {
        const float f = (float)((d + 0.5) * scale - 0.5);
        int s0 = (int)floorf(f);
        float w = f - (float)s0;
        if (s0 < 0) {
            s0 = 0;
            w = 0.0f;
        }
        if (s0 >= src - 1) {
            s0 = src - 1;
            w = 0.0f;
        }
        int s1 = s0 + 1 < src - 1 ? s0 + 1 : src - 1;
        if (mirror) {
            s0 = src - 1 - s0;
            s1 = src - 1 - s1;
        }
        i0[d] = s0;
        i1[d] = s1;
        a[d] = w;
    }
}

void oracle_image_resample(const unsigned char *img, int w, int h, size_t stride, int dw, int dh,
                           unsigned char *out)
{
    int *xi0 = malloc(sizeof(int) * dw), *xi1 = malloc(sizeof(int) * dw);
    int *yi0 = malloc(sizeof(int) * dh), *yi1 = malloc(sizeof(int) * dh);
    float *xa = malloc(sizeof(float) * dw), *ya = malloc(sizeof(float) * dh);
    o_axis(w, dw, 1, xi0, xi1, xa);
    o_axis(h, dh, 0, yi0, yi1, ya);
    for (int j = 0; j < dh; j++) {
        const unsigned char *r0 = img + (size_t)yi0[j] * stride, *r1 = img + (size_t)yi1[j] * stride;
        for (int i = 0; i < dw; i++) {
            for (int k = 0; k < 3; k++) {
                const float ax = xa[i], ay = ya[j];
                const float h0 = (float)r0[3 * xi0[i] + k] * (1.0f - ax) + (float)r0[3 * xi1[i] + k] * ax;
                const float h1 = (float)r1[3 * xi0[i] + k] * (1.0f - ax) + (float)r1[3 * xi1[i] + k] * ax;
                long v = lrintf(h0 * (1.0f - ay) + h1 * ay);
                out[3 * ((size_t)j * dw + i) + k] = (unsigned char)(v < 0 ? 0 : v > 255 ? 255 : v);
            }
        }
    }
    free(xi0);
    free(xi1);
    free(yi0);
    free(yi1);
    free(xa);
    free(ya);
}
