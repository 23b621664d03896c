/* TEST INFRASTRUCTURE: the seeded synthetic initial state, on the CPU side.
 *
 * The benchmark workloads and the parity tests start from a seeded state: a
 * stream function of orthonormal real spherical harmonics (l <= lmax, N(0,1)
 * coefficients) plus an optional Gaussian vortex, its curl evaluated at the
 * staggered (theta, phi) points, velocities scaled so max|u| is
 * velocity_scale; thickness 1 + a U(-1,1); particles uniform on the sphere.
 * The library makes it with kamino_make_initial_state; this file restates the
 * same generator (same splitmix64-seeded xoshiro256** streams, the same
 * Legendre recurrences, the same order of double operations, built without
 * contraction as the library is), so that the CPU arm of the benchmark and
 * the oracle-side tests build the identical inputs without loading the
 * product library.  tests/test_oracle.py checks the two bit for bit.
 *
 * None of this is the reference's: the reference initialises velocity from
 * FBM curl noise and thickness from an image (KaminoInitializer.cu,
 * KaminoSolver.cu:243-277); the seeded spherical-harmonic state is this
 * project's workload definition. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
    uint64_t s[4];
} synth_rng;

static uint64_t synth_splitmix(uint64_t* x)
{
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void synth_seed(synth_rng* r, uint64_t seed)
{
    uint64_t x = seed;
    for (int k = 0; k < 4; k++) r->s[k] = synth_splitmix(&x);
}

static uint64_t synth_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t synth_next(synth_rng* r)
{
    uint64_t* s = r->s;
    uint64_t res = synth_rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = synth_rotl(s[3], 45);
    return res;
}

static double synth_uniform(synth_rng* r) { return (double)(synth_next(r) >> 11) * (1.0 / 9007199254740992.0); }

static double synth_normal(synth_rng* r)
{
    double u1 = synth_uniform(r), u2 = synth_uniform(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

/* one stream per quantity, so adding particles leaves the velocity alone */
enum { SYNTH_SH = 1, SYNTH_THICK = 2, SYNTH_PART = 3, SYNTH_VORTEX = 4 };
static uint64_t synth_stream(uint64_t seed, int stream)
{
    return seed * 0x2545F4914F6CDD1Dull + 0x9E37u * (uint64_t)stream;
}

/* Orthonormal associated Legendre Pbar_l^m(cos theta), l <= L, and their
 * theta-derivatives, [l][m] with row width L + 1. */
static void synth_legendre(int L, double theta, double* P, double* dP)
{
    const int W = L + 1;
    memset(P, 0, sizeof(double) * W * W);
    memset(dP, 0, sizeof(double) * W * W);
    double x = cos(theta), s = sin(theta);
    P[0] = sqrt(1.0 / (4.0 * M_PI));
    for (int m = 1; m <= L; m++) P[(size_t)m * W + m] = sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * P[(size_t)(m - 1) * W + m - 1];
    for (int m = 0; m < L; m++) P[(size_t)(m + 1) * W + m] = sqrt(2.0 * m + 3.0) * x * P[(size_t)m * W + m];
    for (int m = 0; m <= L; m++)
        for (int l = m + 2; l <= L; l++) {
            double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
            P[(size_t)l * W + m] = a * (x * P[(size_t)(l - 1) * W + m] - b * P[(size_t)(l - 2) * W + m]);
        }
    /* sin(theta) dPbar_l^m/dtheta = l cos(theta) Pbar_l^m
     *                               - sqrt((l^2-m^2)(2l+1)/(2l-1)) Pbar_{l-1}^m */
    for (int l = 0; l <= L; l++)
        for (int m = 0; m <= l; m++) {
            double v = l * x * P[(size_t)l * W + m];
            if (l > m) v -= sqrt(((double)l * l - (double)m * m) * (2.0 * l + 1.0) / (2.0 * l - 1.0)) * P[(size_t)(l - 1) * W + m];
            dP[(size_t)l * W + m] = v / s;
        }
}

/* Returns 0, or -1 for an invalid argument.  u_phi [nt][2nt], u_theta
 * [nt-1][2nt], thickness [nt][2nt], particles [n][2] (phi, theta); any may be
 * NULL.  vortex_out: centre theta, centre phi, amplitude after scaling. */
int oracle_make_initial_state(int nt, int lmax, uint64_t seed, double radius, double thickness_noise, int vortex,
                              double vortex_sigma, double vortex_amplitude, double velocity_scale,
                              int64_t n_particles, float* u_phi, float* u_theta, float* thickness,
                              float* particles, double* vortex_out)
{
    if (nt < 4 || (nt & (nt - 1)) || lmax < 1 || lmax > 256 || !(radius > 0)) return -1;
    const int np = 2 * nt, L = lmax, W = L + 1;
    const double h = M_PI / nt, R = radius;
    double* ca = calloc((size_t)W * W, sizeof(double));
    double* cb = calloc((size_t)W * W, sizeof(double));
    double* up = malloc(sizeof(double) * (size_t)nt * np);
    double* vt = malloc(sizeof(double) * (size_t)(nt - 1) * np);
    if (!ca || !cb || !up || !vt) {
        free(ca), free(cb), free(up), free(vt);
        return -1;
    }
    {
        synth_rng rng;
        synth_seed(&rng, synth_stream(seed, SYNTH_SH));
        for (int l = 1; l <= L; l++)
            for (int m = 0; m <= l; m++) {
                double s = m ? sqrt(2.0) : 1.0;
                ca[(size_t)l * W + m] = s * synth_normal(&rng);
                cb[(size_t)l * W + m] = m ? s * synth_normal(&rng) : 0.0;
            }
    }
    double vth = 0, vph = 0, vamp = 0, vsig = vortex_sigma;
    if (vortex) {
        synth_rng rng;
        synth_seed(&rng, synth_stream(seed, SYNTH_VORTEX));
        vth = acos(1.0 - 2.0 * synth_uniform(&rng));
        vph = 2.0 * M_PI * synth_uniform(&rng);
        double a = 0.5 + synth_uniform(&rng);
        if (synth_uniform(&rng) < 0.5) a = -a;
        vamp = vortex_amplitude != 0.0 ? vortex_amplitude : a * vsig * exp(0.5);
        if (!(vsig > 0)) {
            free(ca), free(cb), free(up), free(vt);
            return -1;
        }
    }
    const double cc = cos(vth), sc = sin(vth);
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < 2 * nt - 1; j++) {
        const int isu = j < nt, row = isu ? j : j - nt;
        const double theta = isu ? (row + 0.5) * h : (row + 1.0) * h;
        double* P = malloc(sizeof(double) * W * W * 2 + sizeof(double) * W * 4);
        double *dP = P + W * W, *Ac = dP + W * W, *As = Ac + W, *dAc = As + W, *dAs = dAc + W;
        synth_legendre(L, theta, P, dP);
        for (int m = 0; m < W; m++) Ac[m] = As[m] = dAc[m] = dAs[m] = 0.0;
        for (int m = 0; m <= L; m++)
            for (int l = m > 1 ? m : 1; l <= L; l++) {
                size_t k = (size_t)l * W + m;
                Ac[m] += ca[k] * P[k];
                As[m] += cb[k] * P[k];
                dAc[m] += ca[k] * dP[k];
                dAs[m] += cb[k] * dP[k];
            }
        for (int i = 0; i < np; i++) {
            const double phi = isu ? (i - 0.5) * h : i * h;
            double dth = 0, dph = 0;
            for (int m = 0; m <= L; m++) {
                double cm = cos(m * phi), sm = sin(m * phi);
                dth += dAc[m] * cm + dAs[m] * sm;
                dph += m * (-Ac[m] * sm + As[m] * cm);
            }
            if (vortex) {
                double ct = cos(theta), st = sin(theta);
                double dp = phi - vph;
                double cosd = ct * cc + st * sc * cos(dp);
                double psi = vamp * exp((cosd - 1.0) / (vsig * vsig));
                dth += psi / (vsig * vsig) * (-st * cc + ct * sc * cos(dp));
                dph += psi / (vsig * vsig) * (-st * sc * sin(dp));
            }
            if (isu)
                up[(size_t)row * np + i] = -dth / R;
            else
                vt[(size_t)row * np + i] = dph / (R * sin(theta));
        }
        free(P);
    }
    double scale = 1.0;
    if (velocity_scale > 0) {
        double mx = 0;
        for (size_t k = 0; k < (size_t)nt * np; k++) mx = fmax(mx, fabs(up[k]));
        for (size_t k = 0; k < (size_t)(nt - 1) * np; k++) mx = fmax(mx, fabs(vt[k]));
        if (mx > 0) scale = velocity_scale / mx;
    }
    if (u_phi)
        for (size_t k = 0; k < (size_t)nt * np; k++) u_phi[k] = (float)(up[k] * scale);
    if (u_theta)
        for (size_t k = 0; k < (size_t)(nt - 1) * np; k++) u_theta[k] = (float)(vt[k] * scale);
    if (thickness) {
        synth_rng rng;
        synth_seed(&rng, synth_stream(seed, SYNTH_THICK));
        for (size_t k = 0; k < (size_t)nt * np; k++)
            thickness[k] = (float)(1.0 + thickness_noise * (2.0 * synth_uniform(&rng) - 1.0));
    }
    if (particles && n_particles > 0) {
        synth_rng rng;
        synth_seed(&rng, synth_stream(seed, SYNTH_PART));
        for (int64_t k = 0; k < n_particles; k++) {
            double th = acos(1.0 - 2.0 * synth_uniform(&rng));
            double ph = 2.0 * M_PI * synth_uniform(&rng);
            particles[2 * k] = (float)ph;
            particles[2 * k + 1] = (float)th;
        }
    }
    if (vortex_out) {
        vortex_out[0] = vth;
        vortex_out[1] = vph;
        vortex_out[2] = vamp * scale;
    }
    free(ca), free(cb), free(up), free(vt);
    return 0;
}
