// kamino_common.h — shared host/device declarations of the GB300 solver.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime.h>
#include <vector_types.h>

#include "../../include/kamino_gb300.h"

// Records a formatted message as the thread's last error and returns code.
int kamino_fail(int code, const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;

#ifdef __cplusplus
#include <vector>
// Host tables shared by the solver units (kamino_solver.cu).
void laplacian_rows(int nt, std::vector<double>& A, std::vector<double>& C, std::vector<double>& B0,
                    std::vector<double>& S);
void fp64_tables(int nt, int nmodes, const std::vector<double>& A, const std::vector<double>& C,
                 const std::vector<double>& S, std::vector<double>& out);
#endif

// Internal hooks for the batched and served forms (kamino_batch.cu): they
// advance many handles with shared launches and keep each handle's
// bookkeeping (buffer parity, step count) in step.
struct KGeo;
struct KBufs;
int kamino_internal_desc(kamino_handle h, KGeo* g, KBufs* b, int* nfp64, int* cur_uv, int* cur_r);
int kamino_internal_advance(kamino_handle h, int nsteps);
int kamino_internal_get_counters(kamino_handle h, int* cur_uv, int* cur_r, int64_t* steps, double* time);
int kamino_internal_set_counters(kamino_handle h, int cur_uv, int cur_r, int64_t steps, double time);
// Re-targets a handle of the same nTheta to a new radius / dt / flags and
// zeroes its state, so pooled device memory can serve a new request.
int kamino_internal_reset(kamino_handle h, const kamino_config* cfg);
// Rebuilds the particles' visiting order (KBufs::pperm) on the handle's
// stream when it is due (*launched: whether it did); the batched engine
// calls it before its steps.
int kamino_internal_sort_particles(kamino_handle h, int* launched);
// The handle's own stream (its steps and copies are ordered on it).
cudaStream_t kamino_internal_stream(kamino_handle h);
// The handle's configuration as created.
int kamino_internal_config(kamino_handle h, kamino_config* cfg);
// Evicts the L2 on the handle's stream (a write and a read of a buffer larger
// than L2), for timing entry points.
int kamino_internal_flush_l2(kamino_handle h);
// Frame output (kamino_frames.cu): the handle's frame state, made current
// with the handle's device; released by kamino_destroy.
struct KFrames;
int kamino_internal_frames(kamino_handle h, KFrames*** out);
void kamino_frames_release(KFrames* f);

#define KAMINO_PI_D 3.14159265358979323846   /* M_PI  (KaminoHeader.cuh:26) */
#define KAMINO_2PI_D 6.28318530717958647692  /* M_2PI (KaminoHeader.cuh:27) */

// Per-sphere constants, passed to kernels by value.  They replace the
// reference's process-wide __constant__ parameters (KaminoCore.cu:5-9).
struct KGeo {
    int nt;       // nTheta (power of two)
    int np;       // nPhi = 2 * nTheta
    int mask;     // nPhi - 1
    int half;     // nPhi / 2
    int log2nt;
    float h;      // gridLenGlobal = (float)(M_PI / nTheta), KaminoCore.cu:849
    float halfh;  // 0.5f * h (exact)
    float invh;   // (float)(1.0 / h), the invGridLen of the samplers
    float R;      // radiusGlobal
    float dt;     // timeStepGlobal
    float cofTheta;     // dt / R (float division, KaminoCore.cu:204)
    float cellTheta;    // dt / (R h): theta displacement in cells per unit velocity
    float pi_up;        // smallest float > M_PI: theta > M_PI  <=>  theta >= pi_up
    float wrap_phi_hi;  // smallest float x with floorf((float)(x / M_2PI)) >= 1
    int pitch;          // floats per row (== np)
    int rows;           // rows allocated per field (nt + 2; the last rows read as 0)
    uint32_t flags;     // kamino_flags
};

// Device arrays of one sphere.  Each field is [rows][pitch] floats.
struct KBufs {
    float* u[2];
    float* v[2];
    float* rho[2];
    float2* part[2];
    float* cu;       // geometric scratch: u at cell centres
    float* cv;       // geometric scratch: v at cell centres
    float* p;        // pressure
    float2* spec;    // spectrum, [mode m-1][row], m = 1..nt
    float2* sol;     // per-mode solution, [mode m-1][row]
    double* s64;     // FP64 solve multipliers, s64_stride(nt) doubles per FP64 mode
    // per-row tables
    float* cof_c;    // dt / (R sinf((j+1/2)h))   (centred rows, u_phi rows)
    float* cof_v;    // dt / (R sinf((j+1)h))     (u_theta rows)
    float* cell_c;   // dt / (R sin((j+1/2)h) h): velocity -> cells, centred rows
    float* cell_v;   // dt / (R sin((j+1)h) h):   u_theta rows
    float* gfac;     // G = dt cosf(theta) / (R sinf(theta)) at (j+1/2)h
    float* negHs;    // -h * sinf((j+1/2)h)
    float* divf;     // (1/sinf(theta_j)) / h
    float* sinN;     // sinf(theta_j - h/2)
    float* sinS;     // sinf(theta_j + h/2)
    float* lapA;     // Laplacian rows (FP32): A_i, C_i, B0_i, 1/sin^2
    float* lapC;
    float* lapB0;
    float* lapS;
    double* lapA64;  // same in FP64
    double* lapC64;
    double* lapB064;
    double* lapS64;
    float2* tw;      // e^{-2 pi i k / nt}, k < nt/2
    float2* rt;      // e^{-i pi m / nt},  m <= nt
    int64_t npart;
    // Order in which the advection visits the particles: a permutation of
    // 0 .. npart-1, rebuilt every few steps so that consecutive threads take
    // particles of the same block of cells (their gathers then share cache
    // lines).  Each particle's update does not depend on the order.  Null:
    // index order.
    const int* pperm;
};
