/*
 * kamino_gb300.h — C ABI of the GB300-native Kamino spherical fluid step.
 *
 * This header is the drop-in boundary for the per-timestep solver of Kamino
 * (KaminoGPU).  The reference exposes that solver only as C++ classes:
 *   KaminoSolver(nPhi, nTheta, radius, frameDuration, A, B, C, D, E)
 *                                  KaminoGPU/include/KaminoSolver.cuh:99-100
 *   KaminoSolver::stepForward(dt)  KaminoGPU/kernel/KaminoSolver.cu:197-221
 *   advection() / geometric() / projection()
 *                                  KaminoGPU/kernel/KaminoCore.cu:344, 551, 749
 *   Kamino::run() frame loop       KaminoGPU/kernel/KaminoCore.cu:860-912
 *   main(configKamino.txt)         KaminoGPU/kernel/main.cu:4-59
 * Every entry point below names the reference interface it replaces.
 *
 * Conventions (differences from the reference are deliberate and listed):
 *  - Every call returns an int status (KAMINO_OK == 0).  Nothing calls
 *    exit(); the reference's checkCudaErrors did (helper_cuda.h:981-995).
 *    kamino_last_error() gives the message of the last failing call.
 *  - Handles are independent.  There is no process-wide __constant__ state
 *    (the reference keeps one sphere per process, KaminoCore.cu:5-9).
 *  - A handle is thread-compatible, not thread-safe.  All its work is ordered
 *    on one CUDA stream owned by the handle.
 *  - Fields are row-major [theta][phi] float32 with a caller-chosen pitch in
 *    bytes, exactly like KaminoQuantity::copyToGPU/copyBackToCPU
 *    (KaminoQuantity.cu:3-18).  u_phi and thickness have nTheta rows,
 *    u_theta has nTheta-1 rows, nPhi = 2*nTheta columns.  Particles are
 *    interleaved (phi, theta) float pairs (KaminoParticles.cu:61-62).
 *  - nTheta must be a power of two in [32, 2048]; the reference's cyclic
 *    reduction has the same power-of-two rule (tdm.cu:11-13).
 */
#ifndef KAMINO_GB300_H
#define KAMINO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum kamino_status {
    KAMINO_OK = 0,
    KAMINO_ERR_INVALID = 1,   /* bad argument or unsupported size            */
    KAMINO_ERR_CUDA = 2,      /* a CUDA runtime call failed                  */
    KAMINO_ERR_ALLOC = 3,     /* device or host allocation failed            */
    KAMINO_ERR_IO = 4,        /* config file could not be read or parsed     */
    KAMINO_ERR_BUDGET = 5,    /* request does not fit the admission budget   */
    KAMINO_ERR_TIMEOUT = 6,   /* a bounded device-side wait gave up          */
    KAMINO_ERR_NOT_READY = 7, /* request still running                       */
    KAMINO_ERR_NOT_FOUND = 8  /* unknown request id                          */
};

/* ---------------------------------------------------------------- fields */
enum kamino_field {
    KAMINO_U_PHI = 0,      /* velPhi,   nTheta   x nPhi (KaminoSolver.cu:50) */
    KAMINO_U_THETA = 1,    /* velTheta, nTheta-1 x nPhi (KaminoSolver.cu:52) */
    KAMINO_THICKNESS = 2,  /* "density", nTheta  x nPhi (KaminoSolver.cu:56) */
    KAMINO_PRESSURE = 3,   /* p,        nTheta   x nPhi (KaminoSolver.cu:54) */
    KAMINO_PARTICLES = 4   /* (phi, theta) pairs, n_particles entries        */
};

/* ------------------------------------------------------------------ flags */
enum kamino_flags {
    /* Advect particles with RK2 (midpoint) instead of the reference's forward
     * Euler (KaminoCore.cu:321-342). */
    KAMINO_F_PARTICLE_RK2 = 1u << 0,
    /* Negate u_phi / u_theta samples taken across a pole.  The reference does
     * not (KaminoCore.cu:43,52,93,102); off by default for parity. */
    KAMINO_F_POLE_SIGN_FLIP = 1u << 1,
    /* Use the dt passed to kamino_step().  The reference ignores it and uses
     * the configured dt (KaminoSolver.cu:199, KaminoCore.cu:871). */
    KAMINO_F_HONOR_STEP_DT = 1u << 2,
    /* 1u << 3 is reserved (the pressure is read back by the u_theta
     * gradient, so a step always writes it). */
    /* Evaluate sample positions in radians with the reference's own
     * float/double rounding (KaminoCore.cu:11-52), so the pole-wrap index
     * map is bit-exact with the reference kernels.  Without this flag,
     * positions are kept as an exact integer cell index plus an FP32
     * fraction and the pole remap (theta -> -theta, phi -> phi + pi) is done
     * in index arithmetic; that is the reference's algorithm with less
     * rounding error: the radian form misplaces phi + pi by up to ~3e-5
     * cells at nTheta = 1024 (pi/h != nTheta in float), which the RK2
     * midpoint cancellation on the pole rows turns into O(1) differences. */
    KAMINO_F_REFERENCE_ROUNDING = 1u << 4
};

/* Positional configKamino.txt fields (main.cu:17-45) plus extensions. */
typedef struct kamino_config {
    double radius;            /* sphere radius                      main.cu:17 */
    int32_t n_theta;          /* latitude cells; nPhi = 2*nTheta    main.cu:18 */
    int32_t frames;           /* frames for kamino_run_frames       main.cu:22 */
    double particle_density;  /* particles per cell                 main.cu:19 */
    double dt;                /* time step                          main.cu:20 */
    double frame_dt;          /* DT, frame duration                 main.cu:21 */
    double A;                 /* unused by the reference (N8)       main.cu:23 */
    int32_t B, C, D, E;       /* unused by the reference (N8)    main.cu:24-27 */
    char grid_path[256];      /*                                    main.cu:28 */
    char particle_path[256];  /*                                    main.cu:29 */
    char density_image[256];  /* "" when the file says null      main.cu:31-35 */
    char solid_image[256];    /*                                 main.cu:36-40 */
    char color_image[256];    /*                                 main.cu:41-45 */
    /* extensions */
    int64_t n_particles;      /* <0: count from particle_density as
                                 KaminoParticles.cu:20-26 does          */
    uint32_t flags;           /* kamino_flags                              */
    int32_t fp64_modes;       /* Fourier modes |m| <= this are solved in
                                 FP64 (default 4; 0 = all FP32)            */
    int32_t device;           /* CUDA device ordinal (default 0)           */
    int32_t reserved[7];
} kamino_config;

typedef struct kamino_solver_s* kamino_handle;

/* Fill *cfg with the reference's defaults (KaminoGPU.cuh:40-44). */
int kamino_config_default(kamino_config* cfg);

/* Parse a positional configKamino.txt (main.cu:17-45).  "null" image paths
 * become "" (the reference's solidImage test is a no-op, main.cu:39; here it
 * is honoured). */
int kamino_parse_config(const char* path, kamino_config* cfg);

/* Number of particles the reference would create for a config
 * (KaminoParticles.cu:20-26): 2 * floor(sqrt(d) * nTheta)^2, with d the
 * particle density truncated to an integer (Kamino::run passes it through
 * initParticlesfromPic's size_t parameter, KaminoSolver.cu:278). */
int64_t kamino_particle_count(const kamino_config* cfg);

/* Steps the frame loop of Kamino::run takes (KaminoCore.cu:886-895); -1 on
 * bad input.  Host-only. */
int64_t kamino_frame_steps(double dt, double frame_dt, int frames);

/* sizeof(kamino_config), sizeof(kamino_init_spec), sizeof(kamino_server_config),
 * sizeof(kamino_server_stats), in that order, for binding checks. */
int kamino_abi_sizes(size_t* out, int n);

/* Replaces KaminoSolver::KaminoSolver (KaminoSolver.cu:12-67) together with
 * the parameter upload of Kamino::run (KaminoCore.cu:868-872).  Allocates
 * all device state once; fields start at zero. */
int kamino_create(const kamino_config* cfg, kamino_handle* out);

/* Replaces KaminoSolver::~KaminoSolver (KaminoSolver.cu:69-104), without the
 * cudaDeviceReset the reference does there. */
int kamino_destroy(kamino_handle h);

/* Replaces KaminoQuantity::copyToGPU / copyBackToCPU (KaminoQuantity.cu:3-18)
 * and KaminoParticles::copy2GPU / copyBack2CPU (KaminoParticles.cu:93-109).
 * pitch_bytes is the host row pitch (ignored for particles).  Synchronous. */
int kamino_set_state(kamino_handle h, int field, const float* host, size_t pitch_bytes);
int kamino_get_state(kamino_handle h, int field, float* host, size_t pitch_bytes);

/* The reference's particle placement, KaminoParticles::KaminoParticles
 * without a colour image (KaminoParticles.cu:20-62; reached through
 * KaminoSolver::initParticlesfromPic, KaminoSolver.cu:278-281): a jittered
 * grid of 2 floor(sqrt(d) nTheta)^2 particles drawn with the C library's
 * rand() sequence after srand(seed) (the reference never seeds: seed 1), in
 * its float arithmetic.  kamino_reference_particles fills n (phi, theta)
 * pairs on the host (n must be that count for cfg->particle_density and
 * cfg->n_theta; the caller's rand() state is not touched);
 * kamino_init_particles uploads them to a handle created with that count. */
int kamino_reference_particles(const kamino_config* cfg, uint32_t seed, float* out, int64_t n);
int kamino_init_particles(kamino_handle h, uint32_t seed);

/* Image inputs with the image decoded by the caller (the reference reads it
 * with OpenCV's imread, which is not part of this library): 8-bit pixels in
 * OpenCV's B, G, R order, width x height, row stride in bytes.  As the
 * reference, the image is mirrored left-right (cv::flip code 1) and
 * resampled to nPhi x nTheta pixels (cv::resize, INTER_LINEAR): here on the
 * device, bilinear at half-pixel centres with the edges clamped, each
 * channel rounded to 8 bits.
 *   kamino_init_density_image replaces KaminoSolver::initDensityfromPic
 *   (KaminoSolver.cu:243-277): thickness(i, j) = (B + G + R) / 3 of pixel
 *   (i, j), each channel / 255.
 *   kamino_init_particle_colors_image gives the particles, as placed now,
 *   the colours KaminoParticles takes from its image (KaminoParticles.cu:
 *   6-17, 56-72): (G, R, B) / 255 of the pixel of the particle's cell; they
 *   appear in the particle .bgeo files. */
int kamino_init_density_image(kamino_handle h, const uint8_t* bgr, int width, int height, size_t stride);
int kamino_init_particle_colors_image(kamino_handle h, const uint8_t* bgr, int width, int height,
                                      size_t stride);

/* Replaces KaminoSolver::initialize_velocity (KaminoInitializer.cu:3-85),
 * which the reference's constructor runs (KaminoSolver.cu:59): sets u_phi
 * and u_theta to the reference's FBM curl-noise velocity, evaluated on the
 * device with the reference's float/double arithmetic.  kamino_create
 * leaves every field zero; call this for the reference's default start. */
int kamino_init_fbm(kamino_handle h);

/* One step with the state in host memory: KaminoQuantity::copyToGPU of
 * u_phi, u_theta and the thickness, KaminoSolver::stepForward(dt) and
 * copyBackToCPU of the three (KaminoQuantity.cu:3-18, KaminoSolver.cu:
 * 197-221) in one call, which returns when the outputs are in host memory.
 * The copies overlap the step: u_phi and u_theta are advected while the
 * thickness is still being uploaded, and the thickness and u_phi downloads
 * start as soon as each is final.  Same results as the separate calls; the
 * in and out buffers may be the same.  pitch_bytes: host row pitch (0 =
 * dense); pinned host memory (kamino_host_alloc) copies fastest. */
int kamino_step_host(kamino_handle h, float dt, const float* u_phi_in, const float* u_theta_in,
                     const float* thickness_in, float* u_phi_out, float* u_theta_out, float* thickness_out,
                     size_t pitch_bytes);

/* Same, with a device pointer (row pitch in bytes), ordered on the handle's
 * stream and not synchronised. */
int kamino_set_state_device(kamino_handle h, int field, const float* dev, size_t pitch_bytes);
int kamino_get_state_device(kamino_handle h, int field, float* dev, size_t pitch_bytes);

/* Replaces KaminoSolver::stepForward (KaminoSolver.cu:197-221).  dt is
 * stored and, as in the reference, ignored unless KAMINO_F_HONOR_STEP_DT is
 * set.  Asynchronous on the handle's stream. */
int kamino_step(kamino_handle h, float dt);

/* The three stages of stepForward, callable one by one (KaminoCore.cu:344,
 * 551, 749).  advection+geometric+projection == step. */
int kamino_advection(kamino_handle h);
int kamino_geometric(kamino_handle h);
int kamino_projection(kamino_handle h);

/* Pressure projection of caller-owned fields that allocates no device memory.
 * No counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc (code running inside another framework's memory pool, or whose
 * device memory is fixed at start-up): they pass device pointers to the
 * input and output fields, and the projection's temporaries live in one
 * fixed 1.25 MiB array compiled into the library, which every GPU that loads
 * the library holds until exit.  Limit: n_theta a power of two in [32, 256];
 * larger sizes return KAMINO_ERR_INVALID.  Modes |m| <= 4 are solved in FP64.
 * Dense rows of 2*n_theta floats: u_phi / u_phi_out n_theta rows, u_theta /
 * u_theta_out n_theta-1 rows, pressure_out n_theta rows (outputs may alias
 * inputs); every pointer 16-byte aligned.  stream is a cudaStream_t (NULL: the default stream); the call is
 * asynchronous on it.  The first call on a device looks up the array's
 * device address, so make it before any stream capture on that device.  All
 * calls share the array, which keeps the tables of the last n_theta called
 * and the last call's temporaries: calls whose work overlaps on the GPU race.
 * A call with an n_theta other than the previous call's uploads that size's
 * tables from host memory; on a stream that is capturing, such a call is
 * refused with KAMINO_ERR_INVALID. */
int kamino_projection_noalloc(int n_theta, const float* u_phi, const float* u_theta, float* u_phi_out,
                              float* u_theta_out, float* pressure_out, void* stream);

/* n steps of the configured dt, replayed from CUDA graphs. */
int kamino_step_n(kamino_handle h, int n);

/* The frame loop of Kamino::run (KaminoCore.cu:886-904) without the .bgeo
 * output: for each frame, steps while T < i*DT, then one remainder step;
 * every step uses the configured dt as the reference does (N5). */
int kamino_run_frames(kamino_handle h, int frames, int64_t* steps_taken);

/* ------------------------------------------------------------ frame output
 * The .bgeo files Kamino writes after every frame, through Partio's
 * uncompressed BGEO writer (Houdini classic geometry, big-endian):
 *   KAMINO_FRAME_GRID       KaminoSolver::write_data_bgeo
 *                           (KaminoSolver.cu:284-357): one point per cell
 *                           centre, attributes position, v (the centred
 *                           velocity mapped to 3-D, mapVToSphere :409-423)
 *                           and density (the thickness);
 *   KAMINO_FRAME_PARTICLES  KaminoSolver::write_particles_bgeo (:359-396):
 *                           one point per particle, position, v = 0 and
 *                           color as the reference writes it (components
 *                           3i+1..3i+3 of its per-particle (G, R, B) array,
 *                           :375-377; zero without a colour image, see
 *                           kamino_init_particle_colors_image).
 * The records are computed on the device in the file's byte order and
 * copied to pinned host memory on a second stream, so work issued after a
 * capture overlaps the copy. */
enum kamino_frame_kind { KAMINO_FRAME_GRID = 0, KAMINO_FRAME_PARTICLES = 1 };

/* Size of the file a frame of this kind writes. */
int kamino_frame_bytes(kamino_handle h, int kind, size_t* bytes);

/* Snapshot the current state as a frame: queues the pack kernel on the
 * handle's stream and the device->host copy behind it; returns at once.  At
 * most two captures of a kind wait to be written (a third is an error). */
int kamino_frame_capture(kamino_handle h, int kind);

/* Waits for the oldest captured frame of the kind (capturing the current
 * state first if none waits) and writes its file image to path (if not
 * NULL) and to host (if not NULL; host_bytes >= kamino_frame_bytes). */
int kamino_frame_write(kamino_handle h, int kind, const char* path, void* host, size_t host_bytes);

/* Kamino::run (KaminoCore.cu:860-912) with its output: writes frame 0, then
 * runs every frame's steps (as kamino_run_frames) and writes
 * <grid_path><i>.bgeo and <particle_path><i>.bgeo (a NULL or empty path
 * skips that kind).  Frame i's file is written while the GPU runs frame
 * i+1. */
int kamino_run_frames_bgeo(kamino_handle h, int frames, const char* grid_path, const char* particle_path,
                           int64_t* steps_taken);

/* Device time of one pack kernel launch of the kind, averaged over reps
 * (CUDA events on the handle's stream; flush_l2 evicts the L2 before each
 * launch, outside the timed interval). */
int kamino_frame_time_pack(kamino_handle h, int kind, int reps, int flush_l2, double* ms);

/* Checkpoint and resume: no counterpart in the reference (its .bgeo frames
 * are write-only).  kamino_save_state writes u_phi, u_theta, the thickness,
 * the particles, the step count and the elapsed time to a file with a
 * checksum; kamino_load_state restores them into a handle of the same
 * n_theta, particle count, radius, dt and trajectory flags (particle RK2,
 * pole sign flip, honoured step dt, reference rounding; KAMINO_ERR_INVALID otherwise;
 * KAMINO_ERR_IO for a truncated or corrupted file).  Synchronous. */
int kamino_save_state(kamino_handle h, const char* path);
int kamino_load_state(kamino_handle h, const char* path);

int kamino_synchronize(kamino_handle h);

/* Elapsed simulated time (KaminoSolver.cu:220) and step count. */
int kamino_time_elapsed(kamino_handle h, double* t, int64_t* steps);

/* Device timing of n steps with CUDA events on the handle's stream.  When
 * flush_l2 is set, a buffer larger than L2 is written before every step,
 * outside the timed interval.  *ms_total is the sum over the n steps. */
int kamino_time_steps(kamino_handle h, int n, int flush_l2, double* ms_total);

/* Per-kernel device timing of one step (CUDA events around each launch on
 * the handle's stream, averaged over reps).  Writes up to max entries. */
int kamino_time_kernels(kamino_handle h, int reps, int flush_l2, double* ms, int max,
                        int* count);
const char* kamino_kernel_name(int index);

/* Kernel launches one step issues (for launch accounting). */
int kamino_launches_per_step(kamino_handle h);

/* Device bytes held by the handle. */
int kamino_device_bytes(kamino_handle h, size_t* bytes);

/* Message of the last failure on this thread (never NULL). */
const char* kamino_last_error(void);

/* Page-locked host memory for fast host<->device state copies. */
int kamino_host_alloc(size_t bytes, void** out);
int kamino_host_free(void* p);

/* --------------------------------------------------------- debug probes
 * Evaluate the sampler's index stage (pole wrap, cell index, branch) on
 * given coordinates, with the same device code the step uses.  kind:
 * 0 = u_phi sampler (sampleVPhi, KaminoCore.cu:36-84), 1 = u_theta
 * (sampleVTheta, :86-134), 2 = centred (sampleCentered, :136-184).
 * out[4*i..] = phiIndex, thetaIndex, flipped (1/0), pole branch (1/0);
 * alpha[2*i..] = alphaPhi, alphaTheta.  Host arrays, synchronous. */
int kamino_probe_index(kamino_handle h, int kind, const float* phi, const float* theta,
                       int64_t n, int32_t* out, float* alpha);

/* Apply the reference's validateCoord (KaminoCore.cu:11-29) to n host
 * coordinate pairs on the device and return the particle cell indices
 * floor(phi/h), floor(theta/h) (KaminoParticles.cu:56-57). */
int kamino_probe_wrap(kamino_handle h, float* phi, float* theta, int64_t n, int32_t* cells);

/* ------------------------------------------------ seeded initial states
 * Synthetic inputs: stream function psi = sum_{l<=lmax} a_lm Y_lm with
 * a_lm ~ N(0,1) from the seed, optionally plus a Gaussian vortex, velocity
 * = curl(psi) evaluated at the staggered points; thickness = 1 +
 * amp*U(-1,1); particles uniform on the sphere.  Host arrays (dense, pitch =
 * nPhi floats).  Any output pointer may be NULL. */
typedef struct kamino_init_spec {
    int32_t n_theta;
    int32_t lmax;
    uint64_t seed;
    double radius;
    double thickness_noise;    /* amplitude of the U(-1,1) thickness noise  */
    int32_t vortex;            /* 1: add one seeded Gaussian vortex          */
    double vortex_sigma;       /* radians                                    */
    double vortex_amplitude;   /* 0: draw from the seed                      */
    double velocity_scale;     /* velocities are scaled so max|u| == this;
                                  0 keeps the raw N(0,1) amplitudes          */
    int64_t n_particles;
    double vortex_out[3];      /* written: centre theta, centre phi, amplitude */
} kamino_init_spec;

int kamino_init_spec_default(kamino_init_spec* spec);
int kamino_make_initial_state(kamino_init_spec* spec, float* u_phi, float* u_theta,
                              float* thickness, float* particles);

/* ------------------------------------------------------------- batching
 * Many independent spheres of uneven nTheta advanced together: each stage
 * is one persistent launch that drains a queue of (sphere, row tile) work
 * items, and a whole step is one CUDA graph.  Tile shapes come from the
 * autotuner (kamino_batch_autotune) or its defaults. */
typedef struct kamino_batch_s* kamino_batch;

int kamino_batch_create(const kamino_config* cfgs, int n_spheres, kamino_batch* out);
int kamino_batch_destroy(kamino_batch b);
int kamino_batch_set_state(kamino_batch b, int sphere, int field, const float* host,
                           size_t pitch_bytes);
int kamino_batch_get_state(kamino_batch b, int sphere, int field, float* host,
                           size_t pitch_bytes);
int kamino_batch_step_n(kamino_batch b, int n);
int kamino_batch_synchronize(kamino_batch b);
int kamino_batch_time_steps(kamino_batch b, int n, int flush_l2, double* ms_total);
/* Times candidate tile shapes on the live batch and keeps the fastest.
 * The state is saved and restored around the trials. */
int kamino_batch_autotune(kamino_batch b, int reps, int* chosen, int max_chosen);
int64_t kamino_batch_cells(kamino_batch b);

/* -------------------------------------------------------------- serving
 * Continuous batching: requests (one sphere each) are admitted while their
 * device state fits the budget, advance together with whatever else is
 * resident, and retire independently. */
typedef struct kamino_server_s* kamino_server;

typedef struct kamino_server_config {
    size_t budget_bytes;      /* admission budget for resident state        */
    int32_t max_resident;     /* slot limit (0 = unlimited)                 */
    int32_t steps_per_round;  /* steps every batched sphere takes per round  */
    int32_t device;
    int32_t solo_n_theta;     /* requests with n_theta >= this run all their
                                 steps as one-sphere graphs on their own
                                 stream, concurrently with everything else
                                 (0 = 512); smaller ones advance together in
                                 the batched step                            */
    int32_t solo_slots;       /* solo requests running at once (0 = 3): a few
                                 large spheres together fill the SMs that
                                 one leaves idle in its latency-bound
                                 kernels; more evict each other from the L2.
                                 A solo request waiting for a slot does not
                                 hold back smaller ones                      */
    int32_t reserved[3];
} kamino_server_config;

typedef struct kamino_server_stats {
    int64_t submitted, completed, resident, queued;
    int64_t cell_steps;       /* total cell-steps executed                   */
    double busy_seconds;      /* wall time with at least one resident sphere */
    double p50_latency_s, p99_latency_s, mean_latency_s;
    size_t resident_bytes, peak_resident_bytes;
    /* where the time and the work went */
    int64_t solo_cell_steps;       /* cell-steps of spheres run as one-sphere graphs */
    int64_t batched_cell_steps;    /* cell-steps of the batched rounds            */
    int64_t batched_rounds;        /* batched rounds completed                    */
    double batched_round_seconds;  /* device time of those rounds (CUDA events)   */
    double solo_seconds;           /* device time of the one-sphere runs, summed
                                      (they can overlap each other)              */
    double poll_seconds;           /* host wall time inside kamino_server_poll    */
} kamino_server_stats;

int kamino_server_create(const kamino_server_config* cfg, kamino_server* out);
int kamino_server_destroy(kamino_server s);
/* Submit one sphere: config (n_theta, radius, dt, flags...), initial state
 * (host, dense pitch; u_theta has n_theta-1 rows), and a step count.
 * arrival_time_s is the request's arrival on the caller's clock (for the
 * latency statistics); pass a negative value to use the submit time. */
int kamino_server_submit(kamino_server s, const kamino_config* cfg, const float* u_phi,
                         const float* u_theta, const float* thickness, int32_t steps,
                         double arrival_time_s, int64_t* request_id);
/* One pass of the request loop; never waits for the GPU: retires requests
 * whose work has finished (event queries), admits queued requests that fit
 * (a large one starts its steps on its own stream), and launches the next
 * round of the batched spheres if none is in flight.  n_completed: requests
 * retired by this call.  Call it repeatedly until the work is done. */
int kamino_server_poll(kamino_server s, int* n_completed);
/* Copy a finished request's field to host memory (dense pitch) and, for
 * the last field, release it.  KAMINO_ERR_NOT_READY while it runs. */
int kamino_server_fetch(kamino_server s, int64_t request_id, int field, float* host);
int kamino_server_release(kamino_server s, int64_t request_id);
int kamino_server_get_stats(kamino_server s, kamino_server_stats* st);
/* Seconds on the server's clock (monotonic, same clock as the stats). */
double kamino_server_now(kamino_server s);

#ifdef __cplusplus
}
#endif

#endif /* KAMINO_GB300_H */
