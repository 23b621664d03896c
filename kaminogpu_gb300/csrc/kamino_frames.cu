// kamino_frames.cu — frame I/O: the .bgeo files Kamino writes after every
// frame, built on the device, and the image inputs (thickness and particle
// colours from a decoded image), resampled on the device.
//
// The reference writes two files per frame through Partio
// (KaminoSolver::write_data_bgeo / write_particles_bgeo, KaminoSolver.cu:
// 284-396, called from Kamino::run, KaminoCore.cu:874-903): a grid file with
// one point per cell centre (position on the sphere, centred velocity mapped
// to 3-D, thickness) and a particle file (position, zero velocity, colour).
// It copies the fields back, loops over every cell on the host, adds each
// point to a Partio container and writes it, all while the GPU waits.
//
// Here one kernel per kind computes every point's record and writes it in
// the file's own byte order (big-endian floats, the point layout of the
// uncompressed BGEO writer), so the device->host copy lands the finished
// file body in pinned memory next to a header the host wrote once.  The copy
// runs on a second stream: steps issued after a capture run while it drains,
// and the host writes one frame's file while the GPU computes the next frame.
//
// File layout (Houdini classic geometry, as Partio's BGEO writer emits it
// for ".bgeo"; every integer and float big-endian):
//   int32 magic "Bgeo", char 'V', int32 version 5,
//   int32 nPoints, nPrims 0, nPointGroups 0, nPrimGroups 0,
//         nPointAttrib, nVertexAttrib 0, nPrimAttrib 0, nAttrib 0,
//   per point attribute other than position:
//         uint16 name length, name, uint16 size, int32 type (0 float,
//         5 vector), size x int32 default 0,
//   per point: x, y, z, w = 1, then the attributes' values,
//   trailer bytes 0x00, 0xff.
// Grid records: position(3) w v(3) density(1) = 32 bytes; particle records:
// position(3) w v(3) color(3) = 40 bytes.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <fcntl.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include "kamino_common.h"

#define FCUDA(call)                                                                                  \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return kamino_fail(KAMINO_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                               __FILE__, __LINE__);                                                  \
    } while (0)

namespace {

constexpr int FRAME_THREADS = 256;
constexpr int GRID_FLOATS = 8;       // x y z w | vx vy vz density
constexpr int PARTICLE_FLOATS = 10;  // x y z w | vx vy vz | r g b

__device__ __forceinline__ uint32_t be32(float x) { return __byte_perm(__float_as_uint(x), 0u, 0x0123u); }

// One thread per cell, records in the reference's loop order (row j, then
// column i; KaminoSolver.cu:305-307).  Arithmetic as the reference's, in
// float with the operations in its order: the centred velocity
// (KaminoSolver.cu:309-337), the cell centre ((i + 0) h, (j + 1/2) h)
// (:339), mapVToSphere (:409-423) and mapPToSphere (:398-407).  Only sinf /
// cosf can differ from the host's, by the functions' last-place error.
__global__ void __launch_bounds__(FRAME_THREADS) k_frame_grid(KGeo g, const float* __restrict__ u,
                                                              const float* __restrict__ v,
                                                              const float* __restrict__ rho,
                                                              uint4* __restrict__ out)
{
    const int t = blockIdx.x * FRAME_THREADS + threadIdx.x;
    if (t >= g.nt * g.np) return;
    const int j = t >> (g.log2nt + 1), i = t & g.mask;
    const int ie = (i + 1) & g.mask;  // iEast wraps at the seam (:313)
    int jn, js;                       // the pole rows use u_theta row 0 / nTheta-2 twice (:316-329)
    if (j == 0) {
        jn = js = 0;
    } else if (j == g.nt - 1) {
        jn = js = g.nt - 2;
    } else {
        jn = j - 1;
        js = j;
    }
    const size_t row = (size_t)j * g.pitch;
    const float uw = __ldg(u + row + i), ue = __ldg(u + row + ie);
    const float vn = __ldg(v + (size_t)jn * g.pitch + i), vs = __ldg(v + (size_t)js * g.pitch + i);
    const float d = __ldg(rho + row + i);
    // (uWest + uEast) / 2.0: a float sum, halved exactly
    const float uphi = __fmul_rn(__fadd_rn(uw, ue), 0.5f);
    const float uth = __fmul_rn(__fadd_rn(vn, vs), 0.5f);
    // (i + 0.0) * gridLen and (j + 0.5) * gridLen are exact in double and
    // rounded to float by mapVToSphere's float locals: the rounded products
    const float phi = __fmul_rn((float)i, g.h);
    const float theta = __fmul_rn((float)j + 0.5f, g.h);
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    const float vx = __fsub_rn(__fmul_rn(__fmul_rn(ct, cp), uth), __fmul_rn(sp, uphi));
    const float vz = __fadd_rn(__fmul_rn(__fmul_rn(ct, sp), uth), __fmul_rn(cp, uphi));
    const float vy = __fmul_rn(-st, uth);
    const float rs = __fmul_rn(g.R, st);
    const float x = __fmul_rn(rs, cp), z = __fmul_rn(rs, sp), y = __fmul_rn(g.R, ct);
    out[2 * (size_t)t] = make_uint4(be32(x), be32(y), be32(z), be32(1.0f));
    out[2 * (size_t)t + 1] = make_uint4(be32(vx), be32(vy), be32(vz), be32(d));
}

// One thread per particle: mapPToSphere of (phi, theta) (KaminoSolver.cu:
// 373-393), velocity 0, and the colour the reference writes: components
// colorBGR[3i+1], [3i+2], [3i+3] (KaminoSolver.cu:375-377) of its (G, R, B)
// per-particle array, i.e. (R_i, B_i, G_i+1); for the last particle the third
// read is past the array in the reference and 0 here.  Without a colour image
// every colour is 0 (KaminoParticles.cu:73-78); col is then null.
__global__ void __launch_bounds__(FRAME_THREADS) k_frame_particles(float R, const float2* __restrict__ part,
                                                                   const float* __restrict__ col, int64_t n,
                                                                   uint2* __restrict__ out)
{
    const int64_t t = (int64_t)blockIdx.x * FRAME_THREADS + threadIdx.x;
    if (t >= n) return;
    const float2 pt = __ldg(part + t);  // (phi, theta)
    float st, ct, sp, cp;
    sincosf(pt.y, &st, &ct);
    sincosf(pt.x, &sp, &cp);
    const float rs = __fmul_rn(R, st);
    const float x = __fmul_rn(rs, cp), z = __fmul_rn(rs, sp), y = __fmul_rn(R, ct);
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
    if (col) {
        c0 = __ldg(col + 3 * t + 1);
        c1 = __ldg(col + 3 * t + 2);
        c2 = t + 1 < n ? __ldg(col + 3 * t + 3) : 0.0f;
    }
    uint2* o = out + 5 * t;
    o[0] = make_uint2(be32(x), be32(y));
    o[1] = make_uint2(be32(z), be32(1.0f));
    o[2] = make_uint2(0u, 0u);
    o[3] = make_uint2(0u, be32(c0));
    o[4] = make_uint2(be32(c1), be32(c2));
}

// ------------------------------------------------------------ image input
// The image of initDensityfromPic / KaminoParticles (KaminoSolver.cu:243-277,
// KaminoParticles.cu:6-17), decoded by the caller: 8-bit B, G, R pixels.  The
// reference mirrors it left-right (cv::flip code 1) and resamples it to
// nPhi x nTheta (cv::resize, INTER_LINEAR).  Here the resampling is bilinear
// at half-pixel centres with the edges clamped, separable in the order
// columns then rows, in FP32 with each product and sum rounded as written,
// and each channel rounded to the nearest 8-bit value (ties to even).  The
// per-column and per-row source indices (already mirrored) and weights come
// from the host (image_axis).
struct ImgAxis {
    int i0, i1;  // source pixels
    float a;     // weight of i1
};

__device__ __forceinline__ float lerp_px(float p0, float p1, float a)
{
    return __fadd_rn(__fmul_rn(p0, __fsub_rn(1.0f, a)), __fmul_rn(p1, a));
}

// One thread per destination pixel (i, j); writes the pixel (B, G, R, 0) to
// px and, with rho, the thickness (B + G + R) / 3 of KaminoSolver.cu:265-273:
// each channel / 255.0 rounded to float, a float sum, / 3.0 in double.
__global__ void __launch_bounds__(FRAME_THREADS) k_image_resample(KGeo g, const uint8_t* __restrict__ img,
                                                                  size_t stride, const ImgAxis* __restrict__ ax,
                                                                  const ImgAxis* __restrict__ ay,
                                                                  uchar4* __restrict__ px, float* __restrict__ rho)
{
    const int t = blockIdx.x * FRAME_THREADS + threadIdx.x;
    if (t >= g.nt * g.np) return;
    const int j = t >> (g.log2nt + 1), i = t & g.mask;
    const ImgAxis x = ax[i], y = ay[j];
    const uint8_t* r0 = img + (size_t)y.i0 * stride;
    const uint8_t* r1 = img + (size_t)y.i1 * stride;
    uint8_t c[3];
    for (int k = 0; k < 3; k++) {
        const float h0 = lerp_px(r0[3 * x.i0 + k], r0[3 * x.i1 + k], x.a);
        const float h1 = lerp_px(r1[3 * x.i0 + k], r1[3 * x.i1 + k], x.a);
        c[k] = (uint8_t)min(255, max(0, __float2int_rn(lerp_px(h0, h1, y.a))));
    }
    px[t] = make_uchar4(c[0], c[1], c[2], 0);
    if (rho) {
        const float B = (float)__ddiv_rn((double)c[0], 255.0), G = (float)__ddiv_rn((double)c[1], 255.0),
                    R = (float)__ddiv_rn((double)c[2], 255.0);
        rho[(size_t)j * g.pitch + i] = (float)__ddiv_rn((double)__fadd_rn(__fadd_rn(B, G), R), 3.0);
    }
}

// KaminoParticles.cu:56-57, 64-72: a particle's pixel is its cell
// floor(phi / gridLen), floor(theta / gridLen) (clamped to the grid; the
// reference would read outside the image there), colour (G, R, B) / 255.
__global__ void __launch_bounds__(FRAME_THREADS) k_particle_colors(KGeo g, const float2* __restrict__ part, int64_t n,
                                                                   const uchar4* __restrict__ px, float* __restrict__ col)
{
    const int64_t t = (int64_t)blockIdx.x * FRAME_THREADS + threadIdx.x;
    if (t >= n) return;
    const float2 pt = __ldg(part + t);
    const int xi = min(g.np - 1, max(0, (int)floorf(__fdiv_rn(pt.x, g.h))));
    const int yi = min(g.nt - 1, max(0, (int)floorf(__fdiv_rn(pt.y, g.h))));
    const uchar4 p = px[(size_t)yi * g.np + xi];
    col[3 * t] = (float)__ddiv_rn((double)p.y, 255.0);
    col[3 * t + 1] = (float)__ddiv_rn((double)p.z, 255.0);
    col[3 * t + 2] = (float)__ddiv_rn((double)p.x, 255.0);
}

void put16(std::vector<uint8_t>& o, uint16_t x)
{
    o.push_back((uint8_t)(x >> 8));
    o.push_back((uint8_t)x);
}

void put32(std::vector<uint8_t>& o, uint32_t x)
{
    for (int s = 24; s >= 0; s -= 8) o.push_back((uint8_t)(x >> s));
}

struct Attr {
    const char* name;
    uint16_t size;
    int32_t type;  // Houdini attribute type: 0 float, 5 vector
};

std::vector<uint8_t> bgeo_header(int32_t npoints, const Attr* attrs, int nattr)
{
    std::vector<uint8_t> o;
    put32(o, ((uint32_t)'B' << 24) | ((uint32_t)'g' << 16) | ((uint32_t)'e' << 8) | (uint32_t)'o');
    o.push_back((uint8_t)'V');
    put32(o, 5);
    const int32_t counts[8] = {npoints, 0, 0, 0, nattr, 0, 0, 0};
    for (int32_t c : counts) put32(o, (uint32_t)c);
    for (int a = 0; a < nattr; a++) {
        const uint16_t len = (uint16_t)std::strlen(attrs[a].name);
        put16(o, len);
        o.insert(o.end(), attrs[a].name, attrs[a].name + len);
        put16(o, attrs[a].size);
        put32(o, (uint32_t)attrs[a].type);
        for (int k = 0; k < attrs[a].size; k++) put32(o, 0);
    }
    return o;
}

const Attr kGridAttrs[] = {{"v", 3, 5}, {"density", 1, 0}};
const Attr kParticleAttrs[] = {{"v", 3, 5}, {"color", 3, 5}};

}  // namespace

// One captured frame: device records, and the pinned file image the copy
// fills ([pad][header][records][trailer], the records 256-byte aligned).
struct KFrameSlot {
    void* dev = nullptr;
    uint8_t* host = nullptr;
    size_t file_off = 0;  // start of the header in host
    size_t file_bytes = 0;
    cudaEvent_t copied = nullptr;
    bool pending = false;
};

struct KFrames {
    KFrameSlot slot[2][2];  // [kind][slot]: two captures of each kind may be in flight
    int head[2] = {0, 0};   // slot the next capture fills
    int tail[2] = {0, 0};   // oldest pending capture
    size_t rec_bytes[2] = {0, 0};
    cudaStream_t copy = nullptr;
    cudaEvent_t packed = nullptr;
    float* colors = nullptr;  // per-particle (G, R, B) from a colour image, or null
};

void kamino_frames_release(KFrames* f)
{
    if (!f) return;
    if (f->copy) cudaStreamSynchronize(f->copy);
    for (auto& kind : f->slot)
        for (auto& s : kind) {
            if (s.copied) cudaEventDestroy(s.copied);
            if (s.dev) cudaFree(s.dev);
            if (s.host) cudaFreeHost(s.host);
        }
    if (f->packed) cudaEventDestroy(f->packed);
    if (f->copy) cudaStreamDestroy(f->copy);
    if (f->colors) cudaFree(f->colors);
    delete f;
}

namespace {

int check_kind(int kind)
{
    if (kind != KAMINO_FRAME_GRID && kind != KAMINO_FRAME_PARTICLES)
        return kamino_fail(KAMINO_ERR_INVALID, "unknown frame kind %d", kind);
    return KAMINO_OK;
}

int64_t frame_points(const KGeo& g, const KBufs& b, int kind)
{
    return kind == KAMINO_FRAME_GRID ? (int64_t)g.nt * g.np : b.npart;
}

std::vector<uint8_t> frame_header(const KGeo& g, const KBufs& b, int kind)
{
    return kind == KAMINO_FRAME_GRID ? bgeo_header((int32_t)frame_points(g, b, kind), kGridAttrs, 2)
                                     : bgeo_header((int32_t)frame_points(g, b, kind), kParticleAttrs, 2);
}

size_t record_bytes(int kind) { return sizeof(float) * (kind == KAMINO_FRAME_GRID ? GRID_FLOATS : PARTICLE_FLOATS); }

int frame_state(kamino_handle h, KFrames** out)
{
    KFrames** pf = nullptr;
    int rc = kamino_internal_frames(h, &pf);
    if (rc) return rc;
    if (!*pf) {
        KFrames* f = new KFrames();
        cudaError_t e = cudaStreamCreateWithFlags(&f->copy, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->packed, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            kamino_frames_release(f);
            return kamino_fail(KAMINO_ERR_CUDA, "frame output streams: %s", cudaGetErrorString(e));
        }
        *pf = f;
    }
    *out = *pf;
    return KAMINO_OK;
}

// Allocates a slot's buffers on its first use and writes its header and
// trailer once (they depend only on the point count, fixed per handle).
int prepare_slot(KFrames* f, const KGeo& g, const KBufs& b, int kind, KFrameSlot& s)
{
    if (s.host) return KAMINO_OK;  // set only once every buffer of the slot exists
    const std::vector<uint8_t> head = frame_header(g, b, kind);
    const size_t rec = (size_t)frame_points(g, b, kind) * record_bytes(kind);
    const size_t pad = (256 - head.size() % 256) % 256;
    void* dp = nullptr;
    void* hp = nullptr;
    cudaEvent_t ev = nullptr;
    cudaError_t e = rec ? cudaMalloc(&dp, rec) : cudaSuccess;
    if (e == cudaSuccess) e = cudaHostAlloc(&hp, pad + head.size() + rec + 2, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (dp) cudaFree(dp);
        if (hp) cudaFreeHost(hp);
        return kamino_fail(KAMINO_ERR_ALLOC, "frame buffers (%zu bytes): %s", rec, cudaGetErrorString(e));
    }
    uint8_t* host = (uint8_t*)hp;
    std::memcpy(host + pad, head.data(), head.size());
    host[pad + head.size() + rec] = 0x00;
    host[pad + head.size() + rec + 1] = 0xff;
    s.dev = dp;
    s.copied = ev;
    s.file_off = pad;
    s.file_bytes = head.size() + rec + 2;
    s.host = host;
    f->rec_bytes[kind] = rec;
    return KAMINO_OK;
}

int launch_pack(const KGeo& g, const KBufs& b, int cur_uv, int cur_r, int kind, void* dev, cudaStream_t st,
                const float* colors)
{
    const int64_t n = frame_points(g, b, kind);
    if (n == 0) return KAMINO_OK;
    const unsigned blocks = (unsigned)((n + FRAME_THREADS - 1) / FRAME_THREADS);
    if (kind == KAMINO_FRAME_GRID)
        k_frame_grid<<<blocks, FRAME_THREADS, 0, st>>>(g, b.u[cur_uv], b.v[cur_uv], b.rho[cur_r], (uint4*)dev);
    else
        k_frame_particles<<<blocks, FRAME_THREADS, 0, st>>>(g.R, b.part[cur_r], colors, n, (uint2*)dev);
    FCUDA(cudaGetLastError());
    return KAMINO_OK;
}

int capture(kamino_handle h, KFrames* f, int kind)
{
    KGeo g;
    KBufs b;
    int cu, cr;
    int rc = kamino_internal_desc(h, &g, &b, nullptr, &cu, &cr);
    if (rc) return rc;
    if (kind == KAMINO_FRAME_GRID && (int64_t)g.nt * g.np > INT32_MAX)
        return kamino_fail(KAMINO_ERR_INVALID, "too many points for a .bgeo file");
    if (b.npart > INT32_MAX) return kamino_fail(KAMINO_ERR_INVALID, "too many particles for a .bgeo file");
    KFrameSlot& s = f->slot[kind][f->head[kind]];
    if (s.pending)
        return kamino_fail(KAMINO_ERR_INVALID, "two frames of kind %d are captured and not yet written", kind);
    if ((rc = prepare_slot(f, g, b, kind, s))) return rc;
    cudaStream_t st = kamino_internal_stream(h);
    // The slot's device records were last read by its previous copy, which
    // finished before that capture was written (kamino_frame_write waits).
    if ((rc = launch_pack(g, b, cu, cr, kind, s.dev, st, f->colors))) return rc;
    FCUDA(cudaEventRecord(f->packed, st));
    FCUDA(cudaStreamWaitEvent(f->copy, f->packed, 0));
    const size_t rec = f->rec_bytes[kind];
    const size_t head_bytes = s.file_bytes - rec - 2;
    if (rec)
        FCUDA(cudaMemcpyAsync(s.host + s.file_off + head_bytes, s.dev, rec, cudaMemcpyDeviceToHost, f->copy));
    FCUDA(cudaEventRecord(s.copied, f->copy));
    s.pending = true;
    f->head[kind] ^= 1;
    return KAMINO_OK;
}

// Writes n bytes to path.  (Writing with several threads at disjoint
// offsets was measured: buffered writes to one file take the inode's lock,
// so it gained nothing.)
int write_file(const char* path, const uint8_t* data, size_t n)
{
    const int fd = ::open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return kamino_fail(KAMINO_ERR_IO, "cannot open %s for writing: %s", path, std::strerror(errno));
    size_t done = 0;
    int err = 0;
    while (done < n) {
        const ssize_t w = ::write(fd, data + done, n - done);
        if (w < 0 && errno == EINTR) continue;
        if (w <= 0) {
            err = w < 0 ? errno : EIO;
            break;
        }
        done += (size_t)w;
    }
    if (::close(fd) != 0 && !err) err = errno;
    if (err) return kamino_fail(KAMINO_ERR_IO, "write to %s failed: %s", path, std::strerror(err));
    return KAMINO_OK;
}

// Waits for the oldest pending capture of the kind (capturing now if there is
// none) and hands its file image to the file and/or the caller's buffer.
int finish(kamino_handle h, KFrames* f, int kind, const char* path, void* host, size_t host_bytes)
{
    int rc;
    KFrameSlot* s = &f->slot[kind][f->tail[kind]];
    if (!s->pending) {
        if ((rc = capture(h, f, kind))) return rc;
        s = &f->slot[kind][f->tail[kind]];
    }
    if (host && host_bytes < s->file_bytes)
        return kamino_fail(KAMINO_ERR_INVALID, "buffer of %zu bytes < frame of %zu bytes", host_bytes,
                           s->file_bytes);
    FCUDA(cudaEventSynchronize(s->copied));
    s->pending = false;
    f->tail[kind] ^= 1;
    const uint8_t* img = s->host + s->file_off;
    if (host) std::memcpy(host, img, s->file_bytes);
    if (path && (rc = write_file(path, img, s->file_bytes))) return rc;
    return KAMINO_OK;
}

}  // namespace

extern "C" int kamino_frame_bytes(kamino_handle h, int kind, size_t* bytes)
{
    int rc = check_kind(kind);
    if (rc) return rc;
    KGeo g;
    KBufs b;
    if ((rc = kamino_internal_desc(h, &g, &b, nullptr, nullptr, nullptr))) return rc;
    if (!bytes) return kamino_fail(KAMINO_ERR_INVALID, "null output");
    *bytes = frame_header(g, b, kind).size() + (size_t)frame_points(g, b, kind) * record_bytes(kind) + 2;
    return KAMINO_OK;
}

extern "C" int kamino_frame_capture(kamino_handle h, int kind)
{
    int rc = check_kind(kind);
    if (rc) return rc;
    KFrames* f = nullptr;
    if ((rc = frame_state(h, &f))) return rc;
    return capture(h, f, kind);
}

extern "C" int kamino_frame_write(kamino_handle h, int kind, const char* path, void* host, size_t host_bytes)
{
    int rc = check_kind(kind);
    if (rc) return rc;
    if (!path && !host) return kamino_fail(KAMINO_ERR_INVALID, "kamino_frame_write: no path and no buffer");
    KFrames* f = nullptr;
    if ((rc = frame_state(h, &f))) return rc;
    return finish(h, f, kind, path, host, host_bytes);
}

// Kamino::run (KaminoCore.cu:860-912) with its output: frame 0, then per
// frame the reference's step count and the frame's files.  Frame i's pack
// and copy are queued behind its steps, and its file is written while the
// GPU runs frame i+1's steps.
extern "C" int kamino_run_frames_bgeo(kamino_handle h, int frames, const char* grid_path,
                                      const char* particle_path, int64_t* steps_taken)
{
    if (frames < 0) return kamino_fail(KAMINO_ERR_INVALID, "frames=%d < 0", frames);
    KFrames* f = nullptr;
    int rc = frame_state(h, &f);
    if (rc) return rc;
    double dt = 0, DT = 0;
    {
        kamino_config cfg;
        if ((rc = kamino_internal_config(h, &cfg))) return rc;
        dt = cfg.dt;
        DT = cfg.frame_dt;
    }
    if (kamino_frame_steps(dt, DT, 1) < 0) return kamino_fail(KAMINO_ERR_INVALID, "frame_dt and dt must be > 0");
    const bool want[2] = {grid_path && *grid_path, particle_path && *particle_path};
    const char* base[2] = {grid_path, particle_path};
    for (int k = 0; k < 2; k++)  // no earlier capture may be pending: the files pair with frames
        if (want[k] && f->slot[k][f->tail[k]].pending)
            return kamino_fail(KAMINO_ERR_INVALID, "a captured frame of kind %d is not yet written", k);
    auto name = [&](int k, int i) { return std::string(base[k]) + std::to_string(i) + ".bgeo"; };
    int64_t total = 0;
    auto run = [&]() {
        int r;
        for (int k = 0; k < 2; k++)
            if (want[k] && (r = capture(h, f, k))) return r;
        const float fdt = (float)dt, fDT = (float)DT;
        float T = 0.0f;
        for (int i = 1; i <= frames; i++) {
            int64_t n = 0;  // the reference's step count for frame i (KaminoCore.cu:888-895)
            while (T < i * fDT) {
                n++;
                T += fdt;
            }
            n++;
            T = i * fDT;
            if (n > 0x7fffffff) return kamino_fail(KAMINO_ERR_INVALID, "too many steps in a frame");
            if ((r = kamino_step_n(h, (int)n))) return r;
            total += n;
            for (int k = 0; k < 2; k++)
                if (want[k] && (r = capture(h, f, k))) return r;
            for (int k = 0; k < 2; k++)  // frame i-1, while frame i runs
                if (want[k] && (r = finish(h, f, k, name(k, i - 1).c_str(), nullptr, 0))) return r;
        }
        for (int k = 0; k < 2; k++)
            if (want[k] && (r = finish(h, f, k, name(k, frames).c_str(), nullptr, 0))) return r;
        return (int)KAMINO_OK;
    };
    rc = run();
    if (rc) {  // leave no capture of this loop waiting: later captures and loops start clean
        for (int k = 0; k < 2; k++) {
            if (!want[k]) continue;
            for (auto& sl : f->slot[k]) {
                if (sl.pending) cudaEventSynchronize(sl.copied);
                sl.pending = false;
            }
            f->head[k] = f->tail[k] = 0;
        }
        return rc;
    }
    if (steps_taken) *steps_taken = total;
    return KAMINO_OK;
}

// Device time of the pack kernel alone (CUDA events on the handle's stream,
// averaged over reps; with flush_l2 the L2 is evicted before each launch by
// the solver's flush, outside the timed interval).
extern "C" int kamino_frame_time_pack(kamino_handle h, int kind, int reps, int flush_l2, double* ms)
{
    int rc = check_kind(kind);
    if (rc) return rc;
    if (reps < 1 || !ms) return kamino_fail(KAMINO_ERR_INVALID, "reps must be >= 1 and ms non-null");
    KFrames* f = nullptr;
    if ((rc = frame_state(h, &f))) return rc;
    KGeo g;
    KBufs b;
    int cu, cr;
    if ((rc = kamino_internal_desc(h, &g, &b, nullptr, &cu, &cr))) return rc;
    KFrameSlot& s = f->slot[kind][f->head[kind]];
    if (s.pending) return kamino_fail(KAMINO_ERR_INVALID, "write the captured frames before timing");
    if ((rc = prepare_slot(f, g, b, kind, s))) return rc;
    cudaStream_t st = kamino_internal_stream(h);
    cudaEvent_t e0, e1;
    FCUDA(cudaEventCreate(&e0));
    FCUDA(cudaEventCreate(&e1));
    double total = 0.0;
    for (int r = 0; r < reps && !rc; r++) {
        if (flush_l2 && (rc = kamino_internal_flush_l2(h))) break;
        cudaEventRecord(e0, st);
        rc = launch_pack(g, b, cu, cr, kind, s.dev, st, f->colors);
        cudaEventRecord(e1, st);
        float t = 0.0f;
        if (!rc && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess)
            total += t;
        else if (!rc)
            rc = kamino_fail(KAMINO_ERR_CUDA, "pack timing: %s", cudaGetErrorString(cudaGetLastError()));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *ms = total / reps;
    return KAMINO_OK;
}

// ------------------------------------------------------------ image input
namespace {

// Source pixels and weight of each destination column (or row), as
// cv::resize INTER_LINEAR places them: f = (d + 0.5) * (src / dst) - 0.5 in
// double, rounded to float; s = floor(f), a = f - s; clamped at both edges
// with a = 0.  mirror counts the columns from the right (cv::flip code 1).
std::vector<ImgAxis> image_axis(int src, int dst, bool mirror)
{
    std::vector<ImgAxis> ax((size_t)dst);
    const double scale = (double)src / dst;
    for (int d = 0; d < dst; d++) {
        const float f = (float)((d + 0.5) * scale - 0.5);
        int s0 = (int)std::floor(f);
        float a = f - (float)s0;
        if (s0 < 0) {
            s0 = 0;
            a = 0.0f;
        }
        if (s0 >= src - 1) {
            s0 = src - 1;
            a = 0.0f;
        }
        int s1 = std::min(s0 + 1, src - 1);
        if (mirror) {
            s0 = src - 1 - s0;
            s1 = src - 1 - s1;
        }
        ax[(size_t)d] = {s0, s1, a};
    }
    return ax;
}

// Uploads the image and the axis tables into one scratch allocation and runs
// k_image_resample; on success *scratch holds the allocation, *px the
// nPhi x nTheta resampled pixels inside it (the caller frees *scratch).
int resample(kamino_handle h, const uint8_t* bgr, int width, int height, size_t stride, float* rho, void** scratch,
             uchar4** px)
{
    *scratch = nullptr;
    if (!bgr || width < 1 || height < 1 || (int64_t)width * height > ((int64_t)1 << 28) ||
        stride < 3 * (size_t)width)
        return kamino_fail(KAMINO_ERR_INVALID, "image %dx%d with row stride %zu: bad size or null pixels", width,
                           height, stride);
    KGeo g;
    int rc = kamino_internal_desc(h, &g, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    const std::vector<ImgAxis> ax = image_axis(width, g.np, true), ay = image_axis(height, g.nt, false);
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t row = 3 * (size_t)width, img_b = up(row * height), ax_b = up(sizeof(ImgAxis) * ax.size()),
                 ay_b = up(sizeof(ImgAxis) * ay.size()), px_b = sizeof(uchar4) * (size_t)g.np * g.nt;
    char* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, img_b + ax_b + ay_b + px_b);
    if (e != cudaSuccess) return kamino_fail(KAMINO_ERR_ALLOC, "image scratch: %s", cudaGetErrorString(e));
    *scratch = d;
    cudaStream_t st = kamino_internal_stream(h);
    FCUDA(cudaMemcpy2DAsync(d, row, bgr, stride, row, height, cudaMemcpyHostToDevice, st));
    FCUDA(cudaMemcpyAsync(d + img_b, ax.data(), sizeof(ImgAxis) * ax.size(), cudaMemcpyHostToDevice, st));
    FCUDA(cudaMemcpyAsync(d + img_b + ax_b, ay.data(), sizeof(ImgAxis) * ay.size(), cudaMemcpyHostToDevice, st));
    *px = (uchar4*)(d + img_b + ax_b + ay_b);
    const unsigned blocks = (unsigned)(((size_t)g.np * g.nt + FRAME_THREADS - 1) / FRAME_THREADS);
    k_image_resample<<<blocks, FRAME_THREADS, 0, st>>>(g, (const uint8_t*)d, row, (const ImgAxis*)(d + img_b),
                                                       (const ImgAxis*)(d + img_b + ax_b), *px, rho);
    FCUDA(cudaGetLastError());
    return KAMINO_OK;
}

int finish_image(kamino_handle h, int rc, void* scratch)
{
    if (!rc) {
        const cudaError_t e = cudaStreamSynchronize(kamino_internal_stream(h));
        if (e != cudaSuccess) rc = kamino_fail(KAMINO_ERR_CUDA, "image input: %s", cudaGetErrorString(e));
    } else {
        cudaStreamSynchronize(kamino_internal_stream(h));
    }
    if (scratch) cudaFree(scratch);
    return rc;
}

}  // namespace

// KaminoSolver::initDensityfromPic (KaminoSolver.cu:243-277) with a decoded
// image: the thickness of every cell from the mirrored, resampled image.
extern "C" int kamino_init_density_image(kamino_handle h, const uint8_t* bgr, int width, int height, size_t stride)
{
    KFrames* f = nullptr;
    int rc = frame_state(h, &f);  // makes the handle's device current
    if (rc) return rc;
    KBufs b;
    int cr;
    if ((rc = kamino_internal_desc(h, nullptr, &b, nullptr, nullptr, &cr))) return rc;
    void* scratch = nullptr;
    uchar4* px = nullptr;
    rc = resample(h, bgr, width, height, stride, b.rho[cr], &scratch, &px);
    return finish_image(h, rc, scratch);
}

// The colours KaminoParticles takes from its image (KaminoParticles.cu:6-17,
// 56-72) for the particles as they are now.
extern "C" int kamino_init_particle_colors_image(kamino_handle h, const uint8_t* bgr, int width, int height,
                                                 size_t stride)
{
    KFrames* f = nullptr;
    int rc = frame_state(h, &f);
    if (rc) return rc;
    KGeo g;
    KBufs b;
    int cr;
    if ((rc = kamino_internal_desc(h, &g, &b, nullptr, nullptr, &cr))) return rc;
    if (b.npart == 0) return KAMINO_OK;
    if (!f->colors) {
        const cudaError_t e = cudaMalloc((void**)&f->colors, sizeof(float) * 3 * (size_t)b.npart);
        if (e != cudaSuccess) {
            f->colors = nullptr;
            return kamino_fail(KAMINO_ERR_ALLOC, "particle colours: %s", cudaGetErrorString(e));
        }
    }
    void* scratch = nullptr;
    uchar4* px = nullptr;
    rc = resample(h, bgr, width, height, stride, nullptr, &scratch, &px);
    if (!rc) {
        const unsigned blocks = (unsigned)((b.npart + FRAME_THREADS - 1) / FRAME_THREADS);
        k_particle_colors<<<blocks, FRAME_THREADS, 0, kamino_internal_stream(h)>>>(g, b.part[cr], b.npart, px,
                                                                                   f->colors);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = kamino_fail(KAMINO_ERR_CUDA, "particle colours: %s", cudaGetErrorString(e));
    }
    return finish_image(h, rc, scratch);
}
