// fgpu_disk_force_static: the disk-on-body force and gas-mass reduction with
// no device allocation at all.
//
// Who needs this: code that holds the surface density and scale height in its
// own device buffers and may not allocate device memory when it asks for the
// force -- for example a host driver that runs under a fixed device-memory
// budget negotiated up front, code called back from inside a library that
// forbids allocation on its hot path, or a caller that must not synchronise
// the device (cudaMalloc/cudaFree can).  The regular entry point,
// fgpu_disk_on_planet_accel, needs an engine handle, whose creation allocates
// every field and a scratch buffer for the per-ring partial sums.
//
// Here the per-ring partial sums go to a file-scope static device array of
// fixed size instead, so the call allocates nothing; the caller passes the
// inputs and the output as device pointers.
#include "../../include/fargocpt_gb300.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace {

// Largest ring count the scratch holds: FargoCPT's own MAX1D (src/types.h:76).
constexpr int kMaxRings = 16384;
constexpr int kWidth = 5;  // inner x, inner y, outer x, outer y, mass

// Shared by every call on a device; it keeps the last call's contents.  Every
// call rewrites each row it later reads, so nothing has to be cleared first.
static __device__ __align__(256) double g_ring_partials[kMaxRings * kWidth];

// Device address of the array per device, from cudaGetSymbolAddress.  The
// address is looked up again on every call that is not being captured into a
// CUDA graph (a reset device or a new primary context may load the module at
// another address); a call made while its stream captures uses the address
// the last uncaptured call on that device found.  The mutex orders first
// calls from several host threads.
constexpr int kMaxDevices = 64;
static double *g_scratch_addr[kMaxDevices];
static bool g_scratch_ready[kMaxDevices];
static std::mutex g_scratch_mutex;

__device__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum(double v, double *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double x = lane < nw ? red[lane] : 0.0;
        x = warp_sum(x);
        if (lane == 0) red[32] = x;
    }
    __syncthreads();
    return red[32];
}

// One block per active ring i = 1 .. nrad-2 (ComputeDiskOnPlanetAccel,
// src/Force.cpp:23-122, with the ring-mean density subtracted as
// CorrectDiskSelfgravity, FargoCPT's default without self-gravity, does at
// src/Force.cpp:64-66; gas_total_mass, src/quantities.cpp:51-74).  The ring
// metric is formed from the radii.
__global__ void k_force_rows(const double *__restrict__ S, const double *__restrict__ H,
                             const double *__restrict__ radii, int naz, double G, double eps,
                             double px, double py, double pa, double rsm,
                             double *__restrict__ rows)
{
    __shared__ double red[33];
    const int i = blockIdx.x + 1;
    const size_t row = (size_t)i * naz;
    const double rinf = radii[i], rsup = radii[i + 1];
    const double rmed = 2.0 / 3.0 * (rsup * rsup * rsup - rinf * rinf * rinf) /
                        (rsup * rsup - rinf * rinf);
    const double surf = M_PI * (rsup * rsup - rinf * rinf) / (double)naz;
    const double dphi = 2.0 * M_PI / (double)naz;
    double ps = 0.0;
    for (int j = threadIdx.x; j < naz; j += blockDim.x) ps += S[row + j];
    const double sigma1d = block_sum(ps, red) / naz;
    double ax = 0.0, ay = 0.0, mass = 0.0;
    for (int j = threadIdx.x; j < naz; j += blockDim.x) {
        double sn, cs;
        sincos(dphi * (double)j, &sn, &cs);
        const double smooth = eps * H[row + j];
        const double dx = rmed * cs - px, dy = rmed * sn - py;
        const double dsm2 = dx * dx + dy * dy + smooth * smooth;
        const double dsm = sqrt(dsm2);
        const double inv3 = 1.0 / (dsm2 * dsm);
        double fk = 1.0;
        if (rsm > 0.0 && dsm < rsm) {
            const double q = dsm / rsm;
            fk = -(3.0 * q * q * q * q - 4.0 * q * q * q);
        }
        const double cellmass = surf * (S[row + j] - sigma1d);
        ax += G * cellmass * dx * inv3 * fk;
        ay += G * cellmass * dy * inv3 * fk;
        mass += surf * S[row + j];
    }
    ax = block_sum(ax, red);
    ay = block_sum(ay, red);
    mass = block_sum(mass, red);
    if (threadIdx.x == 0) {
        const bool inner = rmed < pa;
        double *p = rows + (size_t)blockIdx.x * kWidth;
        p[0] = inner ? ax : 0.0;
        p[1] = inner ? ay : 0.0;
        p[2] = inner ? 0.0 : ax;
        p[3] = inner ? 0.0 : ay;
        p[4] = mass;
    }
}

// Adds the rows in ring order with Kahan compensation into out[0 .. 4].
__global__ void k_sum_rows(const double *__restrict__ rows, int nrows, double *__restrict__ out)
{
    const int w = threadIdx.x;
    if (w >= kWidth) return;
    double s = 0.0, c = 0.0;
    for (int r = 0; r < nrows; ++r) {
        const double y = rows[(size_t)r * kWidth + w] - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    out[w] = s;
}

}  // namespace

extern "C" int fgpu_disk_force_static(const double *sigma, const double *scale_height,
                                      const double *radii, int nrad, int naz, double G,
                                      double thickness_smoothing, const fgpu_body *body,
                                      double *out, void *stream)
{
    if (!sigma || !scale_height || !radii || !body || !out || naz < 1) {
        fprintf(stderr, "fgpu_disk_force_static: null pointer or naz < 1\n");
        return FGPU_ERR_BAD_ARG;
    }
    if (nrad < 3 || nrad - 2 > kMaxRings) {
        fprintf(stderr,
                "fgpu_disk_force_static: nrad = %d outside [3, %d]; the static scratch "
                "holds %d active rings\n",
                nrad, kMaxRings + 2, kMaxRings);
        return FGPU_ERR_BAD_ARG;
    }
    // An error the caller left pending on this thread is not this call's:
    // report it without clearing it, so that the caller can still read it.
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        fprintf(stderr, "fgpu_disk_force_static: an earlier CUDA error is pending: %s\n",
                cudaGetErrorString(pending));
        return FGPU_ERR_CUDA;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return FGPU_ERR_NO_DEVICE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;  // treat as capturing: no lookup
    }
    double *rows = nullptr;
    {
        // The device address of the static scratch (host code may not use
        // the symbol itself as a pointer), looked up with this device
        // current.  A capturing stream cannot make the lookup, so the first
        // call on each device has to come before any stream capture.
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (cap == cudaStreamCaptureStatusNone) {
            cudaError_t e = cudaGetSymbolAddress((void **)&g_scratch_addr[dev], g_ring_partials);
            if (e != cudaSuccess) {
                cudaGetLastError();
                g_scratch_ready[dev] = false;
                fprintf(stderr, "fgpu_disk_force_static: cudaGetSymbolAddress: %s\n",
                        cudaGetErrorString(e));
                return FGPU_ERR_CUDA;
            }
            g_scratch_ready[dev] = true;
        } else if (!g_scratch_ready[dev]) {
            fprintf(stderr, "fgpu_disk_force_static: the first call on a device must not be "
                            "made while its stream captures\n");
            return FGPU_ERR_BAD_ARG;
        }
        rows = g_scratch_addr[dev];
    }
    const int nrows = nrad - 2;
    k_force_rows<<<nrows, 256, 0, s>>>(sigma, scale_height, radii, naz, G, thickness_smoothing,
                                       body->x, body->y, body->a, body->r_sm, rows);
    k_sum_rows<<<1, 32, 0, s>>>(rows, nrows, out);
    // nothing was pending before the launches, so an error now is theirs
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "fgpu_disk_force_static: launch: %s\n", cudaGetErrorString(e));
        return FGPU_ERR_CUDA;
    }
    return FGPU_OK;
}
