// FP32-mixed form of the GB300 hydro step.
//
// Storage and arithmetic are FP32 except for a few FP64 islands.  To keep
// FP32 free of cancellation, the state is stored relative to the Keplerian
// disk: v_phi as the residual dv = v_phi - v_K(Rmed), the potential as the
// residual Phi - Phi_K with Phi_K = -G M / Rmed, and the angular momentum as
// sigma * r * dv.  Sigma is a compensated FP32 pair (hi + lo): every kernel
// computes with the hi part, and the places that change sigma (transport,
// FARGO shift, floor, damping, ghost rings) carry the rounding error of the
// update in lo (Fast2Sum), so FP32 storage does not accumulate a rounding
// error of 2^-24 sigma per step.  The large Keplerian terms that cancel in FargoCPT's
// equations -- the centrifugal vs. gravitational balance of
// momentum_update_radial (SourceEuler.cpp:325-372), the Keplerian shear of
// tau_r_phi (viscosity.cpp:201-207), the Keplerian angular momentum carried
// by the radial mass flux (TransportEuler.cpp:545-591) -- become per-ring
// constants computed once in FP64 on the host.  FP64 remains for the FARGO
// shift phase of every ring, the cell-to-body separations (potential and disk
// force), and the accumulation of the force and mass reductions.
//
// The step has the same phases and order as the FP64 form (kernels_fp64.cu)
// and FargoCPT's step_Euler (simulation.cpp:148-267).  The per-cell, per-column
// and per-ring bodies live in fp32_device.cuh, shared with the batched
// many-disk kernels (batch_fp32.cu); this file holds the single-disk kernels
// around them and the host engine.
#include "../../include/fargocpt_gb300.h"
#include "fp32_engine.h"
#include "fp32_device.cuh"
#include "reduce.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <string>
#include <vector>

namespace fgpu32 {

// ---------------------------------------------------------------------------
// single-disk kernels: one thread per cell (blockIdx.y = ring), one thread per
// column and chunk of rings, or one block per ring
// ---------------------------------------------------------------------------
__global__ void f_potential(GeoF g, TablesF t, PhysF ph, BodiesF b, const float *__restrict__ H,
                            float *__restrict__ pot)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    potential_cell(g, t, ph, b, H, pot, blockIdx.y, j);
}

__global__ void f_source(GeoF g, TablesF t, float dt, const float *__restrict__ S,
                         const float *__restrict__ P, const float *__restrict__ pot,
                         const float *__restrict__ vr_in, const float *__restrict__ dv_in,
                         float *__restrict__ vr_out, float *__restrict__ dv_out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    source_cell(g, t, dt, S, P, pot, vr_in, dv_in, vr_out, dv_out, blockIdx.y, j);
}

__global__ void f_artvisc_q(GeoF g, TablesF t, PhysF ph, float dt, const float *__restrict__ S,
                            const float *__restrict__ vr, const float *__restrict__ dv,
                            float *__restrict__ E, float *__restrict__ Qr, float *__restrict__ Qp)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    artvisc_q_cell(g, t, ph, dt, S, vr, dv, E, Qr, Qp, blockIdx.y, j);
}

__global__ void f_artvisc_v(GeoF g, TablesF t, PhysF ph, float dt, const float *__restrict__ S,
                            const float *__restrict__ E, const float *__restrict__ Qr,
                            const float *__restrict__ Qp, float *__restrict__ vr,
                            float *__restrict__ dv, float *__restrict__ cs, float *__restrict__ H,
                            float *__restrict__ nu)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    artvisc_v_cell(g, t, ph, dt, S, E, Qr, Qp, vr, dv, cs, H, nu, blockIdx.y, j);
}

__global__ void f_stress(GeoF g, TablesF t, const float *__restrict__ S, const float *__restrict__ vr,
                         const float *__restrict__ dv, const float *__restrict__ nu,
                         float *__restrict__ divv, float *__restrict__ trr, float *__restrict__ tpp,
                         float *__restrict__ trp)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    stress_cell(g, t, S, vr, dv, nu, divv, trr, tpp, trp, blockIdx.y, j);
}

__global__ void f_viscous(GeoF g, TablesF t, PhysF ph, float dt, float beta_inv, int mode,
                          const float *__restrict__ S, const float *__restrict__ trr,
                          const float *__restrict__ tpp, const float *__restrict__ trp,
                          const float *__restrict__ divv, const float *__restrict__ nu,
                          const float *__restrict__ H, const float *__restrict__ S0,
                          const float *__restrict__ E0, float *__restrict__ vr,
                          float *__restrict__ dv, float *__restrict__ E, float *__restrict__ qplus,
                          float *__restrict__ qminus, const float *__restrict__ corr_phi,
                          const float *__restrict__ corr_r)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    viscous_cell(g, t, ph, dt, beta_inv, mode, S, trr, tpp, trp, divv, nu, H, S0, E0, vr, dv, E,
                 qplus, qminus, corr_phi, corr_r, blockIdx.y, j);
}

// StabilizeViscosity's correction factors, rows 1 .. nr - 1
__global__ void f_visc_corr(GeoF g, TablesF t, const float *__restrict__ S,
                            const float *__restrict__ nu, float *__restrict__ corr_phi,
                            float *__restrict__ corr_r)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y + 1;
    if (j >= g.nz || i >= g.nr) return;
    visc_corr_cell(g, t, S, nu, corr_phi, corr_r, i, j);
}

__global__ void f_ghost(GeoF g, BcF bc, StateF s)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    ghost_col(g, bc, s, j);
}

// 64-thread blocks, 16 per SM (64 registers, about 100 bytes of spills to
// L1, which the kernel leaves unshared).  FP32 step of the 2048 x 6144 disk:
// 2.321 ms, against 2.342 at 80 registers, 2.346 at 96 and 2.399 at 115.
template <int NQ>
__global__ void __launch_bounds__(64, 16) f_transport_radial(GeoF g, TablesF t, float dt, int mc, int chunk,
                                   const float *__restrict__ S, const float *__restrict__ vr,
                                   const float *__restrict__ dv, const float *__restrict__ E,
                                   float *__restrict__ m0, float *__restrict__ m1,
                                   float *__restrict__ m2, float *__restrict__ m3,
                                   float *__restrict__ E_out, float *__restrict__ S_out,
                                   const float *__restrict__ S_lo, float *__restrict__ S_lo_out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    radial_col<NQ>(g, t, dt, mc, chunk, S, vr, dv, E, m0, m1, m2, m3, E_out, S_out, S_lo,
                   S_lo_out, blockIdx.y * chunk, j);
}

template <int PER, int NQ, bool STAGE>
__global__ void __launch_bounds__(512) f_transport_azimuthal(GeoF g, TablesF t, double dt, int mc,
                                                             int fast,
                                                             const float *__restrict__ dv,
                                                             float *m0, float *m1, float *m2,
                                                             float *m3, float *E, float *S,
                                                             float *S_lo, int *ring_shift)
{
    extern __shared__ __align__(16) float smf[];
    __shared__ float redf[33];
    __shared__ long long redl[33];
    azimuthal_ring<PER, NQ, STAGE>(g, t, dt, mc, fast, dv, m0, m1, m2, m3, E, S, S_lo,
                                   blockIdx.x, smf, redf, redl, ring_shift);
}

// the register-blocked ring transport (azimuthal_ring_rb): nz = PER x blockDim.x
template <int PER, int NQ>
__global__ void __launch_bounds__(rb_max_threads(PER)) f_transport_azimuthal_rb(GeoF g, TablesF t, double dt,
                                                                int mc, int fast,
                                                                const float *__restrict__ dv,
                                                                float *m0, float *m1, float *m2,
                                                                float *m3, float *E, float *S,
                                                                float *S_lo, int *ring_shift)
{
    extern __shared__ __align__(16) float smf[];
    __shared__ float redf[33];
    __shared__ long long redl[33];
    azimuthal_ring_rb<PER, NQ>(g, t, dt, mc, fast, dv, m0, m1, m2, m3, E, S, S_lo, blockIdx.x,
                               smf, redf, redl, ring_shift);
}

__global__ void f_pressure(GeoF g, TablesF t, PhysF ph, const float *__restrict__ S,
                           const float *__restrict__ E, float *__restrict__ P)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    pressure_cell(g, t, ph, S, E, P, blockIdx.y, j);
}

__global__ void f_finish(GeoF g, TablesF t, PhysF ph, const float *__restrict__ m0,
                         const float *__restrict__ m1, const float *__restrict__ m2,
                         const float *__restrict__ m3, const float *__restrict__ S_t,
                         const float *__restrict__ E_t, const float *__restrict__ vr_in,
                         float *__restrict__ vr_out, float *__restrict__ dv_out,
                         float *__restrict__ S_out, float *__restrict__ E_out,
                         const float *__restrict__ Slo_t, float *__restrict__ Slo_out,
                         const int *__restrict__ shift)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    finish_cell(g, t, ph, m0, m1, m2, m3, S_t, E_t, vr_in, vr_out, dv_out, S_out, E_out, Slo_t,
                Slo_out, shift, blockIdx.y, j);
}

__global__ void f_damping(GeoF g, DampingF dm, float dt, const int *__restrict__ rings, StateF s)
{
    __shared__ float red[33];
    __shared__ long long redl[33];
    // one block per (ring, damped field)
    damping_ring(g, dm, dt, s, rings[blockIdx.x], red, redl, blockIdx.y, blockIdx.y + 1);
}

__global__ void f_derived_cfl(GeoF g, TablesF t, PhysF ph, int mode, const float *__restrict__ S,
                              const float *__restrict__ E, const float *__restrict__ vr,
                              const float *__restrict__ dv, const float *__restrict__ qplus,
                              const float *__restrict__ qminus, float *__restrict__ cs,
                              float *__restrict__ H, float *__restrict__ P, float *__restrict__ T,
                              float *__restrict__ nu, unsigned int *__restrict__ dt_min,
                              const float *__restrict__ corr_phi,
                              const float *__restrict__ corr_r)
{
    __shared__ float red[33];
    __shared__ longlong2 red2[33];
    derived_cfl_ring(g, t, ph, mode, S, E, vr, dv, qplus, qminus, cs, H, P, T, nu, dt_min,
                     blockIdx.x, red, red2, corr_phi, corr_r);
}

// disk force on up to kForceBodies32 bodies in one pass over the ring, and the
// gas mass: separations as float pairs, sums as compensated float pairs per
// thread and in FP64 across the block.  partial[5 b .. 5 b + 4] of the ring's
// row: inner x, inner y, outer x, outer y, mass (ComputeDiskOnPlanetAccel,
// Force.cpp:23-122; the ring mean removed with CorrectDiskSelfgravity,
// Force.cpp:64-66; gas_total_mass, quantities.cpp:51-74).
constexpr int kForceBodies32 = 4;
struct ForceBodies32 {
    int n;
    double x[kForceBodies32], y[kForceBodies32], a[kForceBodies32], rsm[kForceBodies32];
};

__global__ void f_disk_force_bodies(GeoF g, TablesF t, PhysF ph, ForceBodies32 fb,
                                    const float *__restrict__ S,
                                    const float *__restrict__ S_lo, const float *__restrict__ H,
                                    double *__restrict__ partial, int width)
{
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x + 1;
    const size_t row = (size_t)i * nz;
    // sigma as its compensated pair; the ring sum gives the ring mean and,
    // times the cell area, the ring's mass.  Each thread sums its cells as a
    // compensated float pair (TwoSum, Knuth 1969), the block in FP64.
    float sh_ = 0.f, sl_ = 0.f;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        two_sum_add(sh_, sl_, S[row + j]);
        sl_ += S_lo[row + j];
    }
    const double ring_sum = bsum_d((double)sh_ + (double)sl_, red);
    const double sigma1d = ph.correct_sg ? ring_sum / nz : 0.0;
    const float mh = (float)sigma1d, ml = (float)(sigma1d - (double)mh);
    // cell centres and the bodies as float pairs (see potential_cell): the
    // distance loses nothing to cancellation near a body
    float pxh[kForceBodies32], pxl[kForceBodies32], pyh[kForceBodies32], pyl[kForceBodies32];
    float frsm[kForceBodies32];
#pragma unroll
    for (int b = 0; b < kForceBodies32; ++b) {
        const double px = b < fb.n ? fb.x[b] : 0.0, py = b < fb.n ? fb.y[b] : 0.0;
        pxh[b] = (float)px;
        pxl[b] = (float)(px - (double)pxh[b]);
        pyh[b] = (float)py;
        pyl[b] = (float)(py - (double)pyh[b]);
        frsm[b] = b < fb.n ? (float)fb.rsm[b] : 0.f;
    }
    const float rh = t.Rmed[i], rl = t.RmedLo[i];
    float axh[kForceBodies32], axl[kForceBodies32], ayh[kForceBodies32], ayl[kForceBodies32];
#pragma unroll
    for (int b = 0; b < kForceBodies32; ++b) axh[b] = axl[b] = ayh[b] = ayl[b] = 0.f;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const float ch = t.cosHi[j], cl = t.cosLo[j], sh = t.sinHi[j], sl = t.sinLo[j];
        const float xh = rh * ch, yh = rh * sh;
        const float xl = fmaf(rh, ch, -xh) + fmaf(rh, cl, rl * ch);
        const float yl = fmaf(rh, sh, -yh) + fmaf(rh, sl, rl * sh);
        const float sm = ph.eps_smooth * H[row + j];
        const float sm2 = sm * sm;
        // the ring mean removed (CorrectDiskSelfgravity) from the pair
        const float dsig = ph.correct_sg ? (S[row + j] - mh) + (S_lo[row + j] - ml)
                                         : S[row + j] + S_lo[row + j];
#pragma unroll
        for (int b = 0; b < kForceBodies32; ++b) {
            if (b < fb.n) {
                const float dx = (xh - pxh[b]) + (xl - pxl[b]);
                const float dy = (yh - pyh[b]) + (yl - pyl[b]);
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, sm2));
                const float rinv = rsqrtf(d2);
                float fk = 1.f;
                if (frsm[b] > 0.f) {
                    const float dsm = d2 * rinv;
                    if (dsm < frsm[b]) {
                        const float q = dsm / frsm[b];
                        fk = -(3.f * q * q * q * q - 4.f * q * q * q);
                    }
                }
                const float w = dsig * (rinv * rinv * rinv * fk);
                two_sum_add(axh[b], axl[b], w * dx);
                two_sum_add(ayh[b], ayl[b], w * dy);
            }
        }
    }
    const double f = t.Surf_d[i] * ph.G_d;
    double *p = partial + (size_t)blockIdx.x * width;
#pragma unroll
    for (int b = 0; b < kForceBodies32; ++b) {
        if (b < fb.n) {
            const double ax = bsum_d((double)axh[b] + (double)axl[b], red);
            const double ay = bsum_d((double)ayh[b] + (double)ayl[b], red);
            if (threadIdx.x == 0) {
                const bool inner = t.Rmed_d[i] < fb.a[b];
                p[5 * b + 0] = inner ? f * ax : 0.0;
                p[5 * b + 1] = inner ? f * ay : 0.0;
                p[5 * b + 2] = inner ? 0.0 : f * ax;
                p[5 * b + 3] = inner ? 0.0 : f * ay;
                p[5 * b + 4] = t.Surf_d[i] * ring_sum;
            }
        }
    }
}

// the rows' components, one block (one warp) per component
__global__ void f_reduce_cols(const double *__restrict__ partial, int rows, int width,
                              double *__restrict__ out)
{
    warp_compensated_rows(partial, rows, width, blockIdx.x, out);
}

// one warp per component
__global__ void f_reduce_rows(const double *__restrict__ partial, int rows, double *__restrict__ out)
{
    const int w = threadIdx.x >> 5;
    if (w < 5) warp_compensated_rows(partial, rows, 5, w, out);
}
__global__ void f_reduce_rows2(const double *__restrict__ partial, int rows, double *__restrict__ out)
{
    const int w = threadIdx.x >> 5;
    if (w < 2) warp_compensated_rows(partial, rows, 2, w, out);
}

// gas_total_mass and gas_angular_momentum (quantities.cpp:51-74, 242-276)
// of each active ring with Rmed <= radius: sigma from its compensated pair
// and the inertial azimuthal speed (the stored residual plus v_K(Rmed)), all
// in FP64; one block per ring writes (mass, angular momentum).
__global__ void f_gas_quantities(GeoF g, TablesF t, double radius, const float *__restrict__ S,
                                 const float *__restrict__ S_lo, const float *__restrict__ dv,
                                 double *__restrict__ partial)
{
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x + 1;
    const size_t row = (size_t)i * nz;
    const double vref = t.Vref_d[i];
    double m = 0.0, l = 0.0;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const size_t c = row + j, cm = row + (j == 0 ? nz - 1 : j - 1);
        const double sj = (double)S[c] + (double)S_lo[c];
        const double sm = (double)S[cm] + (double)S_lo[cm];
        m += sj;
        l += 0.5 * (sj + sm) * ((double)dv[c] + vref);
    }
    m = bsum_d(m, red);
    l = bsum_d(l, red);
    if (threadIdx.x == 0) {
        const bool in = t.Rmed_d[i] <= radius;
        partial[(size_t)blockIdx.x * 2] = in ? t.Surf_d[i] * m : 0.0;
        partial[(size_t)blockIdx.x * 2 + 1] = in ? t.Surf_d[i] * t.Rmed_d[i] * l : 0.0;
    }
}

// KeepDiskMassConstant on the compensated pair: (hi + lo) * target / mass
// in FP64, split again into the pair.
__global__ void f_scale_sigma(float *__restrict__ S, float *__restrict__ S_lo, size_t n,
                              double target, const double *__restrict__ mass)
{
    const double factor = target / mass[0];
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x) {
        const double v = ((double)S[k] + (double)S_lo[k]) * factor;
        const float h = (float)v;
        S[k] = h;
        S_lo[k] = (float)(v - (double)h);
    }
}

__global__ void f_check_finite(const float *__restrict__ x, size_t n, unsigned long long *bad)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && !isfinite(x[k])) atomicMin(bad, (unsigned long long)k);
}

// FP64 <-> FP32 field conversion with the per-ring reference profile
__global__ void f_to_f32(const double *__restrict__ in, float *__restrict__ out, size_t n, int nz,
                         const double *__restrict__ ring_offset)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = (float)(in[k] - (ring_offset ? ring_offset[k / nz] : 0.0));
}
__global__ void f_to_f64(const float *__restrict__ in, double *__restrict__ out, size_t n, int nz,
                         const double *__restrict__ ring_offset)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = (double)in[k] + (ring_offset ? ring_offset[k / nz] : 0.0);
}
__global__ void f_split_f32(const double *__restrict__ in, float *__restrict__ hi,
                            float *__restrict__ lo, size_t n)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        const float h = (float)in[k];
        hi[k] = h;
        lo[k] = (float)(in[k] - (double)h);
    }
}
__global__ void f_join_f64(const float *__restrict__ hi, const float *__restrict__ lo,
                           double *__restrict__ out, size_t n)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = (double)hi[k] + (double)lo[k];
}

// ===========================================================================
// host side
// ===========================================================================

static bool is_vec(int f) { return f == FGPU_V_RADIAL || f == FGPU_V_RADIAL0 || f == FGPU_TAU_R_PHI; }

// the launch just made failed: name it
#define CKL(what)                                                           \
    do {                                                                    \
        cudaError_t e_ = cudaGetLastError();                                \
        if (e_ != cudaSuccess) {                                            \
            err = std::string("launch of ") + (what) + ": " + cudaGetErrorString(e_); \
            return FGPU_ERR_CUDA;                                           \
        }                                                                   \
    } while (0)

#define CKF(call)                                                           \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);      \
            return FGPU_ERR_CUDA;                                           \
        }                                                                   \
    } while (0)

int Engine32::create(const fgpu_params &prm, const double *radii, cudaStream_t s)
{
    p = prm;
    stream = s;
    nr = p.nrad;
    nz = p.naz;
    cells = (size_t)nr * nz;
    vcells = (size_t)(nr + 1) * nz;
    const double dphi = 2.0 * M_PI / (double)nz, invdphi = (double)nz / (2.0 * M_PI);
    geo = GeoF{nr, nz, (float)dphi, (float)invdphi, dphi, invdphi};
    const double G = p.G, M = p.hydro_center_mass;
    const int R = nr + 2;
    auto pw = [](double x, double e) { return std::pow(x, e); };
    std::vector<double> Rinf(R), Rsup(R), Rmed(R), Surf(R), Vref(R), PhiK(R), Jref(R);
    for (int n = 0; n <= nr; ++n) {
        Rinf[n] = radii[n];
        Rsup[n] = radii[n + 1];
        Rmed[n] = 2.0 / 3.0 * (pw(Rsup[n], 3) - pw(Rinf[n], 3)) / (pw(Rsup[n], 2) - pw(Rinf[n], 2));
        Surf[n] = M_PI * (pw(Rsup[n], 2) - pw(Rinf[n], 2)) / (double)nz;
        Vref[n] = std::sqrt(G * M / Rmed[n]);
        PhiK[n] = -G * M / Rmed[n];
        Jref[n] = Vref[n] * Rmed[n];
    }
    enum { RINF, RSUP, RMED, SURF, INVRMED, INVSURF, INVDIFFRMED, INVDIFFRSUP, INVDIFFRSUPRB,
           INVRINF, RINFSQ, TWOOVER, OMEGAK, INVOMEGAK, CSISO, INVDXSRC, INVDXTHETA, EMODEL,
           HFACADI, INVCELL, INVCELL2, TWOOVERRMEDSUM, KBAL, AFACE, SHEAR, DJ, JSLOPE, DRMED,
           OMREFDIFF, VREF, DRSUP, RSUPIDRR, LSQTW, TWOOVERDRMED2, RA3IDRMED, F43, CRPP1,
           CRPP2, CRRR1, CRRR2, CRRP, CRSCALE, RMEDLO, RINFOFF, NT };
    std::vector<float> hf((size_t)NT * R, 0.f);
    auto F = [&](int k) { return hf.data() + (size_t)k * R; };
    for (int n = 0; n <= nr; ++n) {
        const double rm = Rmed[n], dxr = Rsup[n] - Rinf[n], dxa = rm * dphi;
        F(DRSUP)[n] = (float)dxr;
        F(RSUPIDRR)[n] = (float)(Rsup[n] / (dxr * rm));
        F(F43)[n] = (float)(4.0 / 3.0 / rm * (1.0 / dphi) * (1.0 / dphi));
        F(CRRP)[n] = (float)(1.0 / (dphi * dphi * Rinf[n]));
        if (n >= 1) {
            F(RA3IDRMED)[n] = (float)(std::pow(Rinf[n], 3) / (rm - Rmed[n - 1]));
        }
        if (n < nr) {
            // artificial_viscosity.cpp:60-73
            const double Dr = Rinf[n + 1] - Rinf[n];
            const double dxtw = nz <= 16 ? std::min(Dr, dxa) : std::max(Dr, dxa);
            F(LSQTW)[n] = (float)(std::pow(p.art_visc_factor, 2) * std::pow(dxtw, 2));
        }
        const double om = std::sqrt(G * M / (rm * rm * rm));
        const double cell = std::min(dxr, dxa);
        F(RINF)[n] = (float)Rinf[n];
        F(RSUP)[n] = (float)Rsup[n];
        F(RMED)[n] = (float)rm;
        F(RMEDLO)[n] = (float)(rm - (double)(float)rm);
        if (n >= 1) F(RINFOFF)[n] = (float)(Rinf[n] - 0.5 * (Rmed[n] + Rmed[n - 1]));
        F(SURF)[n] = (float)Surf[n];
        F(INVRMED)[n] = (float)(1.0 / rm);
        F(INVSURF)[n] = (float)(1.0 / Surf[n]);
        F(INVDIFFRSUP)[n] = (float)(1.0 / dxr);
        F(INVDIFFRSUPRB)[n] = (float)(1.0 / (dxr * rm));
        F(INVRINF)[n] = (float)(1.0 / Rinf[n]);
        F(RINFSQ)[n] = (float)(Rinf[n] * Rinf[n]);
        F(OMEGAK)[n] = (float)om;
        F(INVOMEGAK)[n] = (float)(1.0 / om);
        F(CSISO)[n] = (float)(p.aspect_ratio * pw(rm, p.flaring_index) * std::sqrt(G * M / rm));
        F(INVDXSRC)[n] = (float)(2.0 / (dphi * (Rsup[n] + Rinf[n])));
        F(INVDXTHETA)[n] = (float)(1.0 / (dphi * rm));
        F(EMODEL)[n] = (float)(1.0 / (p.gamma - 1.0) * pw(p.aspect_ratio, 2) *
                               pw(rm, 2.0 * p.flaring_index - 1.0) * G * M);
        F(HFACADI)[n] = (float)(1.0 / om / std::sqrt(p.gamma));
        F(INVCELL)[n] = (float)(1.0 / cell);
        F(INVCELL2)[n] = (float)(1.0 / (cell * cell));
        F(VREF)[n] = (float)Vref[n];
    }
    for (int n = 0; n < nr; ++n) {
        F(TWOOVER)[n] = (float)(2.0 / (Rinf[n + 1] * Rinf[n + 1] - Rinf[n] * Rinf[n]));
        F(JSLOPE)[n] = (float)((Jref[n + 1] - Jref[n]) / (Rmed[n + 1] - Rmed[n]));
        F(OMREFDIFF)[n] = (float)(Vref[n] / Rmed[n] - Vref[n + 1] / Rmed[n + 1]);
    }
    for (int n = 1; n <= nr; ++n) {
        const double idr = 1.0 / (Rmed[n] - Rmed[n - 1]);
        F(INVDIFFRMED)[n] = (float)idr;
        F(TWOOVERRMEDSUM)[n] = (float)(2.0 / (Rmed[n] + Rmed[n - 1]));
        F(DRMED)[n] = (float)(Rmed[n] - Rmed[n - 1]);
        F(TWOOVERDRMED2)[n] = (float)(2.0 / (std::pow(Rmed[n], 2) - std::pow(Rmed[n - 1], 2)));
        {
            // StabilizeViscosity ring terms, viscosity.cpp:280-331 (Ra = Rinf)
            const double ra = Rinf[n], idr_sup = 1.0 / (Rsup[n] - Rinf[n]);
            const double idr_sup_m = 1.0 / (Rsup[n - 1] - Rinf[n - 1]);
            const double irb = 1.0 / ((Rsup[n] - Rinf[n]) * Rmed[n]);
            const double irb_m = 1.0 / ((Rsup[n - 1] - Rinf[n - 1]) * Rmed[n - 1]);
            F(CRPP1)[n] = (float)(2.0 * (0.5 / Rmed[n] + 1.0 / 3.0 * ra * irb));
            F(CRPP2)[n] = (float)(2.0 * (0.5 / Rmed[n - 1] - 1.0 / 3.0 * ra * irb_m));
            F(CRRR1)[n] = (float)(Rmed[n] * 2.0 * (-idr_sup + 1.0 / 3.0 * ra * irb));
            F(CRRR2)[n] = (float)(-1.0 * Rmed[n - 1] * 2.0 * (idr_sup_m - 1.0 / 3.0 * ra * irb_m));
            F(CRSCALE)[n] = (float)(p.radial_viscosity_factor / (0.5 * (Rmed[n] + Rmed[n - 1])));
        }
        F(DJ)[n] = (float)(Jref[n - 1] - Jref[n]);
        F(SHEAR)[n] = (float)((Vref[n] / Rmed[n] - Vref[n - 1] / Rmed[n - 1]) * idr);
        const double A = 0.5 * (Vref[n] + Vref[n - 1]);
        F(AFACE)[n] = (float)A;
        F(KBAL)[n] = (float)(A * A / Rinf[n] - (PhiK[n] - PhiK[n - 1]) * idr);
    }
    F(DRMED)[nr + 1] = (float)(Rmed[nr] - Rmed[nr - 1]);
    // device copies: float tables, then double tables (Rmed, InvRmed, Vref,
    // Surf, PhiK, cos, sin)
    std::vector<double> hd((size_t)5 * R + 2 * (size_t)nz);
    for (int n = 0; n < R; ++n) {
        hd[n] = Rmed[n];
        hd[R + n] = 1.0 / Rmed[n];
        hd[2 * R + n] = Vref[n];
        hd[3 * R + n] = Surf[n];
        hd[4 * R + n] = PhiK[n];
    }
    for (int j = 0; j < nz; ++j) {
        hd[5 * R + j] = std::cos(dphi * (double)j);
        hd[5 * R + nz + j] = std::sin(dphi * (double)j);
    }
    CKF(cudaMalloc(&tab_f, sizeof(float) * hf.size()));
    CKF(cudaMemcpy(tab_f, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice));
    CKF(cudaMalloc(&tab_d, sizeof(double) * hd.size()));
    CKF(cudaMemcpy(tab_d, hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice));
    std::vector<float> hc((size_t)4 * nz);
    for (int j = 0; j < nz; ++j) {
        const double c = hd[5 * R + j], sn = hd[5 * R + nz + j];
        hc[j] = (float)c;
        hc[nz + j] = (float)(c - (double)hc[j]);
        hc[2 * nz + j] = (float)sn;
        hc[3 * nz + j] = (float)(sn - (double)hc[2 * nz + j]);
    }
    CKF(cudaMalloc(&tab_c, sizeof(float) * hc.size()));
    CKF(cudaMemcpy(tab_c, hc.data(), sizeof(float) * hc.size(), cudaMemcpyHostToDevice));
    auto Df = [&](int k) -> const float * { return tab_f + (size_t)k * R; };
    TablesF &t = tabs;
    t.Rinf = Df(RINF); t.Rsup = Df(RSUP); t.Rmed = Df(RMED); t.Surf = Df(SURF);
    t.InvRmed = Df(INVRMED); t.InvSurf = Df(INVSURF); t.InvDiffRmed = Df(INVDIFFRMED);
    t.InvDiffRsup = Df(INVDIFFRSUP); t.InvDiffRsupRb = Df(INVDIFFRSUPRB); t.InvRinf = Df(INVRINF);
    t.RinfSq = Df(RINFSQ); t.TwoOverDRa2 = Df(TWOOVER); t.OmegaK = Df(OMEGAK);
    t.InvOmegaK = Df(INVOMEGAK); t.CsIso = Df(CSISO); t.InvDxSrc = Df(INVDXSRC);
    t.InvDxTheta = Df(INVDXTHETA); t.EModel = Df(EMODEL); t.HFacAdi = Df(HFACADI);
    t.InvCell = Df(INVCELL); t.InvCell2 = Df(INVCELL2); t.TwoOverRmedSum = Df(TWOOVERRMEDSUM);
    t.Kbal = Df(KBAL); t.Aface = Df(AFACE); t.Shear = Df(SHEAR); t.DJ = Df(DJ);
    t.JSlope = Df(JSLOPE); t.DRmed = Df(DRMED); t.DRsup = Df(DRSUP); t.RsupIDRR = Df(RSUPIDRR);
    t.LSqTW = Df(LSQTW); t.TwoOverDRmed2 = Df(TWOOVERDRMED2);
    t.Ra3IDRmed = Df(RA3IDRMED); t.F43 = Df(F43); t.CrPp1 = Df(CRPP1); t.CrPp2 = Df(CRPP2);
    t.CrRr1 = Df(CRRR1); t.CrRr2 = Df(CRRR2); t.CrRp = Df(CRRP); t.CrScale = Df(CRSCALE); t.OmRefDiff = Df(OMREFDIFF); t.Vref = Df(VREF);
    t.Rmed_d = tab_d; t.InvRmed_d = tab_d + R; t.Vref_d = tab_d + 2 * R; t.Surf_d = tab_d + 3 * R;
    t.PhiK_d = tab_d + 4 * R; t.cos_d = tab_d + 5 * R; t.sin_d = tab_d + 5 * R + nz;
    t.RmedLo = Df(RMEDLO);
    t.RinfOff = Df(RINFOFF);
    t.cosHi = tab_c; t.cosLo = tab_c + nz; t.sinHi = tab_c + 2 * nz; t.sinLo = tab_c + 3 * nz;

    // physics
    PhysF &ph = phys;
    ph.adiabatic = p.eos == FGPU_EOS_IDEAL;
    ph.art_visc_sn = p.art_visc == FGPU_ARTVISC_SN;
    ph.art_visc_tw = p.art_visc == FGPU_ARTVISC_TW;
    ph.stabilize = p.stabilize_viscosity;
    ph.dissipation = p.art_visc_dissipation;
    ph.limiter_mc = p.flux_limiter == FGPU_LIMITER_MC;
    ph.fast_transport = p.fast_transport;
    ph.heating_viscous = p.heating_viscous;
    ph.cooling_beta = p.cooling_beta;
    ph.beta_ref = p.cooling_beta_reference;
    ph.gm1 = (float)(p.gamma - 1.0);
    ph.g_gm1 = (float)(p.gamma * (p.gamma - 1.0));
    ph.mu = (float)p.mu;
    ph.alpha = (float)p.viscous_alpha;
    ph.constant_viscosity = (float)p.constant_viscosity;
    ph.C2 = (float)(p.art_visc_factor * p.art_visc_factor);
    ph.four_C2 = 4.f * ph.C2;
    ph.rvf = (float)p.radial_viscosity_factor;
    ph.hvf = (float)p.heating_viscous_factor;
    ph.cfl = (float)p.cfl;
    ph.leapfrog = p.integrator == FGPU_INTEGRATOR_LEAPFROG;
    ph.inv_hc_limit = (float)(1.0 / p.heating_cooling_cfl_limit);
    ph.sigma_min = (float)(p.sigma_floor * p.sigma0);
    ph.sigma_floor10 = (float)(10.0 * p.sigma0 * p.sigma_floor);
    ph.eps_smooth = (float)p.thickness_smoothing;
    ph.correct_sg = p.correct_disk_selfgravity != 0;
    ph.c_v_inv = (float)(p.mu / p.R_gas * (p.gamma - 1.0));
    ph.mu_over_R = (float)(p.mu / p.R_gas);
    ph.cool_const = (float)(8.0 * p.sigma_sb / p.c_light);
    ph.mu_gm1_over_R = (float)(p.mu * (p.gamma - 1.0) / p.R_gas);
    ph.emin_fac = (float)(p.minimum_temperature / p.mu * p.R_gas / (p.gamma - 1.0));
    {
        const double emax = p.maximum_temperature / p.mu * p.R_gas / (p.gamma - 1.0);
        ph.emax_fac = emax > 3.0e38 ? INFINITY : (float)emax;
    }
    ph.G_d = G;

    // fields
    const int nfield = FGPU_FIELD_COUNT;
    for (int f = 0; f < nfield; ++f) {
        const size_t n = is_vec(f) ? vcells : cells;
        CKF(cudaMalloc(&fld[f], n * sizeof(float)));
        CKF(cudaMemset(fld[f], 0, n * sizeof(float)));
    }
    vr_a = fld[FGPU_V_RADIAL];
    dv_a = fld[FGPU_V_AZIMUTHAL];
    CKF(cudaMalloc(&alt_sigma, cells * sizeof(float)));
    CKF(cudaMalloc(&alt_vr, vcells * sizeof(float)));
    CKF(cudaMalloc(&alt_dv, cells * sizeof(float)));
    CKF(cudaMalloc(&alt_e, cells * sizeof(float)));
    CKF(cudaMemset(alt_e, 0, cells * sizeof(float)));
    CKF(cudaMalloc(&sigma_lo, cells * sizeof(float)));
    CKF(cudaMemset(sigma_lo, 0, cells * sizeof(float)));
    CKF(cudaMalloc(&alt_sigma_lo, cells * sizeof(float)));
    CKF(cudaMemset(alt_sigma_lo, 0, cells * sizeof(float)));
    CKF(cudaMalloc(&ring_shift, sizeof(int) * (size_t)nr));
    CKF(cudaMemset(ring_shift, 0, sizeof(int) * (size_t)nr));
    for (int k = 0; k < 4; ++k) CKF(cudaMalloc(&mom[k], cells * sizeof(float)));
    CKF(cudaMalloc(&partial, sizeof(double) * 5 * kForceBodies32 * (size_t)nr));
    CKF(cudaMalloc(&red_out, sizeof(double) * (8 + 5 * kMaxBodies)));
    CKF(cudaMalloc(&d_dtmin, sizeof(unsigned int)));
    CKF(cudaMalloc(&d_bad, sizeof(unsigned long long)));
    CKF(cudaMallocHost(&h_pinned, sizeof(double) * (16 + 5 * kMaxBodies)));
    CKF(cudaMalloc(&stage, sizeof(double) * vcells));
    if (p.stabilize_viscosity) {
        // zero until the first stress evaluation, like the reference's grids
        CKF(cudaMalloc(&corr_phi, cells * sizeof(float)));
        CKF(cudaMalloc(&corr_r, cells * sizeof(float)));
        CKF(cudaMemset(corr_phi, 0, cells * sizeof(float)));
        CKF(cudaMemset(corr_r, 0, cells * sizeof(float)));
    }

    // boundary hooks on the residual v_phi
    bc.sigma_in = p.bc_sigma_inner; bc.sigma_out = p.bc_sigma_outer;
    bc.energy_in = p.bc_energy_inner; bc.energy_out = p.bc_energy_outer;
    bc.vr_in = p.bc_vrad_inner; bc.vr_out = p.bc_vrad_outer;
    bc.vaz_in = p.bc_vaz_inner; bc.vaz_out = p.bc_vaz_outer;
    bc.kep_in = (float)(p.vaz_inner_keplerian_factor * std::sqrt(G * M / Rmed[0]) - Vref[0]);
    bc.kep_out = (float)(p.vaz_outer_keplerian_factor * std::sqrt(G * M / Rmed[nr - 1]) -
                         Vref[nr - 1]);
    zg_in_base = Vref[1] - Vref[0];
    zg_out_base = Vref[nr - 2] - Vref[nr - 1];
    bc.zg_in = (float)zg_in_base;
    bc.zg_out = (float)zg_out_base;
    CKF(cudaMalloc(&vaz_offset, sizeof(double) * nr));
    CKF(cudaMemcpy(vaz_offset, Vref.data(), sizeof(double) * nr, cudaMemcpyHostToDevice));
    bc.nu = fld[FGPU_VISCOSITY];
    visc_recompute = p.eos == FGPU_EOS_IDEAL &&
                     (p.viscous_accretion || p.bc_vrad_inner == FGPU_BC_VISCOUS);
    {
        // the remaining hooks' constants, in the residual form where v_phi is
        // concerned (the FP32 form runs without a rotating frame)
        double vin[4][2], vout[4][2];
        boundary_values(p, Rmed.data(), Rinf.data(), nr, vin, vout);
        const int kin[4] = {p.bc_sigma_inner, p.bc_energy_inner, p.bc_vrad_inner, p.bc_vaz_inner};
        const int kout[4] = {p.bc_sigma_outer, p.bc_energy_outer, p.bc_vrad_outer,
                             p.bc_vaz_outer};
        for (int f = 0; f < 4; ++f) {
            for (int side = 0; side < 2; ++side) {
                const double *v = side ? vout[f] : vin[f];
                float *o = side ? bc.val_out[f] : bc.val_in[f];
                const int kind = side ? kout[f] : kin[f];
                const int edge = side ? nr - 1 : 0, next = side ? nr - 2 : 1;
                o[0] = (float)v[0];
                o[1] = (float)v[1];
                if (f == 0 && kind == FGPU_BC_DISKMODEL) {
                    o[1] = (float)(v[0] - (double)o[0]);
                } else if (f == 3 && kind == FGPU_BC_ZEROSHEAR) {
                    const double ratio = v[0] / v[1];
                    o[0] = (float)ratio;
                    o[1] = (float)(ratio * Vref[next] - Vref[edge]);
                } else if (f == 3 && kind == FGPU_BC_BALANCED) {
                    o[0] = (float)(v[0] - Vref[edge]);
                }
            }
        }
    }

    // damping
    const int dq_field[4] = {FGPU_V_RADIAL, FGPU_V_AZIMUTHAL, FGPU_SIGMA, FGPU_ENERGY};
    std::vector<float> dfac((size_t)4 * (nr + 1)), dzero((size_t)2 * (nr + 1));
    for (int vec = 0; vec < 2; ++vec) {
        const std::vector<double> &rad = vec ? Rinf : Rmed;
        float *fi = dfac.data() + (size_t)(vec ? 2 : 0) * (nr + 1);
        float *fo = fi + (nr + 1);
        for (int n = 0; n <= nr; ++n) {
            fi[n] = (float)pw((rad[n] - p.rmin * p.damping_inner_limit) /
                                  (p.rmin - p.rmin * p.damping_inner_limit), 2);
            fo[n] = (float)pw((rad[n] - p.rmax * p.damping_outer_limit) /
                                  (p.rmax - p.rmax * p.damping_outer_limit), 2);
        }
    }
    for (int n = 0; n <= nr; ++n) dzero[n] = (float)(-Vref[n]);  // v_phi -> 0 (fixed frame)
    host_rmed.assign(Rmed.begin(), Rmed.begin() + nr + 1);
    host_vref.assign(Vref.begin(), Vref.begin() + nr + 1);
    CKF(cudaMalloc(&damp_mem, sizeof(float) * (dfac.size() + dzero.size() + 2)));
    CKF(cudaMemcpy(damp_mem, dfac.data(), sizeof(float) * dfac.size(), cudaMemcpyHostToDevice));
    float *zero_vphi = damp_mem + dfac.size();
    zero_vphi_tab = zero_vphi;
    CKF(cudaMemcpy(zero_vphi, dzero.data(), sizeof(float) * dzero.size(), cudaMemcpyHostToDevice));
    // a zero table for the other quantities and the sigma floor of "zero" damping
    std::vector<float> zf((size_t)(nr + 1), 0.f), sf((size_t)(nr + 1), (float)(p.sigma_floor * p.sigma0));
    CKF(cudaMalloc(&damp_aux, sizeof(float) * 2 * (nr + 1)));
    CKF(cudaMemcpy(damp_aux, zf.data(), sizeof(float) * (nr + 1), cudaMemcpyHostToDevice));
    CKF(cudaMemcpy(damp_aux + nr + 1, sf.data(), sizeof(float) * (nr + 1), cudaMemcpyHostToDevice));
    std::vector<char> on(nr + 1, 0);
    for (int q = 0; q < 4; ++q) {
        DampQF &d = dm.q[q];
        const DampQSpec &sp = damp_spec[q];
        const bool vec = is_vec(dq_field[q]);
        d.vector = vec;
        d.kind_in = sp.kind_in;
        d.kind_out = sp.kind_out;
        d.active_in = sp.active_in;
        d.active_out = sp.active_out;
        d.limit_in = sp.limit_in;
        d.limit_out = sp.limit_out;
        d.tau_in = (float)sp.tau_in;
        d.tau_out = (float)sp.tau_out;
        d.fac_in = damp_mem + (size_t)(vec ? 2 : 0) * (nr + 1);
        d.fac_out = d.fac_in + (nr + 1);
        const float *zero_tab = damp_aux;
        d.x0_zero_in = dq_field[q] == FGPU_SIGMA ? damp_aux + nr + 1
                       : dq_field[q] == FGPU_V_AZIMUTHAL ? zero_vphi : zero_tab;
        d.x0_zero_out = dq_field[q] == FGPU_V_AZIMUTHAL ? zero_vphi : zero_tab;
        const int size = vec ? nr + 1 : nr;
        if (d.kind_in && d.active_in) for (int n = 0; n <= d.limit_in; ++n) on[n] = 1;
        if (d.kind_out && d.active_out) for (int n = d.limit_out; n < size; ++n) on[n] = 1;
    }
    std::vector<int> rings;
    for (int n = 0; n <= nr; ++n) if (on[n]) rings.push_back(n);
    n_rings = (int)rings.size();
    host_damp_rings = rings;
    if (n_rings) {
        CKF(cudaMalloc(&damp_rings, sizeof(int) * rings.size()));
        CKF(cudaMemcpy(damp_rings, rings.data(), sizeof(int) * rings.size(), cudaMemcpyHostToDevice));
    }
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 1;
    }

    // azimuthal kernel configuration
    per = nz <= 2048 ? 4 : (nz <= 4096 ? 8 : (nz <= 6144 ? 12 : 16));
    az_block = std::max(128, std::min(512, ((nz + per - 1) / per + 31) / 32 * 32));
    // cells strided over the block; the transported quantities staged in
    // shared memory when they fit in its 227 KB
    const int nq = phys.adiabatic ? 5 : 4;
    az_stage = azimuthal_smem_floats(nz, nq, true) * sizeof(float) <= kMaxRingSmem;
    az_smem = azimuthal_smem_floats(nz, nq, az_stage) * sizeof(float);
    if (az_smem > kMaxRingSmem) {
        err = "ring too long for the FP32 azimuthal kernel";
        return FGPU_ERR_UNSUPPORTED;
    }
    const void *az_kernels[16] = {
        (const void *)f_transport_azimuthal<4, 4, false>,
        (const void *)f_transport_azimuthal<8, 4, false>,
        (const void *)f_transport_azimuthal<12, 4, false>,
        (const void *)f_transport_azimuthal<16, 4, false>,
        (const void *)f_transport_azimuthal<4, 4, true>,
        (const void *)f_transport_azimuthal<8, 4, true>,
        (const void *)f_transport_azimuthal<12, 4, true>,
        (const void *)f_transport_azimuthal<16, 4, true>,
        (const void *)f_transport_azimuthal<4, 5, false>,
        (const void *)f_transport_azimuthal<8, 5, false>,
        (const void *)f_transport_azimuthal<12, 5, false>,
        (const void *)f_transport_azimuthal<16, 5, false>,
        (const void *)f_transport_azimuthal<4, 5, true>,
        (const void *)f_transport_azimuthal<8, 5, true>,
        (const void *)f_transport_azimuthal<12, 5, true>,
        (const void *)f_transport_azimuthal<16, 5, true>};
    for (const void *fn : az_kernels) {
        if (raise_smem_limit(fn, az_smem) != cudaSuccess) {
            err = "cannot reserve shared memory for the FP32 azimuthal kernel";
            return FGPU_ERR_CUDA;
        }
    }
    // the register-blocked kernel where the ring splits into whole 128-bit
    // segments (rb_default_per), unless FARGO_GB300_AZIMUTHAL asks for
    // "strided" or "blocked<PER>" (an explicit request is honoured or
    // refused, never replaced)
    rb_per = 0;
    {
        const char *env = getenv("FARGO_GB300_AZIMUTHAL");
        const std::string want = env ? env : "";
        if (want.rfind("blocked", 0) == 0) {
            const int pc = atoi(want.c_str() + 7);
            if ((pc == 4 || pc == 8 || pc == 12 || pc == 16) &&
                rb_fits(nz, nq, pc, 1, kMaxRingSmem)) {
                rb_per = pc;
            } else {
                err = "FARGO_GB300_AZIMUTHAL=" + want + " does not fit this ring";
                return FGPU_ERR_UNSUPPORTED;
            }
        } else if (want != "strided") {
            rb_per = rb_default_per(nz, nq, kMaxRingSmem);
        }
    }
    if (rb_per) {
        rb_smem = rb_smem_floats(nz, nq, nz / rb_per) * sizeof(float);
        const void *rb_kernels[8] = {
            (const void *)f_transport_azimuthal_rb<4, 4>, (const void *)f_transport_azimuthal_rb<8, 4>,
            (const void *)f_transport_azimuthal_rb<12, 4>, (const void *)f_transport_azimuthal_rb<16, 4>,
            (const void *)f_transport_azimuthal_rb<4, 5>, (const void *)f_transport_azimuthal_rb<8, 5>,
            (const void *)f_transport_azimuthal_rb<12, 5>, (const void *)f_transport_azimuthal_rb<16, 5>};
        for (const void *fn : rb_kernels) {
            if (raise_smem_limit(fn, rb_smem) != cudaSuccess) {
                err = "cannot reserve shared memory for the FP32 azimuthal kernel";
                return FGPU_ERR_CUDA;
            }
        }
    }

    CKF(cudaDeviceSynchronize());
    return FGPU_OK;
}

void Engine32::destroy()
{
    for (int f = 0; f < FGPU_FIELD_COUNT; ++f) cudaFree(fld[f]);
    cudaFree(alt_sigma); cudaFree(alt_vr); cudaFree(alt_dv); cudaFree(alt_e);
    cudaFree(sigma_lo); cudaFree(alt_sigma_lo); cudaFree(ring_shift);
    for (int k = 0; k < 4; ++k) cudaFree(mom[k]);
    cudaFree(partial); cudaFree(red_out); cudaFree(d_dtmin); cudaFree(d_bad); cudaFree(stage);
    cudaFree(corr_phi); cudaFree(corr_r);
    cudaFree(tab_f); cudaFree(tab_d); cudaFree(tab_c); cudaFree(vaz_offset); cudaFree(damp_mem); cudaFree(damp_aux); cudaFree(damp_rings);
    if (h_pinned) cudaFreeHost(h_pinned);
}

StateF Engine32::state()
{
    StateF s;
    s.sigma = fld[FGPU_SIGMA]; s.vr = fld[FGPU_V_RADIAL]; s.dv = fld[FGPU_V_AZIMUTHAL];
    s.energy = fld[FGPU_ENERGY]; s.sigma0 = fld[FGPU_SIGMA0]; s.vr0 = fld[FGPU_V_RADIAL0];
    s.dv0 = fld[FGPU_V_AZIMUTHAL0]; s.energy0 = fld[FGPU_ENERGY0];
    s.sigma_lo = sigma_lo;
    return s;
}

DiskF Engine32::describe()
{
    DiskF d{};
    d.g = geo;
    d.t = tabs;
    d.ph = phys;
    d.bc = bc;
    d.dm = dm;
    d.s = state();
    d.vr_b = alt_vr;
    d.dv_b = alt_dv;
    d.sigma_t = alt_sigma;
    d.energy_t = alt_e;
    d.sigma_lo_t = alt_sigma_lo;
    d.ring_shift = ring_shift;
    for (int k = 0; k < 4; ++k) d.mom[k] = mom[k];
    d.pot = fld[FGPU_POTENTIAL];
    d.P = fld[FGPU_PRESSURE];
    d.cs = fld[FGPU_SOUNDSPEED];
    d.H = fld[FGPU_SCALE_HEIGHT];
    d.nu = fld[FGPU_VISCOSITY];
    d.T = fld[FGPU_TEMPERATURE];
    d.Qr = fld[FGPU_Q_R];
    d.Qp = fld[FGPU_Q_PHI];
    d.divv = fld[FGPU_DIV_V];
    d.trr = fld[FGPU_TAU_R_R];
    d.tpp = fld[FGPU_TAU_PHI_PHI];
    d.trp = fld[FGPU_TAU_R_PHI];
    d.qplus = fld[FGPU_QPLUS];
    d.qminus = fld[FGPU_QMINUS];
    d.dtmin = d_dtmin;
    d.damping = p.damping && n_rings;
    d.nq = phys.adiabatic ? 5 : 4;
    return d;
}

// rows of a field and the ring offset between stored and FargoCPT values
const double *Engine32::offset_of(int f) const
{
    if (f == FGPU_V_AZIMUTHAL || f == FGPU_V_AZIMUTHAL0) return vaz_offset;
    if (f == FGPU_POTENTIAL) return tabs.PhiK_d;
    return nullptr;
}

int Engine32::upload(int f, const double *host, int rows)
{
    if (int rc_ = sync_frame()) return rc_;
    const size_t n = (size_t)rows * nz;
    CKF(cudaMemcpyAsync(stage, host, n * sizeof(double), cudaMemcpyHostToDevice, stream));
    if (f == FGPU_SIGMA)
        f_split_f32<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(stage, fld[f], sigma_lo, n);
    else
        f_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(stage, fld[f], n, nz, offset_of(f));
    CKF(cudaGetLastError());
    CKF(cudaStreamSynchronize(stream));
    cfl_valid = false;
    return FGPU_OK;
}

// FargoCPT's FP64 values of field f into the device buffer dst, in stream order
int Engine32::to_fp64(int f, double *dst, int rows)
{
    if (int rc_ = sync_frame()) return rc_;
    const size_t n = (size_t)rows * nz;
    if (f == FGPU_SIGMA)
        f_join_f64<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(fld[f], sigma_lo, dst, n);
    else
        f_to_f64<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(fld[f], dst, n, nz, offset_of(f));
    CKF(cudaGetLastError());
    return FGPU_OK;
}

int Engine32::download(int f, double *host, int rows)
{
    if (int rc_ = sync_frame()) return rc_;
    const size_t n = (size_t)rows * nz;
    int rc = to_fp64(f, stage, rows);
    if (rc) return rc;
    CKF(cudaMemcpyAsync(host, stage, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CKF(cudaStreamSynchronize(stream));
    return FGPU_OK;
}

// v_phi += Rmed s on every ring (the frame velocities kept when OmegaFrame
// changes, or shifted by correct_v_azimuthal)
__global__ void f_shift_vaz(GeoF g, const double *__restrict__ rmed, double s_dv, double s_dv0,
                            float *__restrict__ dv, float *__restrict__ dv0)
{
    const int nz = g.nz;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    if (s_dv != 0.0) dv[CELL(i, j)] += (float)(rmed[i] * s_dv);
    if (s_dv0 != 0.0) dv0[CELL(i, j)] += (float)(rmed[i] * s_dv0);
}

int Engine32::sync_frame()
{
    if (pend_dv == 0.0 && pend_dv0 == 0.0) return FGPU_OK;
    f_shift_vaz<<<dim3((nz + 127) / 128, nr), 128, 0, stream>>>(
        geo, tabs.Rmed_d, pend_dv, pend_dv0, fld[FGPU_V_AZIMUTHAL], fld[FGPU_V_AZIMUTHAL0]);
    pend_dv = pend_dv0 = 0.0;
    CKF(cudaGetLastError());
    return FGPU_OK;
}

void Engine32::set_bodies(int n, const fgpu_body *b, double ix, double iy, double omega_frame)
{
    if (omega_frame != geo.omega_frame) {
        // FargoCPT keeps the frame velocities when OmegaFrame changes: the
        // residuals about the inertial Keplerian speed move by Rmed dOmega
        const double d = omega_frame - geo.omega_frame;
        pend_dv += d;
        pend_dv0 += d;
        geo.omega_frame = omega_frame;
        geo.omega_f = (float)omega_frame;
        bc.zg_in = (float)(zg_in_base - omega_frame * (host_rmed[1] - host_rmed[0]));
        bc.zg_out = (float)(zg_out_base - omega_frame * (host_rmed[nr - 2] - host_rmed[nr - 1]));
        std::vector<double> off(nr);
        std::vector<float> z(nr + 1);
        for (int k = 0; k < nr; ++k) off[k] = host_vref[k] - host_rmed[k] * omega_frame;
        for (int k = 0; k <= nr; ++k) z[k] = (float)(host_rmed[k] * omega_frame - host_vref[k]);
        // stream-ordered after the kernels already queued that read the old
        // tables; from pageable memory the call returns once the source is
        // staged, so the local vectors may go
        cudaMemcpyAsync(vaz_offset, off.data(), sizeof(double) * nr, cudaMemcpyHostToDevice,
                        stream);
        cudaMemcpyAsync(zero_vphi_tab, z.data(), sizeof(float) * (nr + 1),
                        cudaMemcpyHostToDevice, stream);
    }
    bodies.n = n;
    bodies.star_at_origin = n > 0 && b[0].x == 0.0 && b[0].y == 0.0 &&
                            b[0].mass == p.hydro_center_mass && b[0].r_sm == 0.0;
    for (int k = 0; k < n; ++k) {
        bodies.x[k] = b[k].x;
        bodies.y[k] = b[k].y;
        split_position(bodies, k);
        bodies.gm[k] = (float)(p.G * b[k].mass);
        bodies.rsm[k] = (float)b[k].r_sm;
        bodies.a[k] = b[k].a;
    }
    bodies.gm_ref = (float)(p.G * p.hydro_center_mass);
    bodies.ix = (float)ix;
    bodies.iy = (float)iy;
}

static dim3 grid2(int nz, int rows) { return dim3((nz + 127) / 128, rows); }

int Engine32::derived_cfl(int mode)
{
    if (int rc_ = sync_frame()) return rc_;
    StateF s = state();
    if (mode & 4) CKF(cudaMemsetAsync(d_dtmin, 0x7f, sizeof(unsigned int), stream));
    f_derived_cfl<<<nr, 256, 0, stream>>>(geo, tabs, phys, mode, s.sigma, s.energy, s.vr, s.dv,
                                          fld[FGPU_QPLUS], fld[FGPU_QMINUS], fld[FGPU_SOUNDSPEED],
                                          fld[FGPU_SCALE_HEIGHT], fld[FGPU_PRESSURE],
                                          fld[FGPU_TEMPERATURE], fld[FGPU_VISCOSITY], d_dtmin,
                                          corr_phi, corr_r);
    CKF(cudaGetLastError());
    if (mode & 4) cfl_valid = true;
    return FGPU_OK;
}

// StabilizeViscosity's correction factors from the current nu and sigma
void Engine32::visc_corr(const StateF &s)
{
    f_visc_corr<<<dim3((nz + 127) / 128, nr - 1), 128, 0, stream>>>(
        geo, tabs, s.sigma, fld[FGPU_VISCOSITY], corr_phi, corr_r);
}

int Engine32::init_euler(double t)
{
    if (int rc_ = sync_frame()) return rc_;
    int rc = derived_cfl(1 | 2);
    if (rc) return rc;
    if (phys.adiabatic) {
        StateF s = state();
        f_stress<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, s.sigma, s.vr, s.dv,
                                                    fld[FGPU_VISCOSITY], fld[FGPU_DIV_V],
                                                    fld[FGPU_TAU_R_R], fld[FGPU_TAU_PHI_PHI],
                                                    fld[FGPU_TAU_R_PHI]);
        if (phys.stabilize) visc_corr(s);
        f_viscous<<<grid2(nz, nr), 128, 0, stream>>>(
            geo, tabs, phys, 0.f, (float)beta_inv(t), 2, s.sigma, fld[FGPU_TAU_R_R],
            fld[FGPU_TAU_PHI_PHI], fld[FGPU_TAU_R_PHI], fld[FGPU_DIV_V], fld[FGPU_VISCOSITY],
            fld[FGPU_SCALE_HEIGHT], s.sigma0, s.energy0, s.vr, s.dv, s.energy, fld[FGPU_QPLUS],
            fld[FGPU_QMINUS], corr_phi, corr_r);
        CKF(cudaGetLastError());
    }
    cfl_valid = false;
    return FGPU_OK;
}

double Engine32::beta_inv(double t) const
{
    double b = 1 / p.cooling_beta_value;
    if (p.cooling_beta_ramp_up > 0.0) b *= 1 - std::exp(-std::pow(2 * t / p.cooling_beta_ramp_up, 2));
    return b;
}

int Engine32::cfl(double *dt_out)
{
    if (!cfl_valid) {
        int rc = derived_cfl(4);
        if (rc) return rc;
    }
    CKF(cudaMemcpyAsync(h_pinned, d_dtmin, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
    CKF(cudaStreamSynchronize(stream));
    float f;
    std::memcpy(&f, h_pinned, sizeof(float));
    *dt_out = (double)f;
    return FGPU_OK;
}

void Engine32::com_boundary(const ComCenter *c)
{
    if (!com_any) return;
    ComSpec cs = com;
    cs.c[0] = c[0];
    cs.c[1] = c[1];
    cs.omf = geo.omega_frame;
    StateF s = state();
    const ComFields32 f{s.sigma, s.sigma_lo, s.vr, s.dv, s.energy, tabs.Vref_d, tabs.Rmed_d,
                        geo.omega_frame};
    k_com_boundary<<<dim3((nz + 127) / 128, 2), 128, 0, stream>>>(cs, nz, nr, f);
}

void Engine32::com_damping(double dt, const ComCenter *c)
{
    if (!com_any || !p.damping) return;
    ComSpec cs = com;
    cs.c[0] = c[0];
    cs.c[1] = c[1];
    cs.omf = geo.omega_frame;
    StateF s = state();
    const ComFields32 f{s.sigma, s.sigma_lo, s.vr, s.dv, s.energy, tabs.Vref_d, tabs.Rmed_d,
                        geo.omega_frame};
    launch_com_damping_sides(cs, nz, dt, f, stream);
}

int Engine32::boundary(double dt, bool final)
{
    if (int rc_ = sync_frame()) return rc_;
    if (final && visc_recompute) {
        // c_s, H, nu of the transported state before the final hooks
        // (simulation.cpp:232-242, 432-441)
        int rc = derived_cfl(1);
        if (rc) return rc;
    }
    if (final && p.damping && n_rings)
        f_damping<<<dim3(n_rings, 4), 256, 0, stream>>>(geo, dm, (float)dt, damp_rings, state());
    if (final) com_damping(dt, com_now);
    f_ghost<<<(nz + 127) / 128, 128, 0, stream>>>(geo, bc, state());
    com_boundary(com_now);
    CKF(cudaGetLastError());
    if (final)
        if (int rc = keep_mass()) return rc;
    cfl_valid = false;
    return FGPU_OK;
}

// The gas kick: potential, source terms, artificial viscosity, viscosity,
// stress, viscous update and SubStep3 (simulation.cpp:170-203).  Leaves the
// updated velocities in the step's buffers.
int Engine32::kick(double dt, double t)
{
    if (int rc_ = sync_frame()) return rc_;
    const float fdt = (float)dt;
    const bool adi = phys.adiabatic;
    auto mark = [&](int k) {
        if (mark_fn) mark_fn(mark_ctx, k);
    };
    f_potential<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, phys, bodies, fld[FGPU_SCALE_HEIGHT],
                                                   fld[FGPU_POTENTIAL]);
    CKL("potential");
    mark(0);
    f_source<<<grid2(nz, nr + 1), 128, 0, stream>>>(geo, tabs, fdt, fld[FGPU_SIGMA],
                                                    fld[FGPU_PRESSURE], fld[FGPU_POTENTIAL],
                                                    fld[FGPU_V_RADIAL], fld[FGPU_V_AZIMUTHAL],
                                                    alt_vr, alt_dv);
    CKL("source");
    std::swap(fld[FGPU_V_RADIAL], alt_vr);
    std::swap(fld[FGPU_V_AZIMUTHAL], alt_dv);
    mark(1);
    StateF s = state();
    if (adi || phys.art_visc_sn || phys.art_visc_tw) {
        f_artvisc_q<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, phys, fdt, s.sigma, s.vr, s.dv,
                                                       s.energy, fld[FGPU_Q_R], fld[FGPU_Q_PHI]);
        CKL("artvisc_q");
        mark(2);
        f_artvisc_v<<<grid2(nz, nr), 128, 0, stream>>>(
            geo, tabs, phys, fdt, s.sigma, s.energy, fld[FGPU_Q_R], fld[FGPU_Q_PHI], s.vr, s.dv,
            fld[FGPU_SOUNDSPEED], fld[FGPU_SCALE_HEIGHT], fld[FGPU_VISCOSITY]);
        CKL("artvisc_v");
        mark(3);
    } else {
        mark(2);
        mark(3);
    }
    f_stress<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, s.sigma, s.vr, s.dv,
                                                fld[FGPU_VISCOSITY], fld[FGPU_DIV_V],
                                                fld[FGPU_TAU_R_R], fld[FGPU_TAU_PHI_PHI],
                                                fld[FGPU_TAU_R_PHI]);
    CKL("stress");
    if (phys.stabilize) visc_corr(s);
    mark(4);
    f_viscous<<<grid2(nz, nr), 128, 0, stream>>>(
        geo, tabs, phys, fdt, (float)beta_inv(t), adi ? 7 : 1, s.sigma, fld[FGPU_TAU_R_R],
        fld[FGPU_TAU_PHI_PHI], fld[FGPU_TAU_R_PHI], fld[FGPU_DIV_V], fld[FGPU_VISCOSITY],
        fld[FGPU_SCALE_HEIGHT], s.sigma0, s.energy0, s.vr, s.dv, s.energy, fld[FGPU_QPLUS],
        fld[FGPU_QMINUS], corr_phi, corr_r);
    CKL("viscous");
    mark(5);
    cfl_valid = false;
    return FGPU_OK;
}

// Transport (TransportEuler.cpp): radial sweep, FARGO azimuthal transport,
// velocities from momenta and floors.
int Engine32::transport(double dt)
{
    if (int rc_ = sync_frame()) return rc_;
    const float fdt = (float)dt;
    const bool adi = phys.adiabatic;
    auto mark = [&](int k) {
        if (mark_fn) mark_fn(mark_ctx, k);
    };
    StateF s = state();
    {
        // rings per thread: the longest walk that still gives every SM
        // sixteen blocks of columns (each thread's rings are a dependent
        // chain of loads, so short grids need short walks to hide latency)
        const int cols = (nz + 63) / 64;
        int chunk = 16;
        while (chunk > 4 && (long long)cols * ((nr + chunk - 1) / chunk) < 16LL * nsm) chunk /= 2;
        dim3 grid(cols, (nr + chunk - 1) / chunk);
        if (adi)
            f_transport_radial<5><<<grid, 64, 0, stream>>>(geo, tabs, fdt, phys.limiter_mc, chunk,
                                                           s.sigma, s.vr, s.dv, s.energy, mom[0],
                                                           mom[1], mom[2], mom[3], alt_e, alt_sigma,
                                                           sigma_lo, alt_sigma_lo);
        else
            f_transport_radial<4><<<grid, 64, 0, stream>>>(geo, tabs, fdt, phys.limiter_mc, chunk,
                                                           s.sigma, s.vr, s.dv, s.energy, mom[0],
                                                           mom[1], mom[2], mom[3], alt_e, alt_sigma,
                                                           sigma_lo, alt_sigma_lo);
    }
    CKL("transport_radial");
    mark(7);
    {
#define AZ32(P, NQ, ST)                                                                          \
    f_transport_azimuthal<P, NQ, ST><<<nr, az_block, az_smem, stream>>>(                         \
        geo, tabs, dt, phys.limiter_mc, phys.fast_transport, s.dv, mom[0], mom[1], mom[2],      \
        mom[3], alt_e, alt_sigma, alt_sigma_lo, ring_shift)
#define AZ32_NQ(NQ)                                      \
    if (az_stage) {                                      \
        if (per == 4) AZ32(4, NQ, true);                 \
        else if (per == 8) AZ32(8, NQ, true);            \
        else if (per == 12) AZ32(12, NQ, true);          \
        else AZ32(16, NQ, true);                         \
    } else {                                             \
        if (per == 4) AZ32(4, NQ, false);                \
        else if (per == 8) AZ32(8, NQ, false);           \
        else if (per == 12) AZ32(12, NQ, false);         \
        else AZ32(16, NQ, false);                        \
    }
#define AZRB(P, NQ)                                                                              \
    f_transport_azimuthal_rb<P, NQ><<<nr, nz / P, rb_smem, stream>>>(                            \
        geo, tabs, dt, phys.limiter_mc, phys.fast_transport, s.dv, mom[0], mom[1], mom[2],      \
        mom[3], alt_e, alt_sigma, alt_sigma_lo, ring_shift)
#define AZRB_NQ(NQ)                         \
    if (rb_per == 4) AZRB(4, NQ);           \
    else if (rb_per == 8) AZRB(8, NQ);      \
    else if (rb_per == 12) AZRB(12, NQ);    \
    else AZRB(16, NQ);
        if (rb_per) {
            if (adi) {
                AZRB_NQ(5)
            } else {
                AZRB_NQ(4)
            }
        } else if (adi) {
            AZ32_NQ(5)
        } else {
            AZ32_NQ(4)
        }
#undef AZRB_NQ
#undef AZRB
#undef AZ32_NQ
#undef AZ32
    }
    CKL("transport_azimuthal");
    mark(8);
    f_finish<<<grid2(nz, nr + 1), 128, 0, stream>>>(geo, tabs, phys, mom[0], mom[1], mom[2],
                                                    mom[3], alt_sigma, alt_e, s.vr, alt_vr,
                                                    alt_dv, s.sigma, s.energy, alt_sigma_lo,
                                                    sigma_lo, ring_shift);
    CKL("finish");
    std::swap(fld[FGPU_V_RADIAL], alt_vr);
    std::swap(fld[FGPU_V_AZIMUTHAL], alt_dv);
    mark(9);
    cfl_valid = false;
    return FGPU_OK;
}

int Engine32::pressure()
{
    f_pressure<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, phys, fld[FGPU_SIGMA],
                                                  fld[FGPU_ENERGY], fld[FGPU_PRESSURE]);
    CKF(cudaGetLastError());
    return FGPU_OK;
}

int Engine32::step(double dt, double t)
{
    auto mark = [&](int k) {
        if (mark_fn) mark_fn(mark_ctx, k);
    };
    mark(-1);
    int rc = kick(dt, t);
    if (rc) return rc;
    f_ghost<<<(nz + 127) / 128, 128, 0, stream>>>(geo, bc, state());
    CKL("ghost");
    com_boundary(com_now);
    CKL("com_boundary");
    mark(6);
    rc = transport(dt);
    if (rc) return rc;
    if (visc_recompute) {
        rc = derived_cfl(1);
        if (rc) return rc;
    }
    StateF s = state();
    if (p.damping && n_rings)
        f_damping<<<dim3(n_rings, 4), 256, 0, stream>>>(geo, dm, (float)dt, damp_rings, s);
    CKL("damping");
    com_damping(dt, com_after);
    CKL("com_damping");
    mark(10);
    f_ghost<<<(nz + 127) / 128, 128, 0, stream>>>(geo, bc, s);
    CKL("ghost");
    com_boundary(com_after);
    CKL("com_boundary");
    rc = keep_mass();
    if (rc) return rc;
    mark(11);
    rc = derived_cfl(1 | 4);
    if (rc) return rc;
    mark(12);
    CKF(cudaGetLastError());
    return FGPU_OK;
}

// the disk force on n <= kMaxBodies bodies, kForceBodies32 per pass over the
// disk, one read-back; out (host, 5 doubles per body) receives the sums
int Engine32::disk_forces(int n, const double *x, const double *y, const double *a,
                          const double *rsm, double *out)
{
    if (n < 0 || n > kMaxBodies) return FGPU_ERR_BAD_ARG;
    const int rows = nr - 2;
    double *dev = red_out + 8;
    for (int b0 = 0; b0 < n; b0 += kForceBodies32) {
        ForceBodies32 fb{};
        fb.n = std::min(kForceBodies32, n - b0);
        for (int b = 0; b < fb.n; ++b) {
            fb.x[b] = x[b0 + b];
            fb.y[b] = y[b0 + b];
            fb.a[b] = a[b0 + b];
            fb.rsm[b] = rsm[b0 + b];
        }
        const int width = 5 * fb.n;
        f_disk_force_bodies<<<rows, 256, 0, stream>>>(geo, tabs, phys, fb, fld[FGPU_SIGMA],
                                                      sigma_lo, fld[FGPU_SCALE_HEIGHT], partial,
                                                      width);
        f_reduce_cols<<<width, 32, 0, stream>>>(partial, rows, width, dev + 5 * b0);
    }
    CKF(cudaGetLastError());
    CKF(cudaMemcpyAsync(h_pinned + 16, dev, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost,
                        stream));
    CKF(cudaStreamSynchronize(stream));
    std::copy(h_pinned + 16, h_pinned + 16 + 5 * n, out);
    return FGPU_OK;
}

int Engine32::gas_quantities(double radius, double out[2])
{
    if (int rc_ = sync_frame()) return rc_;
    const int rows = nr - 2;
    f_gas_quantities<<<rows, 256, 0, stream>>>(geo, tabs, radius, fld[FGPU_SIGMA], sigma_lo,
                                               fld[FGPU_V_AZIMUTHAL], partial);
    f_reduce_rows2<<<1, 64, 0, stream>>>(partial, rows, red_out + 5);
    CKF(cudaGetLastError());
    CKF(cudaMemcpyAsync(h_pinned, red_out + 5, sizeof(double) * 2, cudaMemcpyDeviceToHost,
                        stream));
    CKF(cudaStreamSynchronize(stream));
    out[0] = h_pinned[0];
    out[1] = h_pinned[1];
    return FGPU_OK;
}

// KeepDiskMassConstant after a final boundary call (simulation.cpp:246-251,
// 445-450): the mass at RMAX on the device, then the rescale.
int Engine32::keep_mass()
{
    if (!p.keep_disk_mass_constant) return FGPU_OK;
    const int rows = nr - 2;
    f_gas_quantities<<<rows, 256, 0, stream>>>(geo, tabs, p.rmax, fld[FGPU_SIGMA], sigma_lo,
                                               fld[FGPU_V_AZIMUTHAL], partial);
    f_reduce_rows2<<<1, 64, 0, stream>>>(partial, rows, red_out + 5);
    const size_t n = cells;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    f_scale_sigma<<<blocks, 256, 0, stream>>>(fld[FGPU_SIGMA], sigma_lo, n, mass_target,
                                              red_out + 5);
    CKL("keep_mass");
    return FGPU_OK;
}

int Engine32::disk_force(double px, double py, double pa, double rsm, double out[5])
{
    return disk_forces(1, &px, &py, &pa, &rsm, out);
}

// Accretion onto one planet (accretion.cpp:84-480) on the FP32 state: the
// compensated sigma pair and the cell geometry in FP64, the removed mass and
// momentum summed in FP64 (one block; cells are independent).
__global__ void f_accrete(GeoF g, TablesF t, PhysF ph, AccrF a, float *__restrict__ S,
                          float *__restrict__ S_lo, float *__restrict__ E,
                          const float *__restrict__ vr, const float *__restrict__ dv,
                          const float *__restrict__ nu, double *__restrict__ out)
{
    __shared__ double red[33];
    const int nz = g.nz, nr = g.nr;
    const long long cells = (long long)(a.i1 - a.i0 + 1) * a.ncols;
    double dM = 0.0, dPx = 0.0, dPy = 0.0;
    for (long long k = threadIdx.x; k < cells; k += blockDim.x) {
        const int i = a.i0 + (int)(k / a.ncols);
        int jf = (a.j0 + (int)(k % a.ncols)) % nz;
        if (jf < 0) jf += nz;
        const size_t l = CELL(i, jf);
        const double rm = t.Rmed_d[i];
        const double xc = rm * t.cos_d[jf], yc = rm * t.sin_d[jf];
        const double dx = a.x - xc, dy = a.y - yc;
        const double distance = sqrt(dx * dx + dy * dy);
        // the stored residual is about the inertial Keplerian speed, so this
        // is the inertial v_phi the reference forms as v_phi + Rmed OmegaFrame
        const double vtcell = t.Vref_d[i] + 0.5 * ((double)dv[l] + (double)dv[CELL(i, jnext(jf, nz))]);
        const double vrcell = 0.5 * ((double)vr[l] + (double)vr[l + nz]);
        const double vxcell = (vrcell * xc - vtcell * yc) / rm;
        const double vycell = (vrcell * yc + vtcell * xc) / rm;
        double sig = (double)S[l] + (double)S_lo[l];
        const double sig0 = sig;
        double e = ph.adiabatic ? (double)E[l] : 0.0;
        const double facc_max = 1 - a.density_floor / sig0;
        const bool active = 1 < i && i < nr - 1;
        bool changed = false;
        if (distance < a.frac1 * a.rhill) {
            double f = a.facc1;
            if (a.type == 1 /* viscous */)
                f = a.facc1 * (double)nu[l] * (a.f_const * (1.0 - distance / a.dist_max));
            const double fc = facc_max < f ? facc_max : f;
            const double deltaM = fc * sig * t.Surf_d[i];
            sig *= 1.0 - fc;
            e *= 1.0 - fc;
            changed = true;
            if (active) {
                dPx += deltaM * vxcell;
                dPy += deltaM * vycell;
                dM += deltaM;
            }
        }
        if (a.type == 0 /* Kley */ && distance < a.frac2 * a.rhill) {
            const double fc = facc_max < a.facc2 ? facc_max : a.facc2;
            const double deltaM = fc * sig * t.Surf_d[i];
            sig *= 1.0 - fc;
            // the reference scales the energy by the uncapped factor here
            e *= 1.0 - a.facc2;
            changed = true;
            if (active) {
                dPx += deltaM * vxcell;
                dPy += deltaM * vycell;
                dM += deltaM;
            }
        }
        if (changed) {
            const float hi = (float)sig;
            S[l] = hi;
            S_lo[l] = (float)(sig - (double)hi);
            if (ph.adiabatic) E[l] = (float)e;
        }
    }
    dM = bsum_d(dM, red);
    dPx = bsum_d(dPx, red);
    dPy = bsum_d(dPy, red);
    if (threadIdx.x == 0) {
        out[0] = dM;
        out[1] = dPx;
        out[2] = dPy;
    }
}

int Engine32::accrete(const AccrF &a, double out[3])
{
    if (int rc_ = sync_frame()) return rc_;
    StateF s = state();
    f_accrete<<<1, 512, 0, stream>>>(geo, tabs, phys, a, s.sigma, s.sigma_lo, s.energy, s.vr,
                                     s.dv, fld[FGPU_VISCOSITY], red_out);
    CKF(cudaGetLastError());
    CKF(cudaMemcpyAsync(h_pinned, red_out, sizeof(double) * 3, cudaMemcpyDeviceToHost, stream));
    CKF(cudaStreamSynchronize(stream));
    for (int k = 0; k < 3; ++k) out[k] = h_pinned[k];
    cfl_valid = false;
    return FGPU_OK;
}

int Engine32::check_finite(int *field, int *nr_out, int *naz_out)
{
    const int fields[4] = {FGPU_SIGMA, FGPU_V_RADIAL, FGPU_V_AZIMUTHAL, FGPU_ENERGY};
    for (int k = 0; k < 4; ++k) {
        const size_t n = is_vec(fields[k]) ? vcells : cells;
        CKF(cudaMemsetAsync(d_bad, 0xff, sizeof(unsigned long long), stream));
        f_check_finite<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(fld[fields[k]], n, d_bad);
        CKF(cudaMemcpyAsync(h_pinned, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            stream));
        CKF(cudaStreamSynchronize(stream));
        unsigned long long bad;
        std::memcpy(&bad, h_pinned, sizeof(bad));
        if (bad != ~0ull) {
            if (field) *field = fields[k];
            if (nr_out) *nr_out = (int)(bad / nz);
            if (naz_out) *naz_out = (int)(bad % nz);
            return FGPU_ERR_NONFINITE;
        }
    }
    return FGPU_OK;
}

}  // namespace fgpu32
