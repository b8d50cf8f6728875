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
// and FargoCPT's step_Euler (simulation.cpp:148-267).
#include "../../include/fargocpt_gb300.h"
#include "fp32_engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace fgpu32 {

#define CELL(i, j) ((size_t)(i) * (size_t)nz + (size_t)(j))

__device__ __forceinline__ int jnext(int j, int nz) { return j == nz - 1 ? 0 : j + 1; }
__device__ __forceinline__ int jprev(int j, int nz) { return j == 0 ? nz - 1 : j - 1; }

__device__ __forceinline__ float lim_f(float a, float b, int mc)
{
    if (mc) {
        float mm = 0.f;
        if (a * b > 0.f) mm = fabsf(a) < fabsf(b) ? a : b;
        const float c = 0.5f * (a + b), d = 2.f * mm;
        if (c * d > 0.f) return fabsf(c) < fabsf(d) ? c : d;
        return 0.f;
    }
    if (a * b > 0.f) return __fdividef(2.f * a * b, a + b);
    return 0.f;
}

// hi + lo + inc as a compensated pair: y = lo + inc is small next to hi, so
// Fast2Sum (Dekker 1971) recovers the rounding error of hi + y exactly.
__device__ __forceinline__ void comp_add(float &hi, float &lo, float inc)
{
    const float y = lo + inc;
    const float s = hi + y;
    lo = y - (s - hi);
    hi = s;
}

__device__ __forceinline__ float tfloor(float e, float sigma, const PhysF &ph)
{
    const float emin = sigma * ph.emin_fac;
    const float emax = sigma * ph.emax_fac;
    if (!(e > emin)) e = emin;
    if (!(e < emax)) e = emax;
    return e;
}

__device__ float warp_sum_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ float warp_min_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
template <typename T, T (*WARP)(T)>
__device__ T block_reduce(T v, T *red, T neutral)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = WARP(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        T x = lane < nw ? red[lane] : neutral;
        x = WARP(x);
        if (lane == 0) red[32] = x;
    }
    __syncthreads();
    return red[32];
}
__device__ double bsum_d(double v, double *red) { return block_reduce<double, warp_sum_d>(v, red, 0.0); }
__device__ float bsum_f(float v, float *red) { return block_reduce<float, warp_sum_f>(v, red, 0.f); }
__device__ float bmin_f(float v, float *red) { return block_reduce<float, warp_min_f>(v, red, 3.0e38f); }

// ---------------------------------------------------------------------------
// Potential residual Phi - Phi_K (CalculateNbodyPotential, Pframeforce.cpp:21-86)
// ---------------------------------------------------------------------------
__global__ void f_potential(GeoF g, TablesF t, PhysF ph, BodiesF b, const float *__restrict__ H,
                            float *__restrict__ pot)
{
    const int nz = g.nz;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const double xd = t.Rmed_d[i] * t.cos_d[j];
    const double yd = t.Rmed_d[i] * t.sin_d[j];
    const float eps = ph.eps_smooth * H[CELL(i, j)];
    const float s2 = eps * eps;
    float acc = 0.f;
    for (int k = 0; k < b.n; ++k) {
        float term;
        if (k == 0 && b.star_at_origin) {
            // -G M / sqrt(r^2 + eps^2) + G M / r without cancellation:
            // 1/r - 1/d = (d - r) / (r d) = eps^2 / ((d + r) r d)
            const float r = t.Rmed[i];
            const float d = sqrtf(r * r + s2);
            term = b.gm[0] * s2 / ((d + r) * r * d);
        } else {
            const double dx = xd - b.x[k], dy = yd - b.y[k];
            const float d2 = (float)(dx * dx + dy * dy) + s2;
            const float inv_d = rsqrtf(d2);
            float fk = 1.f;
            if (b.rsm[k] > 0.f) {
                const float dsm = d2 * inv_d;
                if (dsm < b.rsm[k]) {
                    const float q = dsm / b.rsm[k];
                    fk = q * q * q * q - 2.f * q * q * q + 2.f * q;
                }
            }
            if (k == 0) {
                // central object off the origin: residual against -G M / r in FP64
                term = (float)(-(double)b.gm[0] * fk / sqrt(dx * dx + dy * dy + (double)s2) +
                               (double)b.gm_ref * t.InvRmed_d[i]);
            } else {
                term = -b.gm[k] * inv_d * fk;
            }
        }
        acc += term;
    }
    acc += -b.ix * (float)xd - b.iy * (float)yd;
    pot[CELL(i, j)] = acc;
}

// ---------------------------------------------------------------------------
// momentum sources (SourceEuler.cpp:325-428) in residual form
// ---------------------------------------------------------------------------
__global__ void f_source(GeoF g, TablesF t, float dt, const float *__restrict__ S,
                         const float *__restrict__ P, const float *__restrict__ pot,
                         const float *__restrict__ vr_in, const float *__restrict__ dv_in,
                         float *__restrict__ vr_out, float *__restrict__ dv_out)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    float vr = vr_in[CELL(i, j)];
    if (i >= 2 && i < nr - 1) {
        const float gradp = 2.f * __fdividef(P[CELL(i, j)] - P[CELL(i - 1, j)],
                                             S[CELL(i, j)] + S[CELL(i - 1, j)]) *
                            t.InvDiffRmed[i];
        const float gradphi = (pot[CELL(i, j)] - pot[CELL(i - 1, j)]) * t.InvDiffRmed[i];
        const int jn = jnext(j, nz);
        const float d = 0.25f * (dv_in[CELL(i, j)] + dv_in[CELL(i, jn)] + dv_in[CELL(i - 1, j)] +
                                 dv_in[CELL(i - 1, jn)]);
        // vt^2 / r - dPhi_K/dr = Kbal + (2 A d + d^2) / Rinf
        const float centri = t.Kbal[i] + (2.f * t.Aface[i] + d) * d * t.InvRinf[i];
        vr += dt * (-gradp - gradphi + centri);
    }
    vr_out[CELL(i, j)] = vr;
    if (i < nr) {
        float v = dv_in[CELL(i, j)];
        if (i >= 1 && i < nr - 1) {
            const int jp = jprev(j, nz);
            const float invdx = t.InvDxSrc[i];
            const float gradp = 2.f * __fdividef(P[CELL(i, j)] - P[CELL(i, jp)],
                                                 S[CELL(i, j)] + S[CELL(i, jp)]) * invdx;
            const float gradphi = (pot[CELL(i, j)] - pot[CELL(i, jp)]) * invdx;
            v = v + dt * (-gradp - gradphi);
        }
        dv_out[CELL(i, j)] = v;
    }
}

// compression heating + SN q and energy update + T floor
__global__ void f_artvisc_q(GeoF g, TablesF t, PhysF ph, float dt, const float *__restrict__ S,
                            const float *__restrict__ vr, const float *__restrict__ dv,
                            float *__restrict__ E, float *__restrict__ Qr, float *__restrict__ Qp)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jn = jnext(j, nz);
    const float vr0 = vr[c], vr1 = vr[CELL(i + 1, j)];
    const float dvp = dv[CELL(i, jn)] - dv[c];
    float e = 0.f;
    if (ph.adiabatic) {
        e = E[c];
        if (i < nr - 1) {
            const float div_v = (vr1 * t.Rinf[i + 1] - vr0 * t.Rinf[i]) * t.InvDiffRsupRb[i] +
                                dvp * g.invdphi * t.InvRmed[i];
            e = e * __expf(-ph.gm1 * dt * div_v);
        }
    }
    if (ph.art_visc_sn) {
        const float sig = S[c];
        const float dv_r = vr1 - vr0;
        const float qr = dv_r < 0.f ? ph.C2 * sig * (dv_r * dv_r) : 0.f;
        const float qp = dvp < 0.f ? ph.C2 * sig * (dvp * dvp) : 0.f;
        Qr[c] = qr;
        Qp[c] = qp;
        if (ph.adiabatic && ph.dissipation && i >= 1 && i < nr - 1) {
            e = e - dt * qr * dv_r * t.InvDiffRsup[i] - dt * qp * dvp * t.InvDxTheta[i];
        }
    }
    if (ph.adiabatic) {
        if (ph.dissipation) e = tfloor(e, S[c], ph);
        E[c] = e;
    }
}

__global__ void f_artvisc_v(GeoF g, TablesF t, PhysF ph, float dt, const float *__restrict__ S,
                            const float *__restrict__ E, const float *__restrict__ Qr,
                            const float *__restrict__ Qp, float *__restrict__ vr,
                            float *__restrict__ dv, float *__restrict__ cs, float *__restrict__ H,
                            float *__restrict__ nu)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    if (ph.art_visc_sn) {
        if (i >= 2 && i < nr - 1) {
            vr[c] -= dt * 2.f * __fdividef(Qr[c] - Qr[CELL(i - 1, j)], S[c] + S[CELL(i - 1, j)]) *
                     t.InvDiffRmed[i];
        }
        if (i >= 1 && i < nr - 1) {
            const int jp = jprev(j, nz);
            dv[c] -= dt * 2.f * __fdividef(Qp[c] - Qp[CELL(i, jp)], S[c] + S[CELL(i, jp)]) *
                     t.InvDxTheta[i];
        }
    }
    if (ph.adiabatic) {
        const float c_s = sqrtf(ph.g_gm1 * __fdividef(E[c], S[c]));
        const float h = c_s * t.HFacAdi[i];
        cs[c] = c_s;
        H[c] = h;
        nu[c] = ph.alpha > 0.f ? ph.alpha * h * c_s : ph.constant_viscosity;
    }
}

// stress tensor (viscosity.cpp:139-254); tau_r_phi adds the Keplerian shear
__global__ void f_stress(GeoF g, TablesF t, const float *__restrict__ S, const float *__restrict__ vr,
                         const float *__restrict__ dv, const float *__restrict__ nu,
                         float *__restrict__ divv, float *__restrict__ trr, float *__restrict__ tpp,
                         float *__restrict__ trp)
{
    const int nz = g.nz;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jn = jnext(j, nz);
    const float vr0 = vr[c], vr1 = vr[CELL(i + 1, j)];
    const float dvp = dv[CELL(i, jn)] - dv[c];
    const float n = nu[c], sg = S[c];
    const float d = (vr1 * t.Rinf[i + 1] - vr0 * t.Rinf[i]) * t.InvDiffRsupRb[i] +
                    dvp * g.invdphi * t.InvRmed[i];
    divv[c] = d;
    const float drr = (vr1 - vr0) * t.InvDiffRsup[i];
    trr[c] = 2.f * n * sg * (drr - (1.f / 3.f) * d);
    const float dpp = dvp * g.invdphi * t.InvRmed[i] + 0.5f * (vr1 + vr0) * t.InvRmed[i];
    tpp[c] = 2.f * n * sg * (dpp - (1.f / 3.f) * d);
    if (i >= 1) {
        const int jp = jprev(j, nz);
        const float dvazirdr =
            t.Shear[i] + (dv[c] * t.InvRmed[i] - dv[CELL(i - 1, j)] * t.InvRmed[i - 1]) *
                             t.InvDiffRmed[i];
        const float dvrdphi = (vr0 - vr[CELL(i, jp)]) * g.invdphi;
        const float drp = t.Rinf[i] * dvazirdr + dvrdphi * t.InvRinf[i];
        const float n4 = 0.25f * (n + nu[CELL(i - 1, j)] + nu[CELL(i, jp)] + nu[CELL(i - 1, jp)]);
        const float s4 = 0.25f * (sg + S[CELL(i - 1, j)] + S[CELL(i, jp)] + S[CELL(i - 1, jp)]);
        trp[c] = n4 * s4 * drp;
    }
}

// viscous velocity update + SubStep3 (mode bits as in the FP64 form)
__global__ void f_viscous(GeoF g, TablesF t, PhysF ph, float dt, float beta_inv, int mode,
                          const float *__restrict__ S, const float *__restrict__ trr,
                          const float *__restrict__ tpp, const float *__restrict__ trp,
                          const float *__restrict__ divv, const float *__restrict__ nu,
                          const float *__restrict__ H, const float *__restrict__ S0,
                          const float *__restrict__ E0, float *__restrict__ vr,
                          float *__restrict__ dv, float *__restrict__ E, float *__restrict__ qplus,
                          float *__restrict__ qminus)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jp = jprev(j, nz), jn = jnext(j, nz);
    if (mode & 1) {
        if (i >= 1 && i < nr - 1) {
            const float sa = 0.5f * (S[c] + S[CELL(i, jp)]);
            dv[c] += __fdividef(dt * t.InvRmed[i], sa) *
                     (t.TwoOverDRa2[i] * (t.RinfSq[i + 1] * trp[CELL(i + 1, j)] -
                                          t.RinfSq[i] * trp[c]) +
                      (tpp[c] - tpp[CELL(i, jp)]) * g.invdphi);
        }
        if (i >= 2 && i < nr - 1) {
            const float sa = 0.5f * (S[c] + S[CELL(i - 1, j)]);
            vr[c] += __fdividef(dt, sa) * ph.rvf * t.TwoOverRmedSum[i] *
                     ((t.Rmed[i] * trr[c] - t.Rmed[i - 1] * trr[CELL(i - 1, j)]) * t.InvDiffRmed[i] +
                      (trp[CELL(i, jn)] - trp[c]) * g.invdphi - 0.5f * (tpp[c] + tpp[CELL(i - 1, j)]));
        }
    }
    if (!(mode & 6) || !ph.adiabatic) return;
    float qp = 0.f, qm = 0.f;
    const float e = E[c], sig = S[c];
    const bool active = i >= 1 && i < nr - 1;
    if (active) {
        if (ph.cooling_beta) {
            float dE = e;
            if (ph.beta_ref == 1) dE -= __fdividef(E0[c], S0[c]) * sig;
            else if (ph.beta_ref == 2) dE -= t.EModel[i] * sig;
            else if (ph.beta_ref == 3) dE -= sig * ph.emin_fac;
            qm = dE * t.OmegaK[i] * beta_inv;
        }
        if (ph.heating_viscous) {
            const float n = nu[c];
            if (n != 0.f) {
                const float trpa = 0.25f * (trp[c] + trp[CELL(i + 1, j)] + trp[CELL(i, jn)] +
                                            trp[CELL(i + 1, jn)]);
                const float a = trr[c], b2 = tpp[c], dd = divv[c];
                float q = __fdividef(a * a + 2.f * trpa * trpa + b2 * b2, 2.f * n * sig);
                q += (2.f / 9.f) * n * sig * dd * dd;
                qp = q * ph.hvf;
            }
        }
        // radiative alpha: 1 + 8 sigma_SB / c * H * x^4 e^3 with
        // x = mu (gamma-1) / (R sigma), evaluated as x * (x e)^3
        const float x = __fdividef(ph.mu_gm1_over_R, sig);
        const float xe = x * e;
        const float alpha = 1.f + H[c] * ph.cool_const * x * (xe * xe * xe);
        const float ia = __frcp_rn(alpha);
        qp *= ia;
        qm *= ia;
    }
    if (mode & 4) {
        float en = e;
        if (active) {
            en = e + dt * (qp - qm);
            if (sig < ph.sigma_floor10) {
                qm = qp;
                en = 0.f;
            }
        }
        E[c] = tfloor(en, sig, ph);
    }
    qplus[c] = qp;
    qminus[c] = qm;
}

// ghost rings (boundary_conditions.cpp:65-114); v_phi hooks work on the
// residual, with the reference-profile offsets per ring
__device__ void ghost_f(float *x, const float *x0, int kind, int outer, int vec, int nr, int nz, int j,
                        float kep_value, float zg_offset)
{
    const int irad = vec ? nr : nr - 1;
    switch (kind) {
    case 1:
        if (!outer) {
            if (vec) {
                x[CELL(0, j)] = x[CELL(2, j)];
                x[CELL(1, j)] = x[CELL(2, j)];
            } else {
                x[CELL(0, j)] = x[CELL(1, j)] + zg_offset;
            }
        } else {
            if (vec) {
                x[CELL(irad, j)] = x[CELL(irad - 2, j)];
                x[CELL(irad - 1, j)] = x[CELL(irad - 2, j)];
            } else {
                x[CELL(irad, j)] = x[CELL(irad - 1, j)] + zg_offset;
            }
        }
        break;
    case 2:
        if (!outer) {
            const float v2 = x[CELL(2, j)];
            x[CELL(1, j)] = v2 > 0.f ? 0.f : v2;
            x[CELL(0, j)] = v2 > 0.f ? 0.f : v2;
        } else {
            const float v2 = x[CELL(irad - 2, j)];
            x[CELL(irad - 1, j)] = v2 < 0.f ? 0.f : v2;
            x[CELL(irad, j)] = v2 < 0.f ? 0.f : v2;
        }
        break;
    case 3:
        if (!outer) {
            x[CELL(0, j)] = x0[CELL(0, j)];
            if (vec) x[CELL(1, j)] = x0[CELL(1, j)];
        } else {
            x[CELL(irad, j)] = x0[CELL(irad, j)];
            if (vec) x[CELL(irad - 1, j)] = x0[CELL(irad - 1, j)];
        }
        break;
    case 4:
        x[CELL(outer ? irad : 0, j)] = kep_value;
        break;
    default:
        break;
    }
}

__global__ void f_ghost(GeoF g, BcF bc, StateF s)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nz) return;
    ghost_f(s.sigma, s.sigma0, bc.sigma_in, 0, 0, nr, nz, j, 0.f, 0.f);
    ghost_f(s.sigma, s.sigma0, bc.sigma_out, 1, 0, nr, nz, j, 0.f, 0.f);
    // low part of sigma: copied by zero-gradient, cleared by reference hooks
    if (bc.sigma_in == 1) s.sigma_lo[CELL(0, j)] = s.sigma_lo[CELL(1, j)];
    else if (bc.sigma_in == 3) s.sigma_lo[CELL(0, j)] = 0.f;
    if (bc.sigma_out == 1) s.sigma_lo[CELL(nr - 1, j)] = s.sigma_lo[CELL(nr - 2, j)];
    else if (bc.sigma_out == 3) s.sigma_lo[CELL(nr - 1, j)] = 0.f;
    ghost_f(s.energy, s.energy0, bc.energy_in, 0, 0, nr, nz, j, 0.f, 0.f);
    ghost_f(s.energy, s.energy0, bc.energy_out, 1, 0, nr, nz, j, 0.f, 0.f);
    ghost_f(s.vr, s.vr0, bc.vr_in, 0, 1, nr, nz, j, 0.f, 0.f);
    ghost_f(s.vr, s.vr0, bc.vr_out, 1, 1, nr, nz, j, 0.f, 0.f);
    ghost_f(s.dv, s.dv0, bc.vaz_in, 0, 0, nr, nz, j, bc.kep_in, bc.zg_in);
    ghost_f(s.dv, s.dv0, bc.vaz_out, 1, 0, nr, nz, j, bc.kep_out, bc.zg_out);
}

// ---------------------------------------------------------------------------
// radial transport (TransportEuler.cpp:138-167, 349-406, 545-620) with the
// residual angular momentum: quantities 0,1 radial momenta, 2,3 residual
// angular momenta sigma r dv, [4 energy], last sigma.  The angular-momentum
// slopes and the limiter act on the total specific angular momentum
// J_K + r dv (J_K = r v_K per ring), the upwind star value is kept relative to
// J_K of the upwind ring, and the Keplerian part J_K * mass-flux enters the
// residual update through the per-ring differences of J_K.
// ---------------------------------------------------------------------------
template <int NQ>
__device__ __forceinline__ void rad_ring_f(int i, int j, int nz, const float *S, const float *vr,
                                           const float *dv, const float *E, const TablesF &t,
                                           float *w)
{
    const float sg = S[CELL(i, j)];
    const float r = t.Rmed[i];
    w[0] = vr[CELL(i + 1, j)];
    w[1] = vr[CELL(i, j)];
    w[2] = dv[CELL(i, jnext(j, nz))] * r;
    w[3] = dv[CELL(i, j)] * r;
    if (NQ == 5) w[4] = __fdividef(E[CELL(i, j)], sg);
    w[NQ] = sg;
}

template <int NQ>
__global__ void f_transport_radial(GeoF g, TablesF t, float dt, int mc, int chunk,
                                   const float *__restrict__ S, const float *__restrict__ vr,
                                   const float *__restrict__ dv, const float *__restrict__ E,
                                   float *__restrict__ m0, float *__restrict__ m1,
                                   float *__restrict__ m2, float *__restrict__ m3,
                                   float *__restrict__ E_out, float *__restrict__ S_out,
                                   const float *__restrict__ S_lo, float *__restrict__ S_lo_out)
{
    constexpr int NW = NQ + 1;
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nz) return;
    const int i0 = blockIdx.y * chunk;
    if (i0 >= nr) return;
    const int i1 = min(i0 + chunk, nr);
    const float dtdphi = dt * g.dphi;

    // upward difference of ring k (total slope for the angular momenta)
    auto updiff = [&](int k, const float *wlo, const float *whi, int q) -> float {
        float d = (whi[q] - wlo[q]) * t.InvDiffRmed[k + 1];
        if (q == 2 || q == 3) d += t.JSlope[k];
        return d;
    };
    auto lim = [&](int ring, float up, float down) -> float {
        if (ring <= 0 || ring >= nr - 1) return 0.f;
        return lim_f(up, down, mc);
    };

    float wa[NW] = {}, wb[NW] = {}, wn[NW] = {}, da[NW] = {}, db[NW] = {}, ub[NW] = {};
    {
        float wm2[NW] = {};
        const int r0 = i0 - 1;
        if (r0 - 1 >= 0) rad_ring_f<NQ>(r0 - 1, j, nz, S, vr, dv, E, t, wm2);
        if (r0 >= 0) rad_ring_f<NQ>(r0, j, nz, S, vr, dv, E, t, wa);
        rad_ring_f<NQ>(i0, j, nz, S, vr, dv, E, t, wb);
        const bool has_next = i0 + 1 < nr;
        if (has_next) rad_ring_f<NQ>(i0 + 1, j, nz, S, vr, dv, E, t, wn);
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const float downa = (r0 - 1 >= 0) ? updiff(r0 - 1, wm2, wa, q) : 0.f;
            const float upa = (r0 >= 0) ? updiff(r0, wa, wb, q) : 0.f;
            da[q] = r0 >= 0 ? lim(r0, upa, downa) : 0.f;
            const float upb = has_next ? updiff(i0, wb, wn, q) : 0.f;
            db[q] = lim(i0, upb, upa);
            ub[q] = upb;
        }
    }
    float flux_prev[NW] = {}, q_prev[NW] = {};
    float kep_prev = 0.f;  // Keplerian term of ring k-1 from interface k-1
    for (int k = i0; k <= i1; ++k) {
        float flux[NW];
        float kep_lower = 0.f, kep_upper = 0.f;
        if (k == 0 || k >= nr) {
#pragma unroll
            for (int q = 0; q < NW; ++q) flux[q] = 0.f;
        } else {
            const float v = vr[CELL(k, j)];
            const float base = dtdphi * t.Rinf[k];
            const float vdt = v * dt;
            float sstar;
            if (v > 0.f) {
                const float f = (t.DRmed[k] - vdt) * 0.5f;
                sstar = wa[NQ] + f * da[NQ];
#pragma unroll
                for (int q = 0; q < NQ; ++q) flux[q] = base * (wa[q] + f * da[q]) * sstar * v;
            } else {
                const float f = (t.DRmed[k + 1] + vdt) * 0.5f;
                sstar = wb[NQ] - f * db[NQ];
#pragma unroll
                for (int q = 0; q < NQ; ++q) flux[q] = base * (wb[q] - f * db[q]) * sstar * v;
            }
            const float fs = base * sstar * v;
            flux[NQ] = fs;
            // J_K(upwind) - J_K(ring) times the mass flux, for the ring above
            // (inflow from below) and the ring below (outflow upwards)
            if (v > 0.f) kep_upper = t.DJ[k] * fs;
            else kep_lower = -t.DJ[k] * fs;
        }
        if (k > i0) {
            const int i = k - 1;
            const float invs = t.InvSurf[i];
            const size_t c = CELL(i, j);
            m0[c] = q_prev[0] + (flux_prev[0] - flux[0]) * invs;
            m1[c] = q_prev[1] + (flux_prev[1] - flux[1]) * invs;
            m2[c] = q_prev[2] + (flux_prev[2] + kep_prev - flux[2] - kep_lower) * invs;
            m3[c] = q_prev[3] + (flux_prev[3] + kep_prev - flux[3] - kep_lower) * invs;
            if (NQ == 5) E_out[c] = q_prev[4] + (flux_prev[4] - flux[4]) * invs;
            float hi = q_prev[NQ], lo = S_lo[c];
            comp_add(hi, lo, (flux_prev[NQ] - flux[NQ]) * invs);
            S_out[c] = hi;
            S_lo_out[c] = lo;
        }
        if (k < i1) {
#pragma unroll
            for (int q = 0; q < NW; ++q) flux_prev[q] = flux[q];
            kep_prev = kep_upper;
            const float sb = wb[NQ];
            q_prev[0] = sb * wb[0];
            q_prev[1] = sb * wb[1];
            q_prev[2] = sb * wb[2];
            q_prev[3] = sb * wb[3];
            if (NQ == 5) q_prev[4] = E[CELL(k, j)];
            q_prev[NQ] = sb;
            const bool more = k + 2 < nr;
            float w2[NW] = {};
            if (more) rad_ring_f<NQ>(k + 2, j, nz, S, vr, dv, E, t, w2);
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                wa[q] = wb[q];
                da[q] = db[q];
                wb[q] = wn[q];
                const float up = more ? updiff(k + 1, wn, w2, q) : 0.f;
                db[q] = lim(k + 1, up, ub[q]);
                ub[q] = up;
                wn[q] = w2[q];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// azimuthal transport with FARGO (TransportEuler.cpp:174-304, 416-466,
// 630-664): FP32 advection, FP64 ring mean and shift phase.  The residual
// angular momentum is advected like any specific quantity (J_K is constant on
// a ring, so its part cancels exactly).
// ---------------------------------------------------------------------------
template <int PER>
__device__ void ring_pass_f(float *S, float *SS, float *W, float *D, float *const *qrow, int nq,
                            const float *v, float *slo, float dt, float dxtheta, float half_invdx,
                            float dxrad, float invsurf, int nz, int mc, bool uniform, float vconst)
{
    const int tid = threadIdx.x, bs = blockDim.x;
    float invs[PER], f[PER];
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
            D[j] = lim_f(S[jp] - S[j], S[j] - S[jm], mc) * half_invdx;
            invs[n] = __frcp_rn(S[j]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jm = j == 0 ? nz - 1 : j - 1;
            const float vv = uniform ? vconst : v[n];
            const float ksi = vv * dt;
            SS[j] = ksi > 0.f ? S[jm] + (dxtheta - ksi) * D[jm] : S[j] - (dxtheta + ksi) * D[j];
        }
    }
    __syncthreads();
    for (int q = 0; q < nq; ++q) {
        float *Q = qrow[q];
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) W[j] = Q[j] * invs[n];
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
                D[j] = lim_f(W[jp] - W[j], W[j] - W[jm], mc) * half_invdx;
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                const int jm = j == 0 ? nz - 1 : j - 1;
                const float vv = uniform ? vconst : v[n];
                const float ksi = vv * dt;
                const float qs = ksi > 0.f ? W[jm] + (dxtheta - ksi) * D[jm]
                                           : W[j] - (dxtheta + ksi) * D[j];
                f[n] = dxrad * qs * SS[j] * vv;
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) W[j] = f[n];
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) Q[j] += (W[j] - W[j == nz - 1 ? 0 : j + 1]) * invsurf;
        }
        __syncthreads();
    }
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) W[j] = dxrad * SS[j] * (uniform ? vconst : v[n]);
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            f[n] = S[j];
            comp_add(f[n], slo[n], (W[j] - W[j == nz - 1 ? 0 : j + 1]) * invsurf);
        }
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) S[j] = f[n];
    }
    __syncthreads();
}

template <int PER>
__global__ void __launch_bounds__(512) f_transport_azimuthal(GeoF g, TablesF t, double dt, int mc,
                                                             int fast, int nq,
                                                             const float *__restrict__ dv,
                                                             float *m0, float *m1, float *m2,
                                                             float *m3, float *E, float *S,
                                                             float *S_lo)
{
    extern __shared__ float smf[];
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x;
    const int tid = threadIdx.x, bs = blockDim.x;
    const size_t row = (size_t)i * nz;
    float *Sr = smf, *SS = smf + nz, *W = smf + 2 * nz, *D = smf + 3 * nz;

    float vown[PER], slo[PER];
    double part = 0.0;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            vown[n] = dv[row + j];
            part += (double)vown[n];
        }
    }
    // ring mean of v_phi and the FARGO shift phase in FP64 (:174-236)
    const double mean_dv = bsum_d(part, red) / (double)nz;
    const double vmean = t.Vref_d[i] + mean_dv;
    const double Ntilde = vmean * t.InvRmed_d[i] * dt * g.invdphi_d;
    const double Nround = floor(Ntilde + 0.5);
    const int nshift = (int)Nround;
    const float vt = (float)((Ntilde - Nround) * t.Rmed_d[i] * (1.0 / dt) * g.dphi_d);
    const float mdv = (float)mean_dv;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            // residual about the ring mean (compute_residual_velocity, :194-205)
            float vres = vown[n] - mdv;
            if (!fast) vres = vt + vres;
            vown[n] = vres;
            Sr[j] = S[row + j];
            slo[n] = S_lo[row + j];
        }
    }
    __syncthreads();
    float *qrow[5] = {m0 + row, m1 + row, m2 + row, m3 + row, E + row};
    const float dxtheta = g.dphi * t.Rmed[i];
    const float half_invdx = 0.5f / dxtheta;
    const float dxrad = (t.Rsup[i] - t.Rinf[i]) * (float)dt;
    const float invsurf = t.InvSurf[i];
    ring_pass_f<PER>(Sr, SS, W, D, qrow, nq, vown, slo, (float)dt, dxtheta, half_invdx, dxrad,
                     invsurf, nz, mc, false, 0.f);
    if (fast) {
        ring_pass_f<PER>(Sr, SS, W, D, qrow, nq, vown, slo, (float)dt, dxtheta, half_invdx, dxrad,
                         invsurf, nz, mc, true, vt);
    }
    for (int q = 0; q <= nq; ++q) {
        float *Q = q < nq ? qrow[q] : S + row;
        const float *src = q < nq ? qrow[q] : Sr;
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) W[j] = src[j];
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                int ji = (j - nshift) % nz;
                if (ji < 0) ji += nz;
                Q[j] = W[ji];
            }
        }
        __syncthreads();
    }
    // the low part of sigma moves with it
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) W[j] = slo[n];
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            int ji = (j - nshift) % nz;
            if (ji < 0) ji += nz;
            S_lo[row + j] = W[ji];
        }
    }
}

// velocities from momenta (:498-535), floors
__global__ void f_finish(GeoF g, TablesF t, PhysF ph, const float *__restrict__ m0,
                         const float *__restrict__ m1, const float *__restrict__ m2,
                         const float *__restrict__ m3, const float *__restrict__ S_t,
                         const float *__restrict__ E_t, const float *__restrict__ vr_in,
                         float *__restrict__ vr_out, float *__restrict__ dv_out,
                         float *__restrict__ S_out, float *__restrict__ E_out,
                         const float *__restrict__ Slo_t, float *__restrict__ Slo_out)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    if (i == nr) {
        vr_out[c] = vr_in[c];
        return;
    }
    const float s = S_t[c];
    if (i == 0) {
        vr_out[c] = 0.f;
    } else {
        const size_t cm = CELL(i - 1, j);
        vr_out[c] = __fdividef(m0[cm] + m1[c], S_t[cm] + s);
    }
    const size_t cjm = CELL(i, jprev(j, nz));
    dv_out[c] = __fdividef(m2[cjm] + m3[c], S_t[cjm] + s) * t.InvRmed[i];
    const bool floored = s < ph.sigma_min;
    const float sf = floored ? ph.sigma_min : s;
    S_out[c] = sf;
    Slo_out[c] = floored ? 0.f : Slo_t[c];
    if (ph.adiabatic) E_out[c] = tfloor(E_t[c], sf, ph);
}

// damping zones (damping.cpp:311-776)
__device__ void damp_ring_f(float *X, float *X0, const DampQF &d, int i, int nz, int outer, float dt,
                            float *red, float *Xlo)
{
    const int kind = outer ? d.kind_out : d.kind_in;
    const size_t row = (size_t)i * nz;
    float x0c = 0.f;
    if (kind == 3) {
        float part = 0.f;
        for (int j = threadIdx.x; j < nz; j += blockDim.x) part += X[row + j];
        const float mean = bsum_f(part, red) / nz;
        if (threadIdx.x == 0) X0[row] = mean;
        x0c = mean;
    } else if (kind == 2) {
        x0c = outer ? d.x0_zero_out[i] : d.x0_zero_in[i];
    }
    const float factor = outer ? d.fac_out[i] : d.fac_in[i];
    const float tau = outer ? d.tau_out : d.tau_in;
    const float ef = __expf(-dt * factor / tau);
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const float x0 = kind == 1 ? X0[row + j] : x0c;
        X[row + j] = (X[row + j] - x0) * ef + x0;
        if (Xlo) Xlo[row + j] *= ef;
    }
    __syncthreads();
}

__global__ void f_damping(GeoF g, DampingF dm, float dt, const int *__restrict__ rings, StateF s)
{
    __shared__ float red[33];
    const int nz = g.nz, nr = g.nr;
    const int i = rings[blockIdx.x];
    float *X[4] = {s.vr, s.dv, s.sigma, s.energy};
    float *X0[4] = {s.vr0, s.dv0, s.sigma0, s.energy0};
    for (int q = 0; q < 4; ++q) {
        const DampQF &d = dm.q[q];
        const int size = d.vector ? nr + 1 : nr;
        float *lo = q == 2 ? s.sigma_lo : nullptr;
        if (d.kind_in != 0 && d.active_in && i <= d.limit_in)
            damp_ring_f(X[q], X0[q], d, i, nz, 0, dt, red, lo);
        if (d.kind_out != 0 && d.active_out && i >= d.limit_out && i < size)
            damp_ring_f(X[q], X0[q], d, i, nz, 1, dt, red, lo);
    }
}

// derived quantities + CFL (SourceEuler.cpp:225-249, cfl.cpp:185-382)
__global__ void f_derived_cfl(GeoF g, TablesF t, PhysF ph, int mode, const float *__restrict__ S,
                              const float *__restrict__ E, const float *__restrict__ vr,
                              const float *__restrict__ dv, const float *__restrict__ qplus,
                              const float *__restrict__ qminus, float *__restrict__ cs,
                              float *__restrict__ H, float *__restrict__ P, float *__restrict__ T,
                              float *__restrict__ nu, unsigned int *__restrict__ dt_min)
{
    __shared__ float red[33];
    const int nz = g.nz, nr = g.nr;
    const int i = blockIdx.x;
    const size_t row = (size_t)i * nz;
    const bool do_cfl = (mode & 4) != 0;
    float md0 = 0.f, md1 = 0.f;
    if (do_cfl && i < nr - 1) {
        float p0 = 0.f, p1 = 0.f;
        for (int j = threadIdx.x; j < nz; j += blockDim.x) {
            p0 += dv[row + j];
            p1 += dv[row + nz + j];
        }
        md0 = bsum_f(p0, red) / (float)nz;
        md1 = bsum_f(p1, red) / (float)nz;
    }
    float local = 3.0e38f;
    if (do_cfl && i < nr - 1 && i >= 0 && (i == 0 || i < nr - 1)) {
        // shear limit: |vm_i / R_i - vm_{i+1} / R_{i+1}| with vm = Vref + mean dv
        const float denom = fabsf(t.OmRefDiff[i] + md0 * t.InvRmed[i] - md1 * t.InvRmed[i + 1]) +
                            1.0e-30f;
        local = ph.cfl * g.dphi / denom;
    }
    const bool cfl_ring = do_cfl && i >= 1 && i < nr - 1;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const size_t c = row + j;
        float c_s, n;
        if (mode & 1) {
            const float sg = S[c];
            if (ph.adiabatic) {
                const float e = E[c];
                const float es = __fdividef(e, sg);
                T[c] = ph.c_v_inv * es;
                c_s = sqrtf(ph.g_gm1 * es);
                const float h = c_s * t.HFacAdi[i];
                cs[c] = c_s;
                H[c] = h;
                P[c] = ph.gm1 * e;
                n = ph.alpha > 0.f ? ph.alpha * h * c_s : ph.constant_viscosity;
            } else {
                c_s = t.CsIso[i];
                const float h = c_s * t.InvOmegaK[i];
                P[c] = sg * (c_s * c_s);
                if (mode & 2) {
                    cs[c] = c_s;
                    H[c] = h;
                    T[c] = ph.mu_over_R * P[c] / sg;
                }
                n = ph.alpha > 0.f ? ph.alpha * h * c_s : ph.constant_viscosity;
            }
            nu[c] = n;
        } else {
            c_s = cs[c];
            n = nu[c];
        }
        if (cfl_ring) {
            const float d0 = dv[c];
            const float vres = ph.fast_transport ? d0 - md0 : t.Vref[i] + d0;
            const float invdt1 = c_s * t.InvCell[i];
            const float invdt2 = vr[c] * t.InvDiffRsup[i];
            const float invdt3 = vres * t.InvDxTheta[i];
            const float vr1 = vr[c + nz];
            const float dvA = dv[row + (j == nz - 1 ? 0 : j + 1)] - d0;
            float invdt4;
            if (ph.art_visc_sn) {
                const float a = fmaxf(vr[c] - vr1, 0.f) * t.InvDiffRsup[i];
                const float b = fmaxf(-dvA, 0.f) * t.InvDxTheta[i];
                invdt4 = ph.four_C2 * fmaxf(a, b);
            } else {
                const float eps_rr = (vr1 - vr[c]) * t.InvDiffRsup[i];
                const float eps_pp = t.InvRmed[i] * (dvA * g.invdphi + 0.5f * (vr1 + vr[c]));
                invdt4 = ph.four_C2 * fmaxf(-(eps_rr + eps_pp), 0.f);
            }
            const float invdt5 = 4.f * n * t.InvCell2[i];
            float invdt6 = 0.f;
            if (ph.adiabatic) invdt6 = ph.inv_hc_limit * fabsf(__fdividef(qplus[c] - qminus[c], E[c]));
            const float s2 = invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 +
                             invdt4 * invdt4 + invdt5 * invdt5 + invdt6 * invdt6;
            local = fminf(local, ph.cfl * rsqrtf(s2));
        }
    }
    if (do_cfl) {
        const float m = bmin_f(local, red);
        if (threadIdx.x == 0 && m < 3.0e38f) atomicMin(dt_min, __float_as_uint(m));
    }
}

// disk force on a body and gas mass: FP64 separations and accumulation
__global__ void f_disk_force(GeoF g, TablesF t, PhysF ph, double px, double py, double pa,
                             double rsm, const float *__restrict__ S, const float *__restrict__ H,
                             double *__restrict__ partial)
{
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x + 1;
    const size_t row = (size_t)i * nz;
    double ps = 0.0;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) ps += (double)S[row + j];
    const double sigma1d = bsum_d(ps, red) / nz;
    double ax = 0.0, ay = 0.0, mass = 0.0;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const double dx = t.Rmed_d[i] * t.cos_d[j] - px, dy = t.Rmed_d[i] * t.sin_d[j] - py;
        const float sm = ph.eps_smooth * H[row + j];
        const float d2 = (float)(dx * dx + dy * dy) + sm * sm;
        const float rinv = rsqrtf(d2);
        float fk = 1.f;
        if (rsm > 0.0) {
            const float dsm = d2 * rinv;
            if (dsm < (float)rsm) {
                const float q = dsm / (float)rsm;
                fk = -(3.f * q * q * q * q - 4.f * q * q * q);
            }
        }
        const double cellmass = t.Surf_d[i] * ((double)S[row + j] - sigma1d);
        const double w = cellmass * (double)(rinv * rinv * rinv * fk) * ph.G_d;
        ax += w * dx;
        ay += w * dy;
        mass += t.Surf_d[i] * (double)S[row + j];
    }
    ax = bsum_d(ax, red);
    ay = bsum_d(ay, red);
    mass = bsum_d(mass, red);
    if (threadIdx.x == 0) {
        const bool inner = t.Rmed_d[i] < pa;
        double *p = partial + (size_t)blockIdx.x * 5;
        p[0] = inner ? ax : 0.0;
        p[1] = inner ? ay : 0.0;
        p[2] = inner ? 0.0 : ax;
        p[3] = inner ? 0.0 : ay;
        p[4] = mass;
    }
}

__global__ void f_reduce_rows(const double *__restrict__ partial, int rows, double *__restrict__ out)
{
    const int w = threadIdx.x;
    if (w >= 5) return;
    double s = 0.0, comp = 0.0;
    for (int r = 0; r < rows; ++r) {
        const double y = partial[(size_t)r * 5 + w] - comp;
        const double tt = s + y;
        comp = (tt - s) - y;
        s = tt;
    }
    out[w] = s;
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
           OMREFDIFF, VREF, NT };
    std::vector<float> hf((size_t)NT * R, 0.f);
    auto F = [&](int k) { return hf.data() + (size_t)k * R; };
    for (int n = 0; n <= nr; ++n) {
        const double rm = Rmed[n], dxr = Rsup[n] - Rinf[n], dxa = rm * dphi;
        const double om = std::sqrt(G * M / (rm * rm * rm));
        const double cell = std::min(dxr, dxa);
        F(RINF)[n] = (float)Rinf[n];
        F(RSUP)[n] = (float)Rsup[n];
        F(RMED)[n] = (float)rm;
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
    t.JSlope = Df(JSLOPE); t.DRmed = Df(DRMED); t.OmRefDiff = Df(OMREFDIFF); t.Vref = Df(VREF);
    t.Rmed_d = tab_d; t.InvRmed_d = tab_d + R; t.Vref_d = tab_d + 2 * R; t.Surf_d = tab_d + 3 * R;
    t.PhiK_d = tab_d + 4 * R; t.cos_d = tab_d + 5 * R; t.sin_d = tab_d + 5 * R + nz;

    // physics
    PhysF &ph = phys;
    ph.adiabatic = p.eos == FGPU_EOS_IDEAL;
    ph.art_visc_sn = p.art_visc == FGPU_ARTVISC_SN;
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
    ph.inv_hc_limit = (float)(1.0 / p.heating_cooling_cfl_limit);
    ph.sigma_min = (float)(p.sigma_floor * p.sigma0);
    ph.sigma_floor10 = (float)(10.0 * p.sigma0 * p.sigma_floor);
    ph.eps_smooth = (float)p.thickness_smoothing;
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
    CKF(cudaMalloc(&alt_sigma, cells * sizeof(float)));
    CKF(cudaMalloc(&alt_vr, vcells * sizeof(float)));
    CKF(cudaMalloc(&alt_dv, cells * sizeof(float)));
    CKF(cudaMalloc(&alt_e, cells * sizeof(float)));
    CKF(cudaMemset(alt_e, 0, cells * sizeof(float)));
    CKF(cudaMalloc(&sigma_lo, cells * sizeof(float)));
    CKF(cudaMemset(sigma_lo, 0, cells * sizeof(float)));
    CKF(cudaMalloc(&alt_sigma_lo, cells * sizeof(float)));
    CKF(cudaMemset(alt_sigma_lo, 0, cells * sizeof(float)));
    for (int k = 0; k < 4; ++k) CKF(cudaMalloc(&mom[k], cells * sizeof(float)));
    CKF(cudaMalloc(&partial, sizeof(double) * 5 * (size_t)nr));
    CKF(cudaMalloc(&red_out, sizeof(double) * 8));
    CKF(cudaMalloc(&d_dtmin, sizeof(unsigned int)));
    CKF(cudaMalloc(&d_bad, sizeof(unsigned long long)));
    CKF(cudaMallocHost(&h_pinned, sizeof(double) * 16));
    CKF(cudaMalloc(&stage, sizeof(double) * vcells));

    // boundary hooks on the residual v_phi
    bc.sigma_in = p.bc_sigma_inner; bc.sigma_out = p.bc_sigma_outer;
    bc.energy_in = p.bc_energy_inner; bc.energy_out = p.bc_energy_outer;
    bc.vr_in = p.bc_vrad_inner; bc.vr_out = p.bc_vrad_outer;
    bc.vaz_in = p.bc_vaz_inner; bc.vaz_out = p.bc_vaz_outer;
    bc.kep_in = (float)(p.vaz_inner_keplerian_factor * std::sqrt(G * M / Rmed[0]) - Vref[0]);
    bc.kep_out = (float)(p.vaz_outer_keplerian_factor * std::sqrt(G * M / Rmed[nr - 1]) -
                         Vref[nr - 1]);
    bc.zg_in = (float)(Vref[1] - Vref[0]);
    bc.zg_out = (float)(Vref[nr - 2] - Vref[nr - 1]);

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
    for (int n = 0; n <= nr; ++n) dzero[n] = (float)(-Vref[n]);  // v_phi -> 0
    CKF(cudaMalloc(&damp_mem, sizeof(float) * (dfac.size() + dzero.size() + 2)));
    CKF(cudaMemcpy(damp_mem, dfac.data(), sizeof(float) * dfac.size(), cudaMemcpyHostToDevice));
    float *zero_vphi = damp_mem + dfac.size();
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
    if (n_rings) {
        CKF(cudaMalloc(&damp_rings, sizeof(int) * rings.size()));
        CKF(cudaMemcpy(damp_rings, rings.data(), sizeof(int) * rings.size(), cudaMemcpyHostToDevice));
    }
    // azimuthal kernel configuration
    per = nz <= 2048 ? 4 : (nz <= 4096 ? 8 : 16);
    az_block = std::max(128, std::min(512, ((nz + per - 1) / per + 31) / 32 * 32));
    az_smem = (size_t)4 * nz * sizeof(float);
    if (az_smem > 200 * 1024) {
        err = "ring too long for the FP32 azimuthal kernel";
        return FGPU_ERR_UNSUPPORTED;
    }
    cudaError_t e1 = cudaFuncSetAttribute(f_transport_azimuthal<4>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)az_smem);
    cudaError_t e2 = cudaFuncSetAttribute(f_transport_azimuthal<8>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)az_smem);
    cudaError_t e3 = cudaFuncSetAttribute(f_transport_azimuthal<16>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)az_smem);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
        err = "cannot reserve shared memory for the FP32 azimuthal kernel";
        return FGPU_ERR_CUDA;
    }
    CKF(cudaDeviceSynchronize());
    return FGPU_OK;
}

void Engine32::destroy()
{
    for (int f = 0; f < FGPU_FIELD_COUNT; ++f) cudaFree(fld[f]);
    cudaFree(alt_sigma); cudaFree(alt_vr); cudaFree(alt_dv); cudaFree(alt_e);
    cudaFree(sigma_lo); cudaFree(alt_sigma_lo);
    for (int k = 0; k < 4; ++k) cudaFree(mom[k]);
    cudaFree(partial); cudaFree(red_out); cudaFree(d_dtmin); cudaFree(d_bad); cudaFree(stage);
    cudaFree(tab_f); cudaFree(tab_d); cudaFree(damp_mem); cudaFree(damp_aux); cudaFree(damp_rings);
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

// rows of a field and the ring offset between stored and FargoCPT values
const double *Engine32::offset_of(int f) const
{
    if (f == FGPU_V_AZIMUTHAL || f == FGPU_V_AZIMUTHAL0) return tabs.Vref_d;
    if (f == FGPU_POTENTIAL) return tabs.PhiK_d;
    return nullptr;
}

int Engine32::upload(int f, const double *host, int rows)
{
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

int Engine32::download(int f, double *host, int rows)
{
    const size_t n = (size_t)rows * nz;
    if (f == FGPU_SIGMA)
        f_join_f64<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(fld[f], sigma_lo, stage, n);
    else
        f_to_f64<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(fld[f], stage, n, nz, offset_of(f));
    CKF(cudaGetLastError());
    CKF(cudaMemcpyAsync(host, stage, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CKF(cudaStreamSynchronize(stream));
    return FGPU_OK;
}

void Engine32::set_bodies(int n, const fgpu_body *b, double ix, double iy)
{
    bodies.n = n;
    bodies.star_at_origin = n > 0 && b[0].x == 0.0 && b[0].y == 0.0 &&
                            b[0].mass == p.hydro_center_mass && b[0].r_sm == 0.0;
    for (int k = 0; k < n; ++k) {
        bodies.x[k] = b[k].x;
        bodies.y[k] = b[k].y;
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
    StateF s = state();
    if (mode & 4) CKF(cudaMemsetAsync(d_dtmin, 0x7f, sizeof(unsigned int), stream));
    f_derived_cfl<<<nr, 256, 0, stream>>>(geo, tabs, phys, mode, s.sigma, s.energy, s.vr, s.dv,
                                          fld[FGPU_QPLUS], fld[FGPU_QMINUS], fld[FGPU_SOUNDSPEED],
                                          fld[FGPU_SCALE_HEIGHT], fld[FGPU_PRESSURE],
                                          fld[FGPU_TEMPERATURE], fld[FGPU_VISCOSITY], d_dtmin);
    CKF(cudaGetLastError());
    if (mode & 4) cfl_valid = true;
    return FGPU_OK;
}

int Engine32::init_euler(double t)
{
    int rc = derived_cfl(1 | 2);
    if (rc) return rc;
    if (phys.adiabatic) {
        StateF s = state();
        f_stress<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, s.sigma, s.vr, s.dv,
                                                    fld[FGPU_VISCOSITY], fld[FGPU_DIV_V],
                                                    fld[FGPU_TAU_R_R], fld[FGPU_TAU_PHI_PHI],
                                                    fld[FGPU_TAU_R_PHI]);
        f_viscous<<<grid2(nz, nr), 128, 0, stream>>>(
            geo, tabs, phys, 0.f, (float)beta_inv(t), 2, s.sigma, fld[FGPU_TAU_R_R],
            fld[FGPU_TAU_PHI_PHI], fld[FGPU_TAU_R_PHI], fld[FGPU_DIV_V], fld[FGPU_VISCOSITY],
            fld[FGPU_SCALE_HEIGHT], s.sigma0, s.energy0, s.vr, s.dv, s.energy, fld[FGPU_QPLUS],
            fld[FGPU_QMINUS]);
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

int Engine32::boundary(double dt, bool final)
{
    if (final && p.damping && n_rings)
        f_damping<<<n_rings, 256, 0, stream>>>(geo, dm, (float)dt, damp_rings, state());
    f_ghost<<<(nz + 127) / 128, 128, 0, stream>>>(geo, bc, state());
    CKF(cudaGetLastError());
    cfl_valid = false;
    return FGPU_OK;
}

int Engine32::step(double dt, double t)
{
    const float fdt = (float)dt;
    const bool adi = phys.adiabatic;
    auto mark = [&](int k) {
        if (mark_fn) mark_fn(mark_ctx, k);
    };
    mark(-1);
    f_potential<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, phys, bodies, fld[FGPU_SCALE_HEIGHT],
                                                   fld[FGPU_POTENTIAL]);
    mark(0);
    f_source<<<grid2(nz, nr + 1), 128, 0, stream>>>(geo, tabs, fdt, fld[FGPU_SIGMA],
                                                    fld[FGPU_PRESSURE], fld[FGPU_POTENTIAL],
                                                    fld[FGPU_V_RADIAL], fld[FGPU_V_AZIMUTHAL],
                                                    alt_vr, alt_dv);
    std::swap(fld[FGPU_V_RADIAL], alt_vr);
    std::swap(fld[FGPU_V_AZIMUTHAL], alt_dv);
    mark(1);
    StateF s = state();
    if (adi || phys.art_visc_sn) {
        f_artvisc_q<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, phys, fdt, s.sigma, s.vr, s.dv,
                                                       s.energy, fld[FGPU_Q_R], fld[FGPU_Q_PHI]);
        mark(2);
        f_artvisc_v<<<grid2(nz, nr), 128, 0, stream>>>(
            geo, tabs, phys, fdt, s.sigma, s.energy, fld[FGPU_Q_R], fld[FGPU_Q_PHI], s.vr, s.dv,
            fld[FGPU_SOUNDSPEED], fld[FGPU_SCALE_HEIGHT], fld[FGPU_VISCOSITY]);
        mark(3);
    } else {
        mark(2);
        mark(3);
    }
    f_stress<<<grid2(nz, nr), 128, 0, stream>>>(geo, tabs, s.sigma, s.vr, s.dv,
                                                fld[FGPU_VISCOSITY], fld[FGPU_DIV_V],
                                                fld[FGPU_TAU_R_R], fld[FGPU_TAU_PHI_PHI],
                                                fld[FGPU_TAU_R_PHI]);
    mark(4);
    f_viscous<<<grid2(nz, nr), 128, 0, stream>>>(
        geo, tabs, phys, fdt, (float)beta_inv(t), adi ? 7 : 1, s.sigma, fld[FGPU_TAU_R_R],
        fld[FGPU_TAU_PHI_PHI], fld[FGPU_TAU_R_PHI], fld[FGPU_DIV_V], fld[FGPU_VISCOSITY],
        fld[FGPU_SCALE_HEIGHT], s.sigma0, s.energy0, s.vr, s.dv, s.energy, fld[FGPU_QPLUS],
        fld[FGPU_QMINUS]);
    mark(5);
    f_ghost<<<(nz + 127) / 128, 128, 0, stream>>>(geo, bc, s);
    mark(6);
    {
        const int chunk = 16;
        dim3 grid((nz + 63) / 64, (nr + chunk - 1) / chunk);
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
    mark(7);
    {
        const int nq = adi ? 5 : 4;
#define AZ32(P)                                                                                  \
    f_transport_azimuthal<P><<<nr, az_block, az_smem, stream>>>(                                 \
        geo, tabs, dt, phys.limiter_mc, phys.fast_transport, nq, s.dv, mom[0], mom[1], mom[2],  \
        mom[3], alt_e, alt_sigma, alt_sigma_lo)
        if (per == 4) AZ32(4);
        else if (per == 8) AZ32(8);
        else AZ32(16);
#undef AZ32
    }
    mark(8);
    f_finish<<<grid2(nz, nr + 1), 128, 0, stream>>>(geo, tabs, phys, mom[0], mom[1], mom[2],
                                                    mom[3], alt_sigma, alt_e, s.vr, alt_vr,
                                                    alt_dv, s.sigma, s.energy, alt_sigma_lo,
                                                    sigma_lo);
    std::swap(fld[FGPU_V_RADIAL], alt_vr);
    std::swap(fld[FGPU_V_AZIMUTHAL], alt_dv);
    mark(9);
    s = state();
    if (p.damping && n_rings)
        f_damping<<<n_rings, 256, 0, stream>>>(geo, dm, fdt, damp_rings, s);
    mark(10);
    f_ghost<<<(nz + 127) / 128, 128, 0, stream>>>(geo, bc, s);
    mark(11);
    int rc = derived_cfl(1 | 4);
    if (rc) return rc;
    mark(12);
    CKF(cudaGetLastError());
    return FGPU_OK;
}

int Engine32::disk_force(double px, double py, double pa, double rsm, double out[5])
{
    const int rows = nr - 2;
    f_disk_force<<<rows, 256, 0, stream>>>(geo, tabs, phys, px, py, pa, rsm, fld[FGPU_SIGMA],
                                           fld[FGPU_SCALE_HEIGHT], partial);
    f_reduce_rows<<<1, 32, 0, stream>>>(partial, rows, red_out);
    CKF(cudaGetLastError());
    CKF(cudaMemcpyAsync(h_pinned, red_out, sizeof(double) * 5, cudaMemcpyDeviceToHost, stream));
    CKF(cudaStreamSynchronize(stream));
    for (int k = 0; k < 5; ++k) out[k] = h_pinned[k];
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
