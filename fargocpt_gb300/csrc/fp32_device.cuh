// Device bodies of the FP32-mixed hydro step, shared by the single-disk
// kernels (kernels_fp32.cu) and the batched many-disk kernels
// (batch_fp32.cu).  Each body updates one cell, one column or one ring of one
// disk; the kernels around them only decide which disk, ring and column a
// thread works on.  The storage conventions (residual v_phi about v_K(Rmed),
// potential residual about -G M / Rmed, compensated sigma hi + lo) are
// described at the top of kernels_fp32.cu.
#pragma once

#include "fp32_engine.h"

#include <cuda_runtime.h>

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

// The star values and fluxes of the azimuthal passes with the rounding of
// every operation fixed (an explicit FMA where the value is interpolated),
// so that the strided and the register-blocked ring kernels, whose code the
// compiler would otherwise contract differently, give the same bits; the
// passes spell out the specific values (q / sigma as q times 1 / sigma) and
// the slopes' differences and scaling for the same reason (the blocked kernel
// holds a specific value in a register where it is differenced, the strided
// one reloads it from shared memory, and only the former may fuse the two).
//   upwind value on the positive side: W_jm + (dx - ksi) D_jm
//   on the negative side:              W_j  - (dx + ksi) D_j
__device__ __forceinline__ float star_pos(float w, float d, float dx, float ksi)
{
    return __fmaf_rn(__fsub_rn(dx, ksi), d, w);
}
__device__ __forceinline__ float star_neg(float w, float d, float dx, float ksi)
{
    return __fmaf_rn(-__fadd_rn(dx, ksi), d, w);
}
// X_u + a D_u and the neighbour difference (X_u - X_u1) + a (D_u - D_u1)
__device__ __forceinline__ float star_at(float x, float d, float a) { return __fmaf_rn(a, d, x); }
__device__ __forceinline__ float star_diff(float xu, float xu1, float du, float du1, float a)
{
    return __fmaf_rn(a, __fsub_rn(du, du1), __fsub_rn(xu, xu1));
}
// q += c (qs dS* + S*_{j+1} dq*) of the uniform pass
__device__ __forceinline__ float uniform_update(float q, float c, float qs, float dss, float fs,
                                                float dqs)
{
    return __fadd_rn(q, __fmul_rn(c, __fmaf_rn(qs, dss, __fmul_rn(fs, dqs))));
}

// hi + lo += x with the rounding error of hi + x kept in lo (TwoSum,
// Knuth 1969: exact for any order of magnitudes)
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, err);
}

__device__ __forceinline__ float tfloor(float e, float sigma, const PhysF &ph)
{
    const float emin = sigma * ph.emin_fac;
    const float emax = sigma * ph.emax_fac;
    if (!(e > emin)) e = emin;
    if (!(e < emax)) e = emax;
    return e;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_min_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
template <typename T, T (*WARP)(T)>
__device__ __forceinline__ T block_reduce(T v, T *red, T neutral)
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
__device__ __forceinline__ double bsum_d(double v, double *red)
{
    return block_reduce<double, warp_sum_d>(v, red, 0.0);
}
__device__ __forceinline__ float bsum_f(float v, float *red)
{
    return block_reduce<float, warp_sum_f>(v, red, 0.f);
}
__device__ __forceinline__ float bmin_f(float v, float *red)
{
    return block_reduce<float, warp_min_f>(v, red, 3.0e38f);
}

__device__ __forceinline__ float warp_max_f(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Ring sums that do not depend on the block's shape.  Every value is rounded
// to a multiple of 2^-k and the resulting 64-bit integers are added; integer
// addition is associative, so neither the tile shape a kernel runs with nor
// the order of the threads changes a bit of the result.  k is the largest
// exponent for which n values of at most the block's largest |x| stay below
// 2^62 in total; the sum is then within n 2^-k (about 2^-51 n max|x|) of the
// exact one.  Every thread of the block must call both steps.
//
// Step 1: the scale, from the block's largest |x| (an exact reduction).
__device__ __forceinline__ int exact_sum_scale(float local_absmax, int n, float *redf)
{
    const float m = block_reduce<float, warp_max_f>(local_absmax, redf, 0.f);
    int e = 0;
    frexpf(m, &e);                // m < 2^e
    const int ln = 32 - __clz(n);  // n < 2^ln
    return 62 - e - ln;
}
__device__ __forceinline__ long long to_fixed(float x, int k) { return __float2ll_rn(ldexpf(x, k)); }
// Step 2: the sum of the threads' integer partial sums.
__device__ __forceinline__ double exact_sum_result(long long part, int k, long long *redl)
{
    const long long s = block_reduce<long long, warp_sum_ll>(part, redl, 0LL);
    return ldexp((double)s, -k);
}

__device__ __forceinline__ float2 warp_max_f2(float2 v)
{
    for (int o = 16; o > 0; o >>= 1) {
        v.x = fmaxf(v.x, __shfl_down_sync(0xffffffffu, v.x, o));
        v.y = fmaxf(v.y, __shfl_down_sync(0xffffffffu, v.y, o));
    }
    return v;
}
__device__ __forceinline__ longlong2 warp_sum_ll2(longlong2 v)
{
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// Means of two rows at once (the CFL's ring i and ring i + 1), each with its
// own scale, in two block reductions.  red2: 33 float2, redl2: 33 longlong2.
__device__ __forceinline__ float2 exact_row_means2(const float *a, const float *b, int n,
                                                   float2 *red2, longlong2 *redl2)
{
    float2 m = make_float2(0.f, 0.f);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        m.x = fmaxf(m.x, fabsf(a[j]));
        m.y = fmaxf(m.y, fabsf(b[j]));
    }
    m = block_reduce<float2, warp_max_f2>(m, red2, make_float2(0.f, 0.f));
    int ea = 0, eb = 0;
    frexpf(m.x, &ea);
    frexpf(m.y, &eb);
    const int ln = 32 - __clz(n);
    const int ka = 62 - ea - ln, kb = 62 - eb - ln;
    longlong2 part = make_longlong2(0, 0);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        part.x += to_fixed(a[j], ka);
        part.y += to_fixed(b[j], kb);
    }
    part = block_reduce<longlong2, warp_sum_ll2>(part, redl2, make_longlong2(0, 0));
    return make_float2((float)(ldexp((double)part.x, -ka) / (double)n),
                       (float)(ldexp((double)part.y, -kb) / (double)n));
}

// Mean of row[0 .. n-1] (global memory, cells strided over the block).
__device__ __forceinline__ float exact_row_mean(const float *row, int n, float *redf,
                                                long long *redl)
{
    float m = 0.f;
    for (int j = threadIdx.x; j < n; j += blockDim.x) m = fmaxf(m, fabsf(row[j]));
    const int k = exact_sum_scale(m, n, redf);
    long long part = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) part += to_fixed(row[j], k);
    return (float)(exact_sum_result(part, k, redl) / (double)n);
}

// ---------------------------------------------------------------------------
// Potential residual Phi - Phi_K (CalculateNbodyPotential, Pframeforce.cpp:21-86)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void potential_cell(const GeoF &g, const TablesF &t, const PhysF &ph,
                                               const BodiesF &b, const float *__restrict__ H,
                                               float *__restrict__ pot, int i, int j)
{
    const int nz = g.nz;
    // the cell centre as float pairs (x = xh + xl): the product's rounding
    // error by FMA plus the cross terms of the split factors; the distance to
    // a body then loses nothing to cancellation however close the body is
    const float rh = t.Rmed[i], rl = t.RmedLo[i];
    const float ch = t.cosHi[j], cl = t.cosLo[j], sh = t.sinHi[j], sl = t.sinLo[j];
    const float xh = rh * ch, yh = rh * sh;
    const float xl = fmaf(rh, ch, -xh) + fmaf(rh, cl, rl * ch);
    const float yl = fmaf(rh, sh, -yh) + fmaf(rh, sl, rl * sh);
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
        } else if (k == 0) {
            // central object off the origin: residual against -G M / r in FP64
            const double xd = t.Rmed_d[i] * t.cos_d[j], yd = t.Rmed_d[i] * t.sin_d[j];
            const double dx = xd - b.x[0], dy = yd - b.y[0];
            const float d2 = (float)(dx * dx + dy * dy) + s2;
            const float inv_d = rsqrtf(d2);
            float fk = 1.f;
            if (b.rsm[0] > 0.f) {
                const float dsm = d2 * inv_d;
                if (dsm < b.rsm[0]) {
                    const float q = dsm / b.rsm[0];
                    fk = q * q * q * q - 2.f * q * q * q + 2.f * q;
                }
            }
            term = (float)(-(double)b.gm[0] * fk / sqrt(dx * dx + dy * dy + (double)s2) +
                           (double)b.gm_ref * t.InvRmed_d[i]);
        } else {
            const float dx = (xh - b.xh[k]) + (xl - b.xl[k]);
            const float dy = (yh - b.yh[k]) + (yl - b.yl[k]);
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, s2));
            const float inv_d = rsqrtf(d2);
            float fk = 1.f;
            if (b.rsm[k] > 0.f) {
                const float dsm = d2 * inv_d;
                if (dsm < b.rsm[k]) {
                    const float q = dsm / b.rsm[k];
                    fk = q * q * q * q - 2.f * q * q * q + 2.f * q;
                }
            }
            term = -b.gm[k] * inv_d * fk;
        }
        acc += term;
    }
    acc = fmaf(-b.iy, yh + yl, fmaf(-b.ix, xh + xl, acc));
    pot[CELL(i, j)] = acc;
}

// ---------------------------------------------------------------------------
// momentum sources (SourceEuler.cpp:325-428) in residual form; rows 0..nr
// ---------------------------------------------------------------------------
__device__ __forceinline__ void source_cell(const GeoF &g, const TablesF &t, float dt,
                                            const float *__restrict__ S,
                                            const float *__restrict__ P,
                                            const float *__restrict__ pot,
                                            const float *__restrict__ vr_in,
                                            const float *__restrict__ dv_in,
                                            float *__restrict__ vr_out,
                                            float *__restrict__ dv_out, int i, int j)
{
    const int nz = g.nz, nr = g.nr;
    float vr = vr_in[CELL(i, j)];
    if (i >= 2 && i < nr - 1) {
        const float gradp = 2.f * __fdividef(P[CELL(i, j)] - P[CELL(i - 1, j)],
                                             S[CELL(i, j)] + S[CELL(i - 1, j)]) *
                            t.InvDiffRmed[i];
        const float gradphi = (pot[CELL(i, j)] - pot[CELL(i - 1, j)]) * t.InvDiffRmed[i];
        const int jn = jnext(j, nz);
        float d = 0.25f * (dv_in[CELL(i, j)] + dv_in[CELL(i, jn)] + dv_in[CELL(i - 1, j)] +
                           dv_in[CELL(i - 1, jn)]);
        // in a rotating frame the reference's vt (frame velocities averaged,
        // plus Rinf OmegaFrame; SourceEuler.cpp:355-364) is the inertial mean
        // plus OmegaFrame (Rinf - the mean of the two Rmed)
        if (g.omega_f != 0.f) d += g.omega_f * t.RinfOff[i];
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
__device__ __forceinline__ void artvisc_q_cell(const GeoF &g, const TablesF &t, const PhysF &ph,
                                               float dt, const float *__restrict__ S,
                                               const float *__restrict__ vr,
                                               const float *__restrict__ dv, float *__restrict__ E,
                                               float *__restrict__ Qr, float *__restrict__ Qp,
                                               int i, int j)
{
    const int nz = g.nz, nr = g.nr;
    const size_t c = CELL(i, j);
    const int jn = jnext(j, nz);
    const float vr0 = vr[c], vr1 = vr[CELL(i + 1, j)];
    const float dvp = dv[CELL(i, jn)] - dv[c];
    float e = 0.f;
    if (ph.adiabatic) {
        e = E[c];
        if (i < nr - 1) {
            // (vr1 Rinf[i+1] - vr0 Rinf[i]) / ((Rsup - Rinf) Rmed), regrouped
            // exactly (Rinf[i+1] = Rsup[i]) so that no product cancels
            const float div_v = (vr1 - vr0) * t.RsupIDRR[i] + vr0 * t.InvRmed[i] +
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
    if (ph.art_visc_tw) {
        // update_with_artificial_viscosity_TW, artificial_viscosity.cpp:52-91
        // (velocity differences within a ring are the same for the residual)
        const float sig = S[c];
        const float eps_rr = (vr1 - vr0) * t.InvDiffRsup[i];
        const float eps_pp = t.InvRmed[i] * (dvp * g.invdphi + 0.5f * (vr1 + vr0));
        const float div_V = fminf(eps_rr + eps_pp, 0.f);
        const float lsig = t.LSqTW[i] * sig;
        Qr[c] = lsig * -div_V * (eps_rr - (1.f / 3.f) * div_V);
        Qp[c] = lsig * -div_V * (eps_pp - (1.f / 3.f) * div_V);
        if (ph.adiabatic && ph.dissipation && i >= 1 && i < nr - 1) {
            const float d = eps_rr - eps_pp;
            e += -lsig * div_V * (1.f / 3.f) * (eps_rr * eps_rr + eps_pp * eps_pp + d * d) * dt;
        }
    }
    if (ph.adiabatic) {
        if (ph.dissipation) e = tfloor(e, S[c], ph);
        E[c] = e;
    }
}

__device__ __forceinline__ void artvisc_v_cell(const GeoF &g, const TablesF &t, const PhysF &ph,
                                               float dt, const float *__restrict__ S,
                                               const float *__restrict__ E,
                                               const float *__restrict__ Qr,
                                               const float *__restrict__ Qp, float *__restrict__ vr,
                                               float *__restrict__ dv, float *__restrict__ cs,
                                               float *__restrict__ H, float *__restrict__ nu, int i,
                                               int j)
{
    const int nz = g.nz, nr = g.nr;
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
    if (ph.art_visc_tw) {
        // artificial_viscosity.cpp:93-139
        if (i >= 1 && i < nr - 1) {
            const int jp = jprev(j, nz);
            dv[c] += __fdividef(dt, 0.5f * (S[c] + S[CELL(i, jp)])) * t.InvDxSrc[i] *
                     (Qp[c] - Qp[CELL(i, jp)]);
        }
        if (i >= 2 && i < nr - 1) {
            const size_t cm = CELL(i - 1, j);
            vr[c] += ph.rvf * __fdividef(dt, 0.5f * (S[c] + S[cm])) * t.TwoOverDRmed2[i] *
                     ((Qr[c] * t.Rmed[i] - Qr[cm] * t.Rmed[i - 1]) -
                      0.5f * (Qp[c] + Qp[cm]) * t.DRmed[i]);
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
__device__ __forceinline__ void stress_cell(const GeoF &g, const TablesF &t,
                                            const float *__restrict__ S,
                                            const float *__restrict__ vr,
                                            const float *__restrict__ dv,
                                            const float *__restrict__ nu, float *__restrict__ divv,
                                            float *__restrict__ trr, float *__restrict__ tpp,
                                            float *__restrict__ trp, int i, int j)
{
    const int nz = g.nz;
    const size_t c = CELL(i, j);
    const int jn = jnext(j, nz);
    const float vr0 = vr[c], vr1 = vr[CELL(i + 1, j)];
    const float dvp = dv[CELL(i, jn)] - dv[c];
    const float n = nu[c], sg = S[c];
    const float d = (vr1 - vr0) * t.RsupIDRR[i] + vr0 * t.InvRmed[i] +
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

// StabilizeViscosity's correction factors (viscosity.cpp:256-348), rows
// 1 .. nr - 1, from nu and sigma (nu sigma at the centres, the four-cell
// averages at the r-phi corners; row nr of the latter is zero)
__device__ __forceinline__ float nusig_rp_f(const float *nu, const float *S, int nz, int i, int j)
{
    const int jp = jprev(j, nz);
    const float n = 0.25f * (nu[CELL(i, j)] + nu[CELL(i - 1, j)] + nu[CELL(i, jp)] +
                             nu[CELL(i - 1, jp)]);
    const float s = 0.25f * (S[CELL(i, j)] + S[CELL(i - 1, j)] + S[CELL(i, jp)] +
                             S[CELL(i - 1, jp)]);
    return n * s;
}

__device__ __forceinline__ void visc_corr_cell(const GeoF &g, const TablesF &t,
                                               const float *__restrict__ S,
                                               const float *__restrict__ nu,
                                               float *__restrict__ corr_phi,
                                               float *__restrict__ corr_r, int i, int j)
{
    const int nz = g.nz, nr = g.nr;
    const size_t c = CELL(i, j);
    const int jp = jprev(j, nz), jn = jnext(j, nz);
    const float rp = nusig_rp_f(nu, S, nz, i, j);
    const float rp_ip = i + 1 < nr ? nusig_rp_f(nu, S, nz, i + 1, j) : 0.f;
    const float rp_jp = nusig_rp_f(nu, S, nz, i, jn);
    const float ns = nu[c] * S[c];
    const float ns_jm = nu[CELL(i, jp)] * S[CELL(i, jp)];
    const float ns_im = nu[CELL(i - 1, j)] * S[CELL(i - 1, j)];
    const float cphi_rp = -t.InvRmed[i] * t.TwoOverDRa2[i] *
                          (rp_ip * t.Ra3IDRmed[i + 1] + rp * t.Ra3IDRmed[i]);
    const float cphi_pp = -t.F43[i] * (ns + ns_jm);
    corr_phi[c] = (cphi_rp + cphi_pp) / (0.5f * (S[c] + S[CELL(i, jp)]) * t.Rmed[i]);
    const float cr_rp = -(rp_jp + rp) * t.CrRp[i];
    const float cr_pp = -0.5f * (ns * t.CrPp1[i] + ns_im * t.CrPp2[i]);
    const float cr_rr = t.InvDiffRmed[i] * (ns * t.CrRr1[i] + ns_im * t.CrRr2[i]);
    corr_r[c] = t.CrScale[i] * (cr_rr + cr_rp + cr_pp) / (0.5f * (S[c] + S[CELL(i - 1, j)]));
}

// viscous velocity update + SubStep3.  mode bits: 1 velocities
// (viscosity.cpp:355-421), 2 heating/cooling rates, 4 energy update
// (SourceEuler.cpp:859-954)
__device__ __forceinline__ void viscous_cell(
    const GeoF &g, const TablesF &t, const PhysF &ph, float dt, float beta_inv, int mode,
    const float *__restrict__ S, const float *__restrict__ trr, const float *__restrict__ tpp,
    const float *__restrict__ trp, const float *__restrict__ divv, const float *__restrict__ nu,
    const float *__restrict__ H, const float *__restrict__ S0, const float *__restrict__ E0,
    float *__restrict__ vr, float *__restrict__ dv, float *__restrict__ E,
    float *__restrict__ qplus, float *__restrict__ qminus, const float *__restrict__ corr_phi,
    const float *__restrict__ corr_r, int i, int j)
{
    const int nz = g.nz, nr = g.nr;
    const size_t c = CELL(i, j);
    const int jp = jprev(j, nz), jn = jnext(j, nz);
    // pseudo-implicit limiter of StabilizeViscosity 1, viscosity.cpp:395-399
    auto stabilized = [&](float d, float cc) {
        const float a = 1.f + dt * cc;
        return d * (1.f / (fmaxf(a, 0.f) - dt * cc));
    };
    if (mode & 1) {
        if (i >= 1 && i < nr - 1) {
            const float sa = 0.5f * (S[c] + S[CELL(i, jp)]);
            const float fac = __fdividef(dt * t.InvRmed[i], sa);
            const float rhs = t.TwoOverDRa2[i] * (t.RinfSq[i + 1] * trp[CELL(i + 1, j)] -
                                                  t.RinfSq[i] * trp[c]) +
                              (tpp[c] - tpp[CELL(i, jp)]) * g.invdphi;
            // the fused form is spelled out so that every kernel built from
            // this body rounds the update the same way
            if (ph.stabilize == 1)
                dv[c] += stabilized(fac * rhs, corr_phi[c]);
            else
                dv[c] = fmaf(fac, rhs, dv[c]);
        }
        if (i >= 2 && i < nr - 1) {
            const float sa = 0.5f * (S[c] + S[CELL(i - 1, j)]);
            const float fac = __fdividef(dt, sa) * ph.rvf * t.TwoOverRmedSum[i];
            const float rhs =
                (t.Rmed[i] * trr[c] - t.Rmed[i - 1] * trr[CELL(i - 1, j)]) * t.InvDiffRmed[i] +
                (trp[CELL(i, jn)] - trp[c]) * g.invdphi - 0.5f * (tpp[c] + tpp[CELL(i - 1, j)]);
            if (ph.stabilize == 1)
                vr[c] += stabilized(fac * rhs, corr_r[c]);
            else
                vr[c] = fmaf(fac, rhs, vr[c]);
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
__device__ __forceinline__ void ghost_f(float *x, const float *x0, int kind, int outer, int vec,
                                        int nr, int nz, int j, float kep_value, float zg_offset,
                                        const float *val, const float *nu)
{
    const int irad = vec ? nr : nr - 1;
    const int edge = outer ? irad : 0;
    const int next = outer ? irad - 1 : 1;
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
        x[CELL(edge, j)] = x0[CELL(edge, j)];
        if (vec) x[CELL(next, j)] = x0[CELL(next, j)];
        break;
    case 4:
        x[CELL(edge, j)] = kep_value;
        break;
    case 5:   // disk model
    case 10:  // balanced (residual)
        x[CELL(edge, j)] = val[0];
        break;
    case 6:  // reflecting
        x[CELL(edge, j)] = -x[CELL(outer ? irad - 2 : 2, j)];
        x[CELL(next, j)] = 0.f;
        break;
    case 7: {  // viscous outflow (inner edge)
        const float Nu = 0.5f * (nu[CELL(0, j)] + nu[CELL(1, j)]);
        x[CELL(1, j)] = val[1] * Nu;
        x[CELL(0, j)] = val[0] * Nu;
        break;
    }
    case 8:  // Keplerian radial
        x[CELL(edge, j)] = val[0];
        x[CELL(next, j)] = val[1];
        break;
    case 9:  // zero shear on the residual: ratio * dv_active + offset
        x[CELL(edge, j)] = fmaf(val[0], x[CELL(next, j)], val[1]);
        break;
    default:
        break;
    }
}

__device__ __forceinline__ void ghost_col(const GeoF &g, const BcF &bc, const StateF &s, int j)
{
    const int nz = g.nz, nr = g.nr;
    ghost_f(s.sigma, s.sigma0, bc.sigma_in, 0, 0, nr, nz, j, 0.f, 0.f, bc.val_in[0], bc.nu);
    ghost_f(s.sigma, s.sigma0, bc.sigma_out, 1, 0, nr, nz, j, 0.f, 0.f, bc.val_out[0], bc.nu);
    // low part of sigma: copied by zero-gradient, cleared by reference hooks,
    // the disk model's own low part
    if (bc.sigma_in == 1) s.sigma_lo[CELL(0, j)] = s.sigma_lo[CELL(1, j)];
    else if (bc.sigma_in == 3) s.sigma_lo[CELL(0, j)] = 0.f;
    else if (bc.sigma_in == 5) s.sigma_lo[CELL(0, j)] = bc.val_in[0][1];
    if (bc.sigma_out == 1) s.sigma_lo[CELL(nr - 1, j)] = s.sigma_lo[CELL(nr - 2, j)];
    else if (bc.sigma_out == 3) s.sigma_lo[CELL(nr - 1, j)] = 0.f;
    else if (bc.sigma_out == 5) s.sigma_lo[CELL(nr - 1, j)] = bc.val_out[0][1];
    ghost_f(s.energy, s.energy0, bc.energy_in, 0, 0, nr, nz, j, 0.f, 0.f, bc.val_in[1], bc.nu);
    ghost_f(s.energy, s.energy0, bc.energy_out, 1, 0, nr, nz, j, 0.f, 0.f, bc.val_out[1], bc.nu);
    ghost_f(s.vr, s.vr0, bc.vr_in, 0, 1, nr, nz, j, 0.f, 0.f, bc.val_in[2], bc.nu);
    ghost_f(s.vr, s.vr0, bc.vr_out, 1, 1, nr, nz, j, 0.f, 0.f, bc.val_out[2], bc.nu);
    ghost_f(s.dv, s.dv0, bc.vaz_in, 0, 0, nr, nz, j, bc.kep_in, bc.zg_in, bc.val_in[3], bc.nu);
    ghost_f(s.dv, s.dv0, bc.vaz_out, 1, 0, nr, nz, j, bc.kep_out, bc.zg_out, bc.val_out[3],
            bc.nu);
}

// ---------------------------------------------------------------------------
// radial transport (TransportEuler.cpp:138-167, 349-406, 545-620) with the
// residual angular momentum: quantities 0,1 radial momenta, 2,3 residual
// angular momenta sigma r dv, [4 energy], last sigma.  The angular-momentum
// slopes and the limiter act on the total specific angular momentum
// J_K + r dv (J_K = r v_K per ring), the upwind star value is kept relative to
// J_K of the upwind ring, and the Keplerian part J_K * mass-flux enters the
// residual update through the per-ring differences of J_K.  One thread walks
// column j through rings i0 .. i0 + chunk - 1 with a rolling window.
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
__device__ __forceinline__ void radial_col(const GeoF &g, const TablesF &t, float dt, int mc,
                                           int chunk, const float *__restrict__ S,
                                           const float *__restrict__ vr,
                                           const float *__restrict__ dv,
                                           const float *__restrict__ E, float *__restrict__ m0,
                                           float *__restrict__ m1, float *__restrict__ m2,
                                           float *__restrict__ m3, float *__restrict__ E_out,
                                           float *__restrict__ S_out,
                                           const float *__restrict__ S_lo,
                                           float *__restrict__ S_lo_out, int i0, int j)
{
    constexpr int NW = NQ + 1;
    const int nz = g.nz, nr = g.nr;
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
    float flux_prev[NW] = {};
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
            // ring k-1's update; its conserved values are formed here from
            // its specific values (wa, the products rounded as stored
            // values) and its energy re-read, so that the walk carries none
            // of them
            const int i = k - 1;
            const float invs = t.InvSurf[i];
            const size_t c = CELL(i, j);
            const float sa = wa[NQ];
            m0[c] = __fmul_rn(sa, wa[0]) + (flux_prev[0] - flux[0]) * invs;
            m1[c] = __fmul_rn(sa, wa[1]) + (flux_prev[1] - flux[1]) * invs;
            m2[c] = __fmul_rn(sa, wa[2]) + (flux_prev[2] + kep_prev - flux[2] - kep_lower) * invs;
            m3[c] = __fmul_rn(sa, wa[3]) + (flux_prev[3] + kep_prev - flux[3] - kep_lower) * invs;
            if (NQ == 5) E_out[c] = E[c] + (flux_prev[4] - flux[4]) * invs;
            float hi = sa, lo = S_lo[c];
            comp_add(hi, lo, (flux_prev[NQ] - flux[NQ]) * invs);
            S_out[c] = hi;
            S_lo_out[c] = lo;
        }
        if (k < i1) {
#pragma unroll
            for (int q = 0; q < NW; ++q) flux_prev[q] = flux[q];
            kep_prev = kep_upper;
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
// a ring, so its part cancels exactly).  One block per ring; thread tid owns
// cells tid + n * blockDim.x, n < PER, which must cover the ring.  Each
// quantity takes three barriers: specific values, slopes, fluxes (a separate
// flux array lets the update read them while the next quantity starts).
// ---------------------------------------------------------------------------
template <int PER, int NQ>
__device__ __forceinline__ void ring_pass_f(float *S, float *W, float *D, float *F, float *X,
                                            float *const *qrow, const float *v, float *slo,
                                            float dt, float dxtheta, float half_invdx,
                                            float dxrad_invsurf, int nz, int mc)
{
    const int tid = threadIdx.x, bs = blockDim.x;
    // per face: 1 / sigma of the cell and dxrad S* v / Surf, the factor every
    // quantity's flux shares; kept in the X array up to 4 cells per thread
    // (short rings, shared memory to spare) and in registers beyond
    constexpr bool XS = PER <= 4;
    float invs[PER], cfr[XS ? 1 : PER];
    auto cf = [&](int n, int j) -> float & { return XS ? X[j] : cfr[n]; };
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
            D[j] = __fmul_rn(lim_f(__fsub_rn(S[jp], S[j]), __fsub_rn(S[j], S[jm]), mc), half_invdx);
            invs[n] = __frcp_rn(S[j]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jm = j == 0 ? nz - 1 : j - 1;
            const float vv = v[n];
            const float ksi = __fmul_rn(vv, dt);
            const float ss = ksi > 0.f ? star_pos(S[jm], D[jm], dxtheta, ksi)
                                       : star_neg(S[j], D[j], dxtheta, ksi);
            cf(n, j) = __fmul_rn(__fmul_rn(dxrad_invsurf, ss), vv);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        float *Q = qrow[q];
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) W[j] = __fmul_rn(Q[j], invs[n]);
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
                D[j] = __fmul_rn(lim_f(__fsub_rn(W[jp], W[j]), __fsub_rn(W[j], W[jm]), mc), half_invdx);
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                const int jm = j == 0 ? nz - 1 : j - 1;
                const float ksi = __fmul_rn(v[n], dt);
                const float qs = ksi > 0.f ? star_pos(W[jm], D[jm], dxtheta, ksi)
                                           : star_neg(W[j], D[j], dxtheta, ksi);
                F[j] = __fmul_rn(qs, cf(n, j));
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) Q[j] = __fadd_rn(Q[j], __fsub_rn(F[j], F[j == nz - 1 ? 0 : j + 1]));
        }
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) F[j] = cf(n, j);
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            float sn = S[j];
            comp_add(sn, slo[n], F[j] - F[j == nz - 1 ? 0 : j + 1]);
            S[j] = sn;
        }
    }
    __syncthreads();
}

// The uniform pass of FARGO (QuantitiesAdvection with the ring's residual
// shift velocity, TransportEuler.cpp:292-304) in difference form.  The whole
// ring has one upwind direction, so with u the upwind cell of face j
// (j - 1 for a positive shift, j otherwise) and a the interpolation distance
// (dx - ksi, or -(dx + ksi)), face j's star value is X_u + a D_u and cell j
// changes by dxrad v invsurf (q*_j S*_j - q*_{j+1} S*_{j+1})
//   = dxrad v invsurf (q*_j dS*_j + S*_{j+1} dq*_j),
//   dS*_j = (S_u - S_{u+1}) + a (D_u - D_{u+1}),  dq*_j likewise.
// This is the flux form's arithmetic regrouped: forming the neighbour
// differences first keeps FP32's rounding at the size of the changes, where
// the flux form rounds at the size of the fluxes, up to half of the ring's
// content per step, and repeats the same rounding pattern every step.
// dS* goes to the X array (up to 4 cells per thread) or registers, S*_{j+1}
// to the F array; c is dxrad v invsurf and a the interpolation distance.
template <int PER, int NQ>
__device__ __forceinline__ void ring_pass_uniform_f(float *S, float *W, float *D, float *F,
                                                    float *X, float *const *qrow, float *slo,
                                                    bool pos, float a, float c, float half_invdx,
                                                    int nz, int mc)
{
    const int tid = threadIdx.x, bs = blockDim.x;
    constexpr bool XS = PER <= 4;
    float invs[PER], dssr[XS ? 1 : PER];
    auto dss = [&](int n, int j) -> float & { return XS ? X[j] : dssr[n]; };
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
            D[j] = __fmul_rn(lim_f(__fsub_rn(S[jp], S[j]), __fsub_rn(S[j], S[jm]), mc), half_invdx);
            invs[n] = __frcp_rn(S[j]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
            const int u = pos ? jm : j, u1 = pos ? j : jp;
            dss(n, j) = star_diff(S[u], S[u1], D[u], D[u1], a);
            F[j] = star_at(S[u1], D[u1], a);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        float *Q = qrow[q];
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) W[j] = __fmul_rn(Q[j], invs[n]);
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
                D[j] = __fmul_rn(lim_f(__fsub_rn(W[jp], W[j]), __fsub_rn(W[j], W[jm]), mc), half_invdx);
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                const int jp = j == nz - 1 ? 0 : j + 1, jm = j == 0 ? nz - 1 : j - 1;
                const int u = pos ? jm : j, u1 = pos ? j : jp;
                const float qs = star_at(W[u], D[u], a);
                const float dqs = star_diff(W[u], W[u1], D[u], D[u1], a);
                Q[j] = uniform_update(Q[j], c, qs, dss(n, j), F[j], dqs);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            float sn = S[j];
            comp_add(sn, slo[n], __fmul_rn(c, dss(n, j)));
            S[j] = sn;
        }
    }
    __syncthreads();
}

// Shared memory of azimuthal_ring: ring-long work arrays for sigma, the
// specific quantity, its slope and the flux, a fifth for the per-face factors
// on rings up to 2048 cells (where at most 4 cells per thread leave no
// registers for them), plus the nq quantity rows when STAGE (then every row
// is read from HBM once, up front, the passes work in shared memory and the
// rows go back once at the end).
__host__ __device__ constexpr int azimuthal_work_rows(int nz) { return nz <= 2048 ? 5 : 4; }
__host__ __device__ constexpr size_t azimuthal_smem_floats(int nz, int nq, bool stage)
{
    return (size_t)(azimuthal_work_rows(nz) + (stage ? nq : 0)) * (size_t)nz;
}

// smf: azimuthal_smem_floats(nz, nq, STAGE) floats of shared memory; redf: 33
// floats, redl: 33 long longs (shared memory)
template <int PER, int NQ, bool STAGE>
__device__ __forceinline__ void azimuthal_ring(const GeoF &g, const TablesF &t, double dt, int mc,
                                               int fast, const float *__restrict__ dv,
                                               float *m0, float *m1, float *m2, float *m3,
                                               float *E, float *S, float *S_lo, int i, float *smf,
                                               float *redf, long long *redl, int *ring_shift)
{
    const int nz = g.nz;
    const int tid = threadIdx.x, bs = blockDim.x;
    const size_t row = (size_t)i * nz;
    float *Sr = smf, *W = smf + nz, *D = smf + 2 * nz, *Fx = smf + 3 * nz;
    // the per-face array exists when PER <= 4, which needs nz <= 4 x 512
    float *X = smf + 4 * nz;
    const int wr = azimuthal_work_rows(nz);
    float *grow[5] = {m0 + row, m1 + row, m2 + row, m3 + row, E + row};
    float *qrow[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) qrow[q] = STAGE ? smf + (size_t)(wr + q) * nz : grow[q];

    float vown[PER], slo[PER];
    float amax = 0.f;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            vown[n] = dv[row + j];
            amax = fmaxf(amax, fabsf(vown[n]));
            Sr[j] = S[row + j];
            slo[n] = S_lo[row + j];
            if (STAGE) {
#pragma unroll
                for (int q = 0; q < NQ; ++q) qrow[q][j] = grow[q][j];
            }
        }
    }
    // ring mean of v_phi, independent of the block's shape, and the FARGO
    // shift phase in FP64 (:174-236)
    const int ks = exact_sum_scale(amax, nz, redf);
    long long part = 0;
#pragma unroll
    for (int n = 0; n < PER; ++n)
        if (tid + n * bs < nz) part += to_fixed(vown[n], ks);
    const double mean_dv = exact_sum_result(part, ks, redl) / (double)nz;
    // the ring's mean frame velocity (the residual is about the inertial
    // Keplerian speed)
    const double vmean = (t.Vref_d[i] - t.Rmed_d[i] * g.omega_frame) + mean_dv;
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
        }
    }
    const float dxtheta = g.dphi * t.Rmed[i];
    const float half_invdx = 0.5f / dxtheta;
    const float dxrad = t.DRsup[i] * (float)dt;
    const float invsurf = t.InvSurf[i];
    ring_pass_f<PER, NQ>(Sr, W, D, Fx, X, qrow, vown, slo, (float)dt, dxtheta, half_invdx,
                         dxrad * invsurf, nz, mc);
    if (fast) {
        const float ksi = vt * (float)dt;
        const bool pos = ksi > 0.f;
        ring_pass_uniform_f<PER, NQ>(Sr, W, D, Fx, X, qrow, slo, pos,
                                     pos ? dxtheta - ksi : -(dxtheta + ksi),
                                     dxrad * vt * invsurf, half_invdx, nz, mc);
    }
    // AdvectSHIFT (:238-268) is the velocity rebuild's: it reads cell j of
    // this ring from cell j - nshift, so the rows go back unshifted (the
    // quantities are already in place unless staged)
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            S[row + j] = Sr[j];
            S_lo[row + j] = slo[n];
        }
    }
    if (STAGE) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
#pragma unroll
            for (int n = 0; n < PER; ++n) {
                const int j = tid + n * bs;
                if (j < nz) grow[q][j] = qrow[q][j];
            }
        }
    }
    if (tid == 0) ring_shift[i] = ((nshift % nz) + nz) % nz;
    // the caller may reuse smf for the next ring
    __syncthreads();
}

// ---------------------------------------------------------------------------
// The same ring transport with the ring in registers: thread tid owns the
// contiguous cells j0 = tid PER .. j0 + PER - 1 (nz = PER blockDim.x, PER a
// multiple of 4), loads and stores them as 128-bit words, and computes every
// stencil from registers.  The only cross-thread step per transported
// quantity is one exchange of segment ends: each thread publishes its first
// two and last two values, and after one barrier reads the two cells left of
// its segment and the two right of it; with them it forms the slopes of
// cells j0 - 1 .. j0 + PER and the fluxes of faces j0 .. j0 + PER itself, so
// no slope or flux crosses threads.  The exchange area is double-buffered:
// a thread writing buffer b for the next exchange has passed the barrier of
// the exchange in between, which every thread reaches only after reading
// buffer b, so no write overtakes a read.  Every cell's arithmetic is the
// strided kernel's (ring_pass_f, ring_pass_uniform_f, the exact-sum ring mean,
// the shift phase), expression for expression, so both give the same bits.
//
// Shared memory (rb_smem_floats): the NQ transported rows between the two
// passes (staged coalesced from HBM; the last pass writes each segment back
// to its row in place, the integer shift being the velocity rebuild's) and
// 2 x 5 x blockDim.x floats for the exchanges.
// ---------------------------------------------------------------------------
// threads per ring block of the register-blocked kernel: 16 cells per thread
// need more registers than 128 (the budget at 512 threads)
__host__ __device__ constexpr int rb_max_threads(int per) { return per >= 16 ? 384 : 512; }
__host__ __device__ constexpr size_t rb_smem_floats(int nz, int nq, int threads)
{
    return (size_t)nq * (size_t)nz + (size_t)10 * (size_t)threads;
}
// whether a ring of nz cells splits into segments of per cells with between
// min_threads and the kernel's bound of threads, within max_smem bytes
__host__ __device__ inline bool rb_fits(int nz, int nq, int per, int min_threads, size_t max_smem)
{
    if (nz % per != 0) return false;
    const int th = nz / per;
    return th >= min_threads && th <= rb_max_threads(per) &&
           rb_smem_floats(nz, nq, th) * sizeof(float) <= max_smem;
}
// The segment length the register-blocked pass takes for a ring of nz cells
// (0: the strided pass): 12 cells per thread where that leaves at least 128
// threads, else the shortest of 4, 8, 16 that leaves at least 32.  Measured
// FP32 steps: 6144-cell rings 2.34 ms with 12 cells (16: 2.54, strided 2.66),
// 3072: 0.569 ms (8: 0.597, 16: 0.601, strided 0.664), 1536: 0.269 ms
// (8: 0.275, 4: 0.283, strided 0.275), 384: 0.127 ms with 4 (8: 0.139,
// 12: 0.152, strided 0.137).
__host__ inline int rb_default_per(int nz, int nq, size_t max_smem)
{
    if (rb_fits(nz, nq, 12, 128, max_smem)) return 12;
    for (int per : {4, 8, 16})
        if (rb_fits(nz, nq, per, 32, max_smem)) return per;
    return 0;
}

template <int PER, int NQ>
__device__ __forceinline__ void azimuthal_ring_rb(const GeoF &g, const TablesF &t, double dt,
                                                  int mc, int fast, const float *__restrict__ dv,
                                                  float *m0, float *m1, float *m2, float *m3,
                                                  float *E, float *S, float *S_lo, int i,
                                                  float *smf, float *redf, long long *redl,
                                                  int *ring_shift)
{
    static_assert(PER % 4 == 0 && PER >= 4, "segments of whole 128-bit words");
    const int nz = g.nz;  // == PER * blockDim.x
    const int tid = threadIdx.x, bs = blockDim.x;
    const size_t row = (size_t)i * nz;
    const int j0 = tid * PER;
    const int left = tid == 0 ? bs - 1 : tid - 1, right = tid == bs - 1 ? 0 : tid + 1;
    float *qsm = smf;                               // NQ rows
    float *xs = smf + (size_t)NQ * nz;              // [2][5][bs]
    float *grow[5] = {m0 + row, m1 + row, m2 + row, m3 + row, E + row};
    int buf = 0;
    // publishes a0, a1 (first two), a2, a3 (last two) and a4; returns the
    // left neighbour's last two (l2, l3), the right neighbour's first two
    // (r0, r1) and its a4 (r4)
    auto exchange = [&](float a0, float a1, float a2, float a3, float a4, float &l2, float &l3,
                        float &r0, float &r1, float &r4) {
        float *x = xs + (size_t)buf * 5 * bs;
        x[tid] = a0;
        x[bs + tid] = a1;
        x[2 * bs + tid] = a2;
        x[3 * bs + tid] = a3;
        x[4 * bs + tid] = a4;
        __syncthreads();
        l2 = x[2 * bs + left];
        l3 = x[3 * bs + left];
        r0 = x[right];
        r1 = x[bs + right];
        r4 = x[4 * bs + right];
        buf ^= 1;
    };
    auto load_seg = [&](const float *src, float *dst) {
#pragma unroll
        for (int k = 0; k < PER / 4; ++k) {
            const float4 w = reinterpret_cast<const float4 *>(src + j0)[k];
            dst[4 * k] = w.x;
            dst[4 * k + 1] = w.y;
            dst[4 * k + 2] = w.z;
            dst[4 * k + 3] = w.w;
        }
    };
    auto store_seg = [&](float *dst, const float *src) {
#pragma unroll
        for (int k = 0; k < PER / 4; ++k)
            reinterpret_cast<float4 *>(dst + j0)[k] =
                make_float4(src[4 * k], src[4 * k + 1], src[4 * k + 2], src[4 * k + 3]);
    };

    // the transported rows into shared memory (coalesced), the own segment of
    // v_phi and of the sigma pair into registers
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        for (int j = tid; j < nz; j += bs) qsm[(size_t)q * nz + j] = grow[q][j];
    float v[PER + 1], s[PER], slo[PER];
    load_seg(dv + row, v);
    load_seg(S + row, s);
    load_seg(S_lo + row, slo);
    float amax = 0.f;
#pragma unroll
    for (int n = 0; n < PER; ++n) amax = fmaxf(amax, fabsf(v[n]));
    // ring mean of v_phi (exact integer sum: the same bits for any ownership)
    // and the FARGO shift phase in FP64 (:174-236)
    const int ks = exact_sum_scale(amax, nz, redf);
    long long part = 0;
#pragma unroll
    for (int n = 0; n < PER; ++n) part += to_fixed(v[n], ks);
    const double mean_dv = exact_sum_result(part, ks, redl) / (double)nz;
    const double vmean = (t.Vref_d[i] - t.Rmed_d[i] * g.omega_frame) + mean_dv;
    const double Ntilde = vmean * t.InvRmed_d[i] * dt * g.invdphi_d;
    const double Nround = floor(Ntilde + 0.5);
    const int nshift = (int)Nround;
    const float vt = (float)((Ntilde - Nround) * t.Rmed_d[i] * (1.0 / dt) * g.dphi_d);
    const float mdv = (float)mean_dv;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        float vres = v[n] - mdv;
        if (!fast) vres = vt + vres;
        v[n] = vres;
    }
    const float dxtheta = g.dphi * t.Rmed[i];
    const float half_invdx = 0.5f / dxtheta;
    const float dxrad = t.DRsup[i] * (float)dt;
    const float invsurf = t.InvSurf[i];
    const float fdt = (float)dt;
    const float dxrad_invsurf = dxrad * invsurf;
    __syncthreads();  // the staged rows are complete

    // values of cells j0 - 2 .. j0 + PER + 1 at index c + 2; slopes of cells
    // j0 - 1 .. j0 + PER at index c + 1
    float X[PER + 4], D[PER + 2], invs[PER];
    auto slopes = [&]() {
#pragma unroll
        for (int c = -1; c <= PER; ++c)
            D[c + 1] = __fmul_rn(lim_f(__fsub_rn(X[c + 3], X[c + 2]), __fsub_rn(X[c + 2], X[c + 1]), mc),
                                 half_invdx);
    };
    auto sigma_ends = [&](float a4, float &r4) {
        float l2, l3, r0, r1;
        exchange(s[0], s[1], s[PER - 2], s[PER - 1], a4, l2, l3, r0, r1, r4);
        X[0] = l2;
        X[1] = l3;
#pragma unroll
        for (int n = 0; n < PER; ++n) X[n + 2] = s[n];
        X[PER + 2] = r0;
        X[PER + 3] = r1;
    };
    auto specific = [&](const float *q) {
#pragma unroll
        for (int n = 0; n < PER; ++n) X[n + 2] = __fmul_rn(q[n], invs[n]);
        float l2, l3, r0, r1, r4;
        exchange(X[2], X[3], X[PER], X[PER + 1], 0.f, l2, l3, r0, r1, r4);
        X[0] = l2;
        X[1] = l3;
        X[PER + 2] = r0;
        X[PER + 3] = r1;
    };

    // QuantitiesAdvection with the residual velocity (ring_pass_f)
    {
        float cf[PER + 1];
        sigma_ends(v[0], v[PER]);  // face j0 + PER takes the right neighbour's velocity
        slopes();
#pragma unroll
        for (int n = 0; n < PER; ++n) invs[n] = __frcp_rn(s[n]);
#pragma unroll
        for (int f = 0; f <= PER; ++f) {
            const float vv = v[f];
            const float ksi = __fmul_rn(vv, fdt);
            const float ss = ksi > 0.f ? star_pos(X[f + 1], D[f], dxtheta, ksi)
                                       : star_neg(X[f + 2], D[f + 1], dxtheta, ksi);
            cf[f] = __fmul_rn(__fmul_rn(dxrad_invsurf, ss), vv);
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float qv[PER];
            load_seg(qsm + (size_t)q * nz, qv);
            specific(qv);
            slopes();
            float F[PER + 1];
#pragma unroll
            for (int f = 0; f <= PER; ++f) {
                const float ksi = __fmul_rn(v[f], fdt);
                const float qs = ksi > 0.f ? star_pos(X[f + 1], D[f], dxtheta, ksi)
                                           : star_neg(X[f + 2], D[f + 1], dxtheta, ksi);
                F[f] = __fmul_rn(qs, cf[f]);
            }
#pragma unroll
            for (int n = 0; n < PER; ++n) qv[n] = __fadd_rn(qv[n], __fsub_rn(F[n], F[n + 1]));
            // the last pass writes the segment back to its row in place
            store_seg(fast ? qsm + (size_t)q * nz : grow[q], qv);
        }
#pragma unroll
        for (int n = 0; n < PER; ++n) comp_add(s[n], slo[n], cf[n] - cf[n + 1]);
    }
    // the uniform pass in difference form (ring_pass_uniform_f)
    if (fast) {
        const float ksi = vt * fdt;
        const bool pos = ksi > 0.f;
        const float a = pos ? dxtheta - ksi : -(dxtheta + ksi);
        const float c = dxrad * vt * invsurf;
        float dss[PER], Fs[PER];
        float unused;
        sigma_ends(0.f, unused);
        slopes();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            invs[n] = __frcp_rn(s[n]);
            // cells u (upwind of face j) and u1 (of face j + 1): n - 1 and n
            // for a positive shift, n and n + 1 otherwise (X index + 2, D
            // index + 1); both candidates are read and one is selected, so
            // the arrays stay in registers
            const float xu = pos ? X[n + 1] : X[n + 2], xu1 = pos ? X[n + 2] : X[n + 3];
            const float du = pos ? D[n] : D[n + 1], du1 = pos ? D[n + 1] : D[n + 2];
            dss[n] = star_diff(xu, xu1, du, du1, a);
            Fs[n] = star_at(xu1, du1, a);
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float qv[PER];
            load_seg(qsm + (size_t)q * nz, qv);
            specific(qv);
            slopes();
#pragma unroll
            for (int n = 0; n < PER; ++n) {
                const float xu = pos ? X[n + 1] : X[n + 2], xu1 = pos ? X[n + 2] : X[n + 3];
                const float du = pos ? D[n] : D[n + 1], du1 = pos ? D[n + 1] : D[n + 2];
                const float qs = star_at(xu, du, a);
                const float dqs = star_diff(xu, xu1, du, du1, a);
                qv[n] = uniform_update(qv[n], c, qs, dss[n], Fs[n], dqs);
            }
            store_seg(grow[q], qv);
        }
#pragma unroll
        for (int n = 0; n < PER; ++n) comp_add(s[n], slo[n], __fmul_rn(c, dss[n]));
    }

    // AdvectSHIFT (:238-268) is the velocity rebuild's: it reads cell j of
    // this ring from cell j - nshift; the last pass wrote the quantities'
    // segments in place, sigma and its low part follow
    store_seg(S + row, s);
    store_seg(S_lo + row, slo);
    if (tid == 0) ring_shift[i] = ((nshift % nz) + nz) % nz;
    // the caller may reuse smf for the next ring
    __syncthreads();
}

// compute_pressure (SourceEuler.cpp:1345-1376): P alone
__device__ __forceinline__ void pressure_cell(const GeoF &g, const TablesF &t, const PhysF &ph,
                                              const float *__restrict__ S,
                                              const float *__restrict__ E, float *__restrict__ P,
                                              int i, int j)
{
    const int nz = g.nz;
    const size_t c = CELL(i, j);
    if (ph.adiabatic) {
        P[c] = ph.gm1 * E[c];
    } else {
        const float c_s = t.CsIso[i];
        P[c] = S[c] * (c_s * c_s);
    }
}

// velocities from momenta (:498-535), floors; rows 0..nr
__device__ __forceinline__ void finish_cell(
    const GeoF &g, const TablesF &t, const PhysF &ph, const float *__restrict__ m0,
    const float *__restrict__ m1, const float *__restrict__ m2, const float *__restrict__ m3,
    const float *__restrict__ S_t, const float *__restrict__ E_t, const float *__restrict__ vr_in,
    float *__restrict__ vr_out, float *__restrict__ dv_out, float *__restrict__ S_out,
    float *__restrict__ E_out, const float *__restrict__ Slo_t, float *__restrict__ Slo_out,
    const int *__restrict__ shift, int i, int j)
{
    const int nz = g.nz, nr = g.nr;
    const size_t c = CELL(i, j);
    if (i == nr) {
        vr_out[c] = vr_in[c];
        return;
    }
    // AdvectSHIFT: the transported cell j of ring k sits at j - shift[k]
    auto at = [&](int k, int jj) {
        int a = jj - __ldg(shift + k);
        if (a < 0) a += nz;
        return CELL(k, a);
    };
    const size_t cs = at(i, j);
    const float s = S_t[cs];
    if (i == 0) {
        vr_out[c] = 0.f;
    } else {
        const size_t cm = at(i - 1, j);
        vr_out[c] = __fdiv_rn(m0[cm] + m1[cs], S_t[cm] + s);
    }
    const size_t cjm = at(i, jprev(j, nz));
    // the residual angular momenta were formed as sigma (dv Rmed) with the
    // FP32 Rmed of the ring: dividing by that same Rmed returns dv without
    // bias, where multiplying by the FP32 1/Rmed would scale every ring's
    // residual by Rmed 1/Rmed - 1 (up to ~6e-8) in every step, a drift that
    // accumulates over tens of thousands of steps; the divisions are
    // correctly rounded for the same reason
    dv_out[c] = __fdiv_rn(m2[cjm] + m3[cs], __fmul_rn(S_t[cjm] + s, t.Rmed[i]));
    const bool floored = s < ph.sigma_min;
    const float sf = floored ? ph.sigma_min : s;
    S_out[c] = sf;
    Slo_out[c] = floored ? 0.f : Slo_t[cs];
    if (ph.adiabatic) E_out[c] = tfloor(E_t[cs], sf, ph);
}

// damping zones (damping.cpp:311-776); block-wide over ring i
// red: 33 floats, redl: 33 long longs (shared memory)
__device__ __forceinline__ void damp_ring_f(float *X, float *X0, const DampQF &d, int i, int nz,
                                            int outer, float dt, float *red, float *Xlo,
                                            long long *redl)
{
    const int kind = outer ? d.kind_out : d.kind_in;
    const size_t row = (size_t)i * nz;
    float x0c = 0.f;
    if (kind == 3) {
        const float mean = exact_row_mean(X + row, nz, red, redl);
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

// fields q0 .. q1 - 1 of ring i (0 v_r, 1 v_phi residual, 2 sigma, 3 energy:
// independent of one another)
__device__ __forceinline__ void damping_ring(const GeoF &g, const DampingF &dm, float dt,
                                             const StateF &s, int i, float *red, long long *redl,
                                             int q0 = 0, int q1 = 4)
{
    const int nz = g.nz, nr = g.nr;
    float *X[4] = {s.vr, s.dv, s.sigma, s.energy};
    float *X0[4] = {s.vr0, s.dv0, s.sigma0, s.energy0};
    for (int q = q0; q < q1; ++q) {
        const DampQF &d = dm.q[q];
        const int size = d.vector ? nr + 1 : nr;
        float *lo = q == 2 ? s.sigma_lo : nullptr;
        if (d.kind_in != 0 && d.active_in && i <= d.limit_in)
            damp_ring_f(X[q], X0[q], d, i, nz, 0, dt, red, lo, redl);
        if (d.kind_out != 0 && d.active_out && i >= d.limit_out && i < size)
            damp_ring_f(X[q], X0[q], d, i, nz, 1, dt, red, lo, redl);
    }
}

// derived quantities + CFL (SourceEuler.cpp:225-249, cfl.cpp:185-382); block-
// wide over ring i.  mode bits: 1 derived quantities, 2 also c_s, H, T of the
// isothermal disk, 4 CFL minimum into dt_min (float bits, atomicMin)
__device__ __forceinline__ void derived_cfl_ring(
    const GeoF &g, const TablesF &t, const PhysF &ph, int mode, const float *__restrict__ S,
    const float *__restrict__ E, const float *__restrict__ vr, const float *__restrict__ dv,
    const float *__restrict__ qplus, const float *__restrict__ qminus, float *__restrict__ cs,
    float *__restrict__ H, float *__restrict__ P, float *__restrict__ T, float *__restrict__ nu,
    unsigned int *__restrict__ dt_min, int i, float *red, longlong2 *red2,
    const float *__restrict__ corr_phi, const float *__restrict__ corr_r)
{
    const int nz = g.nz, nr = g.nr;
    const size_t row = (size_t)i * nz;
    const bool do_cfl = (mode & 4) != 0;
    float md0 = 0.f, md1 = 0.f;
    if (do_cfl && i < nr - 1) {
        // ring means of dv, independent of the block's shape; red2 (33
        // longlong2) serves both pair reductions one after the other
        const float2 m = exact_row_means2(dv + row, dv + row + nz, nz,
                                          reinterpret_cast<float2 *>(red2), red2);
        md0 = m.x;
        md1 = m.y;
    }
    float local = 3.0e38f;
    if (do_cfl && i < nr - 1 && i >= 0 && (i == 0 || i < nr - 1)) {
        // shear limit: |vm_i / R_i - vm_{i+1} / R_{i+1}| with vm = Vref + mean dv
        const float denom = fabsf(t.OmRefDiff[i] + md0 * t.InvRmed[i] - md1 * t.InvRmed[i + 1]) +
                            1.0e-30f;
        local = ph.cfl * g.dphi / denom;
    }
    const bool cfl_ring = do_cfl && i >= 1 && i < nr - 1;
    // standard transport: the ring's frame speed of the Keplerian reference
    const float vref_frame =
        ph.fast_transport ? 0.f : (float)(t.Vref_d[i] - t.Rmed_d[i] * g.omega_frame);
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
            const float vres = ph.fast_transport ? d0 - md0 : vref_frame + d0;
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
            float invdt5 = 4.f * n * t.InvCell2[i];
            float invdt6 = 0.f;
            if (ph.adiabatic) invdt6 = ph.inv_hc_limit * fabsf(__fdividef(qplus[c] - qminus[c], E[c]));
            if (ph.leapfrog) {
                // LeapFrog applies the source terms twice with dt/2 (cfl.cpp:254-317)
                invdt4 *= 0.6f;
                invdt5 *= 0.6f;
                invdt6 *= 0.6f;
            }
            const float s2 = invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 +
                             invdt4 * invdt4 + invdt5 * invdt5 + invdt6 * invdt6;
            float dt_cell = ph.cfl * rsqrtf(s2);
            if (ph.stabilize == 2) {
                // viscous stability limit, cfl.cpp:332-351
                const float cc = fminf(corr_phi[c], corr_r[c]);
                if (cc != 0.f) dt_cell = fminf(dt_cell, -ph.cfl / cc);
            }
            local = fminf(local, dt_cell);
        }
    }
    if (do_cfl) {
        const float m = bmin_f(local, red);
        if (threadIdx.x == 0 && m < 3.0e38f) atomicMin(dt_min, __float_as_uint(m));
    }
}

}  // namespace fgpu32
