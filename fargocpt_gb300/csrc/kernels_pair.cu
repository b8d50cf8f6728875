// The FP64 form's cell kernels with their arithmetic in float pairs
// (fp64_pair.cuh): source terms, artificial viscosity, the viscous stress
// tensor and velocity update with SubStep3, and the velocities rebuilt from
// the transported momenta.
//
// The FP64 kernels (kernels_fp64.cu) run at 85% of GB300's FP64 pipe and
// 6-17% of its HBM bandwidth: the FP64 pipe is the bound.  Here every stored
// double is split into a pair on the integer pipe, the arithmetic is pair
// arithmetic (48 significant bits, errors within a few 2^-47 of the
// operands), and FP64 is kept for three things:
//  * the state: an update x += dx adds the pair increment, joined into a
//    double, to the FP64 value of x, so that a step loses the pair's
//    rounding of the increment, not of the state;
//  * the differences of stored values whose gradient cancels: the potential
//    and the pressure in the source terms (neighbouring values agree to 2 or
//    3 digits, so a pair's 2^-48 of each value would be 2^-40 of their
//    difference; the FP64 difference is exact, as in the reference);
//  * the floors (temperature_floor, the sigma floor), screened in FP32 so
//    that only values near a bound take the FP64 comparison, which then
//    gives the reference's clamped value exactly.
// Each kernel cites the reference function it follows and has the grid and
// the ring ranges of its FP64 counterpart.
#include "fp64_pair.cuh"
#include "hydro.cuh"
#include "kernels.h"

#include <math.h>

#include <algorithm>

namespace fgpu {
namespace {

#define CELL(i, j) ((size_t)(i) * (size_t)nz + (size_t)(j))

__device__ __forceinline__ int nxt(int j, int nz) { return j == nz - 1 ? 0 : j + 1; }
__device__ __forceinline__ int prv(int j, int nz) { return j == 0 ? nz - 1 : j - 1; }

__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return f2_sadd(a, b); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return f2_ssub(a, b); }
__device__ __forceinline__ f2 operator-(f2 a) { return f2_neg(a); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return f2_smul(a, b); }
__device__ __forceinline__ f2 operator/(f2 a, f2 b) { return f2_sdiv(a, b); }

// a stored double, a kernel argument or a literal as a pair
__device__ __forceinline__ f2 P(double x) { return f2_split(x); }
// ring i's value of one of the per-ring tables as a pair
__device__ __forceinline__ f2 T(const Tables &t, const double *tab, int i)
{
    const float2 v = t.ptab[(tab - t.tbase) + i];
    return f2{v.x, v.y};
}
// a constant the host split (split_pair_host)
__device__ __forceinline__ f2 K(float2 v) { return f2{v.x, v.y}; }
// the FP64 difference of two stored values, as a pair
__device__ __forceinline__ f2 D(double a, double b) { return f2_split(a - b); }
// x s for a power of two s (exact)
__device__ __forceinline__ f2 sc(f2 x, float s) { return f2{__fmul_rn(x.h, s), __fmul_rn(x.l, s)}; }
__device__ __forceinline__ bool negative(f2 x) { return x.h < 0.f; }
// x + dx: the FP64 value plus the joined pair increment
__device__ __forceinline__ double upd(double x, f2 dx) { return x + f2_to_double(dx); }

// x truncated to a float (relative error below 2^-23) for
// 2^-126 <= |x| < 2^128, on the integer pipe; ok is false elsewhere
__device__ __forceinline__ float ftrunc(double x, bool &ok)
{
    const unsigned w1 = (unsigned)__double2hiint(x), w0 = (unsigned)__double2loint(x);
    const unsigned ax = w1 & 0x7fffffffu;
    ok = ax - (897u << 20) < (254u << 20);
    return __uint_as_float(__funnelshift_l(w0, ax - (896u << 20), 3) | (w1 & 0x80000000u));
}

// temperature_floor (the FP64 kernels' helper; floors of Transport,
// TransportEuler.cpp:122-127, and SubStep3): e clamped into
// [sigma emin_fac, sigma emax_fac], NaN to the lower bound, as in the FP64
// form.  The FP32 screen passes e only when it lies inside the bounds by
// more than 2^-20 of them (the truncations and roundings of the screen are
// below 2^-22), so an e it passes is one the FP64 clamp leaves alone.
__device__ __forceinline__ double floor_e(double e, double sigma, const Phys &ph)
{
    const float emin_f = ph.emin_fac_f, emax_f = ph.emax_fac_f;
    bool ok_e, ok_s;
    const float ef = ftrunc(e, ok_e), sf = ftrunc(sigma, ok_s);
    const float lo = __fmul_rn(__fmul_rn(sf, emin_f), 1.0f + 0x1p-20f);
    const float hi = __fmul_rn(__fmul_rn(sf, emax_f), 1.0f - 0x1p-20f);
    if (ok_e && ok_s && ef > lo && ef < hi) return e;
    const double emin = sigma * ph.emin_fac;
    const double emax = sigma * ph.emax_fac;
    if (!(e > emin)) e = emin;
    if (!(e < emax)) e = emax;
    return e;
}

// exp(x) - 1 for |x| <= 1/64 in pairs: x + x^2/2 + x^3/6 in pair arithmetic,
// the x^4 tail (below 6.0e-8) in FP32 (its rounding below 2^-48)
__device__ __forceinline__ f2 f2_expm1_small(f2 x)
{
    const f2 x2 = x * x;
    const f2 x3 = x2 * x;
    const float xh = x.h;
    float p = __fmaf_rn(xh, 1.0f / 5040.0f, 1.0f / 720.0f);
    p = __fmaf_rn(p, xh, 1.0f / 120.0f);
    p = __fmaf_rn(p, xh, 1.0f / 24.0f);
    const float tail = __fmul_rn(__fmul_rn(x2.h, x2.h), p);
    const f2 sixth = P(1.0 / 6.0);
    return x + (sc(x2, 0.5f) + (x3 * sixth + f2{tail, 0.f}));
}

// update_with_sourceterms (SourceEuler.cpp:369-450): the momentum updates
// from the pressure gradient, the potential and the centrifugal term
__global__ void k_source_p(Geo g, Tables t, float2 dtp, float2 omega_frame,
                           const double *__restrict__ S, const double *__restrict__ Pr,
                           const double *__restrict__ pot, const double *__restrict__ vr_in,
                           const double *__restrict__ vaz_in, double *__restrict__ vr_out,
                           double *__restrict__ vaz_out)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr
    if (j >= nz) return;
    const f2 pdt = K(dtp);
    double vr = vr_in[CELL(i, j)];
    if (i >= 2 && i < nr - 1) {
        const size_t c = CELL(i, j), cm = CELL(i - 1, j);
        const f2 idr = T(t, t.InvDiffRmed, i);
        const f2 gradp = sc(D(Pr[c], Pr[cm]), 2.0f) / (P(S[c]) + P(S[cm])) * idr;
        const f2 gradphi = D(pot[c], pot[cm]) * idr;
        const int jn = nxt(j, nz);
        const f2 vsum = (P(vaz_in[c]) + P(vaz_in[CELL(i, jn)])) +
                        (P(vaz_in[cm]) + P(vaz_in[CELL(i - 1, jn)]));
        const f2 vt = sc(vsum, 0.25f) + T(t, t.Rinf, i) * K(omega_frame);
        const f2 centrifugal = vt * vt * T(t, t.InvRinf, i);
        vr = upd(vr, pdt * (centrifugal - (gradp + gradphi)));
    }
    vr_out[CELL(i, j)] = vr;
    if (i < nr) {
        double va = vaz_in[CELL(i, j)];
        if (i >= 1 && i < nr - 1) {
            const size_t c = CELL(i, j), cp = CELL(i, prv(j, nz));
            const f2 invdx = T(t, t.InvDxSrc, i);
            const f2 gradp = sc(D(Pr[c], Pr[cp]), 2.0f) / (P(S[c]) + P(S[cp])) * invdx;
            const f2 gradphi = D(pot[c], pot[cp]) * invdx;
            va = upd(va, -(pdt * (gradp + gradphi)));
        }
        vaz_out[CELL(i, j)] = va;
    }
}

// Fields one float-pair kernel leaves for the next (the artificial
// pressures, div v and the stress tensor): the pair itself in the double's
// 8 bytes (PT), else the joined double
template <bool PT>
__device__ __forceinline__ void put_t(double *x, size_t c, f2 v)
{
    if (PT) reinterpret_cast<f2 *>(x)[c] = v;
    else x[c] = f2_to_double(v);
}
__device__ __forceinline__ f2 get_t(const double *x, size_t c)
{
    return reinterpret_cast<const f2 *>(x)[c];
}

// compression heating (SourceEuler.cpp:1045-1092) and the artificial
// pressures with their dissipation (artificial_viscosity.cpp:35-91,
// 141-230), as k_artvisc_q
__global__ void k_artvisc_q_p(Geo g, Tables t, Phys ph, float2 dtp, const double *__restrict__ S,
                              const double *__restrict__ vr, const double *__restrict__ vaz,
                              double *__restrict__ E, double *__restrict__ Qr,
                              double *__restrict__ Qp)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const int jn = nxt(j, nz);
    const size_t c = CELL(i, j);
    const f2 pdt = K(dtp);
    const f2 vr0 = P(vr[c]), vr1 = P(vr[CELL(i + 1, j)]);
    // the FP64 difference of neighbouring v_phi (they cancel to many digits)
    const f2 dva = D(vaz[CELL(i, jn)], vaz[c]);
    const f2 invdphi = K(g.pk_invdphi);
    double e = 0.0;
    f2 de{0.f, 0.f};  // the energy's increment beyond the compression factor
    if (ph.adiabatic) {
        e = E[c];
        if (i < nr - 1) {
            const f2 div_v = (vr1 * T(t, t.Rinf, i + 1) - vr0 * T(t, t.Rinf, i)) *
                                 T(t, t.InvDiffRsupRb, i) +
                             dva * invdphi * T(t, t.InvRmed, i);
            const f2 x = -(K(ph.pk_gm1) * pdt * div_v);
            if (fabsf(x.h) <= 0.015625f) {
                de = P(e) * f2_expm1_small(x);
            } else {
                e = e * exp(f2_to_double(x));  // shocks: FP64 exp
            }
        }
    }
    if (ph.art_visc_sn) {
        const f2 sig = P(S[c]);
        const f2 C2 = K(ph.pk_C2);
        const f2 dv_r = vr1 - vr0;
        const f2 qr = negative(dv_r) ? C2 * sig * (dv_r * dv_r) : f2{0.f, 0.f};
        const f2 dv_p = dva;
        const f2 qp = negative(dv_p) ? C2 * sig * (dv_p * dv_p) : f2{0.f, 0.f};
        put_t<true>(Qr, c, qr);
        put_t<true>(Qp, c, qp);
        if (ph.adiabatic && ph.dissipation && i >= 1 && i < nr - 1) {
            de = de - pdt * (qr * dv_r * T(t, t.InvDiffRsup, i) + qp * dv_p * T(t, t.InvDxTheta, i));
        }
    }
    if (ph.art_visc_tw) {
        // update_with_artificial_viscosity_TW, artificial_viscosity.cpp:52-91
        const f2 sig = P(S[c]);
        const f2 eps_rr = (vr1 - vr0) * T(t, t.InvDiffRsup, i);
        const f2 eps_pp = T(t, t.InvRmed, i) * (dva * invdphi + sc(vr1 + vr0, 0.5f));
        const f2 sum = eps_rr + eps_pp;
        const f2 div_V = negative(sum) ? sum : f2{0.f, 0.f};
        const f2 third = P(1.0 / 3.0);
        const f2 lsig = T(t, t.LSqTW, i) * sig;
        put_t<true>(Qr, c, -(lsig * div_V) * (eps_rr - third * div_V));
        put_t<true>(Qp, c, -(lsig * div_V) * (eps_pp - third * div_V));
        if (ph.adiabatic && ph.dissipation && i >= 1 && i < nr - 1) {
            const f2 d = eps_rr - eps_pp;
            const f2 qplus = -(T(t, t.LSqTW, i) * div_V * sig * third) *
                             (eps_rr * eps_rr + eps_pp * eps_pp + d * d);
            de = de + qplus * pdt;
        }
    }
    if (ph.adiabatic) {
        e = upd(e, de);
        if (ph.dissipation) e = floor_e(e, S[c], ph);
        E[c] = e;
    }
}

// the artificial-viscosity velocity updates (artificial_viscosity.cpp:
// 93-139, 232-290) and the derived c_s, H, nu of the ideal EOS
// (compute_sound_speed_normal, compute_scale_height_old, update_viscosity),
// as k_artvisc_v
__global__ void k_artvisc_v_p(Geo g, Tables t, Phys ph, float2 dtp, const double *__restrict__ S,
                              const double *__restrict__ E, const double *__restrict__ Qr,
                              const double *__restrict__ Qp, double *__restrict__ vr,
                              double *__restrict__ vaz, double *__restrict__ cs,
                              double *__restrict__ H, double *__restrict__ nu)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const f2 pdt = K(dtp);
    if (ph.art_visc_sn) {
        if (i >= 2 && i < nr - 1) {
            const size_t cm = CELL(i - 1, j);
            const f2 a = sc(pdt, 2.0f) / (P(S[c]) + P(S[cm]));
            vr[c] = upd(vr[c], -(a * (get_t(Qr, c) - get_t(Qr, cm)) * T(t, t.InvDiffRmed, i)));
        }
        if (i >= 1 && i < nr - 1) {
            const size_t cp = CELL(i, prv(j, nz));
            const f2 a = sc(pdt, 2.0f) / (P(S[c]) + P(S[cp]));
            vaz[c] = upd(vaz[c], -(a * (get_t(Qp, c) - get_t(Qp, cp)) * T(t, t.InvDxTheta, i)));
        }
    }
    if (ph.art_visc_tw) {
        if (i >= 1 && i < nr - 1) {
            const size_t cp = CELL(i, prv(j, nz));
            const f2 avg = sc(P(S[c]) + P(S[cp]), 0.5f);
            vaz[c] = upd(vaz[c], pdt / avg * T(t, t.InvDxSrc, i) * (get_t(Qp, c) - get_t(Qp, cp)));
        }
        if (i >= 2 && i < nr - 1) {
            const size_t cm = CELL(i - 1, j);
            const f2 avg = sc(P(S[c]) + P(S[cm]), 0.5f);
            const f2 br = (get_t(Qr, c) * T(t, t.Rmed, i) - get_t(Qr, cm) * T(t, t.Rmed, i - 1)) -
                          sc(get_t(Qp, c) + get_t(Qp, cm), 0.5f) * T(t, t.DiffRmed, i);
            vr[c] = upd(vr[c], K(ph.pk_rvf) * (pdt / avg) * T(t, t.TwoOverDRmed2, i) * br);
        }
    }
    if (ph.adiabatic) {
        const f2 c_s = f2_sqrt(K(ph.pk_g_gm1) * (P(E[c]) / P(S[c])));
        const f2 h = c_s * T(t, t.HFacAdi, i);
        cs[c] = f2_to_double(c_s);
        H[c] = f2_to_double(h);
        nu[c] = ph.alpha > 0 ? f2_to_double(K(ph.pk_alpha) * h * c_s) : ph.constant_viscosity;
    }
}

// the viscous stress tensor (viscosity.cpp:60-247), as k_stress
template <bool PT>
__global__ void k_stress_p(Geo g, Tables t, const double *__restrict__ S,
                           const double *__restrict__ vr, const double *__restrict__ vaz,
                           const double *__restrict__ nu, double *__restrict__ divv,
                           double *__restrict__ trr, double *__restrict__ tpp,
                           double *__restrict__ trp)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jn = nxt(j, nz);
    const f2 vr0 = P(vr[c]), vr1 = P(vr[CELL(i + 1, j)]);
    const double va0d = vaz[c];
    // v_phi of neighbouring cells of a ring agree to many digits (the orbital
    // speed cancels): their FP64 difference, exact as in the reference
    const f2 dva = D(vaz[CELL(i, jn)], va0d);
    const f2 n = P(nu[c]), sg = P(S[c]);
    const f2 invdphi = K(g.pk_invdphi);
    const f2 irm = T(t, t.InvRmed, i);
    const f2 third = P(1.0 / 3.0);
    const f2 dv = (vr1 * T(t, t.Rinf, i + 1) - vr0 * T(t, t.Rinf, i)) * T(t, t.InvDiffRsupRb, i) +
                  dva * invdphi * irm;
    put_t<PT>(divv, c, dv);
    const f2 two_n_sg = sc(n * sg, 2.0f);
    const f2 drr = (vr1 - vr0) * T(t, t.InvDiffRsup, i);
    put_t<PT>(trr, c, two_n_sg * (drr - third * dv));
    const f2 dpp = dva * invdphi * irm + sc(vr1 + vr0, 0.5f) * irm;
    put_t<PT>(tpp, c, two_n_sg * (dpp - third * dv));
    if (i >= 1) {
        const int jp = prv(j, nz);
        const size_t cm = CELL(i - 1, j), cp = CELL(i, jp), cmp = CELL(i - 1, jp);
        const f2 dvazirdr = (P(va0d) * irm - P(vaz[cm]) * T(t, t.InvRmed, i - 1)) *
                            T(t, t.InvDiffRmed, i);
        const f2 dvrdphi = (vr0 - P(vr[cp])) * invdphi;
        const f2 drp = T(t, t.Rinf, i) * dvazirdr + dvrdphi * T(t, t.InvRinf, i);
        const f2 n4 = sc((n + P(nu[cm])) + (P(nu[cp]) + P(nu[cmp])), 0.25f);
        const f2 s4 = sc((sg + P(S[cm])) + (P(S[cp]) + P(S[cmp])), 0.25f);
        put_t<PT>(trp, c, n4 * s4 * drp);
    }
}

// the viscous velocity update (viscosity.cpp:249-348 without
// StabilizeViscosity, which the FP64 kernel serves) and SubStep3:
// thermal relaxation (SourceEuler.cpp:632-690), viscous heating (:496-536),
// the radiative alpha factor (:905-912) and the energy update, as k_viscous
__global__ void k_viscous_p(Geo g, Tables t, Phys ph, float2 dtp, float2 beta_inv, int mode,
                            const double *__restrict__ S, const double *__restrict__ trr,
                            const double *__restrict__ tpp, const double *__restrict__ trp,
                            const double *__restrict__ divv, const double *__restrict__ nu,
                            const double *__restrict__ H, const double *__restrict__ S0,
                            const double *__restrict__ E0, double *__restrict__ vr,
                            double *__restrict__ vaz, double *__restrict__ E,
                            double *__restrict__ qplus, double *__restrict__ qminus)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jp = prv(j, nz), jn = nxt(j, nz);
    const f2 pdt = K(dtp);
    const f2 invdphi = K(g.pk_invdphi);
    if (mode & 1) {
        if (i >= 1 && i < nr - 1) {
            const f2 avg = sc(P(S[c]) + P(S[CELL(i, jp)]), 0.5f);
            const f2 dVp = pdt * T(t, t.InvRmed, i) / avg *
                           (T(t, t.TwoOverDRa2, i) * (T(t, t.RinfSq, i + 1) * get_t(trp, CELL(i + 1, j)) -
                                                      T(t, t.RinfSq, i) * get_t(trp, c)) +
                            (get_t(tpp, c) - get_t(tpp, CELL(i, jp))) * invdphi);
            vaz[c] = upd(vaz[c], dVp);
        }
        if (i >= 2 && i < nr - 1) {
            const size_t cm = CELL(i - 1, j);
            const f2 avg = sc(P(S[c]) + P(S[cm]), 0.5f);
            const f2 dVr = pdt / avg * K(ph.pk_rvf) * T(t, t.TwoOverRmedSum, i) *
                           ((T(t, t.Rmed, i) * get_t(trr, c) - T(t, t.Rmed, i - 1) * get_t(trr, cm)) *
                                T(t, t.InvDiffRmed, i) +
                            (get_t(trp, CELL(i, jn)) - get_t(trp, c)) * invdphi -
                            sc(get_t(tpp, c) + get_t(tpp, cm), 0.5f));
            vr[c] = upd(vr[c], dVr);
        }
    }
    if (!(mode & 6) || !ph.adiabatic) return;
    const f2 zero{0.f, 0.f};
    f2 qp = zero, qm = zero;
    const double e = E[c];
    const double sig_d = S[c];
    const f2 ep = P(e), sig = P(sig_d);
    const bool active = i >= 1 && i < nr - 1;
    if (active) {
        if (ph.cooling_beta) {
            f2 delta_E = ep;
            if (ph.beta_ref == 1) {
                delta_E = delta_E - P(E0[c]) / P(S0[c]) * sig;
            } else if (ph.beta_ref == 2) {
                delta_E = delta_E - T(t, t.EModel, i) * sig;
            } else if (ph.beta_ref == 3) {
                delta_E = delta_E - sig * K(ph.pk_emin_fac);
            }
            qm = delta_E * T(t, t.OmegaK, i) * K(beta_inv);
        }
        if (ph.heating_viscous) {
            const double nd = nu[c];
            if (nd != 0.0) {
                const f2 n = P(nd);
                const f2 tau_r_phi = sc((get_t(trp, c) + get_t(trp, CELL(i + 1, j))) +
                                            (get_t(trp, CELL(i, jn)) + get_t(trp, CELL(i + 1, jn))),
                                        0.25f);
                const f2 t_rr = get_t(trr, c), t_pp = get_t(tpp, c), d = get_t(divv, c);
                const f2 ns = n * sig;
                f2 q = (t_rr * t_rr + sc(tau_r_phi * tau_r_phi, 2.0f) + t_pp * t_pp) / sc(ns, 2.0f);
                q = q + P(2.0 / 9.0) * ns * (d * d);
                qp = q * K(ph.pk_hvf);
            }
        }
        const f2 x = K(ph.pk_mu_gm1_over_R) / sig;
        const f2 x2 = x * x;
        const f2 alpha = P(1.0) + P(H[c]) * K(ph.pk_cool_const) * (x2 * x2) * (ep * ep * ep);
        const f2 inv_alpha = f2_rcp(alpha);
        qp = qp * inv_alpha;
        qm = qm * inv_alpha;
    }
    double qp_d = f2_to_double(qp), qm_d = f2_to_double(qm);
    if (mode & 4) {
        double e_new = e;
        if (active) {
            e_new = upd(e, pdt * (qp - qm));
            if (sig_d < ph.sigma_floor10) {
                // TAU_EFF is zero on this path: the equilibrium energy is 0
                qm_d = qp_d;
                e_new = 0.0;
            }
        }
        E[c] = floor_e(e_new, sig_d, ph);
    }
    qplus[c] = qp_d;
    qminus[c] = qm_d;
}

// compute_velocities_from_momenta (TransportEuler.cpp:498-535), the sigma
// floor (SourceEuler.cpp:102-134) and the temperature floor, as k_finish,
// with the azimuthal transport's AdvectSHIFT (:238-268): the transported
// fields of ring i are read at j - shift[i]
__global__ void k_finish_p(Geo g, Tables t, Phys ph, float2 omf, const double *__restrict__ mom0,
                           const double *__restrict__ mom1, const double *__restrict__ mom2,
                           const double *__restrict__ mom3, const double *__restrict__ S_t,
                           const double *__restrict__ E_t, const double *__restrict__ vr_in,
                           double *__restrict__ vr_out, double *__restrict__ vaz_out,
                           double *__restrict__ S_out, double *__restrict__ E_out,
                           const int *__restrict__ shift)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    if (i == nr) {
        vr_out[c] = vr_in[c];
        return;
    }
    // cell j of ring k before the shift
    auto at = [&](int k, int jj) {
        int a = jj - __ldg(shift + k);
        if (a < 0) a += nz;
        return CELL(k, a);
    };
    const size_t cs = at(i, j);
    const double s = S_t[cs];
    const f2 sp = P(s);
    if (i == 0) {
        vr_out[c] = 0.0;
    } else {
        const size_t cm = at(i - 1, j);
        vr_out[c] = f2_to_double((P(mom0[cm]) + P(mom1[cs])) / (P(S_t[cm]) + sp));
    }
    const size_t cjm = at(i, prv(j, nz));
    vaz_out[c] = f2_to_double((P(mom2[cjm]) + P(mom3[cs])) / (P(S_t[cjm]) + sp) *
                                  T(t, t.InvRmed, i) -
                              T(t, t.Rmed, i) * K(omf));
    // s < sigma_min on the bit patterns (sigma_min >= 0; a NaN stays)
    const long long bs = __double_as_longlong(s);
    const bool nan = (bs & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
    const double sf = (!nan && bs < __double_as_longlong(ph.sigma_min)) ? ph.sigma_min : s;
    S_out[c] = sf;
    if (ph.adiabatic) E_out[c] = floor_e(E_t[cs], sf, ph);
}

__global__ void k_join_pairs(double *__restrict__ x, size_t n)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x)
        x[k] = f2_to_double(reinterpret_cast<const f2 *>(x)[k]);
}

dim3 grid2(int nz, int rows, int bx) { return dim3((nz + bx - 1) / bx, rows); }

}  // namespace

void launch_source_pair(const Launch &L, double dt, double omf, const double *S, const double *Pr,
                        const double *pot, const double *vr_in, const double *vaz_in,
                        double *vr_out, double *vaz_out)
{
    k_source_p<<<grid2(L.g.nz, L.g.nr + 1, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, split_pair_host(dt), split_pair_host(omf), S, Pr, pot, vr_in, vaz_in, vr_out,
        vaz_out);
}

void launch_artvisc_q_pair(const Launch &L, double dt, const double *S, const double *vr,
                           const double *vaz, double *E, double *Qr, double *Qp)
{
    k_artvisc_q_p<<<grid2(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, L.ph, split_pair_host(dt), S, vr, vaz, E, Qr, Qp);
}

void launch_artvisc_v_pair(const Launch &L, double dt, const double *S, const double *E,
                           const double *Qr, const double *Qp, double *vr, double *vaz, double *cs,
                           double *H, double *nu)
{
    k_artvisc_v_p<<<grid2(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, L.ph, split_pair_host(dt), S, E, Qr, Qp, vr, vaz, cs, H, nu);
}

void launch_stress_pair(const Launch &L, const double *S, const double *vr, const double *vaz,
                        const double *nu, double *divv, double *trr, double *tpp, double *trp)
{
    auto k = stress_as_pairs(L) ? k_stress_p<true> : k_stress_p<false>;
    k<<<grid2(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(L.g, L.t, S, vr, vaz, nu, divv, trr, tpp,
                                                          trp);
}

void launch_join_pairs(cudaStream_t stream, double *x, size_t n)
{
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 8192);
    k_join_pairs<<<blocks, 256, 0, stream>>>(x, n);
}

void launch_viscous_pair(const Launch &L, double dt, double beta_inv, int mode, const State &s)
{
    k_viscous_p<<<grid2(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, L.ph, split_pair_host(dt), split_pair_host(beta_inv), mode, s.sigma, s.trr,
        s.tpp, s.trp, s.divv, s.nu, s.H,
        s.sigma0, s.energy0, s.vr, s.vaz, s.energy, s.qplus, s.qminus);
}

void launch_finish_pair(const Launch &L, double omf, double *const mom[4], const double *S_t,
                        const double *E_t, const double *vr_in, double *vr_out, double *vaz_out,
                        double *S_out, double *E_out, const int *ring_shift)
{
    k_finish_p<<<grid2(L.g.nz, L.g.nr + 1, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, L.ph, split_pair_host(omf), mom[0], mom[1], mom[2], mom[3], S_t, E_t, vr_in,
        vr_out, vaz_out,
        S_out, E_out, ring_shift);
}

}  // namespace fgpu
