// FP64 kernels of the GB300 hydro step.
//
// Each kernel restates one or more phases of FargoCPT's sim::step_Euler
// (reference src/simulation.cpp:148-267) with the reference's expression
// order, so the FP64 path reproduces the reference's own FP64 results to
// round-off.  Work is fused where the fusion recomputes nothing: GB300's FP64
// rate is low, so every FP64 operation is done once and intermediates that
// several neighbours reuse go through HBM/L2 instead of being recomputed.
#include "hydro.cuh"
#include "fp64_pair.cuh"
#include "kernels.h"
#include "reduce.cuh"

#include <math.h>

#include <algorithm>

namespace fgpu {

#define CELL(i, j) ((size_t)(i) * (size_t)nz + (size_t)(j))

__device__ __forceinline__ int jnext(int j, int nz) { return j == nz - 1 ? 0 : j + 1; }
__device__ __forceinline__ int jprev(int j, int nz) { return j == 0 ? nz - 1 : j - 1; }

// Sign and magnitude tests on the bit pattern run on the integer pipe, which
// GB300 has plenty of, instead of the FP64 pipe, which it has little of.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool positive(double x)
{
    // x > 0 for finite x
    return dbits(x) > 0;
}
// a * b > 0 for finite a, b (both non-zero, same sign)
__device__ __forceinline__ bool same_sign_nonzero(double a, double b)
{
    const long long ia = dbits(a), ib = dbits(b);
    const long long m = 0x7fffffffffffffffll;
    return ((ia ^ ib) >= 0) && (ia & m) != 0 && (ib & m) != 0;
}
// |a| < |b| for finite a, b
__device__ __forceinline__ bool abs_less(double a, double b)
{
    const long long m = 0x7fffffffffffffffll;
    return (dbits(a) & m) < (dbits(b) & m);
}

// Reciprocal by Newton-Raphson iteration r <- r (2 - b r), written as
// e = 1 - b r, r <- r + r e, from the hardware's approximate reciprocal
// (PTX rcp.approx.ftz.f64).  Two iterations square the seed's relative error
// twice, which takes any seed better than 2^-14 below double rounding; the
// quotient a * (1/b) is then within two units in the last place of a / b.
// Used for divisors that are normal numbers (densities, sums of slopes).
__device__ __forceinline__ double fast_rcp(double b)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
    double e = fma(-b, r, 1.0);
    r = fma(r, e, r);
    e = fma(-b, r, 1.0);
    r = fma(r, e, r);
    return r;
}
__device__ __forceinline__ double fast_div(double a, double b) { return a * fast_rcp(b); }

// The same with one Newton-Raphson iteration: the hardware seed is within
// 2^-20 of 1/b (measured on GB300 over 61 binades), so one iteration leaves
// a relative error below 2^-40 (always low).  Used where the quotient only
// forms an increment or a derived quantity (slopes, source and viscous
// terms, heating and cooling, the sound speed, the radial specific energy);
// the velocities rebuilt from momenta, the azimuthal specific quantities and
// the CFL step keep the two-iteration form, whose one-sided error would
// otherwise accumulate in the state or shift the time step.
__device__ __forceinline__ double fast_rcp1(double b)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
    const double e = fma(-b, r, 1.0);
    return fma(r, e, r);
}

__device__ __forceinline__ double fast_div1(double a, double b) { return a * fast_rcp1(b); }

// van_leer_lim / MC_lim, src/TransportEuler.cpp:306-337
__device__ __forceinline__ double flux_limiter(double a, double b, int mc)
{
    if (mc) {
        const double mm = same_sign_nonzero(a, b) ? (abs_less(a, b) ? a : b) : 0.0;
        const double c = 0.5 * (a + b), d = 2.0 * mm;
        if (same_sign_nonzero(c, d)) return abs_less(c, d) ? c : d;
        return 0.0;
    }
    if (same_sign_nonzero(a, b)) return 2.0 * a * b * fast_rcp1(a + b);
    return 0.0;
}

// The limited slope without its constant factor: van Leer's 2ab/(a+b) less
// the 2, MC's value as is.  The azimuthal pass multiplies the factor (2 or
// 1, and 1/(2 dx)) into each cell's interpolation distance once, instead of
// into every quantity's slope.
__device__ __forceinline__ double flux_limiter_unscaled(double a, double b, int mc)
{
    if (mc) return flux_limiter(a, b, 1);
    if (same_sign_nonzero(a, b)) return a * b * fast_rcp1(a + b);
    return 0.0;
}

// exp(x) by its Taylor series through x^7 for |x| <= 1/64 (the remainder,
// below x^8 / 8! <= 1e-19, is under half an ulp of the result), exp() beyond:
// compression heating's exponent is a fraction of the cell's CFL number, so
// the series covers the disk and exp() the shocks.
__device__ __forceinline__ double exp_small(double x)
{
    if (fabs(x) > 0.015625) return exp(x);
    double p = 1.0 / 5040.0;
    p = fma(p, x, 1.0 / 720.0);
    p = fma(p, x, 1.0 / 120.0);
    p = fma(p, x, 1.0 / 24.0);
    p = fma(p, x, 1.0 / 6.0);
    p = fma(p, x, 0.5);
    p = fma(p, x, 1.0);
    return fma(p, x, 1.0);
}

// assure_temperature_range, src/SourceEuler.cpp:136-202: the bounds are
// Tmin/max * sigma / mu * R / (gamma - 1); the constant factor is folded on
// the host.
__device__ __forceinline__ double temperature_floor(double e, double sigma, const Phys &ph)
{
    const double emin = sigma * ph.emin_fac;
    const double emax = sigma * ph.emax_fac;
    if (!(e > emin)) e = emin;
    if (!(e < emax)) e = emax;
    return e;
}

// ---------------------------------------------------------------------------
// CalculateNbodyPotential, src/Pframeforce.cpp:21-86.  The central object's
// term -G M / sqrt(d^2 + eps^2) stays in FP64: the radial force is a small
// difference of neighbouring potentials that gravity, pressure and the
// centrifugal term nearly cancel, and v_r, itself small, inherits the error
// of the dominant term amplified by both cancellations (with this term in
// float pairs, 2^-46, v_r on the 512 x 1536 disk drifted to 1.1e-10 of its
// largest value in 100 steps).  The other bodies' terms, at most ~1e-3 of it
// away from a body, are formed in float-pair arithmetic (fp64_pair.cuh) and
// summed as a pair: about 60 FP32 operations per body and cell instead of
// about 15 FP64 ones, which GB300 issues 64 times slower.
// ---------------------------------------------------------------------------
// 1 / sqrt(d) for a normal d > 0 to FP64 accuracy: the float-pair estimate
// (within a few 2^-46), then one FP64 Newton step, which squares that error
// and leaves the roundings of the step (about one unit in the last place)
__device__ __forceinline__ double rsqrt_fp64(double d)
{
    const double r = f2_to_double(f2_rsqrt(f2_split(d)));
    const double e = fma(-d, r * r, 1.0);
    return fma(0.5 * r, e, r);
}

// Klahr's smoothing applies inside r_sm: a float screen (the pair's high part
// against r_sm with a 2^-20 margin) passes the cells certainly outside it;
// the others compare in FP64
__device__ __forceinline__ bool maybe_inside(f2 dsm, float rsm_f)
{
    return dsm.h < __fmul_rn(rsm_f, 1.0f + 0x1p-20f);
}

// PAIR and a central object at the origin without Klahr smoothing (the
// heliocentric frame's usual case, a uniform branch): its distance^2 is
// R^2 + s^2 (R = Rmed, s = eps H; cos^2 + sin^2 = 1 within the tables'
// rounding), and its potential -G m / sqrt(R^2 + s^2) = C (1 + g(u)) with
// C = -G m / R in FP64 and, u = (s / R)^2,
//     g(u) = (1 + u)^(-1/2) - 1 = -u / (sqrt(1 + u) (1 + sqrt(1 + u))),
// a form without cancellation.  g is small (u is about (eps h)^2), so C g in
// pairs carries an absolute error of a few 2^-46 |C g|, far below the
// rounding of C itself: the FP64 work per cell is the product C and the
// final sum.  The source terms' FP64 differences of the potential see C's
// per-ring values and the smooth correction.  The indirect term, linear in
// the cell position, joins the planets' pair sum.
template <bool PAIR>
__global__ void k_potential(Geo g, Tables t, Phys ph, Bodies b, const double *__restrict__ H,
                            double *__restrict__ pot)
{
    const int nz = g.nz;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    if (PAIR && b.star_plain) {
        const double C = b.gm0 * t.InvRmed[i];
        const f2 sp = f2_smul(f2_split(H[CELL(i, j)]), f2{ph.pk_eps_smooth.x, ph.pk_eps_smooth.y});
        const float2 ir = t.ptab[(t.InvRmed - t.tbase) + i];
        const f2 q = f2_smul(sp, f2{ir.x, ir.y});
        const f2 u = f2_smul(q, q);
        const f2 one{1.f, 0.f};
        const f2 sq = f2_sqrt(f2_sadd(one, u));
        const f2 g1 = f2_neg(f2_sdiv(u, f2_smul(sq, f2_sadd(one, sq))));
        const f2 star = f2_smul(f2_split(C), g1);
        const f2 rmp{t.RmedHi[i], t.RmedLo[i]};
        const f2 xc = f2_smul(rmp, f2{t.cosHi[j], t.cosLo[j]});
        const f2 yc = f2_smul(rmp, f2{t.sinHi[j], t.sinLo[j]});
        const f2 s2 = f2_smul(sp, sp);
        float ah = 0.f, al = 0.f;
        for (int k = 1; k < b.n; ++k) {
            const f2 dx = f2_ssub(xc, f2{b.xh[k], b.xl[k]});
            const f2 dy = f2_ssub(yc, f2{b.yh[k], b.yl[k]});
            const f2 d2 = f2_sadd(f2_sadd(f2_smul(dx, dx), f2_smul(dy, dy)), s2);
            const f2 inv_d = f2_rsqrt(d2);
            f2 term = f2_smul(inv_d, f2{b.gmh[k], b.gml[k]});
            if ((b.klahr >> k) & 1u) {
                // Klahr's cubic inside r_sm (Pframeforce.cpp:57-66): rare, in FP64
                const double r_sm = b.rsm[k];
                const f2 dsm = f2_smul(d2, inv_d);
                if (maybe_inside(dsm, f2_split(r_sm).h)) {
                    const double d_sm = f2_to_double(dsm);
                    if (d_sm < r_sm) {
                        const double q = d_sm / r_sm;
                        const double fk = q * q * q * q - 2.0 * (q * q * q) + 2.0 * q;
                        term = f2_split(f2_to_double(term) * fk);
                    }
                }
            }
            f2_accumulate(ah, al, term);
        }
        const f2 ind = f2_neg(f2_sadd(f2_smul(f2{b.pk_ix.x, b.pk_ix.y}, xc),
                                      f2_smul(f2{b.pk_iy.x, b.pk_iy.y}, yc)));
        pot[CELL(i, j)] = C + f2_to_double(f2_sadd(f2_sadd(f2{ah, al}, ind), star));
        return;
    }
    const double smooth = ph.eps_smooth * H[CELL(i, j)];
    const double s2d = smooth * smooth;
    const double x = t.Rmed[i] * t.cosj[j];
    const double y = t.Rmed[i] * t.sinj[j];
    double acc = 0.0;
    if (b.n > 0) {
        // the central object in FP64, the reference's expressions
        const double dx = x - b.x[0];
        const double dy = y - b.y[0];
        const double d2 = (dx * dx + dy * dy) + s2d;
        const double inv_d = rsqrt_fp64(d2);
        double fk = 1.0;
        const double r_sm = b.rsm[0];
        if (r_sm > 0.0) {
            const double d_sm = d2 * inv_d;
            if (d_sm < r_sm) {
                const double q = d_sm / r_sm;
                fk = q * q * q * q - 2.0 * (q * q * q) + 2.0 * q;
            }
        }
        acc = -ph.G * b.m[0] * inv_d * fk;
    }
    const f2 rm{t.RmedHi[i], t.RmedLo[i]};
    const f2 xc = f2_mul(rm, f2{t.cosHi[j], t.cosLo[j]});
    const f2 yc = f2_mul(rm, f2{t.sinHi[j], t.sinLo[j]});
    const f2 s2 = f2_split(s2d);
    float ah = 0.f, al = 0.f;
    for (int k = 1; k < b.n; ++k) {
        const f2 dx = f2_sub(xc, f2{b.xh[k], b.xl[k]});
        const f2 dy = f2_sub(yc, f2{b.yh[k], b.yl[k]});
        const f2 d2 = f2_add(f2_add(f2_mul(dx, dx), f2_mul(dy, dy)), s2);
        const f2 inv_d = f2_rsqrt(d2);
        f2 term = f2_mul(inv_d, f2{b.gmh[k], b.gml[k]});
        const double r_sm = b.rsm[k];
        if (r_sm > 0.0) {
            // Klahr's cubic inside r_sm (Pframeforce.cpp:57-66): rare, in FP64
            const f2 dsm = f2_mul(d2, inv_d);
            if (maybe_inside(dsm, f2_split(r_sm).h)) {
                const double d_sm = f2_to_double(dsm);
                if (d_sm < r_sm) {
                    const double q = d_sm / r_sm;
                    const double fk = q * q * q * q - 2.0 * (q * q * q) + 2.0 * q;
                    term = f2_split(f2_to_double(term) * fk);
                }
            }
        }
        f2_accumulate(ah, al, term);
    }
    acc += f2_to_double(f2{ah, al});
    pot[CELL(i, j)] = acc + (-b.ix * x - b.iy * y);
}

// ---------------------------------------------------------------------------
// momentum_update_radial / momentum_update_azimuthal,
// src/SourceEuler.cpp:325-428.  Out of place: v_r needs the old v_phi.
// ---------------------------------------------------------------------------
__global__ void k_source(Geo g, Tables t, double dt, double omega_frame,
                         const double *__restrict__ S, const double *__restrict__ P,
                         const double *__restrict__ pot, const double *__restrict__ vr_in,
                         const double *__restrict__ vaz_in, double *__restrict__ vr_out,
                         double *__restrict__ vaz_out)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr
    if (j >= nz) return;
    // v_radial rows One_no_ghost_vr (2) .. MaxMo_no_ghost_vr (nr - 1)
    double vr = vr_in[CELL(i, j)];
    if (i >= 2 && i < nr - 1) {
        double gradp = 2.0 * fast_rcp1(S[CELL(i, j)] + S[CELL(i - 1, j)]);
        gradp *= (P[CELL(i, j)] - P[CELL(i - 1, j)]);
        gradp *= t.InvDiffRmed[i];
        const double gradphi = (pot[CELL(i, j)] - pot[CELL(i - 1, j)]) * t.InvDiffRmed[i];
        const int jn = jnext(j, nz);
        const double vsum = vaz_in[CELL(i, j)] + vaz_in[CELL(i, jn)] +
                            vaz_in[CELL(i - 1, j)] + vaz_in[CELL(i - 1, jn)];
        const double vt = 0.25 * vsum + t.Rinf[i] * omega_frame;
        const double vt2 = vt * vt;
        const double centrifugal = vt2 * t.InvRinf[i];
        vr += dt * (-gradp - gradphi + centrifugal);
    }
    vr_out[CELL(i, j)] = vr;
    if (i < nr) {
        // v_azimuthal rows Zero_no_ghost (1) .. Max_no_ghost (nr - 1)
        double va = vaz_in[CELL(i, j)];
        if (i >= 1 && i < nr - 1) {
            const int jp = jprev(j, nz);
            const double invdx = t.InvDxSrc[i];
            const double gradp = 2.0 * fast_rcp1(S[CELL(i, j)] + S[CELL(i, jp)]) *
                                 (P[CELL(i, j)] - P[CELL(i, jp)]) * invdx;
            const double gradphi = (pot[CELL(i, j)] - pot[CELL(i, jp)]) * invdx;
            va = va + dt * (-gradp - gradphi);
        }
        vaz_out[CELL(i, j)] = va;
    }
}

// ---------------------------------------------------------------------------
// compression_heating (SourceEuler.cpp:459-493) and the first half of
// update_with_artificial_viscosity_SN (artificial_viscosity.cpp:148-207) or
// _TW (:35-91): q_r, q_phi (TW: the diagonal tensor elements) and the energy
// update, then the temperature floor (artificial_viscosity.cpp:19-21).
// ---------------------------------------------------------------------------
__global__ void k_artvisc_q(Geo g, Tables t, Phys ph, double dt, const double *__restrict__ S,
                            const double *__restrict__ vr, const double *__restrict__ vaz,
                            double *__restrict__ E, double *__restrict__ Qr,
                            double *__restrict__ Qp)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const int jn = jnext(j, nz);
    const size_t c = CELL(i, j);
    const double vr0 = vr[c], vr1 = vr[CELL(i + 1, j)];
    const double va0 = vaz[c], va1 = vaz[CELL(i, jn)];
    double e = 0.0;
    if (ph.adiabatic) {
        e = E[c];
        if (i < nr - 1) {
            const double div_v = (vr1 * t.Rinf[i + 1] - vr0 * t.Rinf[i]) * t.InvDiffRsupRb[i] +
                                 (va1 - va0) * g.invdphi * t.InvRmed[i];
            e = e * exp_small(-ph.gm1 * dt * div_v);
        }
    }
    if (ph.art_visc_sn) {
        const double sig = S[c];
        const double dv_r = vr1 - vr0;
        const double qr = dv_r < 0.0 ? ph.C2 * sig * (dv_r * dv_r) : 0.0;
        const double dv_p = va1 - va0;
        const double qp = dv_p < 0.0 ? ph.C2 * sig * (dv_p * dv_p) : 0.0;
        Qr[c] = qr;
        Qp[c] = qp;
        if (ph.adiabatic && ph.dissipation && i >= 1 && i < nr - 1) {
            e = e - dt * qr * dv_r * t.InvDiffRsup[i] - dt * qp * dv_p * t.InvDxTheta[i];
        }
    }
    if (ph.art_visc_tw) {
        // update_with_artificial_viscosity_TW, artificial_viscosity.cpp:52-91
        const double sig = S[c];
        const double eps_rr = (vr1 - vr0) * t.InvDiffRsup[i];
        const double eps_pp = t.InvRmed[i] * ((va1 - va0) * g.invdphi + 0.5 * (vr1 + vr0));
        const double sum = eps_rr + eps_pp;
        const double div_V = sum < 0.0 ? sum : 0.0;
        const double lsig = t.LSqTW[i] * sig;
        Qr[c] = lsig * -div_V * (eps_rr - 1.0 / 3.0 * div_V);
        Qp[c] = lsig * -div_V * (eps_pp - 1.0 / 3.0 * div_V);
        if (ph.adiabatic && ph.dissipation && i >= 1 && i < nr - 1) {
            const double d = eps_rr - eps_pp;
            const double qplus = -t.LSqTW[i] * div_V * sig * (1.0 / 3.0) *
                                 (eps_rr * eps_rr + eps_pp * eps_pp + d * d);
            e += qplus * dt;
        }
    }
    if (ph.adiabatic) {
        if (ph.dissipation) e = temperature_floor(e, S[c], ph);
        E[c] = e;
    }
}

// ---------------------------------------------------------------------------
// Second half of update_with_artificial_viscosity_SN / _TW (velocity updates,
// artificial_viscosity.cpp:209-248 / :93-139) and recalculate_viscosity
// (SourceEuler.cpp:205-223: c_s, H, nu for the ideal EOS).
// ---------------------------------------------------------------------------
__global__ void k_artvisc_v(Geo g, Tables t, Phys ph, double dt, const double *__restrict__ S,
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
    if (ph.art_visc_sn) {
        if (i >= 2 && i < nr - 1) {
            vr[c] = vr[c] - dt * 2.0 * fast_rcp1(S[c] + S[CELL(i - 1, j)]) *
                                (Qr[c] - Qr[CELL(i - 1, j)]) * t.InvDiffRmed[i];
        }
        if (i >= 1 && i < nr - 1) {
            const int jp = jprev(j, nz);
            vaz[c] = vaz[c] - dt * 2.0 * fast_rcp1(S[c] + S[CELL(i, jp)]) *
                                  (Qp[c] - Qp[CELL(i, jp)]) * t.InvDxTheta[i];
        }
    }
    if (ph.art_visc_tw) {
        // artificial_viscosity.cpp:93-139 (conservative volume-integral form)
        if (i >= 1 && i < nr - 1) {
            const int jp = jprev(j, nz);
            const double sigma_phi_avg = 0.5 * (S[c] + S[CELL(i, jp)]);
            vaz[c] += fast_div1(dt, sigma_phi_avg) * t.InvDxSrc[i] * (Qp[c] - Qp[CELL(i, jp)]);
        }
        if (i >= 2 && i < nr - 1) {
            const double sigma_r_avg = 0.5 * (S[c] + S[CELL(i - 1, j)]);
            vr[c] += ph.rvf * fast_div1(dt, sigma_r_avg) * t.TwoOverDRmed2[i] *
                     ((Qr[c] * t.Rmed[i] - Qr[CELL(i - 1, j)] * t.Rmed[i - 1]) -
                      0.5 * (Qp[c] + Qp[CELL(i - 1, j)]) * t.DiffRmed[i]);
        }
    }
    if (ph.adiabatic) {
        // compute_sound_speed_normal / compute_scale_height_old / update_viscosity
        const double c_s = sqrt(ph.g_gm1 * fast_div1(E[c], S[c]));
        const double h = c_s * t.HFacAdi[i];
        cs[c] = c_s;
        H[c] = h;
        nu[c] = ph.alpha > 0 ? ph.alpha * h * c_s : ph.constant_viscosity;
    }
}

// ---------------------------------------------------------------------------
// viscosity::compute_viscous_stress_tensor, src/viscosity/viscosity.cpp:139-254
// ---------------------------------------------------------------------------
__global__ void k_stress(Geo g, Tables t, const double *__restrict__ S, const double *__restrict__ vr,
                         const double *__restrict__ vaz, const double *__restrict__ nu,
                         double *__restrict__ divv, double *__restrict__ trr,
                         double *__restrict__ tpp, double *__restrict__ trp)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jn = jnext(j, nz);
    const double vr0 = vr[c], vr1 = vr[CELL(i + 1, j)];
    const double va0 = vaz[c], va1 = vaz[CELL(i, jn)];
    const double n = nu[c], sg = S[c];
    const double dv = (vr1 * t.Rinf[i + 1] - vr0 * t.Rinf[i]) * t.InvDiffRsupRb[i] +
                      (va1 - va0) * g.invdphi * t.InvRmed[i];
    divv[c] = dv;
    const double drr = (vr1 - vr0) * t.InvDiffRsup[i];
    trr[c] = 2.0 * n * sg * (drr - 1.0 / 3.0 * dv);
    const double dpp = (va1 - va0) * g.invdphi * t.InvRmed[i] + 0.5 * (vr1 + vr0) * t.InvRmed[i];
    tpp[c] = 2.0 * n * sg * (dpp - 1.0 / 3.0 * dv);
    if (i >= 1) {
        const int jp = jprev(j, nz);
        const double dvazirdr = (va0 * t.InvRmed[i] - vaz[CELL(i - 1, j)] * t.InvRmed[i - 1]) *
                                t.InvDiffRmed[i];
        const double dvrdphi = (vr0 - vr[CELL(i, jp)]) * g.invdphi;
        const double drp = t.Rinf[i] * dvazirdr + dvrdphi * t.InvRinf[i];
        const double n4 = 0.25 * (n + nu[CELL(i - 1, j)] + nu[CELL(i, jp)] + nu[CELL(i - 1, jp)]);
        const double s4 = 0.25 * (sg + S[CELL(i - 1, j)] + S[CELL(i, jp)] + S[CELL(i - 1, jp)]);
        trp[c] = n4 * s4 * drp;
    }
}

// ---------------------------------------------------------------------------
// StabilizeViscosity's pseudo-implicit correction factors, the last loop of
// compute_viscous_stress_tensor (viscosity.cpp:256-348), rows 1 .. nr - 1.
// nu * Sigma at the cell centres and the four-cell averages at the r-phi
// corners are recomputed from nu and Sigma (the reference stores them in
// VISCOSITY_SIGMA / VISCOSITY_SIGMA_RP; row nr of the latter is never written
// and stays zero).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nusig_rp(const double *nu, const double *S, int nz, int i, int j)
{
    const int jp = jprev(j, nz);
    const double n = 0.25 * (nu[CELL(i, j)] + nu[CELL(i - 1, j)] + nu[CELL(i, jp)] +
                             nu[CELL(i - 1, jp)]);
    const double sg = 0.25 * (S[CELL(i, j)] + S[CELL(i - 1, j)] + S[CELL(i, jp)] +
                              S[CELL(i - 1, jp)]);
    return n * sg;
}

__global__ void k_visc_corr(Geo g, Tables t, const double *__restrict__ S,
                            const double *__restrict__ nu, double *__restrict__ corr_phi,
                            double *__restrict__ corr_r)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y + 1;  // 1 .. nr - 1
    if (j >= nz || i >= nr) return;
    const size_t c = CELL(i, j);
    const int jp = jprev(j, nz), jn = jnext(j, nz);
    const double rp = nusig_rp(nu, S, nz, i, j);
    const double rp_ip = i + 1 < nr ? nusig_rp(nu, S, nz, i + 1, j) : 0.0;
    const double rp_jp = nusig_rp(nu, S, nz, i, jn);
    const double ns = nu[c] * S[c];
    const double ns_jm = nu[CELL(i, jp)] * S[CELL(i, jp)];
    const double ns_im = nu[CELL(i - 1, j)] * S[CELL(i - 1, j)];
    // v_phi factor
    const double cphi_rp = -t.InvRmed[i] * t.TwoOverDRa2[i] *
                           (rp_ip * t.Ra3IDRmed[i + 1] + rp * t.Ra3IDRmed[i]);
    const double cphi_pp = -t.F43[i] * (ns + ns_jm);
    const double sigma_avg_phi = 0.5 * (S[c] + S[CELL(i, jp)]);
    corr_phi[c] = fast_div(cphi_rp + cphi_pp, sigma_avg_phi * t.Rmed[i]);
    // v_r factor
    const double sigma_avg_r = 0.5 * (S[c] + S[CELL(i - 1, j)]);
    const double cr_rp = -(rp_jp + rp) * t.CrRp[i];
    const double cr_pp = -0.5 * (ns * t.CrPp1[i] + ns_im * t.CrPp2[i]);
    const double cr_rr = t.InvDiffRmed[i] * (ns * t.CrRr1[i] + ns_im * t.CrRr2[i]);
    corr_r[c] = fast_div(t.CrScale[i] * (cr_rr + cr_rp + cr_pp), sigma_avg_r);
}

// pseudo-implicit limiter of a viscous velocity change, viscosity.cpp:395-399
__device__ __forceinline__ double stabilized(double dv, double dt, double c)
{
    const double a = 1.0 + dt * c;
    return dv * (1.0 / ((a > 0.0 ? a : 0.0) - dt * c));
}

// ---------------------------------------------------------------------------
// update_velocities_with_viscosity (viscosity.cpp:355-421) fused with SubStep3
// (SourceEuler.cpp:859-954: beta cooling, viscous heating, energy update,
// temperature floor).  mode bit 1: velocities, bit 2: heating/cooling rates,
// bit 4: energy update (init_euler's compute_heating_cooling_for_CFL uses 2).
// ---------------------------------------------------------------------------
__global__ void k_viscous(Geo g, Tables t, Phys ph, double dt, double beta_inv, int mode,
                          const double *__restrict__ S, const double *__restrict__ trr,
                          const double *__restrict__ tpp, const double *__restrict__ trp,
                          const double *__restrict__ divv, const double *__restrict__ nu,
                          const double *__restrict__ H, const double *__restrict__ S0,
                          const double *__restrict__ E0, double *__restrict__ vr,
                          double *__restrict__ vaz, double *__restrict__ E,
                          double *__restrict__ qplus, double *__restrict__ qminus,
                          const double *__restrict__ corr_phi, const double *__restrict__ corr_r)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;  // 0 .. nr - 1
    if (j >= nz) return;
    const size_t c = CELL(i, j);
    const int jp = jprev(j, nz), jn = jnext(j, nz);
    if (mode & 1) {
        if (i >= 1 && i < nr - 1) {
            const double sigma_avg = 0.5 * (S[c] + S[CELL(i, jp)]);
            double dVp = fast_div1(dt * t.InvRmed[i], sigma_avg) *
                         (t.TwoOverDRa2[i] * (t.RinfSq[i + 1] * trp[CELL(i + 1, j)] -
                                              t.RinfSq[i] * trp[c]) +
                          (tpp[c] - tpp[CELL(i, jp)]) * g.invdphi);
            if (ph.stabilize == 1) dVp = stabilized(dVp, dt, corr_phi[c]);
            vaz[c] += dVp;
        }
        if (i >= 2 && i < nr - 1) {
            const double sigma_avg = 0.5 * (S[c] + S[CELL(i - 1, j)]);
            double dVr =
                fast_div1(dt, sigma_avg) * ph.rvf * t.TwoOverRmedSum[i] *
                ((t.Rmed[i] * trr[c] - t.Rmed[i - 1] * trr[CELL(i - 1, j)]) * t.InvDiffRmed[i] +
                 (trp[CELL(i, jn)] - trp[c]) * g.invdphi - 0.5 * (tpp[c] + tpp[CELL(i - 1, j)]));
            if (ph.stabilize == 1) dVr = stabilized(dVr, dt, corr_r[c]);
            vr[c] += dVr;
        }
    }
    if (!(mode & 6) || !ph.adiabatic) return;
    double qp = 0.0, qm = 0.0;
    const double e = E[c];
    const double sig = S[c];
    const bool active = i >= 1 && i < nr - 1;
    if (active) {
        if (ph.cooling_beta) {
            // thermal_relaxation, SourceEuler.cpp:632-690
            double delta_E = e;
            if (ph.beta_ref == 1) {
                delta_E -= fast_div1(E0[c], S0[c]) * sig;
            } else if (ph.beta_ref == 2) {
                delta_E -= t.EModel[i] * sig;
            } else if (ph.beta_ref == 3) {
                delta_E -= sig * ph.emin_fac;
            }
            qm = 0.0 + delta_E * t.OmegaK[i] * beta_inv;
        }
        if (ph.heating_viscous) {
            // viscous_heating, SourceEuler.cpp:496-536
            const double n = nu[c];
            if (n != 0.0) {
                const double tau_r_phi = 0.25 * (trp[c] + trp[CELL(i + 1, j)] + trp[CELL(i, jn)] +
                                                 trp[CELL(i + 1, jn)]);
                const double t_rr = trr[c], t_pp = tpp[c], d = divv[c];
                double q = fast_rcp1(2.0 * n * sig) *
                           (t_rr * t_rr + 2 * (tau_r_phi * tau_r_phi) + t_pp * t_pp);
                q += (2.0 / 9.0) * n * sig * (d * d);
                q *= ph.hvf;
                qp = 0.0 + q;
            }
        }
        // radiative alpha factor, SourceEuler.cpp:905-912
        const double x = ph.mu_gm1_over_R * fast_rcp1(sig);
        const double x2 = x * x;
        const double inv_pow4 = x2 * x2;
        const double alpha = 1.0 + H[c] * ph.cool_const * inv_pow4 * (e * e * e);
        const double inv_alpha = fast_rcp1(alpha);
        qp *= inv_alpha;
        qm *= inv_alpha;
    }
    if (mode & 4) {
        double e_new = e;
        if (active) {
            e_new = e + dt * (qp - qm);
            if (sig < ph.sigma_floor10) {
                // TAU_EFF is zero on this path: the equilibrium energy is 0
                qm = qp;
                e_new = 0.0;
            }
        }
        E[c] = temperature_floor(e_new, sig, ph);
    }
    qplus[c] = qp;
    qminus[c] = qm;
}

// ---------------------------------------------------------------------------
// Ghost-ring hooks of apply_boundary_condition (boundary_conditions.cpp:65-114)
// ---------------------------------------------------------------------------
__device__ void ghost_hook(double *x, const double *x0, int kind, int outer, int vec, int nr,
                           int nz, int j, const double *val, const double *nu,
                           double rmed_edge, double omf)
{
    const int irad = vec ? nr : nr - 1;  // get_max_radial()
    const int edge = outer ? irad : 0;
    const int next = outer ? irad - 1 : 1;
    switch (kind) {
    case 1:  // zero_gradient.cpp:14-90
        if (!outer) {
            if (vec) {
                x[CELL(0, j)] = x[CELL(2, j)];
                x[CELL(1, j)] = x[CELL(2, j)];
            } else {
                x[CELL(0, j)] = x[CELL(1, j)];
            }
        } else {
            if (vec) {
                x[CELL(irad, j)] = x[CELL(irad - 2, j)];
                x[CELL(irad - 1, j)] = x[CELL(irad - 2, j)];
            } else {
                x[CELL(irad, j)] = x[CELL(irad - 1, j)];
            }
        }
        break;
    case 2:  // outflow.cpp:16-57
        if (!outer) {
            if (x[CELL(2, j)] > 0.0) {
                x[CELL(1, j)] = 0.0;
                x[CELL(0, j)] = 0.0;
            } else {
                x[CELL(1, j)] = x[CELL(2, j)];
                x[CELL(0, j)] = x[CELL(2, j)];
            }
        } else {
            if (x[CELL(irad - 2, j)] < 0.0) {
                x[CELL(irad - 1, j)] = 0.0;
                x[CELL(irad, j)] = 0.0;
            } else {
                x[CELL(irad - 1, j)] = x[CELL(irad - 2, j)];
                x[CELL(irad, j)] = x[CELL(irad - 2, j)];
            }
        }
        break;
    case 3:  // reference.cpp:17-88
        x[CELL(edge, j)] = x0[CELL(edge, j)];
        if (vec) x[CELL(next, j)] = x0[CELL(next, j)];
        break;
    case 4:   // keplerian_azimuthal.cpp:18-59: c v_K - r Omega_F
    case 10:  // balanced.cpp:20-66: sqrt(v^2) - Rb Omega_F
        x[CELL(edge, j)] = val[0] - rmed_edge * omf;
        break;
    case 5:  // diskmodel.cpp:33-77
        x[CELL(edge, j)] = val[0];
        break;
    case 6:  // reflecting.cpp:15-40
        x[CELL(edge, j)] = -x[CELL(outer ? irad - 2 : 2, j)];
        x[CELL(next, j)] = 0.0;
        break;
    case 7: {  // viscous.cpp:15-40 (inner edge)
        const double Nu = 0.5 * (nu[CELL(0, j)] + nu[CELL(1, j)]);
        x[CELL(1, j)] = val[1] * Nu;
        x[CELL(0, j)] = val[0] * Nu;
        break;
    }
    case 8:  // keplerian_radial.cpp:17-62
        x[CELL(edge, j)] = val[0];
        x[CELL(next, j)] = val[1];
        break;
    case 9:  // zero_shear.cpp:19-53: r_edge (v_active / r_active)
        x[CELL(edge, j)] = val[0] * (x[CELL(next, j)] / val[1]);
        break;
    default:
        break;
    }
}

__global__ void k_ghost(Geo g, Tables t, BcSpec bc, double omf, State s)
{
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nz) return;
    ghost_hook(s.sigma, s.sigma0, bc.sigma_in, 0, 0, nr, nz, j, bc.val_in[0], s.nu, 0, 0);
    ghost_hook(s.sigma, s.sigma0, bc.sigma_out, 1, 0, nr, nz, j, bc.val_out[0], s.nu, 0, 0);
    ghost_hook(s.energy, s.energy0, bc.energy_in, 0, 0, nr, nz, j, bc.val_in[1], s.nu, 0, 0);
    ghost_hook(s.energy, s.energy0, bc.energy_out, 1, 0, nr, nz, j, bc.val_out[1], s.nu, 0, 0);
    ghost_hook(s.vr, s.vr0, bc.vr_in, 0, 1, nr, nz, j, bc.val_in[2], s.nu, 0, 0);
    ghost_hook(s.vr, s.vr0, bc.vr_out, 1, 1, nr, nz, j, bc.val_out[2], s.nu, 0, 0);
    ghost_hook(s.vaz, s.vaz0, bc.vaz_in, 0, 0, nr, nz, j, bc.val_in[3], s.nu, t.Rmed[0], omf);
    ghost_hook(s.vaz, s.vaz0, bc.vaz_out, 1, 0, nr, nz, j, bc.val_out[3], s.nu, t.Rmed[nr - 1],
               omf);
}

// ---------------------------------------------------------------------------
// Radial transport, OneWindRad (TransportEuler.cpp:138-167) with
// compute_momenta_from_velocities (:471-493), compute_star_radial (:349-406)
// and VanLeerRadial (:545-620).  One thread sweeps one azimuth column over a
// chunk of rings with a register window, so every interface value is formed
// once; neighbouring chunks overlap by the 2-ring stencil halo only.
// Quantities: 0..3 momenta, 4 energy, 5 sigma (sigma is advected last, with
// the pre-transport sigma as the reference density).
// ---------------------------------------------------------------------------
// Specific quantities of ring i (quantity / sigma, TransportEuler.cpp:550-551
// via divise_polargrid, SideEuler.cpp:27-41): the momenta's specific values
// are the velocities themselves; energy needs one division.  Slot NQ holds
// sigma, whose star value is built from sigma itself (compute_star_radial on
// Density, :140).
template <int NQ>
__device__ __forceinline__ void rad_ring(int i, int j, int nz, const double *S, const double *vr,
                                         const double *vaz, const double *E, double omf,
                                         const Tables &t, double *w, double &sig)
{
    const double sg = S[CELL(i, j)];
    const double r = t.Rmed[i];
    w[0] = vr[CELL(i + 1, j)];
    w[1] = vr[CELL(i, j)];
    if (omf != 0.0) {
        w[2] = (vaz[CELL(i, jnext(j, nz))] + r * omf) * r;
        w[3] = (vaz[CELL(i, j)] + r * omf) * r;
    } else {
        w[2] = vaz[CELL(i, jnext(j, nz))] * r;
        w[3] = vaz[CELL(i, j)] * r;
    }
    if (NQ == 5) w[4] = fast_div1(E[CELL(i, j)], sg);
    w[NQ] = sg;
    sig = sg;
}

// One thread streams one azimuth column through a chunk of rings.  For every
// ring it forms the specific quantities and their limited slopes once; the
// interface between ring k-1 and k takes its upwind star value from ring k-1
// or k, so each flux is computed exactly once.
template <int NQ>
__global__ void k_transport_radial(Geo g, Tables t, double dt, double omf, int mc, int chunk,
                                   const double *__restrict__ S, const double *__restrict__ vr,
                                   const double *__restrict__ vaz, const double *__restrict__ E,
                                   double *__restrict__ mom0, double *__restrict__ mom1,
                                   double *__restrict__ mom2, double *__restrict__ mom3,
                                   double *__restrict__ E_out, double *__restrict__ S_out)
{
    constexpr int NW = NQ + 1;
    const int nz = g.nz, nr = g.nr;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nz) return;
    const int i0 = blockIdx.y * chunk;
    if (i0 >= nr) return;
    const int i1 = min(i0 + chunk, nr);
    const double dtdphi = dt * g.dphi;

    // rolling state: specific quantities of rings k-1 (wa) and k (wb), their
    // limited slopes (da, db), the upward difference of ring k (ub), the
    // sigma of ring k-1 / k
    double wa[NW] = {}, wb[NW] = {}, da[NW] = {}, db[NW] = {}, ub[NW] = {};
    double sa = 0.0, sb = 0.0;

    // slope of ring `ring` from its down/up differences (compute_star_radial,
    // :357-367: zero on the first and last ring), without van Leer's factor 2,
    // which the interpolation distance below carries instead of its 1/2
    auto lim = [&](int ring, double up, double down) -> double {
        if (ring <= 0 || ring >= nr - 1) return 0.0;
        return flux_limiter_unscaled(up, down, mc);
    };
    auto half = [&](double x) { return mc ? x * 0.5 : x; };

    // prime rings k-1 = i0-1 and k = i0 (their slopes need rings i0-2 .. i0+1)
    {
        double wm2[NW] = {}, wtmp[NW] = {}, s_tmp = 0.0;
        const int r0 = i0 - 1;
        if (r0 - 1 >= 0) rad_ring<NQ>(r0 - 1, j, nz, S, vr, vaz, E, omf, t, wm2, s_tmp);
        if (r0 >= 0) rad_ring<NQ>(r0, j, nz, S, vr, vaz, E, omf, t, wa, sa);
        rad_ring<NQ>(i0, j, nz, S, vr, vaz, E, omf, t, wb, sb);
        double downa[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            downa[q] = (r0 - 1 >= 0 && r0 >= 0) ? (wa[q] - wm2[q]) * t.InvDiffRmed[r0] : 0.0;
            ub[q] = r0 >= 0 ? (wb[q] - wa[q]) * t.InvDiffRmed[i0] : 0.0;  // up of k-1 = down of k
        }
        const bool has_next = i0 + 1 < nr;
        if (has_next) rad_ring<NQ>(i0 + 1, j, nz, S, vr, vaz, E, omf, t, wtmp, s_tmp);
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            da[q] = r0 >= 0 ? lim(r0, ub[q], downa[q]) : 0.0;
            const double up = has_next ? (wtmp[q] - wb[q]) * t.InvDiffRmed[i0 + 1] : 0.0;
            db[q] = lim(i0, up, ub[q]);
            ub[q] = up;
        }
        // keep ring i0+1 for the first shift
#pragma unroll
        for (int q = 0; q < NW; ++q) wm2[q] = wtmp[q];
        // wm2 now holds ring k+1; stash it in registers via the loop below
        double flux_prev[NW], q_prev[NW];
        double wn[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) wn[q] = wm2[q];
        double sn = has_next ? S[CELL(i0 + 1, j)] : 0.0;

        for (int k = i0; k <= i1; ++k) {
            // flux through the interface k (between rings k-1 and k)
            double flux[NW];
            if (k == 0 || k >= nr) {
#pragma unroll
                for (int q = 0; q < NW; ++q) flux[q] = 0.0;
            } else {
                const double v = vr[CELL(k, j)];
                const double base = dtdphi * t.Rinf[k];
                const double vdt = v * dt;
                double sstar;
                const bool up = positive(v);
                // DensityStar, then QRStar of every specific quantity
                // base sigma* v, the factor every quantity's flux shares
                if (up) {
                    const double f = half(t.Rmed[k] - t.Rmed[k - 1] - vdt);
                    sstar = wa[NQ] + f * da[NQ];
                    const double bsv = base * sstar * v;
#pragma unroll
                    for (int q = 0; q < NQ; ++q) flux[q] = (wa[q] + f * da[q]) * bsv;
                    flux[NQ] = bsv;
                } else {
                    const double f = half(t.Rmed[k + 1] - t.Rmed[k] + vdt);
                    sstar = wb[NQ] - f * db[NQ];
                    const double bsv = base * sstar * v;
#pragma unroll
                    for (int q = 0; q < NQ; ++q) flux[q] = (wb[q] - f * db[q]) * bsv;
                    flux[NQ] = bsv;
                }
            }
            if (k > i0) {
                // VanLeerRadial update of ring k-1 (:586-591)
                const int i = k - 1;
                const double invs = t.InvSurf[i];
                const size_t c = CELL(i, j);
                mom0[c] = q_prev[0] + (flux_prev[0] - flux[0]) * invs;
                mom1[c] = q_prev[1] + (flux_prev[1] - flux[1]) * invs;
                mom2[c] = q_prev[2] + (flux_prev[2] - flux[2]) * invs;
                mom3[c] = q_prev[3] + (flux_prev[3] - flux[3]) * invs;
                if (NQ == 5) E_out[c] = q_prev[4] + (flux_prev[4] - flux[4]) * invs;
                S_out[c] = q_prev[NQ] + (flux_prev[NQ] - flux[NQ]) * invs;
            }
            if (k < i1) {
                // conserved quantities of ring k for its update at interface k+1
#pragma unroll
                for (int q = 0; q < NW; ++q) flux_prev[q] = flux[q];
                q_prev[0] = sb * wb[0];
                q_prev[1] = sb * wb[1];
                q_prev[2] = sb * wb[2];
                q_prev[3] = sb * wb[3];
                if (NQ == 5) q_prev[4] = E[CELL(k, j)];
                q_prev[NQ] = sb;
                // advance: ring k becomes k-1, ring k+1 becomes k
                const bool more = k + 2 < nr;
                double w2[NW], s2 = 0.0;
                if (more) rad_ring<NQ>(k + 2, j, nz, S, vr, vaz, E, omf, t, w2, s2);
#pragma unroll
                for (int q = 0; q < NW; ++q) {
                    wa[q] = wb[q];
                    da[q] = db[q];
                    wb[q] = wn[q];
                    const double up = more ? (w2[q] - wn[q]) * t.InvDiffRmed[k + 2] : 0.0;
                    db[q] = lim(k + 1, up, ub[q]);
                    ub[q] = up;
                    wn[q] = more ? w2[q] : 0.0;
                }
                sa = sb;
                sb = sn;
                sn = s2;
            }
        }
    }
}

// flux limiters of the pair-arithmetic transports
__device__ __forceinline__ bool f2_same_sign_nonzero(f2 a, f2 b)
{
    // normalised pairs: the high part carries the sign, and is zero only
    // when the pair is
    const int ia = __float_as_int(a.h), ib = __float_as_int(b.h);
    return ((ia ^ ib) >= 0) && (ia & 0x7fffffff) != 0 && (ib & 0x7fffffff) != 0;
}
__device__ __forceinline__ bool f2_abs_less(f2 a, f2 b)
{
    const float ah = fabsf(a.h), bh = fabsf(b.h);
    if (ah != bh) return ah < bh;
    return (a.h < 0.f ? -a.l : a.l) < (b.h < 0.f ? -b.l : b.l);
}
// flux_limiter_unscaled in pairs, of two normalised differences (a
// difference whose low part were not folded in would carry most of the
// product a b in its low part, and the quotient's one-step correction would
// then keep only float precision of it)
__device__ __forceinline__ f2 lim_f2(f2 a, f2 b, int mc)
{
    const f2 zero{0.f, 0.f};
    if (mc) {
        const f2 mm = f2_same_sign_nonzero(a, b) ? (f2_abs_less(a, b) ? a : b) : zero;
        const f2 s = f2_sadd(a, b);
        const f2 c{__fmul_rn(0.5f, s.h), __fmul_rn(0.5f, s.l)};
        const f2 d{__fmul_rn(2.0f, mm.h), __fmul_rn(2.0f, mm.l)};
        if (f2_same_sign_nonzero(c, d)) return f2_abs_less(c, d) ? c : d;
        return zero;
    }
    // both sides formed, one selected (no branch)
    const f2 r = f2_sdiv(f2_smul(a, b), f2_sadd(a, b));
    return f2_same_sign_nonzero(a, b) ? r : zero;
}

// ---------------------------------------------------------------------------
// The radial transport with its arithmetic in float pairs (fp64_pair.cuh),
// the same column sweep as k_transport_radial: the specific quantities, their
// differences, limited slopes, star values and fluxes are pairs; the momenta
// Sigma v of the update are pair products; the new momenta, energy and sigma
// are joined into doubles once, energy and sigma by adding the pair update to
// their FP64 values.  The upwind choice and the interpolation distance come
// from the FP64 velocity.
// ---------------------------------------------------------------------------
// The specific quantities of ring i (slots 0 .. NQ - 1: the two radial
// momenta's velocities, the two angular momenta's, energy / sigma) and sigma
// (slot NQ)
template <int NQ>
__device__ __forceinline__ void rad_ring_f2(int i, int j, int nz, const double *S, const double *vr,
                                            const double *vaz, const double *E, double omf,
                                            const Tables &t, f2 *w)
{
    const f2 sg = f2_split(S[CELL(i, j)]);
    const f2 r{t.RmedHi[i], t.RmedLo[i]};
#pragma unroll
    for (int s = 0; s < NQ; ++s) {
        const int q = s;
        if (q == 0) w[s] = f2_split(vr[CELL(i + 1, j)]);
        if (q == 1) w[s] = f2_split(vr[CELL(i, j)]);
        if (q == 2 || q == 3) {
            f2 v = f2_split(vaz[CELL(i, q == 2 ? jnext(j, nz) : j)]);
            if (omf != 0.0) v = f2_sadd(v, f2_split(t.Rmed[i] * omf));
            w[s] = f2_smul(v, r);
        }
        if (q == 4) w[s] = f2_sdiv(f2_split(E[CELL(i, j)]), sg);
    }
    w[NQ] = sg;
}

template <int NQ>
__device__ __forceinline__ void radial_sweep_f2(const Geo &g, const Tables &t, double dt,
                                                double omf, int mc, int chunk, int j,
                                                const double *__restrict__ S,
                                                const double *__restrict__ vr,
                                                const double *__restrict__ vaz,
                                                const double *__restrict__ E,
                                                double *__restrict__ mom0,
                                                double *__restrict__ mom1,
                                                double *__restrict__ mom2,
                                                double *__restrict__ mom3,
                                                double *__restrict__ E_out,
                                                double *__restrict__ S_out)
{
    constexpr int NW = NQ + 1, NH = NQ;
    const int nz = g.nz, nr = g.nr;
    const int i0 = blockIdx.y * chunk;
    if (i0 >= nr) return;
    const int i1 = min(i0 + chunk, nr);
    const double dtdphi = dt * g.dphi;
    const f2 zero{0.f, 0.f};
    double *const outq[5] = {mom0, mom1, mom2, mom3, E_out};

    // rolling state as in k_transport_radial: rings k-1 (wa, da), k (wb, db,
    // ub: its upward difference) and k+1 (wn)
    f2 wa[NW], wb[NW], wn[NW], da[NW], db[NW], ub[NW];
#pragma unroll
    for (int q = 0; q < NW; ++q) wa[q] = wb[q] = wn[q] = da[q] = db[q] = ub[q] = zero;

    // slope of a ring from its up/down differences (zero on the first and
    // last ring), without van Leer's factor 2
    auto lim = [&](int ring, f2 up, f2 down) -> f2 {
        const f2 d = lim_f2(up, down, mc);
        return (ring <= 0 || ring >= nr - 1) ? zero : d;
    };
    auto dif = [&](int ring, const f2 &hi, const f2 &lo) {
        return f2_smul(f2_ssub(hi, lo), f2{t.InvDiffRmedHi[ring], t.InvDiffRmedLo[ring]});
    };

    // prime rings k-1 = i0-1 and k = i0 (their slopes need rings i0-2 .. i0+1)
    {
        f2 wm2[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) wm2[q] = zero;
        const int r0 = i0 - 1;
        if (r0 - 1 >= 0) rad_ring_f2<NQ>(r0 - 1, j, nz, S, vr, vaz, E, omf, t, wm2);
        if (r0 >= 0) rad_ring_f2<NQ>(r0, j, nz, S, vr, vaz, E, omf, t, wa);
        rad_ring_f2<NQ>(i0, j, nz, S, vr, vaz, E, omf, t, wb);
        f2 downa[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            downa[q] = (r0 - 1 >= 0 && r0 >= 0) ? dif(r0, wa[q], wm2[q]) : zero;
            ub[q] = r0 >= 0 ? dif(i0, wb[q], wa[q]) : zero;  // up of k-1 = down of k
        }
        const bool has_next = i0 + 1 < nr;
        if (has_next) rad_ring_f2<NQ>(i0 + 1, j, nz, S, vr, vaz, E, omf, t, wn);
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            da[q] = r0 >= 0 ? lim(r0, ub[q], downa[q]) : zero;
            const f2 up = has_next ? dif(i0 + 1, wn[q], wb[q]) : zero;
            db[q] = lim(i0, up, ub[q]);
            ub[q] = up;
        }
    }
    f2 flux_prev[NW];
    for (int k = i0; k <= i1; ++k) {
        // flux through the interface k (between rings k-1 and k)
        f2 flux[NW];
        if (k == 0 || k >= nr) {
#pragma unroll
            for (int q = 0; q < NW; ++q) flux[q] = zero;
        } else {
            const double v = vr[CELL(k, j)];
            const double vdt = v * dt;
            const bool up = positive(v);
            double fd = up ? t.Rmed[k] - t.Rmed[k - 1] - vdt : t.Rmed[k + 1] - t.Rmed[k] + vdt;
            if (mc) fd *= 0.5;
            // the star value from ring k-1 (+f da) or ring k (-f db)
            const f2 f = f2_split(up ? fd : -fd);
            f2 star[NW];
#pragma unroll
            for (int q = 0; q < NW; ++q)
                star[q] = f2_sfma(up ? wa[q] : wb[q], f, up ? da[q] : db[q]);
            // base sigma* v, the factor every quantity's flux shares
            const f2 bsv = f2_smul(f2_smul(f2_split(dtdphi * t.Rinf[k]), star[NH]), f2_split(v));
#pragma unroll
            for (int q = 0; q < NH; ++q) flux[q] = f2_smul(star[q], bsv);
            flux[NH] = bsv;
        }
        if (k > i0) {
            // VanLeerRadial update of ring k-1 (:586-591), whose specific
            // quantities are wa; its conserved momenta sigma w are formed
            // here and its sigma and energy re-read (cache hits), so that
            // the walk carries none of them
            const int i = k - 1;
            const f2 invs{t.InvSurfHi[i], t.InvSurfLo[i]};
            const size_t c = CELL(i, j);
#pragma unroll
            for (int s = 0; s < NW; ++s) {
                const f2 dq = f2_smul(f2_ssub(flux_prev[s], flux[s]), invs);
                if (s < 4 && s < NH)
                    outq[s][c] = f2_to_double(f2_sadd(f2_smul(wa[NH], wa[s]), dq));
                else if (s == 4 && NQ == 5) E_out[c] = E[c] + f2_to_double(dq);
                else S_out[c] = S[c] + f2_to_double(dq);
            }
        }
        if (k < i1) {
            // the fluxes through interface k, for ring k's update at k+1
#pragma unroll
            for (int q = 0; q < NW; ++q) flux_prev[q] = flux[q];
            // advance: ring k becomes k-1, ring k+1 becomes k
            const bool more = k + 2 < nr;
            f2 w2[NW];
#pragma unroll
            for (int q = 0; q < NW; ++q) w2[q] = zero;
            if (more) rad_ring_f2<NQ>(k + 2, j, nz, S, vr, vaz, E, omf, t, w2);
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                wa[q] = wb[q];
                da[q] = db[q];
                wb[q] = wn[q];
                const f2 up = more ? dif(k + 2, w2[q], wn[q]) : zero;
                db[q] = lim(k + 1, up, ub[q]);
                ub[q] = up;
                wn[q] = w2[q];
            }
        }
    }
}

// 64-thread blocks, 8 per SM: 128 registers (84 bytes of spills, to L1,
// which this kernel leaves unshared).  Measured on the 2048 x 6144 disk,
// ms per pass: 0.708 at 128 registers, 0.761 at 156 (no spills), 0.780 at 96.
template <int NQ>
__global__ void __launch_bounds__(64, 8) k_transport_radial_f2(Geo g, Tables t, double dt, double omf, int mc, int chunk,
                                      const double *__restrict__ S, const double *__restrict__ vr,
                                      const double *__restrict__ vaz, const double *__restrict__ E,
                                      double *__restrict__ mom0, double *__restrict__ mom1,
                                      double *__restrict__ mom2, double *__restrict__ mom3,
                                      double *__restrict__ E_out, double *__restrict__ S_out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.nz) return;
    radial_sweep_f2<NQ>(g, t, dt, omf, mc, chunk, j, S, vr, vaz, E, mom0, mom1, mom2, mom3,
                           E_out, S_out);
}

// ---------------------------------------------------------------------------
// Block reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Sum over the block; result valid in every thread.
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

__device__ double block_min(double v, double *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double x = lane < nw ? red[lane] : 1.0e300;
        x = warp_min(x);
        if (lane == 0) red[32] = x;
    }
    __syncthreads();
    return red[32];
}

// ---------------------------------------------------------------------------
// Azimuthal transport with FARGO orbital advection, OneWindTheta
// (TransportEuler.cpp:270-288): ring mean, ComputeConstantResidual (:207-236),
// QuantitiesAdvection with the residual then the uniform velocity (:292-304,
// ComputeStarTheta :416-466, VanLeerTheta :630-664) and AdvectSHIFT
// (:238-268).  One CTA owns one ring; the ring's sigma, specific quantity,
// slopes and fluxes live in shared memory (4 x naz doubles, up to 7040 cells;
// a per-ring global workspace stands in beyond that).  The face factor
// dxrad S* v / Surf that every quantity's flux shares is formed once per face.
// ---------------------------------------------------------------------------
// Each thread owns the cells j = threadIdx.x + n * blockDim.x, n < PER.

// One QuantitiesAdvection pass (TransportEuler.cpp:292-304) over the ring:
// DensityStar from sigma (ComputeStarTheta, :416-466), then VanLeerTheta
// (:630-664) for every quantity with DENSITY_INT = sigma, sigma last.  S holds
// sigma on entry and its advected value on exit.  v[n] is the owned cells'
// velocity (ignored when uniform).
template <int PER>
__device__ void ring_advection_pass(double *S, double *W, double *D, double *F,
                                    double *const *qrow, int nq, double *v, double dt,
                                    double dxtheta, double half_invdx, double dxrad_invsurf,
                                    int nz, int mc, bool uniform, double vconst)
{
    const int tid = threadIdx.x, bs = blockDim.x;
    // the upwind cell and interpolation distance are kept per cell up to 8
    // cells per thread and recomputed beyond (registers)
    constexpr bool KEEP = PER <= 8;
    double invs[PER], cf[PER], am[KEEP ? PER : 1];
    int up[KEEP ? PER : 1];
    // D holds the slopes without their constant factor (van Leer's 2 and
    // 1/(2 dx)); the interpolation distance carries it: with
    // k = 2 / (2 dx) (van Leer) or 1 / (2 dx) (MC), the distance is
    // k (dx - v dt) or -k (dx + v dt).  The velocities are scaled by k dt
    // once (in place: the uniform pass does not read them), so a distance
    // costs one addition where it is recomputed.
    const double kfac = mc ? half_invdx : 2.0 * half_invdx;
    const double kdt = kfac * dt;
    const double dxk = dxtheta * kfac;
    const double cvel = dxrad_invsurf / kdt;  // dxrad S* v / Surf = cvel S* (k dt v)
    const double vkc = vconst * kdt;
    if (!uniform) {
#pragma unroll
        for (int n = 0; n < PER; ++n) v[n] *= kdt;
    }
    auto upwind = [&](int n, int j, int &u, double &a) {
        const double vk = uniform ? vkc : v[n];
        const bool pos = positive(vk);
        u = pos ? (j == 0 ? nz - 1 : j - 1) : j;
        a = pos ? dxk - vk : -(dxk + vk);
    };
    // DensityStar
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            const int jp = j == nz - 1 ? 0 : j + 1;
            const int jm = j == 0 ? nz - 1 : j - 1;
            D[j] = flux_limiter_unscaled(S[jp] - S[j], S[j] - S[jm], mc);
            invs[n] = fast_rcp(S[j]);
        }
    }
    __syncthreads();
    // per face j: the upwind cell, the signed interpolation distance
    // (dx - ksi, or -(dx + ksi)) and dxrad S* v / Surf, the factor every
    // quantity's flux shares
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            int u;
            double a;
            upwind(n, j, u, a);
            if (KEEP) {
                up[n] = u;
                am[n] = a;
            }
            cf[n] = cvel * (S[u] + a * D[u]) * (uniform ? vkc : v[n]);
        }
    }
    __syncthreads();
    // three barriers per quantity: specific values, slopes, fluxes (the
    // update reads F while the next quantity fills W and D)
    for (int q = 0; q < nq; ++q) {
        double *Q = qrow[q];
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
                const int jp = j == nz - 1 ? 0 : j + 1;
                const int jm = j == 0 ? nz - 1 : j - 1;
                D[j] = flux_limiter_unscaled(W[jp] - W[j], W[j] - W[jm], mc);
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) {
                int u;
                double a;
                if (KEEP) {
                    u = up[n];
                    a = am[n];
                } else {
                    upwind(n, j, u, a);
                }
                F[j] = (W[u] + a * D[u]) * cf[n];
            }
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = tid + n * bs;
            if (j < nz) Q[j] += F[j] - F[j == nz - 1 ? 0 : j + 1];
        }
    }
    // sigma: its specific quantity is exactly 1, so QRStar == 1 (the barrier
    // lets the last quantity's update finish reading F)
    __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) F[j] = cf[n];
    }
    __syncthreads();
    double f[PER];
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) f[n] = S[j] + (F[j] - F[j == nz - 1 ? 0 : j + 1]);
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
__global__ void __launch_bounds__(512) k_transport_azimuthal(Geo g, Tables t, double dt, int mc,
                                                             int fast, int nq,
                                      const double *__restrict__ vaz, double *mom0, double *mom1,
                                      double *mom2, double *mom3, double *E, double *S,
                                      double *ring_ws)
{
    extern __shared__ double smem[];
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x;
    const int tid = threadIdx.x, bs = blockDim.x;
    const size_t row = (size_t)i * nz;
    double *base = ring_ws ? ring_ws + (size_t)i * 4 * nz : smem;
    double *Sr = base, *W = base + nz, *D = base + 2 * nz, *F = base + 3 * nz;

    // compute_average_azimuthal_velocity, :174-189
    double vown[PER];
    double part = 0.0;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            vown[n] = vaz[row + j];
            part += vown[n];
        }
    }
    const double vmean = block_sum(part, red) / (double)nz;
    // ComputeConstantResidual, :207-236: FP64 shift phase of the ring
    const double Ntilde = vmean * t.InvRmed[i] * dt * g.invdphi;
    const double Nround = floor(Ntilde + 0.5);
    const int nshift = (int)Nround;
    const double invdt = 1.0 / dt;
    const double vt = (Ntilde - Nround) * t.Rmed[i] * invdt * g.dphi;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (j < nz) {
            double vres = vown[n] - vmean;
            if (!fast) vres = vt + vres;
            vown[n] = vres;
            Sr[j] = S[row + j];
        }
    }
    __syncthreads();

    double *qrow[5] = {mom0 + row, mom1 + row, mom2 + row, mom3 + row, E + row};
    const double dxtheta = g.dphi * t.Rmed[i];
    const double half_invdx = 0.5 * (1.0 / dxtheta);
    const double dxrad = (t.Rsup[i] - t.Rinf[i]) * dt;
    const double invsurf = t.InvSurf[i];
    ring_advection_pass<PER>(Sr, W, D, F, qrow, nq, vown, dt, dxtheta, half_invdx,
                             dxrad * invsurf, nz, mc, false, 0.0);
    if (fast) {
        ring_advection_pass<PER>(Sr, W, D, F, qrow, nq, vown, dt, dxtheta, half_invdx,
                                 dxrad * invsurf, nz, mc, true, vt);
    }
    // AdvectSHIFT of every quantity, sigma last
    for (int q = 0; q <= nq; ++q) {
        double *Q = q < nq ? qrow[q] : S + row;
        const double *src = q < nq ? qrow[q] : Sr;
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
}

// ---------------------------------------------------------------------------
// The same azimuthal transport with its arithmetic in float pairs
// (fp64_pair.cuh).  The ring pass above is bound by GB300's FP64 pipe (about
// 1.6 FP64 results per clock per SM against about 113 FP32); here every
// slope, star value and flux is formed in pair arithmetic (48 significant
// bits, errors within a few 2^-47 of the operands), the doubles are split and
// joined on the integer pipe, and FP64 is kept for the state: each quantity's
// update Q += F_j - F_j+1 adds the pair flux difference, joined into a
// double, to the FP64 value, so what a step loses is the pair's rounding of
// the fluxes, not of the state.  The upwind choice and the interpolation
// distance come from the FP64 velocity as before; the ring mean and the FARGO
// shift phase stay in FP64.
//
// Layout as in the FP64 pass (4 x naz x 8 bytes of shared memory, or the
// per-ring global workspace): the sigma pair, the specific quantity, the
// slopes and the fluxes, each a pair.  Sigma's FP64 values are updated in
// place in its global row (the block owns the ring), the transported
// quantities in theirs, and AdvectSHIFT stages each row through shared
// memory.
// ---------------------------------------------------------------------------
// One QuantitiesAdvection pass (TransportEuler.cpp:292-304) in pairs.  SP
// holds sigma's pair, Sg its FP64 row; both advance.  v[n] is the owned
// cells' FP64 velocity (ignored when uniform).
//
// Each face forms the limited slope of its upwind cell itself, from that
// cell and its two neighbours, instead of reading a slope array: every
// cell's slope is still formed once per face that uses it (van Leer's
// upwind cell of face j is j - 1 or j), the slope array and its barrier
// go, and shared memory holds the face factors in their place, so that a
// thread keeps only its faces' interpolation distances in registers.
//
// The four ring arrays carry the periodic neighbours as halo cells: index -2
// and -1 hold cells nz - 2 and nz - 1, index nz holds cell 0, written by the
// owners of those cells with the cell itself, so that no index wraps.
// EXACT (nz == PER blockDim.x): every thread owns PER cells; otherwise the
// loops compute with the index clamped into the ring and guard only their
// stores.  Either way the loop bodies have no branch.
// The quantity rows, chosen by a select chain: an indexed array of their
// pointers would sit in local memory and put a load before every row access.
struct QRows {
    double *r0, *r1, *r2, *r3, *r4;
    __device__ __forceinline__ double *operator[](int q) const
    {
        return q == 0 ? r0 : q == 1 ? r1 : q == 2 ? r2 : q == 3 ? r3 : r4;
    }
};

// The face fluxes of an exact ring with whole warps (SHFL): each cell's
// update F[j] - F[j + 1] takes the right neighbour's flux from the next lane
// by a shuffle, so no flux array exists.  Its shared memory holds instead
// the quantity's FP64 value of each cell, read from global memory once per
// quantity and pass (the specific value and the update both use it).  Lane
// 31's right neighbour is lane 0 of the next warp (of the next slot after
// the last warp, cell 0 after the last cell): lane 0 publishes its flux, lane
// 31 its flux and value, and after the quantity's closing barrier threads
// 0 .. K - 1 (K = PER x warps, one per lane-31 cell) complete those updates.
// The exchange buffers alternate with the quantity, so that the next
// quantity's writes never meet this one's deferred reads.
template <int K>
struct PairEdges {
    f2 first[2][K];   // lane 0's flux, slot-major: n x warps + warp
    f2 last[2][K];    // lane 31's flux
    double val[2][K]; // lane 31's quantity value
};

template <int PER, int NQ, bool EXACT, bool SHFL, int K>
__device__ void ring_advection_pass_f2(double *Sg, f2 *SP, f2 *W, f2 *CF, f2 *F,
                                       PairEdges<K> &xe, const QRows &qrow, const double *v,
                                       double dt, double dxtheta, double half_invdx,
                                       double dxrad_invsurf, int nz, int mc, bool uniform,
                                       double vconst)
{
    static_assert(!SHFL || EXACT, "the shuffled fluxes need an exact ring");
    const int tid = threadIdx.x, bs = blockDim.x;
    // the slopes carry no constant factor; the distance does (as in
    // ring_advection_pass): k (dx - v dt) or -k (dx + v dt), k = 1 / dx
    // (van Leer) or 1 / (2 dx) (MC)
    const double kfac = mc ? half_invdx : 2.0 * half_invdx;
    const double kdt = kfac * dt;
    const double dxk = dxtheta * kfac;
    const f2 cvel = f2_split(dxrad_invsurf / kdt);
    f2 am[PER];
    unsigned pos = 0;  // bit n: the upwind cell of face tid + n bs is its left neighbour
    auto cell = [&](int n) { return EXACT ? tid + n * bs : min(tid + n * bs, nz - 1); };
    auto owned = [&](int n) { return EXACT || tid + n * bs < nz; };
    // X[j] and its halo copy (cells nz - 2, nz - 1 at -2, -1; cell 0 at nz);
    // n is the compile-time cell slot of j, so that in an exact ring only the
    // first and last slots test for the halo
    auto put = [&](f2 *X, int j, f2 x, int n) {
        X[j] = x;
        if (EXACT) {
            if (n == 0 && tid == 0) X[nz] = x;
            if (n == PER - 1 && tid >= bs - 2) X[j - nz] = x;
        } else {
            if (j >= nz - 2) X[j - nz] = x;
            if (j == 0) X[nz] = x;
        }
    };
    // the star value at a face of the quantity X from its upwind cell u
    // (u in -1 .. nz - 1)
    auto star = [&](const f2 *X, int u, f2 a) {
        const f2 x = X[u];
        const f2 d = lim_f2(f2_ssub(X[u + 1], x), f2_ssub(x, X[u - 1]), mc);
        return f2_sfma(x, a, d);
    };
    // DensityStar and the face factor dxrad S* v / Surf every flux shares
    const double vu = vconst * kdt;
    const bool pu = positive(vu);
    const f2 au = f2_split(pu ? dxk - vu : -(dxk + vu));
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = cell(n);
        const double vk = uniform ? vu : v[n] * kdt;
        const bool p = positive(vk);
        am[n] = uniform ? au : f2_split(p ? dxk - vk : -(dxk + vk));
        pos |= (unsigned)p << n;
        const f2 c = f2_smul(f2_smul(cvel, star(SP, p ? j - 1 : j, am[n])), f2_split(vk));
        if (owned(n)) put(CF, j, c, n);
    }
    if constexpr (SHFL) {
        double *Qs = reinterpret_cast<double *>(F);
        const int lane = tid & 31, w = tid >> 5, nw = bs >> 5, kk = PER * nw;
        // the lane-31 cells' updates of quantity q (slot n, warp ww: cell
        // n bs + 32 ww + 31; the next entry is its right neighbour's lane 0)
        auto complete = [&](int q) {
            if (tid < kk) {
                const int b = q & 1, nx = tid + 1 == kk ? 0 : tid + 1;
                const int n = tid / nw, ww = tid - n * nw;
                qrow[q][n * bs + 32 * ww + 31] =
                    xe.val[b][tid] + f2_to_double(f2_ssub(xe.last[b][tid], xe.first[b][nx]));
            }
        };
#pragma unroll 1
        for (int q = 0; q < NQ; ++q) {
            if (q > 0) complete(q - 1);
            double *Q = qrow[q];
            const int b = q & 1;
#pragma unroll
            for (int n = 0; n < PER; ++n) {
                const int j = tid + n * bs;
                const double x = Q[j];
                Qs[j] = x;
                if (lane == 31) xe.val[b][n * nw + w] = x;
                put(W, j, f2_sdiv(f2_split(x), SP[j]), n);
            }
            __syncthreads();
#pragma unroll
            for (int n = 0; n < PER; ++n) {
                const int j = tid + n * bs;
                const f2 f = f2_smul(star(W, (pos >> n) & 1u ? j - 1 : j, am[n]), CF[j]);
                const f2 fr{__shfl_down_sync(0xffffffffu, f.h, 1),
                            __shfl_down_sync(0xffffffffu, f.l, 1)};
                if (lane == 0) xe.first[b][n * nw + w] = f;
                if (lane == 31) xe.last[b][n * nw + w] = f;
                const double qn = Qs[j] + f2_to_double(f2_ssub(f, fr));
                if (lane != 31) Q[j] = qn;
            }
            __syncthreads();
        }
        if (NQ > 0) complete(NQ - 1);
    } else {
    // per quantity: specific values (with the previous quantity's update),
    // then the fluxes
#pragma unroll 1
    for (int q = 0; q <= NQ; ++q) {
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = cell(n);
            if (q > 0) {
                double *Qp = qrow[q - 1];
                const double qn = Qp[j] + f2_to_double(f2_ssub(F[j], F[j + 1]));
                if (owned(n)) Qp[j] = qn;
            }
            if (q < NQ) {
                const f2 w = f2_sdiv(f2_split(qrow[q][j]), SP[j]);
                if (owned(n)) put(W, j, w, n);
            }
        }
        if (q == NQ) break;
        __syncthreads();
#pragma unroll
        for (int n = 0; n < PER; ++n) {
            const int j = cell(n);
            const f2 f = f2_smul(star(W, (pos >> n) & 1u ? j - 1 : j, am[n]), CF[j]);
            if (owned(n)) put(F, j, f, n);
        }
        __syncthreads();
    }
    }
    // sigma: QRStar == 1, the flux is the face factor itself (CF is
    // complete: the barriers of the quantities, or this one when there are
    // none, separate its writes from these reads)
    if (NQ == 0) __syncthreads();
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = cell(n);
        // nothing reads SP in this phase
        const double s = Sg[j] + f2_to_double(f2_ssub(CF[j], CF[j + 1]));
        const f2 sp = f2_split(s);
        if (owned(n)) {
            Sg[j] = s;
            put(SP, j, sp, n);
        }
    }
    __syncthreads();
}

// Shared memory of the pair kernel per ring: four arrays of nz + 4 pairs
// (two halo cells on either side)
__host__ __device__ constexpr size_t pair_ring_f2s(int nz) { return (size_t)4 * (nz + 4); }

// WS: the ring's arrays in the per-ring global workspace (rings beyond the
// shared memory), else in shared memory
// The integer shift of AdvectSHIFT is not applied here: ring_shift[i]
// receives it (in [0, nz)), and the velocity rebuild (k_finish_p) reads each
// ring's transported cells at their shifted places.
template <int PER, int MAXT, int NQ, bool WS, bool EXACT>
__global__ void __launch_bounds__(MAXT) k_transport_azimuthal_f2(
    Geo g, Tables t, double dt, int mc, int fast, const double *__restrict__ vaz, double *mom0,
    double *mom1, double *mom2, double *mom3, double *E, double *S, double *ring_ws,
    int *__restrict__ ring_shift)
{
    // the shuffled fluxes on exact rings of up to 6 cells per thread (their
    // exchange buffers, 9 KB at 6 x 1024, fit beside the ring's arrays)
    constexpr bool SHFL = EXACT && !WS && PER <= 6;
    constexpr int K = SHFL ? PER * (MAXT / 32) : 1;
    extern __shared__ double smem[];
    __shared__ double red[33];
    __shared__ PairEdges<K> xe;
    const int nz = g.nz;
    const int i = blockIdx.x;
    const int tid = threadIdx.x, bs = blockDim.x;
    const size_t row = (size_t)i * nz;
    f2 *base = WS ? reinterpret_cast<f2 *>(ring_ws) + (size_t)i * pair_ring_f2s(nz)
                  : reinterpret_cast<f2 *>(smem);
    f2 *SP = base + 2, *W = SP + (nz + 4), *CF = W + (nz + 4), *F = CF + (nz + 4);
    double *Sg = S + row;
    auto owned = [&](int n) { return EXACT || tid + n * bs < nz; };
    // the ring's transported rows come from DRAM (the radial pass wrote the
    // whole disk since): ask L2 for all of them now, so that their reads in
    // the first pass, one quantity after the other, find them there
    {
        const int lines = (nz + 15) >> 4;  // 128-byte lines of a row
        const double *rows[6] = {Sg, mom0 + row, mom1 + row, mom2 + row, mom3 + row, E + row};
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            if (r == 5 && NQ < 5) break;
            for (int l = tid; l < lines; l += bs)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(rows[r] + min(16 * l, nz - 1)));
        }
    }

    // compute_average_azimuthal_velocity, :174-189
    double vown[PER];
    double part = 0.0;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (owned(n)) {
            vown[n] = vaz[row + j];
            part += vown[n];
        }
    }
    const double vmean = block_sum(part, red) / (double)nz;
    // ComputeConstantResidual, :207-236: FP64 shift phase of the ring
    const double Ntilde = vmean * t.InvRmed[i] * dt * g.invdphi;
    const double Nround = floor(Ntilde + 0.5);
    const int nshift = (int)Nround;
    const double invdt = 1.0 / dt;
    const double vt = (Ntilde - Nround) * t.Rmed[i] * invdt * g.dphi;
#pragma unroll
    for (int n = 0; n < PER; ++n) {
        const int j = tid + n * bs;
        if (owned(n)) {
            double vres = vown[n] - vmean;
            if (!fast) vres = vt + vres;
            vown[n] = vres;
            const f2 sp = f2_split(Sg[j]);
            SP[j] = sp;
            if (j >= nz - 2) SP[j - nz] = sp;
            if (j == 0) SP[nz] = sp;
        }
    }
    __syncthreads();

    const QRows qrow{mom0 + row, mom1 + row, mom2 + row, mom3 + row, E + row};
    const double dxtheta = g.dphi * t.Rmed[i];
    const double half_invdx = 0.5 * (1.0 / dxtheta);
    const double dxrad = (t.Rsup[i] - t.Rinf[i]) * dt;
    const double invsurf = t.InvSurf[i];
    ring_advection_pass_f2<PER, NQ, EXACT, SHFL>(Sg, SP, W, CF, F, xe, qrow, vown, dt, dxtheta,
                                                 half_invdx, dxrad * invsurf, nz, mc, false, 0.0);
    if (fast) {
        ring_advection_pass_f2<PER, NQ, EXACT, SHFL>(Sg, SP, W, CF, F, xe, qrow, vown, dt,
                                                     dxtheta, half_invdx, dxrad * invsurf, nz,
                                                     mc, true, vt);
    }
    // AdvectSHIFT (:238-268) is the rebuild's: it reads cell j of this ring
    // from cell j - nshift
    if (threadIdx.x == 0) ring_shift[i] = ((nshift % nz) + nz) % nz;
}

// ---------------------------------------------------------------------------
// compute_velocities_from_momenta (TransportEuler.cpp:498-535), the sigma
// floor (assure_minimum_value, SourceEuler.cpp:102-134) and the temperature
// floor (Transport, TransportEuler.cpp:122-127).  Reads the transported
// buffers, writes the new state buffers.
// ---------------------------------------------------------------------------
__global__ void k_finish(Geo g, Tables t, Phys ph, double omf, const double *__restrict__ mom0,
                         const double *__restrict__ mom1, const double *__restrict__ mom2,
                         const double *__restrict__ mom3, const double *__restrict__ S_t,
                         const double *__restrict__ E_t, const double *__restrict__ vr_in,
                         double *__restrict__ vr_out, double *__restrict__ vaz_out,
                         double *__restrict__ S_out, double *__restrict__ E_out)
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
    const double s = S_t[c];
    if (i == 0) {
        vr_out[c] = 0.0;
    } else {
        const size_t cm = CELL(i - 1, j);
        vr_out[c] = fast_div(mom0[cm] + mom1[c], S_t[cm] + s);
    }
    const int jm = jprev(j, nz);
    const size_t cjm = CELL(i, jm);
    vaz_out[c] = fast_div(mom2[cjm] + mom3[c], S_t[cjm] + s) * t.InvRmed[i] - t.Rmed[i] * omf;
    const double sf = s < ph.sigma_min ? ph.sigma_min : s;
    S_out[c] = sf;
    if (ph.adiabatic) E_out[c] = temperature_floor(E_t[c], sf, ph);
}

// ---------------------------------------------------------------------------
// damping (boundary_conditions/damping.cpp:311-752, :754-776): one CTA per
// ring of the damping zones; the "mean" kind writes X0(ring, 0) like the
// reference does.
// ---------------------------------------------------------------------------
__device__ void damp_ring(double *X, double *X0, const DampQ &d, int i, int nz, int outer,
                          double dt, double *red)
{
    const int kind = outer ? d.kind_out : d.kind_in;
    const size_t row = (size_t)i * nz;
    double x0c = 0.0;
    if (kind == 3) {
        double part = 0.0;
        for (int j = threadIdx.x; j < nz; j += blockDim.x) part += X[row + j];
        const double mean = block_sum(part, red) / nz;
        if (threadIdx.x == 0) X0[row] = mean;
        x0c = mean;
    } else if (kind == 2) {
        x0c = outer ? 0.0 : d.x0_zero_in;
    }
    const double factor = outer ? d.fac_out[i] : d.fac_in[i];
    const double tau = outer ? d.tau_out : d.tau_in;
    const double ef = exp(-dt * factor / tau);
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const double x0 = kind == 1 ? X0[row + j] : x0c;
        X[row + j] = (X[row + j] - x0) * ef + x0;
    }
    __syncthreads();
}

__global__ void k_damping(Geo g, Damping dm, double dt, const int *__restrict__ rings,
                          State s)
{
    __shared__ double red[33];
    const int nz = g.nz, nr = g.nr;
    const int i = rings[blockIdx.x];
    // the four damped fields are independent: one block per (ring, field)
    const int q = blockIdx.y;
    double *X[4] = {s.vr, s.vaz, s.sigma, s.energy};
    double *X0[4] = {s.vr0, s.vaz0, s.sigma0, s.energy0};
    const DampQ &d = dm.q[q];
    const int size = d.vector ? nr + 1 : nr;
    if (d.kind_in != 0 && d.active_in && i <= d.limit_in) {
        damp_ring(X[q], X0[q], d, i, nz, 0, dt, red);
    }
    if (d.kind_out != 0 && d.active_out && i >= d.limit_out && i < size) {
        damp_ring(X[q], X0[q], d, i, nz, 1, dt, red);
    }
}

// ---------------------------------------------------------------------------
// recalculate_derived_disk_quantities (SourceEuler.cpp:225-249) fused with
// cfl::condition_cfl (cfl.cpp:185-382).  One CTA per ring; the ring means of
// v_phi for rings i and i + 1 are block reductions; the step minimum is an
// atomic min on the ordered bit pattern of the (positive) dt.
// mode bit 1: derived quantities (bit 2: include T, c_s, H for init),
// bit 4: CFL.
// ---------------------------------------------------------------------------
// The CFL time step of one cell in FP32, to screen the cells whose FP64 dt
// can be the ring's minimum.  The differences that cancel (v_phi - mean,
// the velocity jumps, Q+ - Q-) are taken in FP64 by the caller; the values
// reach FP32 by truncating their FP64 bits to 20 mantissa bits on the integer
// pipe (no FP64 instruction), so every term, and the result, is within
// 2^-19 of its FP64 value.
struct CflRing32 {
    float inv_cell, inv_cell2, inv_drsup, inv_dxtheta, inv_rmed, invdphi, four_C2, inv_hc, cfl;
};

__device__ __forceinline__ float dtrunc_f(double x)
{
    const int hi = __double2hiint(x);
    const int em = ((hi >> 20) & 0x7ff) - 1023 + 127;
    if (em <= 0) return 0.f;
    if (em >= 255) return __int_as_float((hi & 0x80000000) | 0x7f800000);
    return __int_as_float((hi & 0x80000000) | (em << 23) | ((hi & 0xfffff) << 3));
}

__device__ __forceinline__ float cfl_cell32(const CflRing32 &t, const Phys &ph, int sn,
                                            double c_s, double n, double vr0, double vr1,
                                            double va, double va1, double vm0, double qp,
                                            double qm, double e, double cphi, double cr)
{
    const float vres = dtrunc_f(ph.fast_transport ? va - vm0 : va);
    const float i1 = dtrunc_f(c_s) * t.inv_cell;
    const float i2 = dtrunc_f(vr0) * t.inv_drsup;
    const float i3 = vres * t.inv_dxtheta;
    float i4;
    if (sn) {
        const float dvR = dtrunc_f(vr0 - vr1), dvA = dtrunc_f(va - va1);
        i4 = t.four_C2 * fmaxf(fmaxf(dvR, 0.f) * t.inv_drsup, fmaxf(dvA, 0.f) * t.inv_dxtheta);
    } else {
        const float eps_rr = dtrunc_f(vr1 - vr0) * t.inv_drsup;
        const float eps_pp =
            t.inv_rmed * (dtrunc_f(va1 - va) * t.invdphi + 0.5f * (dtrunc_f(vr1) + dtrunc_f(vr0)));
        i4 = t.four_C2 * fmaxf(-(eps_rr + eps_pp), 0.f);
    }
    float i5 = 4.f * dtrunc_f(n) * t.inv_cell2;
    float i6 = 0.f;
    if (ph.adiabatic) i6 = t.inv_hc * fabsf(dtrunc_f(qp - qm) / dtrunc_f(e));
    if (ph.leapfrog) {
        i4 *= 0.6f;
        i5 *= 0.6f;
        i6 *= 0.6f;
    }
    const float sum = i1 * i1 + i2 * i2 + i3 * i3 + i4 * i4 + i5 * i5 + i6 * i6;
    float d = t.cfl / sqrtf(sum);
    if (ph.stabilize == 2) {
        const float fc = fminf(dtrunc_f(cphi), dtrunc_f(cr));
        if (fc != 0.f) d = fminf(d, -t.cfl / fc);
    }
    return d;
}

__device__ __forceinline__ float block_min_f(float v, float *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        float x = lane < nw ? red[lane] : 3.0e38f;
        for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_down_sync(0xffffffffu, x, o));
        if (lane == 0) red[32] = x;
    }
    __syncthreads();
    return red[32];
}

// The FP64 time step of cell (i, j) (cfl.cpp:185-382): the six inverse times
// (sound speed, radial and azimuthal transport, artificial viscosity,
// viscosity, heating and cooling; LeapFrog's 0.6 on the last three) into
// inv[], CFL / sqrt of their squares, and StabilizeViscosity 2's limit.
__device__ __forceinline__ double cfl_cell64(const Geo &g, const Tables &t, const Phys &ph,
                                             int sn, int i, int j, double c_s, double n,
                                             const double *__restrict__ vr,
                                             const double *__restrict__ vaz, double vm0,
                                             const double *__restrict__ qplus,
                                             const double *__restrict__ qminus,
                                             const double *__restrict__ E,
                                             const double *__restrict__ corr_phi,
                                             const double *__restrict__ corr_r, double inv[6])
{
    const int nz = g.nz;
    const size_t row = (size_t)i * nz;
    const size_t c = row + j;
    const double va = vaz[c];
    const double vres = ph.fast_transport ? va - vm0 : va;
    const double invdt1 = c_s * t.InvCell[i];
    const double invdt2 = vr[c] * t.InvDiffRsup[i];
    const double invdt3 = vres * t.InvDxTheta[i];
    const double vr1 = vr[c + nz];
    const double va1 = vaz[row + (j == nz - 1 ? 0 : j + 1)];
    double invdt4;
    if (sn) {
        double dvR = vr1 - vr[c];
        double dvA = va1 - va;
        dvR = dvR > 0.0 ? 0.0 : -dvR;
        dvA = dvA > 0.0 ? 0.0 : -dvA;
        const double a = dvR * t.InvDiffRsup[i], b = dvA * t.InvDxTheta[i];
        invdt4 = ph.four_C2 * (dbits(a) > dbits(b) ? a : b);
    } else {
        const double eps_rr = (vr1 - vr[c]) * t.InvDiffRsup[i];
        const double eps_pp = t.InvRmed[i] * ((va1 - va) * g.invdphi + 0.5 * (vr1 + vr[c]));
        const double d = eps_rr + eps_pp;
        const double mdiv = -(d < 0.0 ? d : 0.0);
        invdt4 = ph.four_C2 * mdiv;
    }
    double invdt5 = 4.0 * n * t.InvCell2[i];
    double invdt6 = 0.0;
    if (ph.adiabatic) {
        invdt6 = ph.inv_hc_limit * fabs(fast_div(qplus[c] - qminus[c], E[c]));
    }
    if (ph.leapfrog) {
        // LeapFrog applies the source terms twice with dt/2 (cfl.cpp:254-317)
        invdt4 *= 0.6;
        invdt5 *= 0.6;
        invdt6 *= 0.6;
    }
    double dt_cell =
        fast_div(ph.cfl, sqrt(invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 +
                              invdt4 * invdt4 + invdt5 * invdt5 + invdt6 * invdt6));
    if (ph.stabilize == 2) {
        // viscous stability limit, cfl.cpp:332-351
        const double cphi = corr_phi[c], cr = corr_r[c];
        const double cc = cr < cphi ? cr : cphi;
        if (cc != 0.0) {
            const double dt_stable = -fast_div(ph.cfl, cc);
            if (dt_stable < dt_cell) dt_cell = dt_stable;
        }
    }
    inv[0] = invdt1;
    inv[1] = invdt2;
    inv[2] = invdt3;
    inv[3] = invdt4;
    inv[4] = invdt5;
    inv[5] = invdt6;
    return dt_cell;
}

// The sum of the squares of cell (i, j)'s six inverse times in float pairs
// (cfl_cell64's; LeapFrog's 0.6 on the last three): the cell's step is CFL
// over its square root, so the ring's smallest step is CFL / sqrt of the
// ring's largest sum, formed once per ring; within a few 2^-46 of the FP64
// value, far inside the CFL step's bar.  The
// differences of stored velocities and Q+ - Q- are FP64 subtractions (they
// cancel); StabilizeViscosity 2 is served by the FP64 path.
__device__ __forceinline__ f2 cfl_cell_f2(const Geo &g, const Tables &t, const Phys &ph, int sn,
                                          int i, int j, f2 c_s, f2 n,
                                          const double *__restrict__ vr,
                                          const double *__restrict__ vaz, double vm0,
                                          const double *__restrict__ qplus,
                                          const double *__restrict__ qminus,
                                          const double *__restrict__ E)
{
    const int nz = g.nz;
    const size_t row = (size_t)i * nz;
    const size_t c = row + j;
    auto tp = [&](const double *tab) {
        const float2 v = t.ptab[(tab - t.tbase) + i];
        return f2{v.x, v.y};
    };
    auto fmax2 = [](f2 a, f2 b) {  // a, b >= 0
        return (a.h > b.h || (a.h == b.h && a.l > b.l)) ? a : b;
    };
    const double va = vaz[c], vr0 = vr[c], vr1 = vr[c + nz];
    const double va1 = vaz[row + (j == nz - 1 ? 0 : j + 1)];
    const f2 inv_drsup = tp(t.InvDiffRsup), inv_dxt = tp(t.InvDxTheta);
    const f2 i1 = f2_smul(c_s, tp(t.InvCell));
    const f2 i2 = f2_smul(f2_split(vr0), inv_drsup);
    const f2 i3 = f2_smul(f2_split(ph.fast_transport ? va - vm0 : va), inv_dxt);
    f2 i4;
    if (sn) {
        const double dvR = vr1 - vr0, dvA = va1 - va;
        const f2 a = f2_smul(f2_split(positive(dvR) ? 0.0 : -dvR), inv_drsup);
        const f2 b = f2_smul(f2_split(positive(dvA) ? 0.0 : -dvA), inv_dxt);
        i4 = f2_smul(f2_split(ph.four_C2), fmax2(a, b));
    } else {
        const f2 eps_rr = f2_smul(f2_split(vr1 - vr0), inv_drsup);
        const f2 h = f2_split(0.5 * (vr1 + vr0));
        const f2 eps_pp = f2_smul(tp(t.InvRmed),
                                  f2_sadd(f2_smul(f2_split(va1 - va), f2_split(g.invdphi)), h));
        const f2 d = f2_sadd(eps_rr, eps_pp);
        i4 = f2_smul(f2_split(ph.four_C2), d.h < 0.f ? f2_neg(d) : f2{0.f, 0.f});
    }
    f2 i5 = f2_smul(n, tp(t.InvCell2));
    i5 = f2{__fmul_rn(4.0f, i5.h), __fmul_rn(4.0f, i5.l)};
    f2 i6{0.f, 0.f};
    if (ph.adiabatic) {
        const f2 q = f2_sdiv(f2_split(qplus[c] - qminus[c]), f2_split(E[c]));
        i6 = f2_smul(f2_split(ph.inv_hc_limit), q.h < 0.f ? f2_neg(q) : q);
    }
    if (ph.leapfrog) {
        const f2 k = f2_split(0.6);
        i4 = f2_smul(i4, k);
        i5 = f2_smul(i5, k);
        i6 = f2_smul(i6, k);
    }
    f2 sum = f2_smul(i1, i1);
    sum = f2_sadd(sum, f2_smul(i2, i2));
    sum = f2_sadd(sum, f2_smul(i3, i3));
    sum = f2_sadd(sum, f2_smul(i4, i4));
    sum = f2_sadd(sum, f2_smul(i5, i5));
    sum = f2_sadd(sum, f2_smul(i6, i6));
    return sum;
}

// the larger of two non-negative pairs
__device__ __forceinline__ f2 pair_max(f2 a, f2 b)
{
    return (b.h > a.h || (b.h == a.h && b.l > a.l)) ? b : a;
}
__device__ f2 block_max_f2(f2 v, float *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1)
        v = pair_max(v, f2{__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)});
    __syncthreads();
    if (lane == 0) {
        red[2 * wid] = v.h;
        red[2 * wid + 1] = v.l;
    }
    __syncthreads();
    if (wid == 0) {
        f2 x = lane < nw ? f2{red[2 * lane], red[2 * lane + 1]} : f2{0.f, 0.f};
        for (int o = 16; o > 0; o >>= 1)
            x = pair_max(x, f2{__shfl_down_sync(0xffffffffu, x.h, o), __shfl_down_sync(0xffffffffu, x.l, o)});
        if (lane == 0) {
            red[64] = x.h;
            red[65] = x.l;
        }
    }
    __syncthreads();
    return f2{red[64], red[65]};
}


// PAIR: the ideal-EOS derived quantities (T, c_s, H, nu) in float-pair
// arithmetic (P = (gamma - 1) e stays one FP64 product: the source terms
// difference it)
// 256-thread blocks; the pair form held to 64 registers, 4 blocks per SM (at
// its free choice of 121 registers, 2 blocks: 0.67 ms on the 2048 x 6144
// disk, at 80: 0.557, at 64: 0.502)
template <bool PAIR>
__global__ void __launch_bounds__(256, PAIR ? 4 : 3) k_derived_cfl(Geo g, Tables t, Phys ph, int mode, int sn, const double *__restrict__ S,
                              const double *__restrict__ E, const double *__restrict__ vr,
                              const double *__restrict__ vaz, const double *__restrict__ qplus,
                              const double *__restrict__ qminus, double *__restrict__ cs,
                              double *__restrict__ H, double *__restrict__ P,
                              double *__restrict__ T, double *__restrict__ nu,
                              const double *__restrict__ corr_phi,
                              const double *__restrict__ corr_r,
                              unsigned long long *__restrict__ dt_min)
{
    __shared__ double red[33];
    __shared__ float redf[66];
    extern __shared__ float d32s[];  // the ring's FP32 cell steps (nz floats)
    // PAIR: every cell's squared inverse step in float pairs, the ring's
    // largest kept as a pair and turned into the ring's step once (no FP32
    // screen: in a nearly axisymmetric ring most cells fall inside any
    // screen's margin, and each would then take FP64)
    const bool pair_cfl = PAIR && ph.stabilize != 2;
    f2 local2{0.f, 0.f};
    const int nz = g.nz, nr = g.nr;
    const int i = blockIdx.x;
    float local32 = 3.0e38f;
    CflRing32 t32;
    t32.inv_cell = (float)t.InvCell[i];
    t32.inv_cell2 = (float)t.InvCell2[i];
    t32.inv_drsup = (float)t.InvDiffRsup[i];
    t32.inv_dxtheta = (float)t.InvDxTheta[i];
    t32.inv_rmed = (float)t.InvRmed[i];
    t32.invdphi = (float)g.invdphi;
    t32.four_C2 = (float)ph.four_C2;
    t32.inv_hc = (float)ph.inv_hc_limit;
    t32.cfl = (float)ph.cfl;
    const size_t row = (size_t)i * nz;
    const bool do_cfl = (mode & 4) != 0;
    double vm0 = 0.0, vm1 = 0.0;
    if (do_cfl && i < nr - 1) {
        double p0 = 0.0, p1 = 0.0;
        for (int j = threadIdx.x; j < nz; j += blockDim.x) {
            p0 += vaz[row + j];
            p1 += vaz[row + nz + j];
        }
        vm0 = block_sum(p0, red) / (double)nz;
        vm1 = block_sum(p1, red) / (double)nz;
    }
    const double dxR = t.Rsup[i] - t.Rinf[i];
    const double dxA = t.Rmed[i] * g.dphi;
    const double cell = dxR < dxA ? dxR : dxA;
    double local = 1.0e300;
    if (do_cfl && i == 0) {
        const double denom = fabs(vm0 * t.InvRmed[0] - vm1 * t.InvRmed[1]) + 1.0e-100;
        local = ph.cfl * g.dphi / denom;
    }
    const bool cfl_ring = do_cfl && i >= 1 && i < nr - 1;
    if (cfl_ring) {
        const double denom = fabs(vm0 * t.InvRmed[i] - vm1 * t.InvRmed[i + 1]) + 1.0e-100;
        local = ph.cfl * g.dphi / denom;
    }
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const size_t c = row + j;
        double c_s, n;
        f2 cp2{0.f, 0.f};  // c_s as a pair where the pair path formed it
        bool have_cp2 = false;
        if (mode & 1) {
            const double sg = S[c];
            if (ph.adiabatic && PAIR) {
                const double e = E[c];
                const f2 es = f2_sdiv(f2_split(e), f2_split(sg));
                T[c] = f2_to_double(f2_smul(f2_split(ph.c_v_inv), es));
                const f2 cp = f2_sqrt(f2_smul(f2_split(ph.g_gm1), es));
                const float2 hf = t.ptab[(t.HFacAdi - t.tbase) + i];
                const f2 hp = f2_smul(cp, f2{hf.x, hf.y});
                cp2 = cp;
                have_cp2 = true;
                c_s = f2_to_double(cp);
                cs[c] = c_s;
                H[c] = f2_to_double(hp);
                P[c] = ph.gm1 * e;
                n = ph.alpha > 0 ? f2_to_double(f2_smul(f2_smul(f2_split(ph.alpha), hp), cp))
                                 : ph.constant_viscosity;
            } else if (ph.adiabatic) {
                const double e = E[c];
                const double es = fast_div1(e, sg);
                T[c] = ph.c_v_inv * es;
                c_s = sqrt(ph.g_gm1 * es);
                const double h = c_s * t.HFacAdi[i];
                cs[c] = c_s;
                H[c] = h;
                P[c] = ph.gm1 * e;
                n = ph.alpha > 0 ? ph.alpha * h * c_s : ph.constant_viscosity;
            } else {
                c_s = t.CsIso[i];
                const double h = c_s * t.InvOmegaK[i];
                P[c] = sg * (c_s * c_s);
                if (mode & 2) {
                    cs[c] = c_s;
                    H[c] = h;
                    T[c] = ph.mu / ph.Rgas * P[c] / sg;  // init only
                }
                n = ph.alpha > 0 ? ph.alpha * h * c_s : ph.constant_viscosity;
            }
            nu[c] = n;
        } else {
            c_s = cs[c];
            n = nu[c];
        }
        if (cfl_ring && pair_cfl) {
            const f2 cpair = have_cp2 ? cp2 : f2_split(c_s);
            local2 = pair_max(local2, cfl_cell_f2(g, t, ph, sn, i, j, cpair, f2_split(n), vr, vaz,
                                                  vm0, qplus, qminus, E));
        } else if (cfl_ring) {
            const float d32 = cfl_cell32(t32, ph, sn, c_s, n, vr[c], vr[c + nz], vaz[c],
                                         vaz[row + (j == nz - 1 ? 0 : j + 1)], vm0,
                                         ph.adiabatic ? qplus[c] : 0.0,
                                         ph.adiabatic ? qminus[c] : 0.0,
                                         ph.adiabatic ? E[c] : 1.0,
                                         ph.stabilize == 2 ? corr_phi[c] : 0.0,
                                         ph.stabilize == 2 ? corr_r[c] : 0.0);
            d32s[j] = d32;
            local32 = fminf(local32, d32);
        }
    }
    if (cfl_ring && pair_cfl) {
        const f2 m = block_max_f2(local2, redf);
        const double d = f2_to_double(f2_sdiv(f2_split(ph.cfl), f2_sqrt(m)));
        if (dbits(d) < dbits(local)) local = d;
    } else if (cfl_ring) {
        // the FP64 dt of the cells the FP32 screen puts within 2^-15 of the
        // ring's FP32 minimum; that set holds the FP64 minimum, since the
        // screen's error is below 2^-19 (each thread reads back the screen
        // values it wrote, and c_s, nu as it wrote them)
        const float ringmin = block_min_f(local32, redf);
        const float thr = ringmin * (1.0f + 0x1p-15f);
        for (int j = threadIdx.x; j < nz; j += blockDim.x) {
            if (!(d32s[j] <= thr)) continue;
            const size_t c = row + j;
            const double c_s = ((mode & 1) && !ph.adiabatic) ? t.CsIso[i] : cs[c];
            const double n = nu[c];
            double inv[6];
            const double dt_cell = cfl_cell64(g, t, ph, sn, i, j, c_s, n, vr, vaz, vm0, qplus,
                                              qminus, E, corr_phi, corr_r, inv);
            // positive doubles order like their bit patterns
            if (dbits(dt_cell) < dbits(local)) local = dt_cell;
        }
    }
    if (do_cfl) {
        const double m = block_min(local, red);
        if (threadIdx.x == 0 && m < 1.0e300) {
            atomicMin(dt_min, (unsigned long long)__double_as_longlong(m));
        }
    }
}

// ---------------------------------------------------------------------------
// Accretion onto one planet (accretion.cpp:84-480): Kley's two zones, the
// sink hole or the viscous profile over the planet's region, one block; the
// mass and momentum taken from the active rings are block sums written to
// out[0 .. 2].  Cells are independent, so the in-place updates do not race.
// ---------------------------------------------------------------------------
__global__ void k_accrete(Geo g, Tables t, Phys ph, AccretionSpec a, double *__restrict__ S,
                          double *__restrict__ E, const double *__restrict__ vr,
                          const double *__restrict__ vaz, const double *__restrict__ nu,
                          double *__restrict__ out)
{
    __shared__ double red[33];
    const int nz = g.nz, nr = g.nr;
    const int rows = a.i1 - a.i0 + 1;
    const long long cells = (long long)rows * a.ncols;
    double dM = 0.0, dPx = 0.0, dPy = 0.0;
    for (long long k = threadIdx.x; k < cells; k += blockDim.x) {
        const int i = a.i0 + (int)(k / a.ncols);
        int jf = a.j0 + (int)(k % a.ncols);
        jf %= nz;
        if (jf < 0) jf += nz;
        const size_t l = CELL(i, jf);
        const double xc = t.Rmed[i] * t.cosj[jf];
        const double yc = t.Rmed[i] * t.sinj[jf];
        const double dx = a.x - xc, dy = a.y - yc;
        const double distance = sqrt(dx * dx + dy * dy);
        const double vtcell = 0.5 * (vaz[l] + vaz[CELL(i, jnext(jf, nz))]) + t.Rmed[i] * a.omf;
        const double vrcell = 0.5 * (vr[l] + vr[l + nz]);
        const double vxcell = (vrcell * xc - vtcell * yc) / t.Rmed[i];
        const double vycell = (vrcell * yc + vtcell * xc) / t.Rmed[i];
        const double facc_max = 1 - a.density_floor / S[l];
        const bool active = 1 < i && i < nr - 1;
        if (distance < a.frac1 * a.rhill) {
            double f = a.facc1;
            if (a.type == 1 /* viscous */)
                f = a.facc1 * nu[l] * (a.f_const * (1.0 - distance / a.dist_max));
            const double fc = facc_max < f ? facc_max : f;
            const double deltaM = fc * S[l] * t.Surf[i];
            S[l] *= 1.0 - fc;
            if (ph.adiabatic) E[l] *= 1.0 - fc;
            if (active) {
                dPx += deltaM * vxcell;
                dPy += deltaM * vycell;
                dM += deltaM;
            }
        }
        if (a.type == 0 /* Kley */ && distance < a.frac2 * a.rhill) {
            const double fc = facc_max < a.facc2 ? facc_max : a.facc2;
            const double deltaM = fc * S[l] * t.Surf[i];
            S[l] *= 1.0 - fc;
            // the reference scales the energy by the uncapped factor here
            if (ph.adiabatic) E[l] *= 1.0 - a.facc2;
            if (active) {
                dPx += deltaM * vxcell;
                dPy += deltaM * vycell;
                dM += deltaM;
            }
        }
    }
    dM = block_sum(dM, red);
    dPx = block_sum(dPx, red);
    dPy = block_sum(dPy, red);
    if (threadIdx.x == 0) {
        out[0] = dM;
        out[1] = dPx;
        out[2] = dPy;
    }
}

// ---------------------------------------------------------------------------
// ComputeDiskOnPlanetAccel (src/Force.cpp:23-122) for up to kForceBodies
// bodies in one pass over the ring: with CorrectDiskSelfgravity the ring mean
// of sigma is subtracted (Force.cpp:64-66), and the gas mass of the ring
// (gas_total_mass, quantities.cpp:51-74) comes along.  One CTA per active
// ring writes, for body b, partial[5 b .. 5 b + 4] = (inner x, inner y,
// outer x, outer y, mass) of its ring (split at Rmed < a, the body's distance
// from the origin); k_reduce_cols adds the rings with compensation in a
// fixed order.  Per body and cell: the separation, its smoothed inverse cube
// (one rsqrt), Klahr's cubic factor inside r_sm, and the two products into
// the sums, all in float-pair arithmetic (fp64_pair.cuh, about 2^-46
// relative; sums of pairs per thread, FP64 across the block); G and the
// ring's Surf multiply the ring's sums once.
// ---------------------------------------------------------------------------
struct ForceBodies {
    int n;  // bodies in this pass (1 .. kForceBodies)
    unsigned klahr;  // bit b: body b has Klahr smoothing (rsm > 0)
    double a[kForceBodies], rsm[kForceBodies];
    float xh[kForceBodies], xl[kForceBodies], yh[kForceBodies], yl[kForceBodies];
};

__global__ void __launch_bounds__(256, 4) k_disk_force_bodies(Geo g, Tables t, Phys ph, ForceBodies fb,
                                    const double *__restrict__ S, const double *__restrict__ H,
                                    double *__restrict__ partial, int width)
{
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x + 1;  // radial_first_active .. radial_active_size - 1
    const size_t row = (size_t)i * nz;
    double ps = 0.0;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) ps += S[row + j];
    const double ring_sum = block_sum(ps, red);
    const double sigma1d = ph.correct_sg ? ring_sum / nz : 0.0;
    const double rmed = t.Rmed[i];
    const f2 rm{t.RmedHi[i], t.RmedLo[i]};
    // per body and thread, the sums of the x and y terms as float pairs
    float axh[kForceBodies], axl[kForceBodies], ayh[kForceBodies], ayl[kForceBodies];
#pragma unroll
    for (int b = 0; b < kForceBodies; ++b) axh[b] = axl[b] = ayh[b] = ayl[b] = 0.f;
    const f2 eps = f2_split(ph.eps_smooth);
    float rsm_f[kForceBodies];
#pragma unroll
    for (int b = 0; b < kForceBodies; ++b) rsm_f[b] = b < fb.n ? f2_split(fb.rsm[b]).h : 0.f;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const f2 smooth = f2_smul(eps, f2_split(H[row + j]));
        const f2 s2 = f2_smul(smooth, smooth);
        const f2 xc = f2_smul(rm, f2{t.cosHi[j], t.cosLo[j]});
        const f2 yc = f2_smul(rm, f2{t.sinHi[j], t.sinLo[j]});
        // sigma less the ring mean: the FP64 difference (they agree closely)
        const f2 dsig = f2_split(S[row + j] - sigma1d);
#pragma unroll
        for (int b = 0; b < kForceBodies; ++b) {
            if (b < fb.n) {
                const f2 dx = f2_ssub(xc, f2{fb.xh[b], fb.xl[b]});
                const f2 dy = f2_ssub(yc, f2{fb.yh[b], fb.yl[b]});
                const f2 dsm2 = f2_sadd(f2_sadd(f2_smul(dx, dx), f2_smul(dy, dy)), s2);
                const f2 rinv = f2_rsqrt(dsm2);
                f2 w = f2_smul(dsig, f2_smul(f2_smul(rinv, rinv), rinv));
                if ((fb.klahr >> b) & 1u) {
                    // Klahr's factor inside r_sm (Force.cpp:88-100): rare, in FP64
                    const f2 dsm_p = f2_mul(dsm2, rinv);
                    if (maybe_inside(dsm_p, rsm_f[b])) {
                        const double dsm = f2_to_double(dsm_p);
                        if (dsm < fb.rsm[b]) {
                            const double q = dsm / fb.rsm[b];
                            w = f2_split(f2_to_double(w) *
                                         -(3.0 * (q * q * q * q) - 4.0 * (q * q * q)));
                        }
                    }
                }
                f2_accumulate(axh[b], axl[b], f2_smul(w, dx));
                f2_accumulate(ayh[b], ayl[b], f2_smul(w, dy));
            }
        }
    }
    const double gs = ph.G * t.Surf[i];
    double *p = partial + (size_t)blockIdx.x * width;
#pragma unroll
    for (int b = 0; b < kForceBodies; ++b) {
        if (b < fb.n) {
            const double sx = block_sum((double)axh[b] + (double)axl[b], red) * gs;
            const double sy = block_sum((double)ayh[b] + (double)ayl[b], red) * gs;
            if (threadIdx.x == 0) {
                const bool inner = rmed < fb.a[b];
                p[5 * b + 0] = inner ? sx : 0.0;
                p[5 * b + 1] = inner ? sy : 0.0;
                p[5 * b + 2] = inner ? 0.0 : sx;
                p[5 * b + 3] = inner ? 0.0 : sy;
                p[5 * b + 4] = t.Surf[i] * ring_sum;
            }
        }
    }
}

// gas_total_mass (quantities.cpp:51-74) and gas_angular_momentum
// (quantities.cpp:242-276) of each active ring with Rmed <= radius (zero
// otherwise): one CTA per ring writes (mass, angular momentum).  The ring's
// Surf and Rmed multiply its sums once; the angular momentum takes sigma at
// the v_phi interface (cells j and j - 1) and the inertial speed.
__global__ void k_gas_quantities(Geo g, Tables t, double radius, double omf,
                                 const double *__restrict__ S, const double *__restrict__ vaz,
                                 double *__restrict__ partial)
{
    __shared__ double red[33];
    const int nz = g.nz;
    const int i = blockIdx.x + 1;
    const size_t row = (size_t)i * nz;
    const double rmed = t.Rmed[i];
    const double vframe = omf * rmed;
    double m = 0.0, l = 0.0;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        const double sj = S[row + j];
        const double sm = S[row + (j == 0 ? nz - 1 : j - 1)];
        m += sj;
        l += 0.5 * (sj + sm) * (vaz[row + j] + vframe);
    }
    m = block_sum(m, red);
    l = block_sum(l, red);
    if (threadIdx.x == 0) {
        const bool in = rmed <= radius;
        partial[(size_t)blockIdx.x * 2] = in ? t.Surf[i] * m : 0.0;
        partial[(size_t)blockIdx.x * 2 + 1] = in ? t.Surf[i] * rmed * l : 0.0;
    }
}

// KeepDiskMassConstant (simulation.cpp:246-251): sigma *= target / mass over
// every cell, the mass read on the device (no host round trip).
__global__ void k_scale_sigma(double *__restrict__ S, size_t n, double target,
                              const double *__restrict__ mass)
{
    const double factor = target / mass[0];
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x)
        S[k] *= factor;
}

// Kahan-compensated sum of `rows` records of `width` doubles, in order.
// one warp per component
__global__ void k_reduce_rows(const double *__restrict__ partial, int rows, int width,
                              double *__restrict__ out)
{
    const int w = threadIdx.x >> 5;
    if (w < width) warp_compensated_rows(partial, rows, width, w, out);
}
// the same with one block (one warp) per component, for wide records
__global__ void k_reduce_cols(const double *__restrict__ partial, int rows, int width,
                              double *__restrict__ out)
{
    warp_compensated_rows(partial, rows, width, blockIdx.x, out);
}

// NaN/Inf scan of one field: records the first bad flat index (atomicMin).
__global__ void k_check_finite(const double *__restrict__ x, size_t n, unsigned long long *bad)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && !isfinite(x[k])) atomicMin(bad, (unsigned long long)k);
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
static inline dim3 grid2d(int nz, int rows, int bx) { return dim3((nz + bx - 1) / bx, rows); }

void launch_potential(const Launch &L, const Bodies &b, const double *H, double *pot)
{
    auto k = L.pair ? k_potential<true> : k_potential<false>;
    k<<<grid2d(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(L.g, L.t, L.ph, b, H, pot);
}

void launch_source(const Launch &L, double dt, double omf, const double *S, const double *P,
                   const double *pot, const double *vr_in, const double *vaz_in, double *vr_out,
                   double *vaz_out)
{
    if (L.pair) return launch_source_pair(L, dt, omf, S, P, pot, vr_in, vaz_in, vr_out, vaz_out);
    k_source<<<grid2d(L.g.nz, L.g.nr + 1, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, dt, omf, S, P, pot, vr_in, vaz_in, vr_out, vaz_out);
}

void launch_artvisc_q(const Launch &L, double dt, const double *S, const double *vr,
                      const double *vaz, double *E, double *Qr, double *Qp)
{
    if (L.pair) return launch_artvisc_q_pair(L, dt, S, vr, vaz, E, Qr, Qp);
    k_artvisc_q<<<grid2d(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(L.g, L.t, L.ph, dt, S, vr,
                                                                      vaz, E, Qr, Qp);
}

void launch_artvisc_v(const Launch &L, double dt, const double *S, const double *E,
                      const double *Qr, const double *Qp, double *vr, double *vaz, double *cs,
                      double *H, double *nu)
{
    if (L.pair) return launch_artvisc_v_pair(L, dt, S, E, Qr, Qp, vr, vaz, cs, H, nu);
    k_artvisc_v<<<grid2d(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(L.g, L.t, L.ph, dt, S, E, Qr,
                                                                      Qp, vr, vaz, cs, H, nu);
}

void launch_stress(const Launch &L, const double *S, const double *vr, const double *vaz,
                   const double *nu, double *divv, double *trr, double *tpp, double *trp)
{
    if (L.pair) return launch_stress_pair(L, S, vr, vaz, nu, divv, trr, tpp, trp);
    k_stress<<<grid2d(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(L.g, L.t, S, vr, vaz, nu, divv,
                                                                   trr, tpp, trp);
}

void launch_viscous(const Launch &L, double dt, double beta_inv, int mode, const State &s)
{
    // StabilizeViscosity's corrected update is the FP64 kernel's
    if (L.pair && L.ph.stabilize != 1) return launch_viscous_pair(L, dt, beta_inv, mode, s);
    k_viscous<<<grid2d(L.g.nz, L.g.nr, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, L.ph, dt, beta_inv, mode, s.sigma, s.trr, s.tpp, s.trp, s.divv, s.nu, s.H,
        s.sigma0, s.energy0, s.vr, s.vaz, s.energy, s.qplus, s.qminus, s.corr_phi, s.corr_r);
}

void launch_accrete(const Launch &L, const AccretionSpec &a, double *S, double *E,
                    const double *vr, const double *vaz, const double *nu, double *out)
{
    k_accrete<<<1, 512, 0, L.stream>>>(L.g, L.t, L.ph, a, S, E, vr, vaz, nu, out);
}

void launch_visc_corr(const Launch &L, const State &s)
{
    k_visc_corr<<<grid2d(L.g.nz, L.g.nr - 1, L.bx), L.bx, 0, L.stream>>>(L.g, L.t, s.sigma, s.nu,
                                                                          s.corr_phi, s.corr_r);
}

// correct_v_azimuthal, SideEuler.cpp:79-95
__global__ void k_correct_vaz(Geo g, Tables t, double domega, double *__restrict__ vaz)
{
    const int nz = g.nz;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j < nz) vaz[CELL(i, j)] -= domega * t.Rmed[i];
}

void launch_correct_vaz(const Launch &L, double domega, double *vaz)
{
    k_correct_vaz<<<dim3((L.g.nz + 127) / 128, L.g.nr), 128, 0, L.stream>>>(L.g, L.t, domega,
                                                                         vaz);
}

// The centre-of-mass composite (com_boundary.cuh) on the FP64 fields.
void launch_com_boundary(const Launch &L, const ComSpec &c, const State &s)
{
    const ComFields64 f{s.sigma, s.vr, s.vaz, s.energy};
    k_com_boundary<<<dim3((L.g.nz + 127) / 128, 2), 128, 0, L.stream>>>(c, L.g.nz, L.g.nr, f);
}

void launch_com_damping(const Launch &L, const ComSpec &c, double dt, const State &s)
{
    const ComFields64 f{s.sigma, s.vr, s.vaz, s.energy};
    launch_com_damping_sides(c, L.g.nz, dt, f, L.stream);
}

void launch_ghost(const Launch &L, const BcSpec &bc, double omf, const State &s)
{
    k_ghost<<<(L.g.nz + 127) / 128, 128, 0, L.stream>>>(L.g, L.t, bc, omf, s);
}

int radial_chunk_for(bool pair, bool adiabatic, int nr, int nz)
{
    // resident 64-thread blocks per SM of the kernel this engine launches
    const void *fn = pair ? (adiabatic ? (const void *)k_transport_radial_f2<5>
                                       : (const void *)k_transport_radial_f2<4>)
                          : (adiabatic ? (const void *)k_transport_radial<5>
                                       : (const void *)k_transport_radial<4>);
    int per_sm = 0, dev = 0, nsm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 64, 0) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        per_sm <= 0 || nsm <= 0) {
        cudaGetLastError();
        return (size_t)nr * nz >= ((size_t)8 << 20) ? 32 : 16;
    }
    if ((size_t)nr * nz < ((size_t)8 << 20)) return 16;
    // large disks: the chunk of 28 .. 40 rings whose grid fills the fewest
    // waves of resident blocks for the rings walked (each chunk also primes
    // about three rings)
    const long long cols = (nz + 63) / 64, slots = (long long)per_sm * nsm;
    int best = 32;
    long long best_cost = -1;
    for (int c = 28; c <= 40; ++c) {
        const long long blocks = cols * ((nr + c - 1) / c);
        const long long cost = (blocks + slots - 1) / slots * (c + 3);
        if (best_cost < 0 || cost < best_cost) {
            best = c;
            best_cost = cost;
        }
    }
    return best;
}

void launch_transport_radial(const Launch &L, double dt, double omf, int chunk, const double *S,
                             const double *vr, const double *vaz, const double *E,
                             double *const mom[4], double *E_out, double *S_out)
{
    const bool pair = L.pair;
    const int chunks = (L.g.nr + chunk - 1) / chunk;
    const int bx = 64;
    dim3 grid((L.g.nz + bx - 1) / bx, chunks);
    if (pair) {
        if (L.ph.adiabatic) {
            k_transport_radial_f2<5><<<grid, bx, 0, L.stream>>>(
                L.g, L.t, dt, omf, L.ph.limiter_mc, chunk, S, vr, vaz, E, mom[0], mom[1], mom[2],
                mom[3], E_out, S_out);
        } else {
            k_transport_radial_f2<4><<<grid, bx, 0, L.stream>>>(
                L.g, L.t, dt, omf, L.ph.limiter_mc, chunk, S, vr, vaz, E, mom[0], mom[1], mom[2],
                mom[3], E_out, S_out);
        }
        return;
    }
    if (L.ph.adiabatic) {
        k_transport_radial<5><<<grid, bx, 0, L.stream>>>(L.g, L.t, dt, omf, L.ph.limiter_mc, chunk,
                                                         S, vr, vaz, E, mom[0], mom[1], mom[2],
                                                         mom[3], E_out, S_out);
    } else {
        k_transport_radial<4><<<grid, bx, 0, L.stream>>>(L.g, L.t, dt, omf, L.ph.limiter_mc, chunk,
                                                         S, vr, vaz, E, mom[0], mom[1], mom[2],
                                                         mom[3], E_out, S_out);
    }
}

// the larger of the two kernels' rings: the pair kernel's halo cells
size_t azimuthal_smem_bytes(int nz) { return pair_ring_f2s(nz) * sizeof(f2); }

// Cells per thread of the azimuthal kernel: blocks stay at <= 512 threads so
// that the per-thread cell arrays fit 128 registers.
int azimuthal_cells_per_thread(int nz) { return nz <= 2048 ? 4 : (nz <= 4096 ? 8 : 16); }

cudaError_t prepare_azimuthal(size_t smem)
{
    cudaError_t e = raise_smem_limit((const void *)k_transport_azimuthal<4>, smem);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_transport_azimuthal<8>, smem);
    if (e == cudaSuccess) e = raise_smem_limit((const void *)k_transport_azimuthal<16>, smem);
#define AZ2_FN(P, T, Q, X) (const void *)k_transport_azimuthal_f2<P, T, Q, false, X>
    const void *pair_kernels[12] = {
        AZ2_FN(2, 1024, 4, false), AZ2_FN(2, 1024, 5, false), AZ2_FN(2, 1024, 4, true),
        AZ2_FN(2, 1024, 5, true), AZ2_FN(6, 1024, 4, false), AZ2_FN(6, 1024, 5, false),
        AZ2_FN(6, 1024, 4, true), AZ2_FN(6, 1024, 5, true), AZ2_FN(16, 512, 4, false),
        AZ2_FN(16, 512, 5, false), AZ2_FN(16, 512, 4, true), AZ2_FN(16, 512, 5, true)};
#undef AZ2_FN
    for (const void *fn : pair_kernels)
        if (e == cudaSuccess) e = raise_smem_limit(fn, smem);
    return e;
}

// Cells per thread of the pair kernel: 2 up to 1024 cells (<= 512 threads),
// 6 up to 6144 (<= 1024), 16 beyond (<= 512 threads for 8192 cells); the
// thread count is the ring length over that, in whole warps.  Measured
// (ms per azimuthal pass): 384-cell rings 0.021 with 2 cells per thread
// (4: 0.029, 6: 0.039); 1536: 0.127 with 6 (4: 0.132, 8: 0.135, 2: 0.169);
// 3072: 0.378 with 6 (8: 0.412); 6144: 1.87 with 6 (8: 2.01, 12: 2.55).
int azimuthal_pair_cells_per_thread(int nz) { return nz <= 1024 ? 2 : (nz <= 6144 ? 6 : 16); }

void launch_transport_azimuthal(const Launch &L, double dt, int block, double *const mom[4],
                                double *E, double *S, const double *vaz, double *ring_ws,
                                size_t smem, int *ring_shift)
{
    const bool pair = L.pair;
    const int nq = L.ph.adiabatic ? 5 : 4;
    const size_t dyn = ring_ws ? 0 : smem;
    if (pair) {
        const int per = azimuthal_pair_cells_per_thread(L.g.nz);
        const int threads = ((L.g.nz + per - 1) / per + 31) / 32 * 32;
        const bool exact = L.g.nz == per * threads;
#define AZ2_LAUNCH1(P, T, Q, WS, X)                                                             \
    k_transport_azimuthal_f2<P, T, Q, WS, X><<<L.g.nr, threads, dyn, L.stream>>>(                \
        L.g, L.t, dt, L.ph.limiter_mc, L.ph.fast_transport, vaz, mom[0], mom[1], mom[2], mom[3], \
        E, S, ring_ws, ring_shift)
#define AZ2_LAUNCH2(P, T, Q)                                                                    \
    if (exact) AZ2_LAUNCH1(P, T, Q, false, true); else AZ2_LAUNCH1(P, T, Q, false, false)
#define AZ2_LAUNCH(P, T)                                                                        \
    if (nq == 5) { AZ2_LAUNCH2(P, T, 5); } else { AZ2_LAUNCH2(P, T, 4); }
        if (ring_ws) {
            // rings beyond the shared memory: 16 cells per thread
            if (nq == 5) AZ2_LAUNCH1(16, 512, 5, true, false);
            else AZ2_LAUNCH1(16, 512, 4, true, false);
        } else if (per == 2) {
            AZ2_LAUNCH(2, 1024);
        } else if (per == 6) {
            AZ2_LAUNCH(6, 1024);
        } else {
            AZ2_LAUNCH(16, 512);
        }
#undef AZ2_LAUNCH
#undef AZ2_LAUNCH1
#undef AZ2_LAUNCH2
        return;
    }
    const int per = azimuthal_cells_per_thread(L.g.nz);
#define AZ_LAUNCH(P)                                                                          \
    k_transport_azimuthal<P><<<L.g.nr, block, dyn, L.stream>>>(                               \
        L.g, L.t, dt, L.ph.limiter_mc, L.ph.fast_transport, nq, vaz, mom[0], mom[1], mom[2], \
        mom[3], E, S, ring_ws)
    if (per == 4) {
        AZ_LAUNCH(4);
    } else if (per == 8) {
        AZ_LAUNCH(8);
    } else {
        AZ_LAUNCH(16);
    }
#undef AZ_LAUNCH
}

void launch_finish(const Launch &L, double omf, double *const mom[4], const double *S_t,
                   const double *E_t, const double *vr_in, double *vr_out, double *vaz_out,
                   double *S_out, double *E_out, const int *ring_shift)
{
    if (L.pair)
        return launch_finish_pair(L, omf, mom, S_t, E_t, vr_in, vr_out, vaz_out, S_out, E_out,
                                  ring_shift);
    k_finish<<<grid2d(L.g.nz, L.g.nr + 1, L.bx), L.bx, 0, L.stream>>>(
        L.g, L.t, L.ph, omf, mom[0], mom[1], mom[2], mom[3], S_t, E_t, vr_in, vr_out, vaz_out,
        S_out, E_out);
}

void launch_damping(const Launch &L, const Damping &dm, double dt, const int *rings, int nrings,
                    const State &s)
{
    if (nrings <= 0) return;
    k_damping<<<dim3(nrings, 4), 256, 0, L.stream>>>(L.g, dm, dt, rings, s);
}

// compute_pressure (SourceEuler.cpp:1345-1376): P alone, from sigma and c_s
// (isothermal, axisymmetric c_s) or e (ideal EOS)
__global__ void k_pressure(Geo g, Tables t, Phys ph, const double *__restrict__ S,
                           const double *__restrict__ E, double *__restrict__ P)
{
    const int nz = g.nz;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= nz) return;
    const size_t c = (size_t)i * nz + j;
    if (ph.adiabatic) {
        P[c] = ph.gm1 * E[c];
    } else {
        const double c_s = t.CsIso[i];
        P[c] = S[c] * (c_s * c_s);
    }
}

void launch_pressure(const Launch &L, const double *S, const double *E, double *P)
{
    k_pressure<<<dim3((L.g.nz + 127) / 128, L.g.nr), 128, 0, L.stream>>>(L.g, L.t, L.ph, S, E, P);
}

// The step's limiting cell, as cfl.cpp's timestep_debug_report (:38-182)
// names it: per ring i (0 .. nr - 2) the shear limit and, on the CFL rings
// (1 .. nr - 2), the smallest cell dt, its azimuth (the first on ties) and
// its six inverse times, written as out[10 i .. 10 i + 9] =
// {dt, azimuth, shear dt, invdt 1..6}.  Same arithmetic as k_derived_cfl.
__global__ void k_cfl_cells(Geo g, Tables t, Phys ph, int sn, const double *__restrict__ vr,
                            const double *__restrict__ vaz, const double *__restrict__ cs,
                            const double *__restrict__ nu, const double *__restrict__ qplus,
                            const double *__restrict__ qminus, const double *__restrict__ E,
                            const double *__restrict__ corr_phi,
                            const double *__restrict__ corr_r, double *__restrict__ out)
{
    __shared__ double red[33];
    __shared__ int jmin;
    const int nz = g.nz;
    const int i = blockIdx.x;
    const size_t row = (size_t)i * nz;
    double p0 = 0.0, p1 = 0.0;
    for (int j = threadIdx.x; j < nz; j += blockDim.x) {
        p0 += vaz[row + j];
        p1 += vaz[row + nz + j];
    }
    const double vm0 = block_sum(p0, red) / (double)nz;
    const double vm1 = block_sum(p1, red) / (double)nz;
    const double denom = fabs(vm0 * t.InvRmed[i] - vm1 * t.InvRmed[i + 1]) + 1.0e-100;
    const double shear = ph.cfl * g.dphi / denom;
    const bool cfl_ring = i >= 1;
    double local = 1.0e300;
    double inv[6];
    if (cfl_ring) {
        for (int j = threadIdx.x; j < nz; j += blockDim.x) {
            const size_t c = row + j;
            const double c_s = ph.adiabatic ? cs[c] : t.CsIso[i];
            const double d = cfl_cell64(g, t, ph, sn, i, j, c_s, nu[c], vr, vaz, vm0, qplus,
                                        qminus, E, corr_phi, corr_r, inv);
            if (d < local) local = d;
        }
    }
    if (threadIdx.x == 0) jmin = nz;
    const double m = block_min(local, red);
    if (cfl_ring) {
        for (int j = threadIdx.x; j < nz; j += blockDim.x) {
            const size_t c = row + j;
            const double c_s = ph.adiabatic ? cs[c] : t.CsIso[i];
            const double d = cfl_cell64(g, t, ph, sn, i, j, c_s, nu[c], vr, vaz, vm0, qplus,
                                        qminus, E, corr_phi, corr_r, inv);
            if (d == m) atomicMin(&jmin, j);
        }
    }
    __syncthreads();
    double *o = out + (size_t)10 * i;
    if (threadIdx.x == 0) {
        o[0] = cfl_ring ? m : 1.0e300;
        o[1] = cfl_ring ? (double)jmin : -1.0;
        o[2] = shear;
        for (int k = 0; k < 6; ++k) o[3 + k] = 0.0;
        if (cfl_ring && jmin < nz) {
            const size_t c = row + jmin;
            const double c_s = ph.adiabatic ? cs[c] : t.CsIso[i];
            cfl_cell64(g, t, ph, sn, i, jmin, c_s, nu[c], vr, vaz, vm0, qplus, qminus, E,
                       corr_phi, corr_r, inv);
            for (int k = 0; k < 6; ++k) o[3 + k] = inv[k];
        }
    }
}

void launch_cfl_cells(const Launch &L, const State &s, double *out)
{
    k_cfl_cells<<<L.g.nr - 1, 256, 0, L.stream>>>(L.g, L.t, L.ph, L.ph.art_visc_sn, s.vr, s.vaz,
                                                  s.cs, s.nu, s.qplus, s.qminus, s.energy,
                                                  s.corr_phi, s.corr_r, out);
}

void launch_derived_cfl(const Launch &L, int mode, const State &s, unsigned long long *dt_min)
{
    auto k = L.pair ? k_derived_cfl<true> : k_derived_cfl<false>;
    // the FP32 screen's per-cell steps: only the FP64-arithmetic kernel and
    // StabilizeViscosity 2 use them (the pair kernel keeps the shared memory
    // for L1)
    const bool screen = !L.pair || L.ph.stabilize == 2;
    k<<<L.g.nr, 256, screen ? (size_t)L.g.nz * sizeof(float) : 0, L.stream>>>(
        L.g, L.t, L.ph, mode, L.ph.art_visc_sn, s.sigma, s.energy, s.vr, s.vaz, s.qplus,
        s.qminus, s.cs, s.H, s.P, s.T, s.nu, s.corr_phi, s.corr_r, dt_min);
}

void launch_gas_quantities(const Launch &L, double radius, double omf, const double *S,
                           const double *vaz, double *partial, double *out)
{
    const int rows = L.g.nr - 2;
    k_gas_quantities<<<rows, 256, 0, L.stream>>>(L.g, L.t, radius, omf, S, vaz, partial);
    k_reduce_rows<<<1, 32 * 2, 0, L.stream>>>(partial, rows, 2, out);
}

void launch_scale_sigma(const Launch &L, double *S, double target, const double *mass)
{
    const size_t n = (size_t)L.g.nr * L.g.nz;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    k_scale_sigma<<<blocks, 256, 0, L.stream>>>(S, n, target, mass);
}

void launch_disk_force(const Launch &L, int n, const double *px, const double *py,
                       const double *pa, const double *rsm, const double *S, const double *H,
                       double *partial, double *out)
{
    const int rows = L.g.nr - 2;
    for (int b0 = 0; b0 < n; b0 += kForceBodies) {
        ForceBodies fb{};
        fb.n = std::min(kForceBodies, n - b0);
        for (int b = 0; b < fb.n; ++b) {
            fb.xh[b] = (float)px[b0 + b];
            fb.xl[b] = (float)(px[b0 + b] - (double)fb.xh[b]);
            fb.yh[b] = (float)py[b0 + b];
            fb.yl[b] = (float)(py[b0 + b] - (double)fb.yh[b]);
            fb.a[b] = pa[b0 + b];
            fb.rsm[b] = rsm[b0 + b];
            if (fb.rsm[b] > 0.0) fb.klahr |= 1u << b;
        }
        const int width = 5 * fb.n;
        k_disk_force_bodies<<<rows, 256, 0, L.stream>>>(L.g, L.t, L.ph, fb, S, H, partial, width);
        k_reduce_cols<<<width, 32, 0, L.stream>>>(partial, rows, width, out + 5 * b0);
    }
}

void launch_check_finite(const Launch &L, const double *x, size_t n, unsigned long long *bad)
{
    const int bx = 256;
    k_check_finite<<<(unsigned)((n + bx - 1) / bx), bx, 0, L.stream>>>(x, n, bad);
}

}  // namespace fgpu
