// Device-side data structures shared by the GB300 hydro kernels and the C ABI.
//
// Layout (FargoCPT's t_polargrid, src/polargrid.h:111-133): row-major double,
// ring-major, cell(i, j) = j + i * nz, azimuth contiguous.  Scalar grids have
// nr rows, vector grids (v_radial, tau_r_phi) nr + 1 rows.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "com_boundary.cuh"

namespace fgpu {

constexpr int kMaxBodies = 16;

// Per-ring metric tables, uploaded once (host computes them with the same
// expressions FargoCPT's init_radialarrays uses, src/init.cpp:188-225, so the
// device sees bit-identical values).
struct Tables {
    const double *Rinf, *Rsup, *Rmed, *Surf, *InvRmed, *InvSurf, *InvDiffRmed,
        *InvDiffRsup, *InvDiffRsupRb, *InvRinf;
    const double *RinfSq;      // pow(Rinf, 2)
    const double *TwoOverDRa2; // 2 / (pow(Ra[i+1],2) - pow(Ra[i],2))
    const double *OmegaK;      // calculate_omega_kepler(Rmed)
    const double *InvOmegaK;   // 1 / calculate_omega_kepler(Rmed)
    const double *CsIso;       // isothermal c_s per ring (SourceEuler.cpp:983-990)
    const double *InvDxSrc;    // 2 / (dphi (Rsup + Rinf))  (SourceEuler.cpp:387)
    const double *InvDxTheta;  // 1 / (dphi Rmed)
    const double *EModel;      // beta-cooling disk-model energy per unit sigma
    const double *HFacAdi;     // 1 / (Omega_K sqrt(gamma)): H = c_s * HFacAdi (ideal EOS)
    const double *InvCell;     // 1 / min(Rsup - Rinf, Rmed dphi)  (cfl.cpp:223-225)
    const double *InvCell2;    // InvCell^2
    const double *TwoOverRmedSum; // 2 / (Rmed[i] + Rmed[i-1])  (viscosity.cpp:407)
    // Tscharnuter-Winkler artificial viscosity (artificial_viscosity.cpp:35-140)
    const double *LSqTW;       // pow(C, 2) * pow(max(Ra[i+1] - Ra[i], Rmed dphi), 2)
    const double *TwoOverDRmed2; // 2 / (pow(Rmed[i], 2) - pow(Rmed[i-1], 2))
    const double *DiffRmed;    // Rmed[i] - Rmed[i-1]
    // StabilizeViscosity correction factors (viscosity.cpp:256-348)
    const double *Ra3IDRmed;   // pow(Ra[i], 3) * InvDiffRmed[i]
    const double *F43;         // FourThirdInvRbInvdphiSq (init.cpp:213-214)
    const double *CrPp1, *CrPp2, *CrRr1, *CrRr2; // ring factors of c_r's four terms
    const double *CrRp;        // 1 / (dphi dphi Ra[i])
    const double *CrScale;     // RadialViscosityFactor / (0.5 (Rmed[i] + Rmed[i-1]))
    const double *cosj, *sinj; // cos / sin (dphi j)
    // the same as float pairs hi + lo (for the pair-arithmetic kernels)
    const float *RmedHi, *RmedLo, *cosHi, *cosLo, *sinHi, *sinLo;
    const float *InvDiffRmedHi, *InvDiffRmedLo, *InvSurfHi, *InvSurfLo;
    // every table above as float pairs: the pair of tab[i] is
    // ptab[(tab - tbase) + i]
    const double *tbase;
    const float2 *ptab;
};

struct Geo {
    int nr, nz;
    double dphi, invdphi;
    float2 pk_invdphi;    // invdphi as a float pair (split_pair_host)
};

// x as the float pair hi + lo of the float-pair kernels, computed on the
// host with the device split's bits (f2_split in fp64_pair.cuh: hi the top 24
// significant bits, lo the remaining 29 rounded to a float; zero below
// 2^-74, NaN from 2^128), so that a constant split once here is the pair
// those kernels would form from it.
inline float2 split_pair_host(double x)
{
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    const uint32_t w1 = (uint32_t)(b >> 32), w0 = (uint32_t)b;
    const uint32_t ax = w1 & 0x7fffffffu, sign = w1 & 0x80000000u;
    const uint32_t hb = ((ax - (896u << 20)) << 3) | (w0 >> 29);
    const uint32_t sbits = (hb & 0x7f800000u) - (52u << 23);
    float scale;
    memcpy(&scale, &sbits, sizeof scale);
    const float lf = (float)(w0 & 0x1fffffffu) * scale;
    uint32_t lb;
    memcpy(&lb, &lf, sizeof lb);
    const bool in = ax - (949u << 20) < (202u << 20);
    const uint32_t out = ax < (949u << 20) ? 0u : (0x7fc00000u | sign);
    const uint32_t rh = in ? (hb | sign) : out, rl = in ? (lb | sign) : out;
    float2 r;
    memcpy(&r.x, &rh, sizeof rh);
    memcpy(&r.y, &rl, sizeof rl);
    return r;
}

// Physics switches and constants (a flat copy of the fgpu_params subset the
// kernels read, plus host-precomputed products).
struct Phys {
    int adiabatic, art_visc_sn, dissipation, limiter_mc, fast_transport;
    int heating_viscous, cooling_beta, beta_ref;
    int leapfrog;         // LeapFrog integrator: three CFL limits x 0.6
    int art_visc_tw;      // Tscharnuter-Winkler artificial viscosity
    int stabilize;        // StabilizeViscosity 0 / 1 / 2
    int correct_sg;       // CorrectDiskSelfgravity: disk force from sigma less its ring mean
    double gamma, gm1, g_gm1, sqrt_gamma, mu, alpha, constant_viscosity;
    double C2;            // pow(ArtificialViscosityFactor, 2)
    double rvf, hvf, cfl, inv_hc_limit, sigma_min, sigma_floor10;
    double eps_smooth;    // ThicknessSmoothing
    double tmin, tmax, Rgas, sigma_sb, c_light, G, Mc;
    double c_v_inv;       // mu / R * (gamma - 1)
    double four_C2;       // 4 * pow(C, 2)
    double cool_const;    // 2 * 4 * sigma_sb / c (SubStep3's radiative alpha)
    double mu_gm1_over_R; // mu (gamma - 1) / R
    double emin_fac, emax_fac; // Tmin|Tmax / mu * R / (gamma - 1)
    float emin_fac_f, emax_fac_f;  // the same rounded to float (FP32 screens)
    // constants of the float-pair kernels as pairs (split_pair_host)
    float2 pk_gm1, pk_g_gm1, pk_alpha, pk_C2, pk_rvf, pk_hvf, pk_mu_gm1_over_R, pk_cool_const,
        pk_emin_fac, pk_eps_smooth;
};

struct Bodies {
    int n;
    double x[kMaxBodies], y[kMaxBodies], m[kMaxBodies], rsm[kMaxBodies], a[kMaxBodies];
    // positions and -G m as float pairs hi + lo, split on the host
    float xh[kMaxBodies], xl[kMaxBodies], yh[kMaxBodies], yl[kMaxBodies];
    float gmh[kMaxBodies], gml[kMaxBodies];
    double ix, iy;        // indirect term
    float2 pk_ix, pk_iy;  // the same as float pairs (split_pair_host)
    double omega_frame;
    // decided on the host, so that no kernel compares doubles per cell:
    // bit k set when body k has Klahr smoothing (rsm[k] > 0); the central
    // object at the origin without it; -G m of the central object
    unsigned klahr;
    int star_plain;
    double gm0;
};

// Ghost-ring hooks of one step (FGPU_BC_* per field and side).  val_in /
// val_out hold each hook's host-computed constants per field (0 sigma,
// 1 energy, 2 v_radial, 3 v_azimuthal): Keplerian c v_K; disk-model values;
// the viscous-outflow factors -1.5 s / Rinf[k]; Keplerian-radial values of the
// two ghost rings; zero-shear radii (edge ring, active ring); the balanced
// velocity before the frame correction.
struct BcSpec {
    int sigma_in, sigma_out, energy_in, energy_out, vr_in, vr_out, vaz_in, vaz_out;
    double val_in[4][2], val_out[4][2];
};

// Damping set-up of one quantity (boundary_conditions/damping.cpp:311-752).
struct DampQ {
    int kind_in, kind_out;      // FGPU_DAMP_*
    int active_in, active_out;
    int limit_in, limit_out;    // ring limits
    int vector;                 // uses Rinf (v_radial) instead of Rmed
    int is_density;
    double tau_in, tau_out;
    double x0_zero_in;          // X0 of "zero" damping at the inner edge
    const double *fac_in, *fac_out; // per-ring pow((r - r_lim)/(r_edge - r_lim), 2)
};

struct Damping {
    DampQ q[4];                 // v_radial, v_azimuthal, sigma, energy
};

// One planet's accretion region and constants (accretion.cpp:84-480); the
// region's rings and azimuthal indices are found on the host exactly as
// hill_radial_index / hill_azimuthal_index do.
struct AccretionSpec {
    int type;                   // FGPU_ACCRETION_*
    int i0, i1;                 // rings i0 .. i1
    int j0, ncols;              // azimuthal indices j0 .. j0 + ncols - 1 (wrapped)
    double x, y, rhill;
    double frac1, frac2;        // zone radii in Hill radii (frac2: Kley's inner zone)
    double facc1, facc2;        // removal fractions per call
    double f_const, dist_max;   // viscous accretion profile
    double density_floor, omf;
};

// Pointers of the evolved state and the work arrays of one step.
struct State {
    double *sigma, *vr, *vaz, *energy;        // current state
    double *sigma0, *vr0, *vaz0, *energy0;    // reference values
    double *cs, *H, *P, *T, *nu, *qplus, *qminus, *pot;
    double *divv, *trr, *tpp, *trp, *qr, *qphi;
    double *corr_phi, *corr_r;                // StabilizeViscosity factors (or null)
};

}  // namespace fgpu
