// FP32-mixed form of the hydro step: device structures and the host engine
// (kernels_fp32.cu).  The C ABI (api.cu) routes a handle created with
// precision = FGPU_PRECISION_FP32_MIXED here.
#pragma once

#include "../../include/fargocpt_gb300.h"
#include "com_boundary.cuh"

#include <cuda_runtime.h>
#include <stddef.h>

#include <string>
#include <vector>

// raises a kernel's dynamic shared-memory limit, never lowers it (api.cu)
cudaError_t raise_smem_limit(const void *fn, size_t bytes);

namespace fgpu32 {

constexpr int kMaxBodies = 16;
// dynamic shared memory a ring kernel may ask for (227 KB less static use)
constexpr size_t kMaxRingSmem = 220 * 1024;

struct GeoF {
    int nr, nz;
    float dphi, invdphi;
    double dphi_d, invdphi_d;
    // OmegaFrame: the stored v_phi residual is about the inertial Keplerian
    // speed, so the frame enters only where frame velocities are asked for
    double omega_frame;
    float omega_f;  // the same in FP32
};

// Per-ring tables in FP32, plus the FP64 values the FP64 islands need.
struct TablesF {
    const float *Rinf, *Rsup, *Rmed, *Surf, *InvRmed, *InvSurf, *InvDiffRmed, *InvDiffRsup,
        *InvDiffRsupRb, *InvRinf, *RinfSq, *TwoOverDRa2, *OmegaK, *InvOmegaK, *CsIso,
        *InvDxSrc, *InvDxTheta, *EModel, *HFacAdi, *InvCell, *InvCell2, *TwoOverRmedSum;
    // Keplerian reference terms
    const float *Kbal;      // (v_K face)^2 / Rinf - dPhi_K/dr at interface i
    const float *Aface;     // 0.5 (v_K(i) + v_K(i-1))
    const float *Shear;     // d(v_K / r)/dr at interface i
    const float *DJ;        // J_K(i-1) - J_K(i), J_K = r v_K
    const float *JSlope;    // (J_K(i+1) - J_K(i)) / (Rmed(i+1) - Rmed(i))
    const float *DRmed;     // Rmed(i) - Rmed(i-1)
    const float *LSqTW;     // TW length scale squared, pow(C, 2) pow(max(dr, r dphi), 2)
    const float *TwoOverDRmed2; // 2 / (Rmed(i)^2 - Rmed(i-1)^2)
    // StabilizeViscosity correction-factor ring terms (viscosity.cpp:280-331)
    const float *Ra3IDRmed, *F43, *CrPp1, *CrPp2, *CrRr1, *CrRr2, *CrRp, *CrScale;
    const float *DRsup;     // Rsup(i) - Rinf(i), formed in FP64 (an FP32 difference of
                            // the radii loses ~1e-4 of it on fine grids)
    const float *RsupIDRR;  // Rsup(i) / ((Rsup(i) - Rinf(i)) Rmed(i)): div v without
                            // the cancelling v_r Rinf products
    const float *OmRefDiff; // v_K(i)/R(i) - v_K(i+1)/R(i+1)
    const float *Vref;      // v_K(Rmed)
    const double *Rmed_d, *InvRmed_d, *Vref_d, *Surf_d, *PhiK_d, *cos_d, *sin_d;
    // cell centres as float pairs: Rmed = Rmed + RmedLo, cos (j dphi) =
    // cosHi + cosLo, sin likewise
    const float *RmedLo, *cosHi, *cosLo, *sinHi, *sinLo;
    // Rinf - (Rmed(i) + Rmed(i-1)) / 2: the reference's interface azimuthal
    // speed, the mean of four frame velocities plus Rinf OmegaFrame, exceeds
    // the mean inertial speed by OmegaFrame times it
    const float *RinfOff;
};

struct PhysF {
    int adiabatic, art_visc_sn, dissipation, limiter_mc, fast_transport;
    int art_visc_tw;  // Tscharnuter-Winkler artificial viscosity
    int stabilize;    // StabilizeViscosity 0 / 1 / 2
    int heating_viscous, cooling_beta, beta_ref;
    int leapfrog;  // LeapFrog integrator: three CFL limits x 0.6
    int correct_sg;  // CorrectDiskSelfgravity: disk force from sigma less its ring mean
    float gm1, g_gm1, mu, alpha, constant_viscosity, C2, four_C2, rvf, hvf, cfl, inv_hc_limit;
    float sigma_min, sigma_floor10, eps_smooth, c_v_inv, mu_over_R, cool_const, mu_gm1_over_R;
    float emin_fac, emax_fac;
    double G_d;
};

struct BodiesF {
    int n;
    int star_at_origin;
    double x[kMaxBodies], y[kMaxBodies], a[kMaxBodies];
    float xh[kMaxBodies], xl[kMaxBodies], yh[kMaxBodies], yl[kMaxBodies]; // x = xh + xl
    float gm[kMaxBodies], rsm[kMaxBodies];
    float gm_ref, ix, iy;
};

// the position of body k as an unevaluated pair of floats
__host__ __device__ inline void split_position(BodiesF &b, int k)
{
    b.xh[k] = (float)b.x[k];
    b.xl[k] = (float)(b.x[k] - (double)b.xh[k]);
    b.yh[k] = (float)b.y[k];
    b.yl[k] = (float)(b.y[k] - (double)b.yh[k]);
}

struct BcF {
    int sigma_in, sigma_out, energy_in, energy_out, vr_in, vr_out, vaz_in, vaz_out;
    float kep_in, kep_out;  // Keplerian-hook value of the residual
    float zg_in, zg_out;    // zero-gradient offset of the residual between rings
    // per field (0 sigma, 1 energy, 2 v_r, 3 v_phi residual) and side: the
    // disk-model value (sigma: high and low part), the viscous-outflow factors,
    // the Keplerian-radial values, the zero-shear ratio and offset of the
    // residual, the balanced residual
    float val_in[4][2], val_out[4][2];
    const float *nu;        // viscosity (viscous-outflow hook)
};

struct DampQF {
    int kind_in, kind_out, active_in, active_out, limit_in, limit_out, vector;
    float tau_in, tau_out;
    const float *fac_in, *fac_out;
    const float *x0_zero_in, *x0_zero_out;  // per-ring X0 of the "zero" kind
};
struct DampingF {
    DampQF q[4];
};

// One planet's accretion region and constants (accretion.cpp:84-480), as the
// host finds them (see fgpu_accrete_onto_planet).
struct AccrF {
    int type, i0, i1, j0, ncols;
    double x, y, rhill, frac1, frac2, facc1, facc2, f_const, dist_max, density_floor, omf;
};

// Host constants of every boundary hook in FP64 (api.cu), shared by both forms.
void boundary_values(const fgpu_params &p, const double *Rmed, const double *Rinf, int nr,
                     double vin[4][2], double vout[4][2]);

struct StateF {
    float *sigma, *vr, *dv, *energy, *sigma0, *vr0, *dv0, *energy0;
    float *sigma_lo;  // low part of the compensated sigma (sigma = sigma + sigma_lo)
};

// Every buffer and constant one disk's step touches, as the batched kernels
// read it from device memory.  s holds the step-start state (vr, dv buffers
// A); the source terms write the B buffers, transport writes back to A, so
// the buffers a step uses are the same every step (graph-capturable).
struct DiskF {
    GeoF g;
    TablesF t;
    PhysF ph;
    BcF bc;
    DampingF dm;
    StateF s;
    float *vr_b, *dv_b;
    float *sigma_t, *energy_t, *sigma_lo_t;  // after radial transport
    int *ring_shift;  // the azimuthal pass's integer shift per ring (AdvectSHIFT)
    float *mom[4];
    float *pot, *P, *cs, *H, *nu, *T, *Qr, *Qp, *divv, *trr, *tpp, *trp, *qplus, *qminus;
    unsigned int *dtmin;
    int damping, nq;
};

// The per-step inputs of one disk: dt (FP64 for the FARGO phase, FP32 for
// the rest), the start time, the cooling rate factor and the bodies.
struct StepF {
    double dt, t;
    float fdt, beta_inv;
    int run, pad;
    BodiesF b;
};

// Device-side run clock of one disk (sim::CalculateTimeStep and the monitor
// clamp of sim::run, simulation.cpp:100-118, 505-558) and the circular
// orbits its planets follow around the central star.
struct ClockF {
    double t, last_dt, t_end, monitor_dt, cfl_max_var;
    double G, mstar, beta_inv0, beta_ramp;
    int n_monitor, steps, active, n_planets;
    double q[kMaxBodies], a[kMaxBodies], phase[kMaxBodies];
};

// Damping ring set-up, computed by the FP64 set-up code (the same ring search).
struct DampQSpec {
    int kind_in = 0, kind_out = 0, active_in = 0, active_out = 0, limit_in = 0, limit_out = 0;
    double tau_in = 1.0, tau_out = 1.0;
};

class Engine32 {
  public:
    int create(const fgpu_params &p, const double *radii, cudaStream_t stream);
    void destroy();
    int upload(int field, const double *host, int rows);
    int download(int field, double *host, int rows);
    int to_fp64(int field, double *dst, int rows);
    void set_bodies(int n, const fgpu_body *b, double ix, double iy, double omega_frame = 0.0);
    // correct_v_azimuthal: the frame velocities less dOmega * Rmed
    void correct_v_azimuthal(double domega) { pend_dv -= domega; }
    int init_euler(double t);
    int derived_cfl(int mode);
    int cfl(double *dt_out);
    int boundary(double dt, bool final);
    int step(double dt, double t);
    // the phases step_LeapFrog composes (simulation.cpp:276-459)
    int kick(double dt, double t);
    int transport(double dt);
    int pressure();
    // the step's buffers are the ones the batched kernels were given
    bool canonical() const { return fld[FGPU_V_RADIAL] == vr_a && fld[FGPU_V_AZIMUTHAL] == dv_a; }
    int disk_force(double px, double py, double pa, double rsm, double out[5]);
    int disk_forces(int n, const double *x, const double *y, const double *a,
                    const double *rsm, double *out);
    // gas_total_mass and gas_angular_momentum within radius (out[0], out[1])
    int gas_quantities(double radius, double out[2]);
    // KeepDiskMassConstant's target mass
    void set_mass_target(double m) { mass_target = m; }
    int accrete(const AccrF &a, double out[3]);

    // centre-of-mass composite boundary: the constants and tables (owned by
    // the ABI handle) and the centres of the two boundary calls of a step
    bool com_any = false;
    ComSpec com{};
    ComCenter com_now[2]{}, com_after[2]{};
    void com_boundary(const ComCenter *c);
    void com_damping(double dt, const ComCenter *c);
    int check_finite(int *field, int *nr_out, int *naz_out);
    // the device description used by the batched kernels
    DiskF describe();
    const BodiesF &current_bodies() const { return bodies; }
    double beta_inv_at(double t) const { return beta_inv(t); }
    int rings() const { return nr; }
    int azimuthal() const { return nz; }
    const int *damping_rings(int *n) const
    {
        *n = (p.damping && n_rings) ? n_rings : 0;
        return host_damp_rings.data();
    }
    const fgpu_params &params() const { return p; }
    void set_cfl_valid(bool v) { cfl_valid = v; }

    DampQSpec damp_spec[4];
    std::string err;
    // phase marker: called with -1 before the first kernel of a step and with
    // the phase index after each phase (the FP64 form's phase list)
    void (*mark_fn)(void *, int) = nullptr;
    void *mark_ctx = nullptr;

  private:
    double beta_inv(double t) const;
    const double *offset_of(int f) const;
    StateF state();
    // applies the pending frame shifts of v_phi and its reference values
    int sync_frame();
    double pend_dv = 0.0, pend_dv0 = 0.0;  // shifts, per unit radius
    double *vaz_offset = nullptr;          // per ring: Vref - Rmed OmegaFrame
    std::vector<double> host_rmed, host_vref;
    double zg_in_base = 0.0, zg_out_base = 0.0;
    float *zero_vphi_tab = nullptr;        // damping target of v_phi -> 0 (frame)

    fgpu_params p{};
    cudaStream_t stream = nullptr;
    int nr = 0, nz = 0;
    size_t cells = 0, vcells = 0;
    GeoF geo{};
    TablesF tabs{};
    PhysF phys{};
    BodiesF bodies{};
    BcF bc{};
    DampingF dm{};
    float *fld[FGPU_FIELD_COUNT] = {};
    float *alt_sigma = nullptr, *alt_vr = nullptr, *alt_dv = nullptr, *alt_e = nullptr;
    float *vr_a = nullptr, *dv_a = nullptr;  // v_r, v_phi buffers at creation
    float *sigma_lo = nullptr, *alt_sigma_lo = nullptr;
    int *ring_shift = nullptr;  // AdvectSHIFT per ring, applied by the velocity rebuild
    float *mom[4] = {};
    float *tab_f = nullptr;
    double *tab_d = nullptr;
    float *tab_c = nullptr;  // cosHi, cosLo, sinHi, sinLo
    int nsm = 1;             // streaming multiprocessors of the device
    float *damp_mem = nullptr, *damp_aux = nullptr;
    int *damp_rings = nullptr;
    int n_rings = 0;
    std::vector<int> host_damp_rings;
    double *partial = nullptr, *red_out = nullptr, *stage = nullptr;
    unsigned int *d_dtmin = nullptr;
    unsigned long long *d_bad = nullptr;
    double *h_pinned = nullptr;
    int per = 4, az_block = 128;
    size_t az_smem = 0;
    int rb_per = 0;      // register-blocked azimuthal kernel: cells per thread (0: strided)
    size_t rb_smem = 0;
    bool az_stage = false;
    bool visc_recompute = false;  // c_s, H, nu before the final hooks (adiabatic)
    float *corr_phi = nullptr, *corr_r = nullptr;  // StabilizeViscosity factors
    void visc_corr(const StateF &s);
    int keep_mass();
    double mass_target = 0.0;
    bool cfl_valid = false;
};

}  // namespace fgpu32
