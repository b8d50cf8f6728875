// C ABI of the GB300 hydro engine (include/fargocpt_gb300.h).
//
// Host side: owns the device buffers, computes the per-ring metric tables with
// the expressions of FargoCPT's init_radialarrays (src/init.cpp:188-225) so the
// device sees bit-identical metric values, resolves boundary and damping
// set-up, and sequences the kernels of one hydro step on the handle's stream.
#include "../../include/fargocpt_gb300.h"
#include "hydro.cuh"
#include "kernels.h"
#include "fp32_engine.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <mutex>
#include <unordered_map>
#include <vector>

using namespace fgpu;

struct fgpu_engine {
    fgpu_params p;
    int nr = 0, nz = 0;
    size_t cells = 0, vcells = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    double *field[FGPU_FIELD_COUNT] = {};
    double *sigma_alt = nullptr, *vr_alt = nullptr, *vaz_alt = nullptr, *energy_alt = nullptr;
    double *mom[4] = {};
    double *ring_ws = nullptr;
    int *ring_shift = nullptr;  // the pair azimuthal pass's shift per ring
    size_t az_smem = 0;
    int az_block = 256;
    bool pair_arith = true;  // the kernels' arithmetic in float pairs (else FP64)
    // div v and the stress tensor hold the stress kernel's float pairs
    // (stress_as_pairs), the artificial pressures those of the float-pair
    // artificial viscosity, until join_pair_fields turns them into doubles
    bool stress_pairs = false, q_pairs = false;
    int radial_chunk = 16;

    double *tables_mem = nullptr;
    float *pair_mem = nullptr;  // Rmed, cos, sin as float pairs
    Tables tabs{};
    double *damp_mem = nullptr;
    int *damp_rings = nullptr;
    int n_damp_rings = 0;
    double *partial = nullptr, *red_out = nullptr;
    unsigned long long *d_dtmin = nullptr, *d_bad = nullptr;
    double *h_pinned = nullptr;

    Geo geo{};
    Phys ph{};
    Bodies bodies{};
    BcSpec bc{};
    Damping dm{};
    bool cfl_valid = false;
    std::vector<double> host_radii;

    // phase timing: one row of events per recorded step
    bool timing = false;
    std::vector<std::vector<cudaEvent_t>> ev_rows;
    std::vector<cudaEvent_t> ev_free;
    int ev_cursor = 0;

    // asynchronous snapshots: device staging, a copy stream and its events
    double *snap_stage = nullptr;
    // StabilizeViscosity correction factors (VISCOSITY_CORRECTION_FACTOR_PHI/R),
    // zero until the first stress evaluation like the reference's grids
    double *corr_phi = nullptr, *corr_r = nullptr;
    size_t snap_capacity = 0;  // doubles
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_staged = nullptr, snap_copied = nullptr;
    bool snap_pending = false;

    // centre-of-mass composite boundary: constants, tables on the device
    // (com_mem), and the centres of the current and the post-N-body state
    ComSpec com{};
    bool com_any = false, com_ready = false;
    ComCenter com_now[2]{}, com_after[2]{};
    double *com_mem = nullptr;

    // KeepDiskMassConstant: the mass sigma is rescaled to after each final
    // boundary call (sim::init's total_disk_mass_old)
    double mass_target = 0.0;
    bool mass_target_set = false;

    fgpu32::Engine32 *e32 = nullptr;  // FP32-mixed form, when selected
    bool owns_stream = true;          // false for the disks of a batch
    bool batch_owned = false;         // disks of a batch are freed by the batch
};

static const char *kPhaseNames[] = {
    "potential", "source", "artvisc_q", "artvisc_v", "stress", "viscous_substep3",
    "ghost_pre", "transport_radial", "transport_azimuthal", "finish", "damping",
    "ghost_post", "derived_cfl"};
constexpr int kPhases = sizeof(kPhaseNames) / sizeof(kPhaseNames[0]);

static cudaEvent_t take_event(fgpu_engine *e)
{
    if (!e->ev_free.empty()) {
        cudaEvent_t ev = e->ev_free.back();
        e->ev_free.pop_back();
        return ev;
    }
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    return ev;
}

// Marks the end of phase `k` of the current step (k = -1 opens the step).
static void mark(fgpu_engine *e, int k)
{
    if (!e->timing) return;
    if (k < 0) {
        e->ev_rows.emplace_back();
        e->ev_rows.back().reserve(kPhases + 1);
    }
    cudaEvent_t ev = take_event(e);
    cudaEventRecord(ev, e->stream);
    e->ev_rows.back().push_back(ev);
}

// A named NVTX range around each ABI call that enqueues GPU work, so that
// profilers (ncu --nvtx, Nsight Systems) group the kernels by the FargoCPT
// function they replace.  NVTX v3 is header-only and costs a few
// nanoseconds when no tool is attached.
struct NvtxCall {
    explicit NvtxCall(const char *name) { nvtxRangePushA(name); }
    ~NvtxCall() { nvtxRangePop(); }
};

#define CK(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            eng->err = std::string(#call) + ": " + cudaGetErrorString(e_);       \
            return FGPU_ERR_CUDA;                                                 \
        }                                                                         \
    } while (0)

static bool is_vector_field(int f)
{
    return f == FGPU_V_RADIAL || f == FGPU_V_RADIAL0 || f == FGPU_TAU_R_PHI;
}

static int field_rows(const fgpu_engine *e, int f) { return is_vector_field(f) ? e->nr + 1 : e->nr; }

static bool is_pair_field(int f)
{
    return f == FGPU_DIV_V || f == FGPU_TAU_R_R || f == FGPU_TAU_PHI_PHI || f == FGPU_TAU_R_PHI ||
           f == FGPU_Q_R || f == FGPU_Q_PHI;
}

// The fields the float-pair kernels pass on as pairs, as doubles again
// before anything outside the step reads or overwrites them: the rows the
// last evaluation wrote (every ring of div v, tau_rr, tau_phiphi and the
// artificial pressures; rings 1 .. nr - 1 of tau_rphi)
static int join_pair_fields(fgpu_engine *eng)
{
    const size_t nz = eng->nz, rows = eng->nr;
    if (eng->stress_pairs) {
        launch_join_pairs(eng->stream, eng->field[FGPU_DIV_V], rows * nz);
        launch_join_pairs(eng->stream, eng->field[FGPU_TAU_R_R], rows * nz);
        launch_join_pairs(eng->stream, eng->field[FGPU_TAU_PHI_PHI], rows * nz);
        launch_join_pairs(eng->stream, eng->field[FGPU_TAU_R_PHI] + nz, (rows - 1) * nz);
        eng->stress_pairs = false;
    }
    if (eng->q_pairs) {
        launch_join_pairs(eng->stream, eng->field[FGPU_Q_R], rows * nz);
        launch_join_pairs(eng->stream, eng->field[FGPU_Q_PHI], rows * nz);
        eng->q_pairs = false;
    }
    CK(cudaGetLastError());
    return FGPU_OK;
}

extern "C" int fgpu_grid_radii(int spacing, double rmin, double rmax, int nrad, double *radii)
{
    if (!radii || nrad < 4 || !(rmax > rmin) || !(rmin > 0.0)) return FGPU_ERR_BAD_ARG;
    if (spacing == FGPU_SPACING_LOGARITHMIC) {
        // init.cpp:93-100
        const double q = std::pow((rmax / rmin), 1.0 / ((double)nrad - 2.0));
        for (int n = 0; n <= nrad + 1; ++n) radii[n] = rmin * std::pow(q, (double)n - 1.0);
    } else if (spacing == FGPU_SPACING_ARITHMETIC) {
        // init.cpp:103-110
        const double interval = (rmax - rmin) / (double)(nrad - 2.0);
        for (int n = 0; n <= nrad + 1; ++n) radii[n] = rmin + interval * (double)(n - 1.0);
    } else {
        return FGPU_ERR_BAD_ARG;
    }
    return FGPU_OK;
}

extern "C" const char *fgpu_last_error(const fgpu_engine *eng)
{
    return eng ? eng->err.c_str() : "null engine";
}

extern "C" int fgpu_get_stream(const fgpu_engine *eng, void **stream)
{
    if (!eng || !stream) return FGPU_ERR_BAD_ARG;
    *stream = (void *)eng->stream;
    return FGPU_OK;
}

// ------------------------------------------------------------------------
// damping ring search (find_cell_id.cpp:222-452 with NDEBUG clamping)
// ------------------------------------------------------------------------
static int cell_id_p(const fgpu_params &p, int nr, const double *Rmed, double r, bool rinf)
{
    int id;
    if (p.radial_spacing == FGPU_SPACING_LOGARITHMIC) {
        const double g = std::pow(p.rmax / p.rmin, 1.0 / ((double)p.nrad - 2.0));
        const double ilg = 1.0 / std::log(g);
        if (rinf) {
            id = (int)std::floor(std::log(r / p.rmin) * ilg) + 1;
        } else {
            const double oc = 3.0 / 2.0 / p.rmin * (1 - std::pow(g, 2.0)) / (1 - std::pow(g, 3.0));
            id = (int)std::floor(std::log(r * oc) * ilg) + 1;
        }
    } else {
        const double g = ((double)p.nrad - 2.0) / (p.rmax - p.rmin);
        id = (int)std::floor((r - p.rmin) * g) + 1;
        if (!rinf && id >= 0 && id <= nr && Rmed[id] > r) id--;
    }
    if (id < 0) id = 0;
    if (id > nr - 1) id = nr - 1;
    return id;
}

static int cell_id(const fgpu_engine *e, const std::vector<double> &Rmed, double r, bool rinf)
{
    return cell_id_p(e->p, e->nr, Rmed.data(), r, rinf);
}

// Dynamic shared-memory limits belong to the kernel, process-wide: an engine
// may only raise a limit, or a later engine with shorter rings would shrink
// it under the launches of an earlier one.
cudaError_t raise_smem_limit(const void *fn, size_t bytes)
{
    static std::mutex mu;
    static std::unordered_map<const void *, size_t> limit;
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = limit[fn];
    if (bytes <= cur) return cudaSuccess;
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

// nodes of each viscous-speed lookup table (viscous_radial_speed.cpp:256)
constexpr int kComTableNodes = 1000;

static int clamp_id(int id, bool vec, int nr)
{
    const int mx = nr - (vec ? 0 : 1);
    return std::min(std::max(id, 0), mx);
}

static double omega_kepler(const fgpu_params &p, double r)
{
    return std::sqrt(p.G * p.hydro_center_mass / (r * r * r));  // Theo.cpp:246-249
}

static bool hook_allowed(int field, int kind, bool outer);

static int validate(const fgpu_params *p, std::string &why)
{
    if (p->nrad < 6 || p->naz < 8) { why = "nrad >= 6 and naz >= 8 required"; return FGPU_ERR_BAD_ARG; }
    if (p->naz > 8192) { why = "naz > 8192 not supported by the azimuthal kernel (16 cells x 512 threads per ring)"; return FGPU_ERR_UNSUPPORTED; }
    if (p->eos != FGPU_EOS_ISOTHERMAL && p->eos != FGPU_EOS_IDEAL) { why = "eos"; return FGPU_ERR_BAD_ARG; }
    if (p->art_visc != FGPU_ARTVISC_NONE && p->art_visc != FGPU_ARTVISC_SN && p->art_visc != FGPU_ARTVISC_TW) { why = "art_visc"; return FGPU_ERR_BAD_ARG; }
    if (p->stabilize_viscosity < 0 || p->stabilize_viscosity > 2) { why = "stabilize_viscosity must be 0, 1 or 2"; return FGPU_ERR_BAD_ARG; }
    if (p->precision != FGPU_PRECISION_FP64 && p->precision != FGPU_PRECISION_FP32_MIXED) { why = "precision"; return FGPU_ERR_BAD_ARG; }
    if (p->integrator != FGPU_INTEGRATOR_EULER && p->integrator != FGPU_INTEGRATOR_LEAPFROG) { why = "integrator"; return FGPU_ERR_BAD_ARG; }
    if (p->radial_spacing != FGPU_SPACING_LOGARITHMIC && p->radial_spacing != FGPU_SPACING_ARITHMETIC) { why = "radial_spacing"; return FGPU_ERR_BAD_ARG; }
    const int bcs[8] = {p->bc_sigma_inner, p->bc_sigma_outer, p->bc_energy_inner, p->bc_energy_outer,
                        p->bc_vrad_inner, p->bc_vrad_outer, p->bc_vaz_inner, p->bc_vaz_outer};
    for (int k = 0; k < 8; ++k) {
        if (bcs[k] < FGPU_BC_NONE || bcs[k] > FGPU_BC_BALANCED) { why = "boundary kind"; return FGPU_ERR_BAD_ARG; }
        if (!hook_allowed(k / 2, bcs[k], k % 2 == 1)) {
            why = bcs[k] == FGPU_BC_VISCOUS
                      ? "the viscous v_radial hook exists at the inner edge only (the reference's "
                        "outer version reads past the viscosity grid)"
                      : "boundary kind not available for this field";
            return bcs[k] == FGPU_BC_VISCOUS ? FGPU_ERR_UNSUPPORTED : FGPU_ERR_BAD_ARG;
        }
    }
    for (int q = 0; q < 4; ++q) {
        if (p->damping_inner[q] < 0 || p->damping_inner[q] > FGPU_DAMP_MEAN ||
            p->damping_outer[q] < 0 || p->damping_outer[q] > FGPU_DAMP_MEAN) {
            why = "damping kind"; return FGPU_ERR_BAD_ARG;
        }
    }
    if (!(p->cfl > 0) || !(p->G > 0) || !(p->hydro_center_mass > 0)) { why = "cfl, G, mass must be > 0"; return FGPU_ERR_BAD_ARG; }
    const int comp[2] = {p->composite_inner, p->composite_outer};
    for (int side = 0; side < 2; ++side) {
        if (comp[side] != FGPU_COMPOSITE_INDIVIDUAL && comp[side] != FGPU_COMPOSITE_CENTER_OF_MASS) {
            why = "composite boundary kind"; return FGPU_ERR_BAD_ARG;
        }
        if (comp[side] != FGPU_COMPOSITE_CENTER_OF_MASS) continue;
        // boundary_conditions/config.cpp:512-528
        for (int q = 0; q < 4; ++q) {
            if ((side ? p->damping_outer[q] : p->damping_inner[q]) != FGPU_DAMP_NONE) {
                why = "damping is enabled twice: per field and through the center-of-mass boundary";
                return FGPU_ERR_BAD_ARG;
            }
        }
    }
    return FGPU_OK;
}

// compute_v_kepler, Theo.cpp:207-211
static double v_kepler(const fgpu_params &p, double r)
{
    return std::sqrt(p.G * p.hydro_center_mass / r);
}

// The constants of every boundary hook (see BcSpec), with the reference's
// expressions: keplerian_azimuthal.cpp:27-31, diskmodel.cpp:18-31,
// viscous.cpp:33-35, keplerian_radial.cpp:31-33 and 55-57, zero_shear.cpp:28-32,
// balanced.cpp:20-66 with support_azi_* (Theo.cpp:131-157).
namespace fgpu32 {
void boundary_values(const fgpu_params &p, const double *Rmed, const double *Rinf, int nr,
                     double vin[4][2], double vout[4][2])
{
    for (int f = 0; f < 4; ++f) vin[f][0] = vin[f][1] = vout[f][0] = vout[f][1] = 0.0;
    const double sigexp = -p.sigma_slope;
    auto calc_sig = [&](double R) { return p.sigma0 * std::pow(R, sigexp); };
    auto calc_eng = [&](double R) {
        return 1.0 / (p.gamma - 1.0) * p.sigma0 * std::pow(p.aspect_ratio, 2) *
               std::pow(R, sigexp - 1.0 + 2.0 * p.flaring_index);
    };
    auto balanced = [&](double R) {
        const double vk_2 = std::pow(v_kepler(p, R), 2);
        double support = 0.0;
        if (!p.profile_cutoff_outer) {
            const double F = p.flaring_index, S = p.sigma_slope;
            const double h = p.aspect_ratio * std::pow(R, F);
            support += (2.0 * F - 1.0 - S) * std::pow(h, 2);
            const double eps = p.thickness_smoothing;
            support += (1.0 + (F + 1.0) * std::pow(h * eps, 2)) /
                       std::pow(std::sqrt(1 + std::pow(h * eps, 2)), 3);
        }
        if (p.binary_quadrupole_moment > 0.0) {
            support += 3.0 * p.binary_quadrupole_moment / std::pow(R, 2);
        }
        return std::sqrt(vk_2 * support);
    };
    const int kinds_in[4] = {p.bc_sigma_inner, p.bc_energy_inner, p.bc_vrad_inner, p.bc_vaz_inner};
    const int kinds_out[4] = {p.bc_sigma_outer, p.bc_energy_outer, p.bc_vrad_outer,
                              p.bc_vaz_outer};
    for (int f = 0; f < 4; ++f) {
        for (int side = 0; side < 2; ++side) {
            const int kind = side ? kinds_out[f] : kinds_in[f];
            double *v = side ? vout[f] : vin[f];
            const bool vec = f == 2;
            const int edge = side ? (vec ? nr : nr - 1) : 0;
            const int next = side ? edge - 1 : 1;
            switch (kind) {
            case FGPU_BC_KEPLERIAN:
                v[0] = (side ? p.vaz_outer_keplerian_factor : p.vaz_inner_keplerian_factor) *
                       v_kepler(p, Rmed[edge]);
                break;
            case FGPU_BC_DISKMODEL:
                v[0] = f == 0 ? calc_sig(Rmed[edge]) : calc_eng(Rmed[edge]);
                break;
            case FGPU_BC_VISCOUS:
                v[0] = -1.5 * p.viscous_outflow_speed / Rinf[0];
                v[1] = -1.5 * p.viscous_outflow_speed / Rinf[1];
                break;
            case FGPU_BC_KEPLERIAN_RADIAL: {
                const double c = side ? p.vrad_outer_keplerian_factor : p.vrad_inner_keplerian_factor;
                v[0] = c * v_kepler(p, Rmed[edge]);
                v[1] = c * v_kepler(p, Rmed[next]);
                break;
            }
            case FGPU_BC_ZEROSHEAR:
                v[0] = Rmed[edge];
                v[1] = Rmed[next];
                break;
            case FGPU_BC_BALANCED:
                v[0] = balanced(Rmed[edge]);
                break;
            default:
                break;
            }
        }
    }
}

// viscous_speed::init_vr_table_boundary (viscosity/viscous_radial_speed.cpp:
// 269-347) with the model functions it evaluates (get_sigma, get_nu2, get_w,
// derive, get_vr_with_numerical_viscous_speed and the outer grid correction,
// viscous_radial_speed.cpp:14-254; Theo.cpp:131-200).  radii holds nr + 2
// interface radii (Radii[0 .. nr + 1]).  Each table gets n + 1 nodes: the
// reference interpolates from node i to node i + 1 and has n, so that a radius
// in its last bin reads past the table; the extra node is that next node of
// the same formula.
void viscous_speed_tables(const fgpu_params &p, const double *radii, const double *Rmed, int nr,
                          double mass_all, double mass_center, bool binary_on_primary,
                          double com_max_dist, int n, double min_r[2], double dlog[2],
                          double *r_tab, double *vr_tab)
{
    const bool adi = p.eos == FGPU_EOS_IDEAL;
    auto cut_out = [&](double x) {
        return 1.0 / (1.0 + std::exp((x - p.profile_cutoff_point_outer) / p.profile_cutoff_width_outer));
    };
    auto cut_in = [&](double x) {
        return 1.0 / (1.0 + std::exp((p.profile_cutoff_point_inner - x) / p.profile_cutoff_width_inner));
    };
    auto get_sigma = [&](double R) {
        double d = p.sigma0 * std::pow(R, -p.sigma_slope);
        const double floor = p.sigma_floor * p.sigma0;
        if (p.profile_cutoff_outer) d *= cut_out(R);
        if (p.profile_cutoff_inner) d *= cut_in(R);
        return std::max(d, floor);
    };
    auto get_nu2 = [&](double R, double M, double Sigma) {
        const double v_k = std::sqrt(p.G * M / R);
        const double h = p.aspect_ratio * std::pow(R, p.flaring_index);
        double cutoff = 1.0;
        if (p.profile_cutoff_outer) cutoff *= cut_out(R);
        if (p.profile_cutoff_inner) cutoff *= cut_in(R);
        double cs_adb, H;
        if (adi) {
            const double gamma = p.gamma;
            double energy = cutoff * 1.0 / (gamma - 1.0) * Sigma * std::pow(h * v_k, 2);
            const double energy_floor = p.minimum_temperature * Sigma / p.mu * p.R_gas / (gamma - 1.0);
            const double energy_ceil = p.maximum_temperature * Sigma / p.mu * p.R_gas / (gamma - 1.0);
            energy = std::max(energy, energy_floor);
            energy = std::min(energy, energy_ceil);
            cs_adb = std::sqrt(gamma * (gamma - 1.0) * energy / Sigma);
            const double cs_iso = std::sqrt((gamma - 1.0) * energy / Sigma);
            H = cs_iso / (v_k / R);
        } else {
            cs_adb = h * v_k;
            H = h * R;
        }
        return p.viscous_alpha * cs_adb * H;
    };
    // the smoothed, pressure-supported angular velocity; the quadrupole term
    // is zero unless VazimuthalConsidersQuadropoleMoment is set
    auto get_w = [&](double R, double M) {
        const double F = p.flaring_index, S = p.sigma_slope;
        const double h = p.aspect_ratio * std::pow(R, F);
        const double eps = p.thickness_smoothing;
        const double smooth = (1.0 + (F + 1.0) * std::pow(h * eps, 2)) /
                              std::pow(std::sqrt(1 + std::pow(h * eps, 2)), 3);
        const double press = (2.0 * F - 1.0 - S) * std::pow(h, 2);
        const double quad = p.binary_quadrupole_moment > 0.0
                                ? 3.0 * p.binary_quadrupole_moment / std::pow(R, 2) : 0.0;
        const double vk_2 = p.G * M / R;
        return std::sqrt(vk_2 * (quad + smooth + press)) / R;
    };
    auto derive = [](double x, auto &&f) {
        const double h = 8.0e-4 * x;
        const double f1 = -1.0 * f(x + 2.0 * h);
        const double f2 = 8.0 * f(x + h);
        const double f3 = -8.0 * f(x - h);
        const double f4 = 1.0 * f(x - 2.0 * h);
        return (f1 + f2 + f3 + f4) / (12.0 * h);
    };
    auto vr_numerical = [&](double r, double M) {
        auto w = [&](double x) { return get_w(x, M); };
        auto nu_S_r3_dwdr = [&](double x) {
            const double dw_dr = derive(x, w);
            const double Sigma = get_sigma(x);
            return get_nu2(x, M, Sigma) * Sigma * std::pow(x, 3) * dw_dr;
        };
        auto r2_w = [&](double x) { return std::pow(x, 2) * get_w(x, M); };
        const double num = 1.0 / r * derive(r, nu_S_r3_dwdr);
        const double den = get_sigma(r) * derive(r, r2_w);
        return num / den;
    };
    // GlobalRmed (init.cpp:176-179) up to index nr
    std::vector<double> grmed(nr + 1);
    for (int k = 0; k <= nr; ++k) {
        grmed[k] = 2.0 / 3.0 * (std::pow(radii[k + 1], 3) - std::pow(radii[k], 3));
        grmed[k] = grmed[k] / (std::pow(radii[k + 1], 2) - std::pow(radii[k], 2));
    }
    auto outer_correction = [&](double r, double M) {
        const int id = cell_id_p(p, nr, Rmed, r, false);
        const int k = std::max(2, std::min(std::max(id, 0), nr));
        const double rinf = radii[k];
        const double rmed_p = grmed[k + 1], rmed = grmed[k], rmed_m = grmed[k - 1],
                     rmed_m2 = grmed[k - 2];
        const double w_p = get_w(rmed_p, M), w = get_w(rmed, M), w_m = get_w(rmed_m, M),
                     w_m2 = get_w(rmed_m2, M);
        const double dw_dr = (0.5 * (w_p + w) - 0.5 * (w + w_m)) / (radii[k + 1] - radii[k]);
        const double dw_dr_m = (0.5 * (w + w_m) - 0.5 * (w_m + w_m2)) / (radii[k] - radii[k - 1]);
        const double Sigma = get_sigma(rmed);
        const double nu = get_nu2(rmed, M, Sigma);
        const double Sigma_m = get_sigma(rmed_m);
        const double nu_m = get_nu2(rmed_m, M, Sigma_m);
        const double a = nu * Sigma * std::pow(rmed, 3) * dw_dr;
        const double a_m = nu_m * Sigma_m * std::pow(rmed_m, 3) * dw_dr_m;
        const double num = 1.0 / rinf * (a - a_m) / (rmed - rmed_m);
        const double r2w = std::pow(rmed, 2) * get_w(rmed, M);
        const double r2w_m = std::pow(rmed_m, 2) * get_w(rmed_m, M);
        const double den = Sigma_m * ((r2w - r2w_m) / (rmed - rmed_m));
        return (num / den) / vr_numerical(rinf, M);
    };
    const double *Rinf = radii, *Rsup = radii + 1;
    // outer edge
    {
        const double safety = Rsup[nr - 1] - Rinf[nr - 1];
        double lo, hi;
        if (binary_on_primary) {
            lo = Rinf[nr - 1] * p.damping_outer_limit - com_max_dist - safety;
            hi = Rsup[nr - 1] + com_max_dist + safety;
        } else {
            lo = Rinf[nr - 1] * p.damping_outer_limit - safety;
            hi = Rsup[nr - 1] + safety;
        }
        lo = std::max(p.rmin, lo);
        min_r[1] = lo;
        dlog[1] = std::log10(hi / lo) / (double)n;
        for (int i = 0; i <= n; ++i) {
            const double r = lo * std::pow(10.0, (dlog[1] * (double)i));
            r_tab[(n + 1) + i] = r;
            vr_tab[(n + 1) + i] = vr_numerical(r, mass_all) * outer_correction(r, mass_all);
        }
    }
    // inner edge
    {
        const int lim = clamp_id(cell_id_p(p, nr, Rmed, p.rmin * p.damping_inner_limit, false),
                                 false, nr) + 1;
        const double safety = Rsup[lim] - Rinf[lim];
        double lo, hi;
        if (binary_on_primary) {
            lo = Rinf[1] - com_max_dist - safety;
            lo = std::max(lo, Rsup[0] - Rinf[0]);
            hi = Rsup[1] * p.damping_inner_limit + com_max_dist + safety;
        } else {
            lo = Rinf[1] - safety;
            hi = Rsup[1] * p.damping_inner_limit + safety;
        }
        min_r[0] = lo;
        dlog[0] = std::log10(hi / lo) / (double)n;
        for (int i = 0; i <= n; ++i) {
            const double r = lo * std::pow(10.0, (dlog[0] * (double)i));
            r_tab[i] = r;
            vr_tab[i] = vr_numerical(r, mass_center);
        }
    }
}

}  // namespace fgpu32
using fgpu32::boundary_values;

// Which hooks exist for which field (boundary_conditions/config.cpp:95-340).
static bool hook_allowed(int field, int kind, bool outer)
{
    switch (kind) {
    case FGPU_BC_NONE: case FGPU_BC_ZEROGRADIENT: case FGPU_BC_REFERENCE: return true;
    case FGPU_BC_DISKMODEL: return field == 0 || field == 1;
    case FGPU_BC_OUTFLOW: case FGPU_BC_REFLECTING: case FGPU_BC_KEPLERIAN_RADIAL:
        return field == 2;
    case FGPU_BC_VISCOUS: return field == 2 && !outer;
    case FGPU_BC_KEPLERIAN: case FGPU_BC_ZEROSHEAR: case FGPU_BC_BALANCED: return field == 3;
    default: return false;
    }
}

static int setup_tables(fgpu_engine *eng, const double *radii)
{
    const fgpu_params &p = eng->p;
    const int nr = eng->nr, nz = eng->nz;
    const int R = nr + 2;
    const double dphi = 2.0 * M_PI / (double)nz;      // Interpret.cpp:230
    const double invdphi = (double)nz / (2.0 * M_PI); // Interpret.cpp:231
    eng->geo = Geo{nr, nz, dphi, invdphi, split_pair_host(invdphi)};
    enum { RINF, RSUP, RMED, SURF, INVRMED, INVSURF, INVDIFFRMED, INVDIFFRSUP, INVDIFFRSUPRB,
           INVRINF, RINFSQ, TWOOVER, OMEGAK, INVOMEGAK, CSISO, INVDXSRC, INVDXTHETA, EMODEL,
           HFACADI, INVCELL, INVCELL2, TWOOVERRMEDSUM, LSQTW, TWOOVERDRMED2, DIFFRMED,
           RA3IDRMED, F43, CRPP1, CRPP2, CRRR1, CRRR2, CRRP, CRSCALE, NTAB };
    std::vector<double> h((size_t)NTAB * R, 0.0);
    auto T = [&](int k) { return h.data() + (size_t)k * R; };
    for (int n = 0; n <= nr; ++n) {
        T(RINF)[n] = radii[n];
        T(RSUP)[n] = radii[n + 1];
        double rm = 2.0 / 3.0 * (std::pow(T(RSUP)[n], 3) - std::pow(T(RINF)[n], 3));
        rm = rm / (std::pow(T(RSUP)[n], 2) - std::pow(T(RINF)[n], 2));
        T(RMED)[n] = rm;
        T(SURF)[n] = M_PI * (std::pow(T(RSUP)[n], 2) - std::pow(T(RINF)[n], 2)) / (double)nz;
        T(INVRMED)[n] = 1.0 / rm;
        T(INVSURF)[n] = 1.0 / T(SURF)[n];
        T(INVDIFFRSUP)[n] = 1.0 / (T(RSUP)[n] - T(RINF)[n]);
        T(INVDIFFRSUPRB)[n] = 1.0 / ((T(RSUP)[n] - T(RINF)[n]) * rm);
        T(INVRINF)[n] = 1.0 / T(RINF)[n];
        T(RINFSQ)[n] = std::pow(T(RINF)[n], 2);
        T(OMEGAK)[n] = omega_kepler(p, rm);
        T(INVOMEGAK)[n] = 1.0 / omega_kepler(p, rm);
        {   // compute_sound_speed_normal, isothermal branch (SourceEuler.cpp:983-990)
            const double vK = std::sqrt(p.G * p.hydro_center_mass / rm);
            const double hh = p.aspect_ratio * std::pow(rm, p.flaring_index);
            T(CSISO)[n] = hh * vK;
        }
        T(INVDXSRC)[n] = 2.0 / (dphi * (T(RSUP)[n] + T(RINF)[n]));
        T(INVDXTHETA)[n] = 1.0 / (dphi * rm);
        T(EMODEL)[n] = 1.0 / (p.gamma - 1.0) * std::pow(p.aspect_ratio, 2) *
                       std::pow(rm, 2.0 * p.flaring_index - 1.0) * p.G * p.hydro_center_mass;
        T(HFACADI)[n] = 1.0 / omega_kepler(p, rm) / std::sqrt(p.gamma);
        const double dxr = T(RSUP)[n] - T(RINF)[n], dxa = rm * dphi;
        const double cell = std::min(dxr, dxa);
        T(INVCELL)[n] = 1.0 / cell;
        T(INVCELL2)[n] = 1.0 / (cell * cell);
    }
    for (int n = 1; n <= nr; ++n) T(TWOOVERRMEDSUM)[n] = 2.0 / (T(RMED)[n] + T(RMED)[n - 1]);
    for (int n = 1; n <= nr; ++n) T(INVDIFFRMED)[n] = 1.0 / (T(RMED)[n] - T(RMED)[n - 1]);
    for (int n = 0; n < nr; ++n) {
        T(TWOOVER)[n] = 2.0 / (std::pow(T(RINF)[n + 1], 2) - std::pow(T(RINF)[n], 2));
    }
    for (int n = 0; n <= nr; ++n) {
        // Tscharnuter-Winkler length scale, artificial_viscosity.cpp:60-73
        if (n < nr) {
            const double Dr = T(RINF)[n + 1] - T(RINF)[n], rDphi = T(RMED)[n] * dphi;
            const double dx = nz <= 16 ? std::min(Dr, rDphi) : std::max(Dr, rDphi);
            T(LSQTW)[n] = std::pow(p.art_visc_factor, 2) * std::pow(dx, 2);
        }
        // StabilizeViscosity ring factors, viscosity.cpp:280-331 (Ra = Rinf)
        const double ra = T(RINF)[n];
        T(RA3IDRMED)[n] = std::pow(ra, 3) * T(INVDIFFRMED)[n];
        T(F43)[n] = 4.0 / 3.0 / T(RMED)[n] * invdphi * invdphi;
        T(CRRP)[n] = 1.0 / (dphi * dphi * ra);
        if (n >= 1) {
            T(TWOOVERDRMED2)[n] = 2.0 / (std::pow(T(RMED)[n], 2) - std::pow(T(RMED)[n - 1], 2));
            T(DIFFRMED)[n] = T(RMED)[n] - T(RMED)[n - 1];
            T(CRPP1)[n] = 2.0 * (0.5 * T(INVRMED)[n] + 1.0 / 3.0 * ra * T(INVDIFFRSUPRB)[n]);
            T(CRPP2)[n] = 2.0 * (0.5 * T(INVRMED)[n - 1] - 1.0 / 3.0 * ra * T(INVDIFFRSUPRB)[n - 1]);
            T(CRRR1)[n] = T(RMED)[n] * 2.0 *
                          (-T(INVDIFFRSUP)[n] + 1.0 / 3.0 * ra * T(INVDIFFRSUPRB)[n]);
            T(CRRR2)[n] = -1.0 * T(RMED)[n - 1] * 2.0 *
                          (T(INVDIFFRSUP)[n - 1] - 1.0 / 3.0 * ra * T(INVDIFFRSUPRB)[n - 1]);
            T(CRSCALE)[n] = p.radial_viscosity_factor / (0.5 * (T(RMED)[n] + T(RMED)[n - 1]));
        }
    }
    std::vector<double> cs(nz), sn(nz);
    for (int j = 0; j < nz; ++j) {
        cs[j] = std::cos(dphi * (double)j);  // SideEuler.cpp:56-61
        sn[j] = std::sin(dphi * (double)j);
    }
    const size_t bytes = sizeof(double) * ((size_t)NTAB * R + 2 * (size_t)nz);
    CK(cudaMalloc(&eng->tables_mem, bytes));
    CK(cudaMemcpy(eng->tables_mem, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    double *tc = eng->tables_mem + (size_t)NTAB * R;
    CK(cudaMemcpy(tc, cs.data(), sizeof(double) * nz, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(tc + nz, sn.data(), sizeof(double) * nz, cudaMemcpyHostToDevice));
    auto D = [&](int k) -> const double * { return eng->tables_mem + (size_t)k * R; };
    Tables &t = eng->tabs;
    t.Rinf = D(RINF); t.Rsup = D(RSUP); t.Rmed = D(RMED); t.Surf = D(SURF);
    t.InvRmed = D(INVRMED); t.InvSurf = D(INVSURF); t.InvDiffRmed = D(INVDIFFRMED);
    t.InvDiffRsup = D(INVDIFFRSUP); t.InvDiffRsupRb = D(INVDIFFRSUPRB); t.InvRinf = D(INVRINF);
    t.RinfSq = D(RINFSQ); t.TwoOverDRa2 = D(TWOOVER); t.OmegaK = D(OMEGAK);
    t.InvOmegaK = D(INVOMEGAK); t.CsIso = D(CSISO); t.InvDxSrc = D(INVDXSRC);
    t.InvDxTheta = D(INVDXTHETA); t.EModel = D(EMODEL); t.HFacAdi = D(HFACADI);
    t.InvCell = D(INVCELL); t.InvCell2 = D(INVCELL2); t.TwoOverRmedSum = D(TWOOVERRMEDSUM);
    t.LSqTW = D(LSQTW); t.TwoOverDRmed2 = D(TWOOVERDRMED2); t.DiffRmed = D(DIFFRMED);
    t.Ra3IDRmed = D(RA3IDRMED); t.F43 = D(F43); t.CrPp1 = D(CRPP1); t.CrPp2 = D(CRPP2);
    t.CrRr1 = D(CRRR1); t.CrRr2 = D(CRRR2); t.CrRp = D(CRRP); t.CrScale = D(CRSCALE);
    t.cosj = tc; t.sinj = tc + nz;
    {
        // Rmed, cos and sin, InvDiffRmed and InvSurf as float pairs hi + lo
        std::vector<float> pr((size_t)6 * R + (size_t)4 * nz);
        auto split = [](double v, float &h, float &l) {
            h = (float)v;
            l = (float)(v - (double)h);
        };
        for (int n = 0; n < R; ++n) split(T(RMED)[n], pr[(size_t)n], pr[(size_t)R + n]);
        float *c = pr.data() + 2 * (size_t)R;
        for (int j = 0; j < nz; ++j) {
            split(cs[j], c[j], c[(size_t)nz + j]);
            split(sn[j], c[2 * (size_t)nz + j], c[3 * (size_t)nz + j]);
        }
        float *e = c + 4 * (size_t)nz;
        for (int n = 0; n < R; ++n) {
            split(T(INVDIFFRMED)[n], e[(size_t)n], e[(size_t)R + n]);
            split(T(INVSURF)[n], e[2 * (size_t)R + n], e[3 * (size_t)R + n]);
        }
        // every per-ring table as float pairs, at the same index as its doubles
        pr.resize(pr.size() + (size_t)2 * NTAB * R);
        float *m = pr.data() + (pr.size() - (size_t)2 * NTAB * R);
        for (size_t k = 0; k < (size_t)NTAB * R; ++k) split(h[k], m[2 * k], m[2 * k + 1]);
        CK(cudaMalloc(&eng->pair_mem, sizeof(float) * pr.size()));
        CK(cudaMemcpy(eng->pair_mem, pr.data(), sizeof(float) * pr.size(), cudaMemcpyHostToDevice));
        const float *q = eng->pair_mem;
        t.RmedHi = q; t.RmedLo = q + R;
        t.cosHi = q + 2 * R; t.cosLo = t.cosHi + nz; t.sinHi = t.cosLo + nz; t.sinLo = t.sinHi + nz;
        t.InvDiffRmedHi = t.sinLo + nz; t.InvDiffRmedLo = t.InvDiffRmedHi + R;
        t.InvSurfHi = t.InvDiffRmedLo + R; t.InvSurfLo = t.InvSurfHi + R;
        t.tbase = eng->tables_mem;
        t.ptab = reinterpret_cast<const float2 *>(q + (pr.size() - (size_t)2 * NTAB * R));
    }

    // boundary hooks
    BcSpec &bc = eng->bc;
    bc.sigma_in = p.bc_sigma_inner; bc.sigma_out = p.bc_sigma_outer;
    bc.energy_in = p.bc_energy_inner; bc.energy_out = p.bc_energy_outer;
    bc.vr_in = p.bc_vrad_inner; bc.vr_out = p.bc_vrad_outer;
    bc.vaz_in = p.bc_vaz_inner; bc.vaz_out = p.bc_vaz_outer;
    boundary_values(p, T(RMED), T(RINF), nr, bc.val_in, bc.val_out);

    // damping (damping.cpp:311-752)
    std::vector<double> Rmed(T(RMED), T(RMED) + R);
    std::vector<double> fac((size_t)4 * (nr + 1), 0.0);  // inner S, outer S, inner V, outer V
    for (int vec = 0; vec < 2; ++vec) {
        const double *radius = vec ? T(RINF) : T(RMED);
        double *fi = fac.data() + (size_t)(vec ? 2 : 0) * (nr + 1);
        double *fo = fi + (nr + 1);
        for (int n = 0; n <= nr; ++n) {
            fi[n] = std::pow((radius[n] - p.rmin * p.damping_inner_limit) /
                                 (p.rmin - p.rmin * p.damping_inner_limit), 2);
            fo[n] = std::pow((radius[n] - p.rmax * p.damping_outer_limit) /
                                 (p.rmax - p.rmax * p.damping_outer_limit), 2);
        }
    }
    CK(cudaMalloc(&eng->damp_mem, sizeof(double) * fac.size()));
    CK(cudaMemcpy(eng->damp_mem, fac.data(), sizeof(double) * fac.size(), cudaMemcpyHostToDevice));
    const int dq_field[4] = {FGPU_V_RADIAL, FGPU_V_AZIMUTHAL, FGPU_SIGMA, FGPU_ENERGY};
    std::vector<char> ring_on(nr + 1, 0);
    for (int q = 0; q < 4; ++q) {
        DampQ &d = eng->dm.q[q];
        const bool vec = is_vector_field(dq_field[q]);
        const double *radius = vec ? T(RINF) : T(RMED);
        d.vector = vec;
        d.is_density = dq_field[q] == FGPU_SIGMA;
        d.kind_in = p.damping ? p.damping_inner[q] : 0;
        d.kind_out = p.damping ? p.damping_outer[q] : 0;
        d.active_in = (p.damping_inner_limit > 1.0) && (radius[0] < p.rmin * p.damping_inner_limit);
        d.limit_in = vec ? clamp_id(cell_id(eng, Rmed, p.rmin * p.damping_inner_limit, true), true, nr)
                         : clamp_id(cell_id(eng, Rmed, p.rmin * p.damping_inner_limit, false), false, nr);
        const int maxr = vec ? nr : nr - 1;
        d.active_out = (p.damping_outer_limit < 1.0) && (radius[maxr] > p.rmax * p.damping_outer_limit);
        d.limit_out = vec ? clamp_id(cell_id(eng, Rmed, p.rmax * p.damping_outer_limit, true) + 1, true, nr)
                          : clamp_id(cell_id(eng, Rmed, p.rmax * p.damping_outer_limit, false) + 1, false, nr);
        d.tau_in = p.damping_time_factor * 2.0 * M_PI / omega_kepler(p, p.rmin);
        d.tau_out = p.damping_time_factor * 2.0 * M_PI / omega_kepler(p, p.damping_time_radius_outer);
        d.x0_zero_in = d.is_density ? p.sigma_floor * p.sigma0 : 0.0;
        d.fac_in = eng->damp_mem + (size_t)(vec ? 2 : 0) * (nr + 1);
        d.fac_out = d.fac_in + (nr + 1);
        const int size = vec ? nr + 1 : nr;
        if (d.kind_in && d.active_in) for (int n = 0; n <= d.limit_in; ++n) ring_on[n] = 1;
        if (d.kind_out && d.active_out) for (int n = d.limit_out; n < size; ++n) ring_on[n] = 1;
    }
    std::vector<int> rings;
    for (int n = 0; n <= nr; ++n) if (ring_on[n]) rings.push_back(n);
    eng->n_damp_rings = (int)rings.size();
    if (!rings.empty()) {
        CK(cudaMalloc(&eng->damp_rings, sizeof(int) * rings.size()));
        CK(cudaMemcpy(eng->damp_rings, rings.data(), sizeof(int) * rings.size(), cudaMemcpyHostToDevice));
    }

    // centre-of-mass composite boundary: constants, half-cell trig tables and
    // the damping rings of center_of_mass.cpp:339-720
    eng->com_any = p.composite_inner == FGPU_COMPOSITE_CENTER_OF_MASS ||
                   p.composite_outer == FGPU_COMPOSITE_CENTER_OF_MASS;
    if (eng->com_any) {
        ComSpec &c = eng->com;
        c.active[0] = p.composite_inner == FGPU_COMPOSITE_CENTER_OF_MASS;
        c.active[1] = p.composite_outer == FGPU_COMPOSITE_CENTER_OF_MASS;
        c.pure_keplerian = p.initialize_pure_keplerian;
        c.vr_zero = p.initialize_vradial_zero;
        c.adiabatic = p.eos == FGPU_EOS_IDEAL;
        c.G = p.G; c.h0 = p.aspect_ratio; c.F = p.flaring_index; c.S = p.sigma_slope;
        c.eps = p.thickness_smoothing; c.Q = p.binary_quadrupole_moment;
        c.sigma0 = p.sigma0; c.gamma_m1 = p.gamma - 1.0;
        c.alpha = p.viscous_alpha; c.nu_const = p.constant_viscosity;
        c.sqrt_gamma = c.adiabatic ? std::sqrt(p.gamma) : 1.0;
        c.energy_floor = p.minimum_temperature * p.temperature_cgs_to_code / p.mu * p.R_gas /
                         (p.gamma - 1.0);
        c.n = kComTableNodes;
        const size_t N1 = (size_t)kComTableNodes + 1;
        // cos_h, sin_h, fac_vr[2], fac_az[2], r_tab[2], vr_tab[2]
        const size_t count = 2 * (size_t)nz + 4 * (size_t)(nr + 1) + 4 * N1;
        CK(cudaMalloc(&eng->com_mem, sizeof(double) * count));
        std::vector<double> hc(count, 0.0);
        double *ch = hc.data(), *sh = ch + nz;
        for (int j = 0; j < nz; ++j) {
            const double phi = ((double)j - 0.5) * dphi;  // center_of_mass.cpp:60
            ch[j] = std::cos(phi);
            sh[j] = std::sin(phi);
        }
        double *fv[2] = {sh + nz, sh + nz + (nr + 1)};
        double *fa[2] = {sh + nz + 2 * (nr + 1), sh + nz + 3 * (nr + 1)};
        const double rin = p.rmin * p.damping_inner_limit, rout = p.rmax * p.damping_outer_limit;
        for (int n = 0; n <= nr; ++n) {
            fv[0][n] = std::pow((T(RINF)[n] - rin) / (p.rmin - rin), 2);
            fv[1][n] = std::pow((T(RINF)[n] - rout) / (p.rmax - rout), 2);
            // the inner v_phi and energy damping use the outer zone's profile
            // (center_of_mass.cpp:628-631, 689-692)
            fa[0][n] = std::pow((T(RMED)[n] - rout) / (p.rmax - rout), 2);
            fa[1][n] = fa[0][n];
        }
        CK(cudaMemcpy(eng->com_mem, hc.data(), sizeof(double) * count, cudaMemcpyHostToDevice));
        double *dm = eng->com_mem;
        c.cos_h = dm; c.sin_h = dm + nz;
        c.Rinf = eng->tabs.Rinf; c.Rsup = eng->tabs.Rsup; c.Rmed = eng->tabs.Rmed;
        c.cos_j = eng->tabs.cosj; c.sin_j = eng->tabs.sinj;
        for (int k = 0; k < 2; ++k) {
            c.fac_vr[k] = dm + 2 * nz + k * (nr + 1);
            c.fac_az[k] = dm + 2 * nz + (2 + k) * (nr + 1);
            c.r_tab[k] = dm + 2 * nz + 4 * (nr + 1) + k * N1;
            c.vr_tab[k] = dm + 2 * nz + 4 * (nr + 1) + (2 + k) * N1;
        }
        // inner: damping_diskmodel_center_of_mass_inner (center_of_mass.cpp:552-720)
        const bool din = p.damping && c.active[0] && p.damping_inner_limit > 1.0 &&
                         T(RMED)[0] < rin;
        c.vr_lo[0] = 2;  // One_no_ghost_vr
        c.vr_hi[0] = din ? clamp_id(cell_id(eng, Rmed, rin, true), true, nr) + 1 : 0;
        c.az_lo[0] = 1;  // Zero_no_ghost
        c.az_hi[0] = din ? clamp_id(cell_id(eng, Rmed, rin, false), false, nr) + 1 : 0;
        c.tau[0] = p.damping_time_factor * 2.0 * M_PI / omega_kepler(p, p.rmin);
        // outer: damping_diskmodel_center_of_mass_outer (:339-549)
        const bool dout = p.damping && c.active[1] && p.damping_outer_limit < 1.0 &&
                          T(RINF)[nr] > rout;
        c.vr_lo[1] = clamp_id(cell_id(eng, Rmed, rout, true), true, nr) + 1;
        c.vr_hi[1] = dout ? nr - 1 : 0;  // MaxMo_no_ghost_vr
        c.az_lo[1] = clamp_id(cell_id(eng, Rmed, rout, false), false, nr) + 1;
        c.az_hi[1] = dout ? nr - 1 : 0;  // Max_no_ghost
        c.tau[1] = p.damping_time_factor * 2.0 * M_PI / omega_kepler(p, p.damping_time_radius_outer);
    }

    // physics constants
    Phys &ph = eng->ph;
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
    ph.gamma = p.gamma;
    ph.gm1 = p.gamma - 1.0;
    ph.g_gm1 = p.gamma * (p.gamma - 1.0);
    ph.sqrt_gamma = std::sqrt(p.gamma);
    ph.mu = p.mu;
    ph.alpha = p.viscous_alpha;
    ph.constant_viscosity = p.constant_viscosity;
    ph.C2 = std::pow(p.art_visc_factor, 2);
    ph.four_C2 = 4.0 * std::pow(p.art_visc_factor, 2);
    ph.rvf = p.radial_viscosity_factor;
    ph.hvf = p.heating_viscous_factor;
    ph.cfl = p.cfl;
    ph.leapfrog = p.integrator == FGPU_INTEGRATOR_LEAPFROG;
    ph.inv_hc_limit = 1.0 / p.heating_cooling_cfl_limit;
    ph.sigma_min = p.sigma_floor * p.sigma0;
    ph.sigma_floor10 = 10.0 * p.sigma0 * p.sigma_floor;
    ph.eps_smooth = p.thickness_smoothing;
    ph.correct_sg = p.correct_disk_selfgravity != 0;
    ph.tmin = p.minimum_temperature;
    ph.tmax = p.maximum_temperature;
    ph.Rgas = p.R_gas;
    ph.sigma_sb = p.sigma_sb;
    ph.c_light = p.c_light;
    ph.G = p.G;
    ph.Mc = p.hydro_center_mass;
    ph.c_v_inv = p.mu / p.R_gas * (p.gamma - 1.0);
    ph.cool_const = 2.0 * 4.0 * p.sigma_sb / p.c_light;
    ph.mu_gm1_over_R = p.mu * (p.gamma - 1.0) / p.R_gas;
    ph.emin_fac = p.minimum_temperature / p.mu * p.R_gas / (p.gamma - 1.0);
    ph.emax_fac = p.maximum_temperature / p.mu * p.R_gas / (p.gamma - 1.0);
    ph.emin_fac_f = (float)ph.emin_fac;
    ph.emax_fac_f = (float)ph.emax_fac;  // may round to infinity: the screen then has no upper bound
    ph.pk_gm1 = split_pair_host(ph.gm1);
    ph.pk_g_gm1 = split_pair_host(ph.g_gm1);
    ph.pk_alpha = split_pair_host(ph.alpha);
    ph.pk_C2 = split_pair_host(ph.C2);
    ph.pk_rvf = split_pair_host(ph.rvf);
    ph.pk_hvf = split_pair_host(ph.hvf);
    ph.pk_mu_gm1_over_R = split_pair_host(ph.mu_gm1_over_R);
    ph.pk_cool_const = split_pair_host(ph.cool_const);
    ph.pk_emin_fac = split_pair_host(ph.emin_fac);
    ph.pk_eps_smooth = split_pair_host(ph.eps_smooth);
    return FGPU_OK;
}

// Creates an engine on the given stream (owned by the caller), or on a new
// stream of its own when shared is null.
static int create_engine(const fgpu_params *params, const double *radii, cudaStream_t shared,
                         fgpu_engine **out)
{
    if (!params || !radii || !out) return FGPU_ERR_BAD_ARG;
    *out = nullptr;
    std::string why;
    int rc = validate(params, why);
    if (rc != FGPU_OK) {
        fprintf(stderr, "fgpu_create: %s\n", why.c_str());
        return rc;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FGPU_ERR_NO_DEVICE;
    }
    fgpu_engine *eng = new (std::nothrow) fgpu_engine();
    if (!eng) return FGPU_ERR_OOM;
    eng->p = *params;
    eng->nr = params->nrad;
    eng->nz = params->naz;
    eng->cells = (size_t)eng->nr * eng->nz;
    eng->vcells = (size_t)(eng->nr + 1) * eng->nz;
    eng->host_radii.assign(radii, radii + eng->nr + 2);
    auto fail = [&](int code) {
        fprintf(stderr, "fgpu_create: %s\n", eng->err.c_str());
        fgpu_destroy(eng);
        return code;
    };
    if (shared) {
        eng->stream = shared;
        eng->owns_stream = false;
    } else if (cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking) != cudaSuccess) {
        eng->err = "stream";
        return fail(FGPU_ERR_CUDA);
    }
    if (params->precision == FGPU_PRECISION_FP32_MIXED) {
        rc = setup_tables(eng, radii);
        if (rc != FGPU_OK) return fail(rc);
        eng->e32 = new (std::nothrow) fgpu32::Engine32();
        if (!eng->e32) return fail(FGPU_ERR_OOM);
        for (int q = 0; q < 4; ++q) {
            const DampQ &d = eng->dm.q[q];
            fgpu32::DampQSpec &sp = eng->e32->damp_spec[q];
            sp.kind_in = d.kind_in; sp.kind_out = d.kind_out;
            sp.active_in = d.active_in; sp.active_out = d.active_out;
            sp.limit_in = d.limit_in; sp.limit_out = d.limit_out;
            sp.tau_in = d.tau_in; sp.tau_out = d.tau_out;
        }
        eng->e32->mark_fn = [](void *ctx, int k) { mark((fgpu_engine *)ctx, k); };
        eng->e32->mark_ctx = eng;
        rc = eng->e32->create(*params, radii, eng->stream);
        if (rc != FGPU_OK) {
            eng->err = eng->e32->err;
            return fail(rc);
        }
        *out = eng;
        return FGPU_OK;
    }
    int rc2 = FGPU_OK;
    (void)rc2;
    for (int f = 0; f < FGPU_FIELD_COUNT; ++f) {
        const size_t n = (size_t)field_rows(eng, f) * eng->nz;
        if (cudaMalloc(&eng->field[f], n * sizeof(double)) != cudaSuccess) {
            eng->err = "out of device memory (fields)";
            return fail(FGPU_ERR_OOM);
        }
        cudaMemset(eng->field[f], 0, n * sizeof(double));
    }
    double **alts[4] = {&eng->sigma_alt, &eng->vr_alt, &eng->vaz_alt, &eng->energy_alt};
    for (int k = 0; k < 4; ++k) {
        const size_t n = k == 1 ? eng->vcells : eng->cells;
        if (cudaMalloc(alts[k], n * sizeof(double)) != cudaSuccess) {
            eng->err = "out of device memory (state)";
            return fail(FGPU_ERR_OOM);
        }
        cudaMemset(*alts[k], 0, n * sizeof(double));
    }
    if (params->stabilize_viscosity) {
        if (cudaMalloc(&eng->corr_phi, eng->cells * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&eng->corr_r, eng->cells * sizeof(double)) != cudaSuccess) {
            eng->err = "out of device memory (viscosity correction factors)";
            return fail(FGPU_ERR_OOM);
        }
        cudaMemset(eng->corr_phi, 0, eng->cells * sizeof(double));
        cudaMemset(eng->corr_r, 0, eng->cells * sizeof(double));
    }
    for (int k = 0; k < 4; ++k) {
        if (cudaMalloc(&eng->mom[k], eng->cells * sizeof(double)) != cudaSuccess) {
            eng->err = "out of device memory (momenta)";
            return fail(FGPU_ERR_OOM);
        }
    }
    if (cudaMalloc(&eng->partial, sizeof(double) * 5 * kForceBodies * (size_t)eng->nr) !=
            cudaSuccess ||
        cudaMalloc(&eng->red_out, sizeof(double) * (8 + 5 * kMaxBodies)) != cudaSuccess ||
        cudaMalloc(&eng->d_dtmin, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&eng->d_bad, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost(&eng->h_pinned, sizeof(double) * (16 + 5 * kMaxBodies)) != cudaSuccess) {
        eng->err = "out of memory (reductions)";
        return fail(FGPU_ERR_OOM);
    }
    rc = setup_tables(eng, radii);
    if (rc != FGPU_OK) return fail(rc);

    // the kernels' arithmetic: float pairs unless FARGO_GB300_FP64_ARITH
    // asks for "fp64" ("pair" or unset: pairs)
    {
        const char *env = getenv("FARGO_GB300_FP64_ARITH");
        const std::string want = env ? env : "pair";
        if (want == "fp64") {
            eng->pair_arith = false;
        } else if (want != "pair") {
            eng->err = "FARGO_GB300_FP64_ARITH=" + want + " is neither pair nor fp64";
            return fail(FGPU_ERR_BAD_ARG);
        }
    }
    // rings per radial sweep chunk (radial_chunk_for): longer chunks prime
    // fewer rings, shorter ones give more blocks; 16 below 8M cells
    // (measured, ms per radial pass on 512x1536: 0.064 with 16, 0.068 with
    // 8, 0.098 with 32), else the chunk whose grid fills the fewest waves of
    // resident blocks (2048x6144 in float pairs: 0.707 ms with 32 rings, six
    // waves; 0.694 with 33 and 0.683 with 34, five)
    eng->radial_chunk = radial_chunk_for(eng->pair_arith, eng->ph.adiabatic, eng->nr, eng->nz);
    // azimuthal transport: whole ring in shared memory when it fits
    {
        const int per = azimuthal_cells_per_thread(eng->nz);
        eng->az_block = std::max(128, std::min(512, ((eng->nz + per - 1) / per + 31) / 32 * 32));
    }
    if (cudaMalloc(&eng->ring_shift, sizeof(int) * (size_t)eng->nr) != cudaSuccess ||
        cudaMemsetAsync(eng->ring_shift, 0, sizeof(int) * (size_t)eng->nr, eng->stream) !=
            cudaSuccess) {
        eng->err = "out of device memory (ring shifts)";
        return fail(FGPU_ERR_OOM);
    }
    eng->az_smem = azimuthal_smem_bytes(eng->nz);
    if (eng->az_smem > 220 * 1024) {
        if (cudaMalloc(&eng->ring_ws, eng->az_smem * (size_t)eng->nr) != cudaSuccess) {
            eng->err = "out of device memory (ring workspace)";
            return fail(FGPU_ERR_OOM);
        }
    } else {
        // the kernel also has static shared memory: opt in for the dynamic size
        // whatever it is
        if (prepare_azimuthal(eng->az_smem) != cudaSuccess) {
            eng->err = "cannot reserve shared memory for the azimuthal kernel";
            return fail(FGPU_ERR_CUDA);
        }
    }
    if (cudaStreamSynchronize(eng->stream) != cudaSuccess) {
        eng->err = cudaGetErrorString(cudaGetLastError());
        return fail(FGPU_ERR_CUDA);
    }
    *out = eng;
    return FGPU_OK;
}

extern "C" int fgpu_destroy(fgpu_engine *eng)
{
    if (!eng || eng->batch_owned) return FGPU_ERR_BAD_ARG;
    if (eng->stream) cudaStreamSynchronize(eng->stream);
    if (eng->e32) {
        eng->e32->destroy();
        delete eng->e32;
    }
    for (auto &row : eng->ev_rows)
        for (auto ev : row) cudaEventDestroy(ev);
    for (auto ev : eng->ev_free) cudaEventDestroy(ev);
    for (int f = 0; f < FGPU_FIELD_COUNT; ++f) cudaFree(eng->field[f]);
    cudaFree(eng->sigma_alt); cudaFree(eng->vr_alt); cudaFree(eng->vaz_alt); cudaFree(eng->energy_alt);
    for (int k = 0; k < 4; ++k) cudaFree(eng->mom[k]);
    cudaFree(eng->ring_ws); cudaFree(eng->ring_shift); cudaFree(eng->tables_mem);
    cudaFree(eng->damp_mem);
    cudaFree(eng->damp_rings); cudaFree(eng->partial); cudaFree(eng->red_out);
    cudaFree(eng->pair_mem);
    cudaFree(eng->com_mem);
    cudaFree(eng->d_dtmin); cudaFree(eng->d_bad);
    cudaFree(eng->corr_phi); cudaFree(eng->corr_r);
    if (eng->h_pinned) cudaFreeHost(eng->h_pinned);
    if (eng->copy_stream) {
        cudaStreamSynchronize(eng->copy_stream);
        cudaStreamDestroy(eng->copy_stream);
    }
    if (eng->snap_staged) cudaEventDestroy(eng->snap_staged);
    if (eng->snap_copied) cudaEventDestroy(eng->snap_copied);
    cudaFree(eng->snap_stage);
    if (eng->stream && eng->owns_stream) cudaStreamDestroy(eng->stream);
    delete eng;
    return FGPU_OK;
}

extern "C" int fgpu_create(const fgpu_params *params, const double *radii, fgpu_engine **out)
{
    return create_engine(params, radii, nullptr, out);
}

namespace fgpu32 {
// FP32-mixed disks of a batch: created on the batch's stream
int create_disk(const fgpu_params *params, const double *radii, cudaStream_t stream,
                fgpu_engine **out)
{
    if (!params || params->precision != FGPU_PRECISION_FP32_MIXED) return FGPU_ERR_UNSUPPORTED;
    const int rc = create_engine(params, radii, stream, out);
    if (rc == FGPU_OK) (*out)->batch_owned = true;
    return rc;
}
int destroy_disk(fgpu_engine *eng)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    eng->batch_owned = false;
    return fgpu_destroy(eng);
}
Engine32 *engine32_of(fgpu_engine *eng) { return eng ? eng->e32 : nullptr; }
}  // namespace fgpu32

static Launch launch_of(const fgpu_engine *eng)
{
    Launch L;
    L.g = eng->geo;
    L.t = eng->tabs;
    L.ph = eng->ph;
    L.stream = eng->stream;
    L.bx = 128;
    L.pair = eng->pair_arith;
    return L;
}

static State state_of(fgpu_engine *eng)
{
    State s;
    double **f = eng->field;
    s.sigma = f[FGPU_SIGMA]; s.vr = f[FGPU_V_RADIAL]; s.vaz = f[FGPU_V_AZIMUTHAL];
    s.energy = f[FGPU_ENERGY]; s.sigma0 = f[FGPU_SIGMA0]; s.vr0 = f[FGPU_V_RADIAL0];
    s.vaz0 = f[FGPU_V_AZIMUTHAL0]; s.energy0 = f[FGPU_ENERGY0]; s.cs = f[FGPU_SOUNDSPEED];
    s.H = f[FGPU_SCALE_HEIGHT]; s.P = f[FGPU_PRESSURE]; s.T = f[FGPU_TEMPERATURE];
    s.nu = f[FGPU_VISCOSITY]; s.qplus = f[FGPU_QPLUS]; s.qminus = f[FGPU_QMINUS];
    s.pot = f[FGPU_POTENTIAL]; s.divv = f[FGPU_DIV_V]; s.trr = f[FGPU_TAU_R_R];
    s.tpp = f[FGPU_TAU_PHI_PHI]; s.trp = f[FGPU_TAU_R_PHI]; s.qr = f[FGPU_Q_R];
    s.qphi = f[FGPU_Q_PHI];
    s.corr_phi = eng->corr_phi; s.corr_r = eng->corr_r;
    return s;
}

static int check_launch(fgpu_engine *eng)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        eng->err = std::string("kernel launch: ") + cudaGetErrorString(e);
        return FGPU_ERR_CUDA;
    }
    return FGPU_OK;
}

extern "C" int fgpu_upload_field(fgpu_engine *eng, int field, const double *host, int rows, int cols)
{
    if (!eng || !host || field < 0 || field >= FGPU_FIELD_COUNT) return FGPU_ERR_BAD_ARG;
    if (rows != field_rows(eng, field) || cols != eng->nz) {
        eng->err = "upload_field: shape mismatch";
        return FGPU_ERR_BAD_ARG;
    }
    if (eng->e32) {
        int rc = eng->e32->upload(field, host, rows);
        if (rc) eng->err = eng->e32->err;
        return rc;
    }
    if (is_pair_field(field)) {
        const int rc = join_pair_fields(eng);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(eng->field[field], host, sizeof(double) * (size_t)rows * cols,
                       cudaMemcpyHostToDevice, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    eng->cfl_valid = false;
    return FGPU_OK;
}

extern "C" int fgpu_download_field(fgpu_engine *eng, int field, double *host, int rows, int cols)
{
    if (!eng || !host || field < 0 || field >= FGPU_FIELD_COUNT) return FGPU_ERR_BAD_ARG;
    if (rows != field_rows(eng, field) || cols != eng->nz) {
        eng->err = "download_field: shape mismatch";
        return FGPU_ERR_BAD_ARG;
    }
    if (eng->e32) {
        int rc = eng->e32->download(field, host, rows);
        if (rc) eng->err = eng->e32->err;
        return rc;
    }
    if (is_pair_field(field)) {
        const int rc = join_pair_fields(eng);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(host, eng->field[field], sizeof(double) * (size_t)rows * cols,
                       cudaMemcpyDeviceToHost, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    return FGPU_OK;
}

extern "C" int fgpu_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr || bytes == 0) return FGPU_ERR_BAD_ARG;
    *ptr = nullptr;
    if (cudaMallocHost(ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return FGPU_ERR_OOM;
    }
    return FGPU_OK;
}

extern "C" int fgpu_host_free(void *ptr)
{
    if (!ptr) return FGPU_ERR_BAD_ARG;
    return cudaFreeHost(ptr) == cudaSuccess ? FGPU_OK : FGPU_ERR_CUDA;
}

extern "C" int fgpu_snapshot_wait(fgpu_engine *eng)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    if (!eng->snap_pending) return FGPU_OK;
    eng->snap_pending = false;
    CK(cudaEventSynchronize(eng->snap_copied));
    return FGPU_OK;
}

extern "C" int fgpu_snapshot_begin(fgpu_engine *eng, int n, const int *fields,
                                   double *const *host)
{
    NvtxCall nvtx_("fgpu_snapshot_begin");
    if (!eng || n < 1 || n > FGPU_FIELD_COUNT || !fields || !host) return FGPU_ERR_BAD_ARG;
    for (int k = 0; k < n; ++k) {
        if (fields[k] < 0 || fields[k] >= FGPU_FIELD_COUNT || !host[k]) return FGPU_ERR_BAD_ARG;
    }
    int rc = fgpu_snapshot_wait(eng);  // one snapshot in flight at a time
    if (rc) return rc;
    if (!eng->copy_stream) {
        CK(cudaStreamCreateWithFlags(&eng->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&eng->snap_staged, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&eng->snap_copied, cudaEventDisableTiming));
    }
    const size_t need = (size_t)n * eng->vcells;
    if (need > eng->snap_capacity) {
        cudaFree(eng->snap_stage);
        eng->snap_stage = nullptr;
        eng->snap_capacity = 0;
        if (cudaMalloc(&eng->snap_stage, need * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            eng->err = "snapshot: out of device memory for the staging buffers";
            return FGPU_ERR_OOM;
        }
        eng->snap_capacity = need;
    }
    for (int k = 0; k < n && !eng->e32; ++k) {
        if (is_pair_field(fields[k])) {
            rc = join_pair_fields(eng);
            if (rc) return rc;
            break;
        }
    }
    // the staging copies are ordered with the steps on the engine's stream
    for (int k = 0; k < n; ++k) {
        const int rows = field_rows(eng, fields[k]);
        double *dst = eng->snap_stage + (size_t)k * eng->vcells;
        if (eng->e32) {
            rc = eng->e32->to_fp64(fields[k], dst, rows);
            if (rc) {
                eng->err = eng->e32->err;
                return rc;
            }
        } else {
            CK(cudaMemcpyAsync(dst, eng->field[fields[k]], sizeof(double) * rows * eng->nz,
                               cudaMemcpyDeviceToDevice, eng->stream));
        }
    }
    CK(cudaEventRecord(eng->snap_staged, eng->stream));
    // the copies to the host drain on the copy stream while the steps go on
    CK(cudaStreamWaitEvent(eng->copy_stream, eng->snap_staged, 0));
    for (int k = 0; k < n; ++k) {
        const int rows = field_rows(eng, fields[k]);
        CK(cudaMemcpyAsync(host[k], eng->snap_stage + (size_t)k * eng->vcells,
                           sizeof(double) * rows * eng->nz, cudaMemcpyDeviceToHost,
                           eng->copy_stream));
    }
    CK(cudaEventRecord(eng->snap_copied, eng->copy_stream));
    eng->snap_pending = true;
    return FGPU_OK;
}

extern "C" int fgpu_set_bodies(fgpu_engine *eng, int n, const fgpu_body *bodies, double ix,
                               double iy, double omega_frame)
{
    if (!eng || n < 0 || n > kMaxBodies || (n > 0 && !bodies)) return FGPU_ERR_BAD_ARG;
    Bodies &b = eng->bodies;
    b.n = n;
    for (int k = 0; k < n; ++k) {
        b.x[k] = bodies[k].x;
        b.y[k] = bodies[k].y;
        b.m[k] = bodies[k].mass;
        b.rsm[k] = bodies[k].r_sm;
        b.a[k] = bodies[k].a;
    }
    b.ix = ix;
    b.iy = iy;
    b.pk_ix = split_pair_host(ix);
    b.pk_iy = split_pair_host(iy);
    b.omega_frame = omega_frame;
    auto split = [](double v, float &h, float &l) {
        h = (float)v;
        l = (float)(v - (double)h);
    };
    b.klahr = 0;
    for (int k = 0; k < n; ++k) {
        split(b.x[k], b.xh[k], b.xl[k]);
        split(b.y[k], b.yh[k], b.yl[k]);
        split(-eng->p.G * b.m[k], b.gmh[k], b.gml[k]);
        if (b.rsm[k] > 0.0) b.klahr |= 1u << k;
    }
    b.star_plain = n > 0 && b.x[0] == 0.0 && b.y[0] == 0.0 && !(b.rsm[0] > 0.0);
    b.gm0 = n > 0 ? -eng->p.G * b.m[0] : 0.0;
    if (eng->e32) {
        if (omega_frame != 0.0 && eng->batch_owned) {
            eng->err = "the batched form runs in the fixed (non-rotating) frame";
            return FGPU_ERR_UNSUPPORTED;
        }
        eng->e32->set_bodies(n, bodies, ix, iy, omega_frame);
    }
    return FGPU_OK;
}

static double beta_inv_at(const fgpu_params &p, double t)
{
    // thermal_relaxation, SourceEuler.cpp:645-653
    double beta_inv = 1 / p.cooling_beta_value;
    if (p.cooling_beta_ramp_up > 0.0) {
        const double ramp = 1 - std::exp(-std::pow(2 * t / p.cooling_beta_ramp_up, 2));
        beta_inv = beta_inv * ramp;
    }
    return beta_inv;
}

#define ROUTE32(expr)                           \
    if (eng->e32) {                             \
        int rc_ = (expr);                       \
        if (rc_) eng->err = eng->e32->err;      \
        return rc_;                             \
    }

extern "C" int fgpu_init_euler(fgpu_engine *eng, double t)
{
    NvtxCall nvtx_("fgpu_init_euler");
    if (!eng) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->init_euler(t));
    Launch L = launch_of(eng);
    State s = state_of(eng);
    launch_derived_cfl(L, 1 | 2, s, nullptr);
    if (eng->ph.adiabatic) {
        // compute_heating_cooling_for_CFL, SourceEuler.cpp:1410-1450
        launch_stress(L, s.sigma, s.vr, s.vaz, s.nu, s.divv, s.trr, s.tpp, s.trp);
        eng->stress_pairs = stress_as_pairs(L);
        if (eng->ph.stabilize) launch_visc_corr(L, s);
        launch_viscous(L, 0.0, beta_inv_at(eng->p, t), 2, s);
    }
    eng->cfl_valid = false;
    return check_launch(eng);
}

extern "C" int fgpu_recalculate_derived(fgpu_engine *eng, double t)
{
    NvtxCall nvtx_("fgpu_recalculate_derived");
    (void)t;
    if (!eng) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->derived_cfl(1));
    Launch L = launch_of(eng);
    launch_derived_cfl(L, 1, state_of(eng), nullptr);
    eng->cfl_valid = false;
    return check_launch(eng);
}

extern "C" int fgpu_condition_cfl(fgpu_engine *eng, double *dt_out)
{
    NvtxCall nvtx_("fgpu_condition_cfl");
    if (!eng || !dt_out) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->cfl(dt_out));
    if (!eng->cfl_valid) {
        CK(cudaMemsetAsync(eng->d_dtmin, 0x7f, sizeof(unsigned long long), eng->stream));
        launch_derived_cfl(launch_of(eng), 4, state_of(eng), eng->d_dtmin);
        int rc = check_launch(eng);
        if (rc) return rc;
        eng->cfl_valid = true;
    }
    CK(cudaMemcpyAsync(eng->h_pinned, eng->d_dtmin, sizeof(double), cudaMemcpyDeviceToHost,
                       eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    *dt_out = eng->h_pinned[0];
    return FGPU_OK;
}

// parameters::VISCOUS_ACCRETION (Interpret.cpp:704-707): with the viscous
// v_radial hook or viscous accretion, c_s, H and nu of the transported state
// before the final boundary call (simulation.cpp:232-242, 432-441); only the
// ideal EOS changes them.
static void viscous_recompute(fgpu_engine *eng, const Launch &L)
{
    const fgpu_params &p = eng->p;
    if (eng->ph.adiabatic && (p.viscous_accretion || p.bc_vrad_inner == FGPU_BC_VISCOUS)) {
        launch_derived_cfl(L, 1, state_of(eng), nullptr);
    }
}

static void ghost(fgpu_engine *eng, const Launch &L)
{
    launch_ghost(L, eng->bc, eng->bodies.omega_frame, state_of(eng));
}

// The centre-of-mass composite: its damping runs after the regular damping
// in the final boundary call, its ghost rings after the per-field hooks
// (boundary_conditions.cpp:46-110).
static ComSpec com_spec(const fgpu_engine *eng, const ComCenter *c)
{
    ComSpec cs = eng->com;
    cs.c[0] = c[0];
    cs.c[1] = c[1];
    cs.omf = eng->bodies.omega_frame;
    return cs;
}

static void com_boundary(fgpu_engine *eng, const Launch &L, const ComCenter *c)
{
    if (eng->com_any) launch_com_boundary(L, com_spec(eng, c), state_of(eng));
}

static void com_damping(fgpu_engine *eng, const Launch &L, double dt, const ComCenter *c)
{
    if (eng->com_any && eng->p.damping) launch_com_damping(L, com_spec(eng, c), dt, state_of(eng));
}

static int com_unready(fgpu_engine *eng)
{
    if (eng->com_any && !eng->com_ready) {
        eng->err = "a centerofmass composite boundary needs fgpu_init_center_of_mass_boundary first";
        return FGPU_ERR_BAD_ARG;
    }
    return FGPU_OK;
}

extern "C" int fgpu_init_center_of_mass_boundary(fgpu_engine *eng, double mass_all,
                                                 double mass_center, int binary_on_primary,
                                                 double com_max_dist)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    if (!eng->com_any) {
        eng->err = "no composite boundary is centerofmass";
        return FGPU_ERR_BAD_ARG;
    }
    if (!(mass_all > 0.0) || !(mass_center > 0.0) || !(com_max_dist >= 0.0)) {
        eng->err = "masses must be > 0 and com_max_dist >= 0";
        return FGPU_ERR_BAD_ARG;
    }
    const int nr = eng->nr, n = kComTableNodes;
    const double *radii = eng->host_radii.data();
    std::vector<double> Rmed(nr + 2, 0.0);
    for (int k = 0; k <= nr; ++k) {
        double rm = 2.0 / 3.0 * (std::pow(radii[k + 1], 3) - std::pow(radii[k], 3));
        Rmed[k] = rm / (std::pow(radii[k + 1], 2) - std::pow(radii[k], 2));
    }
    std::vector<double> tabs(4 * (size_t)(n + 1));
    double *rt = tabs.data(), *vt = rt + 2 * (n + 1);
    ComSpec &c = eng->com;
    fgpu32::viscous_speed_tables(eng->p, radii, Rmed.data(), nr, mass_all, mass_center,
                                 binary_on_primary != 0, com_max_dist, n, c.min_r, c.dlog, rt,
                                 vt);
    for (int k = 0; k < 2; ++k) {
        if (!std::isfinite(c.min_r[k]) || !std::isfinite(c.dlog[k]) || !(c.dlog[k] > 0.0)) {
            eng->err = "viscous-speed table range is empty";
            return FGPU_ERR_BAD_ARG;
        }
    }
    // the four tables lie back to back in com_mem: r_tab[0], r_tab[1], vr_tab[0], vr_tab[1]
    CK(cudaMemcpyAsync(const_cast<double *>(c.r_tab[0]), tabs.data(), sizeof(double) * tabs.size(),
                       cudaMemcpyHostToDevice, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    eng->com_ready = true;
    if (eng->e32) {
        eng->e32->com = eng->com;
        eng->e32->com_any = true;
    }
    return FGPU_OK;
}

extern "C" int fgpu_cfl_limiting_cell(fgpu_engine *eng, fgpu_cfl_cell *out)
{
    if (!eng || !out) return FGPU_ERR_BAD_ARG;
    if (eng->e32) {
        eng->err = "the CFL report is a diagnostic of the FP64 form";
        return FGPU_ERR_UNSUPPORTED;
    }
    double dt = 0.0;
    if (int rc = fgpu_condition_cfl(eng, &dt)) return rc;  // derived quantities current
    NvtxCall nvtx_("fgpu_cfl_limiting_cell");
    const int rows = eng->nr - 1;
    double *d = nullptr;
    CK(cudaMalloc(&d, sizeof(double) * 10 * (size_t)rows));
    launch_cfl_cells(launch_of(eng), state_of(eng), d);
    std::vector<double> h(10 * (size_t)rows);
    const cudaError_t e1 = cudaMemcpyAsync(h.data(), d, sizeof(double) * h.size(),
                                           cudaMemcpyDeviceToHost, eng->stream);
    const cudaError_t e2 = cudaStreamSynchronize(eng->stream);
    cudaFree(d);
    CK(e1);
    CK(e2);
    *out = fgpu_cfl_cell{};
    out->ring = out->azimuth = out->shear_ring = -1;
    out->dt_cell = out->dt_shear = 1.0e300;
    for (int i = 0; i < rows; ++i) {
        const double *o = h.data() + (size_t)10 * i;
        if (o[1] >= 0.0 && o[0] < out->dt_cell) {
            out->dt_cell = o[0];
            out->ring = i;
            out->azimuth = (int)o[1];
            for (int k = 0; k < 6; ++k) out->invdt[k] = o[3 + k];
        }
        if (o[2] < out->dt_shear) {
            out->dt_shear = o[2];
            out->shear_ring = i;
        }
    }
    return FGPU_OK;
}

extern "C" int fgpu_correct_v_azimuthal(fgpu_engine *eng, double domega)
{
    if (!eng || !std::isfinite(domega)) return FGPU_ERR_BAD_ARG;
    if (domega == 0.0) return FGPU_OK;
    if (eng->e32) {
        if (eng->batch_owned) {
            eng->err = "the batched form runs in the fixed (non-rotating) frame";
            return FGPU_ERR_UNSUPPORTED;
        }
        eng->e32->correct_v_azimuthal(domega);
        return FGPU_OK;
    }
    NvtxCall nvtx_("fgpu_correct_v_azimuthal");
    launch_correct_vaz(launch_of(eng), domega, eng->field[FGPU_V_AZIMUTHAL]);
    eng->cfl_valid = false;
    return check_launch(eng);
}

extern "C" int fgpu_set_frame_centers(fgpu_engine *eng, const fgpu_frame_center now[2],
                                      const fgpu_frame_center *after)
{
    if (!eng || !now) return FGPU_ERR_BAD_ARG;
    const fgpu_frame_center *a = after ? after : now;
    for (int k = 0; k < 2; ++k) {
        eng->com_now[k] = ComCenter{now[k].x, now[k].y, now[k].vx, now[k].vy, now[k].mass};
        eng->com_after[k] = ComCenter{a[k].x, a[k].y, a[k].vx, a[k].vy, a[k].mass};
        if (eng->e32) {
            eng->e32->com_now[k] = eng->com_now[k];
            eng->e32->com_after[k] = eng->com_after[k];
        }
    }
    return FGPU_OK;
}

// KeepDiskMassConstant (simulation.cpp:246-251, 445-450): gas_total_mass at
// RMAX on the device, then sigma *= target / mass over the whole grid.
static void keep_mass(fgpu_engine *eng, const Launch &L)
{
    if (!eng->p.keep_disk_mass_constant) return;
    launch_gas_quantities(L, eng->p.rmax, eng->bodies.omega_frame, eng->field[FGPU_SIGMA],
                          eng->field[FGPU_V_AZIMUTHAL], eng->partial, eng->red_out + 5);
    launch_scale_sigma(L, eng->field[FGPU_SIGMA], eng->mass_target, eng->red_out + 5);
}

static int mass_target_missing(fgpu_engine *eng)
{
    if (!eng->p.keep_disk_mass_constant || eng->mass_target_set) return FGPU_OK;
    eng->err = "keep_disk_mass_constant needs fgpu_set_disk_mass_target first";
    return FGPU_ERR_BAD_ARG;
}

extern "C" int fgpu_set_disk_mass_target(fgpu_engine *eng, double mass)
{
    if (!eng || !(mass > 0.0) || !std::isfinite(mass)) return FGPU_ERR_BAD_ARG;
    eng->mass_target = mass;
    eng->mass_target_set = true;
    if (eng->e32) eng->e32->set_mass_target(mass);
    return FGPU_OK;
}

extern "C" int fgpu_apply_boundary_condition(fgpu_engine *eng, double t, double dt, int final)
{
    NvtxCall nvtx_("fgpu_apply_boundary_condition");
    (void)t;
    if (!eng) return FGPU_ERR_BAD_ARG;
    if (int rc = com_unready(eng)) return rc;
    if (final)
        if (int rc = mass_target_missing(eng)) return rc;
    ROUTE32(eng->e32->boundary(dt, final != 0));
    Launch L = launch_of(eng);
    if (final) viscous_recompute(eng, L);
    if (final && eng->p.damping) {
        launch_damping(L, eng->dm, dt, eng->damp_rings, eng->n_damp_rings, state_of(eng));
        com_damping(eng, L, dt, eng->com_now);
    }
    ghost(eng, L);
    com_boundary(eng, L, eng->com_now);
    if (final) keep_mass(eng, L);
    eng->cfl_valid = false;
    return check_launch(eng);
}

// The gas kick of step_Euler (simulation.cpp:170-203), and of each half of
// step_LeapFrog (:312-331, :352-384): potential, source terms, artificial
// viscosity, viscosity, stress, viscous update, SubStep3.
static void gas_kick(fgpu_engine *eng, double dt, double t)
{
    Launch L = launch_of(eng);
    const double omf = eng->bodies.omega_frame;
    double **f = eng->field;
    const bool adi = eng->ph.adiabatic;
    // CalculateNbodyPotential (simulation.cpp:170-174)
    launch_potential(L, eng->bodies, f[FGPU_SCALE_HEIGHT], f[FGPU_POTENTIAL]);
    mark(eng, 0);
    // update_with_sourceterms (simulation.cpp:190): momentum updates
    launch_source(L, dt, omf, f[FGPU_SIGMA], f[FGPU_PRESSURE], f[FGPU_POTENTIAL],
                  f[FGPU_V_RADIAL], f[FGPU_V_AZIMUTHAL], eng->vr_alt, eng->vaz_alt);
    std::swap(f[FGPU_V_RADIAL], eng->vr_alt);
    std::swap(f[FGPU_V_AZIMUTHAL], eng->vaz_alt);
    mark(eng, 1);
    State s = state_of(eng);
    // compression heating + artificial viscosity (simulation.cpp:190-194)
    if (adi || eng->ph.art_visc_sn || eng->ph.art_visc_tw) {
        launch_artvisc_q(L, dt, s.sigma, s.vr, s.vaz, s.energy, s.qr, s.qphi);
        if (L.pair && (eng->ph.art_visc_sn || eng->ph.art_visc_tw)) eng->q_pairs = true;
        mark(eng, 2);
        launch_artvisc_v(L, dt, s.sigma, s.energy, s.qr, s.qphi, s.vr, s.vaz, s.cs, s.H, s.nu);
        mark(eng, 3);
    } else {
        mark(eng, 2);
        mark(eng, 3);
    }
    // viscous stress and velocity update, SubStep3 (simulation.cpp:196-203)
    launch_stress(L, s.sigma, s.vr, s.vaz, s.nu, s.divv, s.trr, s.tpp, s.trp);
    eng->stress_pairs = stress_as_pairs(L);
    if (eng->ph.stabilize) launch_visc_corr(L, s);
    mark(eng, 4);
    launch_viscous(L, dt, beta_inv_at(eng->p, t), adi ? 7 : 1, s);
    mark(eng, 5);
}

// Transport (TransportEuler.cpp; simulation.cpp:215-217)
static void transport(fgpu_engine *eng, double dt)
{
    Launch L = launch_of(eng);
    const double omf = eng->bodies.omega_frame;
    double **f = eng->field;
    State s = state_of(eng);
    launch_transport_radial(L, dt, omf, eng->radial_chunk, s.sigma, s.vr, s.vaz, s.energy,
                            eng->mom, eng->energy_alt, eng->sigma_alt);
    mark(eng, 7);
    launch_transport_azimuthal(L, dt, eng->az_block, eng->mom, eng->energy_alt, eng->sigma_alt,
                               s.vaz, eng->ring_ws, eng->az_smem, eng->ring_shift);
    mark(eng, 8);
    launch_finish(L, omf, eng->mom, eng->sigma_alt, eng->energy_alt, s.vr, eng->vr_alt,
                  eng->vaz_alt, s.sigma, s.energy, eng->ring_shift);
    std::swap(f[FGPU_V_RADIAL], eng->vr_alt);
    std::swap(f[FGPU_V_AZIMUTHAL], eng->vaz_alt);
    mark(eng, 9);
}

extern "C" int fgpu_step_euler(fgpu_engine *eng, double dt, double t)
{
    NvtxCall nvtx_("fgpu_step_euler");
    if (!eng || !(dt > 0.0)) return FGPU_ERR_BAD_ARG;
    if (int rc = com_unready(eng)) return rc;
    if (int rc = mass_target_missing(eng)) return rc;
    ROUTE32(eng->e32->step(dt, t));
    Launch L = launch_of(eng);
    mark(eng, -1);
    gas_kick(eng, dt, t);
    // apply_boundary_condition(final = false) (simulation.cpp:213)
    ghost(eng, L);
    com_boundary(eng, L, eng->com_now);
    mark(eng, 6);
    transport(eng, dt);
    viscous_recompute(eng, L);
    State s = state_of(eng);
    // apply_boundary_condition(final = true) (simulation.cpp:244)
    if (eng->p.damping) {
        launch_damping(L, eng->dm, dt, eng->damp_rings, eng->n_damp_rings, s);
        com_damping(eng, L, dt, eng->com_after);
    }
    mark(eng, 10);
    ghost(eng, L);
    com_boundary(eng, L, eng->com_after);
    keep_mass(eng, L);
    mark(eng, 11);
    // recalculate_derived_disk_quantities (simulation.cpp:265) + the next CFL
    CK(cudaMemsetAsync(eng->d_dtmin, 0x7f, sizeof(unsigned long long), eng->stream));
    launch_derived_cfl(L, 1 | 4, s, eng->d_dtmin);
    mark(eng, 12);
    eng->cfl_valid = true;
    return check_launch(eng);
}

extern "C" int fgpu_gas_kick(fgpu_engine *eng, double dt, double t)
{
    NvtxCall nvtx_("fgpu_gas_kick");
    if (!eng || !(dt > 0.0)) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->kick(dt, t));
    gas_kick(eng, dt, t);
    eng->cfl_valid = false;
    return check_launch(eng);
}

extern "C" int fgpu_transport(fgpu_engine *eng, double dt)
{
    NvtxCall nvtx_("fgpu_transport");
    if (!eng || !(dt > 0.0)) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->transport(dt));
    transport(eng, dt);
    eng->cfl_valid = false;
    return check_launch(eng);
}

extern "C" int fgpu_compute_pressure(fgpu_engine *eng)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->pressure());
    Launch L = launch_of(eng);
    launch_pressure(L, eng->field[FGPU_SIGMA], eng->field[FGPU_ENERGY],
                    eng->field[FGPU_PRESSURE]);
    return check_launch(eng);
}

extern "C" int fgpu_disk_on_planet_accel(fgpu_engine *eng, int k, double accel[2])
{
    NvtxCall nvtx_("fgpu_disk_on_planet_accel");
    if (!eng || !accel || k < 0 || k >= eng->bodies.n) return FGPU_ERR_BAD_ARG;
    const Bodies &b = eng->bodies;
    if (eng->e32) {
        double o[5];
        int rc = eng->e32->disk_force(b.x[k], b.y[k], b.a[k], b.rsm[k], o);
        if (rc) {
            eng->err = eng->e32->err;
            return rc;
        }
        accel[0] = o[0] + o[2];
        accel[1] = o[1] + o[3];
        return FGPU_OK;
    }
    // inner/outer split at the body's distance from the origin (t_planet::get_r);
    // the cubic smoothing radius is the same r_sm the gas feels
    launch_disk_force(launch_of(eng), 1, &b.x[k], &b.y[k], &b.a[k], &b.rsm[k],
                      eng->field[FGPU_SIGMA], eng->field[FGPU_SCALE_HEIGHT], eng->partial,
                      eng->red_out);
    int rc = check_launch(eng);
    if (rc) return rc;
    CK(cudaMemcpyAsync(eng->h_pinned, eng->red_out, sizeof(double) * 5, cudaMemcpyDeviceToHost,
                       eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    accel[0] = eng->h_pinned[0] + eng->h_pinned[2];
    accel[1] = eng->h_pinned[1] + eng->h_pinned[3];
    return FGPU_OK;
}

// ComputeDiskOnNbodyAccel (Pframeforce.cpp:194-220): the disk force on every
// body of the last fgpu_set_bodies, all launches queued before one read-back.
extern "C" int fgpu_disk_on_nbody_accel(fgpu_engine *eng, double *accel)
{
    NvtxCall nvtx_("fgpu_disk_on_nbody_accel");
    if (!eng || !accel) return FGPU_ERR_BAD_ARG;
    const Bodies &b = eng->bodies;
    const int n = b.n;
    if (n == 0) return FGPU_OK;
    double sums[5 * kMaxBodies];     // 5 doubles per body
    if (eng->e32) {
        int rc = eng->e32->disk_forces(n, b.x, b.y, b.a, b.rsm, sums);
        if (rc) {
            eng->err = eng->e32->err;
            return rc;
        }
    } else {
        double *out = eng->red_out + 8;
        launch_disk_force(launch_of(eng), n, b.x, b.y, b.a, b.rsm, eng->field[FGPU_SIGMA],
                          eng->field[FGPU_SCALE_HEIGHT], eng->partial, out);
        int rc = check_launch(eng);
        if (rc) return rc;
        CK(cudaMemcpyAsync(eng->h_pinned + 16, out, sizeof(double) * 5 * n,
                           cudaMemcpyDeviceToHost, eng->stream));
        CK(cudaStreamSynchronize(eng->stream));
        std::copy(eng->h_pinned + 16, eng->h_pinned + 16 + 5 * n, sums);
    }
    for (int k = 0; k < n; ++k) {
        const double *o = sums + 5 * k;
        accel[2 * k] = o[0] + o[2];
        accel[2 * k + 1] = o[1] + o[3];
    }
    return FGPU_OK;
}

extern "C" int fgpu_total_mass(fgpu_engine *eng, double *mass)
{
    if (!eng || !mass) return FGPU_ERR_BAD_ARG;
    if (eng->e32) {
        double o[5];
        int rc = eng->e32->disk_force(0.0, 0.0, 0.0, 0.0, o);
        if (rc) eng->err = eng->e32->err;
        *mass = o[4];
        return rc;
    }
    // gas_total_mass over every active ring
    launch_gas_quantities(launch_of(eng), INFINITY, eng->bodies.omega_frame,
                          eng->field[FGPU_SIGMA], eng->field[FGPU_V_AZIMUTHAL], eng->partial,
                          eng->red_out + 5);
    int rc = check_launch(eng);
    if (rc) return rc;
    CK(cudaMemcpyAsync(eng->h_pinned, eng->red_out + 5, sizeof(double), cudaMemcpyDeviceToHost,
                       eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    *mass = eng->h_pinned[0];
    return FGPU_OK;
}

// gas_total_mass / gas_angular_momentum within a radius (quantities.cpp:51-74,
// 242-276): out[0] mass, out[1] angular momentum.
static int gas_quantities(fgpu_engine *eng, double radius, double out[2])
{
    if (eng->e32) {
        int rc = eng->e32->gas_quantities(radius, out);
        if (rc) eng->err = eng->e32->err;
        return rc;
    }
    launch_gas_quantities(launch_of(eng), radius, eng->bodies.omega_frame,
                          eng->field[FGPU_SIGMA], eng->field[FGPU_V_AZIMUTHAL], eng->partial,
                          eng->red_out + 5);
    int rc = check_launch(eng);
    if (rc) return rc;
    CK(cudaMemcpyAsync(eng->h_pinned, eng->red_out + 5, sizeof(double) * 2,
                       cudaMemcpyDeviceToHost, eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    out[0] = eng->h_pinned[0];
    out[1] = eng->h_pinned[1];
    return FGPU_OK;
}

extern "C" int fgpu_gas_total_mass(fgpu_engine *eng, double radius, double *mass)
{
    NvtxCall nvtx_("fgpu_gas_total_mass");
    if (!eng || !mass) return FGPU_ERR_BAD_ARG;
    double o[2];
    int rc = gas_quantities(eng, radius, o);
    if (rc == FGPU_OK) *mass = o[0];
    return rc;
}

extern "C" int fgpu_gas_angular_momentum(fgpu_engine *eng, double radius, double *momentum)
{
    NvtxCall nvtx_("fgpu_gas_angular_momentum");
    if (!eng || !momentum) return FGPU_ERR_BAD_ARG;
    double o[2];
    int rc = gas_quantities(eng, radius, o);
    if (rc == FGPU_OK) *momentum = o[1];
    return rc;
}

// accretion::AccreteOntoPlanets for one planet (accretion.cpp:84-480): the
// constants of the planet's kind and its region (hill_radial_index /
// hill_azimuthal_index, :21-58, with get_rinf_id and get_med_azimuthal_id of
// find_cell_id.cpp under NDEBUG) on the host, the cells on the device.
extern "C" int fgpu_accrete_onto_planet(fgpu_engine *eng, const fgpu_accretor *a, double dt,
                                        double out[3])
{
    NvtxCall nvtx_("fgpu_accrete_onto_planet");
    if (!eng || !a || !out || !(dt >= 0.0)) return FGPU_ERR_BAD_ARG;
    if (a->type != FGPU_ACCRETION_KLEY && a->type != FGPU_ACCRETION_VISCOUS &&
        a->type != FGPU_ACCRETION_SINKHOLE) {
        eng->err = "accretion type";
        return FGPU_ERR_BAD_ARG;
    }
    if (!(a->orbital_period > 0.0) && a->type != FGPU_ACCRETION_VISCOUS) {
        eng->err = "accretion needs the planet's orbital period";
        return FGPU_ERR_BAD_ARG;
    }
    const fgpu_params &p = eng->p;
    const int nr = eng->nr, ns = eng->nz;
    AccretionSpec sp{};
    sp.type = a->type;
    sp.x = a->x;
    sp.y = a->y;
    sp.rhill = a->roche_radius;
    sp.density_floor = p.sigma_floor * p.sigma0;
    sp.omf = eng->bodies.omega_frame;
    const double frac = p.accretion_radius_fraction;
    if (a->type == FGPU_ACCRETION_KLEY) {
        const double facc = dt * a->efficiency / a->orbital_period * std::log(2);
        sp.facc1 = 1.0 / 3.0 * facc;
        sp.facc2 = 2.0 / 3.0 * facc;
        sp.frac1 = frac;
        sp.frac2 = 0.5 * frac;
    } else if (a->type == FGPU_ACCRETION_SINKHOLE) {
        sp.facc1 = dt * a->efficiency / a->orbital_period * std::log(2.0);
        sp.frac1 = frac;
    } else {
        sp.facc1 = dt * 3.0 * M_PI * a->efficiency;
        sp.frac1 = frac;
        sp.dist_max = a->roche_radius * frac;
        sp.f_const = 3.0 / M_PI / std::pow(sp.dist_max, 2);
    }
    const double R = a->r;
    const double search = a->roche_radius * sp.frac1 + 2.0 * R / ns;
    std::vector<double> Rmed;  // unused by the rinf search
    sp.i0 = (R - search < p.rmin) ? 0 : clamp_id(cell_id(eng, Rmed, R - search, true), false, nr);
    sp.i1 = clamp_id(cell_id(eng, Rmed, R + search, true) + 1, false, nr);
    const double max_angle = R == 0.0 ? 2.0 * M_PI : std::min(2.0 * M_PI, 2.0 * search / R);
    const double cell = 2.0 * M_PI / (double)ns, inv = (double)ns / 2.0 / M_PI;
    const int j_min = (int)std::floor((a->phi - max_angle - 0.5 * cell) * inv);
    int j_max = (int)std::floor((a->phi + max_angle - 0.5 * cell) * inv) + 1;
    j_max = j_min + std::min(j_max - j_min, ns - 1);
    sp.j0 = j_min;
    sp.ncols = j_max - j_min + 1;
    if (sp.i1 < sp.i0 || sp.ncols < 1) {
        out[0] = out[1] = out[2] = 0.0;
        return FGPU_OK;
    }
    if (eng->e32) {
        const fgpu32::AccrF af{sp.type, sp.i0, sp.i1, sp.j0, sp.ncols, sp.x, sp.y, sp.rhill,
                               sp.frac1, sp.frac2, sp.facc1, sp.facc2, sp.f_const, sp.dist_max,
                               sp.density_floor, sp.omf};
        ROUTE32(eng->e32->accrete(af, out));
    }
    double **f = eng->field;
    launch_accrete(launch_of(eng), sp, f[FGPU_SIGMA], f[FGPU_ENERGY], f[FGPU_V_RADIAL],
                   f[FGPU_V_AZIMUTHAL], f[FGPU_VISCOSITY], eng->red_out);
    int rc = check_launch(eng);
    if (rc) return rc;
    CK(cudaMemcpyAsync(eng->h_pinned, eng->red_out, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                       eng->stream));
    CK(cudaStreamSynchronize(eng->stream));
    for (int k = 0; k < 3; ++k) out[k] = eng->h_pinned[k];
    eng->cfl_valid = false;
    return FGPU_OK;
}

extern "C" int fgpu_check_finite(fgpu_engine *eng, int *field, int *nr, int *naz)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    ROUTE32(eng->e32->check_finite(field, nr, naz));
    const int fields[4] = {FGPU_SIGMA, FGPU_V_RADIAL, FGPU_V_AZIMUTHAL, FGPU_ENERGY};
    Launch L = launch_of(eng);
    for (int k = 0; k < 4; ++k) {
        const int f = fields[k];
        const size_t n = (size_t)field_rows(eng, f) * eng->nz;
        CK(cudaMemsetAsync(eng->d_bad, 0xff, sizeof(unsigned long long), eng->stream));
        launch_check_finite(L, eng->field[f], n, eng->d_bad);
        CK(cudaMemcpyAsync(eng->h_pinned, eng->d_bad, sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, eng->stream));
        CK(cudaStreamSynchronize(eng->stream));
        unsigned long long bad;
        std::memcpy(&bad, eng->h_pinned, sizeof(bad));
        if (bad != ~0ull) {
            if (field) *field = f;
            if (nr) *nr = (int)(bad / eng->nz);
            if (naz) *naz = (int)(bad % eng->nz);
            return FGPU_ERR_NONFINITE;
        }
    }
    return FGPU_OK;
}

extern "C" int fgpu_synchronize(fgpu_engine *eng)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(eng->stream));
    return FGPU_OK;
}

extern "C" int fgpu_set_phase_timing(fgpu_engine *eng, int enable)
{
    if (!eng) return FGPU_ERR_BAD_ARG;
    eng->timing = enable != 0;
    return FGPU_OK;
}

extern "C" const char *fgpu_phase_name(int k)
{
    return (k >= 0 && k < kPhases) ? kPhaseNames[k] : nullptr;
}

extern "C" int fgpu_phase_times(fgpu_engine *eng, double *ms, int capacity, int *count,
                                int *steps)
{
    if (!eng || !ms || capacity < kPhases) return FGPU_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(eng->stream));
    for (int k = 0; k < kPhases; ++k) ms[k] = 0.0;
    int n = 0;
    for (auto &row : eng->ev_rows) {
        if ((int)row.size() == kPhases + 1) {
            for (int k = 0; k < kPhases; ++k) {
                float t = 0.f;
                CK(cudaEventElapsedTime(&t, row[k], row[k + 1]));
                ms[k] += t;
            }
            ++n;
        }
        for (auto ev : row) eng->ev_free.push_back(ev);
    }
    eng->ev_rows.clear();
    if (count) *count = kPhases;
    if (steps) *steps = n;
    return FGPU_OK;
}
