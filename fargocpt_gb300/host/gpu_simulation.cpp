/*
 * gpu_simulation.cpp -- FargoCPT's run loop with the gas step on the GB300
 * engine.
 *
 * A drop-in translation unit: a FargoCPT build compiles it in place of
 * src/simulation.cpp and links libfargocpt_gb300.so.  It defines the same
 * namespace sim symbols (src/simulation.h) with the same call order as
 * sim::run / sim::init / step_Euler / step_LeapFrog (src/simulation.cpp:
 * 100-118, 148-267, 276-459, 462-558); everything else -- configuration,
 * initial conditions, the N-body system, boundaries' host set-up, output and
 * restart -- is FargoCPT's own code.  The gas step, the CFL time step, the
 * disk force on the bodies, accretion's cell updates, the boundary hooks and
 * damping, KeepDiskMassConstant and the corotating frame's v_phi correction
 * run on the GPU through include/fargocpt_gb300.h; the fields live in HBM and
 * are copied to the host grids before every output (and uploaded again after
 * a restart), so the files are FargoCPT's own.
 *
 * Options the engine does not cover stop the run at start-up with a message
 * (die), never silently: self-gravity, radiative diffusion, particles,
 * variable gamma, polytropic or non-default aspect-ratio modes, the
 * Roche-lobe overflow and custom boundaries, viscous damping of v_radial,
 * gas-acceleration forces instead of the potential, and the time-integrated
 * torque / alpha outputs that read the host fields every step.
 *
 * FGPU_PRECISION=fp32 in the environment selects the FP32-mixed form;
 * FGPU_DUMP_PARAMS=<file> writes the fgpu_params block the run derived from
 * the configuration (for comparing the mapping with other front ends).
 */
#include "simulation.h"

#include "LowTasks.h"
#include "Pframeforce.h"
#include "SourceEuler.h"
#include "Theo.h"
#include "accretion.h"
#include "boundary_conditions/boundary_conditions.h"
#include "cfl.h"
#include "circumplanetary_mass.h"
#include "commbound.h"
#include "constants.h"
#include "fld.h"
#include "frame_of_reference.h"
#include "global.h"
#include "logging.h"
#include "options.h"
#include "output.h"
#include "parameters.h"
#include "quantities.h"
#include "start_mode.h"
#include "units.h"

#include "fargocpt_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace sim
{

double last_dt;
double time, timeInitial;
unsigned int N_snapshot = 0;
unsigned int N_monitor = 0;
unsigned long int N_hydro_iter = 0;

double total_disk_mass_old;

namespace
{

fgpu_engine *g_gpu = nullptr;

void gpu_check(int rc, const char *what)
{
    if (rc != FGPU_OK) {
	die("GB300 engine: %s failed with status %d: %s\n", what, rc,
	    g_gpu ? fgpu_last_error(g_gpu) : "(no engine)");
    }
}

// The engine's fields and the t_data grids that hold them on the host.
struct FieldPair {
    int engine;
    t_data::t_polargrid_type host;
};
const FieldPair kFields[] = {
    {FGPU_SIGMA, t_data::SIGMA},
    {FGPU_V_RADIAL, t_data::V_RADIAL},
    {FGPU_V_AZIMUTHAL, t_data::V_AZIMUTHAL},
    {FGPU_ENERGY, t_data::ENERGY},
    {FGPU_SIGMA0, t_data::SIGMA0},
    {FGPU_V_RADIAL0, t_data::V_RADIAL0},
    {FGPU_V_AZIMUTHAL0, t_data::V_AZIMUTHAL0},
    {FGPU_ENERGY0, t_data::ENERGY0},
    {FGPU_SOUNDSPEED, t_data::SOUNDSPEED},
    {FGPU_SCALE_HEIGHT, t_data::SCALE_HEIGHT},
    {FGPU_PRESSURE, t_data::PRESSURE},
    {FGPU_TEMPERATURE, t_data::TEMPERATURE},
    {FGPU_VISCOSITY, t_data::VISCOSITY},
    {FGPU_QPLUS, t_data::QPLUS},
    {FGPU_QMINUS, t_data::QMINUS},
    {FGPU_POTENTIAL, t_data::POTENTIAL},
    {FGPU_DIV_V, t_data::DIV_V},
    {FGPU_TAU_R_R, t_data::TAU_R_R},
    {FGPU_TAU_PHI_PHI, t_data::TAU_PHI_PHI},
    {FGPU_TAU_R_PHI, t_data::TAU_R_PHI},
    {FGPU_Q_R, t_data::Q_R},
    {FGPU_Q_PHI, t_data::Q_PHI},
};

void upload_all(t_data &data)
{
    for (const FieldPair &f : kFields) {
	t_polargrid &g = data[f.host];
	gpu_check(fgpu_upload_field(g_gpu, f.engine, g.Field, (int)g.get_size_radial(),
				    (int)g.get_size_azimuthal()),
		  "fgpu_upload_field");
    }
}

void download_all(t_data &data)
{
    for (const FieldPair &f : kFields) {
	t_polargrid &g = data[f.host];
	gpu_check(fgpu_download_field(g_gpu, f.engine, g.Field, (int)g.get_size_radial(),
				      (int)g.get_size_azimuthal()),
		  "fgpu_download_field");
    }
}

// The hook a boundary function pointer selects (boundary_conditions/config.cpp
// sets them; comparing the pointers carries every quirk of that set-up).
using hook_fn = void (*)(t_polargrid &, t_polargrid &, t_data &);
int hook_kind(hook_fn fn, const char *what)
{
    namespace bc = boundary_conditions;
    struct {
	hook_fn fn;
	int kind;
    } const table[] = {
	{bc::zero_gradient_inner, FGPU_BC_ZEROGRADIENT},
	{bc::zero_gradient_outer, FGPU_BC_ZEROGRADIENT},
	{bc::outflow_inner, FGPU_BC_OUTFLOW},
	{bc::outflow_outer, FGPU_BC_OUTFLOW},
	{bc::reference_inner, FGPU_BC_REFERENCE},
	{bc::reference_outer, FGPU_BC_REFERENCE},
	{bc::keplerian_azimuthal_inner, FGPU_BC_KEPLERIAN},
	{bc::keplerian_azimuthal_outer, FGPU_BC_KEPLERIAN},
	{bc::diskmodel_inner_sigma, FGPU_BC_DISKMODEL},
	{bc::diskmodel_outer_sigma, FGPU_BC_DISKMODEL},
	{bc::diskmodel_inner_energy, FGPU_BC_DISKMODEL},
	{bc::diskmodel_outer_energy, FGPU_BC_DISKMODEL},
	{bc::reflecting_inner, FGPU_BC_REFLECTING},
	{bc::reflecting_outer, FGPU_BC_REFLECTING},
	{bc::viscous_outflow_inner, FGPU_BC_VISCOUS},
	{bc::viscous_inflow_outer, FGPU_BC_VISCOUS},
	{bc::keplerian_radial_inner, FGPU_BC_KEPLERIAN_RADIAL},
	{bc::keplerian_radial_outer, FGPU_BC_KEPLERIAN_RADIAL},
	{bc::zero_shear_inner, FGPU_BC_ZEROSHEAR},
	{bc::zero_shear_outer, FGPU_BC_ZEROSHEAR},
	{bc::balanced_inner, FGPU_BC_BALANCED},
	{bc::balanced_outer, FGPU_BC_BALANCED},
	{bc::no_operation, FGPU_BC_NONE},
    };
    if (fn == nullptr) return FGPU_BC_NONE;
    for (const auto &e : table) {
	if (e.fn == fn) return e.kind;
    }
    die("GB300 engine: the %s boundary hook has no GPU form\n", what);
    return FGPU_BC_NONE;
}

int damping_kind(boundary_conditions::t_damping_type t, const char *what)
{
    using namespace boundary_conditions;
    switch (t) {
    case damping_none: return FGPU_DAMP_NONE;
    case damping_reference: return FGPU_DAMP_REFERENCE;
    case damping_zero: return FGPU_DAMP_ZERO;
    case damping_mean: return FGPU_DAMP_MEAN;
    default: break;
    }
    die("GB300 engine: the %s damping kind has no GPU form\n", what);
    return FGPU_DAMP_NONE;
}

int composite_kind(const std::string &name)
{
    return name == "centerofmass" ? FGPU_COMPOSITE_CENTER_OF_MASS : FGPU_COMPOSITE_INDIVIDUAL;
}

// The fgpu_params block of this run, from parameters:: and the boundary
// set-up (the header names the source of each field).
fgpu_params engine_params(t_data &data)
{
    namespace bc = boundary_conditions;
    if (parameters::self_gravity) die("GB300 engine: self-gravity is not on the GPU path\n");
    if (fld::radiative_diffusion_enabled)
	die("GB300 engine: radiative diffusion is not on the GPU path\n");
    if (parameters::integrate_particles) die("GB300 engine: particles are not on the GPU path\n");
    if (parameters::variableGamma || parameters::Polytropic)
	die("GB300 engine: only the isothermal and ideal equations of state\n");
    if (parameters::aspectratio_mode != 0)
	die("GB300 engine: only AspectRatioMode 0\n");
    if (!parameters::body_force_from_potential)
	die("GB300 engine: the gas feels the bodies through the potential only\n");
    if (bc::rochelobe_overflow) die("GB300 engine: no Roche-lobe overflow boundary\n");
    if (bc::special_inner_func != nullptr || bc::special_outer_func != nullptr ||
	bc::composite_inner_name == "custom" || bc::composite_outer_name == "custom")
	die("GB300 engine: no custom boundaries\n");
    if (data[t_data::ADVECTION_TORQUE].get_write() || data[t_data::VISCOUS_TORQUE].get_write() ||
	data[t_data::GRAVITATIONAL_TORQUE_NOT_INTEGRATED].get_write() ||
	data[t_data::ALPHA_GRAV_MEAN].get_write() || data[t_data::ALPHA_REYNOLDS_MEAN].get_write())
	die("GB300 engine: time-integrated torque and alpha outputs read the host fields every "
	    "step; disable them\n");

    fgpu_params p;
    std::memset(&p, 0, sizeof p);
    p.nrad = (int)data[t_data::SIGMA].get_size_radial();
    p.naz = (int)data[t_data::SIGMA].get_size_azimuthal();
    p.eos = parameters::Adiabatic ? FGPU_EOS_IDEAL : FGPU_EOS_ISOTHERMAL;
    switch (parameters::artificial_viscosity) {
    case parameters::artificial_viscosity_SN: p.art_visc = FGPU_ARTVISC_SN; break;
    case parameters::artificial_viscosity_TW: p.art_visc = FGPU_ARTVISC_TW; break;
    default: p.art_visc = FGPU_ARTVISC_NONE; break;
    }
    p.art_visc_dissipation = parameters::artificial_viscosity_dissipation ? 1 : 0;
    p.flux_limiter = flux_limiter_type == 1 ? FGPU_LIMITER_MC : FGPU_LIMITER_VANLEER;
    p.fast_transport = parameters::fast_transport ? 1 : 0;
    p.heating_viscous = parameters::heating_viscous_enabled ? 1 : 0;
    p.cooling_beta = parameters::cooling_beta_enabled ? 1 : 0;
    p.cooling_beta_reference = parameters::cooling_beta_reference ? FGPU_BETA_REF_REFERENCE
			       : parameters::cooling_beta_model   ? FGPU_BETA_REF_DISKMODEL
			       : parameters::cooling_beta_floor   ? FGPU_BETA_REF_FLOOR
								  : FGPU_BETA_REF_ZERO;
    p.damping = bc::damping_enabled ? 1 : 0;
    for (const auto &d : bc::damping_vector) {
	int q = -1;
	switch (d.array_to_damp) {
	case t_data::V_RADIAL: q = FGPU_DQ_VRAD; break;
	case t_data::V_AZIMUTHAL: q = FGPU_DQ_VAZI; break;
	case t_data::SIGMA: q = FGPU_DQ_SIGMA; break;
	case t_data::ENERGY: q = FGPU_DQ_ENERGY; break;
	default: die("GB300 engine: damping of an unexpected field\n");
	}
	p.damping_inner[q] = damping_kind(d.type_inner, "inner");
	p.damping_outer[q] = damping_kind(d.type_outer, "outer");
    }
    p.bc_sigma_inner = hook_kind(bc::sigma_inner_func, "inner sigma");
    p.bc_sigma_outer = hook_kind(bc::sigma_outer_func, "outer sigma");
    p.bc_energy_inner = hook_kind(bc::energy_inner_func, "inner energy");
    p.bc_energy_outer = hook_kind(bc::energy_outer_func, "outer energy");
    p.bc_vrad_inner = hook_kind(bc::vrad_inner_func, "inner v_radial");
    p.bc_vrad_outer = hook_kind(bc::vrad_outer_func, "outer v_radial");
    p.bc_vaz_inner = hook_kind(bc::vaz_inner_func, "inner v_azimuthal");
    p.bc_vaz_outer = hook_kind(bc::vaz_outer_func, "outer v_azimuthal");
    const char *prec = std::getenv("FGPU_PRECISION");
    p.precision = (prec && std::strcmp(prec, "fp32") == 0) ? FGPU_PRECISION_FP32_MIXED
							      : FGPU_PRECISION_FP64;
    p.integrator = parameters::hydro_integrator == LEAPFROG_INTEGRATOR
		       ? FGPU_INTEGRATOR_LEAPFROG
		       : FGPU_INTEGRATOR_EULER;
    p.stabilize_viscosity = StabilizeViscosity;
    p.profile_cutoff_outer = parameters::profile_cutoff_outer ? 1 : 0;
    p.viscous_accretion = parameters::VISCOUS_ACCRETION ? 1 : 0;
    p.composite_inner = composite_kind(bc::composite_inner_name);
    p.composite_outer = composite_kind(bc::composite_outer_name);
    p.initialize_pure_keplerian = parameters::initialize_pure_keplerian ? 1 : 0;
    p.initialize_vradial_zero = parameters::initialize_vradial_zero ? 1 : 0;
    p.profile_cutoff_inner = parameters::profile_cutoff_inner ? 1 : 0;
    p.keep_disk_mass_constant = parameters::keep_mass_constant ? 1 : 0;

    p.gamma = parameters::ADIABATICINDEX;
    p.mu = parameters::MU;
    p.aspect_ratio = parameters::aspectratio_ref;
    p.flaring_index = parameters::flaring_index;
    p.viscous_alpha = parameters::viscous_alpha;
    p.constant_viscosity = parameters::constant_viscosity;
    p.art_visc_factor = parameters::artificial_viscosity_factor;
    p.radial_viscosity_factor = parameters::radial_viscosity_factor;
    p.heating_viscous_factor = parameters::heating_viscous_factor;
    p.cfl = parameters::CFL;
    p.cfl_max_var = parameters::CFL_max_var;
    p.heating_cooling_cfl_limit = parameters::HEATING_COOLING_CFL_LIMIT;
    p.sigma0 = parameters::sigma0;
    p.sigma_floor = parameters::sigma_floor;
    p.thickness_smoothing = parameters::thickness_smoothing;
    p.cooling_beta_value = parameters::cooling_beta;
    p.cooling_beta_ramp_up = parameters::cooling_beta_ramp_up;
    p.minimum_temperature = parameters::minimum_temperature;
    p.maximum_temperature = parameters::maximum_temperature;
    p.G = constants::G;
    p.R_gas = constants::R;
    p.sigma_sb = constants::sigma;
    p.c_light = constants::c;
    p.hydro_center_mass = hydro_center_mass;
    p.damping_inner_limit = bc::damping_inner_limit;
    p.damping_outer_limit = bc::damping_outer_limit;
    p.damping_time_factor = bc::damping_time_factor;
    p.damping_time_radius_outer = bc::damping_time_radius_outer;
    p.vaz_inner_keplerian_factor = bc::keplerian_azimuthal_inner_factor;
    p.vaz_outer_keplerian_factor = bc::keplerian_azimuthal_outer_factor;
    p.rmin = RMIN;
    p.rmax = RMAX;
    p.radial_spacing = parameters::radial_grid_type == parameters::arithmetic_spacing
			   ? FGPU_SPACING_ARITHMETIC
			   : FGPU_SPACING_LOGARITHMIC;
    if (parameters::radial_grid_type != parameters::arithmetic_spacing &&
	parameters::radial_grid_type != parameters::logarithmic_spacing)
	die("GB300 engine: only arithmetic and logarithmic radial grids\n");
    p.correct_disk_selfgravity = parameters::correct_disk_selfgravity ? 1 : 0;
    p.accretion_radius_fraction = parameters::accretion_radius_fraction;
    p.sigma_slope = parameters::sigma_slope;
    p.viscous_outflow_speed = bc::viscous_outflow_speed;
    p.vrad_inner_keplerian_factor = bc::keplerian_radial_inner_factor;
    p.vrad_outer_keplerian_factor = bc::keplerian_radial_outer_factor;
    p.binary_quadrupole_moment = binary_quadropole_moment;
    p.profile_cutoff_point_outer = parameters::profile_cutoff_point_outer;
    p.profile_cutoff_width_outer = parameters::profile_cutoff_width_outer;
    p.profile_cutoff_point_inner = parameters::profile_cutoff_point_inner;
    p.profile_cutoff_width_inner = parameters::profile_cutoff_width_inner;
    p.temperature_cgs_to_code = units::temperature.get_cgs_to_code_factor();
    return p;
}

// The bodies as the potential sees them at current_time
// (CalculateNbodyPotential, Pframeforce.cpp:21-40).
int collect_bodies(t_data &data, const double current_time, fgpu_body *b)
{
    auto &ps = data.get_planetary_system();
    const int n = (int)ps.get_number_of_planets();
    if (n > 16) die("GB300 engine: at most 16 bodies\n");
    for (int k = 0; k < n; ++k) {
	t_planet &pl = ps.get_planet(k);
	b[k].x = pl.get_x();
	b[k].y = pl.get_y();
	b[k].mass = pl.get_rampup_mass(current_time);
	b[k].r_sm = pl.get_dimensionless_roche_radius() * pl.get_distance_to_primary() *
		    pl.get_cubic_smoothing_factor();
	b[k].a = pl.get_r();
    }
    return n;
}

void set_bodies(int n, const fgpu_body *b)
{
    gpu_check(fgpu_set_bodies(g_gpu, n, b, refframe::IndirectTerm.x, refframe::IndirectTerm.y,
			      refframe::OmegaFrame),
	      "fgpu_set_bodies");
}

// ComputeDiskOnNbodyAccel (Pframeforce.cpp:194-220) with the forces from the GPU.
void disk_on_nbody_accel(t_data &data)
{
    auto &ps = data.get_planetary_system();
    fgpu_body b[16];
    const int n = collect_bodies(data, time, b);
    set_bodies(n, b);
    double acc[32];
    gpu_check(fgpu_disk_on_nbody_accel(g_gpu, acc), "fgpu_disk_on_nbody_accel");
    for (int k = 0; k < n; ++k) {
	t_planet &pl = ps.get_planet(k);
	if (parameters::planet_orbit_disk_test && k == 0) {
	    pl.set_disk_on_planet_acceleration(Pair{0.0, 0.0});
	    continue;
	}
	const Pair a{acc[2 * k], acc[2 * k + 1]};
	pl.set_disk_on_planet_acceleration(a);
	pl.set_torque((pl.get_x() * a.y - pl.get_y() * a.x) * pl.get_mass());
    }
}

// accretion::AccreteOntoPlanets (accretion.cpp:482-516) with the cells updated
// on the GPU and the planets on the host (update_planet, accretion.cpp:60-82).
void accrete_onto_planets(t_data &data, const double dt)
{
    auto &ps = data.get_planetary_system();
    bool masses_changed = false;
    for (unsigned int k = 0; k < ps.get_number_of_planets(); ++k) {
	t_planet &pl = ps.get_planet(k);
	const int type = pl.get_accretion_type();
	if (type != ACCRETION_TYPE_KLEY && type != ACCRETION_TYPE_VISCOUS &&
	    type != ACCRETION_TYPE_SINKHOLE)
	    continue;
	fgpu_accretor a;
	std::memset(&a, 0, sizeof a);
	a.type = type == ACCRETION_TYPE_KLEY      ? FGPU_ACCRETION_KLEY
		 : type == ACCRETION_TYPE_VISCOUS ? FGPU_ACCRETION_VISCOUS
						  : FGPU_ACCRETION_SINKHOLE;
	a.x = pl.get_x();
	a.y = pl.get_y();
	a.r = pl.get_r();
	a.phi = pl.get_phi();
	a.roche_radius = pl.get_dimensionless_roche_radius() * pl.get_distance_to_primary();
	a.efficiency = pl.get_accretion_efficiency();
	a.orbital_period = pl.get_orbital_period();
	double got[3];
	gpu_check(fgpu_accrete_onto_planet(g_gpu, &a, dt, got), "fgpu_accrete_onto_planet");
	pl.add_accreted_mass(got[0]);
	if (parameters::disk_feedback || parameters::accrete_without_disk_feedback) {
	    const double m_old = pl.get_mass();
	    const double px = m_old * pl.get_vx() + got[1];
	    const double py = m_old * pl.get_vy() + got[2];
	    const double m_new = m_old + got[0];
	    pl.add_accretion_torque(pl.get_x() * got[2] - pl.get_y() * got[1]);
	    pl.set_vx(px / m_new);
	    pl.set_vy(py / m_new);
	    pl.set_mass(m_new);
	    masses_changed = masses_changed || got[0] > 0;
	}
    }
    if (masses_changed) {
	ps.update_global_hydro_frame_center_mass();
	ps.update_roche_radii();
    }
}

// the centres the centre-of-mass boundary reads (planetary_system.cpp:580-650)
fgpu_frame_center frame_center(t_data &data, unsigned int n)
{
    auto &ps = data.get_planetary_system();
    const Pair x = ps.get_center_of_mass(n), v = ps.get_center_of_mass_velocity(n);
    return fgpu_frame_center{x.x, x.y, v.x, v.y, ps.get_mass(n)};
}

bool center_of_mass_boundary()
{
    return boundary_conditions::composite_inner_name == "centerofmass" ||
	   boundary_conditions::composite_outer_name == "centerofmass";
}

// OmegaFrame before and after handle_corotation: the engine corrects v_phi
// (correct_v_azimuthal, SideEuler.cpp:79-95); the host copy it also changes is
// overwritten at the next download.
void corotation(t_data &data, const double dt)
{
    const double omega_old = refframe::OmegaFrame;
    refframe::handle_corotation(data, dt);
    if (parameters::calculate_disk && refframe::OmegaFrame != omega_old)
	gpu_check(fgpu_correct_v_azimuthal(g_gpu, refframe::OmegaFrame - omega_old),
		  "fgpu_correct_v_azimuthal");
}

void write_snapshot(t_data &data)
{
    output::last_snapshot_dir = output::snapshot_dir;
    output::write_full_output(data, std::to_string(N_snapshot));
    output::cleanup_autosave();
    if (N_snapshot == 0 && boundary_conditions::initial_values_needed()) {
	const std::string snapshot_dir_old = output::snapshot_dir;
	output::write_full_output(data, "reference", false);
	output::snapshot_dir = snapshot_dir_old;
    }
}

} // namespace

// sim::handle_outputs (simulation.cpp:50-98): the host grids are refreshed
// from the GPU first, then FargoCPT writes its own files.
void handle_outputs(t_data &data)
{
    if (g_gpu) download_all(data);
    bool need_update_for_output = true;
    N_snapshot = (N_monitor / parameters::Nmonitor);
    const bool to_write_snapshot = (parameters::Nmonitor * N_snapshot == N_monitor);
    const bool to_write_monitor = to_write_snapshot || parameters::write_at_every_timestep;

    if (!parameters::disk_feedback && to_write_monitor) {
	if (g_gpu)
	    disk_on_nbody_accel(data);
	else
	    ComputeDiskOnNbodyAccel(data);
    }
    if (to_write_snapshot) {
	need_update_for_output = false;
	write_snapshot(data);
    }
    if (to_write_snapshot && parameters::write_torques) {
	need_update_for_output = true;
	output::write_torques(data, need_update_for_output);
	need_update_for_output = false;
    }
    if (to_write_monitor) {
	dt_logger.write(N_snapshot, N_monitor);
	if (ECC_GROWTH_MONITOR) {
	    output::write_ecc_peri_changes(sim::N_snapshot, sim::N_monitor);
	}
	output::write_monitor_time();
	ComputeCircumPlanetaryMasses(data);
	data.get_planetary_system().write_planets(1);
	if (parameters::write_lightcurves) {
	    output::write_lightcurves(data, N_snapshot, need_update_for_output);
	}
	fld::write_logfile(output::outdir + "/monitor/fld.log");
    }
    if ((to_write_monitor) && parameters::write_disk_quantities) {
	output::write_quantities(data, need_update_for_output);
    }
}

// sim::CalculateTimeStep (simulation.cpp:100-118) with the CFL step of the GPU.
double CalculateTimeStep(t_data &data)
{
    double rv = last_dt;
    if (parameters::calculate_disk) {
	// main() asks once before sim::run creates the engine (main.cpp:117):
	// that call reads the host state init_physics built
	double cfl_dt;
	if (g_gpu)
	    gpu_check(fgpu_condition_cfl(g_gpu, &cfl_dt), "fgpu_condition_cfl");
	else
	    cfl_dt = cfl::condition_cfl(data);
	rv = std::min(parameters::CFL_max_var * last_dt, cfl_dt);
	last_dt = rv;
	if (PRINT_SIG_INFO && g_gpu) {
	    // the limiting cell of the GPU's own step, FargoCPT's report format
	    fgpu_cfl_cell c;
	    gpu_check(fgpu_cfl_limiting_cell(g_gpu, &c), "fgpu_cfl_limiting_cell");
	    logging::print_master(LOG_INFO
				  "CFL: limiting cell (%d, %d), dt %g; inverse times "
				  "%g %g %g %g %g %g; shear limit %g at ring %d\n",
				  c.ring, c.azimuth, c.dt_cell, c.invdt[0], c.invdt[1], c.invdt[2],
				  c.invdt[3], c.invdt[4], c.invdt[5], c.dt_shear, c.shear_ring);
	    PRINT_SIG_INFO = false;
	}
    }
    dt_logger.update(rv);
    return rv;
}

// step_Euler (simulation.cpp:148-267)
static void step_Euler(t_data &data, const double dt)
{
    auto &ps = data.get_planetary_system();
    if (parameters::calculate_disk) accrete_onto_planets(data, dt);
    if (parameters::disk_feedback) {
	disk_on_nbody_accel(data);
	UpdatePlanetVelocitiesWithDiskForce(data, dt);
    }
    refframe::ComputeIndirectTermDisk(data, dt);
    refframe::ComputeIndirectTermNbody(data, time, dt);
    refframe::ComputeIndirectTermFully();
    ps.apply_indirect_term_on_Nbody(refframe::IndirectTerm, dt);

    // the potential's bodies as CalculateNbodyPotential takes them, before
    // handle_corotation rotates them; the frame speed after it
    fgpu_body bodies[16];
    const int nb = collect_bodies(data, time, bodies);
    fgpu_frame_center now[2];
    const bool com = center_of_mass_boundary();
    if (com) {
	now[0] = frame_center(data, parameters::n_bodies_for_hydroframe_center);
	now[1] = frame_center(data, ps.get_number_of_planets());
    }
    corotation(data, dt);
    set_bodies(nb, bodies);

    if (com) {
	// the final boundary call of the step reads the centres after the
	// N-body step, so the N-body step goes first; the gas does not feed it
	ps.integrate(time, dt);
	ps.copy_data_from_rebound();
	ps.move_to_hydro_center_and_update_orbital_parameters();
	fgpu_frame_center after[2] = {
	    frame_center(data, parameters::n_bodies_for_hydroframe_center),
	    frame_center(data, ps.get_number_of_planets())};
	gpu_check(fgpu_set_frame_centers(g_gpu, now, after), "fgpu_set_frame_centers");
	if (parameters::calculate_disk) gpu_check(fgpu_step_euler(g_gpu, dt, time), "fgpu_step_euler");
    } else {
	// the gas step is queued first: the host's N-body step overlaps it
	if (parameters::calculate_disk) gpu_check(fgpu_step_euler(g_gpu, dt, time), "fgpu_step_euler");
	ps.integrate(time, dt);
	ps.copy_data_from_rebound();
	ps.move_to_hydro_center_and_update_orbital_parameters();
    }
    time += dt;
    N_hydro_iter = N_hydro_iter + 1;
    logging::print_runtime_info();
}

// step_LeapFrog (simulation.cpp:276-459): the N-body drift-kick-drift on the
// host as there, the gas kick-drift-kick from the engine's phases
static void step_LeapFrog(t_data &data, const double step_dt)
{
    auto &ps = data.get_planetary_system();
    const double frog_dt = step_dt / 2;
    const double start_time = time;
    const double midstep_time = time + frog_dt;
    const double end_time = time + step_dt;
    fgpu_body bodies[16];

    refframe::ComputeIndirectTermNbody(data, start_time, frog_dt);
    refframe::init_corotation(data);
    ps.integrate(start_time, frog_dt);
    ps.copy_data_from_rebound();
    ps.move_to_hydro_center_and_update_orbital_parameters();
    if (parameters::disk_feedback) disk_on_nbody_accel(data);
    refframe::ComputeIndirectTermDisk(data, frog_dt);
    refframe::ComputeIndirectTermFully();

    if (parameters::calculate_disk) accrete_onto_planets(data, frog_dt);
    if (parameters::disk_feedback) UpdatePlanetVelocitiesWithDiskForce(data, frog_dt);
    ps.apply_indirect_term_on_Nbody(refframe::IndirectTerm, frog_dt);
    corotation(data, frog_dt);

    if (parameters::calculate_disk) {
	set_bodies(collect_bodies(data, start_time, bodies), bodies);
	gpu_check(fgpu_gas_kick(g_gpu, frog_dt, start_time), "fgpu_gas_kick");
	gpu_check(fgpu_apply_boundary_condition(g_gpu, start_time, 0.0, 0),
		  "fgpu_apply_boundary_condition");
	gpu_check(fgpu_transport(g_gpu, step_dt), "fgpu_transport");
    }

    if (parameters::disk_feedback) disk_on_nbody_accel(data);
    refframe::ComputeIndirectTermDisk(data, frog_dt);
    refframe::ComputeIndirectTermNbody(data, midstep_time, frog_dt);
    refframe::ComputeIndirectTermFully();

    if (parameters::calculate_disk) {
	set_bodies(collect_bodies(data, midstep_time, bodies), bodies);
	gpu_check(fgpu_compute_pressure(g_gpu), "fgpu_compute_pressure");
	gpu_check(fgpu_gas_kick(g_gpu, frog_dt, midstep_time), "fgpu_gas_kick");
    }

    if (parameters::calculate_disk) accrete_onto_planets(data, frog_dt);
    if (parameters::disk_feedback) UpdatePlanetVelocitiesWithDiskForce(data, frog_dt);
    ps.apply_indirect_term_on_Nbody(refframe::IndirectTerm, frog_dt);
    refframe::init_corotation(data);
    ps.integrate(midstep_time, frog_dt);
    ps.copy_data_from_rebound();
    ps.move_to_hydro_center_and_update_orbital_parameters();
    corotation(data, frog_dt);

    time = end_time;
    N_hydro_iter += 1;
    logging::print_runtime_info();

    if (parameters::calculate_disk) {
	if (center_of_mass_boundary()) {
	    fgpu_frame_center c[2] = {
		frame_center(data, parameters::n_bodies_for_hydroframe_center),
		frame_center(data, ps.get_number_of_planets())};
	    gpu_check(fgpu_set_frame_centers(g_gpu, c, nullptr), "fgpu_set_frame_centers");
	}
	// the viscous recompute, the final boundary call and
	// KeepDiskMassConstant (:436-450)
	gpu_check(fgpu_apply_boundary_condition(g_gpu, end_time, step_dt, 1),
		  "fgpu_apply_boundary_condition");
	gpu_check(fgpu_recalculate_derived(g_gpu, end_time), "fgpu_recalculate_derived");
    }
}

// sim::init (simulation.cpp:462-481): the engine takes the host state that
// init_physics built, then the start-up calls run on it
void init(t_data &data)
{
    fgpu_params p = engine_params(data);
    if (const char *dump = std::getenv("FGPU_DUMP_PARAMS")) {
	if (FILE *f = std::fopen(dump, "wb")) {
	    std::fwrite(&p, sizeof p, 1, f);
	    std::fclose(f);
	}
    }
    // the radii FargoCPT built (init.cpp:93-110): Radii[0 .. nrad + 1]
    std::vector<double> radii((size_t)p.nrad + 2);
    for (int k = 0; k < p.nrad + 2; ++k) radii[(size_t)k] = Radii[k];
    gpu_check(fgpu_create(&p, radii.data(), &g_gpu), "fgpu_create");
    upload_all(data);
    if (center_of_mass_boundary()) {
	auto &ps = data.get_planetary_system();
	const unsigned int np = ps.get_number_of_planets();
	const unsigned int nc = parameters::n_bodies_for_hydroframe_center;
	double dist = 0.0;
	const bool binary = np == 2 && nc == 1;
	if (binary) {
	    const t_planet &pl = ps.get_planet(1);
	    dist = pl.get_semi_major_axis() * (1.0 + pl.get_eccentricity()) * pl.get_mass() /
		   (pl.get_mass() + ps.get_planet(0).get_mass());
	}
	gpu_check(fgpu_init_center_of_mass_boundary(g_gpu, ps.get_mass(np), ps.get_mass(nc),
						    binary ? 1 : 0, dist),
		  "fgpu_init_center_of_mass_boundary");
	fgpu_frame_center c[2] = {frame_center(data, nc), frame_center(data, np)};
	gpu_check(fgpu_set_frame_centers(g_gpu, c, nullptr), "fgpu_set_frame_centers");
    }
    fgpu_body bodies[16];
    set_bodies(collect_bodies(data, time, bodies), bodies);

    gpu_check(fgpu_apply_boundary_condition(g_gpu, time, 0.0, 0),
	      "fgpu_apply_boundary_condition");
    refframe::init_corotation(data);
    if (start_mode::mode != start_mode::mode_restart) {
	CalculateTimeStep(data);
    }
    total_disk_mass_old = 1.0;
    if (parameters::keep_mass_constant) {
	gpu_check(fgpu_gas_total_mass(g_gpu, RMAX, &total_disk_mass_old), "fgpu_gas_total_mass");
	gpu_check(fgpu_set_disk_mass_target(g_gpu, total_disk_mass_old),
		  "fgpu_set_disk_mass_target");
    }
}

static bool exit_on_signal() { return SIGTERM_RECEIVED != 0; }

// sim::run (simulation.cpp:505-558)
void run(t_data &data)
{
    double step_dt = last_dt;
    double cfl_dt = last_dt;
    init(data);
    const double t_final =
	parameters::Nsnap * parameters::Nmonitor * parameters::monitor_timestep;
    const bool iteration_restriction = options::max_iteration_number >= 0;
    for (; time < t_final;) {
	if (iteration_restriction &&
	    N_hydro_iter >= (long unsigned int)options::max_iteration_number) {
	    break;
	}
	if (exit_on_signal()) {
	    download_all(data);
	    output::write_full_output(data, "autosave");
	    break;
	}
	cfl_dt = CalculateTimeStep(data);
	const double time_next_monitor = (N_monitor + 1) * parameters::monitor_timestep;
	const double time_left_till_write = time_next_monitor - time;
	const bool overshoot = cfl_dt > time_left_till_write;
	const bool almost_there = time_left_till_write < cfl_dt * (1 + 0.05);
	step_dt = (overshoot || almost_there) ? time_left_till_write : cfl_dt;
	if (parameters::hydro_integrator == LEAPFROG_INTEGRATOR)
	    step_LeapFrog(data, step_dt);
	else
	    step_Euler(data, step_dt);
	if (std::fabs(time_next_monitor - time) < 1e-6 * cfl_dt) {
	    N_monitor++;
	    handle_outputs(data);
	    logging::print_runtime_info();
	}
    }
    logging::print_runtime_final();
    download_all(data);
    gpu_check(fgpu_destroy(g_gpu), "fgpu_destroy");
    g_gpu = nullptr;
}

} // namespace sim
