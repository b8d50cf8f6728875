/*
 * fargocpt_gb300 — C ABI of the GB300 (sm_103a) engine for FargoCPT's
 * per-timestep gas-hydrodynamics step on the 2D polar staggered grid.
 *
 * The engine owns every hydro field in HBM.  The caller (FargoCPT's C++
 * driver, or any host that keeps the N-body system, configuration and I/O)
 * hands in planet positions and scalars each step and reads back dt and
 * disk-on-planet forces; whole fields cross the boundary only on request
 * (initialisation, snapshots, restarts).
 *
 * Layout contract (identical to FargoCPT's t_polargrid, src/polargrid.h:111-133):
 *   row-major double, ring-major: cell(nr, naz) = naz + nr * naz_count,
 *   azimuth contiguous.  Scalar grids have nrad rows, vector grids
 *   (V_RADIAL, V_RADIAL0, TAU_R_PHI) have nrad + 1 rows.  nrad counts the two
 *   ghost rings exactly like FargoCPT's "Nrad" key (src/init.cpp:93-100).
 *
 * Every entry point returns FGPU_OK (0) or a negative fgpu_status; the text of
 * the last error of a handle is available from fgpu_last_error().  A handle is
 * not thread-safe; all of its work is ordered on one CUDA stream.
 */
#ifndef FARGOCPT_GB300_H
#define FARGOCPT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FGPU_ABI_VERSION 2

typedef enum fgpu_status {
    FGPU_OK = 0,
    FGPU_ERR_BAD_ARG = -1,   /* invalid handle, size, enum or option      */
    FGPU_ERR_OOM = -2,       /* device allocation failed                  */
    FGPU_ERR_CUDA = -3,      /* a CUDA call failed (text in last_error)   */
    FGPU_ERR_UNSUPPORTED = -4, /* option outside the GPU path's scope     */
    FGPU_ERR_NONFINITE = -5, /* NaN/Inf found by fgpu_check_finite        */
    FGPU_ERR_NO_DEVICE = -6  /* no CUDA device or the kernels are absent  */
} fgpu_status;

/* Fields, named after FargoCPT's t_data::t_polargrid_type (src/data.h:17-86). */
typedef enum fgpu_field {
    FGPU_SIGMA = 0,
    FGPU_V_RADIAL = 1,      /* vector grid: nrad + 1 rows */
    FGPU_V_AZIMUTHAL = 2,
    FGPU_ENERGY = 3,
    FGPU_SIGMA0 = 4,        /* damping / reference values */
    FGPU_V_RADIAL0 = 5,     /* vector grid */
    FGPU_V_AZIMUTHAL0 = 6,
    FGPU_ENERGY0 = 7,
    FGPU_SOUNDSPEED = 8,
    FGPU_SCALE_HEIGHT = 9,
    FGPU_PRESSURE = 10,
    FGPU_TEMPERATURE = 11,
    FGPU_VISCOSITY = 12,
    FGPU_QPLUS = 13,
    FGPU_QMINUS = 14,
    FGPU_POTENTIAL = 15,
    FGPU_DIV_V = 16,
    FGPU_TAU_R_R = 17,
    FGPU_TAU_PHI_PHI = 18,
    FGPU_TAU_R_PHI = 19,    /* vector grid */
    FGPU_Q_R = 20,
    FGPU_Q_PHI = 21,
    FGPU_FIELD_COUNT = 22
} fgpu_field;

/* Per-field ghost-ring boundary hooks (src/boundary_conditions/config.cpp:86-330). */
typedef enum fgpu_bc {
    FGPU_BC_NONE = 0,
    FGPU_BC_ZEROGRADIENT = 1,  /* zero_gradient.cpp:39-90 */
    FGPU_BC_OUTFLOW = 2,       /* outflow.cpp:16-57 (v_radial only) */
    FGPU_BC_REFERENCE = 3,     /* reference.cpp:17-88 */
    FGPU_BC_KEPLERIAN = 4,     /* keplerian_azimuthal.cpp:18-59 (v_azimuthal only) */
    FGPU_BC_DISKMODEL = 5,     /* diskmodel.cpp:18-77 (sigma, energy) */
    FGPU_BC_REFLECTING = 6,    /* reflecting.cpp:15-40 (v_radial) */
    FGPU_BC_VISCOUS = 7,       /* viscous.cpp:15-40 (v_radial, inner edge only: the
                                  outer version reads one ring past the viscosity
                                  grid, viscous.cpp:46-66, and is refused) */
    FGPU_BC_KEPLERIAN_RADIAL = 8, /* keplerian_radial.cpp:17-62 (v_radial) */
    FGPU_BC_ZEROSHEAR = 9,     /* zero_shear.cpp:19-53 (v_azimuthal) */
    FGPU_BC_BALANCED = 10      /* balanced.cpp:20-94 (v_azimuthal; no self-gravity) */
} fgpu_bc;

/* Damping kinds (src/boundary_conditions/boundary_conditions.h:93-99). */
typedef enum fgpu_damping {
    FGPU_DAMP_NONE = 0,
    FGPU_DAMP_REFERENCE = 1,   /* damping.cpp:311-427 */
    FGPU_DAMP_ZERO = 2,        /* damping.cpp:429-549 */
    FGPU_DAMP_MEAN = 3         /* damping.cpp:551-617, 682-752 */
} fgpu_damping;

/* Index of a damped quantity in fgpu_params.damping_inner/outer, in the order
 * of FargoCPT's damping_vector (damping.cpp:214-271). */
enum { FGPU_DQ_VRAD = 0, FGPU_DQ_VAZI = 1, FGPU_DQ_SIGMA = 2, FGPU_DQ_ENERGY = 3 };

enum { FGPU_EOS_ISOTHERMAL = 0, FGPU_EOS_IDEAL = 1 };
enum { FGPU_SPACING_ARITHMETIC = 0, FGPU_SPACING_LOGARITHMIC = 1 };
enum { FGPU_ARTVISC_NONE = 0, FGPU_ARTVISC_SN = 1, FGPU_ARTVISC_TW = 2 };
enum { FGPU_LIMITER_VANLEER = 0, FGPU_LIMITER_MC = 1 };
enum { FGPU_BETA_REF_ZERO = 0, FGPU_BETA_REF_REFERENCE = 1,
       FGPU_BETA_REF_DISKMODEL = 2, FGPU_BETA_REF_FLOOR = 3 };
/* FGPU_PRECISION_FP64: FargoCPT's FP64 fields and FP64 state updates; the
 * kernels compute in float pairs (48 significant bits) unless the environment
 * variable FARGO_GB300_FP64_ARITH is "fp64" when fgpu_create runs (then in
 * FP64; "pair" or unset: pairs; any other value: FGPU_ERR_BAD_ARG).
 * FGPU_PRECISION_FP32_MIXED: FP32 fields in HBM (v_phi and the potential
 * relative to the Keplerian disk), FargoCPT's FP64 fields on upload and
 * download. */
enum { FGPU_PRECISION_FP64 = 0, FGPU_PRECISION_FP32_MIXED = 1 };
enum { FGPU_INTEGRATOR_EULER = 0, FGPU_INTEGRATOR_LEAPFROG = 1 };
/* composite boundaries (boundary_conditions/config.cpp:344-430): "individual"
 * composites run the per-field hooks; "centerofmass" imposes the initial disk
 * model about the centre of mass of the bodies on that edge's ghost ring and,
 * with damping on, damps towards it (center_of_mass.cpp); the per-field hooks
 * of that edge should then be FGPU_BC_NONE and its damping kinds none. */
enum { FGPU_COMPOSITE_INDIVIDUAL = 0, FGPU_COMPOSITE_CENTER_OF_MASS = 1 };

/*
 * Flat parameter block: the subset of FargoCPT's parameters:: namespace and
 * globals that the hydro step reads, already converted to code units by the
 * caller (src/parameters.cpp, src/Interpret.cpp, src/constants.cpp).
 */
typedef struct fgpu_params {
    int nrad;               /* Nrad incl. 2 ghost rings (parameters.cpp:506) */
    int naz;                /* Naz (parameters.cpp:507) */
    int eos;                /* FGPU_EOS_* (Interpret.cpp:398-460) */
    int art_visc;           /* FGPU_ARTVISC_* (parameters.cpp:637-655) */
    int art_visc_dissipation;
    int flux_limiter;       /* FGPU_LIMITER_* (TransportEuler.cpp:306-337) */
    int fast_transport;     /* 1: FARGO (Interpret.cpp:158-171) */
    int heating_viscous;    /* HeatingViscous (parameters.cpp:560) */
    int cooling_beta;       /* CoolingBetaLocal (parameters.cpp:439) */
    int cooling_beta_reference; /* FGPU_BETA_REF_* (parameters.cpp:451-463) */
    int damping;            /* Damping (damping.cpp:188) */
    int damping_inner[4];   /* FGPU_DAMP_* per FGPU_DQ_* */
    int damping_outer[4];
    int bc_sigma_inner, bc_sigma_outer;   /* FGPU_BC_* */
    int bc_energy_inner, bc_energy_outer;
    int bc_vrad_inner, bc_vrad_outer;
    int bc_vaz_inner, bc_vaz_outer;
    int precision;          /* FGPU_PRECISION_* */
    int integrator;         /* FGPU_INTEGRATOR_* (Interpret.cpp:174-185); LeapFrog
                               scales three CFL limits by 0.6 (cfl.cpp:254-317) */
    int stabilize_viscosity; /* StabilizeViscosity (Interpret.cpp:669-681): 0 off,
                               1 pseudo-implicit viscous update, 2 viscous dt limit
                               (viscosity.cpp:256-348, 395-417; cfl.cpp:332-351);
                               not in the batched form */
    int profile_cutoff_outer; /* ProfileCutoffOuter (parameters.cpp:730): balanced
                                 boundary without pressure support */
    int viscous_accretion;  /* a planet accretes with the viscous profile
                               (planetary_system.cpp:255-257); with it, or with the
                               viscous v_radial hook, c_s, H and nu are recomputed
                               before the final boundary call (simulation.cpp:232-242,
                               432-441; Interpret.cpp:704-707) */
    int composite_inner;    /* FGPU_COMPOSITE_* (InnerBoundary, config.cpp:344-380) */
    int composite_outer;    /* FGPU_COMPOSITE_* (OuterBoundary, config.cpp:384-430) */
    int initialize_pure_keplerian; /* InitializePureKeplerian (parameters.cpp:568):
                                      the centre-of-mass model disk is Keplerian */
    int initialize_vradial_zero;   /* InitializeVradialZero (parameters.cpp:570) */
    int profile_cutoff_inner;      /* ProfileCutoffInner (parameters.cpp:738) */
    int keep_disk_mass_constant;   /* KeepDiskMassConstant (parameters.cpp:660-661): after
                                      every final boundary call sigma is rescaled to the
                                      mass given to fgpu_set_disk_mass_target
                                      (simulation.cpp:246-251, 445-450) */

    double gamma;           /* AdiabaticIndex */
    double mu;              /* mean molecular weight */
    double aspect_ratio;    /* AspectRatio h0 */
    double flaring_index;   /* FlaringIndex */
    double viscous_alpha;   /* ViscousAlpha (> 0 selects alpha viscosity) */
    double constant_viscosity; /* used when viscous_alpha <= 0 */
    double art_visc_factor; /* ArtificialViscosityFactor */
    double radial_viscosity_factor;
    double heating_viscous_factor;
    double cfl;             /* CFL */
    double cfl_max_var;     /* CFLmaxVar */
    double heating_cooling_cfl_limit;
    double sigma0;          /* Sigma0 */
    double sigma_floor;     /* SigmaFloor (multiples of sigma0) */
    double thickness_smoothing; /* ThicknessSmoothing */
    double cooling_beta_value;  /* CoolingBeta */
    double cooling_beta_ramp_up;/* CoolingBetaRampUp */
    double minimum_temperature; /* code units */
    double maximum_temperature; /* code units */
    double G;               /* constants::G in code units */
    double R_gas;           /* constants::R in code units */
    double sigma_sb;        /* constants::sigma in code units */
    double c_light;         /* constants::c in code units */
    double hydro_center_mass;
    double damping_inner_limit;
    double damping_outer_limit;
    double damping_time_factor;
    double damping_time_radius_outer;
    double vaz_inner_keplerian_factor;
    double vaz_outer_keplerian_factor;
    double rmin, rmax;      /* RMIN, RMAX */
    int radial_spacing;     /* FGPU_SPACING_* (used for damping ring search) */
    int correct_disk_selfgravity; /* CorrectDiskSelfgravity (parameters.cpp:699; FargoCPT's
                                     default 1 without self-gravity): the disk force on a
                                     body uses sigma less its ring mean (Force.cpp:64-66) */
    double accretion_radius_fraction; /* MassAccretionRadius (parameters.cpp:789-790,
                                         FargoCPT's default 1.0) */
    double sigma_slope;     /* SigmaSlope (Interpret.cpp:88): disk-model and balanced
                               boundaries */
    double viscous_outflow_speed; /* ViscousOutflowSpeed (config.cpp:498, default 1) */
    double vrad_inner_keplerian_factor; /* InnerBoundaryVradKeplerianFactor (config.cpp:220,
                                           default 0.1) */
    double vrad_outer_keplerian_factor; /* OuterBoundaryVradKeplerianFactor (default 0.1) */
    double binary_quadrupole_moment;    /* Theo.cpp:74 when
                                           VazimuthalConsidersQuadropoleMoment is set,
                                           else 0 (balanced and centre-of-mass
                                           boundaries) */
    double profile_cutoff_point_outer, profile_cutoff_width_outer; /* parameters.cpp:732-735 */
    double profile_cutoff_point_inner, profile_cutoff_width_inner; /* parameters.cpp:740-743 */
    double temperature_cgs_to_code; /* units::temperature.get_cgs_to_code_factor(): the
                                       centre-of-mass boundary scales its temperature
                                       floor by it once more (center_of_mass.cpp:196-200) */
    double reserved_d[2];
} fgpu_params;

/* One N-body object as the gas sees it (src/Pframeforce.cpp:24-35). */
typedef struct fgpu_body {
    double x, y;            /* position in the hydro frame */
    double mass;            /* ramped mass, t_planet::get_rampup_mass(t) */
    double r_sm;            /* Klahr cubic smoothing radius
                               (roche radius * distance * factor), 0 = off */
    double a;               /* distance from the origin, t_planet::get_r() */
} fgpu_body;

typedef struct fgpu_engine fgpu_engine;

/* Fills radii[0 .. nrad + 1] with the interface radii FargoCPT builds in
 * init_radialarrays (src/init.cpp:93-110): Radii[n] for n = 0 .. nrad + 1.
 * Host-only helper; needs no device. */
int fgpu_grid_radii(int spacing, double rmin, double rmax, int nrad,
		    double *radii);

/* Creates an engine on the current CUDA device.  radii: nrad + 2 values
 * (FargoCPT's Radii[0 .. nrad + 1]).  Replaces the allocations of
 * t_data::set_size (src/data.cpp), InitTransport (src/TransportEuler.cpp:57)
 * and init_radialarrays (src/init.cpp:178-225). */
int fgpu_create(const fgpu_params *params, const double *radii,
		fgpu_engine **out);
int fgpu_destroy(fgpu_engine *eng);
const char *fgpu_last_error(const fgpu_engine *eng);
/* CUDA stream (cudaStream_t) that orders all work of the handle. */
int fgpu_get_stream(const fgpu_engine *eng, void **stream);

/* Host <-> device copies of whole fields; rows must be the field's row count
 * (nrad or nrad + 1) and cols == naz.  Synchronous with respect to the host. */
int fgpu_upload_field(fgpu_engine *eng, int field, const double *host,
		      int rows, int cols);
int fgpu_download_field(fgpu_engine *eng, int field, double *host, int rows,
			int cols);

/* Per-step N-body state seen by the gas: bodies[0] is the central object.
 * indirect_x/y: refframe::IndirectTerm (src/frame_of_reference.cpp:166-170);
 * omega_frame: refframe::OmegaFrame.  Replaces the g_xpl/g_ypl/g_mpl set-up of
 * CalculateNbodyPotential (src/Pframeforce.cpp:24-35). */
int fgpu_set_bodies(fgpu_engine *eng, int n, const fgpu_body *bodies,
		    double indirect_x, double indirect_y, double omega_frame);

/* init_euler (src/SourceEuler.cpp:251-285): derived quantities (c_s, P, T, H,
 * nu) and the heating/cooling rates the first CFL call reads
 * (compute_heating_cooling_for_CFL, src/SourceEuler.cpp:1410-1450). */
int fgpu_init_euler(fgpu_engine *eng, double t);

/* recalculate_derived_disk_quantities (src/SourceEuler.cpp:225-249). */
int fgpu_recalculate_derived(fgpu_engine *eng, double t);

/* cfl::condition_cfl (src/cfl.cpp:185-382): the global CFL time step. */
int fgpu_condition_cfl(fgpu_engine *eng, double *dt_out);

/* boundary_conditions::apply_boundary_condition
 * (src/boundary_conditions/boundary_conditions.cpp:65-114). */
int fgpu_apply_boundary_condition(fgpu_engine *eng, double t, double dt,
				  int final);

/* The gas part of sim::step_Euler (src/simulation.cpp:170-265):
 * CalculateNbodyPotential, update_with_sourceterms,
 * update_with_artificial_viscosity, recalculate_viscosity,
 * compute_viscous_stress_tensor, update_velocities_with_viscosity, SubStep3,
 * apply_boundary_condition(final=false), Transport,
 * apply_boundary_condition(final=true), recalculate_derived_disk_quantities.
 * t is sim::time at the start of the step.  Asynchronous. */
int fgpu_step_euler(fgpu_engine *eng, double dt, double t);

/* ComputeDiskOnPlanetAccel (src/Force.cpp:23-122) for body k: accel[0..1]
 * receive the x/y acceleration of the disk on the body. */
int fgpu_disk_on_planet_accel(fgpu_engine *eng, int k, double accel[2]);

/* ComputeDiskOnNbodyAccel (src/Pframeforce.cpp:194-220): the disk force on
 * every body of the last fgpu_set_bodies (ComputeDiskOnPlanetAccel each,
 * Force.cpp:23-122), accel[2k], accel[2k + 1] for body k; all bodies are
 * computed before one read-back (one host synchronisation per call). */
int fgpu_disk_on_nbody_accel(fgpu_engine *eng, double *accel);

/* quantities::gas_total_mass (src/quantities.cpp:51-74) over the active rings. */
int fgpu_total_mass(fgpu_engine *eng, double *mass);

/* quantities::gas_total_mass (src/quantities.cpp:51-74) and
 * quantities::gas_angular_momentum (src/quantities.cpp:242-276) over the
 * active rings whose Rmed <= radius, as the monitor output asks for them
 * (output.cpp:380-390).  Per-ring partial sums in FP64, added across rings
 * with Kahan compensation in a fixed order (both forms). */
int fgpu_gas_total_mass(fgpu_engine *eng, double radius, double *mass);
int fgpu_gas_angular_momentum(fgpu_engine *eng, double radius, double *momentum);

/* KeepDiskMassConstant: the mass sigma is rescaled to after each final
 * boundary call, FargoCPT's total_disk_mass_old (gas_total_mass at RMAX in
 * sim::init, simulation.cpp:476-480).  Needed before the first step when
 * fgpu_params.keep_disk_mass_constant is set; a step or final boundary call
 * without it returns FGPU_ERR_BAD_ARG. */
int fgpu_set_disk_mass_target(fgpu_engine *eng, double mass);

/* Accretion kinds of t_planet (src/nbody/planet.h:6-9). */
enum { FGPU_ACCRETION_KLEY = 0, FGPU_ACCRETION_VISCOUS = 1, FGPU_ACCRETION_SINKHOLE = 2 };

/* One accreting planet as accretion::AccreteOntoPlanets reads it
 * (src/accretion.cpp:84-480); the host's t_planet supplies every value. */
typedef struct fgpu_accretor {
    int type;               /* FGPU_ACCRETION_* (t_planet::get_accretion_type) */
    int reserved;
    double x, y;            /* get_x(), get_y() */
    double r, phi;          /* get_r(), get_phi() (planet.cpp:159-160) */
    double roche_radius;    /* get_dimensionless_roche_radius() *
                               get_distance_to_primary() */
    double efficiency;      /* get_accretion_efficiency() */
    double orbital_period;  /* get_orbital_period() */
} fgpu_accretor;

/* One planet's part of accretion::AccreteOntoPlanets (src/accretion.cpp:84-480,
 * Kley's two zones, the sink hole, or the viscous profile): removes gas, and
 * energy with it, from the cells around the planet, down to the density
 * floor, and returns in out[0 .. 2] the mass and the x/y momentum taken from
 * the active rings.  The host adds them to the planet (update_planet,
 * accretion.cpp:60-82) and its accreted-mass monitor.  Call it for each
 * accreting planet where step_Euler / step_LeapFrog call AccreteOntoPlanets
 * (simulation.cpp:150-153, 301-304, 402-405).  In the FP32-mixed form the
 * removal acts on the compensated sigma pair and the sums are formed in FP64. */
int fgpu_accrete_onto_planet(fgpu_engine *eng, const fgpu_accretor *a, double dt,
			     double out[3]);

/* The centre of a set of bodies as the centre-of-mass boundary reads it from
 * the planetary system (nbody/planetary_system.cpp:580-650). */
typedef struct fgpu_frame_center {
    double x, y;            /* get_center_of_mass(n) */
    double vx, vy;          /* get_center_of_mass_velocity(n) */
    double mass;            /* get_mass(n) */
} fgpu_frame_center;

/* init_center_of_mass (center_of_mass.cpp:25-27): builds the viscous-speed
 * lookup tables of viscous_speed::init_vr_table_boundary
 * (viscosity/viscous_radial_speed.cpp:269-347) for both edges.  mass_all is
 * get_mass() of all bodies, mass_center get_mass(n_bodies_for_hydroframe_center);
 * binary_on_primary is 1 when the system has two bodies and the hydro frame is
 * centred on the first, and com_max_dist is then a (1 + e) q of the second
 * (q = m2 / (m1 + m2)).  Call it once after fgpu_create when a composite is
 * FGPU_COMPOSITE_CENTER_OF_MASS. */
int fgpu_init_center_of_mass_boundary(fgpu_engine *eng, double mass_all, double mass_center,
				      int binary_on_primary, double com_max_dist);

/* The centres each boundary call uses: c[0] of the first
 * n_bodies_for_hydroframe_center bodies (inner edge), c[1] of all bodies
 * (outer edge).  now[] serves fgpu_apply_boundary_condition and the boundary
 * call before transport in fgpu_step_euler; after[] (NULL: now[]) serves the
 * final call of fgpu_step_euler, which FargoCPT makes after the N-body step
 * (simulation.cpp:219-244). */
int fgpu_set_frame_centers(fgpu_engine *eng, const fgpu_frame_center now[2],
			   const fgpu_frame_center *after);

/* correct_v_azimuthal (src/SideEuler.cpp:79-95): v_phi -= dOmega * Rmed on
 * every ring, ghost rings included.  refframe::handle_corotation
 * (src/frame_of_reference.cpp:30-60) calls it when the corotating frame's
 * OmegaFrame changes by dOmega, before the gas step; the engine then takes the
 * new OmegaFrame through fgpu_set_bodies.  Not for the disks of a batch
 * (fixed frame). */
int fgpu_correct_v_azimuthal(fgpu_engine *eng, double domega);

/* The cell that limits the CFL time step, as FargoCPT's SIGUSR1 report
 * (timestep_debug_report, src/cfl.cpp:38-182) names it: ring and azimuth of
 * the smallest cell time step (the first in ring-major order on ties), that
 * time step, its six inverse times (sound speed, radial and azimuthal
 * transport, artificial viscosity, viscosity, heating/cooling; after
 * LeapFrog's factor) and the smallest ring shear limit with its ring.  The
 * step FargoCPT takes is the smaller of dt_cell and dt_shear (before
 * CFLmaxVar).  FP64 form only; a diagnostic, it allocates. */
typedef struct fgpu_cfl_cell {
    int ring, azimuth;
    int shear_ring, reserved;
    double dt_cell;
    double invdt[6];
    double dt_shear;
} fgpu_cfl_cell;

int fgpu_cfl_limiting_cell(fgpu_engine *eng, fgpu_cfl_cell *out);

/* Scans the evolved fields for NaN/Inf; returns FGPU_ERR_NONFINITE and the
 * first bad (field, ring, azimuth) when one is found. */
int fgpu_check_finite(fgpu_engine *eng, int *field, int *nr, int *naz);

/* Blocks until all queued work of the handle is done. */
int fgpu_synchronize(fgpu_engine *eng);

/* Phase timing (no counterpart in the reference, whose only timer is the
 * wall clock per step, src/logging.cpp:179-201): when enabled, every
 * fgpu_step_euler records CUDA events between its kernels on the handle's
 * stream.  fgpu_phase_times waits for the recorded steps, writes the summed
 * milliseconds of each phase into ms[0 .. count-1] (count = number of
 * phases, at most capacity), the number of steps into *steps, and clears the
 * record.  fgpu_phase_name(k) names phase k. */
int fgpu_set_phase_timing(fgpu_engine *eng, int enable);
int fgpu_phase_times(fgpu_engine *eng, double *ms, int capacity, int *count,
		     int *steps);
const char *fgpu_phase_name(int k);

/* Asynchronous snapshots (the payload of FargoCPT's write2D,
 * src/polargrid.cpp:135-180: every row of the grid, row-major FP64, the
 * FP32-mixed form converted back to FargoCPT's values).  fgpu_snapshot_begin
 * copies fields[0 .. n-1] into device staging buffers in order with the
 * steps, then copies them to host[k] (rows x naz doubles each) on a second
 * stream, so the steps that follow run while the copy drains; host[k] must
 * stay valid until fgpu_snapshot_wait returns.  One snapshot is in flight at
 * a time (begin waits for the previous one).  Page-locked buffers from
 * fgpu_host_alloc copy at full speed.  No counterpart in the reference, whose
 * output stops the run while it writes (src/output.cpp:249-304). */
int fgpu_snapshot_begin(fgpu_engine *eng, int n, const int *fields, double *const *host);
int fgpu_snapshot_wait(fgpu_engine *eng);
int fgpu_host_alloc(size_t bytes, void **ptr);
int fgpu_host_free(void *ptr);

/* The phases of the step, for hosts that compose their own integrator
 * (step_LeapFrog, src/simulation.cpp:276-459, kicks with dt/2 around one
 * transport over dt):
 *   fgpu_gas_kick       potential, update_with_sourceterms, artificial
 *                       viscosity, recalculate_viscosity, stress tensor,
 *                       update_velocities_with_viscosity, SubStep3 (the gas
 *                       kick, :312-331 and :352-384), with the bodies of the
 *                       last fgpu_set_bodies; t is the time the kick sees;
 *   fgpu_transport      Transport (TransportEuler.cpp) over dt;
 *   fgpu_compute_pressure  compute_pressure (SourceEuler.cpp:1345-1376).
 * fgpu_step_euler is gas_kick(dt, t), the non-final boundary condition,
 * transport(dt), the final boundary condition and the derived quantities. */
int fgpu_gas_kick(fgpu_engine *eng, double dt, double t);
int fgpu_transport(fgpu_engine *eng, double dt);
int fgpu_compute_pressure(fgpu_engine *eng);

/* Disk-on-body force and gas mass without any device allocation.  No
 * counterpart in the reference: it serves callers that keep sigma and the
 * scale height in their own device buffers and may not allocate device
 * memory when they ask for the force (fixed memory budgets, allocation-free
 * hot paths, code that must not synchronise the device).  The per-ring
 * partial sums live in a static device array of 16384 rings (FargoCPT's
 * MAX1D), so nrad - 2 must not exceed 16384; larger grids get
 * FGPU_ERR_BAD_ARG.  sigma, scale_height: device, nrad x naz; radii: device,
 * nrad + 2 values; out: device, 5 doubles (inner x, inner y, outer x, outer y
 * acceleration, gas mass of the active rings).  The force uses sigma less its
 * ring mean, as FargoCPT's CorrectDiskSelfgravity (its default without
 * self-gravity) does.  The first call on a device looks up the array's
 * address; make it before any stream capture.  All calls share the array:
 * calls that overlap on the GPU race.  A CUDA error left pending by the
 * caller is reported as FGPU_ERR_CUDA and left pending. */
int fgpu_disk_force_static(const double *sigma, const double *scale_height,
			   const double *radii, int nrad, int naz, double G,
			   double thickness_smoothing, const fgpu_body *body,
			   double *out, void *stream);

/* ------------------------------------------------------------------------
 * Batched many-disk form.  No counterpart in the reference, which runs one
 * disk per process (src/main.cpp); a parameter sweep there is many runs.  A
 * batch holds n independent FP32-mixed disks of any sizes; every phase of
 * the step is one grid-stride launch over all disks, each disk with its own
 * dt.  The per-disk handles of fgpu_batch_disk take every single-disk call
 * (upload, download, bodies, init_euler, CFL, boundary, force, mass,
 * finiteness) and share the batch's stream; they belong to the batch
 * (fgpu_destroy refuses them).
 * ---------------------------------------------------------------------- */
typedef struct fgpu_batch fgpu_batch;

/* Tile shape of one batched kernel: threads per block and, for the per-cell
 * kernels, rings per block (cells per thread along the radius); for the
 * radial transport, rings one thread walks.  Ring kernels (azimuthal
 * transport, damping, CFL) use one block per ring; their cells per thread
 * follow from threads and the longest ring. */
typedef struct {
	int threads;
	int rings;
} fgpu_tile;

enum fgpu_batch_kernel {
	FGPU_BK_POTENTIAL = 0,
	FGPU_BK_SOURCE,
	FGPU_BK_ARTVISC_Q,
	FGPU_BK_ARTVISC_V,
	FGPU_BK_STRESS,
	FGPU_BK_VISCOUS,
	FGPU_BK_GHOST,
	FGPU_BK_TRANSPORT_RADIAL,
	FGPU_BK_TRANSPORT_AZIMUTHAL,
	FGPU_BK_FINISH,
	FGPU_BK_DAMPING,
	FGPU_BK_DERIVED_CFL,
	FGPU_BK_COUNT
};

typedef struct {
	fgpu_tile k[FGPU_BK_COUNT];
} fgpu_tiles;

/* Device-side run clock of one disk: FargoCPT's CalculateTimeStep
 * (src/simulation.cpp:100-118) and the monitor-time clamp of sim::run
 * (:505-558), evaluated on the GPU so that a captured sequence of steps needs
 * no host round trip.  The star (star_mass, at the origin) holds n_planets
 * planets on circular orbits: planet k at radius a[k], angular speed
 * sqrt(G (star_mass + mass[k]) / a^3), initial angle phase[k]; the indirect
 * term is the one of the star-centred frame.  A disk steps while
 * time < t_end.  steps counts the steps taken; active is 1 while the disk
 * still steps. */
typedef struct {
	double time, last_dt, t_end, monitor_dt, cfl_max_var;
	double star_mass;
	int n_monitor, steps, active, n_planets;
	double mass[16], a[16], phase[16];
} fgpu_clock;

/* params[k], radii[k]: disk k as for fgpu_create; every disk must select
 * FGPU_PRECISION_FP32_MIXED and the Euler integrator (the batched step is
 * step_Euler); StabilizeViscosity, the centre-of-mass composite boundary,
 * and adiabatic disks with the viscous v_radial hook or viscous accretion,
 * are refused (FGPU_ERR_UNSUPPORTED); the longest ring must fit the
 * azimuthal transport's shared memory (naz <= 6257 with the energy equation,
 * 7040 without).  1 <= n <= 1024. */
int fgpu_batch_create(int n, const fgpu_params *params,
		      const double *const *radii, fgpu_batch **out);
int fgpu_batch_destroy(fgpu_batch *b);
const char *fgpu_batch_last_error(const fgpu_batch *b);
int fgpu_batch_size(const fgpu_batch *b, int *n);
int fgpu_batch_disk(fgpu_batch *b, int k, fgpu_engine **disk);

/* Tile shapes in use; fgpu_batch_set_tiles checks and applies them (a
 * captured step sequence is rebuilt).  fgpu_batch_autotune times candidate
 * shapes of every kernel on the batch's current state with CUDA events
 * (reps timed launches each), keeps the fastest, writes them to *best and
 * restores the state it started from. */
int fgpu_batch_get_tiles(const fgpu_batch *b, fgpu_tiles *tiles);
int fgpu_batch_set_tiles(fgpu_batch *b, const fgpu_tiles *tiles);
int fgpu_batch_autotune(fgpu_batch *b, int reps, fgpu_tiles *best);

/* How a step's substeps are launched.  FGPU_BATCH_LAUNCHES (the default):
 * one grid-stride launch over all disks per substep, each with its
 * autotuned tile shape.  FGPU_BATCH_PERSISTENT: the gas kick's substeps
 * (potential, source terms, artificial viscosity, stress, viscous update,
 * the mid-step ghost rings) as one persistent cooperative launch, the
 * closing substeps (velocities from momenta, damping, ghost rings, CFL) as
 * another, the grid synchronising between substeps (128 threads per block,
 * the autotuned rings per tile); the transports stay separate launches.
 * Both give the same bits; the persistent form is the slower on GB300 (one
 * block shape and register budget for every substep).  A captured step
 * sequence is rebuilt; FGPU_ERR_UNSUPPORTED without cooperative launch. */
enum { FGPU_BATCH_LAUNCHES = 0, FGPU_BATCH_PERSISTENT = 1 };
int fgpu_batch_set_mode(fgpu_batch *b, int mode);
int fgpu_batch_get_mode(const fgpu_batch *b, int *mode);

/* One step of every disk with host-given dt[k] and t[k] (dt[k] = 0 skips
 * disk k) and the bodies last given to each disk's handle: fgpu_step_euler
 * of all disks at once. */
int fgpu_batch_step(fgpu_batch *b, const double *dt, const double *t);

/* Device clock: set or read disk k's clock.  fgpu_batch_run advances every
 * disk by up to max_steps steps with its own CFL dt, stopping disks at
 * their t_end, as CUDA graphs of steps_per_graph steps (captured once and
 * relaunched); *n_active receives the number of disks still below t_end.
 * Before the first run the disks need their initial state, init_euler and
 * a valid CFL time step (fgpu_condition_cfl), as FargoCPT's start-up has. */
int fgpu_batch_set_clock(fgpu_batch *b, int k, const fgpu_clock *clock);
int fgpu_batch_get_clock(fgpu_batch *b, int k, fgpu_clock *clock);
int fgpu_batch_run(fgpu_batch *b, int max_steps, int steps_per_graph,
		   int *n_active);

#ifdef __cplusplus
}
#endif

#endif /* FARGOCPT_GB300_H */
