/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of FargoCPT's per-timestep gas step on the 2D polar
 * staggered grid (reference: rometsch/fargocpt src/), used only as the
 * checker by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm.  The GPU engine never links or calls it.
 *
 * Parity pin: this restatement is checked field by field against snapshots of
 * the reference itself (built from its own sources by oracle/ref/Makefile and
 * run by tests/golden/make_golden.py); the fixtures live in tests/golden/.
 *
 * The state mirrors t_data: every field is a row-major double array,
 * cell(nr, naz) = naz + nr * naz_count; vector grids have nrad + 1 rows.
 */
#ifndef FARGO_ORACLE_H
#define FARGO_ORACLE_H

#include "../include/fargocpt_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_state or_state;

int or_create(const fgpu_params *p, const double *radii, or_state **out);
void or_destroy(or_state *s);
int or_field_rows(const or_state *s, int field);
int or_set_field(or_state *s, int field, const double *src, int rows, int cols);
int or_get_field(const or_state *s, int field, double *dst, int rows, int cols);
int or_set_bodies(or_state *s, int n, const fgpu_body *b, double ix, double iy,
		  double omega_frame);
int or_set_threads(int n);

int or_init_euler(or_state *s, double t);
int or_recalculate_derived(or_state *s, double t);
double or_condition_cfl(or_state *s);
int or_apply_boundary_condition(or_state *s, double t, double dt, int final);
int or_step_euler(or_state *s, double dt, double t);
void or_gas_kick(or_state *s, double dt, double t);
void or_compute_pressure(or_state *s);
int or_disk_on_planet_accel(or_state *s, int k, double accel[2]);
double or_total_mass(or_state *s);
double or_gas_total_mass(or_state *s, double radius);
double or_gas_angular_momentum(or_state *s, double radius);
int or_set_disk_mass_target(or_state *s, double mass);
int or_accrete_onto_planet(or_state *s, const fgpu_accretor *a, double dt, double out[3]);
int or_init_center_of_mass_boundary(or_state *s, double mass_all, double mass_center,
				    int binary_on_primary, double com_max_dist);
int or_correct_v_azimuthal(or_state *s, double domega);
int or_cfl_limiting_cell(or_state *s, fgpu_cfl_cell *out);
int or_set_frame_centers(or_state *s, const fgpu_frame_center now[2],
			 const fgpu_frame_center *after);

/* Sub-steps, exported so tests can check the GPU kernels one phase at a time. */
void or_calculate_potential(or_state *s);
void or_update_with_sourceterms(or_state *s, double dt);
void or_artificial_viscosity(or_state *s, double dt);
void or_recalculate_viscosity(or_state *s, double t);
void or_viscous_stress_tensor(or_state *s);
void or_update_velocities_with_viscosity(or_state *s, double dt);
void or_substep3(or_state *s, double t, double dt);
void or_transport(or_state *s, double dt);

#ifdef __cplusplus
}
#endif

#endif
