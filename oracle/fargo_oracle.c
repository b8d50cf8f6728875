/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C restatement of the gas part of FargoCPT's sim::step_Euler
 * (reference src/simulation.cpp:148-267) and of the functions it calls.
 * Each function names the reference function and lines it restates.  The
 * loops keep the reference's order of operations so that results agree with
 * the reference's FP64 build to round-off; OpenMP parallelises the outer loops
 * the same way the reference does, which is what the CPU baseline times.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load this
 * library, and only as the checker / baseline.
 */
#include "fargo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define MAX_BODIES 16

struct or_state {
    fgpu_params p;
    int nr;  /* Nrad (scalar rows) */
    int nz;  /* Naz */
    double dphi, invdphi;

    /* radial arrays, index 0 .. nr (some read at nr) */
    double *Rinf, *Rsup, *Rmed, *Surf, *InvRmed, *InvSurf, *InvDiffRmed,
	*InvDiffRsup, *InvDiffRsupRb, *TwoDiffRaSq, *InvRinf;
    double *cosj, *sinj;

    double *f[FGPU_FIELD_COUNT];

    /* transport scratch (TransportEuler.cpp:31-52) */
    double *rmp, *rmm, *amp, *amm;
    double *vres, *vmean, *work, *qrstar, *densstar, *tempshift, *dq,
	*density_int;
    int *nshift, *nosplit;
    int uniform_transport;

    double *sigma1d;

    /* StabilizeViscosity (viscosity.cpp:256-348): nu*Sigma at cell centres
       and at the r-phi corners, and the correction factors; cleared at
       creation like every t_polargrid (polargrid.cpp:51-64) */
    double *visc_sigma, *visc_sigma_rp, *corr_phi, *corr_r;
    double *FourThirdInvRbInvdphiSq;

    /* KeepDiskMassConstant: sim::init's total_disk_mass_old
       (simulation.cpp:476-480), set by or_set_disk_mass_target */
    double mass_target;
    int mass_target_set;

    int nb;
    fgpu_body b[MAX_BODIES];
    double ix, iy, omega_frame;

    /* centre-of-mass composite boundary: viscous-speed tables (inner 0,
       outer 1; N + 1 nodes) and the centres of the two boundary calls */
    int com_ready;
    double com_min_r[2], com_dlog[2];
    double *com_r[2], *com_vr[2];
    fgpu_frame_center com_now[2], com_after[2];

    /* damping ring limits (damping.cpp:311-427), per quantity */
    int damp_limit_inner[4];
    int damp_limit_outer[4];
    int damp_active_inner[4];
    int damp_active_outer[4];
};

static int is_vector_field(int f)
{
    return f == FGPU_V_RADIAL || f == FGPU_V_RADIAL0 || f == FGPU_TAU_R_PHI;
}

int or_field_rows(const or_state *s, int field)
{
    return is_vector_field(field) ? s->nr + 1 : s->nr;
}

#define F(s, id) ((s)->f[id])
#define AT(a, i, j) (a)[(size_t)(i) * (size_t)s->nz + (size_t)(j)]

int or_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) {
	omp_set_num_threads(n);
    }
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* grid: init_radialarrays (src/init.cpp:178-225) and the damping ring */
/* search of src/find_cell_id.cpp:222-452                              */
/* ------------------------------------------------------------------ */

static int cell_id_rmed(const or_state *s, double r)
{
    const fgpu_params *p = &s->p;
    int id;
    if (p->radial_spacing == FGPU_SPACING_LOGARITHMIC) {
	/* get_rmed_id_log, find_cell_id.cpp:222-228 */
	const double g = pow(p->rmax / p->rmin, 1.0 / ((double)p->nrad - 2.0));
	const double oc = 3.0 / 2.0 / p->rmin * (1 - pow(g, 2.0)) /
			  (1 - pow(g, 3.0));
	const double ilg = 1.0 / log(g);
	double did = log(r * oc) * ilg;
	id = (int)floor(did) + 1;
    } else {
	/* get_rmed_id_arith, find_cell_id.cpp:230-238 */
	const double g = ((double)p->nrad - 2.0) / (p->rmax - p->rmin);
	double did = (r - p->rmin) * g;
	id = (int)floor(did) + 1;
	if (id >= 0 && id <= s->nr && s->Rmed[id] > r) {
	    id--;
	}
    }
    /* rmed_id_error_check with NDEBUG: clamp (find_cell_id.cpp:159-166) */
    if (id < 0) id = 0;
    if (id > s->nr - 1) id = s->nr - 1;
    return id;
}

static int cell_id_rinf(const or_state *s, double r)
{
    const fgpu_params *p = &s->p;
    int id;
    if (p->radial_spacing == FGPU_SPACING_LOGARITHMIC) {
	/* get_rinf_id_log, find_cell_id.cpp:259-264 */
	const double g = pow(p->rmax / p->rmin, 1.0 / ((double)p->nrad - 2.0));
	const double ilg = 1.0 / log(g);
	double did = log(r / p->rmin) * ilg;
	id = (int)floor(did) + 1;
    } else {
	const double g = ((double)p->nrad - 2.0) / (p->rmax - p->rmin);
	double did = (r - p->rmin) * g;
	id = (int)floor(did) + 1;
    }
    if (id < 0) id = 0;
    if (id > s->nr - 1) id = s->nr - 1;
    return id;
}

static int clamp_id(int id, int vec, int nr)
{
    /* clamp_r_id_to_rmed_grid / clamp_r_id_to_radii_grid, find_cell_id.cpp:14-38 */
    const int mx = nr - (vec ? 0 : 1);
    if (id < 0) id = 0;
    if (id > mx) id = mx;
    return id;
}

static const int dq_field[4] = {FGPU_V_RADIAL, FGPU_V_AZIMUTHAL, FGPU_SIGMA,
				FGPU_ENERGY};

static double omega_kepler(const or_state *s, double r)
{
    /* calculate_omega_kepler, src/Theo.cpp:246-249 */
    return sqrt(s->p.G * s->p.hydro_center_mass / (r * r * r));
}

static void setup_damping(or_state *s)
{
    const fgpu_params *p = &s->p;
    for (int q = 0; q < 4; ++q) {
	const int vec = is_vector_field(dq_field[q]);
	const double *radius = vec ? s->Rinf : s->Rmed;
	s->damp_active_inner[q] = (p->damping_inner_limit > 1.0) &&
				  (radius[0] < p->rmin * p->damping_inner_limit);
	if (vec) {
	    s->damp_limit_inner[q] = clamp_id(
		cell_id_rinf(s, p->rmin * p->damping_inner_limit), 1, s->nr);
	} else {
	    s->damp_limit_inner[q] = clamp_id(
		cell_id_rmed(s, p->rmin * p->damping_inner_limit), 0, s->nr);
	}
	const int maxr = vec ? s->nr : s->nr - 1;
	s->damp_active_outer[q] = (p->damping_outer_limit < 1.0) &&
				  (radius[maxr] > p->rmax * p->damping_outer_limit);
	if (vec) {
	    s->damp_limit_outer[q] = clamp_id(
		cell_id_rinf(s, p->rmax * p->damping_outer_limit) + 1, 1, s->nr);
	} else {
	    s->damp_limit_outer[q] = clamp_id(
		cell_id_rmed(s, p->rmax * p->damping_outer_limit) + 1, 0, s->nr);
	}
    }
}

int or_create(const fgpu_params *p, const double *radii, or_state **out)
{
    if (!p || !radii || !out || p->nrad < 4 || p->naz < 4) {
	return FGPU_ERR_BAD_ARG;
    }
    or_state *s = calloc(1, sizeof(*s));
    s->p = *p;
    s->nr = p->nrad;
    s->nz = p->naz;
    const int nr = s->nr, nz = s->nz;
    /* Interpret.cpp:230-231 */
    s->dphi = 2.0 * M_PI / (double)nz;
    s->invdphi = (double)nz / (2.0 * M_PI);

    const int R = nr + 2;
    double **rad[] = {&s->Rinf, &s->Rsup, &s->Rmed, &s->Surf, &s->InvRmed,
		      &s->InvSurf, &s->InvDiffRmed, &s->InvDiffRsup,
		      &s->InvDiffRsupRb, &s->TwoDiffRaSq, &s->InvRinf};
    for (size_t i = 0; i < sizeof(rad) / sizeof(rad[0]); ++i) {
	*rad[i] = calloc((size_t)R, sizeof(double));
    }
    /* init.cpp:189-225 (single rank: IMIN = 0) */
    for (int n = 0; n <= nr; ++n) {
	s->Rinf[n] = radii[n];
	s->Rsup[n] = radii[n + 1];
	s->Rmed[n] = 2.0 / 3.0 * (pow(s->Rsup[n], 3) - pow(s->Rinf[n], 3));
	s->Rmed[n] = s->Rmed[n] / (pow(s->Rsup[n], 2) - pow(s->Rinf[n], 2));
	s->Surf[n] = M_PI * (pow(s->Rsup[n], 2) - pow(s->Rinf[n], 2)) /
		     (double)nz;
	s->InvRmed[n] = 1.0 / s->Rmed[n];
	s->InvSurf[n] = 1.0 / s->Surf[n];
	s->InvDiffRsup[n] = 1.0 / (s->Rsup[n] - s->Rinf[n]);
	s->InvDiffRsupRb[n] = 1.0 / ((s->Rsup[n] - s->Rinf[n]) * s->Rmed[n]);
	s->TwoDiffRaSq[n] =
	    2.0 / (s->Rsup[n] * s->Rsup[n] - s->Rinf[n] * s->Rinf[n]);
	s->InvRinf[n] = 1.0 / s->Rinf[n];
    }
    for (int n = 1; n <= nr; ++n) {
	s->InvDiffRmed[n] = 1.0 / (s->Rmed[n] - s->Rmed[n - 1]);
    }
    s->cosj = malloc(sizeof(double) * (size_t)nz);
    s->sinj = malloc(sizeof(double) * (size_t)nz);
    for (int j = 0; j < nz; ++j) {
	/* SideEuler.cpp:56-61 */
	s->cosj[j] = cos(s->dphi * (double)j);
	s->sinj[j] = sin(s->dphi * (double)j);
    }
    for (int f = 0; f < FGPU_FIELD_COUNT; ++f) {
	s->f[f] = calloc((size_t)or_field_rows(s, f) * (size_t)nz,
			 sizeof(double));
    }
    const size_t cells = (size_t)nr * nz, vcells = (size_t)(nr + 1) * nz;
    s->rmp = calloc(cells, sizeof(double));
    s->rmm = calloc(cells, sizeof(double));
    s->amp = calloc(cells, sizeof(double));
    s->amm = calloc(cells, sizeof(double));
    s->vres = calloc(cells, sizeof(double));
    s->vmean = calloc((size_t)nr + 1, sizeof(double));
    s->work = calloc(cells, sizeof(double));
    s->qrstar = calloc(vcells, sizeof(double));
    s->densstar = calloc(vcells, sizeof(double));
    s->tempshift = calloc(cells, sizeof(double));
    s->dq = calloc(cells, sizeof(double));
    s->density_int = calloc(cells, sizeof(double));
    s->nshift = calloc((size_t)nr, sizeof(int));
    s->nosplit = calloc((size_t)nr, sizeof(int));
    s->sigma1d = calloc((size_t)nr, sizeof(double));
    s->visc_sigma = calloc(cells, sizeof(double));
    s->visc_sigma_rp = calloc(vcells, sizeof(double));
    s->corr_phi = calloc(cells, sizeof(double));
    s->corr_r = calloc(cells, sizeof(double));
    /* init.cpp:213-214 */
    s->FourThirdInvRbInvdphiSq = calloc((size_t)R, sizeof(double));
    for (int n = 0; n <= nr; ++n) {
	s->FourThirdInvRbInvdphiSq[n] = 4.0 / 3.0 / s->Rmed[n] * s->invdphi * s->invdphi;
    }
    setup_damping(s);
    *out = s;
    return FGPU_OK;
}

void or_destroy(or_state *s)
{
    if (!s) return;
    double *ptrs[] = {s->Rinf, s->Rsup, s->Rmed, s->Surf, s->InvRmed,
		      s->InvSurf, s->InvDiffRmed, s->InvDiffRsup,
		      s->InvDiffRsupRb, s->TwoDiffRaSq, s->InvRinf, s->cosj,
		      s->sinj, s->rmp, s->rmm, s->amp, s->amm, s->vres,
		      s->vmean, s->work, s->qrstar, s->densstar, s->tempshift,
		      s->dq, s->density_int, s->sigma1d, s->visc_sigma,
		      s->visc_sigma_rp, s->corr_phi, s->corr_r,
		      s->FourThirdInvRbInvdphiSq};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    for (int f = 0; f < FGPU_FIELD_COUNT; ++f) free(s->f[f]);
    for (int k = 0; k < 2; ++k) {
	free(s->com_r[k]);
	free(s->com_vr[k]);
    }
    free(s->nshift);
    free(s->nosplit);
    free(s);
}

int or_set_field(or_state *s, int field, const double *src, int rows, int cols)
{
    if (field < 0 || field >= FGPU_FIELD_COUNT || rows != or_field_rows(s, field) ||
	cols != s->nz) {
	return FGPU_ERR_BAD_ARG;
    }
    memcpy(s->f[field], src, sizeof(double) * (size_t)rows * (size_t)cols);
    return FGPU_OK;
}

int or_get_field(const or_state *s, int field, double *dst, int rows, int cols)
{
    if (field < 0 || field >= FGPU_FIELD_COUNT || rows != or_field_rows(s, field) ||
	cols != s->nz) {
	return FGPU_ERR_BAD_ARG;
    }
    memcpy(dst, s->f[field], sizeof(double) * (size_t)rows * (size_t)cols);
    return FGPU_OK;
}

int or_set_bodies(or_state *s, int n, const fgpu_body *b, double ix, double iy,
		  double omega_frame)
{
    if (n < 0 || n > MAX_BODIES) return FGPU_ERR_BAD_ARG;
    s->nb = n;
    memcpy(s->b, b, sizeof(fgpu_body) * (size_t)n);
    s->ix = ix;
    s->iy = iy;
    s->omega_frame = omega_frame;
    return FGPU_OK;
}

/* ------------------------------------------------------------------ */
/* derived quantities                                                 */
/* ------------------------------------------------------------------ */

static int adiabatic(const or_state *s) { return s->p.eos == FGPU_EOS_IDEAL; }

/* compute_sound_speed_normal, src/SourceEuler.cpp:957-995 */
static void compute_sound_speed(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *cs = F(s, FGPU_SOUNDSPEED), *E = F(s, FGPU_ENERGY),
	   *S = F(s, FGPU_SIGMA);
    const double g = s->p.gamma;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    if (adiabatic(s)) {
		AT(cs, i, j) = sqrt(g * (g - 1.0) * AT(E, i, j) / AT(S, i, j));
	    } else {
		const double vK = sqrt(s->p.G * s->p.hydro_center_mass / s->Rmed[i]);
		const double h = s->p.aspect_ratio * pow(s->Rmed[i], s->p.flaring_index);
		AT(cs, i, j) = h * vK;
	    }
	}
    }
}

/* compute_scale_height_old, src/SourceEuler.cpp:1121-1154 */
static void compute_scale_height(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *H = F(s, FGPU_SCALE_HEIGHT), *cs = F(s, FGPU_SOUNDSPEED);
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	const double inv_omega_kepler = 1.0 / omega_kepler(s, s->Rmed[i]);
	for (int j = 0; j < nz; ++j) {
	    if (adiabatic(s)) {
		AT(H, i, j) = AT(cs, i, j) / (sqrt(s->p.gamma)) * inv_omega_kepler;
	    } else {
		AT(H, i, j) = AT(cs, i, j) * inv_omega_kepler;
	    }
	}
    }
}

/* compute_pressure, src/SourceEuler.cpp:1345-1376 */
void or_compute_pressure(or_state *s)
{
    const size_t n = (size_t)s->nr * s->nz;
    double *P = F(s, FGPU_PRESSURE), *E = F(s, FGPU_ENERGY),
	   *S = F(s, FGPU_SIGMA), *cs = F(s, FGPU_SOUNDSPEED);
#pragma omp parallel for
    for (size_t c = 0; c < n; ++c) {
	if (adiabatic(s)) {
	    P[c] = (s->p.gamma - 1.0) * E[c];
	} else {
	    P[c] = S[c] * pow(cs[c], 2);
	}
    }
}

/* compute_temperature, src/SourceEuler.cpp:1378-1408 */
static void compute_temperature(or_state *s)
{
    const size_t n = (size_t)s->nr * s->nz;
    double *T = F(s, FGPU_TEMPERATURE), *E = F(s, FGPU_ENERGY),
	   *S = F(s, FGPU_SIGMA), *P = F(s, FGPU_PRESSURE);
    const double Rgas = s->p.R_gas;
#pragma omp parallel for
    for (size_t c = 0; c < n; ++c) {
	if (adiabatic(s)) {
	    const double c_v_inv = s->p.mu / Rgas * (s->p.gamma - 1.0);
	    T[c] = c_v_inv * E[c] / S[c];
	} else {
	    T[c] = s->p.mu / Rgas * P[c] / S[c];
	}
    }
}

/* viscosity::update_viscosity, src/viscosity/viscosity.cpp:98-137 */
static void update_viscosity(or_state *s)
{
    const size_t n = (size_t)s->nr * s->nz;
    double *nu = F(s, FGPU_VISCOSITY), *cs = F(s, FGPU_SOUNDSPEED),
	   *H = F(s, FGPU_SCALE_HEIGHT);
#pragma omp parallel for
    for (size_t c = 0; c < n; ++c) {
	if (s->p.viscous_alpha > 0) {
	    nu[c] = s->p.viscous_alpha * H[c] * cs[c];
	} else {
	    nu[c] = s->p.constant_viscosity;
	}
    }
}

/* assure_temperature_range, src/SourceEuler.cpp:136-202 */
static void assure_temperature_range(or_state *s)
{
    const size_t n = (size_t)s->nr * s->nz;
    double *E = F(s, FGPU_ENERGY), *S = F(s, FGPU_SIGMA);
    const double mu = s->p.mu, g = s->p.gamma, R = s->p.R_gas;
    const double Tmin = s->p.minimum_temperature, Tmax = s->p.maximum_temperature;
#pragma omp parallel for
    for (size_t c = 0; c < n; ++c) {
	const double emin = Tmin * S[c] / mu * R / (g - 1.0);
	const double emax = Tmax * S[c] / mu * R / (g - 1.0);
	if (!(E[c] > emin)) {
	    E[c] = Tmin * S[c] / mu * R / (g - 1.0);
	}
	if (!(E[c] < emax)) {
	    E[c] = Tmax * S[c] / mu * R / (g - 1.0);
	}
    }
}

/* calculate_qminus (beta cooling only), src/SourceEuler.cpp:632-690, 830-852 */
static void calculate_qminus(or_state *s, double t)
{
    const int nr = s->nr, nz = s->nz;
    double *Qm = F(s, FGPU_QMINUS), *E = F(s, FGPU_ENERGY), *S = F(s, FGPU_SIGMA),
	   *S0 = F(s, FGPU_SIGMA0), *E0 = F(s, FGPU_ENERGY0);
    memset(Qm, 0, sizeof(double) * (size_t)nr * nz);
    if (!s->p.cooling_beta) return;
#pragma omp parallel for
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double r = s->Rmed[i];
	    const double omega_k = omega_kepler(s, r);
	    const double Ev = AT(E, i, j);
	    const double t_ramp_up = s->p.cooling_beta_ramp_up;
	    double beta_inv = 1 / s->p.cooling_beta_value;
	    if (t_ramp_up > 0.0) {
		double ramp = 1 - exp(-pow(2 * t / t_ramp_up, 2));
		beta_inv = beta_inv * ramp;
	    }
	    double delta_E = Ev;
	    if (s->p.cooling_beta_reference == FGPU_BETA_REF_REFERENCE) {
		delta_E -= AT(E0, i, j) / AT(S0, i, j) * AT(S, i, j);
	    } else if (s->p.cooling_beta_reference == FGPU_BETA_REF_DISKMODEL) {
		const double e0 = 1.0 / (s->p.gamma - 1.0) * pow(s->p.aspect_ratio, 2) *
				  pow(s->Rmed[i], 2.0 * s->p.flaring_index - 1.0) *
				  s->p.G * s->p.hydro_center_mass * AT(S, i, j);
		delta_E -= e0;
	    } else if (s->p.cooling_beta_reference == FGPU_BETA_REF_FLOOR) {
		const double emin = s->p.minimum_temperature * AT(S, i, j) / s->p.mu *
				    s->p.R_gas / (s->p.gamma - 1.0);
		delta_E -= emin;
	    }
	    const double qminus = delta_E * omega_k * beta_inv;
	    AT(Qm, i, j) += qminus;
	}
    }
}

/* calculate_qplus -> viscous_heating, src/SourceEuler.cpp:496-536, 616-630 */
static void calculate_qplus(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *Qp = F(s, FGPU_QPLUS), *nu = F(s, FGPU_VISCOSITY),
	   *S = F(s, FGPU_SIGMA), *Trp = F(s, FGPU_TAU_R_PHI),
	   *Trr = F(s, FGPU_TAU_R_R), *Tpp = F(s, FGPU_TAU_PHI_PHI),
	   *dv = F(s, FGPU_DIV_V);
    memset(Qp, 0, sizeof(double) * (size_t)nr * nz);
    if (!s->p.heating_viscous) return;
#pragma omp parallel for
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    if (AT(nu, i, j) != 0.0) {
		const int jn = j == nz - 1 ? 0 : j + 1;
		const double trp = 0.25 * (AT(Trp, i, j) + AT(Trp, i + 1, j) +
					   AT(Trp, i, jn) + AT(Trp, i + 1, jn));
		double qplus = 1.0 / (2.0 * AT(nu, i, j) * AT(S, i, j)) *
			       (pow(AT(Trr, i, j), 2) + 2 * pow(trp, 2) +
				pow(AT(Tpp, i, j), 2));
		qplus += (2.0 / 9.0) * AT(nu, i, j) * AT(S, i, j) *
			 pow(AT(dv, i, j), 2);
		qplus *= s->p.heating_viscous_factor;
		AT(Qp, i, j) += qplus;
	    }
	}
    }
}

/* alpha_rad factor of SubStep3 / compute_heating_cooling_for_CFL */
static double rad_alpha(const or_state *s, double H, double sigma, double energy)
{
    const double inv_pow4 =
	pow(s->p.mu * (s->p.gamma - 1.0) / (s->p.R_gas * sigma), 4);
    return 1.0 + 2.0 * H * 4.0 * s->p.sigma_sb / s->p.c_light * inv_pow4 *
		     pow(energy, 3);
}

int or_recalculate_derived(or_state *s, double t)
{
    (void)t;
    /* recalculate_derived_disk_quantities, src/SourceEuler.cpp:225-249
       (AspectRatioMode 0 only) */
    if (adiabatic(s)) {
	compute_temperature(s);
	compute_sound_speed(s);
	compute_scale_height(s);
	or_compute_pressure(s);
    } else {
	or_compute_pressure(s);
    }
    update_viscosity(s);
    return FGPU_OK;
}

/* ------------------------------------------------------------------ */
/* potential: CalculateNbodyPotential, src/Pframeforce.cpp:21-86        */
/* ------------------------------------------------------------------ */
void or_calculate_potential(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *pot = F(s, FGPU_POTENTIAL), *H = F(s, FGPU_SCALE_HEIGHT);
    const double G = s->p.G;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double x = s->Rmed[i] * s->cosj[j];
	    const double y = s->Rmed[i] * s->sinj[j];
	    double acc = 0.0;
	    for (int k = 0; k < s->nb; ++k) {
		const double smooth = s->p.thickness_smoothing * AT(H, i, j);
		const double dx = x - s->b[k].x;
		const double dy = y - s->b[k].y;
		const double dist_2 = pow(dx, 2) + pow(dy, 2);
		const double d_sm = sqrt(dist_2 + pow(smooth, 2));
		double fk = 1.0;
		if (s->b[k].r_sm > 0.0) {
		    const double r_sm = s->b[k].r_sm;
		    if (d_sm < r_sm) {
			fk = pow(d_sm / r_sm, 4.0) - 2.0 * pow(d_sm / r_sm, 3.0) +
			     2.0 * d_sm / r_sm;
		    }
		}
		acc += -G * s->b[k].mass / d_sm * fk;
	    }
	    acc += -s->ix * x - s->iy * y;
	    AT(pot, i, j) = acc;
	}
    }
}

/* ------------------------------------------------------------------ */
/* source terms: update_with_sourceterms, src/SourceEuler.cpp:325-493   */
/* ------------------------------------------------------------------ */
void or_update_with_sourceterms(or_state *s, double dt)
{
    const int nr = s->nr, nz = s->nz;
    double *S = F(s, FGPU_SIGMA), *P = F(s, FGPU_PRESSURE),
	   *Phi = F(s, FGPU_POTENTIAL), *vaz = F(s, FGPU_V_AZIMUTHAL),
	   *vr = F(s, FGPU_V_RADIAL), *E = F(s, FGPU_ENERGY);
    const double OmegaF = s->omega_frame;

    /* momentum_update_radial, :325-372 (One_no_ghost_vr = 2 .. MaxMo = nr-1) */
#pragma omp parallel for
    for (int i = 2; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    double gradp = 2.0 / (AT(S, i, j) + AT(S, i - 1, j));
	    gradp *= (AT(P, i, j) - AT(P, i - 1, j));
	    gradp *= s->InvDiffRmed[i];
	    const double gradphi = (AT(Phi, i, j) - AT(Phi, i - 1, j)) * s->InvDiffRmed[i];
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    const double vsum = AT(vaz, i, j) + AT(vaz, i, jn) + AT(vaz, i - 1, j) +
				AT(vaz, i - 1, jn);
	    const double vt = 0.25 * vsum + s->Rinf[i] * OmegaF;
	    const double vt2 = vt * vt;
	    const double centrifugal = vt2 * s->InvRinf[i];
	    AT(vr, i, j) += dt * (-gradp - gradphi + centrifugal);
	}
    }
    /* momentum_update_azimuthal, :375-428 (Zero_no_ghost = 1 .. Max = nr-1) */
#pragma omp parallel for
    for (int i = 1; i < nr - 1; ++i) {
	const double invdxtheta = 2.0 / (s->dphi * (s->Rsup[i] + s->Rinf[i]));
	for (int j = 0; j < nz; ++j) {
	    const int jp = j == 0 ? nz - 1 : j - 1;
	    const double gradp = 2.0 / (AT(S, i, j) + AT(S, i, jp)) *
				 (AT(P, i, j) - AT(P, i, jp)) * invdxtheta;
	    const double gradphi = (AT(Phi, i, j) - AT(Phi, i, jp)) * invdxtheta;
	    AT(vaz, i, j) = AT(vaz, i, j) + dt * (-gradp - gradphi);
	}
    }
    /* compression_heating, :459-493 (nr 0 .. max_radial-1) */
    if (adiabatic(s)) {
#pragma omp parallel for
	for (int i = 0; i < nr - 1; ++i) {
	    for (int j = 0; j < nz; ++j) {
		const int jn = j == nz - 1 ? 0 : j + 1;
		const double div_v =
		    (AT(vr, i + 1, j) * s->Rinf[i + 1] - AT(vr, i, j) * s->Rinf[i]) *
			s->InvDiffRsupRb[i] +
		    (AT(vaz, i, jn) - AT(vaz, i, j)) * s->invdphi * s->InvRmed[i];
		const double e_old = AT(E, i, j);
		AT(E, i, j) = e_old * exp(-(s->p.gamma - 1.0) * dt * div_v);
	    }
	}
    }
}

/* update_with_artificial_viscosity_TW, artificial_viscosity.cpp:35-140:
   tensor artificial viscosity of Tscharnuter & Winkler with only the
   diagonal elements, its dissipation, then the velocity updates */
static void artificial_viscosity_tw(or_state *s, double dt)
{
    const int nr = s->nr, nz = s->nz;
    double *E = F(s, FGPU_ENERGY), *S = F(s, FGPU_SIGMA), *vr = F(s, FGPU_V_RADIAL),
	   *vaz = F(s, FGPU_V_AZIMUTHAL), *Qrr = F(s, FGPU_Q_R), *Qpp = F(s, FGPU_Q_PHI);
    const int dissipate = adiabatic(s) && s->p.art_visc_dissipation;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    const double eps_rr = (AT(vr, i + 1, j) - AT(vr, i, j)) * s->InvDiffRsup[i];
	    const double eps_pp =
		s->InvRmed[i] * ((AT(vaz, i, jn) - AT(vaz, i, j)) * s->invdphi +
				 0.5 * (AT(vr, i + 1, j) + AT(vr, i, j)));
	    const double sum = eps_rr + eps_pp;
	    const double div_V = sum < 0.0 ? sum : 0.0;
	    const double Dr = s->Rinf[i + 1] - s->Rinf[i];
	    const double rDphi = s->Rmed[i] * s->dphi;
	    double dx_sq;
	    if (nz <= 16) {
		dx_sq = pow(Dr < rDphi ? Dr : rDphi, 2);
	    } else {
		dx_sq = pow(Dr > rDphi ? Dr : rDphi, 2);
	    }
	    const double l_sq = pow(s->p.art_visc_factor, 2) * dx_sq;
	    AT(Qrr, i, j) = l_sq * AT(S, i, j) * -div_V * (eps_rr - 1.0 / 3.0 * div_V);
	    AT(Qpp, i, j) = l_sq * AT(S, i, j) * -div_V * (eps_pp - 1.0 / 3.0 * div_V);
	    if (dissipate && i > 0 && i < nr - 1) {
		const double Qplus = -l_sq * div_V * AT(S, i, j) * 1.0 / 3.0 *
				     (pow(eps_rr, 2) + pow(eps_pp, 2) + pow((eps_rr - eps_pp), 2));
		AT(E, i, j) += Qplus * dt;
	    }
	}
    }
#pragma omp parallel for
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jp = j == 0 ? nz - 1 : j - 1;
	    const double sigma_phi_avg = 0.5 * (AT(S, i, j) + AT(S, i, jp));
	    const double dVp = 2.0 * dt / ((s->Rsup[i] + s->Rinf[i]) * sigma_phi_avg) *
			       (AT(Qpp, i, j) - AT(Qpp, i, jp)) * s->invdphi;
	    AT(vaz, i, j) += dVp;
	}
    }
#pragma omp parallel for
    for (int i = 2; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double sigma_r_avg = 0.5 * (AT(S, i, j) + AT(S, i - 1, j));
	    const double dVr =
		s->p.radial_viscosity_factor * dt / sigma_r_avg * 2.0 /
		(pow(s->Rmed[i], 2) - pow(s->Rmed[i - 1], 2)) *
		((AT(Qrr, i, j) * s->Rmed[i] - AT(Qrr, i - 1, j) * s->Rmed[i - 1]) -
		 0.5 * (AT(Qpp, i, j) + AT(Qpp, i - 1, j)) * (s->Rmed[i] - s->Rmed[i - 1]));
	    AT(vr, i, j) += dVr;
	}
    }
}

/* ------------------------------------------------------------------ */
/* art_visc::update_with_artificial_viscosity(_SN),                     */
/* src/viscosity/artificial_viscosity.cpp:11-28, 148-250                */
/* ------------------------------------------------------------------ */
void or_artificial_viscosity(or_state *s, double dt)
{
    const int nr = s->nr, nz = s->nz;
    if (s->p.art_visc == FGPU_ARTVISC_SN) {
	double *E = F(s, FGPU_ENERGY), *S = F(s, FGPU_SIGMA),
	       *vr = F(s, FGPU_V_RADIAL), *vaz = F(s, FGPU_V_AZIMUTHAL),
	       *Qr = F(s, FGPU_Q_R), *Qp = F(s, FGPU_Q_PHI);
	const double C = s->p.art_visc_factor;
#pragma omp parallel for
	for (int i = 0; i < nr; ++i) {
	    for (int j = 0; j < nz; ++j) {
		const double dv_r = AT(vr, i + 1, j) - AT(vr, i, j);
		AT(Qr, i, j) = dv_r < 0.0 ? pow(C, 2) * AT(S, i, j) * pow(dv_r, 2) : 0.0;
		const int jn = j == nz - 1 ? 0 : j + 1;
		const double dv_p = AT(vaz, i, jn) - AT(vaz, i, j);
		AT(Qp, i, j) = dv_p < 0.0 ? pow(C, 2) * AT(S, i, j) * pow(dv_p, 2) : 0.0;
	    }
	}
	if (adiabatic(s) && s->p.art_visc_dissipation) {
#pragma omp parallel for
	    for (int i = 1; i < nr - 1; ++i) {
		const double invdxtheta = 1.0 / (s->dphi * s->Rmed[i]);
		for (int j = 0; j < nz; ++j) {
		    const int jn = j == nz - 1 ? 0 : j + 1;
		    const double dv_r = AT(vr, i + 1, j) - AT(vr, i, j);
		    const double dv_p = AT(vaz, i, jn) - AT(vaz, i, j);
		    AT(E, i, j) = AT(E, i, j) -
				  dt * AT(Qr, i, j) * dv_r * s->InvDiffRsup[i] -
				  dt * AT(Qp, i, j) * dv_p * invdxtheta;
		}
	    }
	}
#pragma omp parallel for
	for (int i = 2; i < nr - 1; ++i) {
	    for (int j = 0; j < nz; ++j) {
		AT(vr, i, j) = AT(vr, i, j) -
			       dt * 2.0 / (AT(S, i, j) + AT(S, i - 1, j)) *
				   (AT(Qr, i, j) - AT(Qr, i - 1, j)) * s->InvDiffRmed[i];
	    }
	}
#pragma omp parallel for
	for (int i = 1; i < nr - 1; ++i) {
	    const double invdxtheta = 1.0 / (s->dphi * s->Rmed[i]);
	    for (int j = 0; j < nz; ++j) {
		const int jp = j == 0 ? nz - 1 : j - 1;
		AT(vaz, i, j) = AT(vaz, i, j) -
				dt * 2.0 / (AT(S, i, j) + AT(S, i, jp)) *
				    (AT(Qp, i, j) - AT(Qp, i, jp)) * invdxtheta;
	    }
	}
    }
    if (s->p.art_visc == FGPU_ARTVISC_TW) {
	artificial_viscosity_tw(s, dt);
    }
    if (adiabatic(s) && s->p.art_visc_dissipation) {
	assure_temperature_range(s);
    }
}

/* recalculate_viscosity, src/SourceEuler.cpp:205-223 */
void or_recalculate_viscosity(or_state *s, double t)
{
    (void)t;
    if (adiabatic(s)) {
	compute_sound_speed(s);
	compute_scale_height(s);
    }
    update_viscosity(s);
}

/* The pseudo-implicit correction factors of StabilizeViscosity,
   viscosity.cpp:256-348: c_phi at v_phi and c_r at v_r positions, rows
   1 .. Nrad-1 */
static void viscosity_correction_factors(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    const double *S = F(s, FGPU_SIGMA);
    const double *NS = s->visc_sigma, *NSrp = s->visc_sigma_rp;
    const double *Ra = s->Rinf;
#pragma omp parallel for
    for (int i = 1; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jp = j == 0 ? nz - 1 : j - 1;
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    const double NuSig_rp = AT(NSrp, i, j);
	    const double NuSig_rp_ip = AT(NSrp, i + 1, j);
	    const double NuSig_rp_jp = AT(NSrp, i, jn);
	    const double NuSigma = AT(NS, i, j);
	    const double NuSigma_jm = AT(NS, i, jp);
	    const double NuSigma_im = AT(NS, i - 1, j);

	    const double a3 = NuSig_rp * pow(Ra[i], 3) * s->InvDiffRmed[i];
	    const double a3p = NuSig_rp_ip * pow(Ra[i + 1], 3) * s->InvDiffRmed[i + 1];
	    const double cphi_rp = -s->InvRmed[i] * s->TwoDiffRaSq[i] * (a3p + a3);
	    const double cphi_pp = -s->FourThirdInvRbInvdphiSq[i] * (NuSigma + NuSigma_jm);
	    const double sigma_avg_phi = 0.5 * (AT(S, i, j) + AT(S, i, jp));
	    AT(s->corr_phi, i, j) = (cphi_rp + cphi_pp) / (sigma_avg_phi * s->Rmed[i]);

	    const double sigma_avg_r = 0.5 * (AT(S, i, j) + AT(S, i - 1, j));
	    const double cr_rp = -(NuSig_rp_jp + NuSig_rp) / (s->dphi * s->dphi * Ra[i]);
	    const double cr_pp_1 = 2.0 * NuSigma *
				   (0.5 * s->InvRmed[i] + 1.0 / 3.0 * Ra[i] * s->InvDiffRsupRb[i]);
	    const double cr_pp_2 =
		2.0 * NuSigma_im *
		(0.5 * s->InvRmed[i - 1] - 1.0 / 3.0 * Ra[i] * s->InvDiffRsupRb[i - 1]);
	    const double cr_rr_1 = s->Rmed[i] * 2.0 * NuSigma *
				   (-s->InvDiffRsup[i] + 1.0 / 3.0 * Ra[i] * s->InvDiffRsupRb[i]);
	    const double cr_rr_2 =
		-1.0 * s->Rmed[i - 1] * 2.0 * NuSigma_im *
		(s->InvDiffRsup[i - 1] - 1.0 / 3.0 * Ra[i] * s->InvDiffRsupRb[i - 1]);
	    const double cr_pp = -0.5 * (cr_pp_1 + cr_pp_2);
	    const double cr_rr = s->InvDiffRmed[i] * (cr_rr_1 + cr_rr_2);
	    const double Rmed_mid = 0.5 * (s->Rmed[i] + s->Rmed[i - 1]);
	    AT(s->corr_r, i, j) = s->p.radial_viscosity_factor * (cr_rr + cr_rp + cr_pp) /
				  (sigma_avg_r * Rmed_mid);
	}
    }
}

/* viscosity::compute_viscous_stress_tensor, src/viscosity/viscosity.cpp:139-254 */
void or_viscous_stress_tensor(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *dv = F(s, FGPU_DIV_V), *vr = F(s, FGPU_V_RADIAL),
	   *vaz = F(s, FGPU_V_AZIMUTHAL), *nu = F(s, FGPU_VISCOSITY),
	   *S = F(s, FGPU_SIGMA), *Trr = F(s, FGPU_TAU_R_R),
	   *Tpp = F(s, FGPU_TAU_PHI_PHI), *Trp = F(s, FGPU_TAU_R_PHI);
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    AT(dv, i, j) =
		(AT(vr, i + 1, j) * s->Rinf[i + 1] - AT(vr, i, j) * s->Rinf[i]) *
		    s->InvDiffRsupRb[i] +
		(AT(vaz, i, jn) - AT(vaz, i, j)) * s->invdphi * s->InvRmed[i];
	}
    }
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    const double drr = (AT(vr, i + 1, j) - AT(vr, i, j)) * s->InvDiffRsup[i];
	    AT(Trr, i, j) = 2.0 * AT(nu, i, j) * AT(S, i, j) *
			    (drr - 1.0 / 3.0 * AT(dv, i, j));
	    const double dpp =
		(AT(vaz, i, jn) - AT(vaz, i, j)) * s->invdphi * s->InvRmed[i] +
		0.5 * (AT(vr, i + 1, j) + AT(vr, i, j)) * s->InvRmed[i];
	    const double n = AT(nu, i, j), sg = AT(S, i, j);
	    AT(Tpp, i, j) = 2.0 * n * sg * (dpp - 1.0 / 3.0 * AT(dv, i, j));
	    AT(s->visc_sigma, i, j) = n * sg;
	}
    }
#pragma omp parallel for
    for (int i = 1; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jp = j == 0 ? nz - 1 : j - 1;
	    const double dvazirdr =
		(AT(vaz, i, j) * s->InvRmed[i] - AT(vaz, i - 1, j) * s->InvRmed[i - 1]) *
		s->InvDiffRmed[i];
	    const double dvrdphi = (AT(vr, i, j) - AT(vr, i, jp)) * s->invdphi;
	    const double drp = s->Rinf[i] * dvazirdr + dvrdphi * s->InvRinf[i];
	    const double n = 0.25 * (AT(nu, i, j) + AT(nu, i - 1, j) + AT(nu, i, jp) +
				     AT(nu, i - 1, jp));
	    const double sg = 0.25 * (AT(S, i, j) + AT(S, i - 1, j) + AT(S, i, jp) +
				      AT(S, i - 1, jp));
	    AT(Trp, i, j) = n * sg * drp;
	    AT(s->visc_sigma_rp, i, j) = n * sg;
	}
    }
    if (s->p.stabilize_viscosity) {
	viscosity_correction_factors(s);
    }
}

/* viscosity::update_velocities_with_viscosity, viscosity.cpp:355-421 */
void or_update_velocities_with_viscosity(or_state *s, double dt)
{
    const int nr = s->nr, nz = s->nz;
    double *vaz = F(s, FGPU_V_AZIMUTHAL), *vr = F(s, FGPU_V_RADIAL),
	   *S = F(s, FGPU_SIGMA), *Trp = F(s, FGPU_TAU_R_PHI),
	   *Trr = F(s, FGPU_TAU_R_R), *Tpp = F(s, FGPU_TAU_PHI_PHI);
#pragma omp parallel for
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jp = j == 0 ? nz - 1 : j - 1;
	    const double sigma_avg = 0.5 * (AT(S, i, j) + AT(S, i, jp));
	    double dVp =
		dt * s->InvRmed[i] / (sigma_avg) *
		((2.0 / (pow(s->Rinf[i + 1], 2) - pow(s->Rinf[i], 2))) *
		     (pow(s->Rinf[i + 1], 2) * AT(Trp, i + 1, j) -
		      pow(s->Rinf[i], 2) * AT(Trp, i, j)) +
		 (AT(Tpp, i, j) - AT(Tpp, i, jp)) * s->invdphi);
	    if (s->p.stabilize_viscosity == 1) {
		const double cphi = AT(s->corr_phi, i, j);
		const double a = 1.0 + dt * cphi;
		dVp *= 1.0 / ((a > 0.0 ? a : 0.0) - dt * cphi);
	    }
	    AT(vaz, i, j) += dVp;
	}
    }
#pragma omp parallel for
    for (int i = 2; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    const double sigma_avg = 0.5 * (AT(S, i, j) + AT(S, i - 1, j));
	    double dVr =
		dt / (sigma_avg)*s->p.radial_viscosity_factor * 2.0 /
		(s->Rmed[i] + s->Rmed[i - 1]) *
		((s->Rmed[i] * AT(Trr, i, j) - s->Rmed[i - 1] * AT(Trr, i - 1, j)) *
		     s->InvDiffRmed[i] +
		 (AT(Trp, i, jn) - AT(Trp, i, j)) * s->invdphi -
		 0.5 * (AT(Tpp, i, j) + AT(Tpp, i - 1, j)));
	    if (s->p.stabilize_viscosity == 1) {
		const double cr = AT(s->corr_r, i, j);
		const double a = 1.0 + dt * cr;
		dVr *= 1.0 / ((a > 0.0 ? a : 0.0) - dt * cr);
	    }
	    AT(vr, i, j) += dVr;
	}
    }
}

/* SubStep3, src/SourceEuler.cpp:859-954 (beta cooling + viscous heating) */
void or_substep3(or_state *s, double t, double dt)
{
    const int nr = s->nr, nz = s->nz;
    compute_temperature(s);
    calculate_qminus(s, t);
    calculate_qplus(s);
    double *Qp = F(s, FGPU_QPLUS), *Qm = F(s, FGPU_QMINUS), *E = F(s, FGPU_ENERGY),
	   *S = F(s, FGPU_SIGMA), *H = F(s, FGPU_SCALE_HEIGHT);
#pragma omp parallel for
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double sigma = AT(S, i, j), energy = AT(E, i, j);
	    const double alpha = rad_alpha(s, AT(H, i, j), sigma, energy);
	    AT(Qp, i, j) /= alpha;
	    AT(Qm, i, j) /= alpha;
	    const double qp = AT(Qp, i, j), qm = AT(Qm, i, j);
	    double energy_new = energy + dt * (qp - qm);
	    const double sigma_floor = 10.0 * s->p.sigma0 * s->p.sigma_floor;
	    if (sigma < sigma_floor) {
		/* TAU_EFF is never computed on this path (no surface cooling):
		   it is zero, so the equilibrium energy is zero. */
		const double tau_eff = 0.0;
		const double e4 = qp * tau_eff / (2.0 * s->p.sigma_sb);
		const double cst = (s->p.R_gas / s->p.mu * sigma / (s->p.gamma - 1.0));
		AT(Qm, i, j) = qp;
		energy_new = pow(e4, 1.0 / 4.0) * cst;
	    }
	    AT(E, i, j) = energy_new;
	}
    }
    assure_temperature_range(s);
}

/* ------------------------------------------------------------------ */
/* boundary conditions and damping                                     */
/* ------------------------------------------------------------------ */

/* damping_single_{inner,outer}{,_zero,_mean}, damping.cpp:311-752 */
static void damp_one(or_state *s, int q, int outer, double dt)
{
    const fgpu_params *p = &s->p;
    const int kind = outer ? p->damping_outer[q] : p->damping_inner[q];
    if (kind == FGPU_DAMP_NONE) return;
    const int field = dq_field[q];
    const int vec = is_vector_field(field);
    const double *radius = vec ? s->Rinf : s->Rmed;
    const int is_density = field == FGPU_SIGMA;
    double *X = F(s, field);
    double *X0 = F(s, field + 4); /* SIGMA0 .. ENERGY0 follow in the enum */
    const int nz = s->nz;
    if (!outer) {
	if (!s->damp_active_inner[q]) return;
	const int limit = s->damp_limit_inner[q];
	const double tau = p->damping_time_factor * 2.0 * M_PI / omega_kepler(s, p->rmin);
	if (kind == FGPU_DAMP_MEAN) {
	    for (int i = 0; i <= limit; ++i) {
		AT(X0, i, 0) = 0.0;
		for (int j = 0; j < nz; ++j) AT(X0, i, 0) += AT(X, i, j);
		AT(X0, i, 0) /= nz;
	    }
	}
#pragma omp parallel for
	for (int i = 0; i <= limit; ++i) {
	    const double factor = pow((radius[i] - p->rmin * p->damping_inner_limit) /
					  (p->rmin - p->rmin * p->damping_inner_limit),
				      2);
	    const double ef = exp(-dt * factor / tau);
	    for (int j = 0; j < nz; ++j) {
		double x0;
		if (kind == FGPU_DAMP_REFERENCE) x0 = AT(X0, i, j);
		else if (kind == FGPU_DAMP_ZERO) x0 = is_density ? p->sigma_floor * p->sigma0 : 0.0;
		else x0 = AT(X0, i, 0);
		AT(X, i, j) = (AT(X, i, j) - x0) * ef + x0;
	    }
	}
    } else {
	if (!s->damp_active_outer[q]) return;
	const int limit = s->damp_limit_outer[q];
	const int size = vec ? s->nr + 1 : s->nr;
	const double tau = p->damping_time_factor * 2.0 * M_PI /
			   omega_kepler(s, p->damping_time_radius_outer);
	if (kind == FGPU_DAMP_MEAN) {
	    for (int i = limit; i < size; ++i) {
		AT(X0, i, 0) = 0.0;
		for (int j = 0; j < nz; ++j) AT(X0, i, 0) += AT(X, i, j);
		AT(X0, i, 0) /= nz;
	    }
	}
#pragma omp parallel for
	for (int i = limit; i < size; ++i) {
	    const double factor = pow((radius[i] - p->rmax * p->damping_outer_limit) /
					  (p->rmax - p->rmax * p->damping_outer_limit),
				      2);
	    const double ef = exp(-dt * factor / tau);
	    for (int j = 0; j < nz; ++j) {
		double x0;
		if (kind == FGPU_DAMP_REFERENCE) x0 = AT(X0, i, j);
		else if (kind == FGPU_DAMP_ZERO) x0 = 0.0; /* damping.cpp:531 */
		else x0 = AT(X0, i, 0);
		AT(X, i, j) = (AT(X, i, j) - x0) * ef + x0;
	    }
	}
    }
}

/* per-field ghost hooks: zero_gradient.cpp, outflow.cpp, reference.cpp,
   keplerian_azimuthal.cpp */
static void ghost_hook(or_state *s, int field, int kind, int outer)
{
    const int nz = s->nz;
    const int vec = is_vector_field(field);
    double *x = F(s, field), *x0 = F(s, field + 4);
    const int irad = vec ? s->nr : s->nr - 1; /* get_max_radial() */
    for (int j = 0; j < nz; ++j) {
	switch (kind) {
	case FGPU_BC_NONE:
	    break;
	case FGPU_BC_ZEROGRADIENT:
	    if (!outer) {
		if (vec) { AT(x, 0, j) = AT(x, 2, j); AT(x, 1, j) = AT(x, 2, j); }
		else AT(x, 0, j) = AT(x, 1, j);
	    } else {
		if (vec) { AT(x, irad, j) = AT(x, irad - 2, j); AT(x, irad - 1, j) = AT(x, irad - 2, j); }
		else AT(x, irad, j) = AT(x, irad - 1, j);
	    }
	    break;
	case FGPU_BC_OUTFLOW:
	    if (!outer) {
		if (AT(x, 2, j) > 0.0) { AT(x, 1, j) = 0.0; AT(x, 0, j) = 0.0; }
		else { AT(x, 1, j) = AT(x, 2, j); AT(x, 0, j) = AT(x, 2, j); }
	    } else {
		if (AT(x, irad - 2, j) < 0.0) { AT(x, irad - 1, j) = 0.0; AT(x, irad, j) = 0.0; }
		else { AT(x, irad - 1, j) = AT(x, irad - 2, j); AT(x, irad, j) = AT(x, irad - 2, j); }
	    }
	    break;
	case FGPU_BC_REFERENCE:
	    if (!outer) {
		AT(x, 0, j) = AT(x0, 0, j);
		if (vec) AT(x, 1, j) = AT(x0, 1, j);
	    } else {
		AT(x, irad, j) = AT(x0, irad, j);
		if (vec) AT(x, irad - 1, j) = AT(x0, irad - 1, j);
	    }
	    break;
	case FGPU_BC_KEPLERIAN: {
	    const int i = outer ? irad : 0;
	    const double r = s->Rmed[i];
	    const double vK = sqrt(s->p.G * s->p.hydro_center_mass / r);
	    const double c = outer ? s->p.vaz_outer_keplerian_factor
				   : s->p.vaz_inner_keplerian_factor;
	    AT(x, i, j) = c * vK - r * s->omega_frame;
	    break;
	}
	case FGPU_BC_DISKMODEL: {
	    /* diskmodel.cpp:18-77 (calc_sig, calc_eng at Rmed of the ghost ring) */
	    const double R = s->Rmed[outer ? irad : 0];
	    const double sig0 = s->p.sigma0, sigexp = -s->p.sigma_slope;
	    double v;
	    if (field == FGPU_SIGMA) {
		v = sig0 * pow(R, sigexp);
	    } else {
		v = 1.0 / (s->p.gamma - 1.0) * sig0 * pow(s->p.aspect_ratio, 2) *
		    pow(R, sigexp - 1.0 + 2.0 * s->p.flaring_index);
	    }
	    AT(x, outer ? irad : 0, j) = v;
	    break;
	}
	case FGPU_BC_REFLECTING:
	    /* reflecting.cpp:15-40 */
	    if (!outer) {
		AT(x, 0, j) = -AT(x, 2, j);
		AT(x, 1, j) = 0;
	    } else {
		AT(x, irad, j) = -AT(x, irad - 2, j);
		AT(x, irad - 1, j) = 0;
	    }
	    break;
	case FGPU_BC_VISCOUS:
	    /* viscous_outflow_inner, viscous.cpp:15-40 */
	    if (!outer) {
		const double *visc = F(s, FGPU_VISCOSITY);
		const double sp = s->p.viscous_outflow_speed;
		const double Nu = 0.5 * (AT(visc, 0, j) + AT(visc, 1, j));
		AT(x, 1, j) = -1.5 * sp / s->Rinf[1] * Nu;
		AT(x, 0, j) = -1.5 * sp / s->Rinf[0] * Nu;
	    }
	    break;
	case FGPU_BC_KEPLERIAN_RADIAL: {
	    /* keplerian_radial.cpp:17-62 */
	    const double c = outer ? s->p.vrad_outer_keplerian_factor
				   : s->p.vrad_inner_keplerian_factor;
	    const int k0 = outer ? irad : 0, k1 = outer ? irad - 1 : 1;
	    AT(x, k0, j) = c * sqrt(s->p.G * s->p.hydro_center_mass / s->Rmed[k0]);
	    AT(x, k1, j) = c * sqrt(s->p.G * s->p.hydro_center_mass / s->Rmed[k1]);
	    break;
	}
	case FGPU_BC_ZEROSHEAR: {
	    /* zero_shear.cpp:19-53 */
	    const int e = outer ? irad : 0, a = outer ? irad - 1 : 1;
	    const double Omega_active = AT(x, a, j) / s->Rmed[a];
	    AT(x, e, j) = s->Rmed[e] * Omega_active;
	    break;
	}
	case FGPU_BC_BALANCED: {
	    /* balanced_boundary, balanced.cpp:20-66, support_azi_*
	       Theo.cpp:131-157 (no self-gravity) */
	    const int e = outer ? irad : 0;
	    const double R = s->Rmed[e];
	    const double vk = sqrt(s->p.G * s->p.hydro_center_mass / R);
	    const double vk_2 = pow(vk, 2);
	    double support = 0.0;
	    if (!s->p.profile_cutoff_outer) {
		const double F = s->p.flaring_index, S = s->p.sigma_slope;
		const double h = s->p.aspect_ratio * pow(R, F);
		support += (2.0 * F - 1.0 - S) * pow(h, 2);
		const double eps = s->p.thickness_smoothing;
		support += (1.0 + (F + 1.0) * pow(h * eps, 2)) / pow(sqrt(1 + pow(h * eps, 2)), 3);
	    }
	    if (s->p.binary_quadrupole_moment > 0.0) {
		support += 3.0 * s->p.binary_quadrupole_moment / pow(R, 2);
	    }
	    double vaz_balanced = sqrt(vk_2 * support);
	    vaz_balanced -= R * s->omega_frame;
	    AT(x, e, j) = vaz_balanced;
	    break;
	}
	}
    }
}

/* ------------------------------------------------------------------ */
/* centre-of-mass composite boundary: src/boundary_conditions/         */
/* center_of_mass.cpp, the model of src/Theo.cpp:86-243 and the        */
/* viscous-speed tables of src/viscosity/viscous_radial_speed.cpp      */
/* ------------------------------------------------------------------ */

#define OR_VR_TABLE_N 1000 /* viscous_radial_speed.cpp:256 */

static double th_h(const or_state *s, double R)
{
    return s->p.aspect_ratio * pow(R, s->p.flaring_index);
}

/* support_azi_pressure / _smoothing_derivative / _quadrupole, Theo.cpp:131-157 */
static double th_pressure(const or_state *s, double R)
{
    const double F = s->p.flaring_index, S = s->p.sigma_slope;
    return (2.0 * F - 1.0 - S) * pow(th_h(s, R), 2);
}

static double th_smoothing(const or_state *s, double R)
{
    const double F = s->p.flaring_index, eps = s->p.thickness_smoothing;
    const double h = th_h(s, R);
    return (1.0 + (F + 1.0) * pow(h * eps, 2)) / pow(sqrt(1 + pow(h * eps, 2)), 3);
}

static double th_quadrupole(const or_state *s, double R)
{
    const double Q = s->p.binary_quadrupole_moment;
    return Q > 0.0 ? 3.0 * Q / pow(R, 2) : 0.0;
}

/* initial_locally_isothermal_smoothed_v_az (Theo.cpp:166-181) and the
   variant with the quadrupole moment (:183-200); the quadrupole moment is
   zero unless VazimuthalConsidersQuadropoleMoment is set */
static double th_vaz(const or_state *s, double R, double M, int quad)
{
    double support;
    if (quad) {
	support = th_quadrupole(s, R) + th_smoothing(s, R) + th_pressure(s, R);
    } else {
	const double sm = th_smoothing(s, R);
	support = sm + th_pressure(s, R);
    }
    const double vk_2 = s->p.G * M / R;
    return sqrt(vk_2 * support);
}

/* initial_viscous_radial_speed, Theo.cpp:220-243 */
static double th_vr_steady(const or_state *s, double R, double M)
{
    const fgpu_params *p = &s->p;
    if (p->viscous_alpha > 0) {
	const double sqrt_gamma = adiabatic(s) ? sqrt(p->gamma) : 1.0;
	const double v_k = sqrt(p->G * M / R);
	const double h = p->aspect_ratio * pow(R, p->flaring_index);
	const double cs = sqrt_gamma * h * v_k;
	const double H = h * R;
	const double nu = p->viscous_alpha * cs * H;
	return -3.0 * nu / R * (-p->sigma_slope + 2.0 * p->flaring_index + 1.0);
    }
    return -3.0 * p->constant_viscosity / R * (-p->sigma_slope + .5);
}

/* initial_energy, Theo.cpp:86-99 */
static double th_energy(const or_state *s, double R, double M)
{
    const fgpu_params *p = &s->p;
    return 1.0 / (p->gamma - 1.0) * p->sigma0 * pow(p->aspect_ratio, 2) *
	   pow(R, -p->sigma_slope - 1.0 + 2.0 * p->flaring_index) * p->G * M;
}

/* cutoff_outer / cutoff_inner, util.cpp:69-93 */
static double cutoff_out(const or_state *s, double x)
{
    return 1.0 / (1.0 + exp((x - s->p.profile_cutoff_point_outer) /
			    s->p.profile_cutoff_width_outer));
}

static double cutoff_in(const or_state *s, double x)
{
    return 1.0 / (1.0 + exp((s->p.profile_cutoff_point_inner - x) /
			    s->p.profile_cutoff_width_inner));
}

/* get_sigma, viscous_radial_speed.cpp:92-115 */
static double vs_sigma(const or_state *s, double R)
{
    const fgpu_params *p = &s->p;
    double d = p->sigma0 * pow(R, -p->sigma_slope);
    const double floor_ = p->sigma_floor * p->sigma0;
    if (p->profile_cutoff_outer) d *= cutoff_out(s, R);
    if (p->profile_cutoff_inner) d *= cutoff_in(s, R);
    return d > floor_ ? d : floor_;
}

/* get_nu2, viscous_radial_speed.cpp:37-90 */
static double vs_nu2(const or_state *s, double R, double M, double Sigma)
{
    const fgpu_params *p = &s->p;
    const double v_k = sqrt(p->G * M / R);
    const double h = p->aspect_ratio * pow(R, p->flaring_index);
    double cutoff = 1.0;
    if (p->profile_cutoff_outer) cutoff *= cutoff_out(s, R);
    if (p->profile_cutoff_inner) cutoff *= cutoff_in(s, R);
    double cs_adb, H;
    if (adiabatic(s)) {
	const double gamma = p->gamma;
	double energy = cutoff * 1.0 / (gamma - 1.0) * Sigma * pow(h * v_k, 2);
	const double efloor = p->minimum_temperature * Sigma / p->mu * p->R_gas / (gamma - 1.0);
	const double eceil = p->maximum_temperature * Sigma / p->mu * p->R_gas / (gamma - 1.0);
	energy = fmax(energy, efloor);
	energy = fmin(energy, eceil);
	cs_adb = sqrt(gamma * (gamma - 1.0) * energy / Sigma);
	const double cs_iso = sqrt((gamma - 1.0) * energy / Sigma);
	const double omega_k = v_k / R;
	H = cs_iso / omega_k;
    } else {
	cs_adb = h * v_k;
	H = h * R;
    }
    return p->viscous_alpha * cs_adb * H;
}

typedef double (*vs_fn)(const or_state *, double, double);

/* derive, viscous_radial_speed.cpp:122-135 */
static double vs_derive(const or_state *s, double x, double M, vs_fn f)
{
    const double h = 8.0e-4 * x;
    const double f1 = -1.0 * f(s, x + 2.0 * h, M);
    const double f2 = 8.0 * f(s, x + h, M);
    const double f3 = -8.0 * f(s, x - h, M);
    const double f4 = 1.0 * f(s, x - 2.0 * h, M);
    return (f1 + f2 + f3 + f4) / (12.0 * h);
}

/* get_w with VazimuthalConsidersQuadropoleMoment folded into the moment */
static double vs_w(const or_state *s, double r, double M)
{
    return th_vaz(s, r, M, 1) / r;
}

static double vs_r2_w(const or_state *s, double r, double M)
{
    return pow(r, 2) * vs_w(s, r, M);
}

static double vs_nu_S_r3_dwdr(const or_state *s, double r, double M)
{
    const double dw_dr = vs_derive(s, r, M, vs_w);
    const double Sigma = vs_sigma(s, r);
    const double nu = vs_nu2(s, r, M, Sigma);
    return nu * Sigma * pow(r, 3) * dw_dr;
}

/* get_vr_with_numerical_viscous_speed, viscous_radial_speed.cpp:184-200 */
static double vs_vr(const or_state *s, double r, double M)
{
    const double num = 1.0 / r * vs_derive(s, r, M, vs_nu_S_r3_dwdr);
    const double den = vs_sigma(s, r) * vs_derive(s, r, M, vs_r2_w);
    return num / den;
}

/* interface radius k (Radii[k]) and GlobalRmed[k] (init.cpp:176-179) */
static double radii_at(const or_state *s, int k)
{
    return k <= s->nr ? s->Rinf[k] : s->Rsup[k - 1];
}

static double global_rmed(const or_state *s, int k)
{
    const double a = radii_at(s, k), b = radii_at(s, k + 1);
    double r = 2.0 / 3.0 * (pow(b, 3) - pow(a, 3));
    return r / (pow(b, 2) - pow(a, 2));
}

/* get_vr_outer_viscous_speed_correction_factor, viscous_radial_speed.cpp:207-254 */
static double vs_outer_correction(const or_state *s, double r, double M)
{
    int k = clamp_id(cell_id_rmed(s, r), 1, s->nr);
    if (k < 2) k = 2;
    const double rinf = radii_at(s, k);
    const double rmed_p = global_rmed(s, k + 1), rmed = global_rmed(s, k);
    const double rmed_m = global_rmed(s, k - 1), rmed_m2 = global_rmed(s, k - 2);
    const double w_p = vs_w(s, rmed_p, M), w = vs_w(s, rmed, M);
    const double w_m = vs_w(s, rmed_m, M), w_m2 = vs_w(s, rmed_m2, M);
    const double dw_dr = (0.5 * (w_p + w) - 0.5 * (w + w_m)) / (radii_at(s, k + 1) - radii_at(s, k));
    const double dw_dr_m = (0.5 * (w + w_m) - 0.5 * (w_m + w_m2)) / (radii_at(s, k) - radii_at(s, k - 1));
    const double Sigma = vs_sigma(s, rmed);
    const double nu = vs_nu2(s, rmed, M, Sigma);
    const double Sigma_m = vs_sigma(s, rmed_m);
    const double nu_m = vs_nu2(s, rmed_m, M, Sigma_m);
    const double a = nu * Sigma * pow(rmed, 3) * dw_dr;
    const double a_m = nu_m * Sigma_m * pow(rmed_m, 3) * dw_dr_m;
    const double dr = rmed - rmed_m;
    const double num = 1.0 / rinf * (a - a_m) / dr;
    const double r2w = pow(rmed, 2) * vs_w(s, rmed, M);
    const double r2w_m = pow(rmed_m, 2) * vs_w(s, rmed_m, M);
    const double dr2w_dr = (r2w - r2w_m) / (rmed - rmed_m);
    const double den = Sigma_m * dr2w_dr;
    const double vr = num / den;
    return vr / vs_vr(s, rinf, M);
}

/* init_vr_table_boundary, viscous_radial_speed.cpp:269-347; the tables get
   one node more than the reference's so that the last bin has a right node */
int or_init_center_of_mass_boundary(or_state *s, double mass_all, double mass_center,
				    int binary_on_primary, double com_max_dist)
{
    const fgpu_params *p = &s->p;
    const int nr = s->nr, N = OR_VR_TABLE_N;
    for (int k = 0; k < 2; ++k) {
	free(s->com_r[k]);
	free(s->com_vr[k]);
	s->com_r[k] = calloc(N + 1, sizeof(double));
	s->com_vr[k] = calloc(N + 1, sizeof(double));
    }
    {
	const double safety = s->Rsup[nr - 1] - s->Rinf[nr - 1];
	double lo, hi;
	if (binary_on_primary) {
	    lo = s->Rinf[nr - 1] * p->damping_outer_limit - com_max_dist - safety;
	    hi = s->Rsup[nr - 1] + com_max_dist + safety;
	} else {
	    lo = s->Rinf[nr - 1] * p->damping_outer_limit - safety;
	    hi = s->Rsup[nr - 1] + safety;
	}
	if (lo < p->rmin) lo = p->rmin;
	s->com_min_r[1] = lo;
	s->com_dlog[1] = log10(hi / lo) / (double)N;
	for (int i = 0; i <= N; ++i) {
	    const double r = lo * pow(10.0, (s->com_dlog[1] * (double)i));
	    s->com_r[1][i] = r;
	    s->com_vr[1][i] = vs_vr(s, r, mass_all) * vs_outer_correction(s, r, mass_all);
	}
    }
    {
	const int lim = clamp_id(cell_id_rmed(s, p->rmin * p->damping_inner_limit), 0, nr) + 1;
	const double safety = s->Rsup[lim] - s->Rinf[lim];
	double lo, hi;
	if (binary_on_primary) {
	    lo = s->Rinf[1] - com_max_dist - safety;
	    if (lo < s->Rsup[0] - s->Rinf[0]) lo = s->Rsup[0] - s->Rinf[0];
	    hi = s->Rsup[1] * p->damping_inner_limit + com_max_dist + safety;
	} else {
	    lo = s->Rinf[1] - safety;
	    hi = s->Rsup[1] * p->damping_inner_limit + safety;
	}
	s->com_min_r[0] = lo;
	s->com_dlog[0] = log10(hi / lo) / (double)N;
	for (int i = 0; i <= N; ++i) {
	    const double r = lo * pow(10.0, (s->com_dlog[0] * (double)i));
	    s->com_r[0][i] = r;
	    s->com_vr[0][i] = vs_vr(s, r, mass_center);
	}
    }
    s->com_ready = 1;
    return FGPU_OK;
}

/* correct_v_azimuthal, src/SideEuler.cpp:79-95 */
int or_correct_v_azimuthal(or_state *s, double domega)
{
    double *vaz = s->f[FGPU_V_AZIMUTHAL];
    for (int i = 0; i < s->nr; ++i)
	for (int j = 0; j < s->nz; ++j) vaz[(size_t)i * s->nz + j] -= domega * s->Rmed[i];
    return FGPU_OK;
}

int or_set_frame_centers(or_state *s, const fgpu_frame_center now[2],
			 const fgpu_frame_center *after)
{
    for (int k = 0; k < 2; ++k) {
	s->com_now[k] = now[k];
	s->com_after[k] = after ? after[k] : now[k];
    }
    return FGPU_OK;
}

/* lookup_initial_vr_outer / _inner, viscous_radial_speed.cpp:350-407 */
static double com_lookup(const or_state *s, int side, double r)
{
    const int N = OR_VR_TABLE_N;
    const int i = (int)floor(log10(r / s->com_min_r[side]) / s->com_dlog[side]);
    const double *rt = s->com_r[side], *vt = s->com_vr[side];
    if (i > N - 1) return vt[N - 1];
    if (i < 0) return vt[0];
    const double x = (r - rt[i]) / (rt[i + 1] - rt[i]);
    return (1.0 - x) * vt[i] + x * vt[i + 1];
}

/* the model velocity at (cx, cy) in the primary's frame; side 0 is the
   inner edge (no quadrupole term), 1 the outer edge */
static void com_velocity(const or_state *s, int side, int damping, const fgpu_frame_center *c,
			 double cx, double cy, double *vx, double *vy)
{
    const double x_com = cx - c->x, y_com = cy - c->y;
    const double r_com = sqrt(x_com * x_com + y_com * y_com);
    double vazi0, vr0;
    if (s->p.initialize_pure_keplerian) {
	vazi0 = sqrt(s->p.G * c->mass / r_com); /* compute_v_kepler */
	vr0 = (damping && s->p.initialize_vradial_zero) ? 0.0
						       : th_vr_steady(s, r_com, c->mass);
    } else {
	vazi0 = th_vaz(s, r_com, c->mass, side == 1);
	vr0 = com_lookup(s, side, r_com);
    }
    const double vx_com = (vr0 * x_com - vazi0 * y_com) / r_com;
    const double vy_com = (vr0 * y_com + vazi0 * x_com) / r_com;
    *vx = vx_com + c->vx;
    *vy = vy_com + c->vy;
}

/* diskmodel_center_of_mass_boundary_inner / _outer, center_of_mass.cpp:38-336 */
static void com_ghost(or_state *s, int side, const fgpu_frame_center *c)
{
    const fgpu_params *p = &s->p;
    const int nz = s->nz;
    const int i = side ? s->nr - 1 : 0;
    double *sig = s->f[FGPU_SIGMA], *en = s->f[FGPU_ENERGY];
    double *vr = s->f[FGPU_V_RADIAL], *vaz = s->f[FGPU_V_AZIMUTHAL];
    for (int j = 0; j < nz; ++j) {
	double vx, vy;
	{
	    const double phi = ((double)j - 0.5) * s->dphi;
	    const double rmed = s->Rmed[i];
	    const double cx = rmed * cos(phi), cy = rmed * sin(phi);
	    com_velocity(s, side, 0, c, cx, cy, &vx, &vy);
	    vaz[(size_t)i * nz + j] = (cx * vy - vx * cy) / rmed - s->omega_frame * rmed;
	}
	for (int k = 0; k < 2; ++k) {
	    const double phi = (double)j * s->dphi;
	    const double rr = k ? s->Rsup[i] : s->Rinf[i];
	    const double cx = rr * cos(phi), cy = rr * sin(phi);
	    com_velocity(s, side, 0, c, cx, cy, &vx, &vy);
	    vr[(size_t)(i + k) * nz + j] = (cx * vx + cy * vy) / rr;
	}
	{
	    const double cx = s->Rmed[i] * s->cosj[j], cy = s->Rmed[i] * s->sinj[j];
	    const double x_com = cx - c->x, y_com = cy - c->y;
	    const double r_com = sqrt(x_com * x_com + y_com * y_com);
	    const double cell_sigma = p->sigma0 * pow(r_com, -p->sigma_slope);
	    sig[(size_t)i * nz + j] = cell_sigma;
	    const double cell_energy = th_energy(s, r_com, c->mass);
	    const double tfloor = p->minimum_temperature * p->temperature_cgs_to_code;
	    const double efloor = tfloor * cell_sigma / p->mu * p->R_gas / (p->gamma - 1.0);
	    en[(size_t)i * nz + j] = fmax(cell_energy, efloor);
	}
    }
}

/* damping_diskmodel_center_of_mass_outer / _inner, center_of_mass.cpp:339-720 */
static void com_damp(or_state *s, int side, const fgpu_frame_center *c, double dt)
{
    const fgpu_params *p = &s->p;
    const int nr = s->nr, nz = s->nz;
    double *vr = s->f[FGPU_V_RADIAL], *vaz = s->f[FGPU_V_AZIMUTHAL], *en = s->f[FGPU_ENERGY];
    const double rin = p->rmin * p->damping_inner_limit, rout = p->rmax * p->damping_outer_limit;
    int vr_lo, vr_hi, az_lo, az_hi;
    double tau;
    if (side) {
	if (!(p->damping_outer_limit < 1.0 && s->Rinf[nr] > rout)) return;
	vr_lo = clamp_id(cell_id_rinf(s, rout), 1, nr) + 1;
	vr_hi = nr - 1; /* MaxMo_no_ghost_vr */
	az_lo = clamp_id(cell_id_rmed(s, rout), 0, nr) + 1;
	az_hi = nr - 1; /* Max_no_ghost */
	tau = p->damping_time_factor * 2.0 * M_PI / omega_kepler(s, p->damping_time_radius_outer);
    } else {
	if (!(p->damping_inner_limit > 1.0 && s->Rmed[0] < rin)) return;
	vr_lo = 2; /* One_no_ghost_vr */
	vr_hi = clamp_id(cell_id_rinf(s, rin), 1, nr) + 1;
	az_lo = 1; /* Zero_no_ghost */
	az_hi = clamp_id(cell_id_rmed(s, rin), 0, nr) + 1;
	tau = p->damping_time_factor * 2.0 * M_PI / omega_kepler(s, p->rmin);
    }
    for (int i = vr_lo; i < vr_hi; ++i) {
	const double factor = side ? pow((s->Rinf[i] - rout) / (p->rmax - rout), 2)
				   : pow((s->Rinf[i] - rin) / (p->rmin - rin), 2);
	const double ef = exp(-dt * factor / tau);
	for (int j = 0; j < nz; ++j) {
	    const double phi = (double)j * s->dphi;
	    const double rinf = s->Rinf[i];
	    const double cx = rinf * cos(phi), cy = rinf * sin(phi);
	    double vx, vy;
	    com_velocity(s, side, 1, c, cx, cy, &vx, &vy);
	    const double v0 = (cx * vx + cy * vy) / rinf;
	    double *v = &vr[(size_t)i * nz + j];
	    *v = (*v - v0) * ef + v0;
	}
    }
    for (int i = az_lo; i < az_hi; ++i) {
	/* both sides use the outer zone's profile here (center_of_mass.cpp:491-494,
	   628-631) */
	const double factor = pow((s->Rmed[i] - rout) / (p->rmax - rout), 2);
	const double ef = exp(-dt * factor / tau);
	for (int j = 0; j < nz; ++j) {
	    const double phi = ((double)j - 0.5) * s->dphi;
	    const double rmed = s->Rmed[i];
	    const double cx = rmed * cos(phi), cy = rmed * sin(phi);
	    double vx, vy;
	    com_velocity(s, side, 1, c, cx, cy, &vx, &vy);
	    const double v0 = (cx * vy - vx * cy) / rmed - s->omega_frame * rmed;
	    double *v = &vaz[(size_t)i * nz + j];
	    *v = (*v - v0) * ef + v0;
	}
    }
    if (adiabatic(s)) {
	for (int i = az_lo; i < az_hi; ++i) {
	    const double factor = pow((s->Rmed[i] - rout) / (p->rmax - rout), 2);
	    const double ef = exp(-dt * factor / tau);
	    for (int j = 0; j < nz; ++j) {
		const double cx = s->Rmed[i] * s->cosj[j], cy = s->Rmed[i] * s->sinj[j];
		const double x_com = cx - c->x, y_com = cy - c->y;
		const double r_com = sqrt(x_com * x_com + y_com * y_com);
		const double e0 = th_energy(s, r_com, c->mass);
		double *e = &en[(size_t)i * nz + j];
		*e = (*e - e0) * ef + e0;
	    }
	}
    }
}

static int com_active(const or_state *s, int side)
{
    return (side ? s->p.composite_outer : s->p.composite_inner) == FGPU_COMPOSITE_CENTER_OF_MASS;
}

static int apply_bc(or_state *s, double dt, int final, const fgpu_frame_center *c);

int or_apply_boundary_condition(or_state *s, double t, double dt, int final)
{
    (void)t;
    return apply_bc(s, dt, final, s->com_now);
}

static int apply_bc(or_state *s, double dt, int final, const fgpu_frame_center *c)
{
    const fgpu_params *p = &s->p;
    if ((com_active(s, 0) || com_active(s, 1)) && !s->com_ready) return FGPU_ERR_BAD_ARG;
    if (final && (p->viscous_accretion || p->bc_vrad_inner == FGPU_BC_VISCOUS)) {
	/* parameters::VISCOUS_ACCRETION (Interpret.cpp:704-707): c_s, H, nu of
	   the transported state before the final boundary call
	   (simulation.cpp:232-242, 432-441) */
	compute_sound_speed(s);
	compute_scale_height(s);
	update_viscosity(s);
    }
    if (final && p->damping) {
	for (int q = 0; q < 4; ++q) {
	    damp_one(s, q, 0, dt);
	    damp_one(s, q, 1, dt);
	}
	/* boundary_conditions.cpp:46-60 */
	if (com_active(s, 0)) com_damp(s, 0, &c[0], dt);
	if (com_active(s, 1)) com_damp(s, 1, &c[1], dt);
    }
    ghost_hook(s, FGPU_SIGMA, p->bc_sigma_inner, 0);
    ghost_hook(s, FGPU_SIGMA, p->bc_sigma_outer, 1);
    ghost_hook(s, FGPU_ENERGY, p->bc_energy_inner, 0);
    ghost_hook(s, FGPU_ENERGY, p->bc_energy_outer, 1);
    ghost_hook(s, FGPU_V_RADIAL, p->bc_vrad_inner, 0);
    ghost_hook(s, FGPU_V_RADIAL, p->bc_vrad_outer, 1);
    ghost_hook(s, FGPU_V_AZIMUTHAL, p->bc_vaz_inner, 0);
    ghost_hook(s, FGPU_V_AZIMUTHAL, p->bc_vaz_outer, 1);
    /* the composite after the per-field hooks, boundary_conditions.cpp:92-102 */
    if (com_active(s, 0)) com_ghost(s, 0, &c[0]);
    if (com_active(s, 1)) com_ghost(s, 1, &c[1]);
    if (final && p->keep_disk_mass_constant) {
	/* KeepDiskMassConstant right after the final boundary call
	   (simulation.cpp:246-251, 445-450): sigma *= old / new over the whole
	   grid (t_polargrid::operator*=, polargrid.cpp:496-505) */
	if (!s->mass_target_set) return FGPU_ERR_BAD_ARG;
	const double factor = s->mass_target / or_gas_total_mass(s, p->rmax);
	double *S = F(s, FGPU_SIGMA);
	const size_t n = (size_t)s->nr * s->nz;
	for (size_t k = 0; k < n; ++k) S[k] *= factor;
    }
    return FGPU_OK;
}

/* ------------------------------------------------------------------ */
/* transport: src/TransportEuler.cpp                                   */
/* ------------------------------------------------------------------ */

static double limiter(const or_state *s, double a, double b)
{
    if (s->p.flux_limiter == FGPU_LIMITER_MC) {
	/* MC_lim / minmod, :314-323 */
	double mm;
	if (a * b > 0.0) mm = fabs(a) < fabs(b) ? a : b;
	else mm = 0.0;
	const double c = 0.5 * (a + b), d = 2.0 * mm;
	if (c * d > 0.0) return fabs(c) < fabs(d) ? c : d;
	return 0.0;
    }
    /* van_leer_lim, :306-312 */
    if (a * b > 0.0) return 2.0 * a * b / (a + b);
    return 0;
}

/* compute_star_radial, :349-406 */
static void star_radial(or_state *s, const double *Q, const double *vr,
			double *Qs, double dt)
{
    const int nr = s->nr, nz = s->nz;
    double *dq = s->dq;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    if (i == 0 || i == nr - 1) {
		AT(dq, i, j) = 0.0;
	    } else {
		const double dqm = (AT(Q, i, j) - AT(Q, i - 1, j)) * s->InvDiffRmed[i];
		const double dqp = (AT(Q, i + 1, j) - AT(Q, i, j)) * s->InvDiffRmed[i + 1];
		AT(dq, i, j) = limiter(s, dqp, dqm);
	    }
	}
    }
#pragma omp parallel for
    for (int i = 1; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double v = AT(vr, i, j);
	    if (v > 0.0) {
		AT(Qs, i, j) = AT(Q, i - 1, j) +
			       (s->Rmed[i] - s->Rmed[i - 1] - v * dt) * 0.5 * AT(dq, i - 1, j);
	    } else {
		AT(Qs, i, j) = AT(Q, i, j) -
			       (s->Rmed[i + 1] - s->Rmed[i] + v * dt) * 0.5 * AT(dq, i, j);
	    }
	}
    }
    for (int j = 0; j < nz; ++j) AT(Qs, 0, j) = 0.0;
}

/* VanLeerRadial, :545-620 (monitor-only mass-flow sums omitted) */
static void van_leer_radial(or_state *s, const double *vr, double *Q, double dt)
{
    const int nr = s->nr, nz = s->nz;
    const size_t n = (size_t)nr * nz;
    for (size_t c = 0; c < n; ++c) s->work[c] = Q[c] / s->density_int[c];
    star_radial(s, s->work, vr, s->qrstar, dt);
    const double *QR = s->qrstar, *DS = s->densstar;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double varq_inf = dt * s->dphi * s->Rinf[i] * AT(QR, i, j) *
				    AT(DS, i, j) * AT(vr, i, j);
	    const double varq_sup = dt * s->dphi * s->Rsup[i] * AT(QR, i + 1, j) *
				    AT(DS, i + 1, j) * AT(vr, i + 1, j);
	    AT(Q, i, j) += (varq_inf - varq_sup) * s->InvSurf[i];
	}
    }
}

/* ComputeStarTheta, :416-466 */
static void star_theta(or_state *s, const double *Q, const double *v,
		       double *Qs, double dt)
{
    const int nr = s->nr, nz = s->nz;
    double *dq = s->dq;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	const double dxtheta = s->dphi * s->Rmed[i];
	const double invdxtheta = 1.0 / dxtheta;
	for (int j = 0; j < nz; ++j) {
	    const int jp = j == nz - 1 ? 0 : j + 1;
	    const int jm = j == 0 ? nz - 1 : j - 1;
	    const double dqm = AT(Q, i, j) - AT(Q, i, jm);
	    const double dqp = AT(Q, i, jp) - AT(Q, i, j);
	    AT(dq, i, j) = 0.5 * limiter(s, dqp, dqm) * invdxtheta;
	}
    }
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	const double dxtheta = s->dphi * s->Rmed[i];
	for (int j = 0; j < nz; ++j) {
	    const int jm = j == 0 ? nz - 1 : j - 1;
	    const double ksi = AT(v, i, j) * dt;
	    if (ksi > 0.0) {
		AT(Qs, i, j) = AT(Q, i, jm) + (dxtheta - ksi) * AT(dq, i, jm);
	    } else {
		AT(Qs, i, j) = AT(Q, i, j) - (dxtheta + ksi) * AT(dq, i, j);
	    }
	}
    }
}

/* VanLeerTheta, :630-664 */
static void van_leer_theta(or_state *s, const double *v, double *Q, double dt)
{
    const int nr = s->nr, nz = s->nz;
    const size_t n = (size_t)nr * nz;
    for (size_t c = 0; c < n; ++c) s->work[c] = Q[c] / s->density_int[c];
    star_theta(s, s->work, v, s->qrstar, dt);
    const double *QR = s->qrstar, *DS = s->densstar;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	const double dxrad = (s->Rsup[i] - s->Rinf[i]) * dt;
	const double invsurf = s->InvSurf[i];
	if (!s->uniform_transport || !s->nosplit[i]) {
	    for (int j = 0; j < nz; ++j) {
		const int jp = j == nz - 1 ? 0 : j + 1;
		double varq = dxrad * AT(QR, i, j) * AT(DS, i, j) * AT(v, i, j);
		varq -= dxrad * AT(QR, i, jp) * AT(DS, i, jp) * AT(v, i, jp);
		AT(Q, i, j) += varq * invsurf;
	    }
	}
    }
}

/* QuantitiesAdvection, :292-304 */
static void quantities_advection(or_state *s, const double *v, double dt)
{
    double *S = F(s, FGPU_SIGMA);
    star_theta(s, S, v, s->densstar, dt);
    memcpy(s->density_int, S, sizeof(double) * (size_t)s->nr * s->nz);
    van_leer_theta(s, v, s->rmp, dt);
    van_leer_theta(s, v, s->rmm, dt);
    van_leer_theta(s, v, s->amp, dt);
    van_leer_theta(s, v, s->amm, dt);
    if (adiabatic(s)) van_leer_theta(s, v, F(s, FGPU_ENERGY), dt);
    van_leer_theta(s, v, S, dt);
}

/* AdvectSHIFT, :238-268 */
static void advect_shift(or_state *s, double *val)
{
    const int nr = s->nr, nz = s->nz;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    int ji = j - s->nshift[i];
	    while (ji < 0) ji += nz;
	    while (ji >= nz) ji -= nz;
	    AT(s->tempshift, i, j) = AT(val, i, ji);
	}
    }
    memcpy(val, s->tempshift, sizeof(double) * (size_t)nr * nz);
}

void or_transport(or_state *s, double dt)
{
    const int nr = s->nr, nz = s->nz;
    double *S = F(s, FGPU_SIGMA), *vr = F(s, FGPU_V_RADIAL),
	   *vaz = F(s, FGPU_V_AZIMUTHAL), *E = F(s, FGPU_ENERGY);
    const double OmegaF = s->omega_frame;

    /* compute_momenta_from_velocities, :471-493 */
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    AT(s->rmp, i, j) = AT(S, i, j) * AT(vr, i + 1, j);
	    AT(s->rmm, i, j) = AT(S, i, j) * AT(vr, i, j);
	    const int jn = j == nz - 1 ? 0 : j + 1;
	    const double r = s->Rmed[i];
	    AT(s->amp, i, j) = AT(S, i, j) * (AT(vaz, i, jn) + r * OmegaF) * r;
	    AT(s->amm, i, j) = AT(S, i, j) * (AT(vaz, i, j) + r * OmegaF) * r;
	}
    }

    /* OneWindRad, :138-167 */
    star_radial(s, S, vr, s->densstar, dt);
    memcpy(s->density_int, S, sizeof(double) * (size_t)nr * nz);
    van_leer_radial(s, vr, s->rmp, dt);
    van_leer_radial(s, vr, s->rmm, dt);
    van_leer_radial(s, vr, s->amp, dt);
    van_leer_radial(s, vr, s->amm, dt);
    if (adiabatic(s)) van_leer_radial(s, vr, E, dt);
    van_leer_radial(s, vr, S, dt);

    /* OneWindTheta, :270-288 */
    for (int i = 0; i < nr; ++i) {
	/* compute_average_azimuthal_velocity, :174-189 */
	double sum = 0.0;
	for (int j = 0; j < nz; ++j) sum += AT(vaz, i, j);
	s->vmean[i] = sum / (double)nz;
    }
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) AT(s->vres, i, j) = AT(vaz, i, j) - s->vmean[i];
    }
    /* ComputeConstantResidual, :207-236 */
    const double invdt = 1.0 / dt;
    for (int i = 0; i < nr; ++i) {
	const double Ntilde = s->vmean[i] * s->InvRmed[i] * dt * s->invdphi;
	const double Nround = floor(Ntilde + 0.5);
	s->nshift[i] = (int)Nround;
	for (int j = 0; j < nz; ++j) {
	    AT(vaz, i, j) = (Ntilde - Nround) * s->Rmed[i] * invdt * s->dphi;
	}
	if (!s->p.fast_transport) {
	    s->nosplit[i] = 1;
	    for (int j = 0; j < nz; ++j) {
		AT(s->vres, i, j) = AT(vaz, i, j) + AT(s->vres, i, j);
		AT(vaz, i, j) = 0.0;
	    }
	} else {
	    s->nosplit[i] = 0;
	}
    }
    s->uniform_transport = 0;
    quantities_advection(s, s->vres, dt);
    s->uniform_transport = 1;
    quantities_advection(s, vaz, dt);
    advect_shift(s, s->rmp);
    advect_shift(s, s->rmm);
    advect_shift(s, s->amp);
    advect_shift(s, s->amm);
    if (adiabatic(s)) advect_shift(s, E);
    advect_shift(s, S);

    /* compute_velocities_from_momenta, :498-535 */
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const int jm = j == 0 ? nz - 1 : j - 1;
	    if (i == 0) {
		AT(vr, i, j) = 0.0;
	    } else {
		AT(vr, i, j) = (AT(s->rmp, i - 1, j) + AT(s->rmm, i, j)) /
			       (AT(S, i - 1, j) + AT(S, i, j));
	    }
	    AT(vaz, i, j) = (AT(s->amp, i, jm) + AT(s->amm, i, j)) /
				(AT(S, i, jm) + AT(S, i, j)) * s->InvRmed[i] -
			    s->Rmed[i] * OmegaF;
	}
    }
    /* assure_minimum_value(SIGMA, sigma_floor * sigma0), SourceEuler.cpp:102-134 */
    const double smin = s->p.sigma_floor * s->p.sigma0;
    const size_t n = (size_t)nr * nz;
#pragma omp parallel for
    for (size_t c = 0; c < n; ++c) {
	if (S[c] < smin) S[c] = smin;
    }
    if (adiabatic(s)) assure_temperature_range(s);
}

/* ------------------------------------------------------------------ */
/* step, init, CFL, forces                                             */
/* ------------------------------------------------------------------ */

/* The gas kick of step_Euler (src/simulation.cpp:170-203) and of each half
   of step_LeapFrog (:312-331, :352-384): potential, source terms, artificial
   viscosity, viscosity, viscous stress and velocity update, SubStep3. */
void or_gas_kick(or_state *s, double dt, double t)
{
    or_calculate_potential(s);
    or_update_with_sourceterms(s, dt);
    or_artificial_viscosity(s, dt);
    or_recalculate_viscosity(s, t);
    or_viscous_stress_tensor(s);
    or_update_velocities_with_viscosity(s, dt);
    if (adiabatic(s)) or_substep3(s, t, dt);
}

int or_step_euler(or_state *s, double dt, double t)
{
    if ((com_active(s, 0) || com_active(s, 1)) && !s->com_ready) return FGPU_ERR_BAD_ARG;
    or_gas_kick(s, dt, t);
    apply_bc(s, 0.0, 0, s->com_now);
    or_transport(s, dt);
    /* the final call sees the bodies after the N-body step (simulation.cpp:219-244) */
    const int rc = apply_bc(s, dt, 1, s->com_after);
    if (rc) return rc;
    or_recalculate_derived(s, t + dt);
    return FGPU_OK;
}

int or_init_euler(or_state *s, double t)
{
    /* init_euler, src/SourceEuler.cpp:251-285 (AspectRatioMode 0) */
    if (adiabatic(s)) {
	compute_temperature(s);
	compute_sound_speed(s);
	compute_scale_height(s);
	or_compute_pressure(s);
    } else {
	compute_sound_speed(s);
	or_compute_pressure(s);
	compute_temperature(s);
	compute_scale_height(s);
    }
    update_viscosity(s);
    /* compute_heating_cooling_for_CFL, :1410-1450 */
    if (adiabatic(s)) {
	update_viscosity(s);
	or_viscous_stress_tensor(s);
	calculate_qminus(s, t);
	calculate_qplus(s);
	const int nr = s->nr, nz = s->nz;
	double *Qp = F(s, FGPU_QPLUS), *Qm = F(s, FGPU_QMINUS),
	       *E = F(s, FGPU_ENERGY), *S = F(s, FGPU_SIGMA),
	       *H = F(s, FGPU_SCALE_HEIGHT);
	for (int i = 1; i < nr - 1; ++i) {
	    for (int j = 0; j < nz; ++j) {
		const double a = rad_alpha(s, AT(H, i, j), AT(S, i, j), AT(E, i, j));
		AT(Qp, i, j) /= a;
		AT(Qm, i, j) /= a;
	    }
	}
    }
    return FGPU_OK;
}

/* cfl::condition_cfl, src/cfl.cpp:185-382; the LeapFrog integrator allows
   the source-term limits (artificial viscosity, viscosity, heating/cooling)
   a 0.6 factor (:254-317) */
/* The time step of cell (i, j), cfl.cpp:185-382: the six inverse times
   (LeapFrog's 0.6 on the last three) into inv[], CFL over the root of their
   squares, and StabilizeViscosity 2's limit. */
static double cfl_cell(const or_state *s, int i, int j, double vm_i, double inv[6])
{
    const int nz = s->nz;
    const double *vr = F(s, FGPU_V_RADIAL), *vaz = F(s, FGPU_V_AZIMUTHAL),
         *cs = F(s, FGPU_SOUNDSPEED), *nu = F(s, FGPU_VISCOSITY),
         *Qp = F(s, FGPU_QPLUS), *Qm = F(s, FGPU_QMINUS), *E = F(s, FGPU_ENERGY);
    const fgpu_params *p = &s->p;
    const double lf = p->integrator == FGPU_INTEGRATOR_LEAPFROG ? 0.6 : 1.0;
    const double dxR = s->Rsup[i] - s->Rinf[i];
    const double dxA = s->Rmed[i] * s->dphi;
    const double cell = dxR < dxA ? dxR : dxA;
    const double vres = p->fast_transport ? AT(vaz, i, j) - vm_i : AT(vaz, i, j);
    const double invdt1 = AT(cs, i, j) / cell;
    const double invdt2 = AT(vr, i, j) / dxR;
    const double invdt3 = vres / dxA;
    const int jn = j == nz - 1 ? 0 : j + 1;
    double invdt4;
    if (p->art_visc == FGPU_ARTVISC_SN) {
        double dvR = AT(vr, i + 1, j) - AT(vr, i, j);
        double dvA = AT(vaz, i, jn) - AT(vaz, i, j);
        dvR = dvR > 0.0 ? 0.0 : -dvR;
        dvA = dvA > 0.0 ? 0.0 : -dvA;
        const double a = dvR / dxR, b = dvA / dxA;
        invdt4 = 4.0 * pow(p->art_visc_factor, 2) * (a > b ? a : b) * lf;
    } else {
        const double eps_rr = (AT(vr, i + 1, j) - AT(vr, i, j)) * s->InvDiffRsup[i];
        const double eps_pp =
            s->InvRmed[i] * ((AT(vaz, i, jn) - AT(vaz, i, j)) * s->invdphi +
        		     0.5 * (AT(vr, i + 1, j) + AT(vr, i, j)));
        const double d = eps_rr + eps_pp;
        const double mdiv = -(d < 0.0 ? d : 0.0);
        invdt4 = 4.0 * pow(p->art_visc_factor, 2) * mdiv * lf;
    }
    const double invdt5 = 4.0 * AT(nu, i, j) / pow(cell, 2) * lf;
    double invdt6 = 0.0;
    if (adiabatic(s)) {
        const double inv_limit = 1.0 / p->heating_cooling_cfl_limit;
        invdt6 = inv_limit * fabs((AT(Qp, i, j) - AT(Qm, i, j)) / AT(E, i, j)) * lf;
    }
    double dt_cell =
        p->cfl / sqrt(pow(invdt1, 2) + pow(invdt2, 2) + pow(invdt3, 2) +
        	      pow(invdt4, 2) + pow(invdt5, 2) + pow(invdt6, 2));
    if (p->stabilize_viscosity == 2) {
        /* cfl.cpp:332-351 */
        const double cphi = AT(s->corr_phi, i, j), cr = AT(s->corr_r, i, j);
        const double c = cphi < cr ? cphi : cr;
        if (c != 0.0) {
            const double dt_stable = -p->cfl / c;
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

double or_condition_cfl(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *vaz = F(s, FGPU_V_AZIMUTHAL);
    const fgpu_params *p = &s->p;
    double *vm = s->vmean;
#pragma omp parallel for
    for (int i = 0; i < nr; ++i) {
	vm[i] = 0.0;
	for (int j = 0; j < nz; ++j) vm[i] += AT(vaz, i, j);
	vm[i] /= (double)nz;
    }
    const double denom0 =
	fabs(vm[0] * s->InvRmed[0] - vm[1] * s->InvRmed[1]) + 1.0e-100;
    double dt_core = p->cfl * s->dphi / denom0;
#pragma omp parallel for reduction(min : dt_core)
    for (int i = 1; i < nr - 1; ++i) {
	const double denom =
	    fabs(vm[i] * s->InvRmed[i] - vm[i + 1] * s->InvRmed[i + 1]) + 1.0e-100;
	const double shear_dt = p->cfl * s->dphi / denom;
	if (shear_dt < dt_core) dt_core = shear_dt;
	for (int j = 0; j < nz; ++j) {
	    double inv[6];
	    const double dt_cell = cfl_cell(s, i, j, vm[i], inv);
	    if (dt_cell < dt_core) dt_core = dt_cell;
	}
    }
    return dt_core;
}

/* The limiting cell of the CFL step (timestep_debug_report, cfl.cpp:38-182):
   the smallest cell time step on rings 1 .. nr - 2 (the first in ring-major
   order on ties) with its inverse times, and the smallest ring shear limit
   (rings 0 .. nr - 2). */
int or_cfl_limiting_cell(or_state *s, fgpu_cfl_cell *out)
{
    const int nr = s->nr, nz = s->nz;
    const double *vaz = F(s, FGPU_V_AZIMUTHAL);
    const fgpu_params *p = &s->p;
    double *vm = s->vmean;
    for (int i = 0; i < nr; ++i) {
	vm[i] = 0.0;
	for (int j = 0; j < nz; ++j) vm[i] += AT(vaz, i, j);
	vm[i] /= (double)nz;
    }
    memset(out, 0, sizeof(*out));
    out->ring = out->azimuth = out->shear_ring = -1;
    out->dt_cell = out->dt_shear = 1.0e300;
    for (int i = 0; i < nr - 1; ++i) {
	const double denom =
	    fabs(vm[i] * s->InvRmed[i] - vm[i + 1] * s->InvRmed[i + 1]) + 1.0e-100;
	const double shear_dt = p->cfl * s->dphi / denom;
	if (shear_dt < out->dt_shear) {
	    out->dt_shear = shear_dt;
	    out->shear_ring = i;
	}
	if (i < 1) continue;
	for (int j = 0; j < nz; ++j) {
	    double inv[6];
	    const double dt_cell = cfl_cell(s, i, j, vm[i], inv);
	    if (dt_cell < out->dt_cell) {
		out->dt_cell = dt_cell;
		out->ring = i;
		out->azimuth = j;
		for (int k = 0; k < 6; ++k) out->invdt[k] = inv[k];
	    }
	}
    }
    return FGPU_OK;
}

/* ComputeDiskOnPlanetAccel, src/Force.cpp:23-122; with CorrectDiskSelfgravity
   (FargoCPT's default without self-gravity) the ring-mean density is
   subtracted (Force.cpp:64-66). */
int or_disk_on_planet_accel(or_state *s, int k, double accel[2])
{
    if (k < 0 || k >= s->nb) return FGPU_ERR_BAD_ARG;
    const int nr = s->nr, nz = s->nz;
    double *S = F(s, FGPU_SIGMA), *H = F(s, FGPU_SCALE_HEIGHT);
    for (int i = 1; i < nr - 1; ++i) {
	double sum = 0;
	for (int j = 0; j < nz; ++j) sum += AT(S, i, j);
	s->sigma1d[i] = sum / nz;
    }
    const double x = s->b[k].x, y = s->b[k].y, a = s->b[k].a, r_sm = s->b[k].r_sm;
    const double G = s->p.G;
    double axi = 0, ayi = 0, axo = 0, ayo = 0;
#pragma omp parallel for reduction(+ : axi, ayi, axo, ayo)
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    const double smooth = s->p.thickness_smoothing * AT(H, i, j);
	    const double xc = s->Rmed[i] * s->cosj[j];
	    const double yc = s->Rmed[i] * s->sinj[j];
	    double cell_sigma = AT(S, i, j);
	    if (s->p.correct_disk_selfgravity) cell_sigma -= s->sigma1d[i];
	    const double cellmass = s->Surf[i] * cell_sigma;
	    const double dx = xc - x, dy = yc - y;
	    const double d2 = pow(dx, 2) + pow(dy, 2);
	    const double dsm2 = d2 + pow(smooth, 2);
	    const double dsm = sqrt(dsm2);
	    const double dsm3 = dsm2 * dsm;
	    const double inv3 = 1.0 / dsm3;
	    double fk = 1.0;
	    if (r_sm > 0.0 && dsm < r_sm) {
		fk = -(3.0 * pow(dsm / r_sm, 4.0) - 4.0 * pow(dsm / r_sm, 3.0));
	    }
	    if (s->Rmed[i] < a) {
		axi += G * cellmass * dx * inv3 * fk;
		ayi += G * cellmass * dy * inv3 * fk;
	    } else {
		axo += G * cellmass * dx * inv3 * fk;
		ayo += G * cellmass * dy * inv3 * fk;
	    }
	}
    }
    accel[0] = axi + axo;
    accel[1] = ayi + ayo;
    return FGPU_OK;
}

/* quantities::gas_total_mass over the active rings, src/quantities.cpp:51-74 */
double or_total_mass(or_state *s)
{
    const int nr = s->nr, nz = s->nz;
    double *S = F(s, FGPU_SIGMA);
    double m = 0.0;
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) m += s->Surf[i] * AT(S, i, j);
    }
    return m;
}

/* quantities::gas_total_mass, src/quantities.cpp:51-74: the active rings
   with Rmed <= radius, ring-major (the order of a one-thread run) */
double or_gas_total_mass(or_state *s, double radius)
{
    const int nr = s->nr, nz = s->nz;
    const double *S = F(s, FGPU_SIGMA);
    double m = 0.0;
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    if (s->Rmed[i] <= radius) m += s->Surf[i] * AT(S, i, j);
	}
    }
    return m;
}

/* quantities::gas_angular_momentum, src/quantities.cpp:242-276: sigma
   averaged onto the v_phi interface (j and j - 1, periodic), times Rmed and
   the inertial azimuthal speed v_phi + OmegaFrame Rmed */
double or_gas_angular_momentum(or_state *s, double radius)
{
    const int nr = s->nr, nz = s->nz;
    const double *S = F(s, FGPU_SIGMA), *V = F(s, FGPU_V_AZIMUTHAL);
    double L = 0.0;
    for (int i = 1; i < nr - 1; ++i) {
	for (int j = 0; j < nz; ++j) {
	    if (s->Rmed[i] <= radius) {
		const int jm = j == 0 ? nz - 1 : j - 1;
		L += s->Surf[i] * 0.5 * (AT(S, i, j) + AT(S, i, jm)) * s->Rmed[i] *
		     (AT(V, i, j) + s->omega_frame * s->Rmed[i]);
	    }
	}
    }
    return L;
}

int or_set_disk_mass_target(or_state *s, double mass)
{
    s->mass_target = mass;
    s->mass_target_set = 1;
    return FGPU_OK;
}

/* ------------------------------------------------------------------ */
/* accretion::AccreteOntoPlanets for one planet, src/accretion.cpp:21-480 */
/* ------------------------------------------------------------------ */
static int med_azimuthal_id(const or_state *s, double phi)
{
    /* get_med_azimuthal_id, find_cell_id.cpp:322-345 (init_cell_finder_*:
       phi_cell_size = 2 pi / Naz, inv_phi_cell_size = Naz / 2 / pi) */
    const double cell = 2.0 * M_PI / (double)s->nz;
    const double inv = (double)s->nz / 2.0 / M_PI;
    return (int)floor((phi - 0.5 * cell) * inv);
}

int or_accrete_onto_planet(or_state *s, const fgpu_accretor *a, double dt, double out[3])
{
    const int nr = s->nr, ns = s->nz;
    double *dens = F(s, FGPU_SIGMA), *energy = F(s, FGPU_ENERGY);
    const double *vrad = F(s, FGPU_V_RADIAL), *vazi = F(s, FGPU_V_AZIMUTHAL);
    const double *nuf = F(s, FGPU_VISCOSITY);
    const double density_floor = s->p.sigma_floor * s->p.sigma0;
    const double RHill = a->roche_radius;
    const double Rplanet = a->r;
    double frac1, frac2 = 0.0, facc1, facc2 = 0.0, f_const = 0.0, dist_max = 0.0;
    const double frac = s->p.accretion_radius_fraction;
    if (a->type == FGPU_ACCRETION_KLEY) {
	/* AccreteOntoSinglePlanet, :84-221 */
	const double facc = dt * a->efficiency / a->orbital_period * log(2);
	facc1 = 1.0 / 3.0 * facc;
	facc2 = 2.0 / 3.0 * facc;
	frac1 = frac;
	frac2 = 0.5 * frac;
    } else if (a->type == FGPU_ACCRETION_SINKHOLE) {
	/* SinkHoleSinglePlanet, :223-333 */
	facc1 = dt * a->efficiency / a->orbital_period * log(2.0);
	frac1 = frac;
    } else if (a->type == FGPU_ACCRETION_VISCOUS) {
	/* AccreteOntoSinglePlanetViscous, :335-480 */
	facc1 = dt * 3.0 * M_PI * a->efficiency;
	frac1 = frac;
	dist_max = RHill * frac;
	f_const = 3.0 / M_PI / pow(dist_max, 2);
    } else {
	return FGPU_ERR_BAD_ARG;
    }
    const double search_radius = RHill * frac1 + 2.0 * Rplanet / ns;
    /* hill_radial_index, :21-38 */
    int i_min;
    if (Rplanet - search_radius < s->p.rmin) {
	i_min = 0;
    } else {
	i_min = clamp_id(cell_id_rinf(s, Rplanet - search_radius), 0, nr);
    }
    const int i_max = clamp_id(cell_id_rinf(s, Rplanet + search_radius) + 1, 0, nr);
    /* hill_azimuthal_index, :40-58 */
    double max_angle;
    if (Rplanet == 0.0) {
	max_angle = 2.0 * M_PI;
    } else {
	const double m = 2.0 * search_radius / Rplanet;
	max_angle = m < 2.0 * M_PI ? m : 2.0 * M_PI;
    }
    const int j_min = med_azimuthal_id(s, a->phi - max_angle);
    int j_max = med_azimuthal_id(s, a->phi + max_angle) + 1;
    j_max = j_min + (j_max - j_min < ns - 1 ? j_max - j_min : ns - 1);

    double dM = 0.0, dPx = 0.0, dPy = 0.0;
    for (int i = i_min; i <= i_max; i++) {
	for (int j = j_min; j <= j_max; j++) {
	    int jf = j;
	    while (jf < 0) jf += ns;
	    while (jf >= ns) jf -= ns;
	    const int l = jf + i * ns;
	    const int lip = l + ns;
	    const int ljp = jf == ns - 1 ? i * ns : l + 1;
	    const double xc = s->Rmed[i] * s->cosj[jf];
	    const double yc = s->Rmed[i] * s->sinj[jf];
	    const double dx = a->x - xc;
	    const double dy = a->y - yc;
	    const double distance = sqrt(dx * dx + dy * dy);
	    const double vtcell = 0.5 * (vazi[l] + vazi[ljp]) + s->Rmed[i] * s->omega_frame;
	    const double vrcell = 0.5 * (vrad[l] + vrad[lip]);
	    const double vxcell = (vrcell * xc - vtcell * yc) / s->Rmed[i];
	    const double vycell = (vrcell * yc + vtcell * xc) / s->Rmed[i];
	    const double facc_max = 1 - density_floor / dens[l];
	    const int active = 1 < i && i < nr - 1;
	    if (distance < frac1 * RHill) {
		double f = facc1;
		if (a->type == FGPU_ACCRETION_VISCOUS) {
		    const double spread = f_const * (1.0 - distance / dist_max);
		    f = facc1 * nuf[l] * spread;
		}
		const double fc = facc_max < f ? facc_max : f;
		const double deltaM = fc * dens[l] * s->Surf[i];
		dens[l] *= 1.0 - fc;
		if (adiabatic(s)) energy[l] *= 1.0 - fc;
		if (active) {
		    dPx += deltaM * vxcell;
		    dPy += deltaM * vycell;
		    dM += deltaM;
		}
	    }
	    if (a->type == FGPU_ACCRETION_KLEY && distance < frac2 * RHill) {
		const double fc = facc_max < facc2 ? facc_max : facc2;
		const double deltaM = fc * dens[l] * s->Surf[i];
		dens[l] *= 1.0 - fc;
		/* the reference scales the energy by the uncapped factor here */
		if (adiabatic(s)) energy[l] *= 1.0 - facc2;
		if (active) {
		    dPx += deltaM * vxcell;
		    dPy += deltaM * vycell;
		    dM += deltaM;
		}
	    }
	}
    }
    out[0] = dM;
    out[1] = dPx;
    out[2] = dPy;
    return FGPU_OK;
}
