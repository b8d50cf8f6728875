// The centre-of-mass composite boundary (boundary_conditions/center_of_mass.cpp):
// the initial disk model about the centre of mass of a set of bodies,
// imposed on the ghost ring of an edge (:38-336) and, in the final boundary
// call with damping on, damped towards in the edge's damping zone (:339-720).
//
// The model about the centre: sigma0 r^-S, the locally isothermal energy
// (Theo.cpp:86-99), the pressure-supported smoothed v_phi (Theo.cpp:131-200;
// the quadrupole term at the outer edge only) with the viscous v_r of the
// lookup tables (viscosity/viscous_radial_speed.cpp:350-407), or with
// InitializePureKeplerian the Keplerian v_phi and the steady viscous v_r
// (Theo.cpp:207-243).  Velocities are rotated into the primary's frame and
// shifted by the centre's velocity.  Side 0 is the inner edge (the first
// n_bodies_for_hydroframe_center bodies), side 1 the outer edge (all bodies).
//
// The model is evaluated in FP64 in both forms; a field policy (ComFields64,
// ComFields32) reads and writes the form's own representation.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

struct ComCenter {
    double x, y, vx, vy, mass;  // get_center_of_mass(n), _velocity(n), get_mass(n)
};

struct ComSpec {
    int active[2];              // composite "centerofmass" on this side
    int pure_keplerian;         // InitializePureKeplerian
    int vr_zero;                // InitializeVradialZero (damping model, Keplerian only)
    int adiabatic;
    double G, h0, F, S, eps, Q; // Q: quadrupole moment, outer model only
    double sigma0, gamma_m1;
    double alpha, nu_const, sqrt_gamma;
    double energy_floor;        // temperature floor * (R / mu) / (gamma - 1), per unit sigma
    double omf;
    int n;                      // nodes per viscous-speed table (+ 1 stored)
    double min_r[2], dlog[2];
    const double *r_tab[2], *vr_tab[2];
    const double *Rinf, *Rsup, *Rmed; // ring radii
    const double *cos_j, *sin_j;      // cos / sin (j dphi)
    const double *cos_h, *sin_h;      // cos / sin ((j - 1/2) dphi)
    // damping: rings [vr_lo, vr_hi) of v_radial and [az_lo, az_hi) of
    // v_azimuthal and energy; per-ring ((r - r_lim) / (r_edge - r_lim))^2
    int vr_lo[2], vr_hi[2], az_lo[2], az_hi[2];
    double tau[2];
    const double *fac_vr[2], *fac_az[2];
    ComCenter c[2];
};

__device__ inline double com_vaz_model(const ComSpec &c, double R, double M, int side)
{
    const double h = c.h0 * pow(R, c.F);
    const double he = h * c.eps;
    const double sq = sqrt(1 + he * he);
    const double smooth = (1.0 + (c.F + 1.0) * (he * he)) / (sq * sq * sq);
    const double press = (2.0 * c.F - 1.0 - c.S) * (h * h);
    double support = smooth + press;
    if (side == 1) support = (c.Q > 0.0 ? 3.0 * c.Q / (R * R) : 0.0) + smooth + press;
    return sqrt(c.G * M / R * support);
}

__device__ inline double com_vr_steady(const ComSpec &c, double R, double M)
{
    if (c.alpha > 0) {
        const double v_k = sqrt(c.G * M / R);
        const double h = c.h0 * pow(R, c.F);
        const double nu = c.alpha * (c.sqrt_gamma * h * v_k) * (h * R);
        return -3.0 * nu / R * (-c.S + 2.0 * c.F + 1.0);
    }
    return -3.0 * c.nu_const / R * (-c.S + .5);
}

__device__ inline double com_vr_lookup(const ComSpec &c, int side, double r)
{
    const int i = (int)floor(log10(r / c.min_r[side]) / c.dlog[side]);
    const double *rt = c.r_tab[side], *vt = c.vr_tab[side];
    if (i > c.n - 1) return vt[c.n - 1];
    if (i < 0) return vt[0];
    // the tables hold n + 1 nodes, so that the last bin has a right node
    const double x = (r - rt[i]) / (rt[i + 1] - rt[i]);
    return (1.0 - x) * vt[i] + x * vt[i + 1];
}

// the model velocity (vx, vy) in the primary's frame at (px, py)
__device__ inline void com_velocity(const ComSpec &c, int side, bool damping, double px,
                                    double py, double &vx, double &vy)
{
    const ComCenter &m = c.c[side];
    const double xc = px - m.x, yc = py - m.y;
    const double r = sqrt(xc * xc + yc * yc);
    double vaz0, vr0;
    if (c.pure_keplerian) {
        vaz0 = sqrt(c.G * m.mass / r);
        vr0 = (damping && c.vr_zero) ? 0.0 : com_vr_steady(c, r, m.mass);
    } else {
        vaz0 = com_vaz_model(c, r, m.mass, side);
        vr0 = com_vr_lookup(c, side, r);
    }
    vx = (vr0 * xc - vaz0 * yc) / r + m.vx;
    vy = (vr0 * yc + vaz0 * xc) / r + m.vy;
}

__device__ inline double com_energy_model(const ComSpec &c, double r, double M)
{
    return 1.0 / c.gamma_m1 * c.sigma0 * (c.h0 * c.h0) * pow(r, -c.S - 1.0 + 2.0 * c.F) * c.G * M;
}

// FP64 fields
struct ComFields64 {
    double *sigma, *vr, *vaz, *energy;
    __device__ double get_vr(int nz, int i, int j) const { return vr[(size_t)i * nz + j]; }
    __device__ void set_vr(int nz, int i, int j, double v) const { vr[(size_t)i * nz + j] = v; }
    __device__ double get_vaz(int nz, int i, int j) const { return vaz[(size_t)i * nz + j]; }
    __device__ void set_vaz(int nz, int i, int j, double v) const { vaz[(size_t)i * nz + j] = v; }
    __device__ double get_energy(int nz, int i, int j) const { return energy[(size_t)i * nz + j]; }
    __device__ void set_energy(int nz, int i, int j, double v) const
    {
        energy[(size_t)i * nz + j] = v;
    }
    __device__ void set_sigma(int nz, int i, int j, double v) const { sigma[(size_t)i * nz + j] = v; }
};

// FP32-mixed fields: sigma as a compensated pair, v_phi as the residual about
// the ring's inertial Keplerian speed (frame v_phi = vref + dv - rmed omega)
struct ComFields32 {
    float *sigma, *sigma_lo, *vr, *dv, *energy;
    const double *vref, *rmed;
    double omega;
    __device__ double get_vr(int nz, int i, int j) const { return (double)vr[(size_t)i * nz + j]; }
    __device__ void set_vr(int nz, int i, int j, double v) const { vr[(size_t)i * nz + j] = (float)v; }
    __device__ double get_vaz(int nz, int i, int j) const
    {
        return vref[i] - rmed[i] * omega + (double)dv[(size_t)i * nz + j];
    }
    __device__ void set_vaz(int nz, int i, int j, double v) const
    {
        dv[(size_t)i * nz + j] = (float)(v - (vref[i] - rmed[i] * omega));
    }
    __device__ double get_energy(int nz, int i, int j) const
    {
        return (double)energy[(size_t)i * nz + j];
    }
    __device__ void set_energy(int nz, int i, int j, double v) const
    {
        energy[(size_t)i * nz + j] = (float)v;
    }
    __device__ void set_sigma(int nz, int i, int j, double v) const
    {
        const float hi = (float)v;
        sigma[(size_t)i * nz + j] = hi;
        sigma_lo[(size_t)i * nz + j] = (float)(v - (double)hi);
    }
};

// ghost ring of each active side: v_phi, v_r on both faces of the ring,
// sigma and energy (blockIdx.y = side)
template <class Fields>
__global__ void k_com_boundary(ComSpec c, int nz, int nr, Fields f)
{
    const int side = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (!c.active[side] || j >= nz) return;
    const int i = side ? nr - 1 : 0;
    double vx, vy;
    {
        const double rm = c.Rmed[i];
        const double px = rm * c.cos_h[j], py = rm * c.sin_h[j];
        com_velocity(c, side, false, px, py, vx, vy);
        f.set_vaz(nz, i, j, (px * vy - vx * py) / rm - c.omf * rm);
    }
    for (int k = 0; k < 2; ++k) {
        const double ri = k ? c.Rsup[i] : c.Rinf[i];
        const double px = ri * c.cos_j[j], py = ri * c.sin_j[j];
        com_velocity(c, side, false, px, py, vx, vy);
        f.set_vr(nz, i + k, j, (px * vx + py * vy) / ri);
    }
    const ComCenter &m = c.c[side];
    const double xc = c.Rmed[i] * c.cos_j[j] - m.x, yc = c.Rmed[i] * c.sin_j[j] - m.y;
    const double r = sqrt(xc * xc + yc * yc);
    const double sig = c.sigma0 * pow(r, -c.S);
    f.set_sigma(nz, i, j, sig);
    f.set_energy(nz, i, j, fmax(com_energy_model(c, r, m.mass), c.energy_floor * sig));
}

// damping of one side towards the model (v_r, v_phi, and energy with the
// ideal EOS; sigma is not damped); blockIdx.y = ring
template <class Fields>
__global__ void k_com_damping(ComSpec c, int nz, int side, double dt, Fields f)
{
    const int i = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nz) return;
    double vx, vy;
    if (i >= c.vr_lo[side] && i < c.vr_hi[side]) {
        const double ef = exp(-dt * c.fac_vr[side][i] / c.tau[side]);
        const double ri = c.Rinf[i];
        const double px = ri * c.cos_j[j], py = ri * c.sin_j[j];
        com_velocity(c, side, true, px, py, vx, vy);
        const double v0 = (px * vx + py * vy) / ri;
        f.set_vr(nz, i, j, (f.get_vr(nz, i, j) - v0) * ef + v0);
    }
    if (i >= c.az_lo[side] && i < c.az_hi[side]) {
        const double ef = exp(-dt * c.fac_az[side][i] / c.tau[side]);
        const double rm = c.Rmed[i];
        const double px = rm * c.cos_h[j], py = rm * c.sin_h[j];
        com_velocity(c, side, true, px, py, vx, vy);
        const double v0 = (px * vy - vx * py) / rm - c.omf * rm;
        f.set_vaz(nz, i, j, (f.get_vaz(nz, i, j) - v0) * ef + v0);
        if (c.adiabatic) {
            const ComCenter &m = c.c[side];
            const double xc = rm * c.cos_j[j] - m.x, yc = rm * c.sin_j[j] - m.y;
            const double e0 = com_energy_model(c, sqrt(xc * xc + yc * yc), m.mass);
            f.set_energy(nz, i, j, (f.get_energy(nz, i, j) - e0) * ef + e0);
        }
    }
}

// inner edge first, as handle_damping calls them (boundary_conditions.cpp:47-60)
template <class Fields>
inline void launch_com_damping_sides(const ComSpec &c, int nz, double dt, const Fields &f,
                                     cudaStream_t stream)
{
    for (int side = 0; side < 2; ++side) {
        const int hi = c.vr_hi[side] > c.az_hi[side] ? c.vr_hi[side] : c.az_hi[side];
        if (!c.active[side] || hi <= 0) continue;
        k_com_damping<<<dim3((nz + 127) / 128, hi), 128, 0, stream>>>(c, nz, side, dt, f);
    }
}
