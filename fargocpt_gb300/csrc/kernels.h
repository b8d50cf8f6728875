// Host-side launchers of the FP64 hydro kernels (kernels_fp64.cu).
#pragma once

#include "hydro.cuh"

#include <stddef.h>

// raises a kernel's dynamic shared-memory limit, never lowers it (api.cu)
cudaError_t raise_smem_limit(const void *fn, size_t bytes);

namespace fgpu {

struct Launch {
    Geo g;
    Tables t;
    Phys ph;
    cudaStream_t stream;
    int bx;  // threads per block along the azimuth for cell kernels
    // the kernels' arithmetic in float pairs (kernels_pair.cu and the pair
    // transports) instead of FP64, with FP64 state updates
    bool pair = false;
};

void launch_potential(const Launch &L, const Bodies &b, const double *H, double *pot);
void launch_source(const Launch &L, double dt, double omf, const double *S, const double *P,
                   const double *pot, const double *vr_in, const double *vaz_in, double *vr_out,
                   double *vaz_out);
void launch_artvisc_q(const Launch &L, double dt, const double *S, const double *vr,
                      const double *vaz, double *E, double *Qr, double *Qp);
void launch_artvisc_v(const Launch &L, double dt, const double *S, const double *E,
                      const double *Qr, const double *Qp, double *vr, double *vaz, double *cs,
                      double *H, double *nu);
void launch_stress(const Launch &L, const double *S, const double *vr, const double *vaz,
                   const double *nu, double *divv, double *trr, double *tpp, double *trp);
void launch_viscous(const Launch &L, double dt, double beta_inv, int mode, const State &s);
void launch_visc_corr(const Launch &L, const State &s);
void launch_ghost(const Launch &L, const BcSpec &bc, double omf, const State &s);
void launch_com_boundary(const Launch &L, const ComSpec &c, const State &s);
void launch_correct_vaz(const Launch &L, double domega, double *vaz);
void launch_cfl_cells(const Launch &L, const State &s, double *out);
void launch_com_damping(const Launch &L, const ComSpec &c, double dt, const State &s);
// rings per radial sweep chunk for this device and disk
int radial_chunk_for(bool pair, bool adiabatic, int nr, int nz);
void launch_transport_radial(const Launch &L, double dt, double omf, int chunk, const double *S,
                             const double *vr, const double *vaz, const double *E,
                             double *const mom[4], double *E_out, double *S_out);
size_t azimuthal_smem_bytes(int nz);
int azimuthal_cells_per_thread(int nz);
cudaError_t prepare_azimuthal(size_t smem);
// block: threads of the FP64 kernel (the pair kernel chooses its own)
// ring_shift (nr ints): the pair kernel leaves AdvectSHIFT to the velocity
// rebuild and writes each ring's shift there
void launch_transport_azimuthal(const Launch &L, double dt, int block, double *const mom[4],
                                double *E, double *S, const double *vaz, double *ring_ws,
                                size_t smem, int *ring_shift);
// ring_shift: the azimuthal shifts the pair rebuild applies (pair form)
void launch_finish(const Launch &L, double omf, double *const mom[4], const double *S_t,
                   const double *E_t, const double *vr_in, double *vr_out, double *vaz_out,
                   double *S_out, double *E_out, const int *ring_shift);
void launch_damping(const Launch &L, const Damping &dm, double dt, const int *rings, int nrings,
                    const State &s);
void launch_derived_cfl(const Launch &L, int mode, const State &s, unsigned long long *dt_min);
void launch_pressure(const Launch &L, const double *S, const double *E, double *P);
// the same cell kernels with their arithmetic in float pairs (kernels_pair.cu);
// the launchers above route to them when L.pair is set
void launch_source_pair(const Launch &L, double dt, double omf, const double *S, const double *Pr,
                        const double *pot, const double *vr_in, const double *vaz_in,
                        double *vr_out, double *vaz_out);
void launch_artvisc_q_pair(const Launch &L, double dt, const double *S, const double *vr,
                           const double *vaz, double *E, double *Qr, double *Qp);
void launch_artvisc_v_pair(const Launch &L, double dt, const double *S, const double *E,
                           const double *Qr, const double *Qp, double *vr, double *vaz, double *cs,
                           double *H, double *nu);
void launch_stress_pair(const Launch &L, const double *S, const double *vr, const double *vaz,
                        const double *nu, double *divv, double *trr, double *tpp, double *trp);
void launch_viscous_pair(const Launch &L, double dt, double beta_inv, int mode, const State &s);
// Whether the stress kernel leaves div v and the stress tensor as float pairs
// (hi, lo in the 8 bytes of each double) for the float-pair viscous kernel,
// which reads them so, instead of joined doubles; StabilizeViscosity 1's
// viscous update is the FP64 kernel's, which reads doubles.
inline bool stress_as_pairs(const Launch &L) { return L.pair && L.ph.stabilize != 1; }
// the pairs of n cells joined into doubles in place (div v and the stress
// tensor before they are read as doubles)
void launch_join_pairs(cudaStream_t stream, double *x, size_t n);
void launch_finish_pair(const Launch &L, double omf, double *const mom[4], const double *S_t,
                        const double *E_t, const double *vr_in, double *vr_out, double *vaz_out,
                        double *S_out, double *E_out, const int *ring_shift);
// bodies one disk-force pass handles
constexpr int kForceBodies = 4;

// the disk force on n bodies (ComputeDiskOnPlanetAccel each) and the gas
// mass: out[5 b .. 5 b + 4] = inner x, inner y, outer x, outer y, mass;
// partial holds 5 min(n, 4) doubles per active ring
void launch_disk_force(const Launch &L, int n, const double *px, const double *py,
                       const double *pa, const double *rsm, const double *S, const double *H,
                       double *partial, double *out);
void launch_gas_quantities(const Launch &L, double radius, double omf, const double *S,
                           const double *vaz, double *partial, double *out);
void launch_scale_sigma(const Launch &L, double *S, double target, const double *mass);
void launch_check_finite(const Launch &L, const double *x, size_t n, unsigned long long *bad);
void launch_accrete(const Launch &L, const AccretionSpec &a, double *S, double *E,
                    const double *vr, const double *vaz, const double *nu, double *out);

}  // namespace fgpu
