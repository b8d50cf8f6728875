// Batched many-disk form of the FP32-mixed hydro step (fgpu_batch_* of the C
// ABI).
//
// A batch holds independent disks of any sizes, each an FP32-mixed engine
// (kernels_fp32.cu) whose buffers, tables and constants the batched kernels
// read through a device array of DiskF descriptions.  Every phase of the step
// is ONE grid-stride launch over all disks: the grid is sized to the SM count
// times the kernel's resident blocks per SM, and each block walks a list of
// tiles (disk, rings, columns) found through a per-kernel prefix table of
// tiles per disk.  The per-cell, per-column and per-ring bodies are the ones
// of the single-disk kernels (fp32_device.cuh), so a disk stepped in a batch
// computes what it computes alone.
//
// Each disk has its own dt.  With the device clock (ClockF), a one-block
// kernel at the start of every step turns each disk's CFL minimum of the
// previous step into its dt (sim::CalculateTimeStep and the monitor-time
// clamp of sim::run, simulation.cpp:100-118, 505-558), places the planets on
// their circular orbits at the disk's time and stops disks that reached
// their end time.  No step then needs the host, so a sequence of steps is
// captured once as a CUDA graph and relaunched.
//
// Tile shapes (threads per block, rings per block or per thread) are
// per-kernel and chosen by an autotuner that times candidates on the batch's
// own state with CUDA events and restores the state afterwards.
#include "../../include/fargocpt_gb300.h"
#include "fp32_device.cuh"
#include "fp32_engine.h"

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <new>
#include <string>
#include <vector>

namespace fgpu32 {

int create_disk(const fgpu_params *params, const double *radii, cudaStream_t stream,
                fgpu_engine **out);
int destroy_disk(fgpu_engine *eng);
Engine32 *engine32_of(fgpu_engine *eng);

// ---------------------------------------------------------------------------
// device side
// ---------------------------------------------------------------------------

// disk owning work item `item`: the largest d with start[d] <= item
__device__ __forceinline__ int disk_of(const int *__restrict__ start, int nd, int item)
{
    int lo = 0, hi = nd;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(start + mid) <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Per-cell tiles: blockDim.x columns x rpb rings of one disk; rows nr + extra.
template <class F>
__device__ __forceinline__ void for_cells(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                                          const int *__restrict__ start, int nd, int rpb,
                                          int extra, F f)
{
    const int total = __ldg(start + nd);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int d = disk_of(start, nd, tile);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        const int nz = k.g.nz;
        const int ncol = (nz + blockDim.x - 1) / blockDim.x;
        const int local = tile - __ldg(start + d);
        const int j = (local % ncol) * blockDim.x + threadIdx.x;
        if (j >= nz) continue;
        const int i0 = (local / ncol) * rpb;
        const int i1 = min(i0 + rpb, k.g.nr + extra);
        for (int i = i0; i < i1; ++i) f(k, S[d], i, j);
    }
}

__global__ void b_potential(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                            const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 0, [&](const DiskF &k, const StepF &st, int i, int j) {
        potential_cell(k.g, k.t, k.ph, st.b, k.H, k.pot, i, j);
    });
}

__global__ void b_source(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                         const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 1, [&](const DiskF &k, const StepF &st, int i, int j) {
        source_cell(k.g, k.t, st.fdt, k.s.sigma, k.P, k.pot, k.s.vr, k.s.dv, k.vr_b, k.dv_b, i, j);
    });
}

__global__ void b_artvisc_q(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                            const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 0, [&](const DiskF &k, const StepF &st, int i, int j) {
        if (!(k.ph.adiabatic || k.ph.art_visc_sn || k.ph.art_visc_tw)) return;
        artvisc_q_cell(k.g, k.t, k.ph, st.fdt, k.s.sigma, k.vr_b, k.dv_b, k.s.energy, k.Qr, k.Qp,
                       i, j);
    });
}

__global__ void b_artvisc_v(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                            const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 0, [&](const DiskF &k, const StepF &st, int i, int j) {
        if (!(k.ph.adiabatic || k.ph.art_visc_sn || k.ph.art_visc_tw)) return;
        artvisc_v_cell(k.g, k.t, k.ph, st.fdt, k.s.sigma, k.s.energy, k.Qr, k.Qp, k.vr_b, k.dv_b,
                       k.cs, k.H, k.nu, i, j);
    });
}

__global__ void b_stress(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                         const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 0, [&](const DiskF &k, const StepF &, int i, int j) {
        stress_cell(k.g, k.t, k.s.sigma, k.vr_b, k.dv_b, k.nu, k.divv, k.trr, k.tpp, k.trp, i, j);
    });
}

__global__ void b_viscous(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                          const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 0, [&](const DiskF &k, const StepF &st, int i, int j) {
        viscous_cell(k.g, k.t, k.ph, st.fdt, st.beta_inv, k.ph.adiabatic ? 7 : 1, k.s.sigma, k.trr,
                     k.tpp, k.trp, k.divv, k.nu, k.H, k.s.sigma0, k.s.energy0, k.vr_b, k.dv_b,
                     k.s.energy, k.qplus, k.qminus, nullptr, nullptr, i, j);
    });
}

__global__ void b_finish(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                         const int *__restrict__ start, int nd, int rpb)
{
    for_cells(D, S, start, nd, rpb, 1, [&](const DiskF &k, const StepF &, int i, int j) {
        finish_cell(k.g, k.t, k.ph, k.mom[0], k.mom[1], k.mom[2], k.mom[3], k.sigma_t, k.energy_t,
                    k.vr_b, k.s.vr, k.s.dv, k.s.sigma, k.s.energy, k.sigma_lo_t, k.s.sigma_lo,
                    k.ring_shift, i,
                    j);
    });
}

// ghost rings of the mid-step (B buffers) or end-of-step (A buffers) state
__global__ void b_ghost(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                        const int *__restrict__ start, int nd, int use_b)
{
    const int total = __ldg(start + nd);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int d = disk_of(start, nd, tile);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        const int j = (tile - __ldg(start + d)) * blockDim.x + threadIdx.x;
        if (j >= k.g.nz) continue;
        StateF st = k.s;
        if (use_b) {
            st.vr = k.vr_b;
            st.dv = k.dv_b;
        }
        ghost_col(k.g, k.bc, st, j);
    }
}

// radial transport tiles: blockDim.x columns x one chunk of rings; one
// instantiation per number of transported quantities, disks of the other
// kind skipped
template <int NQ>
__global__ void b_transport_radial(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                                   const int *__restrict__ start, int nd, int chunk)
{
    const int total = __ldg(start + nd);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int d = disk_of(start, nd, tile);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        if (k.nq != NQ) continue;
        const int nz = k.g.nz;
        const int ncol = (nz + blockDim.x - 1) / blockDim.x;
        const int local = tile - __ldg(start + d);
        const int j = (local % ncol) * blockDim.x + threadIdx.x;
        if (j >= nz) continue;
        const int i0 = (local / ncol) * chunk;
        const StateF &s = k.s;
        radial_col<NQ>(k.g, k.t, S[d].fdt, k.ph.limiter_mc, chunk, s.sigma, k.vr_b, k.dv_b,
                       s.energy, k.mom[0], k.mom[1], k.mom[2], k.mom[3], k.energy_t, k.sigma_t,
                       s.sigma_lo, k.sigma_lo_t, i0, j);
    }
}

// azimuthal transport: one ring per block iteration, PER cells per thread
// strided over the block; PER * blockDim.x covers the longest ring of the
// batch; the transported quantities are staged in dynamic shared memory,
// azimuthal_smem_floats(naz_max, nq_max, true) floats
// (two blocks of up to 384 threads per SM up to 4 cells per thread, 85
// registers).  One instantiation per number of transported quantities (4
// isothermal, 5 with the energy); disks of the other kind are skipped.
template <int PER, int NQ>
__global__ void __launch_bounds__(PER <= 4 ? 384 : 512, PER <= 4 ? 2 : 1)
    b_transport_azimuthal(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                          const int *__restrict__ start, int nd)
{
    extern __shared__ __align__(16) float smf[];
    __shared__ float redf[33];
    __shared__ long long redl[33];
    const int total = __ldg(start + nd);
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int d = disk_of(start, nd, item);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        if (k.nq != NQ) continue;
        const int i = item - __ldg(start + d);
        azimuthal_ring<PER, NQ, true>(k.g, k.t, S[d].dt, k.ph.limiter_mc, k.ph.fast_transport,
                                      k.dv_b, k.mom[0], k.mom[1], k.mom[2], k.mom[3], k.energy_t,
                                      k.sigma_t, k.sigma_lo_t, i, smf, redf, redl,
                                      k.ring_shift);
    }
}

// the register-blocked ring transport (azimuthal_ring_rb) over the rings of
// one group of disks with the same ring length nz = PER x blockDim.x and
// quantity count; start holds only the group's disks' rings
template <int PER, int NQ>
__global__ void __launch_bounds__(rb_max_threads(PER))
    b_transport_azimuthal_rb(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                             const int *__restrict__ start, int nd)
{
    extern __shared__ __align__(16) float smf[];
    __shared__ float redf[33];
    __shared__ long long redl[33];
    const int total = __ldg(start + nd);
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int d = disk_of(start, nd, item);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        const int i = item - __ldg(start + d);
        azimuthal_ring_rb<PER, NQ>(k.g, k.t, S[d].dt, k.ph.limiter_mc, k.ph.fast_transport,
                                   k.dv_b, k.mom[0], k.mom[1], k.mom[2], k.mom[3], k.energy_t,
                                   k.sigma_t, k.sigma_lo_t, i, smf, redf, redl,
                                   k.ring_shift);
    }
}

typedef void (*AzRbFn)(const DiskF *, const StepF *, const int *, int);
template <int NQ>
static AzRbFn az_rb_fn_nq(int per)
{
    switch (per) {
    case 4: return b_transport_azimuthal_rb<4, NQ>;
    case 8: return b_transport_azimuthal_rb<8, NQ>;
    case 12: return b_transport_azimuthal_rb<12, NQ>;
    case 16: return b_transport_azimuthal_rb<16, NQ>;
    default: return nullptr;
    }
}
static AzRbFn az_rb_fn(int per, int nq) { return nq == 5 ? az_rb_fn_nq<5>(per) : az_rb_fn_nq<4>(per); }

// damping rings: items = (disk, ring) of every disk with damping zones, each
// taken four times, once per damped field (the fields are independent)
__global__ void b_damping(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                          const int2 *__restrict__ items, int n)
{
    __shared__ float red[33];
    __shared__ long long redl[33];
    for (int it = blockIdx.x; it < 4 * n; it += gridDim.x) {
        const int2 w = items[it >> 2];
        if (!S[w.x].run) continue;
        const DiskF &k = D[w.x];
        const int q = it & 3;
        damping_ring(k.g, k.dm, S[w.x].fdt, k.s, w.y, red, redl, q, q + 1);
    }
}

// derived quantities and CFL minimum: one ring per block iteration
__global__ void b_derived_cfl(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                              const int *__restrict__ start, int nd, int mode, int all)
{
    __shared__ float red[33];
    __shared__ longlong2 red2[33];
    const int total = __ldg(start + nd);
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int d = disk_of(start, nd, item);
        if (!all && !S[d].run) continue;
        const DiskF &k = D[d];
        const int i = item - __ldg(start + d);
        derived_cfl_ring(k.g, k.t, k.ph, mode, k.s.sigma, k.s.energy, k.s.vr, k.s.dv, k.qplus,
                         k.qminus, k.cs, k.H, k.P, k.T, k.nu, k.dtmin, i, red, red2, nullptr,
                         nullptr);
    }
}

// ---------------------------------------------------------------------------
// Persistent substep sequences (FGPU_BATCH_PERSISTENT): the gas kick's
// substeps and the closing substeps each as one cooperative launch whose
// blocks all stay resident; every block walks a substep's tiles exactly as
// the substep's own kernel does, and the grid synchronises before the next
// substep.  The control flow around each grid.sync() is the same in every
// block (uniform conditions only, no early return once the sequence runs),
// and a launch that is not cooperative does nothing but set *err.  Tile
// tables: tabs holds FGPU_BK_COUNT tables of nd + 1 starts made for
// blockDim.x threads.
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;

__global__ void b_kick_sequence(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                                const int *__restrict__ tabs, int nd, fgpu_tiles tl, int any_art,
                                int *err)
{
    cg::grid_group grid = cg::this_grid();
    if (!grid.is_valid()) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *err = 1;
        return;
    }
    auto tab = [&](int k) { return tabs + (size_t)k * (nd + 1); };
    for_cells(D, S, tab(FGPU_BK_POTENTIAL), nd, tl.k[FGPU_BK_POTENTIAL].rings, 0,
              [&](const DiskF &k, const StepF &st, int i, int j) {
                  potential_cell(k.g, k.t, k.ph, st.b, k.H, k.pot, i, j);
              });
    grid.sync();
    for_cells(D, S, tab(FGPU_BK_SOURCE), nd, tl.k[FGPU_BK_SOURCE].rings, 1,
              [&](const DiskF &k, const StepF &st, int i, int j) {
                  source_cell(k.g, k.t, st.fdt, k.s.sigma, k.P, k.pot, k.s.vr, k.s.dv, k.vr_b,
                              k.dv_b, i, j);
              });
    grid.sync();
    if (any_art) {
        for_cells(D, S, tab(FGPU_BK_ARTVISC_Q), nd, tl.k[FGPU_BK_ARTVISC_Q].rings, 0,
                  [&](const DiskF &k, const StepF &st, int i, int j) {
                      if (!(k.ph.adiabatic || k.ph.art_visc_sn || k.ph.art_visc_tw)) return;
                      artvisc_q_cell(k.g, k.t, k.ph, st.fdt, k.s.sigma, k.vr_b, k.dv_b,
                                     k.s.energy, k.Qr, k.Qp, i, j);
                  });
        grid.sync();
        for_cells(D, S, tab(FGPU_BK_ARTVISC_V), nd, tl.k[FGPU_BK_ARTVISC_V].rings, 0,
                  [&](const DiskF &k, const StepF &st, int i, int j) {
                      if (!(k.ph.adiabatic || k.ph.art_visc_sn || k.ph.art_visc_tw)) return;
                      artvisc_v_cell(k.g, k.t, k.ph, st.fdt, k.s.sigma, k.s.energy, k.Qr, k.Qp,
                                     k.vr_b, k.dv_b, k.cs, k.H, k.nu, i, j);
                  });
        grid.sync();
    }
    for_cells(D, S, tab(FGPU_BK_STRESS), nd, tl.k[FGPU_BK_STRESS].rings, 0,
              [&](const DiskF &k, const StepF &, int i, int j) {
                  stress_cell(k.g, k.t, k.s.sigma, k.vr_b, k.dv_b, k.nu, k.divv, k.trr, k.tpp,
                              k.trp, i, j);
              });
    grid.sync();
    for_cells(D, S, tab(FGPU_BK_VISCOUS), nd, tl.k[FGPU_BK_VISCOUS].rings, 0,
              [&](const DiskF &k, const StepF &st, int i, int j) {
                  viscous_cell(k.g, k.t, k.ph, st.fdt, st.beta_inv, k.ph.adiabatic ? 7 : 1,
                               k.s.sigma, k.trr, k.tpp, k.trp, k.divv, k.nu, k.H, k.s.sigma0,
                               k.s.energy0, k.vr_b, k.dv_b, k.s.energy, k.qplus, k.qminus,
                               nullptr, nullptr, i, j);
              });
    grid.sync();
    // the mid-step ghost rings (B buffers), as b_ghost
    const int *gt = tab(FGPU_BK_GHOST);
    const int total = __ldg(gt + nd);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int d = disk_of(gt, nd, tile);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        const int j = (tile - __ldg(gt + d)) * blockDim.x + threadIdx.x;
        if (j >= k.g.nz) continue;
        StateF st = k.s;
        st.vr = k.vr_b;
        st.dv = k.dv_b;
        ghost_col(k.g, k.bc, st, j);
    }
}

__global__ void b_close_sequence(const DiskF *__restrict__ D, const StepF *__restrict__ S,
                                 const int *__restrict__ tabs, int nd, fgpu_tiles tl,
                                 const int2 *__restrict__ damp_items, int n_damp, int *err)
{
    __shared__ float red[33];
    __shared__ long long redl[33];
    __shared__ longlong2 red2[33];
    cg::grid_group grid = cg::this_grid();
    if (!grid.is_valid()) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *err = 1;
        return;
    }
    auto tab = [&](int k) { return tabs + (size_t)k * (nd + 1); };
    for_cells(D, S, tab(FGPU_BK_FINISH), nd, tl.k[FGPU_BK_FINISH].rings, 1,
              [&](const DiskF &k, const StepF &, int i, int j) {
                  finish_cell(k.g, k.t, k.ph, k.mom[0], k.mom[1], k.mom[2], k.mom[3], k.sigma_t,
                              k.energy_t, k.vr_b, k.s.vr, k.s.dv, k.s.sigma, k.s.energy,
                              k.sigma_lo_t, k.s.sigma_lo, k.ring_shift, i, j);
              });
    grid.sync();
    // damping zones, as b_damping (its block reductions are block-wide)
    for (int it = blockIdx.x; it < 4 * n_damp; it += gridDim.x) {
        const int2 w = damp_items[it >> 2];
        if (!S[w.x].run) continue;
        const DiskF &k = D[w.x];
        const int q = it & 3;
        damping_ring(k.g, k.dm, S[w.x].fdt, k.s, w.y, red, redl, q, q + 1);
    }
    grid.sync();
    // the end-of-step ghost rings (A buffers), as b_ghost
    const int *gt = tab(FGPU_BK_GHOST);
    const int total = __ldg(gt + nd);
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int d = disk_of(gt, nd, tile);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        const int j = (tile - __ldg(gt + d)) * blockDim.x + threadIdx.x;
        if (j >= k.g.nz) continue;
        ghost_col(k.g, k.bc, k.s, j);
    }
    grid.sync();
    // derived quantities and the CFL minimum, as b_derived_cfl
    const int *ct = tab(FGPU_BK_DERIVED_CFL);
    const int ctotal = __ldg(ct + nd);
    for (int item = blockIdx.x; item < ctotal; item += gridDim.x) {
        const int d = disk_of(ct, nd, item);
        if (!S[d].run) continue;
        const DiskF &k = D[d];
        const int i = item - __ldg(ct + d);
        derived_cfl_ring(k.g, k.t, k.ph, 1 | 4, k.s.sigma, k.s.energy, k.s.vr, k.s.dv, k.qplus,
                         k.qminus, k.cs, k.H, k.P, k.T, k.nu, k.dtmin, i, red, red2, nullptr,
                         nullptr);
    }
}

__global__ void b_reset_dtmin(const DiskF *__restrict__ D, const StepF *__restrict__ S, int nd)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < nd && S[d].run) *D[d].dtmin = 0x7f7f7f7fu;
}

// Planets on circular orbits around the star at the origin and the indirect
// term of the star-centred frame; the arithmetic is spelled out with
// round-to-nearest intrinsics so that no step is contracted into an FMA.
__device__ void circular_bodies(const ClockF &c, float gm_ref, int star_is_centre, double t,
                                BodiesF &b)
{
    const double G = c.G;
    b.n = 1 + c.n_planets;
    b.star_at_origin = star_is_centre;
    b.x[0] = 0.0;
    b.y[0] = 0.0;
    b.a[0] = 0.0;
    split_position(b, 0);
    b.gm[0] = (float)__dmul_rn(G, c.mstar);
    b.rsm[0] = 0.f;
    double ax = 0.0, ay = 0.0;
    for (int p = 0; p < c.n_planets; ++p) {
        const double m = c.q[p], a = c.a[p];
        const double om = sqrt(__ddiv_rn(__dmul_rn(G, __dadd_rn(c.mstar, m)), pow(a, 3.0)));
        const double ang = __dadd_rn(__dmul_rn(om, t), c.phase[p]);
        const double x = __dmul_rn(a, cos(ang)), y = __dmul_rn(a, sin(ang));
        b.x[p + 1] = x;
        b.y[p + 1] = y;
        split_position(b, p + 1);
        b.a[p + 1] = a;
        b.gm[p + 1] = (float)__dmul_rn(G, m);
        b.rsm[p + 1] = 0.f;
        const double d3 = pow(__dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))), 3.0);
        const double w = __ddiv_rn(__dmul_rn(G, m), d3);
        ax = __dsub_rn(ax, __dmul_rn(w, __dsub_rn(0.0, x)));
        ay = __dsub_rn(ay, __dmul_rn(w, __dsub_rn(0.0, y)));
    }
    b.gm_ref = gm_ref;
    b.ix = (float)(-ax);
    b.iy = (float)(-ay);
}

struct ClockAux {
    float gm_ref;
    int star_is_centre;
};

// One block, one thread per disk (nd <= 1024).
__global__ void b_clock(const DiskF *__restrict__ D, const ClockAux *__restrict__ aux,
                        ClockF *__restrict__ C, StepF *__restrict__ S, int nd, int *n_active)
{
    const int d = threadIdx.x;
    int act = 0;
    if (d < nd) {
        ClockF c = C[d];
        StepF &s = S[d];
        const int run = c.active && c.t < c.t_end;
        if (run) {
            unsigned int *dtmin = D[d].dtmin;
            const double cfl = (double)__uint_as_float(*dtmin);
            *dtmin = 0x7f7f7f7fu;
            const double grown = __dmul_rn(c.cfl_max_var, c.last_dt);
            const double cfl_dt = cfl < grown ? cfl : grown;
            c.last_dt = cfl_dt;
            const double next_mon = __dmul_rn((double)(c.n_monitor + 1), c.monitor_dt);
            const double left = __dsub_rn(next_mon, c.t);
            const bool clamp = cfl_dt > left || left < __dmul_rn(cfl_dt, 1.05);
            const double dt = clamp ? left : cfl_dt;
            s.dt = dt;
            s.t = c.t;
            s.fdt = (float)dt;
            double bi = c.beta_inv0;
            if (c.beta_ramp > 0.0) {
                const double x = __ddiv_rn(__dmul_rn(2.0, c.t), c.beta_ramp);
                bi = __dmul_rn(bi, __dsub_rn(1.0, exp(-__dmul_rn(x, x))));
            }
            s.beta_inv = (float)bi;
            circular_bodies(c, aux[d].gm_ref, aux[d].star_is_centre, c.t, s.b);
            c.t = __dadd_rn(c.t, dt);
            c.steps += 1;
            if (fabs(__dsub_rn(next_mon, c.t)) < __dmul_rn(1e-6, cfl_dt)) c.n_monitor += 1;
        }
        s.run = run;
        c.active = c.active && c.t < c.t_end;
        act = c.active;
        C[d] = c;
    }
    const int cnt = __syncthreads_count(act);
    if (threadIdx.x == 0) *n_active = cnt;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static bool is_cell_kernel(int k)
{
    return k == FGPU_BK_POTENTIAL || k == FGPU_BK_SOURCE || k == FGPU_BK_ARTVISC_Q ||
           k == FGPU_BK_ARTVISC_V || k == FGPU_BK_STRESS || k == FGPU_BK_VISCOUS ||
           k == FGPU_BK_FINISH;
}
static bool is_ring_kernel(int k)
{
    return k == FGPU_BK_TRANSPORT_AZIMUTHAL || k == FGPU_BK_DAMPING || k == FGPU_BK_DERIVED_CFL;
}

static const int kPerChoices[] = {1, 2, 3, 4, 6, 8, 12, 16};

static int per_for(int nz_max, int threads)
{
    const int need = (nz_max + threads - 1) / threads;
    for (int p : kPerChoices)
        if (p >= need) return p;
    return 0;
}

typedef void (*AzFn)(const DiskF *, const StepF *, const int *, int);
template <int NQ>
static AzFn az_fn_nq(int per)
{
    switch (per) {
    case 1: return b_transport_azimuthal<1, NQ>;
    case 2: return b_transport_azimuthal<2, NQ>;
    case 3: return b_transport_azimuthal<3, NQ>;
    case 4: return b_transport_azimuthal<4, NQ>;
    case 6: return b_transport_azimuthal<6, NQ>;
    case 8: return b_transport_azimuthal<8, NQ>;
    case 12: return b_transport_azimuthal<12, NQ>;
    case 16: return b_transport_azimuthal<16, NQ>;
    default: return nullptr;
    }
}
static AzFn az_fn(int per, int nq) { return nq == 5 ? az_fn_nq<5>(per) : az_fn_nq<4>(per); }

static const void *kernel_fn(int k, int per)
{
    switch (k) {
    case FGPU_BK_POTENTIAL: return (const void *)b_potential;
    case FGPU_BK_SOURCE: return (const void *)b_source;
    case FGPU_BK_ARTVISC_Q: return (const void *)b_artvisc_q;
    case FGPU_BK_ARTVISC_V: return (const void *)b_artvisc_v;
    case FGPU_BK_STRESS: return (const void *)b_stress;
    case FGPU_BK_VISCOUS: return (const void *)b_viscous;
    case FGPU_BK_GHOST: return (const void *)b_ghost;
    case FGPU_BK_TRANSPORT_RADIAL: return (const void *)b_transport_radial<5>;
    case FGPU_BK_TRANSPORT_AZIMUTHAL: return (const void *)az_fn(per, 5);
    case FGPU_BK_FINISH: return (const void *)b_finish;
    case FGPU_BK_DAMPING: return (const void *)b_damping;
    case FGPU_BK_DERIVED_CFL: return (const void *)b_derived_cfl;
    default: return nullptr;
    }
}

}  // namespace fgpu32

using namespace fgpu32;

struct fgpu_batch {
    int nd = 0;
    cudaStream_t stream = nullptr;
    std::vector<fgpu_engine *> handles;
    std::vector<Engine32 *> disks;
    std::vector<int> nr, nz;
    int nz_max = 0, nsm = 0;
    bool any_art = false, any_iso = false, any_adi = false;
    std::string err;

    DiskF *d_disks = nullptr;
    StepF *d_steps = nullptr, *h_steps = nullptr;
    ClockF *d_clocks = nullptr, *h_clocks = nullptr;
    ClockAux *d_aux = nullptr;
    std::vector<ClockAux> aux;
    int *d_active = nullptr, *h_active = nullptr;
    int *d_tables = nullptr;        // FGPU_BK_COUNT tables of nd + 1 tile starts
    int2 *d_damp_items = nullptr;
    int n_damp_items = 0;

    fgpu_tiles tiles{};
    int grid[FGPU_BK_COUNT] = {};
    int az_per = 0;
    size_t az_smem = 0;
    // disks whose rings take the register-blocked pass, grouped by ring
    // length and quantity count (one launch per group); the strided pass
    // takes the rest
    struct RbGroup {
        int nz, nq, per, grid;
        size_t smem;
    };
    std::vector<RbGroup> rb;
    std::vector<char> rb_disk;
    int *d_rb_tables = nullptr;  // rb.size() tables of nd + 1 tile starts
    long long az_strided_rings = 0;

    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;

    // FGPU_BATCH_PERSISTENT: the two substep sequences as cooperative
    // launches of seq_threads threads (measured on the 64-disk sweep: 5.86 ms
    // per step with 128, 6.26 with 256, 8.79 with 512, against 3.80 with one
    // launch per substep); their tile tables and grids
    int mode = FGPU_BATCH_LAUNCHES;
    static constexpr int seq_threads = 128;
    int *d_seq_tables = nullptr;  // FGPU_BK_COUNT tables of nd + 1 tile starts
    int seq_grid[2] = {};
    int *d_seq_err = nullptr;     // set by a sequence launched non-cooperatively

    const int *table(int k) const { return d_tables + (size_t)k * (nd + 1); }
};

#define CKB(call)                                                          \
    do {                                                                   \
        cudaError_t e_ = (call);                                           \
        if (e_ != cudaSuccess) {                                           \
            b->err = std::string(#call) + ": " + cudaGetErrorString(e_);   \
            return FGPU_ERR_CUDA;                                          \
        }                                                                  \
    } while (0)

static int check_tiles(const fgpu_batch *b, const fgpu_tiles &t, std::string &why)
{
    for (int k = 0; k < FGPU_BK_COUNT; ++k) {
        const int th = t.k[k].threads, r = t.k[k].rings;
        const int max_threads = (k == FGPU_BK_TRANSPORT_AZIMUTHAL) ? 512 : 1024;
        if (th < 32 || th > max_threads || th % 32) {
            why = "threads of kernel " + std::to_string(k) + " must be a multiple of 32 in [32, " +
                  std::to_string(max_threads) + "]";
            return FGPU_ERR_BAD_ARG;
        }
        if (is_cell_kernel(k) && (r < 1 || r > 64)) {
            why = "rings per block must be in [1, 64]";
            return FGPU_ERR_BAD_ARG;
        }
        if (k == FGPU_BK_TRANSPORT_RADIAL && (r < 1 || r > 1024)) {
            why = "radial chunk must be in [1, 1024]";
            return FGPU_ERR_BAD_ARG;
        }
    }
    if (!per_for(b->nz_max, t.k[FGPU_BK_TRANSPORT_AZIMUTHAL].threads)) {
        why = "azimuthal transport needs more threads for the longest ring (16 cells per thread "
              "at most)";
        return FGPU_ERR_BAD_ARG;
    }
    return FGPU_OK;
}

// tile tables and grid sizes of the current tile shapes
static int apply_tiles(fgpu_batch *b, const fgpu_tiles &t)
{
    std::string why;
    int rc = check_tiles(b, t, why);
    if (rc) {
        b->err = why;
        return rc;
    }
    b->tiles = t;
    const int nd = b->nd;
    // the persistent sequences' tables: the same tiles with seq_threads
    // threads per block
    {
        std::vector<int> hs((size_t)FGPU_BK_COUNT * (nd + 1), 0);
        for (int k = 0; k < FGPU_BK_COUNT; ++k) {
            int *s = hs.data() + (size_t)k * (nd + 1);
            const int th = fgpu_batch::seq_threads, r = t.k[k].rings;
            long long acc = 0;
            for (int d = 0; d < nd; ++d) {
                s[d] = (int)acc;
                const long long ncol = (b->nz[d] + th - 1) / th;
                long long n = 0;
                if (is_cell_kernel(k)) {
                    const int extra = (k == FGPU_BK_SOURCE || k == FGPU_BK_FINISH) ? 1 : 0;
                    n = ((b->nr[d] + extra + r - 1) / r) * ncol;
                } else if (k == FGPU_BK_GHOST) {
                    n = ncol;
                } else if (k == FGPU_BK_DERIVED_CFL) {
                    n = b->nr[d];
                }
                acc += n;
            }
            if (acc > 0x7fffffffLL) {
                b->err = "too many tiles";
                return FGPU_ERR_UNSUPPORTED;
            }
            s[nd] = (int)acc;
        }
        CKB(cudaMemcpyAsync(b->d_seq_tables, hs.data(), sizeof(int) * hs.size(),
                            cudaMemcpyHostToDevice, b->stream));
        const void *seq_fn[2] = {(const void *)b_kick_sequence, (const void *)b_close_sequence};
        for (int q = 0; q < 2; ++q) {
            int per_sm = 0;
            CKB(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, seq_fn[q],
                                                              fgpu_batch::seq_threads, 0));
            // all blocks resident at once, as a cooperative launch requires
            b->seq_grid[q] = std::max(1, per_sm) * b->nsm;
        }
    }
    std::vector<int> h((size_t)FGPU_BK_COUNT * (nd + 1), 0);
    std::vector<long long> totals(FGPU_BK_COUNT, 0);
    for (int k = 0; k < FGPU_BK_COUNT; ++k) {
        int *s = h.data() + (size_t)k * (nd + 1);
        const int th = t.k[k].threads, r = t.k[k].rings;
        long long acc = 0;
        for (int d = 0; d < nd; ++d) {
            s[d] = (int)acc;
            const long long ncol = (b->nz[d] + th - 1) / th;
            long long n = 0;
            if (is_cell_kernel(k)) {
                const int extra = (k == FGPU_BK_SOURCE || k == FGPU_BK_FINISH) ? 1 : 0;
                n = ((b->nr[d] + extra + r - 1) / r) * ncol;
            } else if (k == FGPU_BK_GHOST) {
                n = ncol;
            } else if (k == FGPU_BK_TRANSPORT_RADIAL) {
                n = ((b->nr[d] + r - 1) / r) * ncol;
            } else if (k == FGPU_BK_TRANSPORT_AZIMUTHAL) {
                n = b->rb_disk[d] ? 0 : b->nr[d];
            } else if (k == FGPU_BK_DERIVED_CFL) {
                n = b->nr[d];
            }
            acc += n;
        }
        if (acc > 0x7fffffffLL) {
            b->err = "too many tiles";
            return FGPU_ERR_UNSUPPORTED;
        }
        s[nd] = (int)acc;
        totals[k] = k == FGPU_BK_DAMPING ? 4LL * b->n_damp_items : acc;
        if (k == FGPU_BK_TRANSPORT_AZIMUTHAL) b->az_strided_rings = acc;
    }
    CKB(cudaMemcpyAsync(b->d_tables, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice,
                        b->stream));
    CKB(cudaStreamSynchronize(b->stream));
    b->az_per = per_for(b->nz_max, t.k[FGPU_BK_TRANSPORT_AZIMUTHAL].threads);
    for (int k = 0; k < FGPU_BK_COUNT; ++k) {
        const void *fn = kernel_fn(k, b->az_per);
        const size_t smem = k == FGPU_BK_TRANSPORT_AZIMUTHAL ? b->az_smem : 0;
        cudaFuncAttributes attr;
        CKB(cudaFuncGetAttributes(&attr, fn));
        if (t.k[k].threads > attr.maxThreadsPerBlock) {
            b->err = "kernel " + std::to_string(k) + " takes at most " +
                     std::to_string(attr.maxThreadsPerBlock) + " threads per block";
            return FGPU_ERR_UNSUPPORTED;
        }
        int per_sm = 0;
        CKB(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, t.k[k].threads, smem));
        if (per_sm < 1) {
            b->err = "kernel " + std::to_string(k) + " cannot run with " +
                     std::to_string(t.k[k].threads) + " threads";
            return FGPU_ERR_UNSUPPORTED;
        }
        const long long full = (long long)per_sm * b->nsm;
        b->grid[k] = (int)std::max(1LL, std::min(full, totals[k]));
    }
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_steps = 0;
    }
    return FGPU_OK;
}

static void default_tiles(const fgpu_batch *b, fgpu_tiles &t)
{
    for (int k = 0; k < FGPU_BK_COUNT; ++k) t.k[k] = {128, 1};
    t.k[FGPU_BK_TRANSPORT_RADIAL] = {64, 16};
    t.k[FGPU_BK_DAMPING] = {256, 1};
    t.k[FGPU_BK_DERIVED_CFL] = {256, 1};
    const int per = b->nz_max <= 2048 ? 4 : (b->nz_max <= 4096 ? 8 : 16);
    int th = ((b->nz_max + per - 1) / per + 31) / 32 * 32;
    th = std::max(128, std::min(512, th));
    t.k[FGPU_BK_TRANSPORT_AZIMUTHAL] = {th, 1};
}

// one batched kernel on the batch stream
static void launch_kernel(fgpu_batch *b, int k, int ghost_b = 0)
{
    const int nd = b->nd, th = b->tiles.k[k].threads, r = b->tiles.k[k].rings, g = b->grid[k];
    const DiskF *D = b->d_disks;
    const StepF *S = b->d_steps;
    cudaStream_t s = b->stream;
    switch (k) {
    case FGPU_BK_POTENTIAL: b_potential<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_SOURCE: b_source<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_ARTVISC_Q: b_artvisc_q<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_ARTVISC_V: b_artvisc_v<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_STRESS: b_stress<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_VISCOUS: b_viscous<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_GHOST: b_ghost<<<g, th, 0, s>>>(D, S, b->table(k), nd, ghost_b); break;
    case FGPU_BK_TRANSPORT_RADIAL:
        if (b->any_iso) b_transport_radial<4><<<g, th, 0, s>>>(D, S, b->table(k), nd, r);
        if (b->any_adi) b_transport_radial<5><<<g, th, 0, s>>>(D, S, b->table(k), nd, r);
        break;
    case FGPU_BK_TRANSPORT_AZIMUTHAL:
        if (b->az_strided_rings > 0) {
            if (b->any_iso) az_fn(b->az_per, 4)<<<g, th, b->az_smem, s>>>(D, S, b->table(k), nd);
            if (b->any_adi) az_fn(b->az_per, 5)<<<g, th, b->az_smem, s>>>(D, S, b->table(k), nd);
        }
        for (size_t q = 0; q < b->rb.size(); ++q) {
            const fgpu_batch::RbGroup &grp = b->rb[q];
            az_rb_fn(grp.per, grp.nq)<<<grp.grid, grp.nz / grp.per, grp.smem, s>>>(
                D, S, b->d_rb_tables + q * (size_t)(nd + 1), nd);
        }
        break;
    case FGPU_BK_FINISH: b_finish<<<g, th, 0, s>>>(D, S, b->table(k), nd, r); break;
    case FGPU_BK_DAMPING:
        if (b->n_damp_items)
            b_damping<<<g, th, 0, s>>>(D, S, b->d_damp_items, b->n_damp_items);
        break;
    case FGPU_BK_DERIVED_CFL:
        b_derived_cfl<<<g, th, 0, s>>>(D, S, b->table(k), nd, 1 | 4, 0);
        break;
    default: break;
    }
}

// the phases of one step in FargoCPT's order (simulation.cpp:148-267)
// one cooperative launch of a persistent substep sequence (q = 0: the gas
// kick, 1: the closing substeps)
static void launch_sequence(fgpu_batch *b, int q)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->seq_grid[q]);
    cfg.blockDim = dim3(fgpu_batch::seq_threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = b->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const DiskF *D = b->d_disks;
    const StepF *S = b->d_steps;
    if (q == 0)
        cudaLaunchKernelEx(&cfg, b_kick_sequence, D, S, (const int *)b->d_seq_tables, b->nd,
                           b->tiles, (int)b->any_art, b->d_seq_err);
    else
        cudaLaunchKernelEx(&cfg, b_close_sequence, D, S, (const int *)b->d_seq_tables, b->nd,
                           b->tiles, (const int2 *)b->d_damp_items, b->n_damp_items,
                           b->d_seq_err);
}

static void enqueue_step(fgpu_batch *b, bool device_clock)
{
    if (device_clock)
        b_clock<<<1, (b->nd + 31) / 32 * 32, 0, b->stream>>>(b->d_disks, b->d_aux, b->d_clocks,
                                                             b->d_steps, b->nd, b->d_active);
    else
        b_reset_dtmin<<<(b->nd + 127) / 128, 128, 0, b->stream>>>(b->d_disks, b->d_steps, b->nd);
    if (b->mode == FGPU_BATCH_PERSISTENT) {
        launch_sequence(b, 0);
        launch_kernel(b, FGPU_BK_TRANSPORT_RADIAL);
        launch_kernel(b, FGPU_BK_TRANSPORT_AZIMUTHAL);
        launch_sequence(b, 1);
        return;
    }
    launch_kernel(b, FGPU_BK_POTENTIAL);
    launch_kernel(b, FGPU_BK_SOURCE);
    if (b->any_art) {
        launch_kernel(b, FGPU_BK_ARTVISC_Q);
        launch_kernel(b, FGPU_BK_ARTVISC_V);
    }
    launch_kernel(b, FGPU_BK_STRESS);
    launch_kernel(b, FGPU_BK_VISCOUS);
    launch_kernel(b, FGPU_BK_GHOST, 1);
    launch_kernel(b, FGPU_BK_TRANSPORT_RADIAL);
    launch_kernel(b, FGPU_BK_TRANSPORT_AZIMUTHAL);
    launch_kernel(b, FGPU_BK_FINISH);
    launch_kernel(b, FGPU_BK_DAMPING);
    launch_kernel(b, FGPU_BK_GHOST, 0);
    launch_kernel(b, FGPU_BK_DERIVED_CFL);
}

static void release(fgpu_batch *b)
{
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (fgpu_engine *h : b->handles)
        if (h) destroy_disk(h);
    cudaFree(b->d_disks);
    cudaFree(b->d_steps);
    cudaFree(b->d_clocks);
    cudaFree(b->d_aux);
    cudaFree(b->d_active);
    cudaFree(b->d_tables);
    cudaFree(b->d_seq_tables);
    cudaFree(b->d_seq_err);
    cudaFree(b->d_rb_tables);
    cudaFree(b->d_damp_items);
    if (b->h_steps) cudaFreeHost(b->h_steps);
    if (b->h_clocks) cudaFreeHost(b->h_clocks);
    if (b->h_active) cudaFreeHost(b->h_active);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

extern "C" int fgpu_batch_create(int n, const fgpu_params *params, const double *const *radii,
                                 fgpu_batch **out)
{
    if (!out) return FGPU_ERR_BAD_ARG;
    *out = nullptr;
    if (!params || !radii || n < 1 || n > 1024) return FGPU_ERR_BAD_ARG;
    for (int k = 0; k < n; ++k) {
        if (!radii[k]) return FGPU_ERR_BAD_ARG;
        if (params[k].precision != FGPU_PRECISION_FP32_MIXED ||
            params[k].integrator != FGPU_INTEGRATOR_EULER)
            return FGPU_ERR_UNSUPPORTED;
        // StabilizeViscosity, KeepDiskMassConstant, the centre-of-mass
        // composite boundary and the recompute of c_s, H, nu before the final
        // hooks are not part of the batched step
        if (params[k].stabilize_viscosity || params[k].keep_disk_mass_constant)
            return FGPU_ERR_UNSUPPORTED;
        if (params[k].composite_inner != FGPU_COMPOSITE_INDIVIDUAL ||
            params[k].composite_outer != FGPU_COMPOSITE_INDIVIDUAL)
            return FGPU_ERR_UNSUPPORTED;
        if (params[k].eos == FGPU_EOS_IDEAL &&
            (params[k].viscous_accretion || params[k].bc_vrad_inner == FGPU_BC_VISCOUS))
            return FGPU_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return FGPU_ERR_NO_DEVICE;
    }
    fgpu_batch *b = new (std::nothrow) fgpu_batch();
    if (!b) return FGPU_ERR_OOM;
    b->nd = n;
    auto fail = [&](int rc) {
        fprintf(stderr, "fgpu_batch_create: %s\n", b->err.c_str());
        release(b);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        b->err = "stream";
        return fail(FGPU_ERR_CUDA);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
    std::vector<DiskF> desc(n);
    std::vector<int2> damp;
    b->handles.assign(n, nullptr);
    b->disks.assign(n, nullptr);
    b->aux.resize(n);
    for (int k = 0; k < n; ++k) {
        int rc = create_disk(&params[k], radii[k], b->stream, &b->handles[k]);
        if (rc) {
            b->err = "disk " + std::to_string(k) + " could not be created";
            return fail(rc);
        }
        Engine32 *e = engine32_of(b->handles[k]);
        b->disks[k] = e;
        b->nr.push_back(e->rings());
        b->nz.push_back(e->azimuthal());
        b->nz_max = std::max(b->nz_max, e->azimuthal());
        desc[k] = e->describe();
        b->any_art = b->any_art || desc[k].ph.adiabatic || desc[k].ph.art_visc_sn ||
                     desc[k].ph.art_visc_tw;
        b->any_iso = b->any_iso || desc[k].nq == 4;
        b->any_adi = b->any_adi || desc[k].nq == 5;
        int nrings = 0;
        const int *rings = e->damping_rings(&nrings);
        for (int q = 0; q < nrings; ++q) damp.push_back(make_int2(k, rings[q]));
        b->aux[k].gm_ref = (float)(params[k].G * params[k].hydro_center_mass);
        b->aux[k].star_is_centre = 0;
    }
    b->n_damp_items = (int)damp.size();
    int nq_max = 4;
    for (int k = 0; k < n; ++k) nq_max = std::max(nq_max, desc[k].nq);
    b->az_smem = azimuthal_smem_floats(b->nz_max, nq_max, true) * sizeof(float);
    if (b->az_smem > kMaxRingSmem) {
        b->err = "ring too long for the batched azimuthal kernel";
        return fail(FGPU_ERR_UNSUPPORTED);
    }
#define CKC(call)                                                        \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) {                                         \
            b->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return fail(FGPU_ERR_CUDA);                                  \
        }                                                                \
    } while (0)
    for (int per : kPerChoices) {
        CKC(raise_smem_limit((const void *)az_fn(per, 4), b->az_smem));
        CKC(raise_smem_limit((const void *)az_fn(per, 5), b->az_smem));
    }
    CKC(cudaMalloc(&b->d_disks, sizeof(DiskF) * n));
    CKC(cudaMemcpy(b->d_disks, desc.data(), sizeof(DiskF) * n, cudaMemcpyHostToDevice));
    CKC(cudaMalloc(&b->d_steps, sizeof(StepF) * n));
    CKC(cudaMemset(b->d_steps, 0, sizeof(StepF) * n));
    CKC(cudaMallocHost(&b->h_steps, sizeof(StepF) * n));
    std::memset(b->h_steps, 0, sizeof(StepF) * n);
    CKC(cudaMalloc(&b->d_clocks, sizeof(ClockF) * n));
    CKC(cudaMemset(b->d_clocks, 0, sizeof(ClockF) * n));
    CKC(cudaMallocHost(&b->h_clocks, sizeof(ClockF) * n));
    std::memset(b->h_clocks, 0, sizeof(ClockF) * n);
    CKC(cudaMalloc(&b->d_aux, sizeof(ClockAux) * n));
    CKC(cudaMemcpy(b->d_aux, b->aux.data(), sizeof(ClockAux) * n, cudaMemcpyHostToDevice));
    CKC(cudaMalloc(&b->d_active, sizeof(int)));
    CKC(cudaMallocHost(&b->h_active, sizeof(int)));
    CKC(cudaMalloc(&b->d_tables, sizeof(int) * FGPU_BK_COUNT * (n + 1)));
    CKC(cudaMalloc(&b->d_seq_tables, sizeof(int) * FGPU_BK_COUNT * (n + 1)));
    CKC(cudaMalloc(&b->d_seq_err, sizeof(int)));
    CKC(cudaMemsetAsync(b->d_seq_err, 0, sizeof(int), b->stream));
    {
        // register-blocked groups: disks with the same ring length and
        // quantity count whose rings split into whole segments
        // (rb_default_per); FARGO_GB300_AZIMUTHAL=strided keeps them all on
        // the strided pass
        const char *env = getenv("FARGO_GB300_AZIMUTHAL");
        const bool strided_only = env && std::string(env) == "strided";
        b->rb_disk.assign(n, 0);
        for (int d = 0; d < n && !strided_only; ++d) {
            const int nq = params[d].eos == FGPU_EOS_IDEAL ? 5 : 4;
            const int per = rb_default_per(b->nz[d], nq, kMaxRingSmem);
            if (!per) continue;
            b->rb_disk[d] = 1;
            bool found = false;
            for (auto &g : b->rb) found = found || (g.nz == b->nz[d] && g.nq == nq);
            if (!found)
                b->rb.push_back({b->nz[d], nq, per, 1,
                                 rb_smem_floats(b->nz[d], nq, b->nz[d] / per) * sizeof(float)});
        }
        if (!b->rb.empty()) {
            std::vector<int> h((size_t)b->rb.size() * (n + 1), 0);
            for (size_t q = 0; q < b->rb.size(); ++q) {
                fgpu_batch::RbGroup &g = b->rb[q];
                int *st = h.data() + q * (size_t)(n + 1);
                long long acc = 0;
                for (int d = 0; d < n; ++d) {
                    st[d] = (int)acc;
                    const int nq = params[d].eos == FGPU_EOS_IDEAL ? 5 : 4;
                    if (b->rb_disk[d] && b->nz[d] == g.nz && nq == g.nq) acc += b->nr[d];
                }
                st[n] = (int)acc;
                const void *fn = (const void *)az_rb_fn(g.per, g.nq);
                CKC(raise_smem_limit(fn, g.smem));
                int per_sm = 0;
                CKC(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, g.nz / g.per,
                                                                  g.smem));
                if (per_sm < 1) {
                    b->err = "the register-blocked ring pass cannot run on this device";
                    return fail(FGPU_ERR_UNSUPPORTED);
                }
                g.grid = (int)std::max(1LL, std::min((long long)per_sm * b->nsm, acc));
            }
            CKC(cudaMalloc(&b->d_rb_tables, sizeof(int) * h.size()));
            CKC(cudaMemcpy(b->d_rb_tables, h.data(), sizeof(int) * h.size(),
                           cudaMemcpyHostToDevice));
        }
    }
    if (!damp.empty()) {
        CKC(cudaMalloc(&b->d_damp_items, sizeof(int2) * damp.size()));
        CKC(cudaMemcpy(b->d_damp_items, damp.data(), sizeof(int2) * damp.size(),
                       cudaMemcpyHostToDevice));
    }
#undef CKC
    fgpu_tiles t;
    default_tiles(b, t);
    int rc = apply_tiles(b, t);
    if (rc) return fail(rc);
    *out = b;
    return FGPU_OK;
}

extern "C" int fgpu_batch_destroy(fgpu_batch *b)
{
    if (!b) return FGPU_ERR_BAD_ARG;
    release(b);
    return FGPU_OK;
}

extern "C" const char *fgpu_batch_last_error(const fgpu_batch *b)
{
    return b ? b->err.c_str() : "null batch";
}

extern "C" int fgpu_batch_size(const fgpu_batch *b, int *n)
{
    if (!b || !n) return FGPU_ERR_BAD_ARG;
    *n = b->nd;
    return FGPU_OK;
}

extern "C" int fgpu_batch_disk(fgpu_batch *b, int k, fgpu_engine **disk)
{
    if (!b || !disk || k < 0 || k >= b->nd) return FGPU_ERR_BAD_ARG;
    *disk = b->handles[k];
    return FGPU_OK;
}

extern "C" int fgpu_batch_get_tiles(const fgpu_batch *b, fgpu_tiles *tiles)
{
    if (!b || !tiles) return FGPU_ERR_BAD_ARG;
    *tiles = b->tiles;
    return FGPU_OK;
}

extern "C" int fgpu_batch_set_tiles(fgpu_batch *b, const fgpu_tiles *tiles)
{
    if (!b || !tiles) return FGPU_ERR_BAD_ARG;
    CKB(cudaStreamSynchronize(b->stream));
    return apply_tiles(b, *tiles);
}

extern "C" int fgpu_batch_set_mode(fgpu_batch *b, int mode)
{
    if (!b || (mode != FGPU_BATCH_LAUNCHES && mode != FGPU_BATCH_PERSISTENT))
        return FGPU_ERR_BAD_ARG;
    CKB(cudaStreamSynchronize(b->stream));
    if (mode == FGPU_BATCH_PERSISTENT) {
        int dev = 0, coop = 0;
        CKB(cudaGetDevice(&dev));
        CKB(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) {
            b->err = "the device has no cooperative launch";
            return FGPU_ERR_UNSUPPORTED;
        }
    }
    b->mode = mode;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_steps = 0;
    }
    return FGPU_OK;
}

extern "C" int fgpu_batch_get_mode(const fgpu_batch *b, int *mode)
{
    if (!b || !mode) return FGPU_ERR_BAD_ARG;
    *mode = b->mode;
    return FGPU_OK;
}

// a sequence launched without cooperation did nothing: report it
static int check_sequences(fgpu_batch *b)
{
    if (b->mode != FGPU_BATCH_PERSISTENT) return FGPU_OK;
    int e = 0;
    CKB(cudaMemcpyAsync(&e, b->d_seq_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CKB(cudaStreamSynchronize(b->stream));
    if (e) {
        b->err = "a persistent substep sequence ran without a cooperative launch";
        return FGPU_ERR_CUDA;
    }
    return FGPU_OK;
}

// The batched kernels were given every disk's step buffers at creation; a
// half step of a disk alone (fgpu_gas_kick without fgpu_transport) leaves its
// velocities in the other pair.
static int check_canonical(fgpu_batch *b)
{
    for (int k = 0; k < b->nd; ++k) {
        if (!b->disks[k]->canonical()) {
            b->err = "disk " + std::to_string(k) +
                     " is between the kick and the transport of a step";
            return FGPU_ERR_BAD_ARG;
        }
    }
    return FGPU_OK;
}

extern "C" int fgpu_batch_step(fgpu_batch *b, const double *dt, const double *t)
{
    nvtxRangePushA("fgpu_batch_step");
    struct Pop { ~Pop() { nvtxRangePop(); } } nvtx_pop_;
    if (!b || !dt || !t) return FGPU_ERR_BAD_ARG;
    for (int k = 0; k < b->nd; ++k) {
        if (!(dt[k] >= 0.0) || !std::isfinite(dt[k])) {
            b->err = "dt must be finite and >= 0";
            return FGPU_ERR_BAD_ARG;
        }
    }
    CKB(cudaStreamSynchronize(b->stream));
    if (int rc = check_canonical(b)) return rc;
    for (int k = 0; k < b->nd; ++k) {
        StepF &s = b->h_steps[k];
        s.dt = dt[k];
        s.t = t[k];
        s.fdt = (float)dt[k];
        s.beta_inv = (float)b->disks[k]->beta_inv_at(t[k]);
        s.run = dt[k] > 0.0;
        s.b = b->disks[k]->current_bodies();
    }
    CKB(cudaMemcpyAsync(b->d_steps, b->h_steps, sizeof(StepF) * b->nd, cudaMemcpyHostToDevice,
                        b->stream));
    enqueue_step(b, false);
    CKB(cudaGetLastError());
    CKB(cudaStreamSynchronize(b->stream));
    if (int rc = check_sequences(b)) return rc;
    for (int k = 0; k < b->nd; ++k)
        if (dt[k] > 0.0) b->disks[k]->set_cfl_valid(true);
    return FGPU_OK;
}

extern "C" int fgpu_batch_set_clock(fgpu_batch *b, int k, const fgpu_clock *c)
{
    if (!b || !c || k < 0 || k >= b->nd) return FGPU_ERR_BAD_ARG;
    if (c->n_planets < 0 || c->n_planets > kMaxBodies - 1 || !(c->monitor_dt > 0.0) ||
        !(c->cfl_max_var > 0.0) || !(c->last_dt > 0.0) || !(c->star_mass > 0.0)) {
        b->err = "clock: need 0 <= n_planets <= 15 and positive monitor_dt, cfl_max_var, "
                 "last_dt, star_mass";
        return FGPU_ERR_BAD_ARG;
    }
    for (int p = 0; p < c->n_planets; ++p) {
        if (!(c->a[p] > 0.0) || !(c->mass[p] >= 0.0)) {
            b->err = "clock: planets need a > 0 and mass >= 0";
            return FGPU_ERR_BAD_ARG;
        }
    }
    CKB(cudaStreamSynchronize(b->stream));
    const fgpu_params &p = b->disks[k]->params();
    ClockF &h = b->h_clocks[k];
    std::memset(&h, 0, sizeof(h));
    h.t = c->time;
    h.last_dt = c->last_dt;
    h.t_end = c->t_end;
    h.monitor_dt = c->monitor_dt;
    h.cfl_max_var = c->cfl_max_var;
    h.G = p.G;
    h.mstar = c->star_mass;
    h.beta_inv0 = 1 / p.cooling_beta_value;
    h.beta_ramp = p.cooling_beta_ramp_up;
    h.n_monitor = c->n_monitor;
    h.steps = c->steps;
    h.active = c->active;
    h.n_planets = c->n_planets;
    for (int q = 0; q < c->n_planets; ++q) {
        h.q[q] = c->mass[q];
        h.a[q] = c->a[q];
        h.phase[q] = c->phase[q];
    }
    b->aux[k].star_is_centre = c->star_mass == p.hydro_center_mass;
    CKB(cudaMemcpyAsync(b->d_clocks + k, &h, sizeof(ClockF), cudaMemcpyHostToDevice, b->stream));
    CKB(cudaMemcpyAsync(b->d_aux + k, &b->aux[k], sizeof(ClockAux), cudaMemcpyHostToDevice,
                        b->stream));
    CKB(cudaStreamSynchronize(b->stream));
    return FGPU_OK;
}

extern "C" int fgpu_batch_get_clock(fgpu_batch *b, int k, fgpu_clock *c)
{
    if (!b || !c || k < 0 || k >= b->nd) return FGPU_ERR_BAD_ARG;
    CKB(cudaMemcpyAsync(b->h_clocks + k, b->d_clocks + k, sizeof(ClockF), cudaMemcpyDeviceToHost,
                        b->stream));
    CKB(cudaStreamSynchronize(b->stream));
    const ClockF &h = b->h_clocks[k];
    std::memset(c, 0, sizeof(*c));
    c->time = h.t;
    c->last_dt = h.last_dt;
    c->t_end = h.t_end;
    c->monitor_dt = h.monitor_dt;
    c->cfl_max_var = h.cfl_max_var;
    c->star_mass = h.mstar;
    c->n_monitor = h.n_monitor;
    c->steps = h.steps;
    c->active = h.active;
    c->n_planets = h.n_planets;
    for (int q = 0; q < h.n_planets; ++q) {
        c->mass[q] = h.q[q];
        c->a[q] = h.a[q];
        c->phase[q] = h.phase[q];
    }
    return FGPU_OK;
}

static int build_graph(fgpu_batch *b, int steps)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_steps = 0;
    }
    CKB(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < steps; ++s) enqueue_step(b, true);
    cudaGraph_t g = nullptr;
    const cudaError_t launch_err = cudaGetLastError();
    const cudaError_t end_err = cudaStreamEndCapture(b->stream, &g);
    if (launch_err != cudaSuccess || end_err != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        b->err = std::string("graph capture: ") +
                 cudaGetErrorString(launch_err != cudaSuccess ? launch_err : end_err);
        return FGPU_ERR_CUDA;
    }
    const cudaError_t inst = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (inst != cudaSuccess) {
        b->graph = nullptr;
        b->err = std::string("graph instantiate: ") + cudaGetErrorString(inst);
        return FGPU_ERR_CUDA;
    }
    b->graph_steps = steps;
    return FGPU_OK;
}

extern "C" int fgpu_batch_run(fgpu_batch *b, int max_steps, int steps_per_graph, int *n_active)
{
    nvtxRangePushA("fgpu_batch_run");
    struct Pop { ~Pop() { nvtxRangePop(); } } nvtx_pop_;
    if (!b || max_steps < 0 || steps_per_graph < 1 || steps_per_graph > 4096)
        return FGPU_ERR_BAD_ARG;
    CKB(cudaStreamSynchronize(b->stream));
    if (int rc = check_canonical(b)) return rc;
    int done = 0;
    int active = -1;
    while (done < max_steps) {
        const int chunk = std::min(steps_per_graph, max_steps - done);
        if (chunk == steps_per_graph) {
            if (!b->graph || b->graph_steps != steps_per_graph) {
                int rc = build_graph(b, steps_per_graph);
                if (rc) return rc;
            }
            CKB(cudaGraphLaunch(b->graph, b->stream));
        } else {
            for (int s = 0; s < chunk; ++s) enqueue_step(b, true);
            CKB(cudaGetLastError());
        }
        done += chunk;
        CKB(cudaMemcpyAsync(b->h_active, b->d_active, sizeof(int), cudaMemcpyDeviceToHost,
                            b->stream));
        CKB(cudaStreamSynchronize(b->stream));
        if (int rc = check_sequences(b)) return rc;
        active = *b->h_active;
        if (active == 0) break;
    }
    if (active < 0) {
        // no step asked: count the active disks on the host copy
        CKB(cudaMemcpyAsync(b->h_clocks, b->d_clocks, sizeof(ClockF) * b->nd,
                            cudaMemcpyDeviceToHost, b->stream));
        CKB(cudaStreamSynchronize(b->stream));
        active = 0;
        for (int k = 0; k < b->nd; ++k)
            active += b->h_clocks[k].active && b->h_clocks[k].t < b->h_clocks[k].t_end;
    }
    for (int k = 0; k < b->nd; ++k) b->disks[k]->set_cfl_valid(true);
    if (n_active) *n_active = active;
    return FGPU_OK;
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
namespace {

struct Snapshot {
    std::vector<float *> dst;
    std::vector<const float *> src;
    std::vector<size_t> count;
    unsigned int *dtmin = nullptr;
    float *mem = nullptr;
};

}  // namespace

// copies of every array the step changes and carries to the next step
static int take_snapshot(fgpu_batch *b, Snapshot &s, bool restore)
{
    if (!restore) {
        size_t total = 0;
        for (int d = 0; d < b->nd; ++d) {
            const DiskF k = b->disks[d]->describe();
            const size_t cells = (size_t)k.g.nr * k.g.nz, vcells = cells + k.g.nz;
            const float *arrays[14] = {k.s.sigma, k.s.vr, k.s.dv, k.s.energy, k.s.sigma0,
                                       k.s.vr0, k.s.dv0, k.s.energy0, k.s.sigma_lo, k.P,
                                       k.cs, k.H, k.nu, k.T};
            const bool vec[14] = {0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int a = 0; a < 14; ++a) {
                s.src.push_back(arrays[a]);
                s.count.push_back(vec[a] ? vcells : cells);
                total += vec[a] ? vcells : cells;
            }
        }
        CKB(cudaMalloc(&s.mem, total * sizeof(float)));
        CKB(cudaMalloc(&s.dtmin, sizeof(unsigned int) * b->nd));
        size_t off = 0;
        for (size_t a = 0; a < s.src.size(); ++a) {
            s.dst.push_back(s.mem + off);
            off += s.count[a];
        }
    }
    for (size_t a = 0; a < s.src.size(); ++a) {
        if (restore)
            CKB(cudaMemcpyAsync((void *)s.src[a], s.dst[a], s.count[a] * sizeof(float),
                                cudaMemcpyDeviceToDevice, b->stream));
        else
            CKB(cudaMemcpyAsync(s.dst[a], s.src[a], s.count[a] * sizeof(float),
                                cudaMemcpyDeviceToDevice, b->stream));
    }
    for (int d = 0; d < b->nd; ++d) {
        const DiskF k = b->disks[d]->describe();
        if (restore)
            CKB(cudaMemcpyAsync(k.dtmin, s.dtmin + d, sizeof(unsigned int),
                                cudaMemcpyDeviceToDevice, b->stream));
        else
            CKB(cudaMemcpyAsync(s.dtmin + d, k.dtmin, sizeof(unsigned int),
                                cudaMemcpyDeviceToDevice, b->stream));
    }
    CKB(cudaStreamSynchronize(b->stream));
    return FGPU_OK;
}

static void candidates(const fgpu_batch *b, int k, std::vector<fgpu_tile> &out)
{
    out.clear();
    if (is_cell_kernel(k)) {
        for (int th : {64, 128, 256, 512})
            for (int r : {1, 2, 4, 8}) out.push_back({th, r});
    } else if (k == FGPU_BK_GHOST) {
        for (int th : {64, 128, 256}) out.push_back({th, 1});
    } else if (k == FGPU_BK_TRANSPORT_RADIAL) {
        for (int th : {32, 64, 128, 256})
            for (int r : {8, 16, 32, 64}) out.push_back({th, r});
    } else if (k == FGPU_BK_TRANSPORT_AZIMUTHAL) {
        for (int th : {96, 128, 192, 256, 384, 512})
            if (per_for(b->nz_max, th)) out.push_back({th, 1});
    } else {
        for (int th : {128, 256, 512}) out.push_back({th, 1});
    }
}

extern "C" int fgpu_batch_autotune(fgpu_batch *b, int reps, fgpu_tiles *best)
{
    if (!b || reps < 1 || reps > 1000) return FGPU_ERR_BAD_ARG;
    CKB(cudaStreamSynchronize(b->stream));
    if (int rc = check_canonical(b)) return rc;
    // a valid step description for every disk: its current CFL dt and bodies
    for (int k = 0; k < b->nd; ++k) {
        double dt = 0.0;
        int rc = b->disks[k]->cfl(&dt);
        if (rc) {
            b->err = b->disks[k]->err;
            return rc;
        }
        StepF &s = b->h_steps[k];
        s.dt = dt;
        s.fdt = (float)dt;
        s.t = b->h_clocks[k].t;
        s.beta_inv = (float)b->disks[k]->beta_inv_at(s.t);
        s.run = 1;
        s.b = b->disks[k]->current_bodies();
    }
    CKB(cudaMemcpyAsync(b->d_steps, b->h_steps, sizeof(StepF) * b->nd, cudaMemcpyHostToDevice,
                        b->stream));
    Snapshot snap;
    int rc = take_snapshot(b, snap, false);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    CKB(cudaEventCreate(&e0));
    CKB(cudaEventCreate(&e1));
    fgpu_tiles cur = b->tiles;
    std::vector<fgpu_tile> cands;
    for (int k = 0; k < FGPU_BK_COUNT && rc == FGPU_OK; ++k) {
        if ((k == FGPU_BK_ARTVISC_Q || k == FGPU_BK_ARTVISC_V) && !b->any_art) continue;
        if (k == FGPU_BK_DAMPING && !b->n_damp_items) continue;
        candidates(b, k, cands);
        float best_ms = 3.0e38f;
        fgpu_tile best_tile = cur.k[k];
        for (const fgpu_tile &c : cands) {
            fgpu_tiles trial = cur;
            trial.k[k] = c;
            if (apply_tiles(b, trial) != FGPU_OK) continue;  // shape not launchable here
            launch_kernel(b, k);
            cudaEventRecord(e0, b->stream);
            for (int r = 0; r < reps; ++r) launch_kernel(b, k);
            cudaEventRecord(e1, b->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
                b->err = "autotune: a candidate launch failed";
                rc = FGPU_ERR_CUDA;
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) {
                best_ms = ms;
                best_tile = c;
            }
        }
        cur.k[k] = best_tile;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == FGPU_OK) b->err.clear();
    const std::string keep = b->err;
    int rc2 = apply_tiles(b, cur);
    if (rc != FGPU_OK) b->err = keep;
    if (rc == FGPU_OK) rc = rc2;
    // put the state (evolved and derived fields, CFL minima) back
    int rc3 = take_snapshot(b, snap, true);
    if (rc == FGPU_OK) rc = rc3;
    cudaFree(snap.mem);
    cudaFree(snap.dtmin);
    if (rc == FGPU_OK && best) *best = b->tiles;
    return rc;
}
