"""GPU FP64 path against the oracle on synthetic disks larger than the
reference fixtures: noisy power-law disks, a planet, CFL-limited steps.
Bar: relative L-infinity <= 1e-10 per evolved field after the run, same CFL
dt sequence to 1e-12.  Also covers the azimuthal transport kernel with the
ring in more than 48 KB of shared memory and at 16 cells per thread."""
import math

import numpy as np
import pytest

from gpu_cases import initial_state, load, make_params
from golden_runner import EVOLVED, rel_linf

pytestmark = pytest.mark.gpu
TOL = 1e-10


def run_both(params, d, steps, planet=True, seed=3):
    from fargocpt_gb300.engine import Engine, grid_radii
    from oracle.oracle_py import OracleState

    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=seed)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0)]
    if planet:
        bodies.append((1.0, 0.05, 1e-3, 0.0, math.hypot(1.0, 0.05)))
    out = []
    for cls in (OracleState, Engine):
        b = cls(params, radii)
        load(b, st, bodies)
        b.apply_boundary_condition(0.0, 0.0, False)
        t, dts = 0.0, []
        for _ in range(steps):
            dt = b.condition_cfl()
            b.step_euler(dt, t)
            t += dt
            dts.append(dt)
        out.append((b, dts))
    return out


@pytest.mark.parametrize("adiabatic", [False, True])
@pytest.mark.parametrize("nrad,naz", [(24, 64), (64, 192)])
def test_gpu_vs_oracle_cfl_steps(adiabatic, nrad, naz):
    params, d = make_params(nrad, naz, adiabatic=adiabatic)
    (o, dto), (g, dtg) = run_both(params, d, steps=12)
    np.testing.assert_allclose(dtg, dto, rtol=1e-12)
    for f in EVOLVED:
        err = rel_linf(g.get_field(f), o.get_field(f))
        assert err <= TOL, f"{f}: {err:.3e}"
    ax_o = o.disk_on_planet_accel(1)
    ax_g = g.disk_on_planet_accel(1)
    np.testing.assert_allclose(ax_g, ax_o, rtol=1e-9, atol=1e-18)
    assert abs(g.total_mass() - o.total_mass()) <= 1e-13 * abs(o.total_mass())


@pytest.mark.parametrize("adiabatic", [True, False])
@pytest.mark.parametrize("naz", [1000, 1536, 4608, 6000, 6150, 7680])
def test_azimuthal_kernel_variants(naz, adiabatic):
    # the float-pair ring pass's variants: 1000 cells, 2 per thread on 512
    # threads with clamped loops; 1536 and 4608, 6 per thread on whole warps
    # (256 and 768 threads) with the shuffled fluxes; 6000, 6 per thread on
    # 1024 threads, clamped; 6150, 16 per thread, clamped, the ring in 197 KB
    # of shared memory; 7680, the ring's arrays in the global workspace (the
    # FP64-arithmetic pass: > 48 KB of shared memory from 1536 cells on)
    params, d = make_params(8, naz, adiabatic=adiabatic)
    (o, dto), (g, dtg) = run_both(params, d, steps=3, planet=False)
    np.testing.assert_allclose(dtg, dto, rtol=1e-12)
    for f in EVOLVED:
        assert rel_linf(g.get_field(f), o.get_field(f)) <= TOL, f


def test_mc_limiter_standard_transport():
    params, d = make_params(32, 96, adiabatic=True, flux_limiter=1, fast_transport=0)
    (o, _), (g, _) = run_both(params, d, steps=8)
    for f in EVOLVED:
        assert rel_linf(g.get_field(f), o.get_field(f)) <= TOL, f


@pytest.mark.parametrize("adiabatic", [False, True])
def test_leapfrog_with_moving_planet(adiabatic):
    """step_LeapFrog's gas part (simulation.cpp:276-459) composed from the
    phase functions: the planet drifted to the half step for the first kick,
    the indirect term renewed for the second, the LeapFrog CFL factor."""
    from fargocpt_gb300.engine import Engine, grid_radii
    from fargocpt_gb300.simulation import indirect_term_euler, step_leapfrog
    from oracle.oracle_py import OracleState

    params, d = make_params(32, 96, adiabatic=adiabatic, integrator=1)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=5)

    def bodies(t):
        x, y = math.cos(0.2 + t), math.sin(0.2 + t)
        return [(0.0, 0.0, 1.0, 0.0, 0.0), (x, y, 1e-3, 0.0, 1.0)]

    hyd = []
    for cls in (OracleState, Engine):
        h = cls(params, radii)
        load(h, st, bodies(0.0))
        h.apply_boundary_condition(0.0, 0.0, False)
        hyd.append(h)
    t = 0.0
    for _ in range(10):
        dts = [h.condition_cfl() for h in hyd]
        np.testing.assert_allclose(dts[1], dts[0], rtol=1e-12)
        dt = dts[0]
        b = bodies(t + dt / 2)
        ix, iy = indirect_term_euler(b)
        first = (b, ix, iy)
        second = (b, 0.9 * ix, 1.1 * iy)
        for h in hyd:
            step_leapfrog(h, dt, t, first, second)
        t += dt
    for f in EVOLVED:
        err = rel_linf(hyd[1].get_field(f), hyd[0].get_field(f))
        assert err <= TOL, f"{f}: {err:.3e}"


@pytest.mark.parametrize("adiabatic,stabilize", [(True, 0), (True, 1), (False, 2)])
def test_tw_artificial_viscosity_and_stabilize(adiabatic, stabilize):
    """Tscharnuter-Winkler artificial viscosity (artificial_viscosity.cpp:35-140)
    and StabilizeViscosity (viscosity.cpp:256-348, 395-417; cfl.cpp:332-351)
    with a constant viscosity that dominates the CFL, at CFL 1.3 so that the
    pseudo-implicit correction acts (dt |c| > 1 in cells) and the viscous dt
    limit binds."""
    params, d = make_params(48, 128, adiabatic=adiabatic, art_visc=2,
                            stabilize_viscosity=stabilize, viscous_alpha=0.0,
                            constant_viscosity=3e-3, cfl=1.3 if stabilize == 1 else 0.5)
    (o, dto), (g, dtg) = run_both(params, d, steps=10)
    np.testing.assert_allclose(dtg, dto, rtol=1e-12)
    for f in EVOLVED:
        err = rel_linf(g.get_field(f), o.get_field(f))
        assert err <= TOL, f"{f}: {err:.3e}"


@pytest.mark.parametrize("kind", ["kley", "sinkhole", "viscous"])
def test_accretion_onto_planet(kind):
    """AccreteOntoPlanets (accretion.cpp:84-480) on a 64 x 192 adiabatic disk:
    the removed mass and momentum (relative 1e-12) and the fields after
    accretion plus a step."""
    from fargocpt_gb300.abi import ACCRETION, FgpuAccretor
    from fargocpt_gb300.engine import Engine, grid_radii
    from oracle.oracle_py import OracleState

    params, d = make_params(64, 192, adiabatic=True, accretion_radius_fraction=1.5)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=7)
    x, y = 1.05 * math.cos(0.3), 1.05 * math.sin(0.3)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (x, y, 3e-3, 0.0, 1.05)]
    acc = FgpuAccretor(type=ACCRETION[kind], x=x, y=y, r=math.hypot(x, y),
                       phi=math.atan2(y, x), roche_radius=0.1 * 1.05,
                       efficiency={"kley": 10.0, "sinkhole": 5.0, "viscous": 300.0}[kind],
                       orbital_period=2 * math.pi * 1.05 ** 1.5)
    res = []
    for cls in (OracleState, Engine):
        h = cls(params, radii)
        load(h, st, bodies)
        h.apply_boundary_condition(0.0, 0.0, False)
        dt = h.condition_cfl()
        sums = h.accrete_onto_planet(acc, dt)
        h.step_euler(dt, 0.0)
        res.append((h, sums))
    (o, so), (g, sg) = res
    assert so[0] > 0
    np.testing.assert_allclose(sg, so, rtol=1e-12, atol=1e-14 * abs(so[0]))
    for f in EVOLVED:
        err = rel_linf(g.get_field(f), o.get_field(f))
        assert err <= TOL, f"{f}: {err:.3e}"


@pytest.mark.parametrize("keplerian", [False, True])
def test_center_of_mass_boundary(keplerian):
    """The centre-of-mass composite (center_of_mass.cpp) at both edges with
    its damping, on a 48 x 128 adiabatic disk in a rotating frame: a centre
    that moves within and between steps, the binary branch of the
    viscous-speed tables, the quadrupole term of the outer model; or the
    Keplerian model with InitializeVradialZero."""
    from fargocpt_gb300.engine import Engine, grid_radii
    from oracle.oracle_py import OracleState

    params, d = make_params(48, 128, adiabatic=True, composite_inner=1, composite_outer=1,
                            damping_inner=[0, 0, 0, 0], damping_outer=[0, 0, 0, 0],
                            damping_inner_limit=1.2, damping_outer_limit=0.85,
                            binary_quadrupole_moment=2e-4,
                            initialize_pure_keplerian=int(keplerian),
                            initialize_vradial_zero=1, temperature_cgs_to_code=1e-3)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=11)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (1.0, 0.05, 1e-3, 0.0, math.hypot(1.0, 0.05))]

    def centres(n):
        ph = 0.3 + 0.05 * n
        q = 1e-3 / 1.001
        return [(0.0, 0.0, 0.0, 0.0, 1.0),
                (q * math.cos(ph), q * math.sin(ph), -q * math.sin(ph), q * math.cos(ph), 1.001)]

    res = []
    for cls in (OracleState, Engine):
        b = cls(params, radii)
        load(b, st, bodies)
        b.set_bodies(bodies, 0.0, 0.0, 0.25)
        b.init_center_of_mass_boundary(1.001, 1.0, 1, 1.0 * 1e-3 / 1.001)
        b.set_frame_centers(centres(0))
        b.apply_boundary_condition(0.0, 0.0, False)
        t = 0.0
        for n in range(8):
            b.set_frame_centers(centres(n), centres(n + 1))
            dt = b.condition_cfl()
            b.step_euler(dt, t)
            t += dt
        res.append(b)
    o, g = res
    for f in EVOLVED:
        err = rel_linf(g.get_field(f), o.get_field(f))
        assert err <= TOL, f"{f}: {err:.3e}"


@pytest.mark.parametrize("precision", [0, 1])
def test_engines_with_different_rings_coexist(precision):
    # A kernel's dynamic shared-memory limit is process-wide: an engine with
    # short rings created after one with long rings (more than 48 KB of ring
    # in shared memory) must not lower the limit the first one launches with.
    from fargocpt_gb300.engine import Engine, grid_radii

    engines = []
    for naz in (1536, 64):
        params, d = make_params(16, naz, precision=precision)
        radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
        e = Engine(params, radii)
        load(e, initial_state(d, radii, seed=5), [(0.0, 0.0, 1.0, 0.0, 0.0)])
        engines.append(e)
    for e in engines:
        e.step_euler(e.condition_cfl(), 0.0)
        assert np.all(np.isfinite(e.get_field("SIGMA")))


@pytest.mark.parametrize("nrad,naz,adiabatic", [(6, 8, False), (6, 9, True), (7, 13, False),
                                                (12, 24, True), (9, 127, True),
                                                (8, 8192, False)])
def test_edge_grids_against_oracle(nrad, naz, adiabatic):
    """The smallest grids the engine takes (6 rings incl. ghosts, 8 cells per
    ring), odd and prime ring lengths (ring ends that do not fill a warp or a
    block), and the longest ring (8192 cells): FP64 within 1e-10 of the
    oracle after five CFL-limited steps with the same dt sequence,
    FP32-mixed finite and within 1e-4 in sigma."""
    from fargocpt_gb300.engine import Engine, grid_radii
    from oracle.oracle_py import OracleState

    params, d = make_params(nrad, naz, adiabatic=adiabatic)
    p32, _ = make_params(nrad, naz, adiabatic=adiabatic, precision=1)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=21)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (1.0, 0.05, 1e-3, 0.0, math.hypot(1.0, 0.05))]
    runs = []
    for cls, p in ((OracleState, params), (Engine, params), (Engine, p32)):
        b = cls(p, radii)
        load(b, st, bodies)
        b.apply_boundary_condition(0.0, 0.0, False)
        t, dts = 0.0, []
        for _ in range(5):
            dt = b.condition_cfl()
            b.step_euler(dt, t)
            t += dt
            dts.append(dt)
        runs.append((b, dts))
    (o, dto), (g, dtg), (f, _) = runs
    np.testing.assert_allclose(dtg, dto, rtol=1e-12)
    for fld in EVOLVED:
        ref = o.get_field(fld)
        if not np.any(ref):
            continue
        err = rel_linf(g.get_field(fld), ref)
        assert err <= TOL, f"FP64 {fld}: {err:.3e}"
        assert np.all(np.isfinite(f.get_field(fld)))
    assert rel_linf(f.get_field("SIGMA"), o.get_field("SIGMA")) <= 1e-4


@pytest.mark.parametrize("adiabatic", [False, True])
def test_cfl_limiting_cell_matches_oracle(adiabatic):
    """The CFL report (timestep_debug_report, cfl.cpp:38-182): the same
    limiting cell as the oracle, its time step to 1e-12 and inverse times to
    1e-11 of the largest, and
    min(dt_cell, dt_shear) equal to the engine's CFL step."""
    params, d = make_params(24, 64, adiabatic=adiabatic)
    (o, _), (g, _) = run_both(params, d, steps=4)
    co, cg = o.cfl_limiting_cell(), g.cfl_limiting_cell()
    assert (cg.ring, cg.azimuth, cg.shear_ring) == (co.ring, co.azimuth, co.shear_ring)
    assert 1 <= cg.ring < d["nrad"] - 1
    assert abs(cg.dt_cell - co.dt_cell) <= 1e-12 * co.dt_cell
    assert abs(cg.dt_shear - co.dt_shear) <= 1e-12 * co.dt_shear
    # the terms enter as a root sum of squares; small ones (v_phi less its
    # ring mean) carry the fields' 1e-13 differences relatively amplified
    scale = max(abs(b) for b in co.invdt)
    for a, b in zip(cg.invdt, co.invdt):
        assert abs(a - b) <= 1e-11 * scale
    assert min(cg.dt_cell, cg.dt_shear) == pytest.approx(g.condition_cfl(), rel=1e-14)
