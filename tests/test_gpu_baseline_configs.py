"""The FP64 drop-in against the oracle on the benchmark disks themselves,
over 100 CFL-limited steps (the FP64 parity bar, 1e-10):

* the locally isothermal 128 x 384 disk (r in [0.4, 2.5], one planet of mass
  ratio 1e-3 at r = 1, FARGO, reference damping, CFL 0.5);
* the adiabatic 512 x 1536 disk (r in [0.3, 3.0], gamma 1.4, beta cooling
  with beta = 10, SN artificial viscosity sqrt(2), flaring 0.25, the planet).

Both start from the same seeded sigma (1e-3 uniform noise) and run FargoCPT's
loop (CalculateTimeStep with CFLmaxVar, the clamp to monitor times every
1/20 orbit; sim::run, simulation.cpp:505-558) with the planet on its
circular orbit at each step's start.  Bars: every dt of the sequence within
1e-12 relative, the same number of monitor outputs, relative L-infinity
<= 1e-10 on sigma, v_r, v_phi and e after 100 steps, the disk force on the
planet within 1e-9 relative, the gas mass and angular momentum within 1e-12.
The oracle runs the 512 x 1536 disk's 100 steps in a few seconds on the
host's cores.  Both arithmetics of the kernels are held to these bars:
float pairs (the default) and FP64 (FARGO_GB300_FP64_ARITH=fp64).
"""
import math
import os

import numpy as np
import pytest

from golden_runner import EVOLVED, rel_linf

pytestmark = pytest.mark.gpu


def _run(cls, name, steps):
    from fargocpt_gb300 import setups
    from fargocpt_gb300.simulation import RunClock, advance, start

    params, d, radii, fields, nbody = setups.build(name)
    h = cls(params, radii)
    for k, a in fields.items():
        h.set_field(k, a)
        h.set_field(k + "0", a)
    b = nbody.bodies(0.0)
    h.set_bodies(b, *nbody.indirect(b), 0.0)
    h.init_euler(0.0)
    clock = RunClock(time=0.0, last_dt=1e-9)
    start(h, clock, d["cfl_max_var"])

    def bodies(c):
        bb = nbody.bodies(c.time)
        return bb, *nbody.indirect(bb)

    monitors = []
    advance(h, clock, cfl_max_var=d["cfl_max_var"], monitor_timestep=2 * math.pi / 20,
            t_final=1e9, max_steps=steps, bodies=bodies,
            on_monitor=lambda c: monitors.append(c.time))
    bb = nbody.bodies(clock.time)
    h.set_bodies(bb, *nbody.indirect(bb), 0.0)
    return h, clock, monitors, d


@pytest.mark.parametrize("arith", ["pair", "fp64"])
@pytest.mark.parametrize("name", ["c1", "c2"])
def test_fp64_benchmark_disk_100_steps_against_oracle(name, arith, monkeypatch):
    from fargocpt_gb300.engine import Engine
    from oracle.oracle_py import OracleState, set_threads

    monkeypatch.setenv("FARGO_GB300_FP64_ARITH", arith)
    set_threads(os.cpu_count() or 1)
    o, co, mo, d = _run(OracleState, name, 100)
    g, cg, mg, _ = _run(Engine, name, 100)
    assert len(cg.dts) == len(co.dts) == 100
    np.testing.assert_allclose(cg.dts, co.dts, rtol=1e-12, atol=0)
    assert len(mg) == len(mo)
    for f in EVOLVED:
        ref = o.get_field(f)
        if not np.any(ref):
            continue
        err = rel_linf(g.get_field(f), ref)
        assert err <= 1e-10, f"{name} {f}: rel Linf {err:.3e}"
    np.testing.assert_allclose(g.disk_on_planet_accel(1), o.disk_on_planet_accel(1),
                               rtol=1e-9, atol=0)
    rmax = d["rmax"]
    assert abs(g.gas_total_mass(rmax) - o.gas_total_mass(rmax)) <= \
        1e-12 * abs(o.gas_total_mass(rmax))
    assert abs(g.gas_angular_momentum(rmax) - o.gas_angular_momentum(rmax)) <= \
        1e-12 * abs(o.gas_angular_momentum(rmax))


def test_transport_arithmetic_request_is_checked(monkeypatch, capfd):
    """An unknown FARGO_GB300_FP64_ARITH value is refused at fgpu_create
    (status BAD_ARG, the message on stderr), never replaced by a default."""
    from fargocpt_gb300 import setups
    from fargocpt_gb300.engine import Engine, EngineError

    params, d, radii, fields, nbody = setups.build("c1")
    monkeypatch.setenv("FARGO_GB300_FP64_ARITH", "fp128")
    with pytest.raises(EngineError, match="BAD_ARG"):
        Engine(params, radii)
    assert "FARGO_GB300_FP64_ARITH=fp128" in capfd.readouterr().err


STRESS = ("DIV_V", "TAU_R_R", "TAU_PHI_PHI", "TAU_R_PHI")


def _perturbed(cls, seed=7):
    """The 512 x 1536 adiabatic disk with seeded relative noise of 1e-3 on
    v_phi and noise of 1e-3 of the orbital speed on v_r, so that div v and
    the stress tensor are of the velocities' own order (in the smooth initial
    disk they vanish or nearly so), after init_euler's stress evaluation."""
    from fargocpt_gb300 import setups

    params, d, radii, fields, nbody = setups.build("c2")
    rng = np.random.default_rng(seed)
    f = dict(fields)
    vaz = f["V_AZIMUTHAL"]
    f["V_AZIMUTHAL"] = vaz * (1.0 + 1e-3 * rng.standard_normal(vaz.shape))
    f["V_RADIAL"] = f["V_RADIAL"] + 1e-3 * float(np.max(np.abs(vaz))) * \
        rng.standard_normal(f["V_RADIAL"].shape)
    h = cls(params, radii)
    for k, a in f.items():
        h.set_field(k, a)
        h.set_field(k + "0", a)
    b = nbody.bodies(0.0)
    h.set_bodies(b, *nbody.indirect(b), 0.0)
    h.init_euler(0.0)
    return h


def _stress_err(got, ref, f, nr):
    # rows a stress evaluation writes (tau_r_phi: rings 1 .. nr - 1)
    rows = slice(1, nr) if f == "TAU_R_PHI" else slice(0, nr)
    scale = float(np.max(np.abs(ref[rows])))
    assert scale > 0.0, f
    return float(np.max(np.abs(got[rows] - ref[rows]))) / scale


@pytest.mark.parametrize("arith", ["pair", "fp64"])
def test_stress_fields_read_back_as_doubles(arith, monkeypatch):
    """div v, the viscous stress tensor and the artificial pressures, which
    the float-pair kernels pass between them as pairs, read back as the
    oracle's doubles through fgpu_download_field and fgpu_snapshot_begin;
    after a step, an upload of one of them (before anything read them) leaves
    the others as the step left them.  Relative L-infinity bars: 1e-11 on the
    same state, 1e-9 after one step of both."""
    from fargocpt_gb300.engine import Engine
    from fargocpt_gb300.output import Snapshotter
    from oracle.oracle_py import OracleState, set_threads

    monkeypatch.setenv("FARGO_GB300_FP64_ARITH", arith)
    set_threads(os.cpu_count() or 1)
    o = _perturbed(OracleState)
    g = _perturbed(Engine)
    snap = Snapshotter(g, fields=STRESS + ("SIGMA",))
    try:
        snap.begin()
        staged = {f: a.copy() for f, a in snap.wait().items()}
    finally:
        snap.close()
    for f in STRESS:
        got = g.get_field(f)
        err = _stress_err(got, o.get_field(f), f, g.nr)
        assert err <= 1e-11, f"{f}: rel Linf {err:.3e}"
        assert np.array_equal(staged[f], got), f
    dt = g.condition_cfl()
    o.condition_cfl()
    g.step_euler(dt, 0.0)
    o.step_euler(dt, 0.0)
    mark = np.full((g.nr, g.nz), 0.25)
    g.set_field("TAU_R_R", mark)
    assert np.array_equal(g.get_field("TAU_R_R"), mark)
    for f in ("DIV_V", "TAU_PHI_PHI", "TAU_R_PHI", "Q_R", "Q_PHI"):
        err = _stress_err(g.get_field(f), o.get_field(f), f, g.nr)
        assert err <= 1e-9, f"{f} after a step and an upload of TAU_R_R: {err:.3e}"


@pytest.mark.parametrize("arith", ["pair", "fp64"])
def test_fp64_full_size_disk_against_oracle(arith, monkeypatch):
    """The 2048 x 6144 three-planet adiabatic disk of the bench line, 10 CFL
    steps against the oracle: the production kernel variants at their full
    size (6 cells per thread on 1024-thread ring blocks with the shuffled
    fluxes, the radial walk's 32-ring chunks, the four-body disk force).
    Bars as for the 100-step runs: dt within 1e-12, fields within 1e-10
    relative L-infinity, the force on the first planet within 1e-9."""
    from fargocpt_gb300.engine import Engine
    from oracle.oracle_py import OracleState, set_threads

    monkeypatch.setenv("FARGO_GB300_FP64_ARITH", arith)
    set_threads(os.cpu_count() or 1)
    o, co, _, _ = _run(OracleState, "c5", 10)
    g, cg, _, _ = _run(Engine, "c5", 10)
    np.testing.assert_allclose(cg.dts, co.dts, rtol=1e-12, atol=0)
    for f in EVOLVED:
        ref = o.get_field(f)
        if not np.any(ref):
            continue
        err = rel_linf(g.get_field(f), ref)
        assert err <= 1e-10, f"c5 {f}: rel Linf {err:.3e}"
    np.testing.assert_allclose(g.disk_on_planet_accel(1), o.disk_on_planet_accel(1),
                               rtol=1e-9, atol=0)
