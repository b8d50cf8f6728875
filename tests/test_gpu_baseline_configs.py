"""The FP64 drop-in against the oracle on the benchmark disks themselves,
over 100 CFL-limited steps (the spec parity bar):

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
