"""Monitor reductions and the two disk-mass / disk-force switches.

* gas_total_mass and gas_angular_momentum within a radius
  (quantities.cpp:51-74, 242-276) against the reference's own Quantities.dat
  (fixture adi_planet_keep_mass_nocorr, 17 significant digits) and against
  the oracle on a 64 x 192 disk in a rotating frame.  Bars: FP64 1e-12
  relative; FP32-mixed 1e-6 relative (sigma is a compensated FP32 pair, the
  v_phi residual FP32, the sums FP64).
* KeepDiskMassConstant (simulation.cpp:246-251): after every step the gas
  mass within RMAX equals the target (FP64 1e-13, FP32-mixed 1e-7), and the
  fields follow the oracle within the FP64 bar (1e-10).
* CorrectDiskSelfgravity off (Force.cpp:64-66): the disk force follows the
  oracle within 1e-9 (FP64) and the FP64 form within 1e-5 (FP32-mixed).
"""
import math

import numpy as np
import pytest

from gpu_cases import initial_state, load, make_params
from golden_runner import EVOLVED, replay, rel_linf

pytestmark = pytest.mark.gpu


def _engine():
    from fargocpt_gb300.engine import Engine
    return Engine


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
def test_quantities_match_reference_monitor(precision, tol):
    quantities = {}
    replay(_engine(), "adi_planet_keep_mass_nocorr", {"precision": precision},
           quantities=quantities)
    from golden_runner import load_case
    _, arrays = load_case("adi_planet_keep_mass_nocorr")
    mon = arrays["quantities_monitor"]
    assert len(quantities) == len(mon)
    for row, n in enumerate(mon):
        m, l = quantities[int(n)]
        m_ref = arrays["quantities_mass"][row]
        l_ref = arrays["quantities_angular_momentum"][row]
        assert abs(m - m_ref) <= tol * abs(m_ref), (n, m, m_ref)
        assert abs(l - l_ref) <= tol * abs(l_ref), (n, l, l_ref)


def _pair(params, d, bodies, steps, omega_frame=0.0, keep_mass=False):
    from fargocpt_gb300.engine import Engine, grid_radii
    from oracle.oracle_py import OracleState

    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=11)
    out = []
    for cls in (OracleState, Engine):
        b = cls(params, radii)
        load(b, st, bodies)
        b.set_bodies(bodies, 0.0, 0.0, omega_frame)
        b.apply_boundary_condition(0.0, 0.0, False)
        if keep_mass:
            b.set_disk_mass_target(b.gas_total_mass(d["rmax"]))
        t = 0.0
        for _ in range(steps):
            dt = b.condition_cfl()
            b.step_euler(dt, t)
            t += dt
        out.append(b)
    return out


PLANET = [(0.0, 0.0, 1.0, 0.0, 0.0), (1.1, 0.2, 1e-3, 0.0, math.hypot(1.1, 0.2))]


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-6)])
def test_quantities_vs_oracle_rotating_frame(precision, tol):
    params, d = make_params(64, 192, adiabatic=True, precision=precision)
    o, g = _pair(params, d, PLANET, steps=8, omega_frame=0.25)
    for radius in (d["rmax"], 1.3, 0.5):
        m_o, l_o = o.gas_total_mass(radius), o.gas_angular_momentum(radius)
        m_g, l_g = g.gas_total_mass(radius), g.gas_angular_momentum(radius)
        assert abs(m_g - m_o) <= tol * abs(m_o), (radius, m_g, m_o)
        assert abs(l_g - l_o) <= tol * abs(l_o), (radius, l_g, l_o)
    # the rings beyond RMAX: none within a radius below the grid
    assert g.gas_total_mass(0.1) == 0.0


@pytest.mark.parametrize("precision", [0, 1])
def test_keep_disk_mass_constant(precision):
    params, d = make_params(64, 192, adiabatic=True, precision=precision,
                            keep_disk_mass_constant=1)
    o, g = _pair(params, d, PLANET, steps=12, keep_mass=True)
    target = o.gas_total_mass(d["rmax"])
    tol = 1e-13 if precision == 0 else 1e-7
    assert abs(g.gas_total_mass(d["rmax"]) - target) <= tol * target
    if precision == 0:
        for f in EVOLVED:
            err = rel_linf(g.get_field(f), o.get_field(f))
            assert err <= 1e-10, f"{f}: {err:.3e}"


def test_keep_disk_mass_constant_needs_a_target():
    from fargocpt_gb300.engine import Engine, EngineError, grid_radii

    params, d = make_params(24, 64, keep_disk_mass_constant=1)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    g = Engine(params, radii)
    load(g, initial_state(d, radii, seed=2), PLANET[:1])
    with pytest.raises(EngineError, match="BAD_ARG"):
        g.step_euler(1e-3, 0.0)


def test_disk_force_without_selfgravity_correction():
    from fargocpt_gb300.abi import params_from_dict

    params, d = make_params(64, 192, adiabatic=True, correct_disk_selfgravity=0)
    o, g = _pair(params, d, PLANET, steps=4)
    np.testing.assert_allclose(g.disk_on_planet_accel(1), o.disk_on_planet_accel(1),
                               rtol=1e-9, atol=1e-18)
    # FP32-mixed against the FP64 form on the same state
    d32 = dict(d, precision=1)
    from fargocpt_gb300.engine import Engine
    e32 = Engine(params_from_dict(d32), g._radii)
    for f in EVOLVED + ["SCALE_HEIGHT"]:
        e32.set_field(f, g.get_field(f))
    e32.set_bodies(PLANET, 0.0, 0.0, 0.0)
    np.testing.assert_allclose(e32.disk_on_planet_accel(1), g.disk_on_planet_accel(1),
                               rtol=1e-5)
    # and the correction changes the force
    params_on, _ = make_params(64, 192, adiabatic=True)
    e_on = Engine(params_on, g._radii)
    for f in EVOLVED + ["SCALE_HEIGHT"]:
        e_on.set_field(f, g.get_field(f))
    e_on.set_bodies(PLANET, 0.0, 0.0, 0.0)
    a_on, a_off = np.array(e_on.disk_on_planet_accel(1)), np.array(g.disk_on_planet_accel(1))
    assert np.max(np.abs(a_on - a_off)) > 1e-3 * np.max(np.abs(a_off))


@pytest.mark.parametrize("precision", [0, 1])
def test_disk_on_nbody_accel_matches_per_body_calls(precision):
    # ComputeDiskOnNbodyAccel (Pframeforce.cpp:194-220): every body in one
    # call equals one ComputeDiskOnPlanetAccel call per body, bit for bit
    from fargocpt_gb300 import setups
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine

    _, d, radii, fields, nbody = setups.build("c1")
    d = dict(d, precision=precision)
    e = Engine(params_from_dict(d), radii)
    for k, a in fields.items():
        e.set_field(k, a)
        e.set_field(k + "0", a)
    bodies = nbody.bodies(0.3) + [(1.7, -0.4, 3e-4, 0.0, math.hypot(1.7, -0.4))]
    e.set_bodies(bodies, 0.0, 0.0, 0.0)
    e.init_euler(0.0)
    all_at_once = e.disk_on_nbody_accel(len(bodies))
    assert len(all_at_once) == len(bodies)
    for k in range(len(bodies)):
        assert all_at_once[k] == e.disk_on_planet_accel(k)
