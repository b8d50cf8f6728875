"""The FP32-mixed form's accuracy bar against the FP64 oracle itself.

The locally isothermal 128 x 384 disk with one planet (r in [0.4, 2.5], FARGO,
SN artificial viscosity, damping, alpha 1e-3) is run for 10 orbits by the
oracle (the CPU restatement of FargoCPT's FP64 step) and by the FP32-mixed
engine from the same seeded state, with the oracle's CFL dt (clamped to the
output time) and the same planet positions every step.  Bar: sigma relative
L1 <= 1e-5 after 10 orbits (sum |a - b| / sum |b|); the v_phi residual about
Keplerian, v_r and the disk torque on the planet are reported alongside.
fargocpt_gb300.accuracy makes the same comparison against the FP64 GPU form
at larger sizes.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _l1(a, b):
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


def test_fp32_mixed_10_orbits_against_oracle():
    from fargocpt_gb300 import setups
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine
    from oracle.oracle_py import OracleState, set_threads

    set_threads(os.cpu_count() or 1)
    p64, d, radii, fields, nbody = setups.build("c1")
    p32 = params_from_dict(dict(d, precision=1))
    ref, fp32 = OracleState(p64, radii), Engine(p32, radii)
    for h in (ref, fp32):
        for k, a in fields.items():
            h.set_field(k, a)
            h.set_field(k + "0", a)
        b = nbody.bodies(0.0)
        h.set_bodies(b, *nbody.indirect(b), 0.0)
        h.init_euler(0.0)
        h.apply_boundary_condition(0.0, 0.0, False)
    t, t_end, steps = 0.0, 10 * 2 * math.pi, 0
    while t < t_end:
        dt = min(ref.condition_cfl(), t_end - t)
        if t_end - t - dt < 1e-12 * t_end:
            dt = t_end - t
        b = nbody.bodies(t)
        for h in (ref, fp32):
            h.set_bodies(b, *nbody.indirect(b), 0.0)
            h.step_euler(dt, t)
        t += dt
        steps += 1
    nr = d["nrad"]
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    vk = np.sqrt(d["G"] * d["hydro_center_mass"] / rmed)[:, None]
    sigma = _l1(fp32.get_field("SIGMA"), ref.get_field("SIGMA"))
    vres = _l1(fp32.get_field("V_AZIMUTHAL") - vk, ref.get_field("V_AZIMUTHAL") - vk)
    vr = _l1(fp32.get_field("V_RADIAL"), ref.get_field("V_RADIAL"))
    b = nbody.bodies(t)
    tq = []
    for h in (ref, fp32):
        h.set_bodies(b, *nbody.indirect(b), 0.0)
        ax, ay = h.disk_on_planet_accel(1)
        tq.append((b[1][0] * ay - b[1][1] * ax) * b[1][2])
    print(f"10 orbits, {steps} steps: sigma L1 {sigma:.2e}, v_phi residual L1 {vres:.2e}, "
          f"v_r L1 {vr:.2e}, torque {abs(tq[1] - tq[0]) / abs(tq[0]):.2e}")
    assert steps > 3000
    assert sigma <= 1e-5, sigma
    assert vres <= 1e-4 and vr <= 1e-4
