"""The FP32-mixed form (precision = FGPU_PRECISION_FP32_MIXED).

Bars (relative, per field):
* against the reference's FP64 snapshots (golden cases, <= 20 steps):
  sigma, v_phi and e within 1e-5 L-infinity; v_r, a small difference of
  large terms, within 1e-3 of its own maximum;
* against the FP64 form on a 128 x 384 disk over 300 steps: sigma L1 <= 2e-6,
  L-infinity <= 2e-5; v_phi residual about Keplerian L1 <= 5e-5;
* the upload/download round trip keeps v_phi to FP32 precision of the
  residual about Keplerian.
"""
import math

import numpy as np
import pytest

from golden_runner import CASES, EVOLVED, replay, rel_linf

pytestmark = pytest.mark.gpu


def _engine():
    from fargocpt_gb300.engine import Engine
    return Engine


def rel_l1(a, b):
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


@pytest.mark.parametrize("name", CASES)
def test_fp32_mixed_against_reference_snapshots(name):
    snaps, times, torques, dts, arrays = replay(_engine(), name, {"precision": 1})
    assert snaps
    for n, fields in snaps.items():
        for f in EVOLVED:
            ref = arrays[f"s{n}_{f}"]
            if not np.any(ref):
                continue
            err = rel_linf(fields[f], ref)
            tol = 1e-3 if f == "V_RADIAL" else 1e-5
            assert err <= tol, f"{name} snap {n} {f}: {err:.3e}"


def test_fp32_mixed_against_fp64_form():
    from fargocpt_gb300 import setups
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine

    p64, d, radii, fields, nbody = setups.build("c1")
    d32 = dict(d)
    d32["precision"] = 1
    engs = [Engine(p64, radii), Engine(params_from_dict(d32), radii)]
    for e in engs:
        for k, a in fields.items():
            e.set_field(k, a)
            e.set_field(k + "0", a)
        b = nbody.bodies(0.0)
        e.set_bodies(b, *nbody.indirect(b), 0.0)
        e.init_euler(0.0)
        e.apply_boundary_condition(0.0, 0.0, False)
    t = 0.0
    for _ in range(300):
        dt = engs[0].condition_cfl()
        b = nbody.bodies(t)
        ix, iy = nbody.indirect(b)
        for e in engs:
            e.set_bodies(b, ix, iy, 0.0)
            e.step_euler(dt, t)
        t += dt
    s64, s32 = engs[0].get_field("SIGMA"), engs[1].get_field("SIGMA")
    assert rel_l1(s32, s64) <= 2e-6
    assert rel_linf(s32, s64) <= 2e-5
    nr = d["nrad"]
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    vk = np.sqrt(1.0 / rmed)[:, None]
    v64, v32 = engs[0].get_field("V_AZIMUTHAL"), engs[1].get_field("V_AZIMUTHAL")
    assert rel_l1(v32 - vk, v64 - vk) <= 5e-5
    assert engs[1].check_finite() is None


def test_fp32_round_trip_keeps_residual_precision():
    from fargocpt_gb300 import setups
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine

    p64, d, radii, fields, nbody = setups.build("c1")
    d32 = dict(d)
    d32["precision"] = 1
    e = Engine(params_from_dict(d32), radii)
    v = fields["V_AZIMUTHAL"]
    e.set_field("V_AZIMUTHAL", v)
    back = e.get_field("V_AZIMUTHAL")
    nr = d["nrad"]
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    vk = np.sqrt(1.0 / rmed)[:, None]
    res = v - vk
    assert np.max(np.abs(back - v)) <= 1e-7 * np.max(np.abs(res))


@pytest.mark.parametrize("naz", [6144, 7680])
def test_fp32_long_rings_against_fp64_form(naz):
    """Long rings: 12 cells per thread with the rows staged in shared memory
    (6144) and 16 cells per thread without staging (7680), adiabatic, against
    the FP64 form after a few CFL steps."""
    from fargocpt_gb300.engine import Engine, grid_radii
    from gpu_cases import initial_state, load, make_params

    p64, d = make_params(8, naz, adiabatic=True)
    p32, _ = make_params(8, naz, adiabatic=True, precision=1)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=9)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0)]
    engs = [Engine(p64, radii), Engine(p32, radii)]
    for e in engs:
        load(e, st, bodies)
        e.apply_boundary_condition(0.0, 0.0, False)
    t = 0.0
    for _ in range(4):
        dt = engs[0].condition_cfl()
        for e in engs:
            e.step_euler(dt, t)
        t += dt
    s64, s32 = engs[0].get_field("SIGMA"), engs[1].get_field("SIGMA")
    assert rel_linf(s32, s64) <= 1e-6
    e64, e32 = engs[0].get_field("ENERGY"), engs[1].get_field("ENERGY")
    assert rel_linf(e32, e64) <= 1e-5


@pytest.mark.parametrize("name", [c for c in CASES if "accretion" in c])
def test_fp32_mixed_accreted_mass_matches_reference_monitor(name):
    # The removal acts on the compensated sigma pair with FP64 sums, so the
    # accreted mass per monitor interval (nbody/planet.cpp:357-369) follows
    # the reference's to the FP32 state's precision.
    from golden_runner import load_case
    accreted = {}
    _, _, _, _, arrays = replay(_engine(), name, {"precision": 1}, accreted=accreted)
    rate = arrays["body1_accretion_rate"]
    dt_mon = load_case(name)[0]["monitor_timestep"]
    assert len(accreted) == len(rate) - 1
    for n, m in accreted.items():
        assert abs(m / dt_mon - rate[n]) <= 1e-5 * rate[n], (n, m / dt_mon, rate[n])


@pytest.mark.parametrize("where", [(1.0, 0.05), (1.002, 0.0021), (1.6, -0.9)])
def test_fp32_disk_force_against_fp64_form(where):
    """ComputeDiskOnPlanetAccel (Force.cpp:23-122) with the ring mean removed
    (Pframeforce.cpp:175-190) on the same state in both forms: the FP32-mixed
    form forms distances as float pairs and sums in FP64, within 1e-6 of the
    FP64 acceleration (inner + outer parts) and 1e-12 of the mass, also with
    the planet inside a cell and with Klahr smoothing."""
    from fargocpt_gb300 import setups
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine

    p64, d, radii, fields, _ = setups.build("c1")
    d32 = dict(d)
    d32["precision"] = 1
    x, y = where
    r = math.hypot(x, y)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (x, y, 1e-3, 0.4 * 0.07 * r, r)]
    out = []
    for e in (Engine(p64, radii), Engine(params_from_dict(d32), radii)):
        for k, a in fields.items():
            e.set_field(k, a)
            e.set_field(k + "0", a)
        e.set_bodies(bodies, 0.0, 0.0, 0.0)
        e.init_euler(0.0)
        out.append((np.array(e.disk_on_planet_accel(1)), e.total_mass()))
    (a64, m64), (a32, m32) = out
    assert np.linalg.norm(a32 - a64) <= 1e-6 * np.linalg.norm(a64)
    assert abs(m32 - m64) <= 1e-12 * m64


def test_fp32_rotating_frame_against_fp64_form():
    """A rotating frame (OmegaFrame 0.25) with a change of OmegaFrame and the
    v_phi correction of handle_corotation half way, on a 48 x 128 adiabatic
    disk with a planet: the FP32-mixed form within 1e-5 of the FP64 form in
    sigma and in the frame's v_phi."""
    from fargocpt_gb300.engine import Engine, grid_radii
    from gpu_cases import initial_state, load, make_params

    p64, d = make_params(48, 128, adiabatic=True)
    p32, _ = make_params(48, 128, adiabatic=True, precision=1)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=13)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (1.0, 0.05, 1e-3, 0.0, math.hypot(1.0, 0.05))]
    engs = [Engine(p64, radii), Engine(p32, radii)]
    for e in engs:
        load(e, st, bodies)
        e.set_bodies(bodies, 0.0, 0.0, 0.25)
        e.apply_boundary_condition(0.0, 0.0, False)
    t, omega = 0.0, 0.25
    for n in range(8):
        if n == 4:
            for e in engs:
                e.correct_v_azimuthal(0.01)
            omega += 0.01
        dt = engs[0].condition_cfl()
        for e in engs:
            e.set_bodies(bodies, 0.0, 0.0, omega)
            e.step_euler(dt, t)
        t += dt
    assert rel_linf(engs[1].get_field("SIGMA"), engs[0].get_field("SIGMA")) <= 1e-5
    assert rel_linf(engs[1].get_field("V_AZIMUTHAL"), engs[0].get_field("V_AZIMUTHAL")) <= 1e-5



@pytest.mark.parametrize("naz,per", [(384, 4), (384, 12), (768, 8), (1536, 16), (6144, 12),
                                     (6144, 16)])
@pytest.mark.parametrize("adiabatic,fargo,mc", [(False, 1, 0), (True, 1, 0), (True, 0, 1)])
def test_register_blocked_ring_pass_matches_strided(naz, per, adiabatic, fargo, mc,
                                                     monkeypatch):
    """The register-blocked azimuthal pass (contiguous segments of `per`
    cells, one exchange of segment ends per quantity) against the strided
    pass: every cell's arithmetic is the same, so the fields after the steps
    are bit-identical, with FARGO (residual and uniform passes and the integer
    shift) and with standard transport and the MC limiter."""
    from gpu_cases import initial_state, load, make_params

    from fargocpt_gb300.engine import Engine, grid_radii

    params, d = make_params(16, naz, adiabatic=adiabatic, precision=1, fast_transport=fargo,
                            flux_limiter=mc)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=21)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (1.0, 0.3, 1e-3, 0.0, math.hypot(1.0, 0.3))]
    out = []
    for variant in ("strided", f"blocked{per}"):
        monkeypatch.setenv("FARGO_GB300_AZIMUTHAL", variant)
        e = Engine(params, radii)
        load(e, st, bodies)
        e.apply_boundary_condition(0.0, 0.0, False)
        t = 0.0
        for _ in range(6):
            dt = e.condition_cfl()
            e.step_euler(dt, t)
            t += dt
        out.append({f: e.get_field(f) for f in EVOLVED})
        e.close()
    for f in EVOLVED:
        assert np.array_equal(out[0][f], out[1][f]), f


def test_register_blocked_request_that_does_not_fit_is_refused(monkeypatch):
    from gpu_cases import make_params

    from fargocpt_gb300.engine import Engine, EngineError, grid_radii

    params, d = make_params(16, 392, precision=1)   # 392 cells: no 12-cell segments
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    monkeypatch.setenv("FARGO_GB300_AZIMUTHAL", "blocked12")
    with pytest.raises(EngineError, match="UNSUPPORTED"):
        Engine(params, radii)
