"""Size-independent properties of the GPU step at full benchmark sizes (the
step-for-step comparison with the oracle at these sizes is in
test_gpu_baseline_configs.py; these properties hold without a second
implementation):

* azimuthal equivariance: with only the central star, rotating the initial
  disk by k cells rotates the result by k cells, within the FP64 bar of
  1e-10 (the ring reductions change summation order with the rotation; v_r
  near the inner damping zone, the most sensitive field, differs by 1.7e-11
  of its largest value after one step, whichever arithmetic the kernels
  use);
* axisymmetry: an axisymmetric disk without a planet stays axisymmetric;
* finiteness after many steps of the C2-size adiabatic disk.
"""
import numpy as np
import pytest

from gpu_cases import initial_state, load, make_params
from golden_runner import EVOLVED, rel_linf

pytestmark = pytest.mark.gpu


def _engine(params, radii):
    from fargocpt_gb300.engine import Engine
    return Engine(params, radii)


def _radii(d):
    from fargocpt_gb300.engine import grid_radii
    return grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])


def _advance(e, steps):
    t = 0.0
    for _ in range(steps):
        dt = e.condition_cfl()
        e.step_euler(dt, t)
        t += dt


def test_rotation_equivariance_c2_size():
    params, d = make_params(512, 1536, adiabatic=True, rmin=0.3, rmax=3.0,
                            damping_time_radius_outer=3.0)
    radii = _radii(d)
    st = initial_state(d, radii, seed=11)
    k = 97
    rot = {f: np.roll(a, k, axis=1) for f, a in st.items()}
    star = [(0.0, 0.0, 1.0, 0.0, 0.0)]
    e1, e2 = _engine(params, radii), _engine(params, radii)
    load(e1, st, star)
    load(e2, rot, star)
    for e in (e1, e2):
        e.apply_boundary_condition(0.0, 0.0, False)
        _advance(e, 5)
    for f in EVOLVED:
        a = np.roll(e1.get_field(f), k, axis=1)
        assert rel_linf(e2.get_field(f), a) <= 1e-10, f


def test_axisymmetric_disk_stays_axisymmetric():
    params, d = make_params(128, 384, adiabatic=False)
    radii = _radii(d)
    st = initial_state(d, radii, seed=5, noise=0.0)
    e = _engine(params, radii)
    load(e, st, [(0.0, 0.0, 1.0, 0.0, 0.0)])
    e.apply_boundary_condition(0.0, 0.0, False)
    _advance(e, 20)
    vscale = np.max(np.abs(e.get_field("V_AZIMUTHAL")))
    for f in EVOLVED:
        a = e.get_field(f)
        spread = np.max(np.abs(a - a[:, :1]))
        scale = vscale if f.startswith("V_") else np.max(np.abs(a))
        assert spread <= 1e-12 * max(1e-300, scale), f


def test_c2_size_stays_finite():
    params, d = make_params(512, 1536, adiabatic=True, rmin=0.3, rmax=3.0,
                            damping_time_radius_outer=3.0)
    radii = _radii(d)
    st = initial_state(d, radii, seed=2)
    e = _engine(params, radii)
    load(e, st, [(0.0, 0.0, 1.0, 0.0, 0.0), (1.0, 0.0, 1e-3, 0.0, 1.0)])
    e.apply_boundary_condition(0.0, 0.0, False)
    _advance(e, 50)
    assert e.check_finite() is None


@pytest.mark.parametrize("precision", [0, 1])
def test_injected_nonfinite_value_is_reported(precision):
    """Failure detection without a GPU fault: a NaN planted on the host in an
    uploaded field is reported by fgpu_check_finite with its field, ring and
    azimuth (both forms); an infinite energy likewise; a clean state reports
    nothing; a non-positive dt is refused before any launch."""
    from fargocpt_gb300.abi import FIELDS
    params, d = make_params(16, 48, adiabatic=True, precision=precision)
    radii = _radii(d)
    st = initial_state(d, radii, seed=4)
    e = _engine(params, radii)
    load(e, st, [(0.0, 0.0, 1.0, 0.0, 0.0)])
    assert e.check_finite() is None
    bad = st["SIGMA"].copy()
    bad[5, 7] = np.nan
    e.set_field("SIGMA", bad)
    assert e.check_finite() == (FIELDS["SIGMA"], 5, 7)
    e.set_field("SIGMA", st["SIGMA"])
    hot = st["ENERGY"].copy()
    hot[9, 40] = np.inf
    e.set_field("ENERGY", hot)
    assert e.check_finite() == (FIELDS["ENERGY"], 9, 40)
    e.set_field("ENERGY", st["ENERGY"])
    assert e.check_finite() is None
    assert e.lib.fgpu_step_euler(e.h, 0.0, 0.0) == -1
    assert e.lib.fgpu_step_euler(e.h, -1.0, 0.0) == -1
