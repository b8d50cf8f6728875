"""Asynchronous snapshots (fgpu_snapshot_begin / fgpu_snapshot_wait): the
copy holds the fields as they were when it was queued, although the steps
queued after it run on; the files read back as FargoCPT's format."""
import numpy as np
import pytest

from gpu_cases import initial_state, load, make_params

pytestmark = pytest.mark.gpu

EVOLVED = ("SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY")


@pytest.mark.parametrize("precision", [0, 1])
def test_snapshot_while_stepping(precision, tmp_path):
    from fargocpt_gb300 import output
    from fargocpt_gb300.engine import Engine, grid_radii

    params, d = make_params(32, 96, adiabatic=True, precision=precision)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    e = Engine(params, radii)
    load(e, initial_state(d, radii, seed=2), [(0.0, 0.0, 1.0, 0.0, 0.0)])
    t = 0.0
    for _ in range(3):
        dt = e.condition_cfl()
        e.step_euler(dt, t)
        t += dt
    ref = {f: e.get_field(f) for f in EVOLVED}
    snap = output.Snapshotter(e)
    snap.begin()
    for _ in range(5):
        e.step_euler(e.condition_cfl(), t)
    got = snap.wait()
    for f in EVOLVED:
        assert np.array_equal(got[f], ref[f]), f
    assert not np.array_equal(e.get_field("SIGMA"), ref["SIGMA"])
    snap.write(str(tmp_path), snapshot=1, monitor=10, time=t, last_dt=1e-3, n_iter=8)
    assert np.array_equal(output.read_grid(str(tmp_path / "Sigma.dat"), d["naz"]), ref["SIGMA"])
    assert np.array_equal(output.read_grid(str(tmp_path / "vrad.dat"), d["naz"]),
                          ref["V_RADIAL"])
    assert output.read_misc(str(tmp_path / "misc.bin"))["n_iter"] == 8
    snap.close()
