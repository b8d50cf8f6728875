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


@pytest.mark.parametrize("name", ["adi_planet_fixed_dt", "c1_cfl_100"])
@pytest.mark.parametrize("precision", [0, 1])
def test_snapshot_files_against_the_references(name, precision, tmp_path):
    """A reference case replayed on the GPU and written through the
    asynchronous snapshot path (staged on the device, copied on the second
    stream, written by fargocpt_gb300.output) against the files the reference
    wrote: every <name>.dat within the FP64 bar (relative L-infinity 1e-10;
    FP32-mixed: sigma, v_phi, e 1e-5 and v_r 1e-3 of its maximum), same
    size; misc.bin's snapshot and monitor numbers byte-equal, its time within
    1e-12 relative, OmegaFrame and FrameAngle equal, and in the FP64 form the
    hydro step count byte-equal and the last dt within 1e-11 (FP32-mixed:
    1e-5) (polargrid.cpp:135-180, output.cpp:494-527).  The CFL step is a
    function of the fields at its limiting cell, so it carries their
    differences: after the 100 steps of c1_cfl_100 the float-pair kernels
    leave the last dt 1.7e-12 from the reference's."""
    import struct

    from fargocpt_gb300 import output
    from golden_runner import replay, rel_linf

    dirs = {}

    def on_snapshot(hyd, n, clock):
        snap = output.Snapshotter(hyd)
        snap.begin()
        d = tmp_path / str(n)
        snap.write(str(d), snapshot=n, monitor=n, time=clock.time, last_dt=clock.last_dt,
                   n_iter=clock.n_hydro_iter)
        snap.close()
        dirs[n] = d

    _, _, _, _, arrays = replay(_engine_cls(), name, {"precision": precision},
                                on_snapshot=on_snapshot)
    assert set(dirs) == set(int(k) for k in arrays["keep"])
    for n, d in dirs.items():
        for f in EVOLVED:
            ref = arrays[f"s{n}_{f}"]
            raw = (d / (output.GRID_NAMES[f] + ".dat")).read_bytes()
            assert len(raw) == ref.size * 8
            got = np.frombuffer(raw, dtype="<f8").reshape(ref.shape)
            if not np.any(ref):
                assert not np.any(got)
                continue
            tol = 1e-10 if precision == 0 else (1e-3 if f == "V_RADIAL" else 1e-5)
            assert rel_linf(got, ref) <= tol, (name, n, f, rel_linf(got, ref))
        mine = (d / "misc.bin").read_bytes()
        theirs = arrays[f"s{n}_misc"].tobytes()
        assert len(mine) == len(theirs) == 48
        assert mine[:8] == theirs[:8]          # snapshot and monitor numbers
        t_m, om_m, fa_m, dt_m = struct.unpack_from("<dddd", mine, 8)
        t_r, om_r, fa_r, dt_r = struct.unpack_from("<dddd", theirs, 8)
        assert abs(t_m - t_r) <= 1e-12 * abs(t_r)
        assert (om_m, fa_m) == (om_r, fa_r)
        if precision == 0:
            assert mine[40:] == theirs[40:]    # the hydro step count
            assert abs(dt_m - dt_r) <= 1e-11 * abs(dt_r)
        else:
            # the FP32-mixed CFL step is within FP32 rounding of FargoCPT's
            assert abs(dt_m - dt_r) <= 1e-5 * abs(dt_r)


def _engine_cls():
    from fargocpt_gb300.engine import Engine
    return Engine
