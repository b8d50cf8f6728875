"""A C program drives the engine through include/fargocpt_gb300.h alone
(tests/abi_client/abi_client.c, built here with the system C compiler and
linked against libfargocpt_gb300.so): a 64 x 192 adiabatic disk with a
planet, the start-up calls and 12 CFL-limited Euler steps.  Its dt sequence,
fields and disk forces must match the oracle's run of the same inputs (dt to
1e-12, fields to relative L-infinity 1e-10, forces to 1e-9) and the Python
front end's run bit for bit: both call the same library."""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from gpu_cases import initial_state, make_params
from golden_runner import EVOLVED, rel_linf

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STEPS = 12


def _build_client(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.join(REPO, "fargocpt_gb300")
    exe = tmp_path / "abi_client"
    subprocess.run([cc, "-std=c99", "-O2", "-Wall", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "abi_client", "abi_client.c"), "-o", str(exe),
                    "-L", libdir, "-lfargocpt_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def _run(backend_cls, params, radii, st, bodies):
    h = backend_cls(params, radii)
    for f, a in st.items():
        h.set_field(f, a)
        h.set_field(f + "0", a)
    h.set_bodies(bodies, 0.0, 0.0, 0.0)
    h.init_euler(0.0)
    h.apply_boundary_condition(0.0, 0.0, False)
    t, dts = 0.0, []
    for _ in range(STEPS):
        dt = h.condition_cfl()
        h.step_euler(dt, t)
        dts.append(dt)
        t += dt
    forces = [h.disk_on_planet_accel(k) for k in range(len(bodies))]
    return {f: h.get_field(f) for f in EVOLVED}, dts, forces


def test_c_caller_matches_oracle_and_python(tmp_path):
    from fargocpt_gb300.abi import FgpuBody
    from fargocpt_gb300.engine import Engine, grid_radii
    from oracle.oracle_py import OracleState

    exe = _build_client(tmp_path)
    params, d = make_params(64, 192, adiabatic=True)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=5)
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (1.05, -0.2, 1e-3, 0.0, math.hypot(1.05, -0.2))]
    (tmp_path / "params.bin").write_bytes(bytes(params))
    radii.astype("<f8").tofile(tmp_path / "radii.bin")
    arr = (FgpuBody * len(bodies))(*[FgpuBody(*b) for b in bodies])
    (tmp_path / "bodies.bin").write_bytes(bytes(arr))
    for f, a in st.items():
        np.ascontiguousarray(a, dtype="<f8").tofile(tmp_path / f"{f}.bin")
    r = subprocess.run([str(exe), str(tmp_path), str(STEPS)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    naz = d["naz"]
    got = {f: np.fromfile(tmp_path / f"out_{f}.bin", dtype="<f8").reshape(-1, naz)
           for f in EVOLVED}
    dts = np.fromfile(tmp_path / "out_dt.bin", dtype="<f8")
    force = np.fromfile(tmp_path / "out_force.bin", dtype="<f8").reshape(-1, 2)

    ref, ref_dts, ref_force = _run(OracleState, params, radii, st, bodies)
    np.testing.assert_allclose(dts, ref_dts, rtol=1e-12, atol=0)
    for f in EVOLVED:
        assert rel_linf(got[f], ref[f]) <= 1e-10, f
    np.testing.assert_allclose(force[1], ref_force[1], rtol=1e-9)

    py, py_dts, py_force = _run(Engine, params, radii, st, bodies)
    assert np.array_equal(dts, py_dts)
    for f in EVOLVED:
        assert np.array_equal(got[f], py[f]), f
    assert np.array_equal(force, np.array(py_force))
