"""The drop-in translation unit (fargocpt_gb300/host/gpu_simulation.cpp, built
into FargoCPT as oracle/_ref/dropin/fargocpt_gpu when the reference's sources
are present) maps FargoCPT's configuration onto fgpu_params itself, from
parameters:: and the boundary set-up's function pointers.  For every golden
case it runs FargoCPT's own start-up on the case's setup file with
FGPU_DUMP_PARAMS set; the block it derives must equal the one the fixtures
were replayed with (tests/golden/<case>.json), which reproduce the reference
bit for bit.  Without a GPU the run then stops at fgpu_create (no device), as
the product path must: there is no CPU fallback."""
import json
import os
import subprocess

import numpy as np
import pytest

from fargocpt_gb300.abi import FgpuParams, params_from_dict, params_to_dict
from golden_runner import CASES, GOLDEN

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(REPO, "oracle", "_ref", "dropin", "fargocpt_gpu")


@pytest.mark.parametrize("name", CASES)
def test_dropin_derives_the_fixture_parameters(name, tmp_path):
    if not os.path.exists(EXE):
        pytest.skip("the drop-in build needs the reference's sources")
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        meta = json.load(f)
    pd = meta["params"]
    (tmp_path / "setup.yml").write_text(open(os.path.join(GOLDEN, f"{name}.yml")).read())
    np.full((pd["nrad"], pd["naz"]), 1e-3).astype("<f8").tofile(tmp_path / "sigma_init.dat")
    dump = tmp_path / "params.bin"
    env = {**os.environ, "FGPU_DUMP_PARAMS": str(dump), "OMP_NUM_THREADS": "1",
           "CUDA_VISIBLE_DEVICES": ""}
    r = subprocess.run([EXE, "start", "setup.yml"], cwd=tmp_path, capture_output=True,
                       text=True, env=env, timeout=120)
    assert dump.exists(), r.stdout[-2000:] + r.stderr[-2000:]
    # no device here: the run must stop at the engine, never fall back
    assert r.returncode != 0
    assert "fgpu_create failed" in r.stdout + r.stderr
    got = params_to_dict(FgpuParams.from_buffer_copy(dump.read_bytes()))
    want = params_to_dict(params_from_dict(pd))
    for key, v in want.items():
        g = got[key]
        if isinstance(v, float):
            assert g == pytest.approx(v, rel=1e-15, abs=0.0), key
        else:
            assert g == v, key
