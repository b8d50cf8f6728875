"""The C-ABI library without a GPU: it loads, exports every symbol of
include/fargocpt_gb300.h, computes the reference's radii on the host, and
reports a missing device instead of falling back to the CPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from fargocpt_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(REPO, "include", "fargocpt_gb300.h")).read()
    return sorted(set(re.findall(r"\b(fgpu_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(abi.LIB_PATH):
        from fargocpt_gb300.build import build
        build()
    return abi.load_library()


def test_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert set(declared) == set(abi.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(lib, name), name


def test_grid_radii_matches_reference_formula(lib):
    from golden_runner import load_case
    meta, arrays = load_case("iso_planet_fixed_dt")
    p = meta["params"]
    out = np.empty(p["nrad"] + 2)
    rc = lib.fgpu_grid_radii(1, p["rmin"], p["rmax"], p["nrad"],
                             out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    assert np.array_equal(out, arrays["radii"])


def test_bad_arguments_are_rejected(lib):
    out = np.empty(8)
    assert lib.fgpu_grid_radii(7, 0.4, 2.5, 6, out.ctypes.data_as(C.POINTER(C.c_double))) == -1
    assert lib.fgpu_grid_radii(1, 2.5, 0.4, 6, out.ctypes.data_as(C.POINTER(C.c_double))) == -1
    h = C.c_void_p()
    p = abi.FgpuParams()
    p.nrad, p.naz = 3, 8
    assert lib.fgpu_create(C.byref(p), out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(h)) == -1
    assert lib.fgpu_destroy(None) == -1


def test_unsupported_options_are_reported(lib):
    from gpu_cases import make_params
    out = np.zeros(40)
    h = C.c_void_p()
    p, _ = make_params(16, 32, stabilize_viscosity=3)
    assert lib.fgpu_create(C.byref(p), out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(h)) == -1
    p, _ = make_params(16, 9000)
    assert lib.fgpu_create(C.byref(p), out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(h)) == -4


def test_center_of_mass_composite_is_validated(lib):
    from gpu_cases import make_params
    radii = np.linspace(0.4, 2.5, 18)
    rd = radii.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    p, _ = make_params(16, 32, composite_outer=2)
    assert lib.fgpu_create(C.byref(p), rd, C.byref(h)) == -1
    # per-field damping on a centre-of-mass edge dies in the reference
    # (boundary_conditions/config.cpp:512-528)
    p, _ = make_params(16, 32, composite_outer=1)
    assert list(p.damping_outer) != [0, 0, 0, 0]
    assert lib.fgpu_create(C.byref(p), rd, C.byref(h)) == -1
    # the batched form has no centre-of-mass boundary
    q, _ = make_params(16, 48, composite_inner=1, damping_inner=[0, 0, 0, 0], precision=1)
    ps = (abi.FgpuParams * 1)(q)
    rp = (C.POINTER(C.c_double) * 1)(rd)
    assert lib.fgpu_batch_create(1, ps, rp, C.byref(h)) == -4
    assert lib.fgpu_init_center_of_mass_boundary(None, 1.0, 1.0, 0, 0.0) == -1
    assert lib.fgpu_set_frame_centers(None, None, None) == -1


def test_no_device_is_an_error_not_a_fallback(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from gpu_cases import make_params
    p, d = make_params(16, 32)
    radii = np.linspace(0.4, 2.5, 18)
    h = C.c_void_p()
    rc = lib.fgpu_create(C.byref(p), radii.ctypes.data_as(C.POINTER(C.c_double)), C.byref(h))
    assert rc == -6


def test_batch_arguments_and_missing_device(lib):
    from gpu_cases import make_params
    radii = np.linspace(0.4, 2.5, 18)
    rp = (C.POINTER(C.c_double) * 2)(*[radii.ctypes.data_as(C.POINTER(C.c_double))] * 2)
    p, _ = make_params(16, 48)
    ps = (abi.FgpuParams * 2)(p, p)
    h = C.c_void_p()
    assert lib.fgpu_batch_create(0, ps, rp, C.byref(h)) == -1
    assert lib.fgpu_batch_create(2, ps, None, C.byref(h)) == -1
    # the batched form is FP32-mixed only
    assert lib.fgpu_batch_create(2, ps, rp, C.byref(h)) == -4
    for q in ps:
        q.precision = 1
    assert lib.fgpu_batch_destroy(None) == -1
    try:
        import torch
        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    assert lib.fgpu_batch_create(2, ps, rp, C.byref(h)) == -6


def test_batch_tile_table_round_trips():
    t = abi.FgpuTiles()
    for i in range(len(abi.BATCH_KERNELS)):
        t.k[i].threads, t.k[i].rings = 32 * (i + 1), i + 1
    d = t.to_dict()
    assert list(d) == abi.BATCH_KERNELS
    back = abi.FgpuTiles.from_dict(d)
    assert bytes(back) == bytes(t)
