"""fgpu_disk_force_static, the allocation-free disk-force entry point.

It exists for callers that hold sigma and the scale height in their own device
buffers and may not allocate device memory when they ask for the force (for
instance under a fixed device-memory budget, or on a hot path where an
allocation would synchronise the device).  Its scratch is a static device
array shared by all calls, so this test calls it several times in a row with
different bodies and checks each result against the regular entry points
(fgpu_disk_on_planet_accel, fgpu_total_mass) of an engine holding the same
disk, and each of the four inner/outer components against a numpy restatement
of ComputeDiskOnPlanetAccel (src/Force.cpp:23-122).  Tolerance: 1e-9 relative
on the force components (plus 1e-18 absolute for components near zero),
1e-12 relative on the mass.  Free device memory must not change across the
calls after the first (the first call on a device may load the module that
holds the static array).

This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C
import math

import numpy as np
import pytest

from gpu_cases import initial_state, load, make_params

pytestmark = pytest.mark.gpu


def split_force(sigma, H, radii, naz, G, eps, body):
    """(inner x, inner y, outer x, outer y) acceleration of the disk on body
    (x, y, m, r_sm, a): sigma less its ring mean (CorrectDiskSelfgravity),
    split at Rmed < a (Force.cpp:23-122), in numpy FP64."""
    nr = sigma.shape[0]
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    surf = math.pi * (rsup ** 2 - rinf ** 2) / naz
    phi = 2.0 * math.pi / naz * np.arange(naz)
    px, py, _, rsm, a = body
    out = np.zeros(4)
    for i in range(1, nr - 1):
        dx = rmed[i] * np.cos(phi) - px
        dy = rmed[i] * np.sin(phi) - py
        dsm2 = dx * dx + dy * dy + (eps * H[i]) ** 2
        dsm = np.sqrt(dsm2)
        fk = np.ones(naz)
        if rsm > 0.0:
            q = dsm / rsm
            fk = np.where(dsm < rsm, -(3.0 * q ** 4 - 4.0 * q ** 3), 1.0)
        w = G * surf[i] * (sigma[i] - sigma[i].mean()) / (dsm2 * dsm) * fk
        k = 0 if rmed[i] < a else 2
        out[k] += np.sum(w * dx)
        out[k + 1] += np.sum(w * dy)
    return out


def test_static_scratch_force_matches_engine_in_a_row():
    import torch

    from fargocpt_gb300.abi import FgpuBody, load_library
    from fargocpt_gb300.engine import Engine, grid_radii

    lib = load_library()
    params, d = make_params(64, 192, adiabatic=True)
    radii = grid_radii(d["radial_spacing"], d["rmin"], d["rmax"], d["nrad"])
    st = initial_state(d, radii, seed=7)
    # the planet's orbit lies inside the grid, so both halves of the split
    # are non-zero; the star at the origin has every ring outside it
    bodies = [(0.0, 0.0, 1.0, 0.0, 0.0), (0.9, 0.3, 1e-3, 0.05, math.hypot(0.9, 0.3))]
    eng = Engine(params, radii)
    load(eng, st, bodies)
    eng.apply_boundary_condition(0.0, 0.0, False)
    t = 0.0
    for _ in range(3):
        dt = eng.condition_cfl()
        eng.step_euler(dt, t)
        t += dt

    dev = torch.device("cuda", torch.cuda.current_device())
    sigma_h = eng.get_field("SIGMA")
    h_h = eng.get_field("SCALE_HEIGHT")
    sig = torch.from_numpy(sigma_h).to(dev)
    hh = torch.from_numpy(h_h).to(dev)
    rad = torch.from_numpy(np.ascontiguousarray(radii)).to(dev)
    out = torch.full((5,), float("nan"), dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    mass_ref = eng.total_mass()
    torch.cuda.synchronize()

    free_after_first = None
    for call, k in enumerate((1, 0, 1)):  # calls in a row, different bodies
        acc_ref = eng.disk_on_planet_accel(k)
        body = FgpuBody(*bodies[k])
        rc = lib.fgpu_disk_force_static(
            C.c_void_p(sig.data_ptr()), C.c_void_p(hh.data_ptr()), C.c_void_p(rad.data_ptr()),
            d["nrad"], d["naz"], d["G"], d["thickness_smoothing"], C.byref(body),
            C.c_void_p(out.data_ptr()), stream)
        assert rc == 0
        torch.cuda.synchronize()
        if call == 0:
            free_after_first = torch.cuda.mem_get_info()[0]
        o = out.cpu().numpy()
        acc = (o[0] + o[2], o[1] + o[3])
        np.testing.assert_allclose(acc, acc_ref, rtol=1e-9, atol=1e-18)
        assert abs(o[4] - mass_ref) <= 1e-12 * abs(mass_ref)
        split = split_force(sigma_h, h_h, radii, d["naz"], d["G"], d["thickness_smoothing"],
                            bodies[k])
        np.testing.assert_allclose(o[:4], split, rtol=1e-9, atol=1e-18)
        if k == 1:
            assert np.all(np.abs(split) > 0.0), "both halves of the split take part"
    assert torch.cuda.mem_get_info()[0] == free_after_first, "device memory was allocated"


def test_static_scratch_rejects_oversized_grids():
    from fargocpt_gb300.abi import FgpuBody, load_library

    lib = load_library()
    body = FgpuBody(1.0, 0.0, 1e-3, 0.0, 1.0)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.fgpu_disk_force_static(dummy, dummy, dummy, 16384 + 3, 64, 1.0, 0.6,
                                    C.byref(body), dummy, None)
    assert rc == -1
