"""ctypes front end of the oracle (test infrastructure, not product code).

Loads oracle/liboracle.so (built by oracle/Makefile from fargo_oracle.c, a CPU
restatement of FargoCPT's hydro step) and exposes the same method names as
fargocpt_gb300.engine.Engine so that one run-loop driver can step either.
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from fargocpt_gb300.abi import (FIELDS, VECTOR_FIELDS, FgpuAccretor, FgpuBody,
                                FgpuCflCell, FgpuFrameCenter, FgpuParams)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
# the same source built with the reference's shipped flags (-Ofast
# -march=native): only the CPU baseline's timing uses it, never a comparison
LIB_TIMING = os.path.join(HERE, "liboracle_timing.so")


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None
_variant = "parity"


def use_timing_build() -> None:
    """Selects the shipped-flags build for this process (CPU baseline timing
    only); call it before the first OracleState."""
    global _variant, _lib
    if _lib is not None and _variant != "timing":
        raise RuntimeError("the parity build is already loaded in this process")
    _variant = "timing"


def _load():
    global _lib
    if _lib is not None:
        return _lib
    path = LIB_TIMING if _variant == "timing" else LIB
    if not os.path.exists(path):
        build_oracle()
    lib = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    lib.or_create.argtypes = [C.POINTER(FgpuParams), dp, C.POINTER(vp)]
    lib.or_destroy.argtypes = [vp]
    lib.or_set_field.argtypes = [vp, C.c_int, dp, C.c_int, C.c_int]
    lib.or_get_field.argtypes = [vp, C.c_int, dp, C.c_int, C.c_int]
    lib.or_set_bodies.argtypes = [vp, C.c_int, C.POINTER(FgpuBody), C.c_double,
                                  C.c_double, C.c_double]
    lib.or_set_threads.argtypes = [C.c_int]
    for name in ("or_init_euler", "or_recalculate_derived"):
        getattr(lib, name).argtypes = [vp, C.c_double]
    lib.or_condition_cfl.argtypes = [vp]
    lib.or_condition_cfl.restype = C.c_double
    lib.or_apply_boundary_condition.argtypes = [vp, C.c_double, C.c_double, C.c_int]
    lib.or_step_euler.argtypes = [vp, C.c_double, C.c_double]
    lib.or_disk_on_planet_accel.argtypes = [vp, C.c_int, dp]
    lib.or_total_mass.argtypes = [vp]
    lib.or_total_mass.restype = C.c_double
    for name in ("or_gas_total_mass", "or_gas_angular_momentum"):
        getattr(lib, name).argtypes = [vp, C.c_double]
        getattr(lib, name).restype = C.c_double
    lib.or_set_disk_mass_target.argtypes = [vp, C.c_double]
    lib.or_accrete_onto_planet.argtypes = [vp, C.POINTER(FgpuAccretor), C.c_double, dp]
    lib.or_init_center_of_mass_boundary.argtypes = [vp, C.c_double, C.c_double, C.c_int,
                                                    C.c_double]
    lib.or_correct_v_azimuthal.argtypes = [vp, C.c_double]
    lib.or_cfl_limiting_cell.argtypes = [vp, C.POINTER(FgpuCflCell)]
    lib.or_set_frame_centers.argtypes = [vp, C.POINTER(FgpuFrameCenter),
                                         C.POINTER(FgpuFrameCenter)]
    for name in ("or_calculate_potential", "or_viscous_stress_tensor"):
        getattr(lib, name).argtypes = [vp]
    for name in ("or_update_with_sourceterms", "or_artificial_viscosity",
                 "or_update_velocities_with_viscosity", "or_transport"):
        getattr(lib, name).argtypes = [vp, C.c_double]
    lib.or_recalculate_viscosity.argtypes = [vp, C.c_double]
    lib.or_substep3.argtypes = [vp, C.c_double, C.c_double]
    lib.or_gas_kick.argtypes = [vp, C.c_double, C.c_double]
    lib.or_transport.argtypes = [vp, C.c_double]
    lib.or_compute_pressure.argtypes = [vp]
    _lib = lib
    return lib


def set_threads(n: int) -> int:
    return _load().or_set_threads(int(n))


class OracleState:
    def __init__(self, params: FgpuParams, radii):
        self.lib = _load()
        self.params = params
        self.nr, self.nz = params.nrad, params.naz
        r = np.ascontiguousarray(radii, dtype=np.float64)
        assert r.size >= self.nr + 2
        h = C.c_void_p()
        rc = self.lib.or_create(C.byref(params), r.ctypes.data_as(C.POINTER(C.c_double)),
                                C.byref(h))
        if rc != 0:
            raise RuntimeError(f"or_create failed: {rc}")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.or_destroy(self.h)
            self.h = None

    def rows(self, name):
        return self.nr + 1 if name in VECTOR_FIELDS else self.nr

    def set_field(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        rc = self.lib.or_set_field(self.h, FIELDS[name], a.ctypes.data_as(C.POINTER(C.c_double)),
                                   self.rows(name), self.nz)
        if rc != 0:
            raise ValueError(f"or_set_field({name}) shape {a.shape}")

    def get_field(self, name):
        a = np.empty((self.rows(name), self.nz), dtype=np.float64)
        rc = self.lib.or_get_field(self.h, FIELDS[name], a.ctypes.data_as(C.POINTER(C.c_double)),
                                   self.rows(name), self.nz)
        if rc != 0:
            raise ValueError(name)
        return a

    def set_bodies(self, bodies, ix, iy, omega_frame=0.0):
        arr = (FgpuBody * max(1, len(bodies)))()
        for k, b in enumerate(bodies):
            vals = list(b) + [0.0] * (5 - len(b))
            arr[k] = FgpuBody(*vals)
        self.lib.or_set_bodies(self.h, len(bodies), arr, ix, iy, omega_frame)

    def init_euler(self, t):
        self.lib.or_init_euler(self.h, t)

    def recalculate_derived(self, t):
        self.lib.or_recalculate_derived(self.h, t)

    def condition_cfl(self):
        return self.lib.or_condition_cfl(self.h)

    def apply_boundary_condition(self, t, dt, final):
        self.lib.or_apply_boundary_condition(self.h, t, dt, 1 if final else 0)

    def step_euler(self, dt, t):
        self.lib.or_step_euler(self.h, dt, t)

    # the phases step_LeapFrog composes (simulation.cpp:276-459)
    def gas_kick(self, dt, t):
        self.lib.or_gas_kick(self.h, dt, t)

    def transport(self, dt):
        self.lib.or_transport(self.h, dt)

    def compute_pressure(self):
        self.lib.or_compute_pressure(self.h)

    def disk_on_planet_accel(self, k):
        out = (C.c_double * 2)()
        rc = self.lib.or_disk_on_planet_accel(self.h, k, out)
        if rc != 0:
            raise ValueError(k)
        return out[0], out[1]

    def total_mass(self):
        return self.lib.or_total_mass(self.h)

    def gas_total_mass(self, radius):
        return self.lib.or_gas_total_mass(self.h, radius)

    def gas_angular_momentum(self, radius):
        return self.lib.or_gas_angular_momentum(self.h, radius)

    def set_disk_mass_target(self, mass):
        self.lib.or_set_disk_mass_target(self.h, mass)

    def accrete_onto_planet(self, accretor, dt):
        out = (C.c_double * 3)()
        rc = self.lib.or_accrete_onto_planet(self.h, C.byref(accretor), dt, out)
        if rc != 0:
            raise ValueError(rc)
        return out[0], out[1], out[2]

    def init_center_of_mass_boundary(self, mass_all, mass_center, binary_on_primary,
                                     com_max_dist):
        rc = self.lib.or_init_center_of_mass_boundary(self.h, mass_all, mass_center,
                                                      int(binary_on_primary), com_max_dist)
        if rc != 0:
            raise ValueError(rc)

    def correct_v_azimuthal(self, domega):
        self.lib.or_correct_v_azimuthal(self.h, domega)

    def cfl_limiting_cell(self):
        out = FgpuCflCell()
        self.lib.or_cfl_limiting_cell(self.h, C.byref(out))
        return out

    def set_frame_centers(self, now, after=None):
        n = (FgpuFrameCenter * 2)(*[FgpuFrameCenter(*c) for c in now])
        a = (FgpuFrameCenter * 2)(*[FgpuFrameCenter(*c) for c in after]) if after else None
        self.lib.or_set_frame_centers(self.h, n, a)

    # phase-by-phase access for kernel tests
    def phase(self, name, *args):
        getattr(self.lib, "or_" + name)(self.h, *args)
