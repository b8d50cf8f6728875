"""Python front end of the GB300 engine's C ABI.

Method names follow FargoCPT's hydro functions (reference src/SourceEuler.h,
src/TransportEuler.h, src/cfl.h, src/Force.h) so that a run loop written
against the reference's call sequence drives the engine unchanged.  Every
call goes through libfargocpt_gb300.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import (FIELDS, STATUS_NAMES, VECTOR_FIELDS, FgpuBody, FgpuCflCell, FgpuFrameCenter, FgpuParams,
                  load_library)


class EngineError(RuntimeError):
    pass


def grid_radii(spacing: int, rmin: float, rmax: float, nrad: int) -> np.ndarray:
    """FargoCPT's Radii[0 .. nrad+1] (init.cpp:93-110), computed by the library."""
    lib = load_library()
    out = np.empty(nrad + 2, dtype=np.float64)
    rc = lib.fgpu_grid_radii(spacing, rmin, rmax, nrad, out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise EngineError(f"fgpu_grid_radii: {STATUS_NAMES.get(rc, rc)}")
    return out


class Engine:
    """One disk resident in HBM.  Not thread-safe; all work on one stream."""

    def __init__(self, params: FgpuParams, radii):
        self.lib = load_library()
        self.params = params
        self.nr, self.nz = params.nrad, params.naz
        r = np.ascontiguousarray(radii, dtype=np.float64)
        if r.size < self.nr + 2:
            raise ValueError("radii must hold nrad + 2 values")
        self._radii = r
        h = C.c_void_p()
        rc = self.lib.fgpu_create(C.byref(params), r.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.byref(h))
        if rc != 0:
            raise EngineError(f"fgpu_create: {STATUS_NAMES.get(rc, rc)}")
        self.h = h

    @classmethod
    def attach(cls, handle, params: FgpuParams, radii, owner) -> "Engine":
        """Front end for a handle owned by someone else (a disk of a batch);
        closing it leaves the handle alone."""
        self = cls.__new__(cls)
        self.lib = load_library()
        self.params = params
        self.nr, self.nz = params.nrad, params.naz
        self._radii = np.ascontiguousarray(radii, dtype=np.float64)
        self.h = handle
        self._owner = owner
        return self

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_owner", None) is not None:
            self.h = None
            return
        if getattr(self, "h", None):
            self.lib.fgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.fgpu_last_error(self.h)
            raise EngineError(f"{what}: {STATUS_NAMES.get(rc, rc)}: "
                              f"{msg.decode() if msg else ''}")

    @property
    def stream(self) -> int:
        p = C.c_void_p()
        self._check(self.lib.fgpu_get_stream(self.h, C.byref(p)), "fgpu_get_stream")
        return p.value or 0

    # -- fields -------------------------------------------------------------
    def rows(self, name):
        return self.nr + 1 if name in VECTOR_FIELDS else self.nr

    def set_field(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.shape != (self.rows(name), self.nz):
            raise ValueError(f"{name}: shape {a.shape} != {(self.rows(name), self.nz)}")
        self._check(self.lib.fgpu_upload_field(self.h, FIELDS[name],
                                               a.ctypes.data_as(C.POINTER(C.c_double)),
                                               a.shape[0], a.shape[1]), f"upload {name}")

    def get_field(self, name):
        a = np.empty((self.rows(name), self.nz), dtype=np.float64)
        self._check(self.lib.fgpu_download_field(self.h, FIELDS[name],
                                                 a.ctypes.data_as(C.POINTER(C.c_double)),
                                                 a.shape[0], a.shape[1]), f"download {name}")
        return a

    # -- per-step host state ------------------------------------------------
    def set_bodies(self, bodies, ix, iy, omega_frame=0.0):
        arr = (FgpuBody * max(1, len(bodies)))()
        for k, b in enumerate(bodies):
            vals = list(b) + [0.0] * (5 - len(b))
            arr[k] = FgpuBody(*vals)
        self._check(self.lib.fgpu_set_bodies(self.h, len(bodies), arr, ix, iy, omega_frame),
                    "fgpu_set_bodies")

    # -- hydro functions ----------------------------------------------------
    def init_euler(self, t):
        self._check(self.lib.fgpu_init_euler(self.h, t), "fgpu_init_euler")

    def recalculate_derived(self, t):
        self._check(self.lib.fgpu_recalculate_derived(self.h, t), "fgpu_recalculate_derived")

    def condition_cfl(self) -> float:
        out = C.c_double()
        self._check(self.lib.fgpu_condition_cfl(self.h, C.byref(out)), "fgpu_condition_cfl")
        return out.value

    def apply_boundary_condition(self, t, dt, final):
        self._check(self.lib.fgpu_apply_boundary_condition(self.h, t, dt, 1 if final else 0),
                    "fgpu_apply_boundary_condition")

    def step_euler(self, dt, t):
        self._check(self.lib.fgpu_step_euler(self.h, dt, t), "fgpu_step_euler")

    # the phases step_LeapFrog composes (simulation.cpp:276-459)
    def gas_kick(self, dt, t):
        self._check(self.lib.fgpu_gas_kick(self.h, dt, t), "fgpu_gas_kick")

    def transport(self, dt):
        self._check(self.lib.fgpu_transport(self.h, dt), "fgpu_transport")

    def compute_pressure(self):
        self._check(self.lib.fgpu_compute_pressure(self.h), "fgpu_compute_pressure")

    def disk_on_planet_accel(self, k):
        out = (C.c_double * 2)()
        self._check(self.lib.fgpu_disk_on_planet_accel(self.h, k, out),
                    "fgpu_disk_on_planet_accel")
        return out[0], out[1]

    def disk_on_nbody_accel(self, n):
        """ComputeDiskOnNbodyAccel: [(ax, ay)] for the n bodies last set."""
        out = (C.c_double * (2 * max(1, n)))()
        self._check(self.lib.fgpu_disk_on_nbody_accel(self.h, out), "fgpu_disk_on_nbody_accel")
        return [(out[2 * k], out[2 * k + 1]) for k in range(n)]

    def total_mass(self):
        out = C.c_double()
        self._check(self.lib.fgpu_total_mass(self.h, C.byref(out)), "fgpu_total_mass")
        return out.value

    def gas_total_mass(self, radius):
        """quantities::gas_total_mass (quantities.cpp:51-74): rings with Rmed <= radius."""
        out = C.c_double()
        self._check(self.lib.fgpu_gas_total_mass(self.h, radius, C.byref(out)),
                    "fgpu_gas_total_mass")
        return out.value

    def gas_angular_momentum(self, radius):
        """quantities::gas_angular_momentum (quantities.cpp:242-276)."""
        out = C.c_double()
        self._check(self.lib.fgpu_gas_angular_momentum(self.h, radius, C.byref(out)),
                    "fgpu_gas_angular_momentum")
        return out.value

    def set_disk_mass_target(self, mass):
        """KeepDiskMassConstant's target, sim::init's total_disk_mass_old
        (simulation.cpp:476-480)."""
        self._check(self.lib.fgpu_set_disk_mass_target(self.h, mass),
                    "fgpu_set_disk_mass_target")

    def accrete_onto_planet(self, accretor, dt):
        """One planet's part of AccreteOntoPlanets; accretor is an
        abi.FgpuAccretor.  Returns (mass, x momentum, y momentum) taken."""
        out = (C.c_double * 3)()
        self._check(self.lib.fgpu_accrete_onto_planet(self.h, C.byref(accretor), dt, out),
                    "fgpu_accrete_onto_planet")
        return out[0], out[1], out[2]

    def init_center_of_mass_boundary(self, mass_all, mass_center, binary_on_primary,
                                     com_max_dist):
        """init_center_of_mass (center_of_mass.cpp:25-27): the viscous-speed
        tables of a centerofmass composite boundary."""
        self._check(self.lib.fgpu_init_center_of_mass_boundary(
            self.h, mass_all, mass_center, int(binary_on_primary), com_max_dist),
            "fgpu_init_center_of_mass_boundary")

    def set_frame_centers(self, now, after=None):
        """now / after: two (x, y, vx, vy, mass) centres, of the first
        n_bodies_for_hydroframe_center bodies and of all bodies."""
        n = (FgpuFrameCenter * 2)(*[FgpuFrameCenter(*c) for c in now])
        a = (FgpuFrameCenter * 2)(*[FgpuFrameCenter(*c) for c in after]) if after else None
        self._check(self.lib.fgpu_set_frame_centers(self.h, n, a), "fgpu_set_frame_centers")

    def cfl_limiting_cell(self):
        """The cell that limits the CFL step (cfl.cpp:38-182): an
        abi.FgpuCflCell with ring, azimuth, dt_cell, invdt[6], shear_ring,
        dt_shear."""
        out = FgpuCflCell()
        self._check(self.lib.fgpu_cfl_limiting_cell(self.h, C.byref(out)),
                    "fgpu_cfl_limiting_cell")
        return out

    def correct_v_azimuthal(self, domega):
        """correct_v_azimuthal (SideEuler.cpp:79-95), for a corotating frame
        whose OmegaFrame changed by domega."""
        self._check(self.lib.fgpu_correct_v_azimuthal(self.h, domega),
                    "fgpu_correct_v_azimuthal")

    def check_finite(self):
        f, i, j = C.c_int(), C.c_int(), C.c_int()
        rc = self.lib.fgpu_check_finite(self.h, C.byref(f), C.byref(i), C.byref(j))
        if rc == -5:
            return (f.value, i.value, j.value)
        self._check(rc, "fgpu_check_finite")
        return None

    def set_phase_timing(self, enable: bool):
        self._check(self.lib.fgpu_set_phase_timing(self.h, 1 if enable else 0),
                    "fgpu_set_phase_timing")

    def phase_times(self):
        """{phase: summed ms} over the steps recorded since the last call, and
        the number of steps."""
        buf = (C.c_double * 64)()
        n, steps = C.c_int(), C.c_int()
        self._check(self.lib.fgpu_phase_times(self.h, buf, 64, C.byref(n), C.byref(steps)),
                    "fgpu_phase_times")
        return ({self.lib.fgpu_phase_name(k).decode(): buf[k] for k in range(n.value)},
                steps.value)

    def synchronize(self):
        self._check(self.lib.fgpu_synchronize(self.h), "fgpu_synchronize")
