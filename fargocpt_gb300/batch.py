"""Python front end of the batched many-disk form (fgpu_batch_* of the C ABI).

A batch advances many independent FP32-mixed disks of different sizes, each
with its own CFL time step, with one launch per phase over all disks.  Each
disk is reachable as an :class:`~fargocpt_gb300.engine.Engine` (``batch.disks``)
for uploads, downloads and every single-disk call.  Two ways to step:

* ``step(dts, ts)``: one step of every disk with host-given dt and time and
  the bodies last given to each disk (``disks[k].set_bodies``);
* ``set_clock`` + ``run``: the device clock picks every disk's dt from its
  CFL minimum (FargoCPT's CalculateTimeStep and monitor clamp,
  simulation.cpp:100-118, 505-558), moves its planets on circular orbits
  and stops it at its end time; ``run`` relaunches CUDA graphs of steps.

There is no CPU fallback: every call goes through libfargocpt_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import math
import os

import numpy as np

from .abi import BATCH_KERNELS, STATUS_NAMES, FgpuClock, FgpuParams, FgpuTiles, load_library
from .engine import Engine, EngineError
from .simulation import RunClock, start


class Batch:
    def __init__(self, params: list[FgpuParams], radii: list):
        self.lib = load_library()
        n = len(params)
        if n == 0:
            raise ValueError("a batch needs at least one disk")
        self._params = (FgpuParams * n)(*params)
        self._radii = [np.ascontiguousarray(r, dtype=np.float64) for r in radii]
        for p, r in zip(params, self._radii):
            if r.size < p.nrad + 2:
                raise ValueError("radii must hold nrad + 2 values")
        ptrs = (C.POINTER(C.c_double) * n)(
            *[r.ctypes.data_as(C.POINTER(C.c_double)) for r in self._radii])
        h = C.c_void_p()
        rc = self.lib.fgpu_batch_create(n, self._params, ptrs, C.byref(h))
        if rc != 0:
            raise EngineError(f"fgpu_batch_create: {STATUS_NAMES.get(rc, rc)}")
        self.h = h
        self.n = n
        self.disks = []
        for k in range(n):
            dh = C.c_void_p()
            self._check(self.lib.fgpu_batch_disk(self.h, k, C.byref(dh)), "fgpu_batch_disk")
            self.disks.append(Engine.attach(dh, params[k], self._radii[k], self))

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.fgpu_batch_last_error(self.h)
            raise EngineError(f"{what}: {STATUS_NAMES.get(rc, rc)}: "
                              f"{msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            for d in self.disks:
                d.close()
            self.lib.fgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self) -> list[int]:
        return [p.nrad * p.naz for p in self._params]

    def signature(self) -> str:
        """Names the batch's shape for the tile cache: sizes and physics per disk."""
        rows = sorted((p.nrad, p.naz, p.eos, p.art_visc, p.damping) for p in self._params)
        return hashlib.sha1(json.dumps(rows).encode()).hexdigest()[:16]

    # -- tiles ----------------------------------------------------------------
    def tiles(self) -> dict:
        t = FgpuTiles()
        self._check(self.lib.fgpu_batch_get_tiles(self.h, C.byref(t)), "fgpu_batch_get_tiles")
        return t.to_dict()

    def set_tiles(self, tiles: dict):
        t = FgpuTiles.from_dict(tiles)
        self._check(self.lib.fgpu_batch_set_tiles(self.h, C.byref(t)), "fgpu_batch_set_tiles")

    def set_mode(self, persistent: bool):
        """One launch per substep (False), or the gas kick's and the closing
        substeps each as one persistent cooperative launch (True)."""
        self._check(self.lib.fgpu_batch_set_mode(self.h, 1 if persistent else 0),
                    "fgpu_batch_set_mode")

    @property
    def persistent(self) -> bool:
        m = C.c_int()
        self._check(self.lib.fgpu_batch_get_mode(self.h, C.byref(m)), "fgpu_batch_get_mode")
        return m.value == 1

    def autotune(self, reps: int = 5, cache: str | None = None, device: str = "cuda") -> dict:
        """Times candidate tile shapes of every kernel on the current state and
        keeps the fastest (the state is restored).  With ``cache``, a JSON file
        of earlier results keyed by device name and batch signature is read
        first and updated after tuning."""
        key = f"{device}|{self.signature()}"
        table = {}
        if cache and os.path.exists(cache):
            with open(cache) as f:
                table = json.load(f)
            if key in table:
                self.set_tiles(table[key])
                return table[key]
        t = FgpuTiles()
        self._check(self.lib.fgpu_batch_autotune(self.h, reps, C.byref(t)), "fgpu_batch_autotune")
        best = t.to_dict()
        if cache:
            table[key] = best
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return best

    # -- stepping ---------------------------------------------------------------
    def step(self, dts, ts):
        dt = np.ascontiguousarray(dts, dtype=np.float64)
        t = np.ascontiguousarray(ts, dtype=np.float64)
        if dt.size != self.n or t.size != self.n:
            raise ValueError("one dt and one t per disk")
        self._check(self.lib.fgpu_batch_step(self.h, dt.ctypes.data_as(C.POINTER(C.c_double)),
                                             t.ctypes.data_as(C.POINTER(C.c_double))),
                    "fgpu_batch_step")

    def set_clock(self, k, *, time, last_dt, t_end, monitor_dt, cfl_max_var, star_mass,
                  planets=(), n_monitor=0, steps=0, active=1):
        """planets: (mass, a, phase) of bodies on circular orbits."""
        c = FgpuClock()
        c.time, c.last_dt, c.t_end, c.monitor_dt = time, last_dt, t_end, monitor_dt
        c.cfl_max_var, c.star_mass = cfl_max_var, star_mass
        c.n_monitor, c.steps, c.active, c.n_planets = n_monitor, steps, active, len(planets)
        for q, (m, a, ph) in enumerate(planets):
            c.mass[q], c.a[q], c.phase[q] = m, a, ph
        self._check(self.lib.fgpu_batch_set_clock(self.h, k, C.byref(c)), "fgpu_batch_set_clock")

    def clock(self, k) -> dict:
        c = FgpuClock()
        self._check(self.lib.fgpu_batch_get_clock(self.h, k, C.byref(c)), "fgpu_batch_get_clock")
        return dict(time=c.time, last_dt=c.last_dt, t_end=c.t_end, monitor_dt=c.monitor_dt,
                    n_monitor=c.n_monitor, steps=c.steps, active=c.active)

    def run(self, max_steps: int, steps_per_graph: int = 16) -> int:
        """Advances every active disk by up to max_steps steps; returns the
        number of disks still below their end time."""
        n = C.c_int()
        self._check(self.lib.fgpu_batch_run(self.h, max_steps, steps_per_graph, C.byref(n)),
                    "fgpu_batch_run")
        return n.value


def start_disks(batch: Batch, disks, *, t_end: float, monitor_dt: float) -> None:
    """Loads every disk's initial state and starts its device clock the way
    FargoCPT starts a run (main.cpp:117, simulation.cpp:462-480): fields and
    reference fields, bodies, init_euler, then the two CFL evaluations around
    the initial boundary condition.  disks[k] is a setups-style tuple
    (params, dict, radii, fields, nbody) with nbody a CircularPlanets."""
    for k, (params, d, radii, fields, nbody) in enumerate(disks):
        e = batch.disks[k]
        for name, a in fields.items():
            e.set_field(name, a)
            e.set_field(name + "0", a)
        b0 = nbody.bodies(0.0)
        e.set_bodies(b0, *nbody.indirect(b0))
        e.init_euler(0.0)
        clock = RunClock()
        start(e, clock, d["cfl_max_var"])
        planets = [(q * nbody.mstar, a, ph) for q, a, ph in nbody.planets]
        batch.set_clock(k, time=clock.time, last_dt=clock.last_dt, t_end=t_end,
                        monitor_dt=monitor_dt, cfl_max_var=d["cfl_max_var"],
                        star_mass=nbody.mstar, planets=planets)


def orbits_to_time(n_orbits: float) -> float:
    """Code time of n orbits at r = 1 around a unit mass (G = 1)."""
    return n_orbits * 2.0 * math.pi


__all__ = ["Batch", "start_disks", "orbits_to_time", "BATCH_KERNELS"]
