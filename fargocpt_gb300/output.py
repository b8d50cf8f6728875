"""FargoCPT snapshot files written from the engine without stopping the run.

FargoCPT writes a snapshot as one raw file per grid, ``<name>.dat`` (every row
of the grid, row-major little-endian FP64: t_polargrid::write2D,
src/polargrid.cpp:135-180, names from src/data.cpp:13-254) and ``misc.bin``
(struct misc_entry, src/output.h:16-24, written by write_misc,
src/output.cpp:494-525).  :class:`Snapshotter` stages the fields on the
device and copies them to page-locked host buffers on a second stream
(fgpu_snapshot_begin), so the next steps run while the copy drains; the files
are written once the copy is done.
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

from .abi import FIELDS, STATUS_NAMES, VECTOR_FIELDS, load_library

# t_data polar-grid names (src/data.cpp:13-254)
GRID_NAMES = {
    "SIGMA": "Sigma", "V_RADIAL": "vrad", "V_AZIMUTHAL": "vazi", "ENERGY": "energy",
    "SIGMA0": "dens0", "V_RADIAL0": "vrad0", "V_AZIMUTHAL0": "vazi0", "ENERGY0": "energy0",
    "TEMPERATURE": "Temperature", "PRESSURE": "pressure", "SOUNDSPEED": "soundspeed",
    "SCALE_HEIGHT": "scale_height", "VISCOSITY": "viscosity", "QPLUS": "Qplus",
    "QMINUS": "Qminus", "POTENTIAL": "potential", "DIV_V": "div_v", "TAU_R_R": "tau_r_r",
    "TAU_PHI_PHI": "tau_phi_phi", "TAU_R_PHI": "tau_r_phi", "Q_R": "q_r", "Q_PHI": "q_phi",
}

# struct misc_entry: unsigned timestep, unsigned nTimeStep, double time,
# double OmegaFrame, double FrameAngle, double last_dt, unsigned long N_iter
MISC_FORMAT = "<IIddddQ"


def write_grid(path: str, array: np.ndarray) -> None:
    np.ascontiguousarray(array, dtype="<f8").tofile(path)


def read_grid(path: str, naz: int) -> np.ndarray:
    return np.fromfile(path, dtype="<f8").reshape(-1, naz)


def write_misc(path: str, *, snapshot: int, monitor: int, time: float, last_dt: float,
               n_iter: int, omega_frame: float = 0.0, frame_angle: float = 0.0) -> None:
    with open(path, "wb") as f:
        f.write(struct.pack(MISC_FORMAT, snapshot, monitor, time, omega_frame, frame_angle,
                            last_dt, n_iter))


def read_misc(path: str) -> dict:
    with open(path, "rb") as f:
        v = struct.unpack(MISC_FORMAT, f.read(struct.calcsize(MISC_FORMAT)))
    keys = ("snapshot", "monitor", "time", "omega_frame", "frame_angle", "last_dt", "n_iter")
    return dict(zip(keys, v))


class Snapshotter:
    """Asynchronous snapshots of one engine into page-locked host buffers."""

    def __init__(self, engine, fields=("SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY")):
        self.lib = load_library()
        self.engine = engine
        self.fields = list(fields)
        self._ptrs, self.arrays = [], {}
        for name in self.fields:
            rows = engine.nr + 1 if name in VECTOR_FIELDS else engine.nr
            n = rows * engine.nz
            p = C.c_void_p()
            rc = self.lib.fgpu_host_alloc(n * 8, C.byref(p))
            if rc != 0:
                self.close()
                raise MemoryError(f"fgpu_host_alloc: {STATUS_NAMES.get(rc, rc)}")
            self._ptrs.append(p.value)
            buf = (C.c_double * n).from_address(p.value)
            self.arrays[name] = np.ctypeslib.as_array(buf).reshape(rows, engine.nz)
        self._ids = (C.c_int * len(self.fields))(*[FIELDS[f] for f in self.fields])
        self._hosts = (C.POINTER(C.c_double) * len(self.fields))(
            *[C.cast(C.c_void_p(p), C.POINTER(C.c_double)) for p in self._ptrs])

    def begin(self) -> None:
        """Stages the fields as they are after the work queued so far."""
        self.engine._check(self.lib.fgpu_snapshot_begin(self.engine.h, len(self.fields),
                                                        self._ids, self._hosts),
                           "fgpu_snapshot_begin")

    def wait(self) -> dict:
        self.engine._check(self.lib.fgpu_snapshot_wait(self.engine.h), "fgpu_snapshot_wait")
        return self.arrays

    def write(self, snapshot_dir: str, **misc) -> None:
        """Waits for the copy and writes <name>.dat for every field and, with
        misc given (snapshot, monitor, time, last_dt, n_iter), misc.bin."""
        self.wait()
        os.makedirs(snapshot_dir, exist_ok=True)
        for name, a in self.arrays.items():
            write_grid(os.path.join(snapshot_dir, GRID_NAMES[name] + ".dat"), a)
        if misc:
            write_misc(os.path.join(snapshot_dir, "misc.bin"), **misc)

    def close(self) -> None:
        if getattr(self, "engine", None) is not None and getattr(self.engine, "h", None):
            self.lib.fgpu_snapshot_wait(self.engine.h)
        for p in getattr(self, "_ptrs", []):
            self.lib.fgpu_host_free(C.c_void_p(p))
        self._ptrs, self.arrays = [], {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
