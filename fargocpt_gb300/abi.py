"""ctypes mirror of include/fargocpt_gb300.h and the loader of the engine.

The engine is the in-tree shared library ``fargocpt_gb300/libfargocpt_gb300.so``
built by :mod:`fargocpt_gb300.build`.  Loading fails loudly when it is missing:
there is no CPU fallback on the product path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfargocpt_gb300.so")

# fgpu_status
FGPU_OK = 0
STATUS_NAMES = {
    0: "FGPU_OK",
    -1: "FGPU_ERR_BAD_ARG",
    -2: "FGPU_ERR_OOM",
    -3: "FGPU_ERR_CUDA",
    -4: "FGPU_ERR_UNSUPPORTED",
    -5: "FGPU_ERR_NONFINITE",
    -6: "FGPU_ERR_NO_DEVICE",
}

# fgpu_field
FIELDS = {
    "SIGMA": 0, "V_RADIAL": 1, "V_AZIMUTHAL": 2, "ENERGY": 3,
    "SIGMA0": 4, "V_RADIAL0": 5, "V_AZIMUTHAL0": 6, "ENERGY0": 7,
    "SOUNDSPEED": 8, "SCALE_HEIGHT": 9, "PRESSURE": 10, "TEMPERATURE": 11,
    "VISCOSITY": 12, "QPLUS": 13, "QMINUS": 14, "POTENTIAL": 15,
    "DIV_V": 16, "TAU_R_R": 17, "TAU_PHI_PHI": 18, "TAU_R_PHI": 19,
    "Q_R": 20, "Q_PHI": 21,
}
VECTOR_FIELDS = {"V_RADIAL", "V_RADIAL0", "TAU_R_PHI"}

BC = {"none": 0, "zerogradient": 1, "outflow": 2, "reference": 3, "keplerian": 4,
      "diskmodel": 5, "reflecting": 6, "viscous": 7, "keplerian_radial": 8, "zeroshear": 9,
      "balanced": 10}
DAMP = {"none": 0, "reference": 1, "zero": 2, "mean": 3}
EOS_ISOTHERMAL, EOS_IDEAL = 0, 1
SPACING_ARITHMETIC, SPACING_LOGARITHMIC = 0, 1
ARTVISC_NONE, ARTVISC_SN, ARTVISC_TW = 0, 1, 2
LIMITER_VANLEER, LIMITER_MC = 0, 1
BETA_REF = {"zero": 0, "reference": 1, "diskmodel": 2, "floor": 3}
PRECISION_FP64, PRECISION_FP32_MIXED = 0, 1


class FgpuParams(C.Structure):
    _fields_ = [
        ("nrad", C.c_int), ("naz", C.c_int), ("eos", C.c_int),
        ("art_visc", C.c_int), ("art_visc_dissipation", C.c_int),
        ("flux_limiter", C.c_int), ("fast_transport", C.c_int),
        ("heating_viscous", C.c_int), ("cooling_beta", C.c_int),
        ("cooling_beta_reference", C.c_int), ("damping", C.c_int),
        ("damping_inner", C.c_int * 4), ("damping_outer", C.c_int * 4),
        ("bc_sigma_inner", C.c_int), ("bc_sigma_outer", C.c_int),
        ("bc_energy_inner", C.c_int), ("bc_energy_outer", C.c_int),
        ("bc_vrad_inner", C.c_int), ("bc_vrad_outer", C.c_int),
        ("bc_vaz_inner", C.c_int), ("bc_vaz_outer", C.c_int),
        ("precision", C.c_int), ("integrator", C.c_int),
        ("stabilize_viscosity", C.c_int), ("profile_cutoff_outer", C.c_int),
        ("viscous_accretion", C.c_int), ("composite_inner", C.c_int),
        ("composite_outer", C.c_int), ("initialize_pure_keplerian", C.c_int),
        ("initialize_vradial_zero", C.c_int), ("profile_cutoff_inner", C.c_int),
        ("keep_disk_mass_constant", C.c_int),
        ("gamma", C.c_double), ("mu", C.c_double), ("aspect_ratio", C.c_double),
        ("flaring_index", C.c_double), ("viscous_alpha", C.c_double),
        ("constant_viscosity", C.c_double), ("art_visc_factor", C.c_double),
        ("radial_viscosity_factor", C.c_double),
        ("heating_viscous_factor", C.c_double), ("cfl", C.c_double),
        ("cfl_max_var", C.c_double), ("heating_cooling_cfl_limit", C.c_double),
        ("sigma0", C.c_double), ("sigma_floor", C.c_double),
        ("thickness_smoothing", C.c_double), ("cooling_beta_value", C.c_double),
        ("cooling_beta_ramp_up", C.c_double),
        ("minimum_temperature", C.c_double), ("maximum_temperature", C.c_double),
        ("G", C.c_double), ("R_gas", C.c_double), ("sigma_sb", C.c_double),
        ("c_light", C.c_double), ("hydro_center_mass", C.c_double),
        ("damping_inner_limit", C.c_double), ("damping_outer_limit", C.c_double),
        ("damping_time_factor", C.c_double),
        ("damping_time_radius_outer", C.c_double),
        ("vaz_inner_keplerian_factor", C.c_double),
        ("vaz_outer_keplerian_factor", C.c_double),
        ("rmin", C.c_double), ("rmax", C.c_double),
        ("radial_spacing", C.c_int), ("correct_disk_selfgravity", C.c_int),
        ("accretion_radius_fraction", C.c_double), ("sigma_slope", C.c_double),
        ("viscous_outflow_speed", C.c_double), ("vrad_inner_keplerian_factor", C.c_double),
        ("vrad_outer_keplerian_factor", C.c_double), ("binary_quadrupole_moment", C.c_double),
        ("profile_cutoff_point_outer", C.c_double), ("profile_cutoff_width_outer", C.c_double),
        ("profile_cutoff_point_inner", C.c_double), ("profile_cutoff_width_inner", C.c_double),
        ("temperature_cgs_to_code", C.c_double),
        ("reserved_d", C.c_double * 2),
    ]


class FgpuBody(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("mass", C.c_double),
                ("r_sm", C.c_double), ("a", C.c_double)]


ACCRETION = {"kley": 0, "viscous": 1, "sinkhole": 2}
COMPOSITE = {"individual": 0, "centerofmass": 1}


class FgpuCflCell(C.Structure):
    """fgpu_cfl_cell: the cell that limits the CFL step (cfl.cpp:38-182)."""
    _fields_ = [("ring", C.c_int), ("azimuth", C.c_int), ("shear_ring", C.c_int),
                ("reserved", C.c_int), ("dt_cell", C.c_double), ("invdt", C.c_double * 6),
                ("dt_shear", C.c_double)]


class FgpuFrameCenter(C.Structure):
    """fgpu_frame_center: centre of mass, its velocity and the mass of a set
    of bodies (nbody/planetary_system.cpp:580-650)."""
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("vx", C.c_double),
                ("vy", C.c_double), ("mass", C.c_double)]


class FgpuAccretor(C.Structure):
    """fgpu_accretor: one accreting planet (accretion.cpp:84-480)."""
    _fields_ = [("type", C.c_int), ("reserved", C.c_int), ("x", C.c_double),
                ("y", C.c_double), ("r", C.c_double), ("phi", C.c_double),
                ("roche_radius", C.c_double), ("efficiency", C.c_double),
                ("orbital_period", C.c_double)]


# FargoCPT's defaults for keys a parameter dict may leave out
# (CorrectDiskSelfgravity defaults to yes without self-gravity, parameters.cpp:699)
PARAM_DEFAULTS = {"correct_disk_selfgravity": 1}


def params_from_dict(d: dict) -> FgpuParams:
    """Fills an FgpuParams from a flat dict of field name -> value; keys the
    dict leaves out are zero, except those of PARAM_DEFAULTS."""
    p = FgpuParams()
    d = {**PARAM_DEFAULTS, **d}
    for name, _ in FgpuParams._fields_:
        if name in d:
            v = d[name]
            if name in ("damping_inner", "damping_outer"):
                arr = getattr(p, name)
                for i in range(4):
                    arr[i] = int(v[i])
            else:
                setattr(p, name, v)
    return p


def params_to_dict(p: FgpuParams) -> dict:
    out = {}
    for name, _ in FgpuParams._fields_:
        if name.startswith("reserved"):
            continue
        v = getattr(p, name)
        if name in ("damping_inner", "damping_outer"):
            v = [int(x) for x in v]
        out[name] = v
    return out


BATCH_KERNELS = ["potential", "source", "artvisc_q", "artvisc_v", "stress", "viscous",
                 "ghost", "transport_radial", "transport_azimuthal", "finish", "damping",
                 "derived_cfl"]


class FgpuTile(C.Structure):
    _fields_ = [("threads", C.c_int), ("rings", C.c_int)]


class FgpuTiles(C.Structure):
    _fields_ = [("k", FgpuTile * len(BATCH_KERNELS))]

    def to_dict(self) -> dict:
        return {n: [self.k[i].threads, self.k[i].rings] for i, n in enumerate(BATCH_KERNELS)}

    @classmethod
    def from_dict(cls, d: dict) -> "FgpuTiles":
        t = cls()
        for i, n in enumerate(BATCH_KERNELS):
            t.k[i].threads, t.k[i].rings = int(d[n][0]), int(d[n][1])
        return t


class FgpuClock(C.Structure):
    _fields_ = [("time", C.c_double), ("last_dt", C.c_double), ("t_end", C.c_double),
                ("monitor_dt", C.c_double), ("cfl_max_var", C.c_double),
                ("star_mass", C.c_double), ("n_monitor", C.c_int), ("steps", C.c_int),
                ("active", C.c_int), ("n_planets", C.c_int), ("mass", C.c_double * 16),
                ("a", C.c_double * 16), ("phase", C.c_double * 16)]


EXPORTED_SYMBOLS = [
    "fgpu_grid_radii", "fgpu_create", "fgpu_destroy", "fgpu_last_error",
    "fgpu_get_stream", "fgpu_upload_field", "fgpu_download_field",
    "fgpu_set_bodies", "fgpu_init_euler", "fgpu_recalculate_derived",
    "fgpu_condition_cfl", "fgpu_apply_boundary_condition", "fgpu_step_euler",
    "fgpu_disk_on_planet_accel", "fgpu_disk_on_nbody_accel", "fgpu_total_mass",
    "fgpu_gas_total_mass",
    "fgpu_gas_angular_momentum", "fgpu_set_disk_mass_target", "fgpu_accrete_onto_planet",
    "fgpu_check_finite", "fgpu_init_center_of_mass_boundary", "fgpu_set_frame_centers",
    "fgpu_correct_v_azimuthal", "fgpu_cfl_limiting_cell",
    "fgpu_synchronize", "fgpu_set_phase_timing", "fgpu_phase_times", "fgpu_phase_name",
    "fgpu_disk_force_static", "fgpu_gas_kick", "fgpu_transport", "fgpu_compute_pressure",
    "fgpu_snapshot_begin", "fgpu_snapshot_wait", "fgpu_host_alloc", "fgpu_host_free",
    "fgpu_batch_create", "fgpu_batch_destroy", "fgpu_batch_last_error", "fgpu_batch_size",
    "fgpu_batch_disk", "fgpu_batch_get_tiles", "fgpu_batch_set_tiles", "fgpu_batch_autotune",
    "fgpu_batch_step", "fgpu_batch_set_clock", "fgpu_batch_get_clock", "fgpu_batch_run",
    "fgpu_batch_set_mode", "fgpu_batch_get_mode",
]


# fgpu_batch_set_mode: one launch per substep, or the persistent sequences
BATCH_LAUNCHES, BATCH_PERSISTENT = 0, 1


def _declare(lib: C.CDLL) -> C.CDLL:
    P = C.POINTER
    dp = P(C.c_double)
    vp = C.c_void_p
    sig = {
        "fgpu_grid_radii": ([C.c_int, C.c_double, C.c_double, C.c_int, dp], C.c_int),
        "fgpu_create": ([P(FgpuParams), dp, P(vp)], C.c_int),
        "fgpu_destroy": ([vp], C.c_int),
        "fgpu_last_error": ([vp], C.c_char_p),
        "fgpu_get_stream": ([vp, P(vp)], C.c_int),
        "fgpu_upload_field": ([vp, C.c_int, dp, C.c_int, C.c_int], C.c_int),
        "fgpu_download_field": ([vp, C.c_int, dp, C.c_int, C.c_int], C.c_int),
        "fgpu_set_bodies": ([vp, C.c_int, P(FgpuBody), C.c_double, C.c_double,
                             C.c_double], C.c_int),
        "fgpu_init_euler": ([vp, C.c_double], C.c_int),
        "fgpu_recalculate_derived": ([vp, C.c_double], C.c_int),
        "fgpu_condition_cfl": ([vp, dp], C.c_int),
        "fgpu_apply_boundary_condition": ([vp, C.c_double, C.c_double, C.c_int], C.c_int),
        "fgpu_step_euler": ([vp, C.c_double, C.c_double], C.c_int),
        "fgpu_disk_on_planet_accel": ([vp, C.c_int, dp], C.c_int),
        "fgpu_disk_on_nbody_accel": ([vp, dp], C.c_int),
        "fgpu_total_mass": ([vp, dp], C.c_int),
        "fgpu_gas_total_mass": ([vp, C.c_double, dp], C.c_int),
        "fgpu_gas_angular_momentum": ([vp, C.c_double, dp], C.c_int),
        "fgpu_set_disk_mass_target": ([vp, C.c_double], C.c_int),
        "fgpu_accrete_onto_planet": ([vp, C.POINTER(FgpuAccretor), C.c_double, dp], C.c_int),
        "fgpu_check_finite": ([vp, P(C.c_int), P(C.c_int), P(C.c_int)], C.c_int),
        "fgpu_init_center_of_mass_boundary": ([vp, C.c_double, C.c_double, C.c_int,
                                               C.c_double], C.c_int),
        "fgpu_set_frame_centers": ([vp, P(FgpuFrameCenter), P(FgpuFrameCenter)], C.c_int),
        "fgpu_correct_v_azimuthal": ([vp, C.c_double], C.c_int),
        "fgpu_cfl_limiting_cell": ([vp, P(FgpuCflCell)], C.c_int),
        "fgpu_synchronize": ([vp], C.c_int),
        "fgpu_set_phase_timing": ([vp, C.c_int], C.c_int),
        "fgpu_phase_times": ([vp, dp, C.c_int, P(C.c_int), P(C.c_int)], C.c_int),
        "fgpu_phase_name": ([C.c_int], C.c_char_p),
        "fgpu_disk_force_static": ([vp, vp, vp, C.c_int, C.c_int, C.c_double, C.c_double,
                                    P(FgpuBody), vp, vp], C.c_int),
        "fgpu_snapshot_begin": ([vp, C.c_int, P(C.c_int), P(dp)], C.c_int),
        "fgpu_snapshot_wait": ([vp], C.c_int),
        "fgpu_host_alloc": ([C.c_size_t, P(vp)], C.c_int),
        "fgpu_host_free": ([vp], C.c_int),
        "fgpu_gas_kick": ([vp, C.c_double, C.c_double], C.c_int),
        "fgpu_transport": ([vp, C.c_double], C.c_int),
        "fgpu_compute_pressure": ([vp], C.c_int),
        "fgpu_batch_create": ([C.c_int, P(FgpuParams), P(dp), P(vp)], C.c_int),
        "fgpu_batch_destroy": ([vp], C.c_int),
        "fgpu_batch_last_error": ([vp], C.c_char_p),
        "fgpu_batch_size": ([vp, P(C.c_int)], C.c_int),
        "fgpu_batch_disk": ([vp, C.c_int, P(vp)], C.c_int),
        "fgpu_batch_get_tiles": ([vp, P(FgpuTiles)], C.c_int),
        "fgpu_batch_set_tiles": ([vp, P(FgpuTiles)], C.c_int),
        "fgpu_batch_autotune": ([vp, C.c_int, P(FgpuTiles)], C.c_int),
        "fgpu_batch_step": ([vp, dp, dp], C.c_int),
        "fgpu_batch_set_clock": ([vp, C.c_int, P(FgpuClock)], C.c_int),
        "fgpu_batch_get_clock": ([vp, C.c_int, P(FgpuClock)], C.c_int),
        "fgpu_batch_run": ([vp, C.c_int, C.c_int, P(C.c_int)], C.c_int),
        "fgpu_batch_set_mode": ([vp, C.c_int], C.c_int),
        "fgpu_batch_get_mode": ([vp, P(C.c_int)], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


_LIB = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads the engine library; raises if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"fargocpt_gb300: engine library {p} is missing; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = _declare(C.CDLL(p))
    if path is None:
        _LIB = lib
    return lib
