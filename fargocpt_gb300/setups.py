"""The benchmark configurations as synthetic FargoCPT disks.

Each builder returns the engine parameters (code units: l0 = 1 au,
m0 = 1 solar mass, G = 1, as FargoCPT sets them, src/units.cpp:172), the
interface radii, the initial fields and the N-body state.  Initial conditions
are seeded power laws shaped like FargoCPT's default profiles
(src/init.cpp:937-1148, :1257, :1467): sigma = Sigma0 r^-p (1 + 1e-3 U(-1,1)),
the locally isothermal sound speed h r^f v_K, a pressure-supported Keplerian
v_phi, v_r = 0 and, for the ideal EOS, e = sigma c_s,iso^2 / (gamma - 1).
"""
from __future__ import annotations

import math

import numpy as np

from .abi import BC, params_from_dict

# Code-unit constants for l0 = 1 au, m0 = 1 solMass, mu = 2.35, as FargoCPT
# derives them from its unit system (constants.yml of a reference run).
CODE_CONSTANTS = dict(
    G=1.0,
    R_gas=1.0000000000000004,
    sigma_sb=468.30692052083845,
    c_light=10065.167938321798,
    minimum_temperature=2.811616511825056e-05,   # 3 K
    maximum_temperature=9.372055039416854e+294,  # 1e300 K
)


def base_params(nrad, naz, rmin, rmax, *, adiabatic, alpha=1e-3, h=0.05, flaring=0.0,
                beta=10.0):
    d = dict(
        nrad=nrad, naz=naz, eos=1 if adiabatic else 0, art_visc=1, art_visc_dissipation=1,
        flux_limiter=0, fast_transport=1, heating_viscous=1,
        cooling_beta=1 if adiabatic else 0, cooling_beta_reference=0, damping=1,
        damping_inner=[1, 1, 1, 1 if adiabatic else 0],
        damping_outer=[1, 1, 1, 1 if adiabatic else 0],
        bc_sigma_inner=BC["zerogradient"], bc_sigma_outer=BC["zerogradient"],
        bc_energy_inner=BC["zerogradient"], bc_energy_outer=BC["zerogradient"],
        bc_vrad_inner=BC["outflow"], bc_vrad_outer=BC["outflow"],
        bc_vaz_inner=BC["keplerian"], bc_vaz_outer=BC["keplerian"], precision=0,
        gamma=1.4, mu=2.35, aspect_ratio=h, flaring_index=flaring, viscous_alpha=alpha,
        constant_viscosity=0.0, art_visc_factor=math.sqrt(2.0) if adiabatic else 1.41,
        radial_viscosity_factor=1.0, heating_viscous_factor=1.0, cfl=0.5, cfl_max_var=1.1,
        heating_cooling_cfl_limit=10.0, sigma0=1e-3, sigma_floor=1e-9,
        thickness_smoothing=0.6, cooling_beta_value=beta, cooling_beta_ramp_up=0.0,
        hydro_center_mass=1.0, damping_inner_limit=1.05, damping_outer_limit=0.95,
        damping_time_factor=1.0, damping_time_radius_outer=rmax,
        vaz_inner_keplerian_factor=1.0, vaz_outer_keplerian_factor=1.0,
        rmin=rmin, rmax=rmax, radial_spacing=1,
    )
    d.update(CODE_CONSTANTS)
    return d


def log_radii(nrad, rmin, rmax):
    """FargoCPT's logarithmic Radii[0 .. nrad+1] (init.cpp:93-100)."""
    q = math.pow(rmax / rmin, 1.0 / (nrad - 2.0))
    return np.array([rmin * math.pow(q, n - 1.0) for n in range(nrad + 2)])


def initial_fields(d, radii, slope, seed):
    nr, nz = d["nrad"], d["naz"]
    rng = np.random.default_rng(seed)
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    sigma = d["sigma0"] * rmed[:, None] ** -slope * (1 + 1e-3 * rng.uniform(-1, 1, (nr, nz)))
    vk = np.sqrt(d["G"] * d["hydro_center_mass"] / rmed)
    h = d["aspect_ratio"] * rmed ** d["flaring_index"]
    dlnp = -slope + 2 * d["flaring_index"] - 1.0
    vaz = np.repeat((vk * np.sqrt(1 + h * h * dlnp))[:, None], nz, axis=1)
    vr = np.zeros((nr + 1, nz))
    if d["eos"] == 1:
        energy = sigma * ((h * vk) ** 2)[:, None] / (d["gamma"] - 1.0)
    else:
        energy = np.zeros((nr, nz))
    return dict(SIGMA=sigma, V_RADIAL=vr, V_AZIMUTHAL=vaz, ENERGY=energy)


class CircularPlanets:
    """Host stand-in for the N-body integrator: planets on fixed circular
    orbits around the primary (the hydro frame's centre)."""

    def __init__(self, planets, G=1.0, mstar=1.0):
        self.planets = planets  # list of (mass_ratio, a, phase)
        self.G, self.mstar = G, mstar

    def bodies(self, t):
        out = [(0.0, 0.0, self.mstar, 0.0, 0.0)]
        for q, a, ph in self.planets:
            om = math.sqrt(self.G * (self.mstar + q * self.mstar) / a ** 3)
            out.append((a * math.cos(om * t + ph), a * math.sin(om * t + ph), q * self.mstar,
                        0.0, a))
        return out

    def indirect(self, bodies):
        # IndirectTermMode Euler with the primary as the frame centre
        ax = ay = 0.0
        for x, y, m, *_ in bodies[1:]:
            d3 = math.pow(math.sqrt(x * x + y * y), 3)
            ax -= self.G * m / d3 * (0.0 - x)
            ay -= self.G * m / d3 * (0.0 - y)
        return -ax, -ay


CONFIGS = {
    # locally isothermal 128 x 384 disk, one planet
    "c1": dict(nrad=128, naz=384, rmin=0.4, rmax=2.5, adiabatic=False, slope=0.5,
               flaring=0.0, planets=[(1e-3, 1.0, 0.0)]),
    # adiabatic 512 x 1536 disk, beta cooling, SN art. visc, one planet
    "c2": dict(nrad=512, naz=1536, rmin=0.3, rmax=3.0, adiabatic=True, slope=1.0,
               flaring=0.25, planets=[(1e-3, 1.0, 0.0)]),
    # locally isothermal 1024 x 3072 disk, one planet
    "c3": dict(nrad=1024, naz=3072, rmin=0.4, rmax=2.5, adiabatic=False, slope=0.5,
               flaring=0.0, planets=[(1e-3, 1.0, 0.0)]),
    # large adiabatic 2048 x 6144 disk with three planets
    "c5": dict(nrad=2048, naz=6144, rmin=0.3, rmax=5.0, adiabatic=True, slope=1.0,
               flaring=0.25, planets=[(1e-3, 1.0, 0.0), (3e-4, 1.6, 2.1), (1e-4, 2.5, 4.2)]),
    # the large disk's set-up with a quarter of its rings (512 x 6144): the
    # same 6144-cell rings for profiler captures that stay small (25 MB per
    # FP64 field, about 0.8 GB on the device)
    "c5s": dict(nrad=512, naz=6144, rmin=0.3, rmax=5.0, adiabatic=True, slope=1.0,
                flaring=0.25, planets=[(1e-3, 1.0, 0.0), (3e-4, 1.6, 2.1), (1e-4, 2.5, 4.2)]),
}


def build(name, seed=1234):
    c = CONFIGS[name]
    d = base_params(c["nrad"], c["naz"], c["rmin"], c["rmax"], adiabatic=c["adiabatic"],
                    flaring=c["flaring"])
    radii = log_radii(c["nrad"], c["rmin"], c["rmax"])
    fields = initial_fields(d, radii, c["slope"], seed)
    nbody = CircularPlanets(c["planets"])
    return params_from_dict(d), d, radii, fields, nbody


# Sweep of independent locally isothermal disks: each draws its grid and
# physics from the seed; the radial range and the rest of the set-up are the
# 128 x 384 single-planet disk's.
SWEEP_NR = (128, 192, 256, 384, 512)


def sweep(n_disks=64, seed=4, nr_choices=SWEEP_NR, precision=1):
    """n_disks setups-style tuples (params, dict, radii, fields, nbody):
    Nr uniform in nr_choices with Naz = 3 Nr, alpha log-uniform in
    [1e-4, 1e-2], planet mass ratio log-uniform in [1e-5, 3e-3] at r = 1,
    aspect ratio uniform in [0.03, 0.07], sigma slope uniform in [0.5, 1.5]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_disks):
        nr = int(rng.choice(nr_choices))
        alpha = 10.0 ** rng.uniform(-4.0, -2.0)
        q = 10.0 ** rng.uniform(math.log10(1e-5), math.log10(3e-3))
        h = rng.uniform(0.03, 0.07)
        slope = rng.uniform(0.5, 1.5)
        d = base_params(nr, 3 * nr, 0.4, 2.5, adiabatic=False, alpha=alpha, h=h)
        d["precision"] = precision
        radii = log_radii(nr, 0.4, 2.5)
        fields = initial_fields(d, radii, slope, seed * 1000 + k)
        out.append((params_from_dict(d), d, radii, fields, CircularPlanets([(q, 1.0, 0.0)])))
    return out
