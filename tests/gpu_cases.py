"""Synthetic disks for GPU-vs-oracle tests at sizes beyond the fixtures."""
import math

import numpy as np

from fargocpt_gb300.abi import BC, params_from_dict


def make_params(nrad, naz, adiabatic=False, **over):
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
        gamma=1.4, mu=2.35, aspect_ratio=0.05, flaring_index=0.25 if adiabatic else 0.0,
        viscous_alpha=1e-3, constant_viscosity=0.0, art_visc_factor=math.sqrt(2.0),
        radial_viscosity_factor=1.0, heating_viscous_factor=1.0, cfl=0.5, cfl_max_var=1.1,
        heating_cooling_cfl_limit=10.0, sigma0=1e-3, sigma_floor=1e-9,
        thickness_smoothing=0.6, cooling_beta_value=10.0, cooling_beta_ramp_up=0.0,
        minimum_temperature=2.811616511825056e-05, maximum_temperature=9.372055039416854e+294,
        G=1.0, R_gas=1.0000000000000004, sigma_sb=468.30692052083845,
        c_light=10065.167938321798,
        hydro_center_mass=1.0, damping_inner_limit=1.1, damping_outer_limit=0.9,
        damping_time_factor=1.0, damping_time_radius_outer=2.5,
        vaz_inner_keplerian_factor=1.0, vaz_outer_keplerian_factor=1.0,
        rmin=0.4, rmax=2.5, radial_spacing=1,
    )
    d.update(over)
    return params_from_dict(d), d


def initial_state(d, radii, seed=0, noise=1e-2):
    """Power-law disk with seeded noise: sigma, a near-Keplerian v_phi with a
    random perturbation, small random v_r, and (ideal EOS) the energy of the
    flared temperature profile."""
    nr, nz = d["nrad"], d["naz"]
    rng = np.random.default_rng(seed)
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    sigma = d["sigma0"] * rmed[:, None] ** -1.0 * (1 + noise * rng.uniform(-1, 1, (nr, nz)))
    vk = np.sqrt(d["G"] / rmed)
    vaz = (vk * np.sqrt(1 - d["aspect_ratio"] ** 2))[:, None] * (
        1 + 0.1 * noise * rng.uniform(-1, 1, (nr, nz)))
    vr = 1e-3 * noise * rng.uniform(-1, 1, (nr + 1, nz))
    h = d["aspect_ratio"] * rmed ** d["flaring_index"]
    cs2 = (h * vk) ** 2
    energy = sigma * cs2[:, None] / (d["gamma"] * (d["gamma"] - 1.0))
    if d["eos"] == 0:
        energy = np.zeros_like(sigma)
    return dict(SIGMA=sigma, V_RADIAL=vr, V_AZIMUTHAL=vaz, ENERGY=energy)


def load(backend, state, bodies, ix=0.0, iy=0.0):
    for f, a in state.items():
        backend.set_field(f, a)
        backend.set_field(f + "0", a)
    backend.set_bodies(bodies, ix, iy, 0.0)
    backend.init_euler(0.0)
