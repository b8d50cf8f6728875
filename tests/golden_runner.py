"""Replays a golden case (tests/golden/<case>.npz, produced by running the
FargoCPT reference) through any hydro backend with the reference's run loop.

The backend is either the GPU engine (fargocpt_gb300.engine.Engine) or the
oracle (oracle.oracle_py.OracleState); both expose the same methods.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from fargocpt_gb300.abi import FgpuAccretor, params_from_dict
from fargocpt_gb300.simulation import (RunClock, advance, center_of_mass, com_boundary_setup,
                                       indirect_term_euler, l1_point, orbital_period, start)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["iso_planet_fixed_dt", "adi_planet_fixed_dt", "iso_star_cfl",
         "adi_star_cfl_mc_std", "iso_star_cfl_leapfrog", "adi_star_cfl_leapfrog",
         "adi_planet_tw", "adi_star_cfl_tw_stab1", "iso_star_cfl_tw_stab2",
         "iso_planet_accretion_kley", "adi_planet_accretion_sinkhole",
         "iso_planet_accretion_viscous", "iso_planet_bc_individual",
         "adi_star_cfl_bc_individual", "iso_planet_bc_com", "adi_star_cfl_bc_com_keplerian",
         "adi_planet_bc_com", "iso_planet_corotating", "adi_planet_keep_mass_nocorr",
         "c1_cfl_100"]
EVOLVED = ["SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY"]


def load_case(name):
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    return meta, arrays


def bodies_at(arrays, nb, row):
    out = []
    for k in range(nb):
        x = float(arrays[f"body{k}_x"][row])
        y = float(arrays[f"body{k}_y"][row])
        m = float(arrays[f"body{k}_mass"][row])
        out.append((x, y, m, 0.0, math.sqrt(x * x + y * y)))
    return out


def circular_bodies_at(arrays, nb, G, t):
    """The bodies at time t when every planet k >= 1 keeps the circular
    orbit of its initial monitor row about the star at the origin."""
    m0 = float(arrays["body0_mass"][0])
    out = [(0.0, 0.0, m0, 0.0, 0.0)]
    for k in range(1, nb):
        x0, y0 = float(arrays[f"body{k}_x"][0]), float(arrays[f"body{k}_y"][0])
        m = float(arrays[f"body{k}_mass"][0])
        a = math.hypot(x0, y0)
        om = math.sqrt(G * (m0 + m) / a ** 3)
        ph = math.atan2(y0, x0) + om * t
        x, y = a * math.cos(ph), a * math.sin(ph)
        out.append((x, y, m, 0.0, math.sqrt(x * x + y * y)))
    return out


def moving_bodies_at(arrays, nb, row):
    """(x, y, vx, vy, mass) of every body at monitor row `row`."""
    return [tuple(float(arrays[f"body{k}_{q}"][row]) for q in ("x", "y", "vx", "vy", "mass"))
            for k in range(nb)]


def frame_centers_at(arrays, nb, row, dt):
    """The centres the two boundary calls of the step after monitor row `row`
    read: before transport, the bodies of the row after
    apply_indirect_term_on_Nbody (planetary_system.cpp:730-744,
    simulation.cpp:165-166); after the N-body step, the next row."""
    mb = moving_bodies_at(arrays, nb, row)
    if nb > 1:
        ix, iy = indirect_term_euler(bodies_at(arrays, nb, row))
    else:
        ix, iy = 0.0, 0.0
    kicked = [(x, y, vx + dt * ix, vy + dt * iy, m) for (x, y, vx, vy, m) in mb]
    nxt = moving_bodies_at(arrays, nb, min(row + 1, len(arrays["body0_x"]) - 1))
    return ([center_of_mass(kicked, 1), center_of_mass(kicked, nb)],
            [center_of_mass(nxt, 1), center_of_mass(nxt, nb)])


def accretor_at(arrays, meta, row):
    """The planet (body 1) as AccreteOntoPlanets sees it at the start of the
    step after monitor row `row`: position, Roche radius (init_l1 times the
    distance to the star, planetary_system.cpp:940-1004) and orbital period
    (calculate_orbital_elements about the star, planetary_system.cpp:773-793)."""
    b = {k: float(arrays[f"body1_{k}"][row]) for k in ("x", "y", "vx", "vy", "mass")}
    s = {k: float(arrays[f"body0_{k}"][row]) for k in ("x", "y", "vx", "vy", "mass")}
    G = float(meta["params"]["G"])
    # get_center_of_mass(1) / get_center_of_mass_velocity(1) of the star alone
    cx, cy = (0.0 + s["x"] * s["mass"]) / s["mass"], (0.0 + s["y"] * s["mass"]) / s["mass"]
    cvx = (0.0 + s["vx"] * s["mass"]) / s["mass"]
    cvy = (0.0 + s["vy"] * s["mass"]) / s["mass"]
    period = orbital_period(b["x"] - cx, b["y"] - cy, b["vx"] - cvx, b["vy"] - cvy,
                            0.0 + s["mass"], b["mass"], G)
    dist = math.sqrt(math.pow(b["x"] - s["x"], 2) + math.pow(b["y"] - s["y"], 2))
    acc = meta["accretion"]
    return FgpuAccretor(type=int(acc["type"]), x=b["x"], y=b["y"],
                        r=math.hypot(b["x"], b["y"]), phi=math.atan2(b["y"], b["x"]),
                        roche_radius=l1_point(s["mass"], b["mass"]) * dist,
                        efficiency=float(acc["efficiency"]), orbital_period=period)


def replay(make_backend, name, params_override=None, accreted=None, quantities=None,
           on_snapshot=None):
    """Runs the case; returns (snapshots, times, torques, dts).  With
    accreted (a dict), the mass each monitor interval accreted is added to
    accreted[monitor]; with quantities (a dict), the gas mass and angular
    momentum within the case's quantities radius at each monitor are stored
    in quantities[monitor]; on_snapshot(backend, n, clock) is called at every
    kept snapshot n (the run clock holds sim::time, last_dt, N_hydro_iter)."""
    meta, arrays = load_case(name)
    pd = dict(meta["params"])
    if params_override:
        pd.update(params_override)
    params = params_from_dict(pd)
    hyd = make_backend(params, arrays["radii"])
    nb = meta["nbodies"]

    def body_state(row):
        b = bodies_at(arrays, nb, row)
        if nb > 1:
            ix, iy = indirect_term_euler(b)
        else:
            ix, iy = 0.0, 0.0
        return b, ix, iy

    for f in EVOLVED:
        hyd.set_field(f, arrays[f"s0_{f}"])
        hyd.set_field(f + "0", arrays[f"s0_{f}"])
    # corotating frame: OmegaFrame of the monitor rows (the value the step
    # that ends at a row used), v_phi corrected by its changes
    corot = bool(meta.get("corotating"))
    omega = arrays["body0_omega_frame"] if corot else None
    b, ix, iy = body_state(0)
    hyd.set_bodies(b, ix, iy, float(omega[0]) if corot else 0.0)
    # init_euler runs before the velocities are initialised in FargoCPT
    # (init.cpp:326-332): the heating/cooling rates the first CFL reads are
    # computed with v = 0.
    zr = np.zeros_like(arrays["s0_V_RADIAL"])
    za = np.zeros_like(arrays["s0_V_AZIMUTHAL"])
    hyd.set_field("V_RADIAL", zr)
    hyd.set_field("V_AZIMUTHAL", za)
    hyd.init_euler(0.0)
    hyd.set_field("V_RADIAL", arrays["s0_V_RADIAL"])
    hyd.set_field("V_AZIMUTHAL", arrays["s0_V_AZIMUTHAL"])

    frame_centers = None
    if int(pd.get("composite_inner", 0)) == 1 or int(pd.get("composite_outer", 0)) == 1:
        mb = moving_bodies_at(arrays, nb, 0)
        hyd.init_center_of_mass_boundary(*com_boundary_setup(mb, float(pd["G"])))
        c0 = [center_of_mass(mb, 1), center_of_mass(mb, nb)]
        hyd.set_frame_centers(c0)

        def frame_centers(c, dt):
            return frame_centers_at(arrays, nb, c.n_monitor, dt)

    clock = RunClock(time=0.0, last_dt=meta["first_dt"])
    cmv = float(pd["cfl_max_var"])
    start(hyd, clock, cmv,
          keep_mass_rmax=float(pd["rmax"]) if int(pd.get("keep_disk_mass_constant", 0)) else None)
    qradius = meta.get("quantities_radius")

    def record_quantities(n):
        if quantities is not None and qradius is not None:
            quantities[n] = (hyd.gas_total_mass(qradius), hyd.gas_angular_momentum(qradius))

    record_quantities(0)
    keep = set(int(k) for k in arrays["keep"])
    snaps, times, torques = {}, {}, {}

    def on_monitor(c):
        times[c.n_monitor] = c.time
        if nb > 1:
            bb, jx, jy = body_state(c.n_monitor)
            hyd.set_bodies(bb, jx, jy, 0.0)
            ax, ay = hyd.disk_on_planet_accel(1)
            x, y, m = bb[1][0], bb[1][1], bb[1][2]
            torques[c.n_monitor] = (x * ay - y * ax) * m
        if c.n_monitor in keep:
            snaps[c.n_monitor] = {f: hyd.get_field(f) for f in EVOLVED}
            if on_snapshot is not None:
                on_snapshot(hyd, c.n_monitor, c)
        record_quantities(c.n_monitor)

    accrete = None
    if "accretion" in meta:
        def accrete(c, dt):
            dm, _, _ = hyd.accrete_onto_planet(accretor_at(arrays, meta, c.n_monitor), dt)
            if accreted is not None:
                accreted[c.n_monitor + 1] = accreted.get(c.n_monitor + 1, 0.0) + dm

    def step_bodies(c):
        if meta.get("circular_bodies"):
            # the planet between monitor outputs: its circular orbit about the
            # star (REBOUND's two-body orbit agrees with it to ~1e-14 at the
            # monitor rows the reference wrote)
            b = circular_bodies_at(arrays, nb, float(pd["G"]), c.time)
            return (b, *indirect_term_euler(b))
        b, ix, iy = body_state(c.n_monitor)
        return (b, ix, iy, float(omega[c.n_monitor + 1])) if corot else (b, ix, iy)

    corotation = None
    if corot:
        def corotation(c):
            return float(omega[c.n_monitor + 1]) - float(omega[c.n_monitor])

    t_final = meta["nsnapshots"] * 1 * meta["monitor_timestep"]
    advance(hyd, clock, cfl_max_var=cmv, monitor_timestep=meta["monitor_timestep"],
            t_final=t_final, bodies=step_bodies, corotation=corotation,
            on_monitor=on_monitor,
            integrator="leapfrog" if int(pd.get("integrator", 0)) == 1 else "euler",
            accrete=accrete, frame_centers=frame_centers)
    return snaps, times, torques, clock.dts, arrays


def rel_linf(a, b, floor=0.0):
    """max |a - b| / max |b| (relative L-infinity of the field)."""
    scale = max(float(np.max(np.abs(b))), floor)
    if scale == 0.0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b))) / scale
