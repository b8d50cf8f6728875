"""Host-side mirror of FargoCPT's run loop (reference src/simulation.cpp).

FargoCPT's C++ driver owns the run; this module restates the part of it that
decides *when* the hydro step is called and with which dt, so that the engine
can be driven exactly like ``sim::run`` drives ``step_Euler``:

* ``CalculateTimeStep`` (simulation.cpp:100-118): dt = min(CFLmaxVar * last_dt,
  CFL dt);
* the clamp of the step to the next monitor time (simulation.cpp:526-540);
* the monitor bookkeeping (simulation.cpp:544-550);
* the gas part of step_LeapFrog (simulation.cpp:276-459) from the phase
  functions (``gas_kick``, ``transport``, ``compute_pressure``).

Any object with the hydro-step methods (``condition_cfl``, ``step_euler``,
``apply_boundary_condition``, ``set_bodies``, and for LeapFrog the phase
functions and ``recalculate_derived``) can be driven; the product uses
:class:`fargocpt_gb300.engine.Engine`.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field


@dataclass
class RunClock:
    """sim::time, sim::last_dt, N_monitor, N_hydro_iter (simulation.cpp:26-31)."""

    time: float = 0.0
    last_dt: float = 1e-9   # FirstDT default, Interpret.cpp:86
    n_monitor: int = 0
    n_hydro_iter: int = 0
    dts: list = field(default_factory=list)


def calculate_time_step(hydro, clock: RunClock, cfl_max_var: float) -> float:
    """sim::CalculateTimeStep, simulation.cpp:100-118."""
    cfl_dt = hydro.condition_cfl()
    rv = min(cfl_max_var * clock.last_dt, cfl_dt)
    clock.last_dt = rv
    return rv


def start(hydro, clock: RunClock, cfl_max_var: float, keep_mass_rmax=None) -> None:
    """The calls main() and sim::init() make before the loop
    (main.cpp:117, simulation.cpp:462-480): one CFL evaluation, the initial
    boundary condition, a second CFL evaluation and, with
    KeepDiskMassConstant (keep_mass_rmax = RMAX), the gas mass within RMAX as
    the target of the rescale (total_disk_mass_old)."""
    calculate_time_step(hydro, clock, cfl_max_var)
    hydro.apply_boundary_condition(clock.time, 0.0, False)
    calculate_time_step(hydro, clock, cfl_max_var)
    if keep_mass_rmax is not None:
        hydro.set_disk_mass_target(hydro.gas_total_mass(keep_mass_rmax))


def step_leapfrog(hydro, dt: float, t: float, first, second) -> None:
    """The gas part of step_LeapFrog (simulation.cpp:276-459): kick dt/2, the
    boundary condition, transport over dt, the pressure of the transported
    state, kick dt/2, then the final boundary condition (damping) and the
    derived quantities.  first and second are (bodies, indirect_x,
    indirect_y) for the two kicks: the host has drifted the bodies to the half
    step before the first kick and recomputed the indirect term before the
    second (:285-302, :338-342)."""
    half = dt / 2
    mid = t + half
    hydro.set_bodies(first[0], first[1], first[2], 0.0)
    hydro.gas_kick(half, t)
    hydro.apply_boundary_condition(t, 0.0, False)
    hydro.transport(dt)
    hydro.set_bodies(second[0], second[1], second[2], 0.0)
    hydro.compute_pressure()
    hydro.gas_kick(half, mid)
    hydro.apply_boundary_condition(t + dt, dt, True)
    hydro.recalculate_derived(t + dt)


def advance(hydro, clock: RunClock, *, cfl_max_var: float,
            monitor_timestep: float, t_final: float, max_steps: int = -1,
            bodies=None, on_monitor=None, integrator: str = "euler",
            bodies_second=None, accrete=None, frame_centers=None,
            corotation=None) -> None:
    """The loop of sim::run (simulation.cpp:505-558) with step_Euler or, for
    integrator "leapfrog", step_LeapFrog's gas part.

    bodies(clock) -> (list_of_body_tuples, indirect_x, indirect_y) is called
    before every step (the N-body state of the host at the start of the step;
    for LeapFrog the state the first kick sees); bodies_second(clock, dt), for
    LeapFrog, gives the second kick's (defaults to the first's);
    accrete(clock, dt), for Euler, runs AccreteOntoPlanets where step_Euler
    does, first in the step (simulation.cpp:150-153);
    frame_centers(clock, dt) -> (now, after), for Euler, gives the centres a
    centre-of-mass boundary reads before transport and after the N-body step;
    corotation(clock) -> dOmega, for Euler, is the change of a corotating
    frame's OmegaFrame in the step (handle_corotation,
    frame_of_reference.cpp:30-60), applied to v_phi before the gas step, the
    new OmegaFrame being the fourth item bodies(clock) returns;
    on_monitor(clock) after every step that lands on a monitor time.
    """
    while clock.time < t_final:
        if max_steps >= 0 and clock.n_hydro_iter >= max_steps:
            break
        cfl_dt = calculate_time_step(hydro, clock, cfl_max_var)
        time_next_monitor = (clock.n_monitor + 1) * monitor_timestep
        time_left = time_next_monitor - clock.time
        overshoot = cfl_dt > time_left
        almost_there = time_left < cfl_dt * (1 + 0.05)
        step_dt = time_left if (overshoot or almost_there) else cfl_dt
        if integrator == "leapfrog":
            first = bodies(clock) if bodies is not None else ([], 0.0, 0.0)
            second = bodies_second(clock, step_dt) if bodies_second is not None else first
            step_leapfrog(hydro, step_dt, clock.time, first, second)
        else:
            if accrete is not None:
                accrete(clock, step_dt)
            if corotation is not None:
                domega = corotation(clock)
                if domega != 0.0:
                    hydro.correct_v_azimuthal(domega)
            if bodies is not None:
                b, ix, iy, *omega = bodies(clock)
                hydro.set_bodies(b, ix, iy, omega[0] if omega else 0.0)
            if frame_centers is not None:
                hydro.set_frame_centers(*frame_centers(clock, step_dt))
            hydro.step_euler(step_dt, clock.time)
        clock.dts.append(step_dt)
        clock.time += step_dt
        clock.n_hydro_iter += 1
        if math.fabs(time_next_monitor - clock.time) < 1e-6 * cfl_dt:
            clock.n_monitor += 1
            if on_monitor is not None:
                on_monitor(clock)


def l1_point(central_mass: float, other_mass: float) -> float:
    """init_l1 (Theo.cpp:251-277): the dimensionless distance of the L1 point
    from the central mass, by Newton-Raphson."""
    q = central_mass / (central_mass + other_mass)
    x = math.pow(other_mass / (3.0 * central_mass), 1.0 / 3.0)
    counter = 0
    while True:
        counter += 1
        if counter > 10:
            break
        f = q / math.pow(1.0 - x, 2) - (1.0 - q) / math.pow(x, 2) - q + x
        df = 2.0 * q / math.pow(1.0 - x, 3) + 2.0 * (1.0 - q) / math.pow(x, 3) + 1.0
        x = x - f / df
        if not math.fabs(f) > 1e-14:
            break
    return x


def orbital_elements(x, y, vx, vy, com_mass, mass, G) -> tuple[float, float, float]:
    """Semi-major axis, eccentricity and period of
    t_planet::calculate_orbital_elements (planet.cpp:488-566) for relative
    position and velocity (x, y, vx, vy) about com_mass; zeros where the
    reference sets the elements to zero."""
    m = com_mass + mass
    h = x * vy - y * vx
    d = math.sqrt(x * x + y * y)
    if d == 0.0 or h == 0.0:
        return 0.0, 0.0, 0.0
    Ax = x * vy * vy - y * vx * vy - G * m * x / d
    Ay = y * vx * vx - x * vx * vy - G * m * y / d
    e = math.sqrt(Ax * Ax + Ay * Ay) / G / m
    a = h * h / G / m / (1.0 - e * e)
    if e > 1.0 or e < 0 or a < 0.0:
        return 0.0, 0.0, 0.0
    return a, e, 2.0 * math.pi * math.sqrt(math.pow(a, 3) / (m * G))


def orbital_period(x, y, vx, vy, com_mass, mass, G) -> float:
    """The period of calculate_orbital_elements (0 where it zeroes them)."""
    return orbital_elements(x, y, vx, vy, com_mass, mass, G)[2]


def center_of_mass(bodies, n) -> tuple[float, float, float, float, float]:
    """get_center_of_mass(n), get_center_of_mass_velocity(n) and get_mass(n)
    (nbody/planetary_system.cpp:580-650) of the first n bodies, each an
    (x, y, vx, vy, mass) tuple: the centre a centre-of-mass boundary reads."""
    x = y = vx = vy = mass = 0.0
    for b in bodies[:n]:
        mass += b[4]
        x += b[0] * b[4]
        y += b[1] * b[4]
        vx += b[2] * b[4]
        vy += b[3] * b[4]
    if mass > 0:
        return (x / mass, y / mass, vx / mass, vy / mass, mass)
    return (0.0, 0.0, 0.0, 0.0, mass)


def com_boundary_setup(bodies, G, n_center=1) -> tuple[float, float, int, float]:
    """The arguments of fgpu_init_center_of_mass_boundary for bodies given
    as (x, y, vx, vy, mass) tuples, as init_vr_table_boundary reads them
    (viscous_radial_speed.cpp:269-347): the mass of all bodies, of the
    hydro-frame centre, whether a two-body system is centred on its first
    body, and then a (1 + e) q of the second."""
    n = len(bodies)
    mass_all = center_of_mass(bodies, n)[4]
    mass_center = center_of_mass(bodies, n_center)[4]
    binary = n == 2 and n_center == 1
    dist = 0.0
    if binary:
        c = center_of_mass(bodies, 1)
        b = bodies[1]
        a, e, _ = orbital_elements(b[0] - c[0], b[1] - c[1], b[2] - c[2], b[3] - c[3],
                                   c[4], b[4], G)
        q = b[4] / (b[4] + bodies[0][4])
        dist = a * (1.0 + e) * q
    return mass_all, mass_center, int(binary), dist


def indirect_term_euler(bodies) -> tuple[float, float]:
    """IndirectTermMode Euler with the primary as frame centre:
    ComputeNbodyOnNbodyAccel (Pframeforce.cpp:225-250) for body 0 and
    ComputeIndirectTermNbodyEuler (frame_of_reference.cpp:118-133)."""
    x, y = bodies[0][0], bodies[0][1]
    ax = 0.0
    ay = 0.0
    for other in bodies[1:]:
        xo, yo, mass = other[0], other[1], other[2]
        dist = math.sqrt(math.pow(x - xo, 2) + math.pow(y - yo, 2))
        ax -= 1.0 * mass / math.pow(dist, 3) * (x - xo)
        ay -= 1.0 * mass / math.pow(dist, 3) * (y - yo)
    m0 = bodies[0][2]
    ix = -(m0 * ax)
    iy = -(m0 * ay)
    return ix / m0, iy / m0
