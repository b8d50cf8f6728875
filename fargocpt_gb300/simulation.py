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


def start(hydro, clock: RunClock, cfl_max_var: float) -> None:
    """The calls main() and sim::init() make before the loop
    (main.cpp:117, simulation.cpp:462-480): one CFL evaluation, the initial
    boundary condition, and a second CFL evaluation."""
    calculate_time_step(hydro, clock, cfl_max_var)
    hydro.apply_boundary_condition(clock.time, 0.0, False)
    calculate_time_step(hydro, clock, cfl_max_var)


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
            bodies_second=None) -> None:
    """The loop of sim::run (simulation.cpp:505-558) with step_Euler or, for
    integrator "leapfrog", step_LeapFrog's gas part.

    bodies(clock) -> (list_of_body_tuples, indirect_x, indirect_y) is called
    before every step (the N-body state of the host at the start of the step;
    for LeapFrog the state the first kick sees); bodies_second(clock, dt), for
    LeapFrog, gives the second kick's (defaults to the first's);
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
            if bodies is not None:
                b, ix, iy = bodies(clock)
                hydro.set_bodies(b, ix, iy, 0.0)
            hydro.step_euler(step_dt, clock.time)
        clock.dts.append(step_dt)
        clock.time += step_dt
        clock.n_hydro_iter += 1
        if math.fabs(time_next_monitor - clock.time) < 1e-6 * cfl_dt:
            clock.n_monitor += 1
            if on_monitor is not None:
                on_monitor(clock)


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
