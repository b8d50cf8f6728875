"""Host-side mirror of FargoCPT's run loop (reference src/simulation.cpp).

FargoCPT's C++ driver owns the run; this module restates the part of it that
decides *when* the hydro step is called and with which dt, so that the engine
can be driven exactly like ``sim::run`` drives ``step_Euler``:

* ``CalculateTimeStep`` (simulation.cpp:100-118): dt = min(CFLmaxVar * last_dt,
  CFL dt);
* the clamp of the step to the next monitor time (simulation.cpp:526-540);
* the monitor bookkeeping (simulation.cpp:544-550).

Any object with the hydro-step methods (``condition_cfl``, ``step_euler``,
``apply_boundary_condition``, ``set_bodies``) can be driven; the product uses
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


def advance(hydro, clock: RunClock, *, cfl_max_var: float,
            monitor_timestep: float, t_final: float, max_steps: int = -1,
            bodies=None, on_monitor=None) -> None:
    """The loop of sim::run (simulation.cpp:505-558) with step_Euler.

    bodies(clock) -> (list_of_body_tuples, indirect_x, indirect_y) is called
    before every step (the N-body state of the host at the start of the step);
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
