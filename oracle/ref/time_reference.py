"""Times FargoCPT itself (built by this directory's Makefile with its shipped
optimisation flags, VARIANT=timing) beside the oracle's C restatement on the
same host cores, for the CPU baseline of the benchmark disks.

Test infrastructure: it runs the reference binary and the oracle, never the
GPU engine.  Needs the reference's sources for the build (REF=... as for the
Makefile; by default a checkout named "reference" beside the repository).

For each workload (the disks of fargocpt_gb300.setups) it writes a FargoCPT
setup with the same grid, physics and planets, and a seeded initial sigma
(SigmaCondition: 2D), then runs the reference for n1 and n2 hydro steps
(-N, options.cpp:157-163) and takes the difference of the walltimes its final
log line reports (logging.cpp:186-201), so the set-up and the initial
snapshot cancel.  The oracle, in the build bench.py's CPU leg times (the reference's shipped
flags), takes the same number of steps of the same call sequence (CFL,
step, disk force on every body).

    python oracle/ref/time_reference.py c2 c5 --threads 8 1 [--n1 2 --n2 12]

prints one JSON line per (workload, threads).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

EXE = os.path.join(REPO, "oracle", "_ref", "timing", "fargocpt")


def setup_text(name):
    from fargocpt_gb300 import setups

    c = setups.CONFIGS[name]
    adi = c["adiabatic"]
    keys = dict(
        l0="1 au", m0="1 solMass", mu=2.35, Sigma0=1e-3, SigmaSlope=c["slope"],
        AspectRatio=0.05, FlaringIndex=c["flaring"], ViscousAlpha=1e-3,
        EquationOfState="Ideal" if adi else "Isothermal", AdiabaticIndex=1.4,
        ArtificialViscosity="SN", ArtificialViscosityFactor=1.41421356 if adi else 1.41,
        ThicknessSmoothing=0.6, Integrator="Euler", InitializeVradialZero="yes",
        FirstDT=1e-9, CFL=0.5, Frame="Fixed", HydroFrameCenter="primary",
        IndirectTermMode=1, DiskFeedback="yes" if name != "c1" else "no",
        RadialSpacing="Logarithmic", Transport="FARGO",
        InnerBoundary="outflow", OuterBoundary="outflow",
        Damping="yes", DampingInnerLimit=1.05, DampingOuterLimit=0.95,
        DampingSurfaceDensityInner="Reference", DampingSurfaceDensityOuter="Reference",
        DampingVRadialInner="Reference", DampingVRadialOuter="Reference",
        DampingVAzimuthalInner="Reference", DampingVAzimuthalOuter="Reference",
        WriteDiskQuantities="no", MonitorTimestep=1000.0, Nmonitor=1, Nsnapshots=1,
        Nrad=c["nrad"], Naz=c["naz"], Rmin=c["rmin"], Rmax=c["rmax"],
        SigmaCondition="2D", SigmaFilename="sigma_init.dat", OutputDir="out")
    if adi:
        keys.update(CoolingBetaLocal="yes", CoolingBeta=10,
                    DampingEnergyInner="Reference", DampingEnergyOuter="Reference")
    lines = [f"{k}: {v}" for k, v in keys.items()]
    lines.append("nbody:")
    lines.append("- name: star\n  semi-major axis: 0.0\n  mass: 1.0")
    for k, (q, a, _) in enumerate(c["planets"]):
        lines.append(f"- name: planet{k}\n  semi-major axis: {a}\n  mass: {q}\n"
                     "  eccentricity: 0.0")
    return "\n".join(lines) + "\n", c


def write_sigma(c, path, seed=1234):
    from fargocpt_gb300.setups import log_radii

    nr, nz = c["nrad"], c["naz"]
    radii = log_radii(nr, c["rmin"], c["rmax"])
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    rng = np.random.default_rng(seed)
    sigma = 1e-3 * rmed[:, None] ** -c["slope"] * (1 + 1e-3 * rng.uniform(-1, 1, (nr, nz)))
    sigma.astype("<f8").tofile(os.path.join(path, "sigma_init.dat"))


def walltime(tmp, steps, threads):
    out = os.path.join(tmp, "out")
    shutil.rmtree(out, ignore_errors=True)
    env = {**os.environ, "OMP_NUM_THREADS": str(threads), "OMP_PROC_BIND": "close"}
    r = subprocess.run([EXE, "-N", str(steps), "start", "setup.yml"], cwd=tmp,
                       capture_output=True, text=True, env=env, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    m = re.search(r"Total Hydrosteps (\d+), Time [^,]+, Walltime ([0-9.]+) seconds",
                  r.stdout)
    if not m or int(m.group(1)) != steps:
        raise RuntimeError("unexpected final line: " + r.stdout.splitlines()[-1])
    return float(m.group(2))


def time_reference(name, threads, n1, n2):
    text, c = setup_text(name)
    tmp = tempfile.mkdtemp(prefix=f"time_{name}_")
    try:
        with open(os.path.join(tmp, "setup.yml"), "w") as f:
            f.write(text)
        write_sigma(c, tmp)
        w1 = walltime(tmp, n1, threads)
        w2 = walltime(tmp, n2, threads)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    ms = (w2 - w1) / (n2 - n1) * 1e3
    return ms, c["nrad"] * c["naz"]


def time_oracle(name, threads, n1, n2):
    from fargocpt_gb300 import setups
    from oracle.oracle_py import OracleState, set_threads, use_timing_build

    use_timing_build()   # the build the CPU baseline times

    set_threads(threads)
    params, d, radii, fields, nbody = setups.build(name)
    o = OracleState(params, radii)
    for k, a in fields.items():
        o.set_field(k, a)
        o.set_field(k + "0", a)
    b = nbody.bodies(0.0)
    o.set_bodies(b, *nbody.indirect(b), 0.0)
    o.init_euler(0.0)
    o.apply_boundary_condition(0.0, 0.0, False)
    t = 0.0
    t0 = None
    for s in range(n2):
        if s == n1:
            t0 = time.perf_counter()
        dt = o.condition_cfl()
        b = nbody.bodies(t)
        o.set_bodies(b, *nbody.indirect(b), 0.0)
        o.step_euler(dt, t)
        if name != "c1":
            for k in range(len(b)):
                o.disk_on_planet_accel(k)
        t += dt
    return (time.perf_counter() - t0) / (n2 - n1) * 1e3


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workloads", nargs="+")
    ap.add_argument("--threads", type=int, nargs="+", default=[os.cpu_count() or 1])
    ap.add_argument("--n1", type=int, default=2)
    ap.add_argument("--n2", type=int, default=12)
    args = ap.parse_args()
    if not os.path.exists(EXE):
        subprocess.run(["make", "-s", "-C", HERE, "VARIANT=timing", "-j8"], check=True)
    for name in args.workloads:
        for th in args.threads:
            ms_ref, cells = time_reference(name, th, args.n1, args.n2)
            ms_or = time_oracle(name, th, args.n1, args.n2)
            print(json.dumps({
                "workload": name, "cells": cells, "threads": th,
                "reference_ms_per_step": ms_ref,
                "reference_cell_updates_per_s": cells / (ms_ref * 1e-3),
                "oracle_ms_per_step": ms_or, "oracle_cell_updates_per_s": cells / (ms_or * 1e-3),
                "reference_over_oracle_speed": ms_or / ms_ref,
                "steps": args.n2 - args.n1}), flush=True)


if __name__ == "__main__":
    main()
