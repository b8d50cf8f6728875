"""Error of the FP32-mixed form against the FP64 form.

    python -m fargocpt_gb300.accuracy --config c3 --orbits 10 [--out file.json]

Both forms start from the same disk and are driven with the same dt sequence
(the FP64 form's CFL dt, clamped to land on every output time) and the same
planet positions.  Reported per field: relative L1 (sum |a - b| / sum |b|) and
relative L-infinity (max |a - b| / max |b|) of sigma, v_r, v_phi, the v_phi
residual about Keplerian, and e, plus the relative error of the disk torque on
the planet.  The FP64 form itself agrees with FargoCPT's own FP64 build to
1e-12 (tests/test_gpu_golden.py), so it stands in for the FP64 reference.

    python -m fargocpt_gb300.accuracy --compare perturbed ...

calibrates how much of that error any FP32 storage must incur: the second
run is the FP64 form again, started from the same disk with v_r and the v_phi
residual about Keplerian rounded once to FP32 (what the FP32-mixed form's
upload does to them; its sigma is a compensated pair and stays exact), plus
optional relative noise of the given size on sigma (--sigma-noise).  The
difference it grows to is the flow's own amplification of FP32-sized
perturbations.

    python -m fargocpt_gb300.accuracy --config c1 --set fast_transport=0 --no-planet ...

changes parameters of both forms (--set name=value, repeatable) or drops the
planet, to see which physics carries the difference.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np


def rel_l1(a, b):
    return float(np.sum(np.abs(a - b)) / max(float(np.sum(np.abs(b))), 1e-300))


def rel_linf(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def run(config="c3", orbits=10.0, outputs=10, seed=1234, log=sys.stderr, compare="fp32",
        sigma_noise=0.0, overrides=None, planet=True):
    from . import setups
    from .abi import params_from_dict
    from .engine import Engine

    p64, d, radii, fields, nbody = setups.build(config, seed=seed)
    if overrides:
        d = dict(d)
        d.update(overrides)
        p64 = params_from_dict(d)
    full_bodies = nbody.bodies

    def bodies_at(t):
        b = full_bodies(t)
        return b if planet else b[:1]

    def indirect(b):
        return nbody.indirect(b) if len(b) > 1 else (0.0, 0.0)
    nr = d["nrad"]
    rinf, rsup = radii[:nr], radii[1:nr + 1]
    rmed = 2.0 / 3.0 * (rsup ** 3 - rinf ** 3) / (rsup ** 2 - rinf ** 2)
    vk = np.sqrt(d["G"] * d["hydro_center_mass"] / rmed)[:, None]
    second = dict(fields)
    if compare == "fp32":
        d32 = dict(d)
        d32["precision"] = 1
        p2 = params_from_dict(d32)
    else:
        p2 = p64
        second["V_RADIAL"] = fields["V_RADIAL"].astype(np.float32).astype(np.float64)
        res = (fields["V_AZIMUTHAL"] - vk).astype(np.float32).astype(np.float64)
        second["V_AZIMUTHAL"] = vk + res
        if sigma_noise > 0:
            rng = np.random.default_rng(seed + 1)
            second["SIGMA"] = fields["SIGMA"] * (1 + sigma_noise * rng.uniform(-1, 1,
                                                                              fields["SIGMA"].shape))
    engines = [Engine(p64, radii), Engine(p2, radii)]
    for e, start in zip(engines, (fields, second)):
        for k, a in start.items():
            e.set_field(k, a)
            e.set_field(k + "0", fields[k])
        b = bodies_at(0.0)
        e.set_bodies(b, *indirect(b), 0.0)
        e.init_euler(0.0)
        e.apply_boundary_condition(0.0, 0.0, False)
    e64, e32 = engines
    t_end = orbits * 2.0 * math.pi
    t, steps, t0 = 0.0, 0, time.time()
    history = []
    for k in range(1, outputs + 1):
        t_out = t_end * k / outputs
        while t < t_out:
            dt = min(e64.condition_cfl(), t_out - t)
            if t_out - t - dt < 1e-12 * t_out:
                dt = t_out - t
            b = bodies_at(t)
            ix, iy = indirect(b)
            for e in engines:
                e.set_bodies(b, ix, iy, 0.0)
                e.step_euler(dt, t)
            t += dt
            steps += 1
        b = bodies_at(t)
        ix, iy = indirect(b)
        rec = {"orbits": t / (2 * math.pi), "steps": steps}
        if planet:
            for name, e in (("fp64", e64), ("fp32", e32)):
                e.set_bodies(b, ix, iy, 0.0)
                ax, ay = e.disk_on_planet_accel(1)
                x, y, m = b[1][0], b[1][1], b[1][2]
                rec[f"torque_{name}"] = (x * ay - y * ax) * m
            rec["torque_rel_err"] = abs(rec["torque_fp32"] - rec["torque_fp64"]) / max(
                abs(rec["torque_fp64"]), 1e-300)
        for f in ("SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY"):
            a, c = e64.get_field(f), e32.get_field(f)
            if f == "ENERGY" and d["eos"] == 0:
                continue
            rec[f"{f}_l1"] = rel_l1(c, a)
            rec[f"{f}_linf"] = rel_linf(c, a)
            if f == "V_AZIMUTHAL":
                rec["V_AZIMUTHAL_residual_l1"] = rel_l1(c - vk, a - vk)
                rec["V_AZIMUTHAL_residual_linf"] = rel_linf(c - vk, a - vk)
        rec["finite_fp32"] = e32.check_finite() is None
        history.append(rec)
        print(json.dumps(rec), file=log, flush=True)
    return {"config": config, "grid": [d["nrad"], d["naz"]], "orbits": orbits,
            "compare": compare, "sigma_noise": sigma_noise, "overrides": overrides or {},
            "planet": planet,
            "steps": steps, "seconds": time.time() - t0, "history": history,
            "final": history[-1]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c3")
    ap.add_argument("--orbits", type=float, default=10.0)
    ap.add_argument("--outputs", type=int, default=10)
    ap.add_argument("--out", default=None)
    ap.add_argument("--compare", default="fp32", choices=["fp32", "perturbed"])
    ap.add_argument("--sigma-noise", type=float, default=0.0)
    ap.add_argument("--set", action="append", default=[], metavar="NAME=VALUE",
                    help="override an fgpu_params field in both forms")
    ap.add_argument("--no-planet", action="store_true")
    a = ap.parse_args()
    overrides = {}
    for item in a.set:
        name, _, value = item.partition("=")
        overrides[name] = float(value) if "." in value or "e" in value else int(value)
    from .build import build
    build()
    res = run(a.config, a.orbits, a.outputs, compare=a.compare, sigma_noise=a.sigma_noise,
              overrides=overrides, planet=not a.no_planet)
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(json.dumps(res["final"]))


if __name__ == "__main__":
    main()
