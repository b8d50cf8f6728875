"""Benchmark of the GB300 hydro step: cell-updates/s on the largest
single-GPU disk of the benchmark set, FargoCPT's adiabatic 2048 x 6144 disk
with three planets (r in [0.3, 5], beta cooling, SN artificial viscosity).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c5]
    python bench.py --impl reference ...     # the CPU restatement, all host cores

One step = one FargoCPT Euler hydro step (sim::step_Euler's gas part plus the
CFL dt for the next step) over the whole disk, and the disk force on every
body (ComputeDiskOnNbodyAccel, which step_Euler runs with DiskFeedback).
value: device time of the steps (CUDA events on the engine's stream around
the step and the force read-back, L2 flushed before every timed step, fields
resident in HBM; every field of the 2048 x 6144 disk is 100 MB, so the step's
working set is far larger than L2 too).  e2e: wall time of the drop-in call
sequence a C++ driver makes every step through the C ABI (CFL read-back,
N-body state in, step, disk forces read back).  Multi-GPU runs are
independent replicas (the path does not shard across GPUs here).

Beside the FP64 headline the line carries the FP32-mixed form on the same
disk (``fp32_mixed``) and the batched form (``batched``): 64 independent
FP32-mixed disks of different sizes, each with its own CFL dt from the
device clock, stepped by one launch per phase over all disks, the timed
steps captured as one CUDA graph, tile shapes from the autotuner; it is
compared with the FP64 form stepping the same disks one after another.
``--forms`` limits the run to some of the forms (for profiling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

# Compulsory HBM bytes per cell of each kernel of the FP64 adiabatic step
# (unique fields read + written, 8 B each; halved for FP32).
KERNEL_BYTES_PER_CELL = {
    "potential": 16, "source": 56, "artvisc_q": 56, "artvisc_v": 88, "stress": 64,
    "viscous_substep3": 120, "ghost_pre": 0, "transport_radial": 80,
    "transport_azimuthal": 104, "finish": 80, "damping": 0, "ghost_post": 0,
    "derived_cfl": 88,
}
STEP_BYTES_PER_CELL = {"adiabatic": 64, "isothermal": 48}   # one read + write of the state
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the dominant
# kernels from one-kernel ncu captures (profiles/ names the capture of each)
NCU_DRAM_BYTES = {
    # 2048 x 6144 three-planet adiabatic disk (profiles/traffic_c5_transports.md;
    # the FP64 form's float-pair kernels)
    ("c5", "fp64", "transport_azimuthal"): 713425664 + 602434048,
    ("c5", "fp64", "transport_radial"): 453888256 + 557087488,
    ("c5", "fp32", "transport_azimuthal"): 402961408 + 288184320,
    ("c5", "fp32", "transport_radial"): 295241216 + 318492928,
    # 512 x 1536 adiabatic disk (--set full captures)
    ("c2", "fp64", "transport_azimuthal"): 44.127e6 + 0.422e6,
    ("c2", "fp64", "transport_radial"): 25.252e6 + 0.738e6,
    ("c2", "fp32", "transport_azimuthal"): 25.286e6 + 0.0005e6,
}
STEP_KERNELS = 13   # the adiabatic step's kernels (the force adds two per 4 bodies)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="c5")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--forms", default="fp64,fp32,batch,fp64disks",
                    help="comma list of the forms to time: fp64 (the headline), fp32 "
                    "(FP32-mixed, same disk), batch (64-disk FP32-mixed sweep), fp64disks "
                    "(the FP64 form on the sweep's disks, one after another)")
    ap.add_argument("--batch-disks", type=int, default=64)
    ap.add_argument("--no-autotune", action="store_true")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows, self.proc = [], None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for k, n in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def load_disk(backend, fields, nbody):
    for k, a in fields.items():
        backend.set_field(k, a)
        backend.set_field(k + "0", a)
    b = nbody.bodies(0.0)
    ix, iy = nbody.indirect(b)
    backend.set_bodies(b, ix, iy, 0.0)
    backend.init_euler(0.0)
    backend.apply_boundary_condition(0.0, 0.0, False)


def cpu_baseline(cfg_name, seconds, threads=None):
    """The oracle (CPU restatement of the reference's step), built with the
    reference's shipped flags (-Ofast -march=native -fopenmp), on this host's
    cores over a bounded sample of the same workload."""
    from fargocpt_gb300 import setups
    from oracle.oracle_py import OracleState, build_oracle, set_threads, use_timing_build

    build_oracle()
    use_timing_build()
    cores = set_threads(threads or os.cpu_count() or 1)
    params, d, radii, fields, nbody = setups.build(cfg_name)
    o = OracleState(params, radii)
    load_disk(o, fields, nbody)
    cells = d["nrad"] * d["naz"]
    t, steps, t0 = 0.0, 0, time.perf_counter()
    while True:
        dt = o.condition_cfl()
        b = nbody.bodies(t)
        ix, iy = nbody.indirect(b)
        o.set_bodies(b, ix, iy, 0.0)
        o.step_euler(dt, t)
        for k in range(len(b)):   # ComputeDiskOnNbodyAccel, as the GPU step
            o.disk_on_planet_accel(k)
        t += dt
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds and steps >= 2:
            break
    return {"value": cells * steps / el, "unit": "cell-updates/s", "cores": cores,
            "kind": "port", "build": "-Ofast -march=native -fopenmp (the reference's shipped "
            "flags)", "sample": f"{steps} full steps of {cfg_name} "
            f"({d['nrad']}x{d['naz']}) in {el:.1f} s"}


def max_over_ranks(vals, dist, torch, device):
    """The slowest rank's times: every rank's list of timings reduced with MAX
    (identity without a process group)."""
    if dist is None:
        return list(vals)
    tt = torch.tensor(vals, device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return [float(x) for x in tt]


def run_reference(args, rank):
    if rank != 0:
        return
    cb = cpu_baseline(args.config, args.cpu_seconds)
    from fargocpt_gb300 import setups
    c = setups.CONFIGS[args.config]
    line = {
        "impl": "reference", "metric": "cell-updates/s/GPU, plain FP64 vs mixed-precision "
        "& batched at stated error", "value": cb["value"], "unit": cb["unit"],
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": c["nrad"] * c["naz"] / cb["value"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.config),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def workload_config(name):
    from fargocpt_gb300 import setups
    c = setups.CONFIGS[name]
    return {"workload": f"FargoCPT {'adiabatic' if c['adiabatic'] else 'locally isothermal'} "
            f"disk {c['nrad']}x{c['naz']} (incl. 2 ghost rings), r in [{c['rmin']}, {c['rmax']}], "
            f"{len(c['planets'])} planet(s), FARGO, SN art. visc, alpha=1e-3"
            + (", beta cooling 10" if c["adiabatic"] else "") + ", FP64",
            "nrad": c["nrad"], "naz": c["naz"], "precision": "fp64",
            "l2": "flushed (256 MB write) before every timed step; each FP64 field of the "
                  f"disk is {c['nrad'] * c['naz'] * 8 / 1e6:.0f} MB"}


def measure(args, precision, cfg_name, torch, dist, local):
    """Times `args.steps` steps of one precision form; returns a dict."""
    from fargocpt_gb300 import setups
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine

    params, d, radii, fields, nbody = setups.build(cfg_name)
    if precision == "fp32":
        d = dict(d)
        d["precision"] = 1
        params = params_from_dict(d)
    eng = Engine(params, radii)
    load_disk(eng, fields, nbody)
    cells = d["nrad"] * d["naz"]
    stream = torch.cuda.ExternalStream(eng.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    state = {"t": 0.0}

    def one_step(timed_events=None):
        t = state["t"]
        dt = eng.condition_cfl()
        b = nbody.bodies(t)
        ix, iy = nbody.indirect(b)
        eng.set_bodies(b, ix, iy, 0.0)
        if timed_events is not None:
            with torch.cuda.stream(stream):
                flush.zero_()
                timed_events[0].record(stream)
        eng.step_euler(dt, t)
        # ComputeDiskOnNbodyAccel: every body, one read-back; the end event
        # follows it, so the device time includes the force kernels
        eng.disk_on_nbody_accel(len(b))
        if timed_events is not None:
            timed_events[1].record(stream)
        state["t"] = t + dt

    for _ in range(args.warmup):
        one_step()
    eng.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        one_step(ev[k])
    eng.synchronize()
    torch.cuda.synchronize()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    if dist is not None:
        dist.barrier()
    eng.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    eng.synchronize()
    e2e_s = time.perf_counter() - t0
    eng.set_phase_timing(True)
    for _ in range(args.steps):
        one_step()
    phases, nsteps = eng.phase_times()
    eng.set_phase_timing(False)
    assert eng.check_finite() is None, "non-finite state after the benchmark"
    return dict(total_ms=total_ms, e2e_s=e2e_s, phases=phases, nsteps=nsteps, cells=cells, d=d,
                nbodies=len(nbody.bodies(0.0)))


def measure_batch(args, torch, dist):
    """The batched form on the sweep of independent locally isothermal disks
    (Nr in {128..512}, Naz = 3 Nr, seeded physics): every disk with its own
    CFL dt from the device clock, `args.steps` steps captured as one CUDA
    graph; inputs (about 1.8 GB of fields) far exceed the 129 MB L2."""
    import numpy as np

    from fargocpt_gb300 import setups
    from fargocpt_gb300.batch import Batch, orbits_to_time, start_disks

    disks = setups.sweep(args.batch_disks, seed=4)
    cells = np.array([x[0].nrad * x[0].naz for x in disks], dtype=np.float64)
    b = Batch([x[0] for x in disks], [x[2] for x in disks])
    t_end = orbits_to_time(2.0)
    start_disks(b, disks, t_end=t_end, monitor_dt=t_end / 20)
    t0 = time.perf_counter()
    tiles = b.tiles() if args.no_autotune else b.autotune(reps=5)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.disks[0].stream)

    def steps():
        return np.array([b.clock(k)["steps"] for k in range(b.n)], dtype=np.float64)

    b.run(args.warmup, steps_per_graph=max(1, args.warmup))
    b.run(args.steps, steps_per_graph=args.steps)   # captures the timed graph
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    s0 = steps()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run(args.steps, steps_per_graph=args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    s1 = steps()
    updates = float(np.sum((s1 - s0) * cells))
    # the same steps with the gas kick's and the closing substeps each as one
    # persistent cooperative launch (fgpu_batch_set_mode); then back
    b.set_mode(True)
    b.run(args.steps, steps_per_graph=args.steps)   # captures its graph
    torch.cuda.synchronize()
    p0 = steps()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    b.run(args.steps, steps_per_graph=args.steps)
    e3.record(stream)
    e3.synchronize()
    pers_ms = e2.elapsed_time(e3)
    pers_updates = float(np.sum((steps() - p0) * cells))
    b.set_mode(False)
    # end to end through the C ABI with host buffers: per step, every disk's
    # CFL dt read back, its bodies and (dt, t) sent (fgpu_batch_step)
    dts = np.empty(b.n)
    ts = np.array([b.clock(k)["time"] for k in range(b.n)])
    e2e_updates = 0.0
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        for k, (_, _, _, _, nbody) in enumerate(disks):
            dts[k] = b.disks[k].condition_cfl()
            bk = nbody.bodies(ts[k])
            b.disks[k].set_bodies(bk, *nbody.indirect(bk), 0.0)
        b.step(dts, ts)
        ts += dts
        e2e_updates += float(np.sum(cells))
    e2e_s = time.perf_counter() - w0
    for e in b.disks:
        assert e.check_finite() is None, "non-finite state after the batched benchmark"
    out = dict(ms=ms, updates=updates, e2e_s=e2e_s, e2e_updates=e2e_updates, tiles=tiles,
               pers_ms=pers_ms, pers_updates=pers_updates,
               tune_s=tune_s, cells=float(np.sum(cells)), n=b.n,
               nr=sorted(set(int(x[0].nrad) for x in disks)))
    b.close()
    return out, disks


def measure_fp64_disks(disks, torch, steps=5, warmup=2):
    """The FP64 form on the same disks, one engine after another (each disk
    alone on the GPU, as FargoCPT runs one disk per process)."""
    from fargocpt_gb300.abi import params_from_dict
    from fargocpt_gb300.engine import Engine

    total_ms, updates = 0.0, 0.0
    for params, d, radii, fields, nbody in disks:
        d64 = dict(d)
        d64["precision"] = 0
        eng = Engine(params_from_dict(d64), radii)
        load_disk(eng, fields, nbody)
        stream = torch.cuda.ExternalStream(eng.stream)
        t = 0.0
        for n in range(warmup + steps):
            if n == warmup:
                eng.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            dt = eng.condition_cfl()
            b = nbody.bodies(t)
            eng.set_bodies(b, *nbody.indirect(b), 0.0)
            eng.step_euler(dt, t)
            t += dt
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        updates += steps * d["nrad"] * d["naz"]
        eng.close()
    return updates / (total_ms * 1e-3)


def roofline(res, steps, bytes_scale, form, cfg_name):
    peak, peak_src = peaks()
    phases, nsteps, cells, d = res["phases"], res["nsteps"], res["cells"], res["d"]
    dom = max(phases, key=phases.get)
    dom_ms = phases[dom] / max(1, nsteps)
    bpc = KERNEL_BYTES_PER_CELL.get(dom, 0) * bytes_scale
    achieved = bpc * cells / (dom_ms * 1e-3) / 1e9
    kind = "adiabatic" if d["eos"] == 1 else "isothermal"
    sbpc = STEP_BYTES_PER_CELL[kind] * bytes_scale
    step_achieved = sbpc * cells * steps / (res["total_ms"] * 1e-3) / 1e9
    traffic = NCU_DRAM_BYTES.get((cfg_name, form, dom))
    # every kernel's algorithmic HBM rate against the peak
    per_kernel = {}
    for k, tot in phases.items():
        ms = tot / max(1, nsteps)
        b = KERNEL_BYTES_PER_CELL.get(k, 0) * bytes_scale
        if ms > 0 and b > 0:
            gbs = b * cells / (ms * 1e-3) / 1e9
            per_kernel[k] = {"ms": ms, "bytes_per_cell": b, "achieved_gbs": gbs,
                             "frac": gbs / peak}
    return ({"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
             "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
             "traffic_unit": "B per launch", "bytes_per_cell": bpc, "ms_per_launch": dom_ms,
             "per_kernel": per_kernel},
            {"achieved": step_achieved, "peak": peak, "unit": "GB/s",
             "frac": step_achieved / peak, "bytes_per_cell": sbpc})


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank)
        if dist is not None:
            dist.barrier()
        return

    import torch

    from fargocpt_gb300.build import build
    if rank == 0:
        build()
    if dist is not None:
        dist.barrier()
    torch.cuda.set_device(local)

    forms = set(args.forms.split(","))
    sampler = ClockSampler(local)
    sampler.start()
    r64 = measure(args, "fp64", args.config, torch, dist, local) if "fp64" in forms else None
    r32 = measure(args, "fp32", args.config, torch, dist, local) if "fp32" in forms else None
    rb, bdisks = measure_batch(args, torch, dist) if "batch" in forms else (None, None)
    clocks = sampler.stop()
    fp64_same = (measure_fp64_disks(bdisks, torch)
                 if rb is not None and "fp64disks" in forms else None)

    vals = [r64["total_ms"] if r64 else 1.0, r64["e2e_s"] if r64 else 1.0,
            r32["total_ms"] if r32 else 1.0, r32["e2e_s"] if r32 else 1.0,
            rb["ms"] if rb else 1.0, rb["e2e_s"] if rb else 1.0]
    vals = max_over_ranks(vals, dist, torch, "cuda")
    if rank != 0:
        return
    batched = None
    if rb is not None:
        bvalue = world * rb["updates"] / (vals[4] * 1e-3)
        peak, peak_src = peaks()
        batched = {
            "value": bvalue, "unit": "cell-updates/s", "ms_per_step": vals[4] / args.steps,
            "workload": f"{rb['n']} independent locally isothermal FP32-mixed disks, Nr in "
                        f"{rb['nr']}, Naz = 3 Nr, {rb['cells']:.0f} cells, own CFL dt each "
                        "(device clock), seeded alpha/q/h/slope, steps as one CUDA graph, "
                        "inputs larger than L2",
            "e2e": {"value": world * rb["e2e_updates"] / vals[5], "unit": "cell-updates/s",
                    "h2d_bytes_per_step": rb["n"] * (2 * 40 + 16),
                    "d2h_bytes_per_step": rb["n"] * 8,
                    "path": "host clock: per step every disk's CFL dt read, bodies and "
                            "(dt, t) sent, fgpu_batch_step"},
            "fp64_same_disks": fp64_same,
            "speedup_vs_fp64_same_disks": bvalue / fp64_same if fp64_same else None,
            "roofline_step": {"achieved": bvalue * 24 / 1e9, "peak": peak, "unit": "GB/s",
                              "frac": bvalue * 24 / 1e9 / peak, "bytes_per_cell": 24,
                              "peak_source": peak_src},
            "tiles": rb["tiles"], "autotune_s": rb["tune_s"],
            "gpu_launches": 14 * args.steps,
            # the same steps with the substeps of the gas kick and of the
            # step's close each as one persistent cooperative launch
            "persistent_sequences": {
                "value": world * rb["pers_updates"] / (rb["pers_ms"] * 1e-3),
                "unit": "cell-updates/s", "ms_per_step": rb["pers_ms"] / args.steps,
                "launches_per_step": "clock, 2 persistent sequences, transports"},
            "error": "per disk the FP32-mixed arithmetic (bit-identical to the single-disk "
                     "FP32-mixed engine); python -m fargocpt_gb300.accuracy gives its error",
        }
    if r64 is None:
        print(json.dumps({"forms": sorted(forms), "batched": batched,
                          "fp32_mixed_ms": vals[2] / args.steps if r32 else None,
                          "clocks": clocks}))
        return
    cells = r64["cells"]
    value = world * cells * args.steps / (vals[0] * 1e-3)
    e2e = world * cells * args.steps / vals[1]
    rl, rls = roofline(r64, args.steps, 1.0, "fp64", args.config)
    # what bounds the float-pair transports (ncu --set full on 512 rings of
    # 6144 cells, profiles/transport_kernels_c5_fp64_pair.md): issue, the
    # FP64 pipe and latency, not DRAM
    rl["ncu_pipes_pct"] = {
        "transport_azimuthal": {"issue_active": 53.4, "fp64_pipe": 54.5, "fma_pipe": 26.4},
        "transport_radial": {"issue_active": 58.8, "fp64_pipe": 42.7, "fma_pipe": 31.6}}
    fp32 = None
    if r32 is not None:
        value32 = world * cells * args.steps / (vals[2] * 1e-3)
        e2e32 = world * cells * args.steps / vals[3]
        rl32, rls32 = roofline(r32, args.steps, 0.5, "fp32", args.config)
        fp32 = {
            "value": value32, "unit": "cell-updates/s", "ms_per_step": vals[2] / args.steps,
            "e2e": {"value": e2e32, "unit": "cell-updates/s",
                    "h2d_bytes_per_step": 40 * r32["nbodies"],
                    "d2h_bytes_per_step": 8 + 40 * r32["nbodies"]},
            "speedup_vs_fp64": value32 / value,
            "roofline": rl32, "roofline_step": rls32,
            "phase_ms_per_step": {k: v / max(1, r32["nsteps"])
                                  for k, v in r32["phases"].items()},
            "error": "see python -m fargocpt_gb300.accuracy (relative L1/Linf vs FP64)",
        }
    line = {
        "metric": "cell-updates/s/GPU, plain FP64 vs mixed-precision & batched at stated error",
        "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": vals[0] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.config),
        "e2e": {"value": e2e, "unit": "cell-updates/s",
                # fgpu_body per body (kernel arguments); CFL dt + 5 force sums per body
                "h2d_bytes_per_step": 40 * r64["nbodies"],
                "d2h_bytes_per_step": 8 + 40 * r64["nbodies"]},
        "roofline": rl,
        "roofline_step": rls,
        "phase_ms_per_step": {k: v / max(1, r64["nsteps"]) for k, v in r64["phases"].items()},
        "fp32_mixed": fp32,
        "batched": batched,
        "gpu_launches": args.steps * (STEP_KERNELS + 2 * ((r64["nbodies"] + 3) // 4)),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.config, args.cpu_seconds)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
