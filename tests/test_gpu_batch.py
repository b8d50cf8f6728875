"""The batched many-disk form (fgpu_batch_*).

Bars:
* host clock: every disk of a batch, stepped with the dt, time and bodies a
  single-disk FP32-mixed engine gets, ends bit-identical to that engine
  (the batched kernels run the single-disk bodies);
* device clock: per disk, the same number of steps and the same end time as
  FargoCPT's run loop (simulation.advance) driving a single-disk engine,
  and fields within 1e-6 relative L1 / 1e-5 relative L-infinity (the planet
  positions come from the device's cos/sin, which may differ from the
  host's in the last bit);
* a step sequence split into CUDA graphs of any length gives bit-identical
  results;
* the autotuner leaves the state as it found it, and the tile shapes it
  picks do not change a bit of the results (ring sums are integer sums of
  fixed-point values, which do not depend on the order of addition).
"""
import ctypes as C

import numpy as np
import pytest

from gpu_cases import initial_state, make_params

pytestmark = pytest.mark.gpu

EVOLVED = ("SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY")


def _small_disks():
    from fargocpt_gb300.setups import log_radii
    specs = [(24, 72, False, 1e-3), (32, 96, False, 3e-3), (16, 48, True, 1e-3),
             (40, 120, False, 1e-4)]
    out = []
    for k, (nr, nz, adi, alpha) in enumerate(specs):
        p, d = make_params(nr, nz, adi, precision=1, viscous_alpha=alpha)
        radii = log_radii(nr, 0.4, 2.5)
        out.append((p, d, radii, initial_state(d, radii, seed=10 + k)))
    return out


def _load(e, state, bodies):
    for f, a in state.items():
        e.set_field(f, a)
        e.set_field(f + "0", a)
    e.set_bodies(bodies, 0.0, 0.0, 0.0)
    e.init_euler(0.0)


def _bodies(t):
    x, y = np.cos(0.3 + t), np.sin(0.3 + t)
    return [(0.0, 0.0, 1.0, 0.0, 0.0), (float(x), float(y), 1e-3, 0.0, 1.0)]


def rel_l1(a, b):
    return float(np.sum(np.abs(a - b)) / max(np.sum(np.abs(b)), 1e-300))


def rel_linf(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_host_clock_matches_single_disks_bit_for_bit():
    from fargocpt_gb300.batch import Batch
    from fargocpt_gb300.engine import Engine

    disks = _small_disks()
    singles = [Engine(p, r) for p, _, r, _ in disks]
    batch = Batch([p for p, *_ in disks], [r for _, _, r, _ in disks])
    b0 = _bodies(0.0)
    for e, (_, _, _, st), be in zip(singles, disks, batch.disks):
        _load(e, st, b0)
        _load(be, st, b0)
    t = np.zeros(len(disks))
    for n in range(15):
        dts = np.empty(len(disks))
        for k, (e, be) in enumerate(zip(singles, batch.disks)):
            ds, db = e.condition_cfl(), be.condition_cfl()
            assert ds == db, (n, k)
            dts[k] = ds
        if n == 7:
            dts[2] = 0.0  # disk 2 sits this step out
        for k, (e, be) in enumerate(zip(singles, batch.disks)):
            bk = _bodies(float(t[k]))
            be.set_bodies(bk, 0.0, 0.0, 0.0)
            if dts[k] > 0:
                e.set_bodies(bk, 0.0, 0.0, 0.0)
                e.step_euler(float(dts[k]), float(t[k]))
        batch.step(dts, t)
        t += dts
    for k, (e, be) in enumerate(zip(singles, batch.disks)):
        for f in EVOLVED:
            a, b = be.get_field(f), e.get_field(f)
            assert np.array_equal(a, b), f"disk {k} {f}: {np.max(np.abs(a - b))}"
    # the disks belong to the batch
    assert batch.lib.fgpu_destroy(batch.disks[0].h) == -1
    batch.close()


def test_accretion_on_a_batch_disk_matches_single_disk():
    # AccreteOntoPlanets (accretion.cpp:84-480) called on a disk of a batch
    # between batch steps acts like the same call on a single-disk engine.
    import math

    from fargocpt_gb300.abi import ACCRETION, FgpuAccretor
    from fargocpt_gb300.batch import Batch
    from fargocpt_gb300.engine import Engine
    from fargocpt_gb300.setups import log_radii

    disks = []
    for k, (nr, nz, adi) in enumerate([(24, 72, False), (16, 48, True)]):
        p, d = make_params(nr, nz, adi, precision=1, viscous_alpha=1e-3,
                           accretion_radius_fraction=1.5)
        radii = log_radii(nr, 0.4, 2.5)
        disks.append((p, radii, initial_state(d, radii, seed=30 + k)))
    singles = [Engine(p, r) for p, r, _ in disks]
    batch = Batch([p for p, *_ in disks], [r for _, r, _ in disks])
    b0 = _bodies(0.0)
    for e, (_, _, st), be in zip(singles, disks, batch.disks):
        _load(e, st, b0)
        _load(be, st, b0)
    x, y = b0[1][0], b0[1][1]
    t = np.zeros(len(disks))
    for n in range(4):
        dts = np.array([e.condition_cfl() for e in singles])
        for k, (e, be) in enumerate(zip(singles, batch.disks)):
            assert be.condition_cfl() == dts[k]
            acc = FgpuAccretor(type=ACCRETION["kley"], x=x, y=y, r=math.hypot(x, y),
                               phi=math.atan2(y, x), roche_radius=(1e-3 / 3) ** (1 / 3),
                               efficiency=10.0, orbital_period=2 * math.pi)
            ss, sb = e.accrete_onto_planet(acc, dts[k]), be.accrete_onto_planet(acc, dts[k])
            assert ss[0] > 0 and ss == sb, (n, k, ss, sb)
            e.step_euler(float(dts[k]), float(t[k]))
        batch.step(dts, t)
        t += dts
    for k, (e, be) in enumerate(zip(singles, batch.disks)):
        for f in EVOLVED:
            a, b = be.get_field(f), e.get_field(f)
            assert np.array_equal(a, b), f"disk {k} {f}: {np.max(np.abs(a - b))}"
    batch.close()


def _sweep(n, seed):
    from fargocpt_gb300 import setups
    return setups.sweep(n_disks=n, seed=seed, nr_choices=(16, 24, 32, 48))


def _host_reference(disk, t_end, monitor_dt):
    from fargocpt_gb300 import simulation
    from fargocpt_gb300.engine import Engine
    params, d, radii, fields, nbody = disk
    e = Engine(params, radii)
    for name, a in fields.items():
        e.set_field(name, a)
        e.set_field(name + "0", a)
    b0 = nbody.bodies(0.0)
    e.set_bodies(b0, *nbody.indirect(b0))
    e.init_euler(0.0)
    clock = simulation.RunClock()
    simulation.start(e, clock, d["cfl_max_var"])

    def bodies(c):
        b = nbody.bodies(c.time)
        return (b, *nbody.indirect(b))

    simulation.advance(e, clock, cfl_max_var=d["cfl_max_var"], monitor_timestep=monitor_dt,
                       t_final=t_end, bodies=bodies)
    return e, clock


def test_device_clock_follows_the_run_loop():
    from fargocpt_gb300.batch import Batch, start_disks
    disks = _sweep(5, seed=11)
    t_end, monitor_dt = 0.06, 0.02
    batch = Batch([x[0] for x in disks], [x[2] for x in disks])
    start_disks(batch, disks, t_end=t_end, monitor_dt=monitor_dt)
    active = batch.run(100000, steps_per_graph=32)
    assert active == 0
    for k, disk in enumerate(disks):
        ref, clock = _host_reference(disk, t_end, monitor_dt)
        c = batch.clock(k)
        assert c["steps"] == clock.n_hydro_iter, (k, c["steps"], clock.n_hydro_iter)
        assert c["n_monitor"] == clock.n_monitor
        assert abs(c["time"] - clock.time) <= 1e-14 * t_end
        assert c["active"] == 0
        for f in ("SIGMA", "V_RADIAL", "V_AZIMUTHAL"):
            a, b = batch.disks[k].get_field(f), ref.get_field(f)
            if f == "V_RADIAL":
                # v_r is a small difference of large terms: scale by its maximum
                assert rel_linf(a, b) <= 1e-3, (k, f)
                continue
            assert rel_l1(a, b) <= 1e-6, (k, f, rel_l1(a, b))
            assert rel_linf(a, b) <= 1e-5, (k, f, rel_linf(a, b))
    batch.close()


def test_graph_length_does_not_change_results():
    from fargocpt_gb300.batch import Batch, start_disks
    disks = _sweep(4, seed=5)
    out = []
    for spg in (12, 5):
        batch = Batch([x[0] for x in disks], [x[2] for x in disks])
        start_disks(batch, disks, t_end=1.0, monitor_dt=0.1)
        batch.run(12, steps_per_graph=spg)
        out.append([{f: e.get_field(f) for f in EVOLVED} for e in batch.disks])
        assert all(batch.clock(k)["steps"] == 12 for k in range(len(disks)))
        batch.close()
    for k in range(len(disks)):
        for f in EVOLVED:
            assert np.array_equal(out[0][k][f], out[1][k][f]), (k, f)


def test_autotune_restores_state_and_keeps_results(tmp_path):
    from fargocpt_gb300.batch import Batch, start_disks
    disks = _sweep(4, seed=9)
    tuned = Batch([x[0] for x in disks], [x[2] for x in disks])
    plain = Batch([x[0] for x in disks], [x[2] for x in disks])
    for b in (tuned, plain):
        start_disks(b, disks, t_end=1.0, monitor_dt=0.1)
        b.run(20, steps_per_graph=10)
    before = [{f: e.get_field(f) for f in EVOLVED} for e in tuned.disks]
    cache = str(tmp_path / "tiles.json")
    best = tuned.autotune(reps=2, cache=cache)
    assert set(best) == set(tuned.tiles())
    after = [{f: e.get_field(f) for f in EVOLVED} for e in tuned.disks]
    for k in range(len(disks)):
        for f in EVOLVED:
            assert np.array_equal(before[k][f], after[k][f]), (k, f)
    # a second call is served by the cache
    assert tuned.autotune(reps=2, cache=cache) == best
    for b in (tuned, plain):
        b.run(20, steps_per_graph=10)
    # ring sums are integer sums, so other tile shapes give the same bits
    for k in range(len(disks)):
        for f in EVOLVED:
            a, b = tuned.disks[k].get_field(f), plain.disks[k].get_field(f)
            assert np.array_equal(a, b), (k, f, rel_linf(a, b))
    tuned.close()
    plain.close()


def test_every_tile_shape_gives_the_same_bits():
    from fargocpt_gb300.batch import Batch, start_disks
    disks = _sweep(3, seed=21)
    ref = None
    shapes = [None, {"transport_azimuthal": [64, 1], "derived_cfl": [512, 1],
                     "potential": [256, 4], "transport_radial": [128, 8]},
              {"transport_azimuthal": [256, 1], "derived_cfl": [128, 1],
               "finish": [64, 8], "transport_radial": [32, 64]}]
    for shape in shapes:
        b = Batch([x[0] for x in disks], [x[2] for x in disks])
        if shape:
            t = b.tiles()
            t.update(shape)
            b.set_tiles(t)
        start_disks(b, disks, t_end=1.0, monitor_dt=0.1)
        b.run(30, steps_per_graph=15)
        out = [{f: e.get_field(f) for f in EVOLVED} for e in b.disks]
        b.close()
        if ref is None:
            ref = out
            continue
        for k in range(len(disks)):
            for f in EVOLVED:
                assert np.array_equal(ref[k][f], out[k][f]), (shape, k, f)


def test_bad_tiles_are_rejected():
    from fargocpt_gb300.batch import Batch
    from fargocpt_gb300.engine import EngineError
    disks = _sweep(2, seed=3)
    batch = Batch([x[0] for x in disks], [x[2] for x in disks])
    t = batch.tiles()
    bad = dict(t)
    bad["potential"] = [100, 1]
    with pytest.raises(EngineError):
        batch.set_tiles(bad)
    assert batch.tiles() == t
    batch.close()


def test_register_blocked_groups_match_strided_pass(monkeypatch):
    """Disks whose rings split into whole segments take the register-blocked
    ring pass in groups of equal ring length, the others the strided pass;
    with FARGO_GB300_AZIMUTHAL=strided every disk takes the strided pass.
    Both give the same bits."""
    from fargocpt_gb300 import setups
    from fargocpt_gb300.batch import Batch, start_disks
    # rings of 96 and 144 cells (strided and blocked), 384 and 576 (blocked)
    disks = setups.sweep(n_disks=6, seed=13, nr_choices=(32, 48, 128, 192))
    out = []
    for variant in ("strided", None):
        if variant:
            monkeypatch.setenv("FARGO_GB300_AZIMUTHAL", variant)
        else:
            monkeypatch.delenv("FARGO_GB300_AZIMUTHAL", raising=False)
        batch = Batch([x[0] for x in disks], [x[2] for x in disks])
        start_disks(batch, disks, t_end=1.0, monitor_dt=0.1)
        batch.run(8, steps_per_graph=4)
        out.append([{f: e.get_field(f) for f in EVOLVED} for e in batch.disks])
        batch.close()
    for k in range(len(disks)):
        for f in EVOLVED:
            assert np.array_equal(out[0][k][f], out[1][k][f]), (k, f)


def test_persistent_substep_sequences_give_the_same_bits():
    """FGPU_BATCH_PERSISTENT runs the gas kick's substeps and the closing
    substeps as two cooperative launches with grid-wide synchronisation
    between substeps: bit-identical to one launch per substep, with the
    host clock (isothermal and adiabatic disks, a disk sitting a step out)
    and with the device clock in CUDA graphs."""
    from fargocpt_gb300.batch import Batch, start_disks

    small = _small_disks()
    host = []
    for persistent in (False, True):
        b = Batch([p for p, *_ in small], [r for _, _, r, _ in small])
        b.set_mode(persistent)
        assert b.persistent == persistent
        b0 = _bodies(0.0)
        for be, (_, _, _, st) in zip(b.disks, small):
            _load(be, st, b0)
        t = np.zeros(len(small))
        for n in range(10):
            dts = np.array([be.condition_cfl() for be in b.disks])
            if n == 4:
                dts[1] = 0.0
            for k, be in enumerate(b.disks):
                be.set_bodies(_bodies(float(t[k])), 0.0, 0.0, 0.0)
            b.step(dts, t)
            t += dts
        host.append([{f: e.get_field(f) for f in EVOLVED} for e in b.disks])
        b.close()
    disks = _sweep(4, seed=31)
    dev = []
    for persistent in (False, True):
        b = Batch([x[0] for x in disks], [x[2] for x in disks])
        b.set_mode(persistent)
        start_disks(b, disks, t_end=1.0, monitor_dt=0.1)
        b.run(24, steps_per_graph=8)
        dev.append([{f: e.get_field(f) for f in EVOLVED} for e in b.disks])
        steps = [b.clock(k)["steps"] for k in range(len(disks))]
        b.close()
        assert all(s == 24 for s in steps)
    for out in (host, dev):
        for k in range(len(out[0])):
            for f in EVOLVED:
                assert np.array_equal(out[0][k][f], out[1][k][f]), (k, f)
