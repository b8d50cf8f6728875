"""The oracle against fixtures produced by the FargoCPT reference itself.

The fixtures (tests/golden/*.npz) are snapshots of the reference built from its
own sources with its FP64 parity flags; make_golden.py regenerates them.  The
oracle follows the reference's operation order, so fields agree bit for bit;
the disk torque is a reduction whose summation order differs (OpenMP), so it
is held to 1e-12 relative.
"""
import re

import numpy as np
import pytest

from golden_runner import CASES, EVOLVED, load_case, replay, rel_linf
from oracle.oracle_py import OracleState


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_snapshots(name):
    snaps, times, torques, dts, arrays = replay(OracleState, name)
    assert snaps, "no snapshot reached"
    meta, _ = load_case(name)
    steps = int(re.search(r"Total Hydrosteps (\d+)", meta["reference_log_tail"]).group(1))
    assert len(dts) == steps
    for n, fields in snaps.items():
        for f in EVOLVED:
            ref = arrays[f"s{n}_{f}"]
            if meta.get("circular_bodies"):
                # the planet's position per step comes from its orbit, not
                # from REBOUND (they agree to ~1e-14): round-off, not bits
                assert rel_linf(fields[f], ref) <= 1e-12, (
                    f"{name} snapshot {n} {f}: rel Linf {rel_linf(fields[f], ref):.3e}")
            else:
                assert np.array_equal(fields[f], ref), (
                    f"{name} snapshot {n} {f}: rel Linf {rel_linf(fields[f], ref):.3e}")
    t_ref = arrays["body0_time"]
    for n, t in times.items():
        assert t == t_ref[n]
    if torques:
        tq = arrays["body1_torque"]
        for n, t in torques.items():
            if meta.get("circular_bodies"):
                # the torque is a sum with cancellation: the orbit-positioned
                # case is held to 1e-10 of the largest torque of the run
                assert abs(t - tq[n]) <= 1e-10 * np.max(np.abs(tq)), (n, t, tq[n])
            else:
                assert abs(t - tq[n]) <= 1e-12 * abs(tq[n]), (n, t, tq[n])


def test_step_counts_follow_cfl():
    # The CFL-limited cases take more hydro steps than monitor outputs; the
    # count is fixed by condition_cfl + CFLmaxVar + the monitor clamp.
    _, _, _, dts, _ = replay(OracleState, "iso_star_cfl")
    assert len(dts) == 22
    _, _, _, dts, _ = replay(OracleState, "adi_star_cfl_mc_std")
    assert len(dts) == 12
    # LeapFrog: the reference's own run logs report 22 and 32 hydro steps
    _, _, _, dts, _ = replay(OracleState, "iso_star_cfl_leapfrog")
    assert len(dts) == 22
    _, _, _, dts, _ = replay(OracleState, "adi_star_cfl_leapfrog")
    assert len(dts) == 32


@pytest.mark.parametrize("name", [c for c in CASES if "accretion" in c])
def test_oracle_accreted_mass_matches_reference_monitor(name):
    # The reference writes accreted mass / monitor interval as the planet's
    # accretion rate (nbody/planet.cpp:357-369).
    accreted = {}
    snaps, _, _, _, arrays = replay(OracleState, name, accreted=accreted)
    rate = arrays["body1_accretion_rate"]
    from golden_runner import load_case
    dt_mon = load_case(name)[0]["monitor_timestep"]
    assert len(accreted) == len(rate) - 1
    for n, m in accreted.items():
        assert m > 0
        assert abs(m / dt_mon - rate[n]) <= 1e-12 * rate[n], (n, m / dt_mon, rate[n])
    # and the accretion is visible in the fields
    plain, _, _, _, _ = replay(OracleState, name, {"accretion_radius_fraction": 0.0})
    last = max(snaps)
    assert rel_linf(plain[last]["SIGMA"], snaps[last]["SIGMA"]) > 1e-4


def test_oracle_quantities_match_reference_monitor():
    # Quantities.dat of the reference (output.cpp:326-470): gas mass and
    # angular momentum within QuantitiesRadiusLimit at every monitor output,
    # written with 17 significant digits; KeepDiskMassConstant holds the
    # mass within RMAX at its initial value (simulation.cpp:246-251).
    name = "adi_planet_keep_mass_nocorr"
    quantities = {}
    snaps, _, _, _, arrays = replay(OracleState, name, quantities=quantities)
    mon = arrays["quantities_monitor"]
    assert len(quantities) == len(mon)
    for row, n in enumerate(mon):
        m, l = quantities[int(n)]
        assert abs(m - arrays["quantities_mass"][row]) <= 1e-13 * abs(m), (n, m)
        assert abs(l - arrays["quantities_angular_momentum"][row]) <= 1e-13 * abs(l), (n, l)
    # the rescale is what keeps the mass: without it the fields differ
    plain, _, _, _, _ = replay(OracleState, name, {"keep_disk_mass_constant": 0})
    last = max(snaps)
    assert rel_linf(plain[last]["SIGMA"], snaps[last]["SIGMA"]) > 1e-12


def test_oracle_disk_force_selfgravity_correction_matters():
    # CorrectDiskSelfgravity off in the fixture: the torques match the
    # reference's above; with the correction on they differ
    _, _, tq_off, _, _ = replay(OracleState, "adi_planet_keep_mass_nocorr")
    _, _, tq_on, _, _ = replay(OracleState, "adi_planet_keep_mass_nocorr",
                               {"correct_disk_selfgravity": 1})
    n = max(tq_off)
    assert abs(tq_off[n] - tq_on[n]) > 1e-6 * abs(tq_off[n])
