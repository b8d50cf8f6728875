"""FargoCPT's snapshot file formats as fargocpt_gb300.output writes them
(no GPU): misc.bin is struct misc_entry (src/output.h:16-24), 48 bytes with
the offsets a C compiler gives it; grids are raw little-endian FP64 rows."""
import struct

import numpy as np

from fargocpt_gb300 import output


def test_misc_entry_layout(tmp_path):
    p = str(tmp_path / "misc.bin")
    output.write_misc(p, snapshot=7, monitor=70, time=1.25, last_dt=3.5e-3, n_iter=12345,
                      omega_frame=0.5, frame_angle=0.25)
    raw = open(p, "rb").read()
    assert len(raw) == 48
    assert struct.unpack_from("<I", raw, 0)[0] == 7
    assert struct.unpack_from("<I", raw, 4)[0] == 70
    assert struct.unpack_from("<d", raw, 8)[0] == 1.25
    assert struct.unpack_from("<d", raw, 16)[0] == 0.5
    assert struct.unpack_from("<d", raw, 24)[0] == 0.25
    assert struct.unpack_from("<d", raw, 32)[0] == 3.5e-3
    assert struct.unpack_from("<Q", raw, 40)[0] == 12345
    assert output.read_misc(p)["n_iter"] == 12345


def test_grid_round_trip(tmp_path):
    a = np.random.default_rng(0).random((9, 12))
    p = str(tmp_path / "Sigma.dat")
    output.write_grid(p, a)
    assert (tmp_path / "Sigma.dat").stat().st_size == a.size * 8
    assert np.array_equal(output.read_grid(p, 12), a)


def _reference_bytes(arrays, n, field):
    # the fixture holds the reference's <name>.dat as read with '<f8'
    return np.ascontiguousarray(arrays[f"s{n}_{field}"], dtype="<f8").tobytes()


def test_oracle_snapshot_files_equal_the_references(tmp_path):
    # A reference case replayed on the oracle (which reproduces the
    # reference bit for bit) and written with fargocpt_gb300.output at every
    # kept snapshot gives files byte-identical to the ones the reference
    # wrote: Sigma.dat, vrad.dat, vazi.dat, energy.dat and misc.bin
    # (polargrid.cpp:135-180, output.cpp:494-527).
    from golden_runner import replay
    from oracle.oracle_py import OracleState

    written = {}

    def on_snapshot(hyd, n, clock):
        d = tmp_path / str(n)
        d.mkdir()
        for f in ("SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY"):
            output.write_grid(str(d / (output.GRID_NAMES[f] + ".dat")), hyd.get_field(f))
        output.write_misc(str(d / "misc.bin"), snapshot=n, monitor=n, time=clock.time,
                          last_dt=clock.last_dt, n_iter=clock.n_hydro_iter)
        written[n] = d

    for name in ("adi_planet_fixed_dt", "adi_star_cfl_mc_std"):
        written.clear()
        _, _, _, _, arrays = replay(OracleState, name, on_snapshot=on_snapshot)
        assert set(written) == set(int(k) for k in arrays["keep"])
        for n, d in written.items():
            for f in ("SIGMA", "V_RADIAL", "V_AZIMUTHAL", "ENERGY"):
                got = (d / (output.GRID_NAMES[f] + ".dat")).read_bytes()
                assert got == _reference_bytes(arrays, n, f), (name, n, f)
            assert (d / "misc.bin").read_bytes() == arrays[f"s{n}_misc"].tobytes(), (name, n)
        for d in written.values():
            for p in d.iterdir():
                p.unlink()
            d.rmdir()
