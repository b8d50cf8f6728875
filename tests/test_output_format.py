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
