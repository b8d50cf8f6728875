"""The host split of constants into float pairs (split_pair_host,
fargocpt_gb300/csrc/hydro.cuh), which the float-pair kernels take in place
of splitting the same constants per thread, against a numpy restatement of
the device split's bit operations (f2_split, csrc/fp64_pair.cuh): hi is the
double truncated to its top 24 significant bits, lo the remaining 29 bits
rounded to a float and scaled; zero below 2^-74, NaN of the sign from 2^128.
Built with nvcc against the header as a host program (no GPU), on seeded
doubles across the range and on the edge cases; the pair must also hold the
double within 2^-48 of it."""
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def split_np(x):
    """f2_split's steps on the bit patterns (uint32 arithmetic wraps)."""
    b = np.frombuffer(np.float64(x).tobytes(), dtype=np.uint64)[0]
    w1, w0 = np.uint32(b >> np.uint64(32)), np.uint32(b & np.uint64(0xFFFFFFFF))
    ax, sign = w1 & np.uint32(0x7FFFFFFF), w1 & np.uint32(0x80000000)
    with np.errstate(over="ignore"):
        hi = np.uint32((int(ax) - (896 << 20)) & 0xFFFFFFFF)
        hb = np.uint32(((int(hi) << 3) & 0xFFFFFFFF) | (int(w0) >> 29))
        sb = np.uint32(((int(hb) & 0x7F800000) - (52 << 23)) & 0xFFFFFFFF)
    scale = np.frombuffer(sb.tobytes(), dtype=np.float32)[0]
    with np.errstate(over="ignore", invalid="ignore"):  # outside the range: replaced below
        lf = np.float32(np.float32(int(w0) & 0x1FFFFFFF) * scale)
    lb = np.frombuffer(lf.tobytes(), dtype=np.uint32)[0]
    inside = ((int(ax) - (949 << 20)) & 0xFFFFFFFF) < (202 << 20)
    out = 0 if int(ax) < (949 << 20) else (0x7FC00000 | int(sign))
    rh = (int(hb) | int(sign)) if inside else out
    rl = (int(lb) | int(sign)) if inside else out
    return rh, rl


def values():
    rng = np.random.default_rng(11)
    v = [float(x) for x in rng.uniform(-1.0, 1.0, 200) * 10.0 ** rng.integers(-30, 30, 200)]
    v += [1.0, -1.0, 0.5, 2.0 ** -74, -(2.0 ** -74) * 1.5, 2.0 ** -80, 2.0 ** 127 * 1.9,
          2.0 ** 128, 1.0 / 3.0, -2.0 / 3.0, 6.283185307179586, 1e-3, 0.0, -0.0]
    return v


def test_host_split_matches_the_device_bits(tmp_path):
    from fargocpt_gb300.build import nvcc

    try:
        cxx = nvcc()
    except RuntimeError:
        pytest.skip("needs nvcc")
    vals = values()
    src = tmp_path / "split.cu"
    body = "\n".join(f"    show({v!r});" for v in vals)
    src.write_text(f'''#include "hydro.cuh"
#include <cstdio>
#include <cstring>
static void show(double x)
{{
    const float2 p = fgpu::split_pair_host(x);
    unsigned h, l;
    std::memcpy(&h, &p.x, 4);
    std::memcpy(&l, &p.y, 4);
    std::printf("%u %u\\n", h, l);
}}
int main()
{{
{body}
    return 0;
}}
''')
    exe = tmp_path / "split"
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", os.path.join(REPO, "fargocpt_gb300", "csrc"), str(src), "-o",
                        str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for v, line in zip(vals, out):
        h, l = (int(s) for s in line.split())
        assert (h, l) == split_np(v), v
        hf = np.frombuffer(np.uint32(h).tobytes(), dtype=np.float32)[0]
        lf = np.frombuffer(np.uint32(l).tobytes(), dtype=np.float32)[0]
        a = abs(v)
        if 2.0 ** -74 <= a < 2.0 ** 128:
            assert abs(float(hf) + float(lf) - v) <= 2.0 ** -48 * a, v
        elif a < 2.0 ** -74:
            assert hf == 0.0 and lf == 0.0, v
        else:
            assert np.isnan(hf) and np.isnan(lf), v
