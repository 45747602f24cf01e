"""The device probes behind the roofline denominators (fg_probe_fp64_pipe, fg_probe_fp64, fg_probe_fp64_tensor,
fg_probe_fp64_lanes): they run, return finite positive rates and times, and are consistent with one another
(fg_probe_fp64 is twice the DFMA instruction rate; the mixed stream runs between the slowest and fastest single
operation; every lane variant runs the same DFMA chains, so its time lies within a factor 40 of the full warp's)."""
import math

import pytest

from flexi_gb300.solver import probe_fp64_lanes, probe_fp64_pipe, probe_fp64_tensor, probe_fp64_tflops

pytestmark = pytest.mark.gpu


def test_fp64_pipe_probe():
    r = probe_fp64_pipe()
    assert all(math.isfinite(v) and v > 0 for v in r.values()), r
    single = [r["dfma"], r["dadd"], r["dmul"]]
    assert 0.9 * min(single) <= r["mixed"] <= 1.1 * max(single), r
    t = probe_fp64_tflops()
    assert abs(t / (2 * r["dfma"]) - 1.0) < 0.1, (t, r)


def test_fp64_tensor_and_lane_probes():
    r = probe_fp64_tensor()
    assert all(math.isfinite(v) and v > 0 for v in r.values()), r
    ms = probe_fp64_lanes()
    assert set(ms) == {"32", "16", "8", "4", "1"}
    assert all(math.isfinite(v) and v > 0 for v in ms.values()), ms
    assert max(ms.values()) <= 40 * ms["32"], ms
