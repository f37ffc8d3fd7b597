"""CPU tests of host-side helpers added for device bodies and the bench:
DeviceParBody's block pointers follow the .par body layout, and bench.py's
histogram-layout choice and committed traffic figure agree with the library's
policy and the profile it names."""
from __future__ import annotations

import ctypes as C
import os
import sys
from pathlib import Path

import pytest

import parent_gb300 as pg

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("n_dih", [0, 1, 7, 100])
def test_device_par_body_pointers_follow_the_body_layout(n_dih):
    base = 1 << 40  # any address: only the offsets are checked
    c = pg.DeviceParBody(n_dih, base).c()
    off = 0
    for k, n in pg.block_sizes(n_dih).items():
        assert C.cast(getattr(c, k), C.c_void_p).value == base + 8 * off, k
        off += n


def test_bench_layout_policy_and_traffic(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    for k in ("PG_HIST_SLOTS", "PG_HIST_STREAM"):
        monkeypatch.delenv(k, raising=False)
    assert bench.hist_layout(50) == "stream32" and bench.hist_layout(30) == "stream32"
    assert bench.hist_layout(51) == "16"
    monkeypatch.setenv("PG_HIST_STREAM", "0")
    assert bench.hist_layout(30) == "ring32" and bench.hist_layout(50) == "16"
    monkeypatch.setenv("PG_HIST_SLOTS", "16")
    assert bench.hist_layout(30) == "16"
    bpu, name = bench.traffic_per_update("stream32")
    assert (ROOT / "profiles" / name).exists()
    assert bpu is not None and 0.0 < bpu < 1.0
