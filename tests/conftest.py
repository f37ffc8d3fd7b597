"""Shared pytest set-up: the `gpu` marker, an in-tree build of the native
library (no-op when up to date), and paths to the golden fixtures."""
from __future__ import annotations

import gzip
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from parent_gb300 import build as b
    b.build()
    b.build_oracle()
    yield


def read_text_gz(name: str) -> list[str]:
    with gzip.open(GOLDEN / name, "rt") as f:
        return f.read().splitlines()


def par_body_from_file(path: Path) -> tuple[int, dict]:
    """(n_dih, blocks) parsed with numpy straight from a .par (io_binary.cpp:446-673)."""
    import numpy as np
    raw = np.fromfile(path, dtype=np.uint8)
    hv = raw[:40].view(np.int32)
    n = int(hv[2])
    hdr = 40 + (n + 3) * 51 + n * 24 + (n + 3) * 4
    body = raw[hdr:].view(np.float64)
    nb, na, nd = n + 2, n + 1, n
    sizes = [("s1_b", nb), ("s1_a", na), ("s1_d", nd), ("bb", nb * (nb - 1) // 2), ("ba", nb * na),
             ("bd", nb * nd), ("aa", na * (na - 1) // 2), ("ad", na * nd), ("dd", nd * (nd - 1) // 2)]
    out, o = {}, 0
    for k, s in sizes:
        out[k] = body[o:o + s].copy()
        o += s
    assert o == body.size
    return n, out


FIXTURES = ["ubq_sub", "synth_small"]
