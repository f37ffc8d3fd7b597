"""The host readers of .bat and .par files (read_BAT_header/read_BAT_frame,
read_PAR_header/read_PAR_body: io_binary.cpp:107-368, :446-673) under damaged
inputs: random byte changes in the header, random truncations. Every case
either reads (a change in a field that is not checked, such as an atom name)
or fails with a PGError whose code is an I/O, format or data error; none may
crash the process or read past the file. Each case runs in a child process so
that a crash is reported as a failure instead of ending the test run."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"

_CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import parent_gb300 as pg
kind, paths = sys.argv[2], sys.argv[3:]
ok = err = 0
for p in paths:
    try:
        if kind == "bat":
            b = pg.BatFile(p)
            v = b.view()
            assert v.n_frames >= 0 and v.n_dihedrals >= 0
        else:
            pg.ParFile(p)
        ok += 1
    except pg.PGError as e:
        assert e.code in (pg.PG_ERR_IO, pg.PG_ERR_FORMAT, pg.PG_ERR_DATA, pg.PG_ERR_NOMEM, pg.PG_ERR_ARG), e.code
        err += 1
print(ok, err)
"""


def _mutants(src: Path, out_dir: Path, n: int, seed: int, header_bytes: int) -> list[Path]:
    raw = np.fromfile(src, dtype=np.uint8)
    rng = np.random.default_rng(seed)
    paths = []
    for k in range(n):
        m = raw.copy()
        if k % 4 == 3:
            m = m[: int(rng.integers(0, raw.size))]  # truncated anywhere
        else:
            for _ in range(int(rng.integers(1, 4))):  # 1-3 changed bytes in the header
                m[int(rng.integers(0, min(header_bytes, raw.size)))] = rng.integers(0, 256)
        p = out_dir / f"m{k}{src.suffix}"
        m.tofile(p)
        paths.append(p)
    return paths


def _run(kind: str, paths: list[Path]) -> tuple[int, int]:
    r = subprocess.run([sys.executable, "-c", _CHILD, str(ROOT), kind, *map(str, paths)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stderr[-3000:])
    ok, err = map(int, r.stdout.split()[-2:])
    return ok, err


def test_damaged_bat_headers(tmp_path):
    src = GOLDEN / "synth_small.bat"
    n_dih = int(np.fromfile(src, dtype=np.int32, count=3)[2])
    header = 16 + 55 * (n_dih + 3) + 24 * n_dih
    ok, err = _run("bat", _mutants(src, tmp_path, 160, 7, header))
    assert ok + err == 160 and err > 0


def test_damaged_par_headers(tmp_path):
    src = GOLDEN / "synth_small_ref.par"
    n_dih = int(np.fromfile(src, dtype=np.int32, count=3)[2])
    header = 40 + (n_dih + 3) * 51 + n_dih * 24 + (n_dih + 3) * 4
    ok, err = _run("par", _mutants(src, tmp_path, 160, 11, header))
    assert ok + err == 160 and err > 0
