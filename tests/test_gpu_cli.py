"""The drop-in CLIs end to end on the GPU, on the reference's own fixtures:
`PARENT_gb300 in.bat out.par b1D a1D d1D b2D a2D d2D` against the reference
`PARENT.x`'s `.par` (header bytes identical, every entropy within 1e-9 nats),
and `get_PAR_MIST_gb300` on the reference's `.par` against the reference
`get_PAR_MIST.x` text (identical bytes)."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import FIXTURES, GOLDEN, ROOT, par_body_from_file, read_text_gz

pytestmark = pytest.mark.gpu

BIN = ROOT / "parent_gb300" / "bin"


def _header_len(n_dih: int) -> int:
    # 10 ints, per-atom strings (8+4+8+31 B), dihedral table (6 ints), masses
    return 40 + (n_dih + 3) * 51 + n_dih * 24 + (n_dih + 3) * 4


@pytest.mark.parametrize("stem", FIXTURES)
def test_parent_cli_matches_reference_par(stem, tmp_path):
    out = tmp_path / f"{stem}.par"
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(GOLDEN / f"{stem}.bat"), str(out)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ref = GOLDEN / f"{stem}_ref.par"
    n, got = par_body_from_file(out)
    n_ref, want = par_body_from_file(ref)
    assert n == n_ref
    hl = _header_len(n)
    assert out.read_bytes()[:hl] == ref.read_bytes()[:hl]
    assert out.stat().st_size == ref.stat().st_size
    for k in want:
        if want[k].size:
            assert np.max(np.abs(got[k] - want[k])) <= 1e-9, k


@pytest.mark.parametrize("stem", FIXTURES)
def test_mist_cli_matches_reference_text(stem, tmp_path):
    out = tmp_path / f"{stem}_MIST.txt"
    r = subprocess.run([str(BIN / "get_PAR_MIST_gb300"), str(GOLDEN / f"{stem}_ref.par"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert out.read_text().splitlines() == read_text_gz(f"{stem}_ref_MIST.txt.gz")


def test_parent_cli_host_reader_same_par(tmp_path):
    """PG_BAT_READ=host (columns transposed on the host) writes the same .par
    as the default device reader."""
    import os
    a, b = tmp_path / "dev.par", tmp_path / "host.par"
    for out, env in ((a, dict(os.environ)), (b, dict(os.environ, PG_BAT_READ="host"))):
        r = subprocess.run([str(BIN / "PARENT_gb300"), str(GOLDEN / "ubq_sub.bat"), str(out)] + ["50"] * 6,
                           capture_output=True, text=True, timeout=300, env=env)
        assert r.returncode == 0, r.stderr
    assert a.read_bytes() == b.read_bytes()


def test_parent_cli_form_override(tmp_path):
    """PG_FORM=onehot runs the tensor-core form through the same CLI."""
    import os
    out = tmp_path / "o.par"
    env = dict(os.environ, PG_FORM="onehot")
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(GOLDEN / "synth_small.bat"), str(out)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    _, got = par_body_from_file(out)
    _, want = par_body_from_file(GOLDEN / "synth_small_ref.par")
    for k in want:
        if want[k].size:
            assert np.max(np.abs(got[k] - want[k])) <= 1e-9, k


def test_parent_cli_checkpoint_resume(tmp_path):
    """PG_SHARDS=4 with an interruption after two shards (exit code 3, a
    checkpoint left behind), then a rerun that resumes: the .par is
    byte-identical to a one-pass run and the checkpoint is removed."""
    import os
    bat = GOLDEN / "synth_small.bat"
    whole = tmp_path / "whole.par"
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(bat), str(whole)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "sharded.par"
    ckpt = tmp_path / "sharded.par.ckpt"
    env = dict(os.environ, PG_SHARDS="4", PG_STOP_AFTER_SHARDS="2")
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(bat), str(out)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 3, r.stdout + r.stderr
    assert ckpt.exists() and not out.exists()
    env = dict(os.environ, PG_SHARDS="4")
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(bat), str(out)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    assert "Resuming" in r.stdout and "2 of 4" in r.stdout
    assert not ckpt.exists()
    assert out.read_bytes() == whole.read_bytes()


def test_parent_cli_ignores_foreign_checkpoint(tmp_path):
    """A checkpoint written for other bin counts is not resumed from."""
    import os
    bat = GOLDEN / "synth_small.bat"
    out = tmp_path / "o.par"
    env = dict(os.environ, PG_SHARDS="3", PG_STOP_AFTER_SHARDS="1")
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(bat), str(out)] + ["40"] * 6,
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 3
    env = dict(os.environ, PG_SHARDS="3")
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(bat), str(out)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    assert "Resuming" not in r.stdout
    whole = tmp_path / "w.par"
    r = subprocess.run([str(BIN / "PARENT_gb300"), str(bat), str(whole)] + ["50"] * 6,
                       capture_output=True, text=True, timeout=300)
    assert out.read_bytes() == whole.read_bytes()
