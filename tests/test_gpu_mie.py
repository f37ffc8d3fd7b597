"""MIE text with the pair lines formatted on the GPU
(pg_write_mie_text_device): byte-identical to the reference get_PAR_MIE.x's
output on the golden fixtures, and to the host writer on synthetic bodies
whose values span the formatter's range, leave it (tiny, huge, inf, nan:
those lines go to the C library) and hit the empty pair blocks of systems
without dihedrals."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import parent_gb300 as pg
from conftest import FIXTURES, GOLDEN, read_text_gz

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = pg.Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("stem", FIXTURES)
def test_device_mie_matches_reference(eng, stem, tmp_path):
    par = pg.ParFile(GOLDEN / f"{stem}_ref.par")
    out = tmp_path / "mie.txt"
    eng.write_mie_text(out, par.body)
    assert out.read_text().splitlines() == read_text_gz(f"{stem}_ref_MIE.txt.gz")


def _random_body(n_dih: int, seed: int, specials: bool) -> pg.ParBody:
    rng = np.random.default_rng(seed)
    b = pg.ParBody.empty(n_dih)
    for k, v in b.blocks.items():
        scale = 10.0 ** rng.uniform(-3, 4, v.size)
        v[:] = rng.normal(0, 1, v.size) * scale
    if specials:
        sp = [0.0, -0.0, 1e-30, -3e60, np.inf, np.nan, 1e-21, 9.9999999999995, 5e-324, 1e46, -1e-5]
        for k in ("bb", "ba", "dd"):
            v = b.blocks[k]
            n = min(v.size, len(sp))
            v[:n] = sp[:n]
        b.blocks["s1_b"][0] = 1e300
    return b


@pytest.mark.parametrize("n_dih,specials", [(300, False), (40, True), (0, False), (1, True), (2, False)])
def test_device_mie_matches_host_writer(eng, tmp_path, n_dih, specials):
    body = _random_body(n_dih, 7 + n_dih, specials)
    host, dev = tmp_path / "host.txt", tmp_path / "dev.txt"
    pg.write_mie_text(host, body)
    eng.write_mie_text(dev, body)
    assert dev.read_bytes() == host.read_bytes()


def test_mie_cli_device_default(tmp_path):
    r = subprocess.run([str(pg.BIN_DIR / "get_PAR_MIE_gb300"), str(GOLDEN / "ubq_sub_ref.par")],
                       capture_output=True, text=True, check=True, env=dict(os.environ))
    assert r.stdout.splitlines() == read_text_gz("ubq_sub_ref_MIE.txt.gz")
