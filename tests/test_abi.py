"""C-ABI library on the CPU: it loads, exports every function the header
declares, and its host-side file formats and text writers are byte-compatible
with the reference (io_binary.cpp, get_PAR_MIE/MIST/info). No GPU calls."""
from __future__ import annotations

import ctypes as C
import gzip
import struct

import numpy as np
import pytest

import parent_gb300 as pg
from conftest import FIXTURES, GOLDEN, par_body_from_file, read_text_gz


def test_library_exports_every_declared_symbol():
    L = pg.lib()
    names = pg.exported_symbols()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), n


@pytest.mark.parametrize("stem", FIXTURES)
def test_par_read_matches_numpy_parse(stem):
    p = pg.ParFile(GOLDEN / f"{stem}_ref.par")
    n, ref = par_body_from_file(GOLDEN / f"{stem}_ref.par")
    assert p.n_dih == n and p.bins == (50,) * 6
    for k in ref:
        assert np.array_equal(p.body.blocks[k], ref[k])


@pytest.mark.parametrize("stem", FIXTURES)
def test_par_write_is_byte_identical_to_reference(stem, tmp_path):
    """.par header copied from the .bat + body, as write_PAR_header/body."""
    bat = pg.BatFile(GOLDEN / f"{stem}.bat")
    ref = pg.ParFile(GOLDEN / f"{stem}_ref.par")
    out = tmp_path / "x.par"
    pg.write_par(out, bat, (50,) * 6, ref.body)
    assert out.read_bytes() == (GOLDEN / f"{stem}_ref.par").read_bytes()


@pytest.mark.parametrize("stem", FIXTURES)
def test_bat_read_columns_match_oracle(stem):
    import oracle
    n, F, prec, b, a, d = oracle.read_bat(GOLDEN / f"{stem}.bat")
    bat = pg.BatFile(GOLDEN / f"{stem}.bat")
    v = bat.view()
    assert (v.n_dihedrals, v.n_frames, v.double_prec) == (n, F, prec)
    dt = np.float64 if prec else np.float32
    cols = np.ctypeslib.as_array(C.cast(v.bonds, C.POINTER(C.c_double if prec else C.c_float)),
                                 ((3 * n + 3) * F,)).reshape(3 * n + 3, F)
    assert np.array_equal(cols.astype(np.float64), np.concatenate([b, a, d]))
    assert cols.dtype == dt


@pytest.mark.parametrize("stem", FIXTURES)
def test_text_writers_byte_identical(stem, tmp_path):
    p = pg.ParFile(GOLDEN / f"{stem}_ref.par")
    pg.write_mie_text(tmp_path / "mie.txt", p.body)
    assert (tmp_path / "mie.txt").read_text().splitlines() == read_text_gz(f"{stem}_ref_MIE.txt.gz")
    pg.write_info_text(tmp_path / "info.txt", p)
    assert (tmp_path / "info.txt").read_text().splitlines() == read_text_gz(f"{stem}_ref_info.txt.gz")


@pytest.mark.parametrize("stem", FIXTURES)
def test_mist_text_writer_matches_reference(stem, tmp_path):
    import oracle
    p = pg.ParFile(GOLDEN / f"{stem}_ref.par")
    edges, totals = oracle.mist(p.n_dih, p.body.blocks)
    pg.write_mist_text(tmp_path / "mist.txt", p.n_dih, edges, totals)
    assert (tmp_path / "mist.txt").read_text().splitlines() == read_text_gz(f"{stem}_ref_MIST.txt.gz")


def _bat_with_header(tmp_path, version=3, prec=1, ndih=1, frames=2, truncate=False):
    t = pg.synth_host(max(ndih, 1) + 3, max(frames, 1), double_prec=1, seed=3)
    path = tmp_path / "h.bat"
    pg.write_bat(path, t)
    raw = bytearray(path.read_bytes())
    raw[0:16] = struct.pack("<4i", version, prec, ndih, frames)
    if truncate:
        raw = raw[: len(raw) - 10]
    path.write_bytes(bytes(raw))
    return path


@pytest.mark.parametrize("kw,code", [
    (dict(version=-1), pg.PG_ERR_FORMAT),
    (dict(prec=2), pg.PG_ERR_FORMAT),
    (dict(ndih=-1), pg.PG_ERR_FORMAT),
    (dict(frames=0), pg.PG_ERR_FORMAT),
    (dict(truncate=True), pg.PG_ERR_IO),
])
def test_bat_header_checks(tmp_path, kw, code):
    """read_BAT_header's checks, io_binary.cpp:127-145 (plus a short file)."""
    path = _bat_with_header(tmp_path, **kw)
    with pytest.raises(pg.PGError) as e:
        pg.BatFile(path)
    assert e.value.code == code


@pytest.mark.parametrize("field,value", [(0, -1), (1, 3), (2, -4), (3, 0), (4, 0), (9, 0)])
def test_par_header_checks(tmp_path, field, value):
    """read_PAR_header's checks, io_binary.cpp:477-519."""
    raw = bytearray((GOLDEN / "synth_small_ref.par").read_bytes())
    struct.pack_into("<i", raw, 4 * field, value)
    path = tmp_path / "bad.par"
    path.write_bytes(bytes(raw))
    with pytest.raises(pg.PGError) as e:
        pg.ParFile(path)
    assert e.value.code == pg.PG_ERR_FORMAT


def test_par_dihedral_table_checks(tmp_path):
    """DIHEDRAL ID < 1 / type / parent checks, io_binary.cpp:558-591."""
    raw = bytearray((GOLDEN / "synth_small_ref.par").read_bytes())
    n = struct.unpack_from("<i", raw, 8)[0]
    off = 40 + (n + 3) * 51
    for k, bad in [(0, 0), (4, 2), (5, -2)]:
        r = bytearray(raw)
        struct.pack_into("<i", r, off + 4 * k, bad)
        path = tmp_path / f"d{k}.par"
        path.write_bytes(bytes(r))
        with pytest.raises(pg.PGError) as e:
            pg.ParFile(path)
        assert e.value.code == pg.PG_ERR_FORMAT


def test_missing_file_is_io_error(tmp_path):
    with pytest.raises(pg.PGError) as e:
        pg.BatFile(tmp_path / "nope.bat")
    assert e.value.code == pg.PG_ERR_IO


def test_cli_usage_errors():
    import subprocess
    for exe, args in [("PARENT_gb300", []), ("PARENT_gb300", ["a.xyz", "b.par"] + ["50"] * 6),
                      ("PARENT_gb300", ["a.bat", "b.par", "x"] + ["50"] * 5), ("get_PAR_MIST_gb300", ["a.par"])]:
        r = subprocess.run([str(pg.BIN_DIR / exe), *args], capture_output=True, text=True)
        assert r.returncode == 1 and ("USAGE" in r.stderr or "ERROR" in r.stderr)


def test_cli_host_formatters(tmp_path):
    """get_PAR_MIE (host writer) / get_PAR_info drop-ins need no GPU:
    byte-identical stdout."""
    import os
    import subprocess
    r = subprocess.run([str(pg.BIN_DIR / "get_PAR_MIE_gb300"), str(GOLDEN / "ubq_sub_ref.par")],
                       capture_output=True, text=True, check=True, env=dict(os.environ, PG_MIE_WRITER="host"))
    assert r.stdout.splitlines() == read_text_gz("ubq_sub_ref_MIE.txt.gz")
    r = subprocess.run([str(pg.BIN_DIR / "get_PAR_info_gb300"), str(GOLDEN / "ubq_sub_ref.par")],
                       capture_output=True, text=True, check=True)
    assert r.stdout.splitlines() == read_text_gz("ubq_sub_ref_info.txt.gz")


def test_engine_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pg.PGError) as e:
        pg.Engine(0)
    assert e.value.code in (pg.PG_ERR_CUDA, pg.PG_ERR_ARG)


def test_mie_text_many_rows_matches_python_formatting(tmp_path):
    """The MIE writer formats its lines on all host threads in row tasks; on a
    body large enough for many tasks every line equals a single-threaded
    %.12g rendering in the reference's order, and the totals match."""
    import numpy as np
    import oracle
    n = 150
    rng = np.random.default_rng(4)
    sizes = pg.block_sizes(n)
    blocks = {k: rng.normal(-3.0, 1.0, v) for k, v in sizes.items()}
    body = pg.ParBody(n, blocks)
    out = tmp_path / "mie.txt"
    pg.write_mie_text(out, body)
    lines = out.read_text().splitlines()
    nb, na, nd = n + 2, n + 1, n
    want = [f"bond {k + 1}   {blocks['s1_b'][k]:.12g}" for k in range(nb)]
    want += [f"angle {k + 1}   {blocks['s1_a'][k]:.12g}" for k in range(na)]
    want += [f"dihedral {k + 1}   {blocks['s1_d'][k]:.12g}" for k in range(nd)]
    specs = [("bond-bond ", "bb", "s1_b", "s1_b", nb, nb, True), ("bond-angle ", "ba", "s1_b", "s1_a", nb, na, False),
             ("bond-dihedral ", "bd", "s1_b", "s1_d", nb, nd, False), ("angle-angle ", "aa", "s1_a", "s1_a", na, na, True),
             ("angle-dihedral ", "ad", "s1_a", "s1_d", na, nd, False),
             ("dihedral-dihedral ", "dd", "s1_d", "s1_d", nd, nd, True)]
    for name, key, a1, a2, n1, n2, same in specs:
        arr = blocks[key]
        if same:
            i, j = np.triu_indices(n1, 1)
            s2 = arr[::-1]
        else:
            i, j = np.divmod(np.arange(n1 * n2), n2)
            s2 = arr
        mu = blocks[a1][i] + blocks[a2][j] - s2
        want += [f"{name}{a + 1}  {c + 1}   {x:.12g}   {y:.12g}" for a, c, x, y in zip(i, j, s2, mu)]
    assert len(lines) == len(want) + 16
    assert lines[:len(want)] == want
    tot = oracle.mie_totals(n, blocks)
    got_tot = np.array([float(ln.split(" = ")[1]) for ln in lines[len(want):]])
    assert np.array_equal(np.array([float(oracle.fmt12(x)) for x in tot]), got_tot)


def test_prefetch_entry_points_reject_a_null_context():
    """pg_prefetch and pg_entropy_ahead check their context before any CUDA
    call (CPU: no device needed)."""
    import ctypes as C
    v = pg.BatView()
    b = (C.c_int * 6)(*(50,) * 6)
    assert pg.lib().pg_prefetch(None, C.byref(v)) == pg.PG_ERR_ARG
    assert pg.lib().pg_entropy_ahead(None, C.byref(v), b, 0, None, C.byref(v)) == pg.PG_ERR_ARG
