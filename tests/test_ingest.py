""".bat ingest: the host reader (parallel positioned reads, column-blocked
transpose) and the device reader (records streamed up in chunks, transposed
by a kernel) give the columns read_BAT_frame + PARENT's scatter give
(io_binary.cpp:281-368, PARENT.cpp:443-473), for FP32 and FP64 files, with
chunk sizes that split the trajectory into many uneven pieces, and both
report a truncated body the way the reference does (an I/O error naming the
frame)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import parent_gb300 as pg
from conftest import FIXTURES, GOLDEN


def _host_cols(v) -> np.ndarray:
    n, F, prec = v.n_dihedrals, v.n_frames, v.double_prec
    ct = C.c_double if prec else C.c_float
    return np.ctypeslib.as_array(C.cast(v.bonds, C.POINTER(ct)), ((3 * n + 3) * v.ld,)).reshape(3 * n + 3, v.ld)[:, :F]


def _device_cols(v) -> np.ndarray:
    """Device columns copied back through torch (zero-copy wrap of the pointer)."""
    import torch
    n, F, prec = v.n_dihedrals, v.n_frames, v.double_prec

    class _Dev:
        __cuda_array_interface__ = {"shape": ((3 * n + 3) * v.ld,), "typestr": "<f8" if prec else "<f4",
                                    "data": (int(v.bonds), False), "version": 3}

    t = torch.as_tensor(_Dev(), device="cuda")
    return t.cpu().numpy().reshape(3 * n + 3, v.ld)[:, :F].copy()


def _synthetic_bat(tmp_path, n_atoms, F, prec, seed):
    t = pg.synth_host(n_atoms, F, double_prec=prec, seed=seed, frac_bimodal_dih=0.3)
    path = tmp_path / f"s{prec}.bat"
    pg.write_bat(path, t)
    return path, np.concatenate([t.bonds, t.angles, t.dihedrals])


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("chunk", [None, 1000, 70000])
def test_host_reader_chunked(tmp_path, monkeypatch, prec, chunk):
    path, want = _synthetic_bat(tmp_path, 23, 997, prec, 5 + prec)
    if chunk:
        monkeypatch.setenv("PG_BAT_CHUNK_BYTES", str(chunk))
    bat = pg.BatFile(path)
    got = _host_cols(bat.view())
    assert got.dtype == want.dtype and np.array_equal(got, want)


def test_host_reader_truncated_body(tmp_path):
    path, _ = _synthetic_bat(tmp_path, 10, 300, 0, 3)
    raw = path.read_bytes()
    path.write_bytes(raw[:-100])
    with pytest.raises(pg.PGError) as e:
        pg.BatFile(path)
    assert e.value.code == pg.PG_ERR_IO and "reading the file" in str(e.value)


def test_host_reader_bad_header(tmp_path):
    path, _ = _synthetic_bat(tmp_path, 10, 50, 0, 3)
    raw = bytearray(path.read_bytes())
    raw[4:8] = (7).to_bytes(4, "little")  # precision flag neither 0 nor 1
    path.write_bytes(bytes(raw))
    with pytest.raises(pg.PGError) as e:
        pg.BatFile(path)
    assert e.value.code == pg.PG_ERR_FORMAT


@pytest.mark.gpu
@pytest.mark.parametrize("stem", FIXTURES)
def test_device_reader_matches_host_reader_fixtures(stem):
    host = pg.BatFile(GOLDEN / f"{stem}.bat")
    dev = pg.BatFile(GOLDEN / f"{stem}.bat", device=0)
    hv, dv = host.view(), dev.view()
    assert dv.on_device == 1 and dv.ld % 32 == 0 and dv.ld >= dv.n_frames
    assert np.array_equal(_device_cols(dv), _host_cols(hv))
    with pg.Engine(0) as eng:
        a = eng.entropy(hv).flat()
        b = eng.entropy(dv).flat()
    assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("chunk", [None, 1, 50000])
def test_device_reader_chunked(tmp_path, monkeypatch, prec, chunk):
    """chunk=1 -> 32-frame chunks (the minimum): 32 chunks through the
    3-buffer staging ring, the last one ragged."""
    path, want = _synthetic_bat(tmp_path, 37, 1013, prec, 11 + prec)
    if chunk:
        monkeypatch.setenv("PG_BAT_CHUNK_BYTES", str(chunk))
    dev = pg.BatFile(path, device=0)
    got = _device_cols(dev.view())
    assert got.dtype == want.dtype and np.array_equal(got, want)


@pytest.mark.gpu
def test_device_reader_truncated_body(tmp_path, monkeypatch):
    path, _ = _synthetic_bat(tmp_path, 12, 500, 1, 4)
    raw = path.read_bytes()
    path.write_bytes(raw[: len(raw) - 3000])
    monkeypatch.setenv("PG_BAT_CHUNK_BYTES", "20000")
    with pytest.raises(pg.PGError) as e:
        pg.BatFile(path, device=0)
    assert e.value.code == pg.PG_ERR_IO and "reading the file" in str(e.value)
    # the device is still usable afterwards
    dev = pg.BatFile(GOLDEN / "synth_small.bat", device=0)
    assert dev.view().on_device == 1


@pytest.mark.gpu
def test_device_reader_allocation_failure(tmp_path):
    """Allocation failure injected through the input: an FP64 header that
    declares 2e9 frames of 24 DOFs (384 GB of columns, more than the GPU
    holds) makes the device allocation fail; the reader returns PG_ERR_NOMEM
    before reading the body, and the device keeps working."""
    import struct
    path, _ = _synthetic_bat(tmp_path, 10, 50, 1, 3)
    raw = bytearray(path.read_bytes())
    raw[12:16] = struct.pack("<i", 2_000_000_000)  # frames
    path.write_bytes(bytes(raw))
    with pytest.raises(pg.PGError) as e:
        pg.BatFile(path, device=0)
    assert e.value.code == pg.PG_ERR_NOMEM
    with pg.Engine(0) as eng:
        with pytest.raises(pg.PGError) as e2:
            big = C.c_void_p()
            pg._check(pg.lib().pg_device_alloc(eng.handle, 1 << 52, C.byref(big)), eng.handle)
        assert e2.value.code == pg.PG_ERR_NOMEM
        dev = pg.BatFile(GOLDEN / "synth_small.bat", device=0)
        body = eng.entropy(dev.view())
        assert np.isfinite(body.flat()).all()
