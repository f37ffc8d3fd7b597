"""Cartesian -> BAT conversion (BAT_builder's per-frame conversion,
BAT_trajectory.cpp:114-125, :209-310) on the GPU.

The oracle's restatement is pinned bit-exactly to the reference BAT_builder's
own output: tests/golden/ubq_sub_xyz.npz holds the Cartesian coordinates
(decoded from the reference's ubiquitin .xtc by its xdrfile library) of the
atoms that the first 30 dihedrals of ubq_sub.bat use, and converting them
reproduces ubq_sub.bat exactly. The GPU conversion is then compared with the
oracle (bonds bit-exact; angles and dihedrals within a few ulp, as CUDA's
acos/atan2 are not glibc's) and, end to end, its entropies with the
reference PARENT.x's .par of the same system."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import parent_gb300 as pg
from conftest import GOLDEN, par_body_from_file

TWO_PI = 2 * np.pi


def _fixture():
    z = np.load(GOLDEN / "ubq_sub_xyz.npz")
    return z["xyz"], z["dih"]


def _chain(n_atoms: int, F: int, seed: int):
    """A jittering random chain (nm) and a linear-chain dihedral table whose
    parents point backwards and forwards (the in-place phase-angle order)."""
    rng = np.random.default_rng(seed)
    steps = rng.normal(size=(n_atoms, 3))
    steps /= np.linalg.norm(steps, axis=1, keepdims=True)
    base = np.cumsum(0.15 * steps, axis=0)
    xyz = (base[None] + 0.01 * rng.normal(size=(F, n_atoms, 3))).astype(np.float32)
    nd = n_atoms - 3
    dih = np.zeros((nd, 6), np.int32)
    for i in range(nd):
        dih[i, :4] = [i + 1, i + 2, i + 3, i + 4]
        dih[i, 5] = -1
        if i % 3 == 1:
            dih[i, 5] = i          # the previous dihedral (1-based)
        elif i % 5 == 2 and i + 2 < nd:
            dih[i, 5] = i + 3      # a later one, still raw when read
    return xyz, dih


def _cols(v):
    from test_ingest import _device_cols
    c = _device_cols(v)
    n = v.n_dihedrals
    return c[: n + 2], c[n + 2: 2 * n + 3], c[2 * n + 3:]


def _angle_close(a, b, tol):
    d = np.abs(a - b)
    return np.all(np.minimum(d, np.abs(d - TWO_PI)) <= tol)


def test_oracle_reproduces_reference_bat_builder():
    xyz, dih = _fixture()
    b, a, d = oracle.bat_from_xyz(xyz, dih)
    n, F, prec, rb, ra, rd = oracle.read_bat(GOLDEN / "ubq_sub.bat")
    assert (n, F, prec) == (dih.shape[0], xyz.shape[0], 1)
    assert np.array_equal(b, rb) and np.array_equal(a, ra) and np.array_equal(d, rd)


def test_bat_dihedral_table_accessor():
    """pg_bat_dihedral_table returns the header table the conversion takes:
    the fixture's subset table maps back onto ubq_sub.bat's own atoms."""
    bat = pg.BatFile(GOLDEN / "ubq_sub.bat")
    tab = bat.dihedral_table()
    assert tab.shape == (30, 6) and tab.dtype == np.int32
    _, dih = _fixture()
    assert np.array_equal(tab[:, 4:], dih[:, 4:])  # types and parents (atoms are renumbered in the fixture)
    assert (tab[:, :4] >= 1).all()


def test_oracle_rejects_bad_tables():
    xyz, dih = _fixture()
    bad = dih.copy()
    bad[3, 2] = xyz.shape[1] + 1
    with pytest.raises(ValueError):
        oracle.bat_from_xyz(xyz, bad)
    bad = dih.copy()
    bad[4, 5] = dih.shape[0] + 1
    with pytest.raises(ValueError):
        oracle.bat_from_xyz(xyz, bad)


@pytest.mark.gpu
def test_gpu_conversion_matches_oracle_ubq():
    xyz, dih = _fixture()
    want = oracle.bat_from_xyz(xyz, dih)
    with pg.Engine(0) as eng:
        v = eng.bat_from_cartesian(xyz, dih, double_prec=1)
        assert v.on_device == 1 and v.n_dihedrals == dih.shape[0] and v.n_frames == xyz.shape[0]
        got = _cols(v)
    assert np.array_equal(got[0], want[0])                      # bonds: sqrt and divisions are IEEE
    assert np.allclose(got[1], want[1], rtol=0, atol=1e-13)     # angles: acos
    assert _angle_close(got[2], want[2], 1e-12)                 # dihedrals: atan2, phase, shift


@pytest.mark.gpu
def test_gpu_conversion_entropies_match_reference_par():
    """xtc coordinates -> BAT (GPU) -> entropies (GPU) equals the reference
    pipeline BAT_builder.x -> PARENT.x on the same system."""
    xyz, dih = _fixture()
    with pg.Engine(0) as eng:
        v = eng.bat_from_cartesian(xyz, dih, double_prec=1)
        body = eng.entropy(v, (50,) * 6)
    _, want = par_body_from_file(GOLDEN / "ubq_sub_ref.par")
    for k in want:
        if want[k].size:
            assert np.max(np.abs(body.blocks[k] - want[k])) <= 1e-9, k


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [1, 0])
def test_gpu_conversion_synthetic_chunks(prec):
    """70,000 frames: two chunks (65,536 + a ragged 4,464); parents before and
    after their dihedral; FP32 output rounds the FP64 values as the .bat writer
    does (io_binary.cpp:238-271)."""
    xyz, dih = _chain(23, 70000, seed=3 + prec)
    want = oracle.bat_from_xyz(xyz, dih)
    with pg.Engine(0) as eng:
        got = _cols(eng.bat_from_cartesian(xyz, dih, double_prec=prec))
    if prec:
        assert np.array_equal(got[0], want[0])
        assert np.allclose(got[1], want[1], rtol=0, atol=1e-13)
        assert _angle_close(got[2], want[2], 1e-12)
    else:
        assert got[0].dtype == np.float32
        assert np.array_equal(got[0], want[0].astype(np.float32))
        for g, w in ((got[1], want[1]), (got[2], want[2])):
            w32 = w.astype(np.float32)
            ulp = np.abs(np.spacing(w32))
            d = np.abs(g.astype(np.float64) - w32.astype(np.float64))
            d = np.minimum(d, np.abs(d - TWO_PI))
            assert np.all(d <= ulp * 1.0001 + 1e-7)
            assert np.mean(g == w32) > 0.999


@pytest.mark.gpu
def test_gpu_conversion_rejects_bad_tables():
    xyz, dih = _fixture()
    bad = dih.copy()
    bad[0, 0] = 0
    with pg.Engine(0) as eng:
        with pytest.raises(pg.PGError) as e:
            eng.bat_from_cartesian(xyz, bad)
        assert e.value.code == pg.PG_ERR_ARG
        bad = dih.copy()
        bad[2, 5] = 999
        with pytest.raises(pg.PGError):
            eng.bat_from_cartesian(xyz, bad)
        v = eng.bat_from_cartesian(xyz, dih)  # the context is still usable
        assert v.on_device == 1


@pytest.mark.gpu
def test_gpu_conversion_from_device_coordinates():
    """xyz_on_device = 1: coordinates already in device memory give the same
    columns as the host-array call."""
    import ctypes as C

    import torch
    xyz, dih = _chain(31, 5000, seed=9)
    with pg.Engine(0) as eng:
        want = [c.copy() for c in _cols(eng.bat_from_cartesian(xyz, dih, double_prec=1))]
        dx = torch.from_numpy(xyz).cuda().contiguous()
        torch.cuda.synchronize()
        v = pg.BatView()
        d = np.ascontiguousarray(dih, dtype=np.int32)
        rc = pg.lib().pg_bat_from_cartesian(eng.handle, C.c_void_p(dx.data_ptr()), 1, xyz.shape[0], dih.shape[0],
                                            d.ctypes.data_as(C.POINTER(C.c_int)), 1, C.byref(v))
        assert rc == pg.PG_OK
        got = _cols(v)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
