"""ORACLE — test infrastructure only.

ctypes access to oracle/liboracle.so, the plain-C restatement of the
reference PARENT algorithm (oracle/parent_oracle.c), and to the reference
programs compiled from their own sources into oracle/_ref/ when this machine
has them. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg import this module, and only to check results or as the timed CPU reference;
the product (parent_gb300) never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF = HERE / "_ref"

_lib = None


def reference_root() -> Path:
    """Where the reference project's sources are (PG_REFERENCE_ROOT, else the
    oracle build recipe's REF_ROOT); the directory may not exist."""
    env = os.environ.get("PG_REFERENCE_ROOT")
    if env:
        return Path(env)
    r = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref-root"], capture_output=True, text=True)
    return Path(r.stdout.strip() or ".") if r.returncode == 0 else Path(".")


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        dp, ip, i, d = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int, C.c_double
        L.or_read_bat.argtypes = [C.c_char_p, ip, ip, ip, C.POINTER(dp), C.POINTER(dp), C.POINTER(dp)]
        L.or_free.argtypes = [C.c_void_p]
        L.or_extrema.argtypes = [i, i, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_entropy1d.restype = d
        L.or_entropy1d.argtypes = [i, dp, i, d, d, i, ip]
        L.or_entropy2d.restype = d
        L.or_entropy2d.argtypes = [i, dp, d, d, i, i, dp, d, d, i, i, C.POINTER(C.c_int64), ip]
        L.or_parent.argtypes = [i, i, dp, dp, dp, ip] + [dp] * 9
        L.or_mutual.restype = d
        L.or_mutual.argtypes = [i, i, i, i] + [dp] * 9
        L.or_mie_totals.argtypes = [i] + [dp] * 9 + [dp]
        L.or_mist.argtypes = [i] + [dp] * 9 + [ip, ip, ip, ip, dp, ip, dp]
        L.or_mist_gap.argtypes = [i] + [dp] * 9 + [ip, ip, ip, ip, dp, ip, dp, dp]
        L.or_sample.argtypes = [i, i, i, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, ip, i, ip, ip,
                                dp, dp, i, C.POINTER(C.c_int64), C.c_longlong, dp, dp, dp]
        L.or_bat_from_xyz.argtypes = [i, i, C.POINTER(C.c_float), ip, dp, dp, dp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


BLOCKS = ("s1_b", "s1_a", "s1_d", "bb", "ba", "bd", "aa", "ad", "dd")


def sizes(n_dih: int) -> dict:
    nb, na, nd = n_dih + 2, n_dih + 1, n_dih
    return dict(s1_b=nb, s1_a=na, s1_d=nd, bb=nb * (nb - 1) // 2, ba=nb * na, bd=nb * nd,
                aa=na * (na - 1) // 2, ad=na * nd, dd=nd * (nd - 1) // 2)


def _cols64(bonds, angles, dihedrals):
    b, a, d = [np.ascontiguousarray(x, dtype=np.float64).copy() for x in (bonds, angles, dihedrals)]
    nd = d.shape[0]
    if b.ndim != 2 or a.ndim != 2 or d.ndim != 2 or b.shape[0] != nd + 2 or a.shape[0] != nd + 1 \
            or not (b.shape[1] == a.shape[1] == d.shape[1]):
        raise ValueError(f"need (nDih+2, F), (nDih+1, F), (nDih, F) columns, got {b.shape}, {a.shape}, {d.shape}")
    return [b, a, d]


def read_bat(path) -> tuple:
    """(n_dih, F, double_prec, bonds, angles, dihedrals) as FP64 DOF-major arrays."""
    L = lib()
    nd, F, prec = C.c_int(), C.c_int(), C.c_int()
    pb, pa, pd = C.POINTER(C.c_double)(), C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
    rc = L.or_read_bat(str(path).encode(), C.byref(nd), C.byref(F), C.byref(prec), C.byref(pb), C.byref(pa), C.byref(pd))
    if rc:
        raise RuntimeError(f"oracle could not read {path}")
    n, f = nd.value, F.value
    out = []
    for ptr, rows in ((pb, n + 2), (pa, n + 1), (pd, n)):
        out.append(np.ctypeslib.as_array(ptr, (max(rows, 1) * f,))[: rows * f].reshape(rows, f).copy())
        L.or_free(ptr)
    return n, f, prec.value, out[0], out[1], out[2]


def extrema(bonds, angles, dihedrals):
    """(min, max, modfit, shifted dihedrals, bad) in global DOF order."""
    b, a, d = _cols64(bonds, angles, dihedrals)
    nd, F = d.shape[0], b.shape[1]
    mn = [np.zeros(x.shape[0]) for x in (b, a, d)]
    mx = [np.zeros(x.shape[0]) for x in (b, a, d)]
    mf = np.zeros(max(nd, 1))
    bad = lib().or_extrema(nd, F, _p(b), _p(a), _p(d), _p(mn[0]), _p(mx[0]), _p(mn[1]), _p(mx[1]),
                           _p(mn[2]), _p(mx[2]), _p(mf))
    return np.concatenate(mn), np.concatenate(mx), np.concatenate([np.zeros(b.shape[0] + a.shape[0]), mf[:nd]]), d, bad


def parent(bonds, angles, dihedrals, bins=(50,) * 6) -> dict:
    """The whole PARENT.x computation; returns the .par body blocks (FP64)."""
    b, a, d = _cols64(bonds, angles, dihedrals)
    nd, F = d.shape[0], b.shape[1]
    out = {k: np.zeros(n) for k, n in sizes(nd).items()}
    bb = (C.c_int * 6)(*bins)
    rc = lib().or_parent(nd, F, _p(b), _p(a), _p(d), bb, *[_p(out[k]) for k in BLOCKS])
    if rc:
        raise RuntimeError(f"oracle rejected the input (code {rc})")
    return out


def pair_counts(bonds, angles, dihedrals, bins, pairs) -> list:
    """Reference 2D counts (int64, B1 x B2) of global DOF pairs (g1 < g2)."""
    b, a, d = _cols64(bonds, angles, dihedrals)
    nd, F = d.shape[0], b.shape[1]
    nb, na = nd + 2, nd + 1
    mn, mx, _, dsh, bad = extrema(b, a, d)
    cols = np.concatenate([b, a, dsh], axis=0)
    res = []
    for g1, g2 in pairs:
        t1 = 0 if g1 < nb else (1 if g1 < nb + na else 2)
        t2 = 0 if g2 < nb else (1 if g2 < nb + na else 2)
        B1, B2 = bins[3 + t1], bins[3 + t2]
        cnt = np.zeros(B1 * B2, dtype=np.int64)
        x = np.ascontiguousarray(cols[g1])
        y = np.ascontiguousarray(cols[g2])
        badi = C.c_int(0)
        lib().or_entropy2d(t1, _p(x), mn[g1], mx[g1], B1, t2, _p(y), mn[g2], mx[g2], B2, F,
                           cnt.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(badi))
        res.append(cnt.reshape(B1, B2))
    return res


def mie_totals(n_dih: int, body: dict) -> np.ndarray:
    t = np.zeros(16)
    lib().or_mie_totals(n_dih, *[_p(np.ascontiguousarray(body[k], dtype=np.float64)) for k in BLOCKS], _p(t))
    return t


def mist(n_dih: int, body: dict, gaps: bool = False):
    """(edges structured array, totals[10]) with the reference's one-thread scan
    order; with gaps=True also each step's gap between the winning MI and the
    largest other candidate (0 where the scan order decided among equal values)."""
    n = 3 * n_dih + 2
    t1, t2, i1, i2, left = (np.zeros(max(n, 1), dtype=np.int32) for _ in range(5))
    mi = np.zeros(max(n, 1))
    gap = np.zeros(max(n, 1))
    tot = np.zeros(10)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    lib().or_mist_gap(n_dih, *[_p(np.ascontiguousarray(body[k], dtype=np.float64)) for k in BLOCKS],
                      ip(t1), ip(t2), ip(i1), ip(i2), _p(mi), ip(left), _p(gap), _p(tot))
    arr = np.zeros(n, dtype=[("t1", "i4"), ("t2", "i4"), ("i1", "i4"), ("i2", "i4"), ("mi", "f8"), ("left", "i4")])
    arr["t1"], arr["t2"], arr["i1"], arr["i2"], arr["mi"], arr["left"] = t1[:n], t2[:n], i1[:n], i2[:n], mi[:n], left[:n]
    if gaps:
        return arr, tot, gap[:n]
    return arr, tot


def sample(bonds, angles, dihedrals, bins, g1, g2, n_counts: int = 0):
    """The oracle at full size on a sample of pairs, without an FP64 copy of the
    trajectory: per-DOF (s1, min, max, modfit) for every DOF and the 2D entropy
    (and, for the first n_counts pairs, the B1 x B2 int64 counts) of each pair
    g1[k] < g2[k] (global DOF indices). Columns: 2D arrays (rows = DOFs of one
    type), float32 or float64, C-contiguous, frames along axis 1."""
    cols = [np.asarray(x) for x in (bonds, angles, dihedrals)]
    dt = cols[0].dtype
    if dt not in (np.float32, np.float64) or any(c.dtype != dt or not c.flags.c_contiguous for c in cols):
        raise ValueError("columns must be C-contiguous float32 or float64 of one dtype")
    nd = cols[2].shape[0]
    F = cols[0].shape[1]
    D = 3 * nd + 3
    g1 = np.ascontiguousarray(g1, dtype=np.int32)
    g2 = np.ascontiguousarray(g2, dtype=np.int32)
    s1, mn, mx, mf = (np.zeros(D) for _ in range(4))
    s2 = np.zeros(max(len(g1), 1))
    bmax = max(bins[3:])
    cnt = np.zeros((max(n_counts, 1), bmax * bmax), dtype=np.int64)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    # an empty dihedral block still needs a valid pointer
    dptr = cols[2].ctypes.data if nd > 0 else cols[1].ctypes.data
    rc = lib().or_sample(nd, F, 1 if dt == np.float64 else 0, cols[0].ctypes.data, cols[1].ctypes.data, dptr,
                         F, ip(np.ascontiguousarray(bins, dtype=np.int32)), len(g1), ip(g1), ip(g2), _p(s1),
                         _p(s2), n_counts, cnt.ctypes.data_as(C.POINTER(C.c_int64)), bmax * bmax,
                         _p(mn), _p(mx), _p(mf))
    if rc:
        raise RuntimeError(f"oracle rejected the input (code {rc})")
    counts = []
    for k in range(n_counts):
        t1 = 0 if g1[k] < nd + 2 else (1 if g1[k] < 2 * nd + 3 else 2)
        t2 = 0 if g2[k] < nd + 2 else (1 if g2[k] < 2 * nd + 3 else 2)
        B1, B2 = bins[3 + t1], bins[3 + t2]
        counts.append(cnt[k, :B1 * B2].reshape(B1, B2).copy())
    return {"s1": s1, "s2": s2[:len(g1)], "min": mn, "max": mx, "modfit": mf, "counts": counts}


def fmt12(x: float) -> str:
    """C++ ostream precision(12) formatting of a double."""
    return "%.12g" % x


def ref_available() -> bool:
    return (REF / "PARENT.x").exists()


def bat_from_xyz(xyz: np.ndarray, dih: np.ndarray):
    """Cartesian (F, nDih+3, 3) float32 in nm + the .bat dihedral table
    (nDih, 6) -> FP64 columns (bonds, angles, dihedrals), as BAT_builder."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    dih = np.ascontiguousarray(dih, dtype=np.int32)
    nf, na, _ = xyz.shape
    nd = dih.shape[0]
    assert na == nd + 3
    b = np.empty((nd + 2, nf)); a = np.empty((nd + 1, nf)); d = np.empty((nd, nf))
    rc = lib().or_bat_from_xyz(nd, nf, xyz.ctypes.data_as(C.POINTER(C.c_float)),
                               dih.ctypes.data_as(C.POINTER(C.c_int)), _p(b), _p(a), _p(d))
    if rc:
        raise ValueError(f"or_bat_from_xyz: bad dihedral table ({rc})")
    return b, a, d
