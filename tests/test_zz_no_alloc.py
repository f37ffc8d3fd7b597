"""pg_mist_noalloc: the MIST entry point that allocates nothing.

Callers that own the whole device memory budget (a pre-allocated pool in the
host program) or that cannot accept an allocation's device-wide
synchronisation pass their own device buffers for the MI matrix and the edge
list; the kernel's scratch is a static device array inside the library. These
tests call it through the C ABI twice in a row and check each result against
pg_mist, the allocating entry point: on the two golden fixtures (the one-CTA
kernel with shared-memory arrays), on 1,194 DOFs (the cluster kernel, also
against the oracle), and on 16,383 then 12,903 DOFs with the cluster kernel
off, the only path whose per-DOF arrays live in the static array (the second
call starts on the first one's leftovers). Plus the size rejection. It sits in
its own file so that pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import parent_gb300 as pg
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MAX_DOFS = 16384


def _noalloc():
    f = pg.lib().pg_mist_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def dense_mi(n: int, body: pg.ParBody) -> np.ndarray:
    """D x D MI as get_mutual (util.cpp:47-81) forms it, same FP64 operation order."""
    b = body.blocks
    nb, na, nd = n + 2, n + 1, n
    D = nb + na + nd
    s1 = np.concatenate([b["s1_b"], b["s1_a"], b["s1_d"]])
    off = {0: 0, 1: nb, 2: nb + na}
    cnt = {0: nb, 1: na, 2: nd}
    M = np.zeros((D, D))
    for t, key in ((0, "bb"), (1, "aa"), (2, "dd")):
        m = cnt[t]
        if m < 2:
            continue
        i, j = np.triu_indices(m, 1)
        mi = s1[off[t] + i] + s1[off[t] + j] - b[key][::-1]
        M[off[t] + i, off[t] + j] = mi
        M[off[t] + j, off[t] + i] = mi
    for (t1, t2), key in (((0, 1), "ba"), ((0, 2), "bd"), ((1, 2), "ad")):
        if cnt[t2] == 0:
            continue
        i, j = np.meshgrid(np.arange(cnt[t1]), np.arange(cnt[t2]), indexing="ij")
        mi = (s1[off[t1] + i] + s1[off[t2] + j]).ravel() - b[key]
        M[off[t1] + i.ravel(), off[t2] + j.ravel()] = mi
        M[off[t2] + j.ravel(), off[t1] + i.ravel()] = mi
    return np.ascontiguousarray(M)


def run_noalloc(eng: pg.Engine, n: int, M: np.ndarray):
    D = M.shape[0]
    dm = eng.alloc(M.nbytes)          # the caller's own buffers
    dmi = eng.alloc(8 * (D - 1))
    dfrom = eng.alloc(4 * (D - 1))
    dto = eng.alloc(4 * (D - 1))
    try:
        eng.memcpy(dm, M.ctypes.data, M.nbytes, 1)
        eng.synchronize()
        rc = _noalloc()(n, dm, dmi, dfrom, dto, eng.stream())
        assert rc == pg.PG_OK, pg.lib().pg_last_global_error()
        mi = np.zeros(D - 1)
        fr = np.zeros(D - 1, dtype=np.int32)
        to = np.zeros(D - 1, dtype=np.int32)
        eng.memcpy(mi.ctypes.data, dmi, mi.nbytes, 2)
        eng.memcpy(fr.ctypes.data, dfrom, fr.nbytes, 2)
        eng.memcpy(to.ctypes.data, dto, to.nbytes, 2)
        eng.synchronize()
    finally:
        for p in (dm, dmi, dfrom, dto):
            eng.free(p)
    return mi, fr, to


def as_edges(n: int, mi, fr, to):
    nb, na = n + 2, n + 1
    t = lambda g: np.where(g < nb, 0, np.where(g < nb + na, 1, 2))
    off = lambda tt: np.where(tt == 0, 0, np.where(tt == 1, nb, nb + na))
    t1, t2 = t(fr), t(to)
    return t1, t2, fr - off(t1) + 1, to - off(t2) + 1, mi


def test_noalloc_matches_pg_mist_on_two_calls():
    with pg.Engine(0) as eng:
        for stem in ("ubq_sub", "synth_small"):
            par = pg.ParFile(GOLDEN / f"{stem}_ref.par")
            ref, _ = eng.mist(par.n_dih, par.body)
            t1, t2, i1, i2, mi = as_edges(par.n_dih, *run_noalloc(eng, par.n_dih, dense_mi(par.n_dih, par.body)))
            assert np.array_equal(t1, ref["t1"]) and np.array_equal(t2, ref["t2"])
            assert np.array_equal(i1, ref["i1"]) and np.array_equal(i2, ref["i2"])
            assert np.max(np.abs(mi - ref["mi"])) <= 1e-9


def dyadic_body(n: int, seed: int) -> pg.ParBody:
    """A random .par body on a grid of 1/64: sums of its values are exact, so
    many MI terms tie exactly and the reference's scan order decides."""
    rng = np.random.default_rng(seed)
    body = pg.ParBody.empty(n)
    for k, v in body.blocks.items():
        mu = 1.0 if k.startswith("s1") else 1.5
        v[:] = np.round(rng.normal(mu, 0.25, v.size) * 64.0) / 64.0
    return body


def check_against(eng, n, body, edges_fn):
    ref, _ = eng.mist(n, body)
    t1, t2, i1, i2, mi = edges_fn()
    assert np.array_equal(t1, ref["t1"]) and np.array_equal(t2, ref["t2"])
    assert np.array_equal(i1, ref["i1"]) and np.array_equal(i2, ref["i2"])
    assert np.array_equal(mi, ref["mi"])
    return ref


def test_noalloc_cluster_kernel_matches_pg_mist_and_the_oracle():
    # from 1,024 DOFs the eight-CTA cluster kernel runs (per-DOF arrays in
    # shared memory); 1,194 DOFs with many exact ties
    import oracle
    n = 397
    body = dyadic_body(n, 11)
    with pg.Engine(0) as eng:
        M = dense_mi(n, body)
        for _ in range(2):
            ref = check_against(eng, n, body, lambda: as_edges(n, *run_noalloc(eng, n, M)))
    oe, _ = oracle.mist(n, body.blocks)
    for f in ("t1", "t2", "i1", "i2"):
        assert np.array_equal(oe[f], ref[f]), f


def test_noalloc_static_array_path_on_two_calls(monkeypatch):
    # one CTA with the cluster kernel off: above 12,800 DOFs its per-DOF arrays
    # leave shared memory for the static array. Two calls in a row, the larger
    # first, so the second starts on the first one's leftover contents; each
    # equals pg_mist with the same setting (the same kernel on allocated
    # scratch) and pg_mist with the cluster kernel (another kernel, checked
    # against the oracle elsewhere).
    with pg.Engine(0) as eng:
        for n, seed in ((5460, 21), (4300, 22)):       # D = 16,383 and 12,903
            body = dyadic_body(n, seed)
            M = dense_mi(n, body)
            monkeypatch.setenv("PG_MIST_CLUSTER", "0")
            got = as_edges(n, *run_noalloc(eng, n, M))
            check_against(eng, n, body, lambda: got)
            monkeypatch.delenv("PG_MIST_CLUSTER")
            check_against(eng, n, body, lambda: got)
            del M


def test_noalloc_rejects_sizes_beyond_its_maximum():
    n = (MAX_DOFS - 3) // 3 + 1          # D = 3n + 3 > MAX_DOFS
    rc = _noalloc()(n, None, None, None, None, None)
    assert rc == pg.PG_ERR_UNSUPPORTED
    assert b"PG_NOALLOC_MAX_DOFS" in pg.lib().pg_last_global_error()
