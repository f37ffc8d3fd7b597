"""GPU parity of the batched entry point (pg_entropy_batch): many independent
trajectories in one run give, system by system, the same .par body and MIST
tree as the oracle and as one pg_entropy + pg_mist call per system, and a
replayed CUDA graph gives the same results as its first capture."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
import parent_gb300 as pg
from test_gpu_parity import compare_bodies, compare_mist

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    e = pg.Engine(0)
    yield e
    e.close()


# (n_atoms, frames, double precision): ragged sizes, both precisions, a
# system without dihedrals and a one-frame system
SYSTEMS = [(40, 12345, 0), (3, 777, 1), (25, 3000, 1), (60, 20000, 0), (4, 1, 1), (17, 4096, 0)]


def _systems(spec, seed0=11):
    return [pg.synth_host(a, f, double_prec=p, seed=seed0 + k, frac_bimodal_dih=0.2, frac_bimodal_bond=0.05)
            for k, (a, f, p) in enumerate(spec)]


def _check_against_oracle(trajs, bodies, trees, bins):
    for t, body, (e, tot) in zip(trajs, bodies, trees):
        ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
        compare_bodies(t.n_dih, body, ref)
        re, rt = oracle.mist(t.n_dih, ref)
        if np.max(np.abs(re["mi"]), initial=0.0) <= 1e-9:
            # one frame: every MI is 0 and the tree order is rounding noise
            assert np.max(np.abs(e["mi"]), initial=0.0) <= 1e-9
            continue
        compare_mist(e, tot, re, rt)


@pytest.mark.parametrize("bins", [(50,) * 6, (7, 64, 100, 10, 20, 30), (50, 50, 50, 100, 100, 100)])
def test_batch_matches_oracle(eng, bins):
    trajs = _systems(SYSTEMS)
    bodies, trees = eng.entropy_batch(trajs, bins)
    assert len(bodies) == len(trajs) and len(trees) == len(trajs)
    _check_against_oracle(trajs, bodies, trees, bins)


@pytest.mark.parametrize("slots", ["16", "32", "stream"])
def test_batch_both_histogram_layouts_at_50_bins(eng, monkeypatch, slots):
    """At 50 bins the batch runs the 32-slot layout with 16-bit counters (row
    codes written per system), streamed from each system's interleaved bin
    matrices or ring-fed, or the 16-slot layout."""
    if slots == "stream":
        monkeypatch.setenv("PG_HIST_STREAM", "1")
    else:
        monkeypatch.setenv("PG_HIST_SLOTS", slots)
    bins = (50, 50, 50, 50, 47, 39)
    # not the one-frame system: its MI values are rounding noise around 0,
    # so its tree order is not defined by the data
    trajs = _systems([s for s in SYSTEMS if s[1] > 1], seed0=21)
    bodies, trees = eng.entropy_batch(trajs, bins)
    _check_against_oracle(trajs, bodies, trees, bins)


def test_batch_at_10_bins_takes_the_onehot_form(eng):
    """At 10 bins the autotuner picks the one-hot form for every system with
    at least 4,096 frames: the batch runs every system's tiles in one
    tensor-core launch; bodies and trees equal the oracle's and the single
    one-hot calls' (bit for bit: each system keeps its own n ln n table)."""
    bins = (10,) * 6
    spec = [(40, 12345, 0), (25, 5000, 1), (60, 20000, 0), (17, 4096, 0)]
    trajs = _systems(spec, seed0=31)
    bodies, trees = eng.entropy_batch(trajs, bins)
    assert eng.last_form() == "onehot"
    _check_against_oracle(trajs, bodies, trees, bins)
    for t, b, (e, tot) in zip(trajs, bodies, trees):
        single = eng.entropy(t, bins, "onehot")
        assert np.array_equal(b.flat(), single.flat())


@pytest.mark.parametrize("pair", ["1", "0"])
def test_batch_onehot_form_on_ragged_systems(eng, monkeypatch, pair):
    """The batched one-hot launch forced on ragged systems (no dihedrals, one
    frame, FP64 and FP32, per-type bin counts), on CTA pairs and on single
    CTAs: the oracle's bodies and trees, the single calls' bodies bit for
    bit, and a replayed graph gives the same results."""
    monkeypatch.setenv("PG_ONEHOT_PAIR", pair)
    bins = (10, 12, 9, 10, 12, 9)
    trajs = _systems(SYSTEMS, seed0=91)
    bodies, trees = eng.entropy_batch(trajs, bins, form="onehot")
    assert eng.last_form() == "onehot"
    _check_against_oracle(trajs, bodies, trees, bins)
    again = eng.entropy_batch(trajs, bins, form="onehot")
    for t, b, b2 in zip(trajs, bodies, again[0]):
        assert np.array_equal(b.flat(), b2.flat())
        single = eng.entropy(t, bins, "onehot")
        assert np.array_equal(b.flat(), single.flat())


def test_batch_equals_single_calls_bitwise(eng):
    bins = (50,) * 6
    trajs = _systems(SYSTEMS, seed0=5)
    bodies, trees = eng.entropy_batch(trajs, bins)
    for t, b, (e, tot) in zip(trajs, bodies, trees):
        single = eng.entropy(t, bins, "hist")
        assert np.array_equal(single.flat(), b.flat())
        e1, tot1 = eng.mist(t.n_dih)
        assert np.array_equal(e1, e)
        assert np.array_equal(tot1, tot)


def test_graph_replay_and_recapture(eng):
    """Same geometry -> the cached graph is replayed on new values; another
    geometry recaptures; the first geometry again gives the first results."""
    bins = (50,) * 6
    a = _systems(SYSTEMS[:3], seed0=21)
    b = _systems(SYSTEMS[:3], seed0=31)          # same shapes, other values
    c = _systems(SYSTEMS[2:5], seed0=41)         # other shapes
    ra = eng.entropy_batch(a, bins)
    rb = eng.entropy_batch(b, bins)
    rc = eng.entropy_batch(c, bins)
    ra2 = eng.entropy_batch(a, bins)
    _check_against_oracle(b, *rb, bins)
    _check_against_oracle(c, *rc, bins)
    for x, y in zip(ra[0], ra2[0]):
        assert np.array_equal(x.flat(), y.flat())
    for (e1, t1), (e2, t2) in zip(ra[1], ra2[1]):
        assert np.array_equal(e1, e2) and np.array_equal(t1, t2)


def test_batch_device_resident_views(eng):
    """Systems whose columns already live on the device (on_device=1, padded
    leading dimension), mixed with host systems."""
    bins = (50,) * 6
    host = _systems([(30, 5000, 0), (20, 3333, 1)], seed0=51)
    views, bufs = [], []
    for t in host:
        es = t.bonds.itemsize
        ld = t.n_frames + 64
        ptrs = []
        for arr in (t.bonds, t.angles, t.dihedrals):
            rows = arr.shape[0]
            p = eng.alloc(max(rows, 1) * ld * es)
            bufs.append(p)
            for r in range(rows):
                eng.memcpy(p + r * ld * es, arr[r].ctypes.data, t.n_frames * es, 1)
            ptrs.append(p)
        views.append(pg.BatView(t.n_dih, t.n_frames, t.double_prec, 1, ld, *ptrs))
    extra = _systems([(12, 2000, 0)], seed0=61)
    try:
        bodies, trees = eng.entropy_batch(views + extra, bins)
        _check_against_oracle(host + extra, bodies, trees, bins)
    finally:
        eng.synchronize()
        for p in bufs:
            eng.free(p)


def test_batch_outputs_optional(eng):
    bins = (50,) * 6
    trajs = _systems(SYSTEMS[:2], seed0=71)
    bodies, trees = eng.entropy_batch(trajs, bins, bodies=False, trees=True)
    assert bodies is None and len(trees) == 2
    bodies, trees = eng.entropy_batch(trajs, bins, bodies=True, trees=False)
    assert trees is None and len(bodies) == 2
    _check_against_oracle(trajs, bodies, [eng.entropy_batch(trajs, bins)[1][k] for k in range(2)], bins)


def test_batch_errors(eng):
    t = _systems([(10, 1000, 1)])[0]
    with pytest.raises(pg.PGError) as ex:   # the one-hot form needs 8..127 bins
        eng.entropy_batch([t], (50, 50, 50, 50, 4, 50), form="onehot")
    assert ex.value.code == pg.PG_ERR_UNSUPPORTED
    with pytest.raises(pg.PGError) as ex:
        eng.entropy_batch([t], (50, 50, 50, 50, 50, 0))
    assert ex.value.code == pg.PG_ERR_ARG
    bad = pg.synth_host(10, 1000, double_prec=1, seed=3)
    bad.bonds[2, 17] = -0.5
    with pytest.raises(pg.PGError) as ex:
        eng.entropy_batch([t, bad], (50,) * 6)
    assert ex.value.code == pg.PG_ERR_DATA
    # the context still works after the failures
    bodies, trees = eng.entropy_batch([t], (50,) * 6)
    _check_against_oracle([t], bodies, trees, (50,) * 6)
    rc = pg.lib().pg_entropy_batch(eng.handle, 0, None, (C.c_int * 6)(*([50] * 6)), 0, None, None, None)
    assert rc == pg.PG_ERR_ARG
