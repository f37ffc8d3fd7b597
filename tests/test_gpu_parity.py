"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's own outputs.

Bars: bin-decision inputs (per-DOF min/max/shift) and every 2D histogram
count bit-exact; 1D/2D entropies and MI within 1e-9 nats of the FP64
oracle (the required bar is 1e-5 nats; the decomposition error is ~1e-12);
MIST edge list identical (types, indices, order), MI of each edge within
1e-9, totals within 1e-7.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import parent_gb300 as pg
from conftest import FIXTURES, GOLDEN, par_body_from_file, read_text_gz

pytestmark = pytest.mark.gpu

S_TOL = 1e-9      # nats, entropies
MI_TOL = 1e-5     # nats, the required bar for every MI term


@pytest.fixture(scope="module")
def eng():
    e = pg.Engine(0)
    yield e
    e.close()


def mutual_all(n: int, body: dict) -> np.ndarray:
    """Every pair's MI as get_mutual (util.cpp:47-81) forms it, in body order."""
    nb, na, nd = n + 2, n + 1, n
    s1b, s1a, s1d = body["s1_b"], body["s1_a"], body["s1_d"]
    out = []
    for key, s1, m in (("bb", s1b, nb), ("aa", s1a, na), ("dd", s1d, nd)):
        if m < 2:
            continue
        i, j = np.triu_indices(m, 1)          # lexicographic
        mi = s1[i] + s1[j] - body[key][::-1]  # stored reversed
        out.append(mi)
    for key, s1, s2 in (("ba", s1b, s1a), ("bd", s1b, s1d), ("ad", s1a, s1d)):
        if s2.size == 0:
            continue
        out.append((s1[:, None] + s2[None, :]).ravel() - body[key])
    return np.concatenate(out) if out else np.zeros(0)


def compare_bodies(n, gpu: pg.ParBody, ref: dict, s_tol=S_TOL):
    for k in oracle.BLOCKS:
        a, b = gpu.blocks[k], ref[k]
        assert a.shape == b.shape, k
        if a.size:
            err = np.max(np.abs(a - b))
            assert err <= s_tol, f"{k}: max |dS| = {err:.3e}"
    dmi = np.abs(mutual_all(n, gpu.blocks) - mutual_all(n, ref))
    if dmi.size:
        assert dmi.max() <= MI_TOL
    return float(dmi.max()) if dmi.size else 0.0


def compare_mist(gpu_edges, gpu_tot, ref_edges, ref_tot):
    for f in ("t1", "t2", "i1", "i2", "left"):
        assert np.array_equal(gpu_edges[f], ref_edges[f]), f
    assert np.max(np.abs(gpu_edges["mi"] - ref_edges["mi"]), initial=0.0) <= S_TOL
    assert np.max(np.abs(gpu_tot - ref_tot)) <= 1e-7


def parse_mist_text(lines):
    ch = {"b": 0, "a": 1, "d": 2}
    edges = []
    for ln in lines:
        if ln.startswith("TOTAL"):
            break
        p = ln.split()
        edges.append((ch[p[0]], ch[p[1]], int(p[2]), int(p[3]), float(p[5]), int(p[9])))
    arr = np.array(edges, dtype=[("t1", "i4"), ("t2", "i4"), ("i1", "i4"), ("i2", "i4"), ("mi", "f8"), ("left", "i4")])
    tot = np.array([float(ln.split(" = ")[1]) for ln in lines if ln.startswith("TOTAL")])
    return arr, tot


# ------------------------------------------------------------ golden fixtures

@pytest.mark.parametrize("stem", FIXTURES)
def test_fixture_par_matches_reference(eng, stem):
    bat = pg.BatFile(GOLDEN / f"{stem}.bat")
    body = eng.entropy(bat.view(), (50,) * 6, "hist")
    n, ref = par_body_from_file(GOLDEN / f"{stem}_ref.par")
    compare_bodies(n, body, ref)
    # MIST on the MI matrix left resident on the device
    e, t = eng.mist(n)
    re, rt = parse_mist_text(read_text_gz(f"{stem}_ref_MIST.txt.gz"))
    for f in ("t1", "t2", "i1", "i2", "left"):
        assert np.array_equal(e[f], re[f]), f
    assert np.max(np.abs(e["mi"] - re["mi"])) <= 1e-9
    assert np.max(np.abs(t - rt) / np.maximum(1.0, np.abs(rt))) <= 1e-10


@pytest.mark.parametrize("stem", FIXTURES)
def test_fixture_mist_from_reference_par(eng, stem):
    """get_PAR_MIST on the reference's own .par: edges and text identical."""
    p = pg.ParFile(GOLDEN / f"{stem}_ref.par")
    e, t = eng.mist(p.n_dih, p.body)
    re, rt = oracle.mist(p.n_dih, p.body.blocks)
    compare_mist(e, t, re, rt)
    lines = []
    import tempfile, os
    with tempfile.TemporaryDirectory() as d:
        pg.write_mist_text(os.path.join(d, "m.txt"), p.n_dih, e, t)
        lines = open(os.path.join(d, "m.txt")).read().splitlines()
    assert lines == read_text_gz(f"{stem}_ref_MIST.txt.gz")


@pytest.mark.parametrize("stem", FIXTURES)
def test_fixture_counts_and_stats_bit_exact(eng, stem):
    n, F, prec, b, a, d = oracle.read_bat(GOLDEN / f"{stem}.bat")
    bat = pg.BatFile(GOLDEN / f"{stem}.bat")
    D = 3 * n + 3
    rng = np.random.default_rng(7)
    pairs = sorted({tuple(sorted(rng.choice(D, 2, replace=False).tolist())) for _ in range(60)})
    pairs += [(0, 1), (0, D - 1), (D - 2, D - 1), (n + 1, n + 2)]
    traj = pg.Trajectory(*(np.ascontiguousarray(x.astype(np.float64 if prec else np.float32)) for x in (b, a, d)))
    got = eng.pair_counts(traj, (50,) * 6, pairs)
    want = oracle.pair_counts(b, a, d, (50,) * 6, pairs)
    for (g1, g2), x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), (g1, g2)
    mn, mx, sh = eng.dof_stats(D)
    omn, omx, osh, _, bad = oracle.extrema(b, a, d)
    assert bad == 0
    assert np.array_equal(mn.view(np.uint64), omn.view(np.uint64))
    assert np.array_equal(mx.view(np.uint64), omx.view(np.uint64))
    assert np.array_equal(sh.view(np.uint64), osh.view(np.uint64))


# ------------------------------------------------------------ synthetic systems

def _synth_case(n_atoms, F, prec, seed, **kw):
    return pg.synth_host(n_atoms, F, double_prec=prec, seed=seed, **kw)


@pytest.mark.parametrize("n_atoms,F,prec,bins", [
    (100, 20000, 1, (50,) * 6),                      # the CPU-runnable config shape (294 DOFs, FP64)
    (40, 12345, 0, (50,) * 6),                       # FP32, ragged frame count
    (30, 5000, 0, (7, 64, 100, 10, 20, 30)),         # different bin counts per type
    (25, 3000, 1, (1, 1, 1, 1, 1, 1)),               # one bin
    (3, 777, 1, (50,) * 6),                          # no dihedrals
    (4, 1, 1, (50,) * 6),                            # one frame: constant columns
    (12, 4096, 0, (50, 50, 50, 100, 100, 100)),      # 2x2 tile kernel
    (9, 2000, 1, (50, 50, 50, 200, 180, 150)),       # 1x1 tile kernel
])
def test_synthetic_matches_oracle(eng, n_atoms, F, prec, bins):
    t = _synth_case(n_atoms, F, prec, seed=n_atoms * 7 + F, frac_bimodal_dih=0.2, frac_bimodal_bond=0.05)
    body = eng.entropy(t, bins, "hist")
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    n = n_atoms - 3
    compare_bodies(n, body, ref)
    e, tot = eng.mist(n)
    re, rt = oracle.mist(n, ref)
    if np.max(np.abs(re["mi"]), initial=0.0) <= 1e-9:
        # one 2D bin or one frame: every MI is exactly 0 in exact arithmetic,
        # so both trees are ordered by ~1e-14 rounding noise; only the values
        # can agree
        assert np.max(np.abs(e["mi"]), initial=0.0) <= 1e-9 and np.max(np.abs(re["mi"]), initial=0.0) <= 1e-9
        assert abs(tot[9] - rt[9]) <= 1e-7
        return
    compare_mist(e, tot, re, rt)


@pytest.mark.parametrize("n_atoms,F,prec,bins", [
    (100, 20000, 1, (50,) * 6),                      # the CPU-runnable config shape, one-hot form
    (40, 12345, 0, (10,) * 6),                       # FP32, ragged frame count, 10 bins
    (30, 5000, 0, (7, 64, 100, 8, 20, 16)),          # different 2D bin counts per type
    (3, 777, 1, (20,) * 6),                          # no dihedrals
    (60, 129, 0, (12,) * 6),                         # one K-block plus one frame
])
@pytest.mark.parametrize("pair", ["1", "0"])
def test_onehot_form_matches_oracle(eng, monkeypatch, n_atoms, F, prec, bins, pair):
    """The tcgen05 one-hot GEMM form, on CTA pairs (cta_group::2, the default)
    and on single CTAs: same S2D/MI bars and the same MIST tree."""
    monkeypatch.setenv("PG_ONEHOT_PAIR", pair)
    t = _synth_case(n_atoms, F, prec, seed=n_atoms * 11 + F, frac_bimodal_dih=0.2, frac_bimodal_bond=0.05)
    body = eng.entropy(t, bins, "onehot")
    assert eng.last_form() == "onehot"
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    n = n_atoms - 3
    compare_bodies(n, body, ref)
    e, tot = eng.mist(n)
    re, rt = oracle.mist(n, ref)
    compare_mist(e, tot, re, rt)


@pytest.mark.parametrize("n_atoms,F,bins", [
    (10, 1_300_000, (10,) * 6),          # two 2^20-frame chunks: one move into the INT32 totals
    (8, 4_500_000, (12, 9, 16, 12, 9, 16)),  # five chunks, past the FP32 accumulators' 2^22-frame limit
])
@pytest.mark.parametrize("pair", ["1", "0"])
def test_onehot_counts_accumulate_over_frame_chunks(eng, monkeypatch, n_atoms, F, bins, pair):
    """Trajectories longer than one 2^20-frame chunk: at each chunk end the
    tensor memory's FP32 counts are moved into INT32 totals and the
    accumulators restart, so the form has no frame limit. Same values as the
    oracle and as the histogram form."""
    monkeypatch.setenv("PG_ONEHOT_PAIR", pair)
    t = _synth_case(n_atoms, F, 0, seed=F + n_atoms, frac_bimodal_dih=0.3, frac_bimodal_bond=0.1)
    body = eng.entropy(t, bins, "onehot")
    assert eng.last_form() == "onehot"
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    compare_bodies(n_atoms - 3, body, ref)
    hist = eng.entropy(t, bins, "hist")
    assert np.max(np.abs(hist.flat() - body.flat())) <= 1e-12


def test_onehot_and_hist_agree_on_fixture(eng):
    bat = pg.BatFile(GOLDEN / "ubq_sub.bat")
    a = eng.entropy(bat.view(), (50,) * 6, "onehot").flat()
    b = eng.entropy(bat.view(), (50,) * 6, "hist").flat()
    assert np.max(np.abs(a - b)) <= S_TOL


@pytest.mark.parametrize("bins", [(50, 50, 50, 4, 50, 50), (50, 50, 50, 50, 128, 50)])
def test_onehot_rejects_unsupported_bins(eng, bins):
    """The one-hot form takes 2D bin counts 8..127 (per-tile DOF tables; bin
    bytes below 128 for its one-hot build)."""
    t = _synth_case(10, 300, 1, seed=4)
    with pytest.raises(pg.PGError) as e:
        eng.entropy(t, bins, "onehot")
    assert e.value.code == pg.PG_ERR_UNSUPPORTED


def test_counts_bit_exact_mixed_bins(eng):
    t = _synth_case(30, 9000, 0, seed=5, frac_bimodal_dih=0.3)
    bins = (13, 50, 77, 17, 33, 50)
    D = 3 * 27 + 3
    pairs = [(i, j) for i in range(0, D, 7) for j in range(i + 1, D, 5)]
    got = eng.pair_counts(t, bins, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, bins, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p


def test_form_auto_and_hist_agree(eng):
    t = _synth_case(20, 3000, 1, seed=11)
    a = eng.entropy(t, (50,) * 6, "auto").flat()
    b = eng.entropy(t, (50,) * 6, "hist").flat()
    assert np.max(np.abs(a - b)) <= S_TOL


def test_repeat_is_deterministic(eng):
    t = _synth_case(50, 10000, 0, seed=3)
    a = eng.entropy(t, (50,) * 6, "hist").flat()
    b = eng.entropy(t, (50,) * 6, "hist").flat()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


# ------------------------------------------------------------ MIST ties

@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mist_tie_order_matches_reference_scan(eng, seed):
    """Quantised MI values make many exact ties; the GPU tree must follow the
    reference's first-maximum scan order (get_PAR_MIST.cpp:481-606)."""
    n = 20
    rng = np.random.default_rng(seed)
    body = {k: np.round(rng.normal(0, 2, s) * 2) / 2 for k, s in oracle.sizes(n).items()}
    for k in ("s1_b", "s1_a", "s1_d"):
        body[k] = np.round(rng.normal(0, 1, oracle.sizes(n)[k]) * 4) / 4
    pb = pg.ParBody(n, {k: np.ascontiguousarray(v) for k, v in body.items()})
    e, t = eng.mist(n, pb)
    re, rt = oracle.mist(n, body)
    compare_mist(e, t, re, rt)


# ------------------------------------------------------------ error paths

@pytest.mark.parametrize("cluster", ["1", "0"])
def test_mist_over_a_cluster_matches_oracle(eng, monkeypatch, cluster):
    """1,194 DOFs: Prim over a cluster of 8 CTAs (the default from 1,024
    vertices) and over one CTA give the oracle's edge list on the same .par
    body, in the reference's tie order."""
    monkeypatch.setenv("PG_MIST_CLUSTER", cluster)
    n_atoms = 400
    t = _synth_case(n_atoms, 3000, 0, seed=17, frac_bimodal_dih=0.2, frac_bimodal_bond=0.05)
    body = eng.entropy(t, (20,) * 6, "hist")
    n = n_atoms - 3
    re, rt = oracle.mist(n, body.blocks)
    e2, tot2 = eng.mist(n)  # on the MI matrix the entropy call left on the device
    compare_mist(e2, tot2, re, rt)
    e, tot = eng.mist(n, body)  # from the .par body
    compare_mist(e, tot, re, rt)


@pytest.mark.parametrize("groups", ["4", "16", "4-ring"])
def test_grouped_upload_schedule_matches(eng, monkeypatch, groups):
    """PG_STREAM_GROUPS > 1 (uploads in DOF groups on the copy stream, pair
    launches alternating between two streams) gives the same body, bit for
    bit, as the default one-group upload; also with the ring-fed 32-slot
    layout instead of the streamed one (their integer n ln n sums are equal
    bit for bit)."""
    t = _synth_case(150, 6000, 0, seed=23, frac_bimodal_dih=0.2)
    base = eng.entropy(t, (50,) * 6, "hist").flat()
    monkeypatch.setenv("PG_STREAM_GROUPS", groups.split("-")[0])
    if groups.endswith("ring"):
        monkeypatch.setenv("PG_HIST_STREAM", "0")
    assert np.array_equal(eng.entropy(t, (50,) * 6, "hist").flat(), base)


def test_negative_bond_is_rejected(eng):
    t = _synth_case(10, 500, 1, seed=1)
    t.bonds[3, 17] = -0.1
    with pytest.raises(pg.PGError) as e:
        eng.entropy(t, (50,) * 6, "hist")
    assert e.value.code == pg.PG_ERR_DATA


def test_dihedral_outside_shift_histogram_is_rejected(eng):
    t = _synth_case(10, 500, 1, seed=1)
    t.dihedrals[2, 5] = 7.0
    with pytest.raises(pg.PGError) as e:
        eng.entropy(t, (50,) * 6, "hist")
    assert e.value.code == pg.PG_ERR_DATA


@pytest.mark.parametrize("bins,code", [((50, 50, 50, 50, 50, 0), pg.PG_ERR_ARG),
                                       ((0, 50, 50, 50, 50, 50), pg.PG_ERR_ARG),
                                       ((50, 50, 50, 219, 50, 50), pg.PG_ERR_UNSUPPORTED)])
def test_bad_bins(eng, bins, code):
    t = _synth_case(10, 100, 1, seed=1)
    with pytest.raises(pg.PGError) as e:
        eng.entropy(t, bins, "hist")
    assert e.value.code == code


def test_context_survives_errors(eng):
    t = _synth_case(10, 500, 1, seed=1)
    bad = _synth_case(10, 500, 1, seed=1)
    bad.bonds[0, 0] = -1.0
    with pytest.raises(pg.PGError):
        eng.entropy(bad, (50,) * 6, "hist")
    body = eng.entropy(t, (50,) * 6, "hist")
    compare_bodies(7, body, oracle.parent(t.bonds, t.angles, t.dihedrals, (50,) * 6))


def test_bounded_wait_times_out_and_context_survives(eng):
    """Failure detection without a fault: a kernel waits, with the pair
    kernels' bounded mbarrier wait, on a barrier nobody arrives on. The wait
    gives up after its limit, the timeout comes back as PG_ERR_TIMEOUT, and
    the context then computes correctly (twice, to check the error word is
    reset between calls)."""
    import time
    for _ in range(2):
        t0 = time.perf_counter()
        rc = pg.lib().pg_check_wait_timeout(eng.handle, 50.0)
        assert rc == pg.PG_ERR_TIMEOUT
        assert b"timed out" in pg.lib().pg_last_error(eng.handle)
        assert time.perf_counter() - t0 < 5.0
    t = _synth_case(10, 500, 1, seed=3)
    body = eng.entropy(t, (50,) * 6, "hist")
    compare_bodies(7, body, oracle.parent(t.bonds, t.angles, t.dihedrals, (50,) * 6))


# ------------------------------------------------------------ size-independent properties

def test_large_properties(eng):
    """A 900-DOF x 100k-frame FP32 system: every sampled pair's counts sum to F
    and equal the oracle's; sampled S2D match the oracle's per-pair value; the
    MI matrix is symmetric; MIST is a spanning tree over all DOFs."""
    n_atoms, F = 302, 100_000
    t = _synth_case(n_atoms, F, 0, seed=99, frac_bimodal_dih=0.2, frac_bimodal_bond=0.05)
    n = n_atoms - 3
    D = 3 * n + 3
    body = eng.entropy(t, (50,) * 6, "hist")
    rng = np.random.default_rng(0)
    pairs = sorted({tuple(sorted(rng.choice(D, 2, replace=False).tolist())) for _ in range(24)})
    got = eng.pair_counts(t, (50,) * 6, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, (50,) * 6, pairs)
    for p, x, y in zip(pairs, got, want):
        assert x.sum() == F and np.array_equal(x, y), p
    # per-pair S2D against the oracle's direct formula
    eng.entropy(t, (50,) * 6, "hist", out=body)
    mn, mx, _, dsh, _ = oracle.extrema(t.bonds, t.angles, t.dihedrals)
    cols = np.concatenate([t.bonds.astype(np.float64), t.angles.astype(np.float64), dsh])
    nb, na = n + 2, n + 1
    typ = lambda g: 0 if g < nb else (1 if g < nb + na else 2)
    off = {0: 0, 1: nb, 2: nb + na}
    import ctypes as C
    for g1, g2 in pairs[:8]:
        t1, t2 = typ(g1), typ(g2)
        s_or = oracle.lib().or_entropy2d(t1, oracle._p(np.ascontiguousarray(cols[g1])), mn[g1], mx[g1], 50,
                                         t2, oracle._p(np.ascontiguousarray(cols[g2])), mn[g2], mx[g2], 50,
                                         F, None, None)
        i1, i2 = g1 - off[t1], g2 - off[t2]
        if t1 == t2:
            m = (nb, na, n)[t1]
            idx = (m - i1) * (m - i1 - 1) // 2 + i1 - i2
            s_gpu = body.blocks[("bb", "aa", "dd")[t1]][idx]
        else:
            key = {(0, 1): "ba", (0, 2): "bd", (1, 2): "ad"}[(t1, t2)]
            s_gpu = body.blocks[key][i1 * (na, n)[t2 - 1] + i2]
        assert abs(s_gpu - s_or) <= S_TOL, (g1, g2)
    e, tot = eng.mist(n)
    assert len(e) == D - 1
    seen = {(0, 1)}
    for x in e:
        assert (x["t1"], x["i1"]) in seen and (x["t2"], x["i2"]) not in seen
        seen.add((x["t2"], x["i2"]))
    assert len(seen) == D


@pytest.mark.parametrize("n_atoms,F,bins", [(40, 70000, (50,) * 6), (20, 3000, (10, 20, 30, 50, 20, 8)),
                                            (30, 20000, (30,) * 6), (25, 5000, (20, 30, 35, 35, 20, 8)),
                                            (22, 4001, (50, 50, 50, 37, 49, 41)), (14, 999, (5, 5, 5, 36, 1, 3))])
@pytest.mark.parametrize("feed", ["ring", "stream"])
def test_hist32_layout_matches_oracle(eng, monkeypatch, n_atoms, F, bins, feed):
    """The 32-slot histogram layout (32-bit counters up to 35 bins, 16-bit
    counters for row-bin pairs above, odd row-bin counts included) gives the
    same counts and values, fed by the TMA ring or streamed from the
    frame-group interleaved bin matrix (ragged last groups included)."""
    if feed == "ring":
        monkeypatch.setenv("PG_HIST_SLOTS", "32")
    else:
        monkeypatch.setenv("PG_HIST_STREAM", "1")
    t = _synth_case(n_atoms, F, 0, seed=n_atoms + F, frac_bimodal_dih=0.2)
    body = eng.entropy(t, bins, "hist")
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    compare_bodies(n_atoms - 3, body, ref)
    D = 3 * n_atoms - 6
    pairs = [(0, 1), (0, D - 1), (5, 17), (D - 2, D - 1)]
    got = eng.pair_counts(t, bins, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, bins, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p


def _boundary_column64(rng, lo, hi, Bs, F, pad=5e-9):
    """FP64 column on [lo, hi] holding the doubles adjacent to every bin edge
    mn + k*bs, closer to the edges than any FP32 value can be."""
    mn, mx = lo - pad, hi + pad
    vals = [lo, hi]
    for B in Bs:
        bs = (mx - mn) / B
        for k in range(1, B):
            e = mn + k * bs
            vals += [np.nextafter(e, -np.inf), e, np.nextafter(e, np.inf)]
    vals = np.array([v for v in vals if lo <= v <= hi], dtype=np.float64)
    fill = rng.uniform(lo, hi, F - vals.size)
    col = np.concatenate([vals, fill])
    rng.shuffle(col)
    return col


def test_fp64_bin_edges_bit_exact(eng):
    """FP64 inputs go through the same FP32 screen after rounding to FP32:
    doubles within one ulp of every 1D and 2D edge get the reference's bins."""
    rng = np.random.default_rng(77)
    n_dih, F = 2, 25000
    B1, B2 = 41, 50
    bins = (B1, B1, B1, B2, B2, B2)
    bonds = np.stack([_boundary_column64(rng, 1.01 + 0.02 * k, 1.09 + 0.01 * k, (B1, B2), F) for k in range(n_dih + 2)])
    angles = np.stack([_boundary_column64(rng, 1.7 + 0.05 * k, 2.2, (B1, B2), F) for k in range(n_dih + 1)])
    base = [rng.uniform(0.5, 5.0, F), rng.uniform(0.0, 2 * np.pi - 1e-3, F)]
    dih = []
    for col in base:
        tb = np.zeros((3, F)) + 1.0
        ta = np.zeros((2, F)) + 1.5
        mn, mx, sh, _, bad = oracle.extrema(tb, ta, col[None, :])
        assert bad == 0
        twopi = 2 * np.pi
        extra = []
        for B in (B1, B2):
            for k in range(1, B):
                t = mn[-1] + k * (mx[-1] - mn[-1]) / B
                x = t - sh[-1]
                if x < 0:
                    x += twopi
                extra += [np.nextafter(x, -np.inf), x, np.nextafter(x, np.inf)]
        e = twopi - sh[-1]
        extra += [np.nextafter(e, -np.inf), e, np.nextafter(e, np.inf)]
        extra = np.array(extra)
        extra = extra[(extra >= col.min()) & (extra <= col.max())]
        c = col.copy()
        c[rng.choice(F, extra.size, replace=False)] = extra
        dih.append(c)
    dih = np.stack(dih)
    traj = pg.Trajectory(np.ascontiguousarray(bonds), np.ascontiguousarray(angles), np.ascontiguousarray(dih))
    D = 3 * n_dih + 3
    pairs = [(i, j) for i in range(D) for j in range(i + 1, D)]
    got = eng.pair_counts(traj, bins, pairs)
    want = oracle.pair_counts(bonds, angles, dih, bins, pairs)
    for p_, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p_
    mn, mx, sh = eng.dof_stats(D)
    omn, omx, osh, _, bad = oracle.extrema(bonds, angles, dih)
    assert bad == 0
    assert np.array_equal(mn.view(np.uint64), omn.view(np.uint64))
    assert np.array_equal(mx.view(np.uint64), omx.view(np.uint64))
    assert np.array_equal(sh.view(np.uint64), osh.view(np.uint64))
    body = eng.entropy(traj, bins, "hist")
    ref = oracle.parent(bonds, angles, dih, bins)
    compare_bodies(n_dih, body, ref)


def _boundary_column(rng, lo, hi, Bs, F, pad=5e-9):
    """FP32 column on [lo, hi] (both present) packed with the float values
    next to every bin edge mn + k*bs (mn = lo - pad, mx = hi + pad) of each
    bin count in Bs: the values whose bin the FP32 screen cannot decide."""
    lo, hi = np.float32(lo), np.float32(hi)
    mn, mx = np.float64(lo) - pad, np.float64(hi) + pad
    vals = [lo, hi]
    for B in Bs:
        bs = (mx - mn) / B
        for k in range(1, B):
            e = np.float32(mn + k * bs)
            vals += [np.nextafter(e, np.float32(-1e9)), e, np.nextafter(e, np.float32(1e9))]
    vals = np.array([v for v in vals if lo <= v <= hi], dtype=np.float32)
    fill = rng.uniform(float(lo), float(hi), F - vals.size).astype(np.float32)
    col = np.concatenate([vals, fill])
    rng.shuffle(col)
    return col


def _dihedral_boundaries(rng, col, B, target_mn, target_mx, shift):
    """Adds to a dihedral column the float x whose shifted value lies next to
    a bin edge of the shifted range (extrema and shift taken from the oracle
    on the column without them) and next to the shift's own 2 pi edge."""
    twopi = 2 * np.pi
    out = []
    for k in range(1, B):
        t = target_mn + k * (target_mx - target_mn) / B
        x = t - shift
        if x < 0:
            x += twopi
        e = np.float32(x)
        out += [np.nextafter(e, np.float32(-1)), e, np.nextafter(e, np.float32(10))]
    e = np.float32(twopi - shift)
    out += [np.nextafter(e, np.float32(-1)), e, np.nextafter(e, np.float32(10))]
    return np.array(out, dtype=np.float32)


def test_fp32_bin_edges_bit_exact(eng):
    """FP32 values adjacent to every 1D and 2D bin edge (and the dihedral
    shift's 2 pi edge) get the reference's bins: pair counts, per-DOF
    extrema/shift and 1D entropies agree with the FP64 oracle."""
    rng = np.random.default_rng(2024)
    n_dih, F = 3, 30000
    B1, B2 = 37, 50
    bins = (B1, B1, B1, B2, B2, B2)
    bonds = np.stack([_boundary_column(rng, 0.14 + 0.01 * k, 0.17 + 0.013 * k, (B1, B2), F) for k in range(n_dih + 2)])
    angles = np.stack([_boundary_column(rng, 1.2 + 0.1 * k, 2.4 + 0.05 * k, (B1, B2), F) for k in range(n_dih + 1)])
    # dihedral 0: a gap at 2 pi (longest empty run); 1: fully occupied (first
    # minimum bin); 2: concentrated near pi
    base = [rng.uniform(0.5, 5.0, F).astype(np.float32),
            rng.uniform(0.0, 2 * np.pi - 1e-3, F).astype(np.float32),
            np.mod(rng.normal(np.pi, 0.4, F), 2 * np.pi).astype(np.float32)]
    dih = []
    for k, col in enumerate(base):
        tb = np.zeros((3, F), np.float32) + 0.15
        ta = np.zeros((2, F), np.float32) + 1.5
        mn, mx, sh, _, bad = oracle.extrema(tb, ta, col[None, :])
        assert bad == 0
        extra = np.concatenate([_dihedral_boundaries(rng, col, B, mn[-1], mx[-1], sh[-1]) for B in (B1, B2)])
        extra = extra[(extra >= col.min()) & (extra <= col.max())]
        c = col.copy()
        c[rng.choice(F, extra.size, replace=False)] = extra
        dih.append(c)
    dih = np.stack(dih)
    traj = pg.Trajectory(np.ascontiguousarray(bonds), np.ascontiguousarray(angles), np.ascontiguousarray(dih))
    D = 3 * n_dih + 3
    pairs = [(i, j) for i in range(D) for j in range(i + 1, D)]
    got = eng.pair_counts(traj, bins, pairs)
    want = oracle.pair_counts(bonds, angles, dih, bins, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p
    mn, mx, sh = eng.dof_stats(D)
    omn, omx, osh, _, bad = oracle.extrema(bonds, angles, dih)
    assert bad == 0
    assert np.array_equal(mn.view(np.uint64), omn.view(np.uint64))
    assert np.array_equal(mx.view(np.uint64), omx.view(np.uint64))
    assert np.array_equal(sh.view(np.uint64), osh.view(np.uint64))
    body = eng.entropy(traj, bins, "hist")
    ref = oracle.parent(bonds, angles, dih, bins)
    compare_bodies(n_dih, body, ref)


def test_hist16_layout_matches_oracle(eng, monkeypatch):
    """The 16-slot histogram layout (32-bit counters, two lanes per pair),
    forced at 50 bins where the 32-slot layout is the default."""
    monkeypatch.setenv("PG_HIST_SLOTS", "16")
    t = _synth_case(40, 30000, 0, seed=99, frac_bimodal_dih=0.2)
    body = eng.entropy(t, (50,) * 6, "hist")
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, (50,) * 6)
    compare_bodies(37, body, ref)
    D = 3 * 40 - 6
    pairs = [(0, 1), (0, D - 1), (5, 17), (D - 2, D - 1)]
    got = eng.pair_counts(t, (50,) * 6, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, (50,) * 6, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p


@pytest.mark.parametrize("slots", ["32", "16", "stream"])
def test_peaked_counts_above_16_bits(eng, monkeypatch, slots):
    """Pairs of DOFs that sit on one value in the same 70% of 150,000 frames:
    one 2D bin holds 105,000 counts, above a 16-bit counter, so the 32-slot
    layouts (ring-fed and streamed) have to move counts out during the run.
    Counts stay bit-exact."""
    if slots == "stream":
        monkeypatch.setenv("PG_HIST_STREAM", "1")
    else:
        monkeypatch.setenv("PG_HIST_SLOTS", slots)
    rng = np.random.default_rng(5)
    n_dih, F = 5, 150000
    t = pg.synth_host(n_dih + 3, F, double_prec=0, seed=77)
    peak = rng.random(F) < 0.7
    t.bonds[0, peak] = np.float32(0.15)
    t.bonds[3, peak] = np.float32(0.16)
    t.angles[2, peak] = np.float32(1.9)
    t.dihedrals[1, peak] = np.float32(2.5)
    t.dihedrals[4, peak[::-1]] = np.float32(1.0)   # a different 70%
    nb, na = n_dih + 2, n_dih + 1
    D = nb + na + n_dih
    peaked = [0, 3, nb + 2, nb + na + 1, nb + na + 4]
    pairs = sorted({tuple(sorted((a, b))) for a in peaked for b in range(D) if a != b})
    got = eng.pair_counts(t, (50,) * 6, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, (50,) * 6, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p
    assert max(int(x.max()) for x in want) > 65535
    body = eng.entropy(t, (50,) * 6, "hist")
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, (50,) * 6)
    compare_bodies(n_dih, body, ref)


@pytest.mark.parametrize("bins", [(16384, 16384, 16384, 218, 218, 218), (16384, 7, 1, 218, 1, 50)])
def test_maximum_bin_counts_match_oracle(eng, bins):
    """The largest bin counts the ABI accepts: 16,384 1D bins and 218 2D bins
    (the 1 x 1 tile layout), next to single-bin types."""
    t = _synth_case(6, 6000, 0, seed=8, frac_bimodal_dih=0.2)
    body = eng.entropy(t, bins, "hist")
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    compare_bodies(3, body, ref)
    D = 12
    pairs = [(0, 1), (2, 9), (5, 11), (10, 11)]
    got = eng.pair_counts(t, bins, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, bins, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), p


def test_one_bin_above_1d_maximum_is_rejected(eng):
    t = _synth_case(6, 100, 0, seed=8)
    with pytest.raises(pg.PGError) as e:
        eng.entropy(t, (16385, 50, 50, 50, 50, 50), "hist")
    assert e.value.code == pg.PG_ERR_UNSUPPORTED


@pytest.mark.parametrize("case", range(10))
def test_random_systems_match_oracle(eng, case):
    """Seeded random systems across the histogram layouts: per-type 2D bin
    counts from 1 to 50 (32-bit and 16-bit counters, odd and even row-bin
    counts), ragged frame counts, FP32 and FP64, and sizes from a few tiles to
    enough tiles that each CTA's queue of finished tiles wraps several times;
    bodies within 1e-9 nats of the oracle, sampled counts bit-exact, MIST
    edge lists identical."""
    rng = np.random.default_rng(1000 + case)
    n_atoms = int(rng.choice([8, 23, 61, 150, 230]))
    F = int(rng.integers(1, 4) * rng.integers(700, 9000) + rng.integers(0, 16))
    prec = int(rng.integers(0, 2))
    b2 = [int(x) for x in rng.integers(1, 51, size=3)]
    b1 = [int(x) for x in rng.integers(1, 80, size=3)]
    bins = tuple(b1 + b2)
    t = _synth_case(n_atoms, F, prec, seed=case, frac_bimodal_dih=0.3)
    body = eng.entropy(t, bins, "hist")
    ref = oracle.parent(t.bonds, t.angles, t.dihedrals, bins)
    n = n_atoms - 3
    compare_bodies(n, body, ref)
    if min(b2) > 1 and F > 1:  # with all-zero MI the tree follows rounding noise
        e1, t1 = eng.mist(n)   # from the resident MI matrix of this call
        e2, t2 = oracle.mist(n, ref)
        compare_mist(e1, t1, e2, t2)
    D = 3 * n_atoms - 6
    pairs = sorted({tuple(sorted(int(x) for x in rng.choice(D, 2, replace=False))) for _ in range(6)})
    got = eng.pair_counts(t, bins, pairs)
    want = oracle.pair_counts(t.bonds, t.angles, t.dihedrals, bins, pairs)
    for p, x, y in zip(pairs, got, want):
        assert np.array_equal(x, y), (p, bins)


def test_entropy_ahead_and_prefetch_give_the_same_bodies(eng):
    """pg_entropy_ahead queues the next call's upload on the copy engine and
    pg_prefetch queues one explicitly: the call that takes the uploaded
    columns, a call on another view (which drops them) and every later call
    give the bodies of plain pg_entropy calls, bit for bit."""
    bins = (50,) * 6
    ta = _synth_case(40, 9000, 0, seed=61, frac_bimodal_dih=0.2)
    tb = _synth_case(40, 9000, 0, seed=62, frac_bimodal_dih=0.2)
    tc = _synth_case(33, 7001, 1, seed=63)
    want = {k: eng.entropy(t, bins, "hist").flat() for k, t in (("a", ta), ("b", tb), ("c", tc))}
    same = lambda body, k: np.array_equal(body.flat().view(np.uint64), want[k].view(np.uint64))
    assert same(eng.entropy(ta, bins, "hist", next=tb), "a")
    assert same(eng.entropy(tb, bins, "hist", next=tb), "b")   # takes tb's columns, queues tb again
    assert same(eng.entropy(tb, bins, "hist"), "b")            # takes them again
    assert same(eng.entropy(ta, bins, "hist", next=tb), "a")
    assert same(eng.entropy(tc, bins, "hist"), "c")            # another view: the prefetch of tb is dropped
    assert same(eng.entropy(tb, bins, "hist"), "b")
    eng.prefetch(tc)
    assert same(eng.entropy(tc, bins, "hist"), "c")
    eng.prefetch(ta)
    part = [eng.entropy_shard(ta, bins, s, 2) for s in range(2)]   # shard 0 takes the prefetched columns
    assert np.array_equal((part[0].flat() + part[1].flat()).view(np.uint64), want["a"].view(np.uint64))
