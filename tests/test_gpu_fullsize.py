"""Full-size parity: whole systems of thousands of DOFs against the FP64 oracle.

The precision-path system (2,994 DOFs x 100,000 frames, FP32) runs through
pg_entropy + pg_mist exactly as a user runs it; the oracle then checks that
run itself (oracle/check.py): 10,000 random pairs' 2D entropies and MI terms
(within 1e-5 nats, observed ~1e-12), bit-exact counts of 50 of those pairs
from the pair kernel, every 1D entropy, and the reference's MIST scan
(get_PAR_MIST.cpp:441-748, first strict maximum in block / In-position /
Out-index order) run on the GPU's own .par body, which must give the GPU's
edge list edge for edge.
"""
from __future__ import annotations

import numpy as np
import pytest

import parent_gb300 as pg
from oracle import check

pytestmark = pytest.mark.gpu


def _run(n_atoms, frames, bins, form="auto", seed=20261, frac_bimodal_dih=0.2, frac_bimodal_bond=0.05,
         monkeypatch=None, stream="1"):
    if monkeypatch is not None:
        # the streamed 32-slot layout (1, the default) or the ring-fed /
        # 16-slot one (0)
        monkeypatch.setenv("PG_HIST_STREAM", stream)
    t = pg.synth_host(n_atoms, frames, double_prec=0, seed=seed, frac_bimodal_dih=frac_bimodal_dih,
                      frac_bimodal_bond=frac_bimodal_bond)
    with pg.Engine(0) as eng:
        body = eng.entropy(t, bins, form)
        used = eng.last_form()
        edges, totals = eng.mist(t.n_dih)
        res = check.check_run(t.bonds, t.angles, t.dihedrals, bins, body.blocks, edges,
                              gpu_counts=lambda pairs: eng.pair_counts(t, bins, pairs),
                              n_pairs=10000, n_count_pairs=50)
    return res, used


def _assert_ok(res):
    assert res["counts_bit_exact"], res
    assert res["max_abs_dMI_nats"] <= 1e-9, res
    assert res["max_abs_dS2D_nats"] <= 1e-9, res
    assert res["max_abs_dS1_nats"] <= 1e-9, res
    assert res["mist_identical"], res
    assert res["mist_max_abs_dMI_nats"] <= 1e-9, res


@pytest.mark.parametrize("stream", ["0", "1"])
def test_precision_path_system_matches_oracle_at_50_bins(monkeypatch, stream):
    res, used = _run(1000, 100_000, (50,) * 6, monkeypatch=monkeypatch, stream=stream)
    assert used == "hist"
    assert res["pairs_total"] == 2994 * 2993 // 2 and res["mist_edges"] == 2993
    _assert_ok(res)


@pytest.mark.parametrize("stream", ["0", "1"])
def test_precision_path_system_matches_oracle_at_30_bins(monkeypatch, stream):
    # the 32-slot layout with 32-bit counters, ring-fed or streamed
    res, used = _run(1000, 100_000, (30,) * 6, seed=777, monkeypatch=monkeypatch, stream=stream)
    assert used == "hist"
    _assert_ok(res)


def test_mixed_bins_system_matches_oracle():
    # per-type 2D bin counts (bonds 50, angles 36, dihedrals 42) and 1D counts of their own
    res, _ = _run(700, 60_000, (40, 30, 20, 50, 36, 42), seed=99)
    _assert_ok(res)
