"""The oracle (oracle/parent_oracle.c) pinned against the reference itself:
the reference programs' outputs on a real-data subset of the ubiquitin test
system and on a synthetic FP32 system (tests/golden/, made by make_golden.py),
and the reference's shipped golden totals for the full test system."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import FIXTURES, GOLDEN, par_body_from_file, read_text_gz

REF_ROOT = oracle.reference_root()

TOTAL_NAMES_MIST = ["TOTAL 1D BONDS ENTROPY", "TOTAL 1D ANGLES ENTROPY", "TOTAL 1D DIHEDRALS ENTROPY",
                    "TOTAL 2D BONDS-BONDS MUTUAL INFORMATION", "TOTAL 2D BONDS-ANGLES MUTUAL INFORMATION",
                    "TOTAL 2D BONDS-DIHEDRALS MUTUAL INFORMATION", "TOTAL 2D ANGLES-ANGLES MUTUAL INFORMATION",
                    "TOTAL 2D ANGLES-DIHEDRALS MUTUAL INFORMATION", "TOTAL 2D DIHEDRALS-DIHEDRALS MUTUAL INFORMATION",
                    "TOTAL CONFIGURATIONAL ENTROPY"]


def mist_lines(edges, totals) -> list[str]:
    ch = "bad"
    out = ["%s %s %d %d   MI: %s   left to process: %d" % (ch[e["t1"]], ch[e["t2"]], e["i1"], e["i2"],
                                                           oracle.fmt12(e["mi"]), e["left"]) for e in edges]
    return out + ["%s = %s" % (n, oracle.fmt12(v)) for n, v in zip(TOTAL_NAMES_MIST, totals)]


@pytest.mark.parametrize("stem", FIXTURES)
def test_oracle_par_bit_identical_to_reference(stem):
    n, F, prec, b, a, d = oracle.read_bat(GOLDEN / f"{stem}.bat")
    body = oracle.parent(b, a, d, (50,) * 6)
    n_ref, ref = par_body_from_file(GOLDEN / f"{stem}_ref.par")
    assert n == n_ref
    for k in oracle.BLOCKS:
        assert np.array_equal(body[k].view(np.uint64), ref[k].view(np.uint64)), k


@pytest.mark.parametrize("stem", FIXTURES)
def test_oracle_mist_matches_reference_text(stem):
    n, ref = par_body_from_file(GOLDEN / f"{stem}_ref.par")
    edges, totals = oracle.mist(n, ref)
    assert mist_lines(edges, totals) == read_text_gz(f"{stem}_ref_MIST.txt.gz")


@pytest.mark.parametrize("stem", FIXTURES)
def test_oracle_mie_totals_match_reference_text(stem):
    n, ref = par_body_from_file(GOLDEN / f"{stem}_ref.par")
    tot = oracle.mie_totals(n, ref)
    tail = read_text_gz(f"{stem}_ref_MIE.txt.gz")[-16:]
    assert [ln.split(" = ")[0] + " = " + oracle.fmt12(v) for ln, v in zip(tail, tot)] == tail


def test_oracle_counts_are_a_histogram():
    """Count-level oracle: every pair's counts sum to the frame count."""
    n, F, prec, b, a, d = oracle.read_bat(GOLDEN / "synth_small.bat")
    D = 3 * n + 3
    pairs = [(0, 1), (0, D - 1), (n + 2, n + 3), (D - 2, D - 1)]
    for c in oracle.pair_counts(b, a, d, (50,) * 6, pairs):
        assert c.sum() == F and c.min() >= 0


@pytest.mark.skipif(not (REF_ROOT / "test_system" / "UBQ_UBM2.xtc").exists() or not oracle.ref_available(),
                    reason="needs the reference test system and oracle/_ref (built where the sources exist)")
def test_oracle_reproduces_full_test_system_golden(tmp_path):
    """The reference's shipped golden totals (test_system/sample_output) from
    the oracle, on the .bat the reference BAT_builder makes from the xtc."""
    bat = tmp_path / "ubq.bat"
    ts = REF_ROOT / "test_system"
    subprocess.run([str(oracle.REF / "BAT_builder.x"), "-t", str(ts / "UBQ_UBM2.top"), "-x", str(ts / "UBQ_UBM2.xtc"),
                    "-o", str(bat), "-bb", "CA C N H1 O1"], check=True, stdout=subprocess.DEVNULL)
    n, F, prec, b, a, d = oracle.read_bat(bat)
    body = oracle.parent(b, a, d, (50,) * 6)
    gold = (GOLDEN / "ubq_full_sample_output_MIE.txt").read_text().splitlines()
    tot = oracle.mie_totals(n, body)
    assert [ln.split(" = ")[0] + " = " + oracle.fmt12(v) for ln, v in zip(gold, tot)] == gold
    gold_mist = (GOLDEN / "ubq_full_sample_output_MIST.txt").read_text().splitlines()
    edges, totals = oracle.mist(n, body)
    assert mist_lines(edges, totals)[-10:] == gold_mist
