"""The form autotuner (pg_autotune.cu): for systems of several shapes around
the crossover between the forms, PG_FORM_AUTO's pair-kernel time is within 5%
of the faster of the two forms timed one after the other, and its model's
prediction of each form is reported beside the measurement."""
from __future__ import annotations

import pytest

import parent_gb300 as pg

pytestmark = pytest.mark.gpu

# (atoms, frames, 2D bins): few and many tiles, short and long trajectories,
# on both sides of the crossover
SHAPES = [(60, 8192, 8), (300, 20000, 10), (1000, 50000, 12), (400, 100000, 16), (700, 30000, 20),
          (2000, 20000, 14), (150, 60000, 24)]


def _pair_ms(eng, view, bins, form, reps=2):
    best = None
    for _ in range(reps):
        eng.entropy(view, bins, form, keep_result=False)
        ms = float(eng.timings()[1])
        best = ms if best is None else min(best, ms)
    return best, eng.last_form()


@pytest.mark.parametrize("atoms,frames,b", SHAPES)
def test_autotuner_pick_is_within_5_percent_of_the_faster_form(atoms, frames, b):
    bins = (b,) * 6
    with pg.Engine(0) as eng:
        nd = atoms - 3
        nb, na = nd + 2, nd + 1
        D = nb + na + nd
        buf = eng.alloc(D * frames * 4)
        try:
            ptrs = (buf, buf + nb * frames * 4, buf + (nb + na) * frames * 4)
            eng.synth_device(atoms, frames, 0, ptrs, frames, seed=atoms + b, frac_bimodal_dih=0.2)
            view = pg.BatView(nd, frames, 0, 1, frames, *ptrs)
            eng.entropy(view, bins, "hist", keep_result=False)     # buffers and tables of this geometry
            eng.entropy(view, bins, "onehot", keep_result=False)
            t_hist, _ = _pair_ms(eng, view, bins, "hist")
            t_oh, _ = _pair_ms(eng, view, bins, "onehot")
            t_auto, form = _pair_ms(eng, view, bins, "auto")
            p_hist = eng.predict_pair_ms(nd, frames, bins, "hist")
            p_oh = eng.predict_pair_ms(nd, frames, bins, "onehot")
        finally:
            eng.synchronize()
            eng.free(buf)
    best = min(t_hist, t_oh)
    msg = (f"{D} DOFs x {frames} frames x {b} bins: hist {t_hist:.3f} ms (model {p_hist:.3f}), "
           f"onehot {t_oh:.3f} ms (model {p_oh:.3f}), auto -> {form} {t_auto:.3f} ms")
    print(msg)
    assert form == ("onehot" if p_oh < p_hist else "hist"), msg
    assert t_auto <= 1.05 * best + 0.05, msg
