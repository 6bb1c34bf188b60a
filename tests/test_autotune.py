"""Batch parameters of the multifrontal factorisation and the autotuner.

The control words panel_rows, fwd_task_kb, lean_task_kb and nd_leaf change
only how fronts are batched into kernels (and, for nd_leaf, the elimination
order inside a subdomain): every setting must give the oracle's solution to
the FP64 bar.  dg_autotune times full solves over a grid of them and must
leave the handle set up with one of the grid's points.
"""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

OPTS = dict(solver=2, method=1, fine_method=1, levels=2, overlap=2, smoothers=1, strong1="0.08",
            radius1=2, solve_tolerance="1.0e-10", solve_maxiters=1000)
GRID = {(24, 512, 96, 80), (16, 512, 96, 80), (32, 512, 96, 80), (24, 256, 96, 80),
        (24, 512, 64, 48), (24, 512, 160, 96)}


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


@pytest.mark.parametrize("word", ["panel_rows", "fwd_task_kb", "lean_task_kb", "thin_level_fronts", "solve_schedule",
                                  "solve_pdl", "factor_overlap"])
def test_tuning_words_reject_bad_values(word):
    s = D.DougSolver({})
    binary = word in ("solve_schedule", "solve_pdl", "factor_overlap")
    s.set_option(word, 1 if binary else 64)
    for bad in ((-3, "x") if word == "thin_level_fronts" else (2, -1, "x") if binary else (0, -3, "x")):
        with pytest.raises(D.DougError):
            s.set_option(word, bad)


@pytest.fixture(scope="module")
def diffusion24():
    n, r, c, v, b = P.diffusion3d_fv(24, seed=13)
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(OPTS))
    assert ro["status"] == 0
    return n, r, c, v, b, ro


@pytest.mark.gpu
@pytest.mark.parametrize("words", [dict(panel_rows=16), dict(panel_rows=48, fwd_task_kb=4, lean_task_kb=1),
                                   dict(fwd_task_kb=1024, lean_task_kb=4096), dict(nd_leaf=8),
                                   dict(thin_level_fronts=0), dict(thin_level_fronts=100000),
                                   dict(solve_schedule=1), dict(solve_schedule=1, thin_level_fronts=0),
                                   dict(solve_pdl=0), dict(factor_overlap=0),
                                   dict(panel_rows=16, tensor_update=0), dict(panel_rows=16, super_panel=32),
                                   dict(panel_rows=16, super_panel=64, factor_overlap=0)])
@pytest.mark.parametrize("precision", [0, 1])
def test_batch_parameters_keep_the_solution(diffusion24, words, precision):
    n, r, c, v, b, ro = diffusion24
    s = D.DougSolver(OPTS)
    s.set_option("precision", precision)
    for k, val in words.items():
        s.set_option(k, val)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.setup()
    x, st = s.solve()
    if precision == 0:
        assert abs(st.iterations - ro["iterations"]) <= 1
        assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
    else:
        assert st.true_rel_residual <= 1.01e-10
        assert np.linalg.norm(x - ro["x"]) <= 1e-7 * np.linalg.norm(ro["x"])


@pytest.mark.gpu
def test_autotune_picks_a_grid_point_and_solves(diffusion24):
    n, r, c, v, b, ro = diffusion24
    s = D.DougSolver(OPTS)
    s.set_option("precision", 1)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    words, best = s.autotune()
    assert (words["nd_leaf"], words["panel_rows"], words["fwd_task_kb"], words["lean_task_kb"]) in GRID
    assert 0 < best < 60
    x, st = s.solve()
    assert st.true_rel_residual <= 1.01e-10
    assert np.linalg.norm(x - ro["x"]) <= 1e-7 * np.linalg.norm(ro["x"])


@pytest.mark.gpu
@pytest.mark.parametrize("word", ["solve_pdl", "factor_overlap"])
@pytest.mark.parametrize("precision", [0, 1])
def test_launch_overlap_gives_identical_results(diffusion24, precision, word):
    """The programmatic dependent launch of the level solves (solve_pdl) and
    the side stream of the one-CTA fronts in the factorisation
    (factor_overlap) change when CTAs start, not what they compute: the
    solutions are bit-identical.  panel_rows 48 gives the factorisation
    levels with both one-CTA and large fronts."""
    n, r, c, v, b, ro = diffusion24
    xs = []
    for on in (0, 1):
        s = D.DougSolver(OPTS)
        s.set_option("precision", precision)
        s.set_option("panel_rows", 48)
        s.set_option(word, on)
        s.set_matrix_coo(n, r, c, v)
        s.set_rhs(b)
        s.setup()
        x, st = s.solve()
        xs.append((x, st.iterations))
    assert xs[0][1] == xs[1][1]
    assert np.array_equal(xs[0][0].view(np.int64), xs[1][0].view(np.int64))
