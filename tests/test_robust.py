"""Robust coarse space (coarse_method 2, §8(f) of the hot-path scope).

The reference builds the coarse space of Graham, Scheichl and Van lent
(CoarsePreconditioner_robust.F90:34-63, RobustCoarseMtx.f90:53-210): g solves
B g = 1 with B = sum_i R_i^T A_i^-1 R_i over the supports of the smoothed
restriction, and row i of the new restriction is A_i^-1 g on support i.  The
oracle solves B g = 1 exactly (dense); the product runs CG on the GPU with the
support matrices factored by the batched multifrontal kernels.  The
restriction's pattern must be equal, its values and the coarse matrix within
rounding of the B-solve, the solution within 1e-10 of the oracle's.
"""
import os

import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

from conftest import GOLDEN


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


def test_oracle_robust_lap16x16_matches_fixture():
    ref = O.read_vector(os.path.join(GOLDEN, "lap16x16", "csolution.xdr"), 2, 225)
    for sm in (0, 1, 2):
        r = O.run_ctl(os.path.join(GOLDEN, "lap16x16", "DOUG.ctl"),
                      f"solver 2\nmethod 1\nfine_method 1\nlevels 2\nsmoothers {sm}\noverlap 1\ncoarse_method 2\n")
        assert r["status"] == 0, r
        assert np.linalg.norm(r["x"] - ref) <= 1e-6
        assert np.linalg.norm(r["x"] - ref) <= 1e-11 * np.linalg.norm(ref)


def test_coarse_method_words():
    # coarse_method 4 is unknown (aggr.F90:155-165: "Wrong coarse method");
    # 3 (the rigid-body coarse space, an extension) needs node coordinates
    n, r, c, v, b = P.laplace2d(8)
    for cm, msg in ((4, "coarse method"), (3, "node coordinates")):
        s = D.DougSolver(dict(solver=2, method=1, fine_method=1, levels=2, coarse_method=cm))
        s.set_matrix_coo(n, r, c, v)
        with pytest.raises(D.DougError) as ei:
            s.setup_host_only()
        assert msg in str(ei.value)
        ro = O.run_coo(n, r, c, v, rhs=b, ctl=f"solver 2\nmethod 1\nfine_method 1\nlevels 2\ncoarse_method {cm}\n")
        assert ro["status"] != 0


CASES = {
    "lap16x16": lambda: (*P.laplace2d(15)[:4], np.ones(225)),
    "p1_33": lambda: P.poisson2d_p1(33, seed=6)[:5],
    "fv_8": lambda: P.diffusion3d_fv(8, seed=4),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("smoothers", [0, 1])
def test_robust_gpu_matches_oracle(case, smoothers):
    n, r, c, v, b = CASES[case]()
    opts = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=smoothers, strong1="0.08",
                radius1=1, coarse_method=2, solve_tolerance="1.0e-10", solve_maxiters=500)
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(opts))
    assert ro["status"] == 0, ro
    s = D.DougSolver(opts)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.setup()
    # restriction: same pattern and entry order, values within the B-solve's rounding
    ri, rj, rv = s.restriction()
    oi, oj, ov = ro["R"][2:]
    assert np.array_equal(ri, oi) and np.array_equal(rj, oj)
    assert np.abs(rv - ov).max() <= 1e-10 * np.abs(ov).max()
    ci, cj, cv = s.coarse_matrix()
    qi, qj, qv = ro["AC"][1:]
    assert np.array_equal(ci, qi) and np.array_equal(cj, qj)
    assert np.abs(cv - qv).max() <= 1e-10 * np.abs(qv).max()
    x, st = s.solve()
    assert abs(st.iterations - ro["iterations"]) <= 1
    assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
