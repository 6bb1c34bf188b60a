"""Symmetric Gauss-Seidel subdomain preconditioner (fine_method 2) and the
`method` variants of the two-level preconditioner.

fine_method 2 runs num_iters (default 3, aggr.F90:221) forward + backward
Gauss-Seidel sweeps per subdomain in global row order on the entries of A
inside the subdomain, from x = 0, and adds the subdomain results
(FinePreconditioner_sgs.F90:69-86, stationary.F90:33-88).  method 5 is the
additive method 1 on one process (pcg.F90:205-208); methods 2 and 3 restrict a
residual vector the one-process reference allocates but never sets
(pcg.F90:146-149), so both the oracle and the library refuse them.
"""
import os

import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

from conftest import GOLDEN

LAP = os.path.join(GOLDEN, "lap16x16", "DOUG.ctl")


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


@pytest.mark.parametrize("m", [2, 3])
def test_methods_2_3_rejected(m):
    s = D.DougSolver(dict(solver=2, method=m, fine_method=1, levels=2, smoothers=1, overlap=1))
    s.load_ctl(LAP)
    with pytest.raises(D.DougError) as ei:
        s.setup_host_only()
    assert ei.value.status == D.DG_BAD_INPUT and "residual" in str(ei.value)


def test_fine_method_2_accepted_on_host():
    s = D.DougSolver(dict(solver=2, method=1, fine_method=2, levels=2, smoothers=1, overlap=1))
    s.load_ctl(LAP)
    s.setup_host_only()
    assert s.sizes()["n"] == 225


@pytest.mark.gpu
@pytest.mark.parametrize("levels,smoothers,overlap,iters", [(2, 1, 1, -1), (2, 0, -1, 2), (1, 0, 0, 4), (2, 2, 0, 1)])
def test_sgs_lap16x16_gpu(levels, smoothers, overlap, iters):
    opts = dict(solver=2, method=1, fine_method=2, levels=levels, smoothers=smoothers, overlap=overlap,
                num_iters=iters)
    s = D.DougSolver(opts)
    s.load_ctl(LAP)
    s.setup()
    x, st = s.solve()
    ref = O.read_vector(os.path.join(GOLDEN, "lap16x16", "csolution.xdr"), 2, 225)
    assert np.linalg.norm(x - ref) <= 1e-9
    ro = O.run_ctl(LAP, _ctl_text(opts))
    assert abs(st.iterations - ro["iterations"]) <= 1
    assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_sgs_poisson2d_gpu(precision):
    n, r, c, v, b, _ = P.poisson2d_p1(65, seed=7)
    opts = dict(solver=2, method=1, fine_method=2, levels=2, overlap=1, smoothers=1, strong1="0.08", radius1=2,
                solve_tolerance="1.0e-10", solve_maxiters=1000)
    s = D.DougSolver(opts)
    if precision:
        s.set_option("precision", precision)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.setup()
    x, st = s.solve()
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(opts))
    if precision == 0:
        assert abs(st.iterations - ro["iterations"]) <= 1
        assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
    else:
        assert np.linalg.norm(x - ro["x"]) <= 1e-7 * np.linalg.norm(ro["x"])


@pytest.mark.gpu
def test_method5_equals_method1_gpu():
    out = []
    for m in (1, 5):
        s = D.DougSolver(dict(solver=2, method=m, fine_method=1, levels=2, smoothers=1, overlap=1))
        s.load_ctl(LAP)
        s.setup()
        out.append(s.solve())
    (x1, s1), (x5, s5) = out
    assert s1.iterations == s5.iterations
    assert np.array_equal(x1, x5)
