"""The small plain case: 2-D P1 Poisson on a 129x129 jittered node grid
(16,129 unknowns), 4 imported subdomains (2x2 quadrants, the stand-in for
METIS), overlap 1, smoothed-aggregation coarse grid with the prolongator
weight omega = 2/3 (the extension word omega; the reference hard-codes 1/3,
CoarseMtx.F90:64-67), PCG to 1e-8.  The host setup must equal the oracle's
bit for bit; the GPU solution the oracle's to 1e-10 (FP64, iterations +-1)
and the FP64 direct solve to 1e-7 at tolerance 1e-10 (mixed).
"""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

OPTS = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08", radius1=2,
            solve_tolerance="1.0e-8", solve_maxiters=1000, omega=repr(2.0 / 3.0))


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


@pytest.fixture(scope="module")
def cfg0():
    n, r, c, v, b, xy = P.poisson2d_p1(129, seed=0)
    part = (1 + (xy[:, 0] >= 0.5) * 2 + (xy[:, 1] >= 0.5)).astype(np.int32)
    return n, r, c, v, b, part


@pytest.mark.parametrize("omega", [None, repr(2.0 / 3.0)])
def test_cfg0_setup_equals_oracle(cfg0, omega):
    n, r, c, v, b, part = cfg0
    opts = dict(OPTS)
    if omega is None:
        del opts["omega"]
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(opts), part=part, setup_only=True)
    assert ro["status"] == 0, ro["errmsg"]
    s = D.DougSolver(opts)
    s.set_matrix_coo(n, r, c, v)
    s.set_partition(part)
    s.setup_host_only()
    ri, rj, rv = s.restriction()
    ci, cj, cv = s.coarse_matrix()
    assert np.array_equal(ri, ro["R"][2]) and np.array_equal(rj, ro["R"][3])
    assert np.array_equal(rv.view(np.int64), ro["R"][4].view(np.int64))
    assert np.array_equal(ci, ro["AC"][1]) and np.array_equal(cj, ro["AC"][2])
    assert np.array_equal(cv.view(np.int64), ro["AC"][3].view(np.int64))
    sd = s.subdomains()
    assert len(sd) == 4 and all(np.array_equal(a, b_) for a, b_ in zip(sd, ro["subdomains"]))


def test_omega_changes_the_prolongator(cfg0):
    n, r, c, v, b, part = cfg0
    base = dict(OPTS)
    del base["omega"]
    r3 = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(base), part=part, setup_only=True)
    r2 = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(OPTS), part=part, setup_only=True)
    assert np.array_equal(r3["R"][2], r2["R"][2]) and not np.array_equal(r3["R"][4], r2["R"][4])


@pytest.mark.gpu
def test_cfg0_gpu_matches_oracle(cfg0):
    n, r, c, v, b, part = cfg0
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(OPTS), part=part)
    assert ro["status"] == 0
    s = D.DougSolver(OPTS)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.set_partition(part)
    s.setup()
    x, st = s.solve()
    assert abs(st.iterations - ro["iterations"]) <= 1
    assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
    assert st.true_rel_residual <= 1.01e-8


@pytest.mark.gpu
def test_cfg0_mixed_vs_direct(cfg0):
    n, r, c, v, b, part = cfg0
    s = D.DougSolver(dict(OPTS, solve_tolerance="1.0e-10"))
    s.set_option("precision", 1)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.set_partition(part)
    s.setup()
    x, st = s.solve()
    xd = O.spd_solve(n, r - 1, c - 1, v, b)
    assert st.true_rel_residual <= 1.01e-10
    assert np.linalg.norm(x - xd) <= 1e-7 * np.linalg.norm(xd)
