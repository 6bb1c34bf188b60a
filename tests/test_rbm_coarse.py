"""coarse_method 3: smoothed aggregation over nodal blocks with a rigid-body
near-nullspace (an extension; the reference's aggregation is scalar,
SpMtx_aggregation.F90:49-641).

The product's host setup (doug_gb300/csrc/host/setup.cpp, build_setup_rbm)
and the oracle's restatement (oracle/doug_oracle.c, run_setup_rbm) run the
same steps in the same order: node aggregates, R and AC must agree bit for
bit.  On the GPU the solve with this coarse space matches the oracle's PCG
(FP64 within 1e-10, iterations +-1; mixed within 1e-7) and needs far fewer
iterations than the scalar coarse space on the same elasticity problem.
"""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08",
           radius1=2, maxasize1=100, coarse_method=3, solve_tolerance="1.0e-8", solve_maxiters=3000)


def _problem(N=8, seed=3, parts=(2, 2, 2)):
    ngf, eptr, efree, emat, erhs, info = P.elasticity3d_p1_elements(N, seed=seed)
    part = P.dof_box_partition(info["node_ijk"], N, parts=parts)
    return ngf, eptr, efree, emat, erhs, info, part


def _solver(prob, ctl=CTL, precision=None):
    ngf, eptr, efree, emat, erhs, info, part = prob
    s = D.DougSolver(ctl)
    if precision is not None:
        s.set_option("precision", precision)
    s.set_elements(ngf, eptr, efree, emat, erhs)
    s.set_node_geometry(info["coords"], info["freemap"])
    s.set_partition(part)
    return s


def _oracle(prob, s, ctl=CTL):
    ngf, eptr, efree, emat, erhs, info, part = prob
    n, r, c, v, b = s.input_matrix()
    # the assembled unknowns are the used freedoms in increasing order
    used = np.unique(efree)
    unode = np.asarray(info["freemap"])[used - 1]
    O.set_geometry(info["coords"], unode)
    try:
        ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(ctl), part=part)
    finally:
        O.set_geometry()
    assert ro["status"] == 0, ro["errmsg"]
    return ro


@pytest.mark.parametrize("N,seed", [(6, 1), (8, 3)])
def test_rbm_setup_bitwise(N, seed):
    prob = _problem(N, seed)
    s = _solver(prob)
    s.setup_host_only()
    ro = _oracle(prob, s)
    f, _ = s.aggregates()
    assert np.array_equal(f, ro["aggr_fine"])
    # aggregates are of mesh nodes: the three freedoms of a node share one
    assert np.all(f.reshape(-1, 3) == f.reshape(-1, 3)[:, :1])
    for x, y in zip(s.restriction(), ro["R"][2:]):
        assert np.array_equal(x, y)
    for x, y in zip(s.coarse_matrix(), ro["AC"][1:]):
        assert np.array_equal(x, y)
    # up to six rigid-body modes per aggregate
    nagr = int(f.max())
    assert nagr < ro["AC"][0] <= 6 * nagr
    sd = s.subdomains()
    assert len(sd) == len(ro["subdomains"]) == 8
    for a, b in zip(sd, ro["subdomains"]):
        assert np.array_equal(a, b)


def test_rbm_needs_geometry_and_partition():
    prob = _problem(4, 0)
    ngf, eptr, efree, emat, erhs, info, part = prob
    s = D.DougSolver(CTL)
    s.set_elements(ngf, eptr, efree, emat, erhs)
    s.set_partition(part)
    with pytest.raises(D.DougError):
        s.setup_host_only()
    s = _solver(prob)
    s.set_partition(np.ones(ngf, dtype=np.int32))  # one part is fine
    s.setup_host_only()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_rbm_solve_matches_oracle(precision):
    prob = _problem(10, 3)
    s = _solver(prob, precision=precision)
    s.setup()
    x, st = s.solve(allow_not_converged=False)
    ro = _oracle(prob, s)
    err = np.linalg.norm(x - ro["x"]) / np.linalg.norm(ro["x"])
    if precision == 0:
        assert abs(st.iterations - ro["iterations"]) <= 1, (st.iterations, ro["iterations"])
        assert err <= 1e-10, err
    else:
        assert err <= 1e-7, err
    # the scalar coarse space of the reference needs many more iterations
    s2 = _solver(prob, ctl=dict(CTL, coarse_method=1), precision=precision)
    s2.setup()
    _, st2 = s2.solve(allow_not_converged=False)
    assert st.iterations < 0.6 * st2.iterations, (st.iterations, st2.iterations)
