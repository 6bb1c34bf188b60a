"""Parity at the benchmark's own controls.

The benchmark solves the 128^3 log-normal diffusion problem with 64 box
subdomains, overlap 2, strong1 0.08, radius1 5, maxasize1 400 and smoothers 1.
These tests run the same controls on the 64^3 grid of the same generator (the
largest the oracle's whole solve finishes in seconds; 64 subdomains of 16^3
cells plus two overlap layers):

* the host setup (aggregates, subdomain lists, R, AC) is bit-equal to the
  oracle's (CPU);
* the FP64 GPU solve matches the oracle's PCG (pcg.F90:387-435) within
  relative 1e-10 with the iteration count within +-1;
* the mixed-precision GPU solve is within relative 1e-7 of the FP64 oracle
  solution at the same tolerance 1e-8.
"""
import os

import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

GRID = 64
CTL = dict(solver=2, method=1, fine_method=1, levels=2, overlap=2, smoothers=1, strong1="0.08",
           radius1=5, maxasize1=400, solve_tolerance="1.0e-8", solve_maxiters=2000)


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


@pytest.fixture(scope="module")
def problem():
    n, r, c, v, b = P.diffusion3d_fv(GRID, sigma=1.0, corr=8.0, seed=0)
    part = P.block_partition(GRID, 4)
    return n, r, c, v, b, part


@pytest.fixture(scope="module")
def oracle_run(problem):
    n, r, c, v, b, part = problem
    O.set_threads(os.cpu_count() or 1)
    try:
        ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(CTL), part=part)
    finally:
        O.set_threads(1)
    assert ro["status"] == 0, ro["errmsg"]
    return ro


def _solver(problem, precision=None, host_only=False):
    n, r, c, v, b, part = problem
    s = D.DougSolver(CTL)
    if precision is not None:
        s.set_option("precision", precision)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.set_partition(part)
    if host_only:
        s.setup_host_only()
    else:
        s.setup()
    return s


def test_setup_bitwise_at_benchmark_controls(problem, oracle_run):
    ro = oracle_run
    s = _solver(problem, host_only=True)
    f, c = s.aggregates()
    assert np.array_equal(f, ro["aggr_fine"])
    assert np.array_equal(c, ro["aggr_coarse"])
    sd = s.subdomains()
    assert len(sd) == len(ro["subdomains"]) == 64
    for a, b in zip(sd, ro["subdomains"]):
        assert np.array_equal(a, b)
    for x, y in zip(s.restriction(), ro["R"][2:]):
        assert np.array_equal(x, y)
    for x, y in zip(s.coarse_matrix(), ro["AC"][1:]):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_fp64_solve_matches_oracle_at_benchmark_controls(problem, oracle_run):
    s = _solver(problem, precision=0)
    x, st = s.solve(allow_not_converged=False)
    ro = oracle_run
    assert abs(st.iterations - ro["iterations"]) <= 1, (st.iterations, ro["iterations"])
    err = np.linalg.norm(x - ro["x"]) / np.linalg.norm(ro["x"])
    assert err <= 1e-10, err
    assert st.nsubdomains == 64
    assert st.ncoarse == ro["AC"][0]


@pytest.mark.gpu
def test_mixed_solve_within_1e7_of_fp64_oracle_at_benchmark_controls(problem, oracle_run):
    s = _solver(problem, precision=1)
    x, st = s.solve(allow_not_converged=False)
    ro = oracle_run
    err = np.linalg.norm(x - ro["x"]) / np.linalg.norm(ro["x"])
    assert err <= 1e-7, err
    assert st.true_rel_residual <= 1.0e-8 * 1.01
    assert abs(st.iterations - ro["iterations"]) <= 3, (st.iterations, ro["iterations"])
