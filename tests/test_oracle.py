"""Pin the CPU oracle against the reference's own fixtures.

The reference's harness accepts a run when ||x - x_ref||_2 <= 1e-6
(scripts/doug/test.py:159-172); its run matrix for doug_aggr on one process
is levels {1,2} x smoothers {0,1,2} x overlap {-1,0,1,2}
(tests/tests_all.conf:32-82).  The fixture solutions are direct solves, and the
control files ask for tolerance 1e-12, so the oracle is also held to 1e-9.
"""
import os

import numpy as np
import pytest

import oracle as O

from conftest import GOLDEN

RUNS_2LEV = [(2, s, o) for s in (0, 1, 2) for o in (-1, 0)]
RUNS_1LEV = [(1, 0, o) for o in (-1, 0, 1, 2)]


def _ov(levels, smoothers, overlap):
    return f"solver 2\nmethod 1\nfine_method 1\nlevels {levels}\nsmoothers {smoothers}\noverlap {overlap}\n"


@pytest.mark.parametrize("levels,smoothers,overlap", RUNS_2LEV + RUNS_1LEV)
def test_lap16x16_matches_reference_solution(levels, smoothers, overlap):
    r = O.run_ctl(os.path.join(GOLDEN, "lap16x16", "DOUG.ctl"), _ov(levels, smoothers, overlap))
    assert r["status"] == 0, r["errmsg"]
    ref = O.read_vector(os.path.join(GOLDEN, "lap16x16", "csolution.xdr"), 2, r["n"])
    err = np.linalg.norm(r["x"] - ref)
    assert err <= 1e-6          # the reference harness rule
    assert err <= 1e-9          # tolerance 1e-12 solve of a well-conditioned system
    assert 1 <= r["iterations"] < 100


@pytest.mark.parametrize("levels,smoothers,overlap", RUNS_2LEV + RUNS_1LEV)
def test_lap4x4_matches_reference_solution(levels, smoothers, overlap):
    r = O.run_ctl(os.path.join(GOLDEN, "lap4x4", "DOUG.ctl"), _ov(levels, smoothers, overlap))
    assert r["status"] == 0, r["errmsg"]
    ref = O.read_vector(os.path.join(GOLDEN, "lap4x4", "solution_correct.dat"), 1, r["n"])
    assert np.linalg.norm(r["x"] - ref) <= 1e-12


def test_rhs_formats_agree():
    n = 225
    b = O.read_vector(os.path.join(GOLDEN, "lap16x16", "rhs.xdr"), 2, n)
    assert np.all(b == 1.0)
    b4 = O.read_vector(os.path.join(GOLDEN, "lap4x4", "rhs.dat"), 1, 9)
    assert b4.shape == (9,) and np.isfinite(b4).all()


def test_direct_solve_oracle_agrees_with_fixture():
    n, nnz, ii, jj, vv = O.read_assembled(os.path.join(GOLDEN, "lap16x16", "Lap16x16.txt"), 0)
    assert (n, nnz) == (225, 1065)
    x = O.spd_solve(n, ii - 1, jj - 1, vv, np.ones(n))
    ref = O.read_vector(os.path.join(GOLDEN, "lap16x16", "csolution.xdr"), 2, n)
    assert np.abs(x - ref).max() < 1e-12


def test_control_value_parsing_quirks():
    # integers: I10 reads the first ten characters, blanks ignored
    assert O.parse_value("i10", "2") == 2
    assert O.parse_value("i10", "-1") == -1
    # reals: F10.5 gives digits without a decimal point five implied decimals
    assert O.parse_value("f10.5", "0.67e0") == pytest.approx(0.67)
    assert O.parse_value("f10.5", "1.0e-12") == pytest.approx(1e-12)
    assert O.parse_value("f10.5", "8") == pytest.approx(8e-5)
    assert O.parse_value("f10.5", "1e-8") == pytest.approx(1e-13)
    assert O.parse_value("l1", "T") == 1 and O.parse_value("l1", "f") == 0


def test_missing_fine_method_is_an_error():
    # doug_aggr aborts with 'Wrong fine method' when fine_method is unset (aggr.F90:216-226)
    r = O.run_ctl(os.path.join(GOLDEN, "lap16x16", "DOUG.ctl"), "")
    assert r["status"] != 0 and "fine method" in r["errmsg"]


def test_setup_structure_lap16x16():
    r = O.run_ctl(os.path.join(GOLDEN, "lap16x16", "DOUG.ctl"), _ov(2, 1, 1))
    assert r["status"] == 0
    n = r["n"]
    # every node is in exactly one fine aggregate; coarse aggregates cover fine aggregates
    assert sorted(set(r["aggr_fine"].tolist())) == list(range(1, r["nagr_fine"] + 1))
    assert sorted(set(r["aggr_coarse"].tolist())) == list(range(1, r["nagr_coarse"] + 1))
    # subdomains = coarse aggregates + one overlap layer, union covers all nodes
    cover = np.zeros(n + 1, int)
    for s in r["subdomains"]:
        assert len(set(s.tolist())) == len(s)
        cover[s] += 1
    assert (cover[1:] >= 1).all()
    nR, ncR, Ri, Rj, Rv = r["R"]
    assert (nR, ncR) == (r["nagr_fine"], n)
    # smoothed prolongator rows sum to (1-omega) + ... ; columns of P sum to one on
    # interior nodes for a Laplacian with zero row sums, so check P^T 1 for those
    P = np.zeros((n, nR))
    P[Rj - 1, Ri - 1] += Rv
    assert np.isfinite(P).all()


@pytest.mark.parametrize("levels,smoothers,overlap,iters", [(2, 1, 1, -1), (2, 0, -1, 2), (1, 0, 0, 4)])
def test_oracle_sgs_fine_preconditioner_matches_fixture(levels, smoothers, overlap, iters):
    # fine_method 2: symmetric Gauss-Seidel on every subdomain (FinePreconditioner_sgs.F90)
    ref = O.read_vector(os.path.join(GOLDEN, "lap16x16", "csolution.xdr"), 2, 225)
    ov = (f"solver 2\nmethod 1\nfine_method 2\nlevels {levels}\nsmoothers {smoothers}\n"
          f"overlap {overlap}\nnum_iters {iters}\n")
    r = O.run_ctl(os.path.join(GOLDEN, "lap16x16", "DOUG.ctl"), ov)
    assert r.get("status", 0) == 0, r
    assert np.linalg.norm(r["x"] - ref) <= 1e-9


def test_oracle_method5_is_additive_and_2_3_are_rejected():
    path = os.path.join(GOLDEN, "lap16x16", "DOUG.ctl")
    base = "solver 2\nfine_method 1\nlevels 2\nsmoothers 1\noverlap 1\n"
    r1 = O.run_ctl(path, "method 1\n" + base)
    r5 = O.run_ctl(path, "method 5\n" + base)
    assert r1["iterations"] == r5["iterations"] and np.array_equal(r1["x"], r5["x"])
    for m in (2, 3):
        r = O.run_ctl(path, f"method {m}\n" + base)
        assert r["status"] != 0 and "residual" in r["errmsg"]


def test_sparse_cholesky_is_an_exact_solve():
    # the oracle's exact subdomain / coarse solver (nested dissection +
    # multifrontal Cholesky, standing in for UMFPACK) against a dense solve
    from doug_gb300 import problems as P
    for N, seed in ((9, 1), (14, 2)):
        n, r, c, v, b = P.diffusion3d_fv(N, seed=seed)
        A = np.zeros((n, n))
        np.add.at(A, (r - 1, c - 1), v)
        x = O.spd_solve(n, r - 1, c - 1, v, b)
        xd = np.linalg.solve(A, b)
        assert np.linalg.norm(x - xd) <= 1e-12 * np.linalg.norm(xd)
    # a non-SPD matrix is refused
    with pytest.raises(RuntimeError):
        O.spd_solve(2, np.array([0, 1, 0, 1]), np.array([0, 1, 1, 0]), np.array([1.0, 1.0, 2.0, 2.0]),
                    np.ones(2))


def test_oracle_threads_do_not_change_results():
    # subdomain factorisations and solves in parallel, summed in subdomain
    # order afterwards: bit-identical solutions for any thread count
    from doug_gb300 import problems as P
    n, r, c, v, b = P.diffusion3d_fv(12, seed=3)
    part = P.block_partition(12, 2)
    ctl = ("solver 2\nmethod 1\nfine_method 1\nlevels 2\noverlap 2\nsmoothers 1\nstrong1 0.08\n"
           "radius1 2\nsolve_tolerance 1.0e-10\n")
    out = []
    for t in (1, 3):
        O.set_threads(t)
        try:
            ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, part=part)
        finally:
            O.set_threads(1)
        assert ro["status"] == 0, ro["errmsg"]
        out.append(ro)
    assert out[0]["iterations"] == out[1]["iterations"]
    assert np.array_equal(out[0]["x"], out[1]["x"])


def test_session_repeats_the_one_shot_run():
    from doug_gb300 import problems as P
    n, r, c, v, b, _ = P.poisson2d_p1(33, seed=2)
    ctl = "solver 2\nmethod 1\nfine_method 1\nlevels 2\noverlap 1\nsmoothers 1\nstrong1 0.08\nradius1 2\n"
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl)
    S = O.Session(n, r, c, v, ctl)
    for _ in range(2):
        rs = S.solve(b)
        assert rs["status"] == 0
        assert rs["iterations"] == ro["iterations"]
        assert np.array_equal(rs["x"], ro["x"])
    S.close()
