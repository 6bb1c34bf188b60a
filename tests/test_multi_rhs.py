"""Several right-hand sides of one matrix solved together (dg_solve_multi).

Each right-hand side runs its own PCG (own scalars and stopping test) while
the factorisations are shared and every kernel covers all of them.  Every
column must match the oracle's solve of that right-hand side (FP64: relative
1e-10, iterations +-1; mixed: 1e-7 against the FP64 direct solve).
"""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

OPTS = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08", radius1=2,
            solve_tolerance="1.0e-10", solve_maxiters=1000)


def _ctl_text(d):
    return "".join(f"{k} {v}\n" for k, v in d.items())


def test_multi_needs_setup():
    n, r, c, v, b = P.laplace2d(6)
    s = D.DougSolver(OPTS)
    s.set_matrix_coo(n, r, c, v)
    with pytest.raises(D.DougError) as ei:
        s.solve_multi(np.ones((n, 3)))
    assert ei.value.status == D.DG_NOT_READY


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_multi_rhs_matches_oracle(precision):
    n, r, c, v, b0, _ = P.poisson2d_p1(41, seed=12)
    rng = np.random.default_rng(3)
    B = np.column_stack([b0] + [rng.uniform(-1, 1, n) for _ in range(4)] + [np.zeros(n) + 1.0])
    s = D.DougSolver(OPTS)
    s.set_option("precision", precision)
    s.set_matrix_coo(n, r, c, v)
    s.setup()
    X, st = s.solve_multi(B)
    ss = s.system_stats()
    assert np.all(ss["status"] == D.DG_OK)
    assert st.iterations == ss["iterations"].max()
    for k in range(B.shape[1]):
        assert ss["rel_residual"][k] <= 1.01e-10
        if precision == 0:
            ro = O.run_coo(n, r, c, v, rhs=B[:, k], ctl=_ctl_text(OPTS))
            assert abs(int(ss["iterations"][k]) - ro["iterations"]) <= 1, k
            assert np.linalg.norm(X[:, k] - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"]), k
        else:
            xd = O.spd_solve(n, r - 1, c - 1, v, B[:, k])
            assert np.linalg.norm(X[:, k] - xd) <= 1e-7 * np.linalg.norm(xd), k
    # a single right-hand side through the single-system path gives the same column
    x1, st1 = s.solve(B[:, 1])
    assert abs(st1.iterations - int(ss["iterations"][1])) <= 1
    assert np.linalg.norm(x1 - X[:, 1]) <= (1e-10 if precision == 0 else 1e-7) * np.linalg.norm(x1)


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", [0, 1])
def test_multi_rhs_3d_with_partition(schedule):
    N = 14
    n, r, c, v, b = P.diffusion3d_fv(N, seed=9)
    part = P.block_partition(N, 2)
    opts = dict(OPTS, overlap=2)
    s = D.DougSolver(opts)
    s.set_option("solve_schedule", schedule)
    s.set_matrix_coo(n, r, c, v)
    s.set_partition(part)
    s.setup()
    rng = np.random.default_rng(8)
    B = rng.uniform(-1, 1, (n, 3))
    X, st = s.solve_multi(B)
    for k in range(3):
        ro = O.run_coo(n, r, c, v, rhs=B[:, k], ctl=_ctl_text(opts), part=part)
        assert np.linalg.norm(X[:, k] - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"]), k


@pytest.mark.gpu
def test_queue_wait_times_out_and_the_handle_recovers():
    # The dependency-driven schedule (solve_schedule 1) with a forward task
    # whose done flag is never published (queue_skip_publish, a failure-test
    # word) and a short wait limit (2e6 cycles, about 1 ms): the tasks waiting
    # on it give up, the kernels finish, and dg_solve reports DG_CUDA_ERROR
    # with the timeout message.  The same handle, set up again without the
    # withheld flag, then solves correctly.
    N = 14
    n, r, c, v, b = P.diffusion3d_fv(N, seed=9)
    part = P.block_partition(N, 2)
    opts = dict(OPTS, overlap=2)
    s = D.DougSolver(opts)
    s.set_option("solve_schedule", 1)
    s.set_option("queue_wait_cycles", 2000000)
    s.set_option("queue_skip_publish", 0)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    s.set_partition(part)
    s.setup()
    with pytest.raises(D.DougError) as ei:
        s.solve()
    assert ei.value.status == D.DG_CUDA_ERROR
    assert "timed out" in str(ei.value)
    s.set_option("queue_skip_publish", -1)
    s.setup()
    x, st = s.solve(allow_not_converged=False)
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(opts), part=part)
    assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
