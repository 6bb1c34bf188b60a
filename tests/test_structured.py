"""Structured input (input_type 3): the reference's generated 5-point Laplacian
on a grid_size x grid_size node grid with b = -1 (Distribution_struct.F90:36-147,
one process).  The generated matrix, the host setup built on it and, on the
GPU, the solution are compared with the oracle's restatement and with a dense
direct solve."""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D

from test_setup_parity import _check


def _laplace5(n):
    rows, cols, vals = [], [], []
    for ri in range(1, n + 1):
        for ci in range(1, n + 1):
            r = (ri - 1) * n + ci
            rows.append(r); cols.append(r); vals.append(4.0)
            for ok, c in ((ci > 1, r - 1), (ci < n, r + 1), (ri > 1, r - n), (ri < n, r + n)):
                if ok:
                    rows.append(r); cols.append(c); vals.append(-1.0)
    return np.array(rows), np.array(cols), np.array(vals)


def _ctl(tmp_path, text):
    p = tmp_path / "DOUG.ctl"
    p.write_text(text)
    return str(p)


@pytest.mark.parametrize("grid", [7, 24])
def test_generated_matrix(tmp_path, grid):
    path = _ctl(tmp_path, f"input_type 3\ngrid_size {grid}\nfine_method 1\n")
    s = D.DougSolver()
    s.load_ctl(path)
    n, r, c, v, b = s.input_matrix()
    er, ec, ev = _laplace5(grid)
    assert n == grid * grid
    assert np.array_equal(r, er) and np.array_equal(c, ec) and np.array_equal(v, ev)
    assert np.all(b == -1.0)


def test_grid_size_default_is_100(tmp_path):
    s = D.DougSolver()
    s.load_ctl(_ctl(tmp_path, "input_type 3\nfine_method 1\n"))
    assert s.input_matrix()[0] == 10000


@pytest.mark.parametrize("smoothers,overlap", [(0, -1), (1, 0), (2, 1)])
def test_structured_setup_bitwise(tmp_path, smoothers, overlap):
    text = (f"solver 2\nmethod 1\nfine_method 1\nlevels 2\nsmoothers {smoothers}\noverlap {overlap}\n"
            "strong1 0.08\nradius1 2\ninput_type 3\ngrid_size 30\n")
    path = _ctl(tmp_path, text)
    ro = O.run_ctl(path)
    assert ro["status"] == 0
    s = D.DougSolver()
    s.load_ctl(path)
    s.setup_host_only()
    _check(s, ro)


@pytest.mark.gpu
def test_structured_gpu_solve(tmp_path):
    text = ("solver 2\nmethod 1\nfine_method 1\nlevels 2\nsmoothers 1\noverlap 1\nstrong1 0.08\n"
            "radius1 2\ninput_type 3\ngrid_size 40\nsolve_tolerance 1.0e-10\n")
    path = _ctl(tmp_path, text)
    s = D.DougSolver()
    s.load_ctl(path)
    s.setup()
    x, st = s.solve()
    ro = O.run_ctl(path)
    assert abs(st.iterations - ro["iterations"]) <= 1
    assert np.linalg.norm(x - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"])
    r, c, v = _laplace5(40)
    A = np.zeros((1600, 1600))
    A[r - 1, c - 1] = v
    xd = np.linalg.solve(A, -np.ones(1600))
    assert np.linalg.norm(x - xd) <= 1e-8 * np.linalg.norm(xd)
