"""The coarse-level setup on the GPU (dg_coarse_setup.cu): prolongator
smoothing, the stable re-bucketings and the three first-touch Galerkin
SpGEMMs (CoarseMtx.F90:128-516, SpMtx_op_AB.f90:39-200,
SpMtx_arrangement.F90:58-292) give R, P and AC bit for bit equal to the
oracle's and to the host path (device_setup 0), and the coarse aggregation
and subdomains built from that AC are the oracle's too.
"""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

BASE = "solver 2\nmethod 1\nfine_method 1\nlevels 2\n"


def _solver(n, r, c, v, b, ctl, part=None, device_setup=1):
    s = D.DougSolver()
    for line in ctl.strip().split("\n"):
        k, val = line.split()
        s.set_option(k, val)
    s.set_option("device_setup", device_setup)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    if part is not None:
        s.set_partition(part)
    s.setup()
    return s


def _check(s, ro):
    f, c = s.aggregates()
    assert np.array_equal(f, ro["aggr_fine"])
    assert np.array_equal(c, ro["aggr_coarse"])
    sd = s.subdomains()
    assert len(sd) == len(ro["subdomains"])
    for a, b in zip(sd, ro["subdomains"]):
        assert np.array_equal(a, b)
    for x, y in zip(s.restriction(), ro["R"][2:]):
        assert np.array_equal(x, y)
    for x, y in zip(s.coarse_matrix(), ro["AC"][1:]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("smoothers,overlap", [(0, -1), (1, -1), (1, 0), (1, 2)])
def test_lap16x16_device_setup_bitwise(smoothers, overlap):
    ov = BASE + f"smoothers {smoothers}\noverlap {overlap}\n"
    ro = O.run_ctl(f"{GOLDEN}/lap16x16/DOUG.ctl", ov)
    assert ro["status"] == 0
    s = D.DougSolver()
    for line in ov.strip().split("\n"):
        k, v = line.split()
        s.set_option(k, v)
    s.load_ctl(f"{GOLDEN}/lap16x16/DOUG.ctl")
    s.setup()
    assert s.setup_phases()["coarse_on_device"]
    _check(s, ro)


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("ctl", [
    BASE + "overlap 1\nsmoothers 1\nstrong1 0.08\nradius1 2\n",
    BASE + "overlap 0\nsmoothers 0\nstrong1 0.67\nradius1 1\n",
    BASE + "overlap 2\nsmoothers 1\nstrong1 0.25\nradius1 3\nradius2 2\n",
])
def test_poisson2d_device_setup_bitwise(seed, ctl):
    n, r, c, v, b, _ = P.poisson2d_p1(41 + 8 * seed, seed=seed)
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, setup_only=True)
    assert ro["status"] == 0, ro["errmsg"]
    s = _solver(n, r, c, v, b, ctl)
    assert s.setup_phases()["coarse_on_device"]
    _check(s, ro)


def test_smoothers_2_stay_on_the_host():
    n, r, c, v, b, _ = P.poisson2d_p1(33, seed=2)
    ctl = BASE + "overlap -1\nsmoothers 2\nstrong1 0.08\nradius1 2\n"
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, setup_only=True)
    s = _solver(n, r, c, v, b, ctl)
    assert not s.setup_phases()["coarse_on_device"]
    _check(s, ro)


def test_benchmark_controls_64cube_device_setup_bitwise():
    n, r, c, v, b = P.diffusion3d_fv(64, sigma=1.0, corr=8.0, seed=0)
    part = P.block_partition(64, 4)
    ctl = BASE + "overlap 2\nsmoothers 1\nstrong1 0.08\nradius1 5\nmaxasize1 400\n"
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, part=part, setup_only=True)
    assert ro["status"] == 0
    s = _solver(n, r, c, v, b, ctl, part=part)
    ph = s.setup_phases()
    assert ph["coarse_on_device"] and ph["coarse_s"] > 0
    _check(s, ro)
    # the host path gives the same bits
    sh = _solver(n, r, c, v, b, ctl, part=part, device_setup=0)
    assert not sh.setup_phases()["coarse_on_device"]
    for x, y in zip(s.restriction(), sh.restriction()):
        assert np.array_equal(x, y)
    for x, y in zip(s.coarse_matrix(), sh.coarse_matrix()):
        assert np.array_equal(x, y)


def test_repeated_input_entries_take_the_one_lane_product():
    # a matrix given with a repeated (row, column) triplet: S^T then repeats
    # a column in a row, and the first-touch product walks those rows with
    # one lane; the oracle keeps both entries as the reference does
    n, r, c, v, b, _ = P.poisson2d_p1(25, seed=3)
    k = np.flatnonzero(r != c)[:40]
    r2 = np.concatenate([r, r[k]])
    c2 = np.concatenate([c, c[k]])
    v2 = np.concatenate([v, 0.25 * v[k]])
    ctl = BASE + "overlap 1\nsmoothers 1\nstrong1 0.08\nradius1 2\n"
    ro = O.run_coo(n, r2, c2, v2, rhs=b, ctl=ctl, setup_only=True)
    assert ro["status"] == 0, ro["errmsg"]
    s = _solver(n, r2, c2, v2, b, ctl)
    assert s.setup_phases()["coarse_on_device"]
    _check(s, ro)
