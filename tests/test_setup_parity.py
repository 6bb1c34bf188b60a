"""Bit-for-bit parity of the product's host setup with the oracle.

Aggregates, subdomain index lists (in the reference's order), the
restriction R and the coarse matrix AC (entry order, pattern and values) must
be identical.  These run without a GPU: dg_setup finishes the host part and
then reports that no device is visible.
"""
import numpy as np
import pytest

import oracle as O
import doug_gb300 as D
from doug_gb300 import problems as P

from conftest import GOLDEN

BASE = "solver 2\nmethod 1\nfine_method 1\nlevels 2\n"


def _solver(n, r, c, v, b, ctl, part=None):
    s = D.DougSolver()
    for line in ctl.strip().split("\n"):
        k, val = line.split()
        s.set_option(k, val)
    s.set_matrix_coo(n, r, c, v)
    s.set_rhs(b)
    if part is not None:
        s.set_partition(part)
    s.setup_host_only()
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


@pytest.mark.parametrize("levels,smoothers,overlap", [(2, s, o) for s in (0, 1, 2) for o in (-1, 0, 1, 2)])
def test_lap16x16_setup_bitwise(levels, smoothers, overlap):
    ov = f"solver 2\nmethod 1\nfine_method 1\nlevels {levels}\nsmoothers {smoothers}\noverlap {overlap}\n"
    ro = O.run_ctl(f"{GOLDEN}/lap16x16/DOUG.ctl", ov)
    assert ro["status"] == 0
    s = D.DougSolver()
    for line in ov.strip().split("\n"):
        k, v = line.split()
        s.set_option(k, v)
    s.load_ctl(f"{GOLDEN}/lap16x16/DOUG.ctl")
    s.setup_host_only()
    _check(s, ro)


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("ctl", [
    BASE + "overlap 1\nsmoothers 1\nstrong1 0.08\nradius1 2\n",
    BASE + "overlap -1\nsmoothers 2\nstrong1 0.08\nradius1 2\nsymmstruct T\nsymmnumeric T\n",
    BASE + "overlap 0\nsmoothers 0\nstrong1 0.67\nradius1 1\n",
    BASE + "overlap 2\nsmoothers 1\nstrong1 0.25\nradius1 3\nradius2 2\n",
])
def test_poisson2d_setup_bitwise(seed, ctl):
    n, r, c, v, b, _ = P.poisson2d_p1(41 + 8 * seed, seed=seed)
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, setup_only=True)
    assert ro["status"] == 0, ro["errmsg"]
    _check(_solver(n, r, c, v, b, ctl), ro)


def test_cartesian_branch_when_strong1_unset():
    # strong1 unset -> theta = -1 (every entry strong); n a perfect square ->
    # Cartesian aggregates (SpMtx_aggregation.F90:124,332-346)
    n, r, c, v, b = P.laplace2d(12)
    ctl = BASE + "overlap 1\nsmoothers 1\nradius1 2\n"
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, setup_only=True)
    assert ro["status"] == 0
    assert ro["nagr_fine"] == 36
    _check(_solver(n, r, c, v, b, ctl), ro)


@pytest.mark.parametrize("parts", [2, 3])
def test_diffusion3d_partition_setup_bitwise(parts):
    n, r, c, v, b = P.diffusion3d_fv(12, seed=3)
    part = P.block_partition(12, parts)
    ctl = BASE + "overlap 2\nsmoothers 1\nstrong1 0.08\nradius1 2\n"
    ro = O.run_coo(n, r, c, v, rhs=b, ctl=ctl, part=part, setup_only=True)
    assert ro["status"] == 0
    assert len(ro["subdomains"]) == parts ** 3
    _check(_solver(n, r, c, v, b, ctl, part=part), ro)


def test_shuffled_input_order_changes_nothing_structural_in_sets():
    # the reference keeps input order inside rows; a permuted triplet order
    # must still give the same aggregates when ties are absent
    n, r, c, v, b, _ = P.poisson2d_p1(33, seed=5)
    ctl = BASE + "overlap 1\nsmoothers 1\nstrong1 0.08\nradius1 2\n"
    perm = np.random.default_rng(0).permutation(len(v))
    ro = O.run_coo(n, r[perm], c[perm], v[perm], rhs=b, ctl=ctl, setup_only=True)
    _check(_solver(n, r[perm], c[perm], v[perm], b, ctl), ro)
