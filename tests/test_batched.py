"""Batched independent systems (dg_set_systems).

Every system of a batch must get exactly the setup and the PCG of its own
one-process run: the host setup (aggregates, subdomains, R, AC) is checked bit
for bit against the oracle run on that system alone, and the GPU solutions and
iteration counts against the oracle's per system (FP64: relative 1e-10 and
+-1 iteration; mixed: 1e-7 relative to the oracle's solution).
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


def _systems():
    """Uneven systems: jittered P1 grids of several sizes, a 5-point grid and a 3D diffusion box."""
    out = []
    for nodes, seed in ((21, 1), (34, 2), (13, 3), (47, 4)):
        n, r, c, v, b, _ = P.poisson2d_p1(nodes, seed=seed)
        out.append((n, r, c, v, b))
    n, r, c, v = P.laplace2d(15)[:4]
    out.append((n, r, c, v, np.random.default_rng(7).uniform(-1, 1, n)))
    n, r, c, v, b = P.diffusion3d_fv(10, seed=8)
    out.append((n, r, c, v, b))
    return out


@pytest.fixture(scope="module")
def batch():
    systems = _systems()
    refs = [O.run_coo(n, r, c, v, rhs=b, ctl=_ctl_text(OPTS)) for (n, r, c, v, b) in systems]
    for ro in refs:
        assert ro["status"] == 0
    return systems, refs


def test_batched_setup_is_each_systems_own(batch):
    systems, refs = batch
    s = D.DougSolver(OPTS)
    s.set_systems([t[:4] for t in systems], [t[4] for t in systems])
    s.setup_host_only()
    f, c = s.aggregates()
    sd = s.subdomains()
    Ri, Rj, Rv = s.restriction()
    Ai, Aj, Av = s.coarse_matrix()
    row = agg = sdi = rq = aq = 0
    for (n, *_), ro in zip(systems, refs):
        nf = len(ro["aggr_coarse"])
        fk = f[row:row + n]
        assert np.array_equal(np.where(fk > 0, fk - agg, 0), ro["aggr_fine"])
        ck = c[agg:agg + nf]
        cagg0 = int(c[:agg].max()) if agg else 0
        assert np.array_equal(np.where(ck > 0, ck - cagg0, 0), ro["aggr_coarse"])
        for a, b in zip(sd[sdi:sdi + len(ro["subdomains"])], ro["subdomains"]):
            assert np.array_equal(a - row, b)
        ri, rj, rv = ro["R"][2:]
        k = len(ri)
        assert np.array_equal(Ri[rq:rq + k] - agg, ri) and np.array_equal(Rj[rq:rq + k] - row, rj)
        assert np.array_equal(Rv[rq:rq + k].view(np.int64), rv.view(np.int64))
        ai, aj, av = ro["AC"][1:]
        k2 = len(ai)
        assert np.array_equal(Ai[aq:aq + k2] - agg, ai) and np.array_equal(Aj[aq:aq + k2] - agg, aj)
        assert np.array_equal(Av[aq:aq + k2].view(np.int64), av.view(np.int64))
        row += n
        agg += nf
        sdi += len(ro["subdomains"])
        rq += k
        aq += k2


def test_batched_input_errors():
    s = D.DougSolver(OPTS)
    n, r, c, v = P.laplace2d(5)[:4]
    r2 = r.copy()
    r2[3] = n + 1   # 1-based within the system: n + 1 is out of range
    with pytest.raises(D.DougError):
        s.set_systems([(n, r, c, v), (n, r2, c, v)])
    s.set_systems([(n, r, c, v)] * 2)
    s.set_partition(np.ones(2 * n, np.int32))
    with pytest.raises(D.DougError):
        s.setup_host_only()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_batched_solve_matches_each_system(batch, precision):
    systems, refs = batch
    s = D.DougSolver(OPTS)
    s.set_option("precision", precision)
    s.set_systems([t[:4] for t in systems], [t[4] for t in systems])
    s.setup()
    x, st = s.solve()
    ss = s.system_stats()
    assert np.all(ss["status"] == D.DG_OK)
    assert st.iterations == ss["iterations"].max()
    for k, (xk, ro) in enumerate(zip(s.split(x), refs)):
        assert ss["rel_residual"][k] <= 1.01e-10
        if precision == 0:
            assert abs(int(ss["iterations"][k]) - ro["iterations"]) <= 1, k
            assert np.linalg.norm(xk - ro["x"]) <= 1e-10 * np.linalg.norm(ro["x"]), k
        else:
            assert np.linalg.norm(xk - ro["x"]) <= 1e-7 * np.linalg.norm(ro["x"]), k
    assert np.all(np.diff(ss["seconds"][np.argsort(ss["iterations"])]) >= 0)
    # a second solve with new right-hand sides reuses the setup
    b2 = np.concatenate([np.random.default_rng(k).uniform(-1, 1, t[0]) for k, t in enumerate(systems)])
    x2, _ = s.solve(b2)
    for k, (t, xk) in enumerate(zip(systems, s.split(x2))):
        n, r, c, v, _ = t
        xd = O.spd_solve(n, r - 1, c - 1, v, b2[sum(u[0] for u in systems[:k]):][:n])
        assert np.linalg.norm(xk - xd) <= 1e-7 * np.linalg.norm(xd), k
