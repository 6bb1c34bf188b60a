"""Adjoint gradients through the GB300 solve (doug_gb300.autograd).

The loss is L = sum over right-hand sides of ||x - x_target||^2.  Gradients
with respect to the COO matrix values, the right-hand sides and per-element
conductivities are checked against an FP64 dense reference gradient
(lambda = A^-1 dL/dx with numpy) and, for the conductivities, against central
finite differences of L computed with the same solver.  The reference has no
gradients; these tests pin the adjoint itself.
"""
import numpy as np
import pytest

import doug_gb300 as D
from doug_gb300 import problems as P

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OPTS = dict(solver=2, method=1, fine_method=1, levels=2, overlap=1, smoothers=1, strong1="0.08", radius1=2,
            solve_tolerance="1.0e-12", solve_maxiters=2000)


def _dense(n, r, c, v):
    A = np.zeros((n, n))
    np.add.at(A, (r - 1, c - 1), v)
    return A


def test_coo_gradients_match_dense_reference():
    from doug_gb300.autograd import coo_solve
    n, r, c, v, b, _ = P.poisson2d_p1(35, seed=11)
    rng = np.random.default_rng(0)
    B = rng.uniform(-1, 1, (n, 3))
    Xt = rng.uniform(-1, 1, (n, 3)) * 1e-2
    vals = torch.tensor(v, dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(B, dtype=torch.float64, device="cuda", requires_grad=True)
    s = D.DougSolver(OPTS)
    X = coo_solve(s, n, r, c, vals, bt)
    L = ((X - torch.tensor(Xt, device="cuda")) ** 2).sum()
    L.backward()
    A = _dense(n, r, c, v)
    Xd = np.linalg.solve(A, B)
    assert np.abs(X.detach().cpu().numpy() - Xd).max() <= 1e-9 * np.abs(Xd).max()
    Lam = np.linalg.solve(A, 2 * (Xd - Xt))
    gb = bt.grad.cpu().numpy()
    assert np.abs(gb - Lam).max() <= 1e-8 * np.abs(Lam).max()
    gv_ref = -(Lam[r - 1] * Xd[c - 1]).sum(axis=1)
    gv = vals.grad.numpy()
    assert np.abs(gv - gv_ref).max() <= 1e-8 * np.abs(gv_ref).max()


@pytest.mark.parametrize("precision", [0, 1])
def test_element_gradients_match_fd_and_dense(precision):
    from doug_gb300.autograd import element_solve
    nodes = 33
    rng = np.random.default_rng(5)
    ntri = 2 * (nodes - 1) ** 2
    kappa0 = np.exp(0.5 * rng.standard_normal(ntri))
    ngf, eptr, efree, Kb, erhs, _ = P.poisson2d_p1_elements(nodes=nodes, seed=2)   # unit conductivities
    B = rng.uniform(-1, 1, (ngf, 2))
    Xt = rng.uniform(-1, 1, (ngf, 2)) * 1e-2
    opts = dict(OPTS, solve_tolerance="1.0e-10" if precision else "1.0e-12")
    s = D.DougSolver(opts)
    if precision:
        s.set_option("precision", precision)
    xt = torch.tensor(Xt, device="cuda")
    bt = torch.tensor(B, device="cuda")

    def loss(kap, grad=False):
        k = torch.tensor(kap, dtype=torch.float64, requires_grad=grad)
        X = element_solve(s, ngf, eptr, efree, Kb, erhs, k, bt)
        L = ((X - xt) ** 2).sum()
        if grad:
            L.backward()
            return L.item(), k.grad.numpy().copy(), X.detach().cpu().numpy()
        return L.item()

    L0, g, X = loss(kappa0, grad=True)
    # dense FP64 reference gradient: dL/dkappa_e = -sum_c lambda_c^T K_e x_c
    nf = np.diff(eptr)
    off = np.concatenate([[0], np.cumsum(nf * nf)])
    A = np.zeros((ngf, ngf))
    for e in range(ntri):
        f = efree[eptr[e]:eptr[e + 1]] - 1
        Ke = Kb[off[e]:off[e + 1]].reshape(nf[e], nf[e]).T
        A[np.ix_(f, f)] += kappa0[e] * Ke
    Xd = np.linalg.solve(A, B)
    Lam = np.linalg.solve(A, 2 * (Xd - Xt))
    g_ref = np.zeros(ntri)
    for e in range(ntri):
        f = efree[eptr[e]:eptr[e + 1]] - 1
        Ke = Kb[off[e]:off[e + 1]].reshape(nf[e], nf[e]).T
        g_ref[e] = -np.einsum("ic,ij,jc->", Lam[f], Ke, Xd[f])
    tol_dense = 1e-5 if precision else 1e-8
    assert np.abs(g - g_ref).max() <= tol_dense * np.abs(g_ref).max()
    # central finite differences on seeded elements
    for e in rng.choice(np.flatnonzero(nf > 0), 6, replace=False):
        h = 1e-4 * kappa0[e]
        kp, km = kappa0.copy(), kappa0.copy()
        kp[e] += h
        km[e] -= h
        fd = (loss(kp) - loss(km)) / (2 * h)
        assert abs(fd - g[e]) <= 1e-5 * max(abs(g_ref).max(), 1e-30) + 1e-5 * abs(fd)
