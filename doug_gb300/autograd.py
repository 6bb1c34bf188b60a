"""Differentiable solves x = A^-1 b through the GB300 solver (torch.autograd).

The forward pass solves A x = b with the library's preconditioned CG (all
right-hand side columns together, dg_solve_multi; the numeric factors are
kept for the backward pass).  The backward pass is the
adjoint: A is symmetric, so lambda = A^-1 dL/dx is one more solve with the
same factors, and

    dL/db    = lambda
    dL/dA_ij = -lambda_i x_j              (on A's pattern, ``dg_grad_matrix``)
    dL/ds_e  = -lambda^T (dA/ds_e) x      (a factor s_e of element e's matrix,
                                            ``dg_grad_elements``)

summed over right-hand sides.  Only x is stored between the passes (no CG
history).  Tensors are FP64 on the current CUDA device; the matrix values
and element factors pass through the host because the setup (aggregation,
restriction, coarse matrix) depends on them.
"""
from __future__ import annotations

import numpy as np
import torch

from . import DougSolver


def _as_cols(b: torch.Tensor) -> torch.Tensor:
    return b.unsqueeze(1) if b.dim() == 1 else b


def _solve_cols(solver: DougSolver, B: torch.Tensor) -> torch.Tensor:
    """Solves A X = B on the current stream (B: n x r, FP64 CUDA): the r
    right-hand sides together (one shared factorisation, every kernel over
    all of them)."""
    stream = torch.cuda.current_stream().cuda_stream
    Bt = B.t().contiguous()                 # columns contiguous
    Xt = torch.empty_like(Bt)
    if Bt.shape[0] == 1:
        solver.solve_device(Bt[0].data_ptr(), Xt[0].data_ptr(), stream)
    else:
        solver.solve_multi_device(Bt.shape[0], Bt.data_ptr(), Xt.data_ptr(), stream)
    return Xt.t()


class _CooSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, b, solver, n, rows1, cols1):
        solver.set_matrix_coo(n, rows1, cols1, values.detach().cpu().numpy())
        solver.setup()
        X = _solve_cols(solver, _as_cols(b).detach())
        ctx.solver = solver
        ctx.squeeze = b.dim() == 1
        ctx.vdev = values.device
        ctx.save_for_backward(X)
        return X[:, 0].clone() if ctx.squeeze else X

    @staticmethod
    def backward(ctx, gx):
        (X,) = ctx.saved_tensors
        solver = ctx.solver
        G = _as_cols(gx.contiguous())
        Lam = _solve_cols(solver, G.contiguous())
        stream = torch.cuda.current_stream().cuda_stream
        nnz = int(solver.input_matrix()[1].shape[0])
        gv = torch.zeros(nnz, dtype=torch.float64, device=X.device)
        vdev = ctx.vdev
        tmp = torch.empty_like(gv)
        for c in range(X.shape[1]):
            lam = Lam[:, c].contiguous()
            x = X[:, c].contiguous()
            solver.grad_matrix(lam.data_ptr(), x.data_ptr(), tmp.data_ptr(), stream)
            gv += tmp
        gb = Lam[:, 0].clone() if ctx.squeeze else Lam
        return gv.to(vdev), gb, None, None, None, None


def coo_solve(solver: DougSolver, n: int, rows1, cols1, values: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """x = A^-1 b with A given by 1-based COO triplets (rows1, cols1, values);
    b of shape (n,) or (n, r).  Differentiable in values and b.  The solver's
    control words (set before the call) choose the preconditioner; the option
    reuse_factors is switched on so that the backward solve reuses the factors."""
    solver.set_option("reuse_factors", 1)
    return _CooSolve.apply(values, b, solver, n, np.asarray(rows1, np.int32), np.asarray(cols1, np.int32))


class _ElementSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kappa, b, solver, ngf, eptr, efree, Kbase, erhs):
        k = kappa.detach().cpu().numpy()
        nf = np.diff(eptr)
        emat = Kbase * np.repeat(k, nf * nf)
        solver.set_elements(ngf, eptr, efree, emat, erhs)
        solver.setup()
        ctx.b_given = b is not None
        if b is None:
            b = torch.tensor(solver.input_matrix()[4], dtype=torch.float64, device="cuda")
        X = _solve_cols(solver, _as_cols(b).detach())
        ctx.solver = solver
        ctx.squeeze = b.dim() == 1
        ctx.kappa = kappa.detach().to(torch.float64)
        ctx.kdev = kappa.device
        ctx.save_for_backward(X)
        return X[:, 0].clone() if ctx.squeeze else X

    @staticmethod
    def backward(ctx, gx):
        (X,) = ctx.saved_tensors
        solver = ctx.solver
        G = _as_cols(gx.contiguous())
        Lam = _solve_cols(solver, G.contiguous())
        stream = torch.cuda.current_stream().cuda_stream
        nell = ctx.kappa.shape[0]
        gs = torch.zeros(nell, dtype=torch.float64, device=X.device)
        tmp = torch.empty_like(gs)
        for c in range(X.shape[1]):
            lam = Lam[:, c].contiguous()
            x = X[:, c].contiguous()
            solver.grad_elements(lam.data_ptr(), x.data_ptr(), tmp.data_ptr(), stream)
            gs += tmp
        # A_e = kappa_e K_e: dL/dkappa_e = dL/ds_e / kappa_e
        gk = (gs / ctx.kappa.to(gs.device)).to(ctx.kdev)
        gb = (Lam[:, 0].clone() if ctx.squeeze else Lam) if ctx.b_given else None
        return gk, gb, None, None, None, None, None, None


def element_solve(solver: DougSolver, ngf: int, eptr, efree, Kbase, erhs, kappa: torch.Tensor,
                  b: torch.Tensor | None = None) -> torch.Tensor:
    """x = A(kappa)^-1 b for A = sum_e kappa_e K_e assembled from element
    matrices K_e (elemental input: freedom lists eptr/efree, Kbase the K_e
    column by column).  b defaults to the assembled element right-hand sides.
    Differentiable in kappa (one value per element) and b."""
    solver.set_option("reuse_factors", 1)
    return _ElementSolve.apply(kappa, b, solver, int(ngf), np.asarray(eptr, np.int32),
                               np.asarray(efree, np.int32), np.asarray(Kbase, np.float64),
                               np.asarray(erhs, np.float64))
