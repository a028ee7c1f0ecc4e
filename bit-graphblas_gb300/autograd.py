"""Differentiable sum aggregation over a B2SR adjacency: Y = A . X.

The binary structure A carries no gradient.  backward computes dX = A^T . dY
with the same dense-RHS kernel on the transposed B2SR, which the library packs
once per matrix and caches; both directions are deterministic (fixed
summation order, no atomics).  FP32 and FP64 features are supported (FP64 for
finite-difference checks).
"""
from __future__ import annotations

import torch

from .matrix import B2SRMatrix


class B2SRAggregate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X: torch.Tensor, A: B2SRMatrix) -> torch.Tensor:
        ctx.A = A
        squeeze = X.dim() == 1
        X2 = X.unsqueeze(1) if squeeze else X
        Y = A.spmm(X2.contiguous())[: A.nrows]
        ctx.squeeze = squeeze
        return Y.squeeze(1) if squeeze else Y

    @staticmethod
    def backward(ctx, dY: torch.Tensor):
        A: B2SRMatrix = ctx.A
        dY2 = dY.unsqueeze(1) if ctx.squeeze else dY
        At = A.transpose()
        # A^T's tile-rows cover A's columns; its B2SR rows past ncols are padding
        dYp = dY2.contiguous()
        if dYp.shape[0] < At.ncols:  # A's padded row count is what A^T reads
            dYp = torch.nn.functional.pad(dYp, (0, 0, 0, At.ncols - dYp.shape[0]))
        dX = At.spmm(dYp)[: A.ncols]
        return (dX.squeeze(1) if ctx.squeeze else dX), None


def aggregate(A: B2SRMatrix, X: torch.Tensor) -> torch.Tensor:
    """Y[i] = sum of X[j] over the neighbours j of i (row i of A), differentiable in X."""
    return B2SRAggregate.apply(X, A)


class SumAggGNN(torch.nn.Module):
    """Two-layer sum-aggregation GNN: Y = A . relu(A . X . W1) . W2."""

    def __init__(self, in_dim: int, hidden: int, out_dim: int, generator: torch.Generator | None = None,
                 dtype=torch.float32, device=None):
        super().__init__()
        w1 = torch.randn(in_dim, hidden, generator=generator, dtype=dtype) / in_dim ** 0.5
        w2 = torch.randn(hidden, out_dim, generator=generator, dtype=dtype) / hidden ** 0.5
        self.W1 = torch.nn.Parameter(w1.to(device))
        self.W2 = torch.nn.Parameter(w2.to(device))

    def forward(self, A: B2SRMatrix, X: torch.Tensor) -> torch.Tensor:
        H = torch.relu(aggregate(A, X) @ self.W1)
        return aggregate(A, H @ self.W2)
