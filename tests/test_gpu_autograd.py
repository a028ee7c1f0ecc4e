"""Differentiable aggregation through the C ABI: FP64 gradcheck (finite
differences) on a 2048-vertex Erdos-Renyi graph of average degree 8, the
adjoint against a cuSPARSE transpose product, and a 2-layer GNN's forward and
backward against dense FP64 torch."""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def dense(g, dtype=torch.float64, device="cuda"):
    D = torch.zeros(g.nrows, g.ncols, dtype=dtype, device=device)
    rows = torch.from_numpy(np.repeat(np.arange(g.nrows), np.diff(g.rowptr))).to(device)
    D[rows, torch.from_numpy(g.colind.astype(np.int64)).to(device)] = 1
    return D


def test_gradcheck_fp64_er2048(pkg, cuda):
    g = pkg.erdos_renyi(2048, 8.0, seed=11)
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    X = torch.randn(g.ncols, 3, dtype=torch.float64, device=cuda, requires_grad=True)
    assert torch.autograd.gradcheck(lambda x: pkg.aggregate(A, x), (X,), eps=1e-6, atol=1e-7, rtol=1e-6)
    v = torch.randn(g.ncols, dtype=torch.float64, device=cuda, requires_grad=True)
    assert torch.autograd.gradcheck(lambda x: pkg.aggregate(A, x), (v,), eps=1e-6, atol=1e-7, rtol=1e-6)


@pytest.mark.parametrize("T", [4, 8, 32])
def test_adjoint_matches_cusparse_transpose(pkg, cuda, T):
    rng = np.random.default_rng(T)
    g = pkg.from_edges(rng.integers(0, 900, 6000), rng.integers(0, 1500, 6000), nrows=900, ncols=1500)
    A = pkg.B2SRMatrix.from_graph(g, T, device=cuda)
    X = torch.randn(g.ncols, 40, dtype=torch.float64, device=cuda, requires_grad=True)
    Y = pkg.aggregate(A, X)
    dY = torch.randn_like(Y)
    (dX,) = torch.autograd.grad(Y, X, dY)
    crow = torch.from_numpy(g.rowptr.astype(np.int64)).to(cuda)
    col = torch.from_numpy(g.colind.astype(np.int64)).to(cuda)
    Acsr = torch.sparse_csr_tensor(crow, col, torch.ones(g.nnz, dtype=torch.float64, device=cuda),
                                   size=(g.nrows, g.ncols))
    want = torch.sparse.mm(Acsr.t().to_sparse_csr(), dY)
    torch.testing.assert_close(dX, want, rtol=1e-12, atol=1e-12)
    torch.testing.assert_close(Y, Acsr @ X.detach(), rtol=1e-12, atol=1e-12)


def test_adjoint_is_deterministic(pkg, cuda):
    g = pkg.rmat(12, 16, seed=4)
    A = pkg.B2SRMatrix.from_graph(g, 4, device=cuda)
    X = torch.randn(g.ncols, 128, device=cuda, requires_grad=True)
    dY = torch.randn(g.nrows, 128, device=cuda)
    grads = []
    for _ in range(3):
        (dX,) = torch.autograd.grad(pkg.aggregate(A, X), X, dY)
        grads.append(dX)
    assert torch.equal(grads[0], grads[1]) and torch.equal(grads[1], grads[2])


def test_two_layer_gnn_forward_backward(pkg, cuda):
    g = pkg.rmat(11, 8, seed=2)
    A = pkg.B2SRMatrix.from_graph(g, 8, device=cuda)
    gen = torch.Generator().manual_seed(0)
    net = pkg.SumAggGNN(16, 128, 8, generator=gen, dtype=torch.float64, device=cuda)
    X = torch.randn(g.ncols, 16, dtype=torch.float64, device=cuda, requires_grad=True)
    out = net(A, X)
    loss = (out ** 2).sum()
    loss.backward()
    D = dense(g)
    W1 = net.W1.detach().clone().requires_grad_(True)
    W2 = net.W2.detach().clone().requires_grad_(True)
    X2 = X.detach().clone().requires_grad_(True)
    ref = D @ (torch.relu(D @ X2 @ W1) @ W2)
    (ref ** 2).sum().backward()
    torch.testing.assert_close(out, ref, rtol=1e-10, atol=1e-10)
    torch.testing.assert_close(X.grad, X2.grad, rtol=1e-10, atol=1e-9)
    torch.testing.assert_close(net.W1.grad, W1.grad, rtol=1e-10, atol=1e-9)
    torch.testing.assert_close(net.W2.grad, W2.grad, rtol=1e-10, atol=1e-9)
