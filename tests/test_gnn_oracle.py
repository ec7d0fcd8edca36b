"""Pins of the learned-preconditioner oracle (CPU): the float64 autograd gradient of
oracle/gnn_oracle.py against central finite differences, and its AdamW step against
torch.optim.AdamW, so that the GPU kernels are checked against a trusted restatement."""
import numpy as np
import pytest

import gnn_oracle as go


def small_graph(num=12, nrhs=2, seed=0):
    rng = np.random.default_rng(seed)
    nbr = np.full((num, go.KNN), -1, dtype=np.int32)
    for i in range(num):
        others = [j for j in range(num) if j != i]
        k = min(go.KNN, len(others) - (i % 3))  # ragged: some slots stay empty
        nbr[i, :k] = rng.permutation(others)[:k]
    xn = rng.standard_normal((num, go.NODE_F))
    ef = rng.standard_normal((num * go.KNN, go.EDGE_F)) * (nbr.reshape(-1, 1) >= 0)
    z = rng.standard_normal((nrhs, num, go.NU))
    u = rng.standard_normal((nrhs, num * go.KNN, go.OUT, go.NU)) * 0.3
    p = rng.uniform(-0.2, 0.2, go.param_count())
    return p, nbr.ravel(), xn.ravel(), ef.ravel(), z.ravel(), u.ravel()


def test_oracle_gradient_matches_finite_differences():
    p, nbr, xn, ef, z, u = small_graph()
    L, g = go.loss_and_grad(p, nbr, xn, ef, z, u)
    rng = np.random.default_rng(1)
    idx = rng.choice(p.size, 40, replace=False)
    # include the output layer and a first-layer weight
    idx = np.concatenate([idx, [p.size - 1, p.size - 2, p.size - 3, 0]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (go.loss_and_grad(pp, nbr, xn, ef, z, u)[0] - go.loss_and_grad(pm, nbr, xn, ef, z, u)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_missing_neighbours_get_zero_weight():
    import torch
    p, nbr, xn, ef, z, u = small_graph()
    w = go.forward(torch.from_numpy(p), torch.from_numpy(nbr), torch.from_numpy(xn).reshape(-1, go.NODE_F),
                   torch.from_numpy(ef)).numpy()
    assert np.all(w[nbr < 0] == 0)
    assert np.any(w[nbr >= 0] != 0)
    assert w.shape == (nbr.size, go.OUT)


def test_oracle_adamw_matches_torch():
    import torch
    rng = np.random.default_rng(2)
    p0 = rng.standard_normal(50)
    t = torch.nn.Parameter(torch.from_numpy(p0.copy()))
    opt = torch.optim.AdamW([t], lr=1e-2, betas=(0.9, 0.999), eps=1e-8, weight_decay=0.05)
    p, m, v = p0.copy(), np.zeros(50), np.zeros(50)
    for step in range(1, 6):
        g = rng.standard_normal(50)
        t.grad = torch.from_numpy(g.copy())
        opt.step()
        p, m, v = go.adamw_step(p, g, m, v, step, 1e-2, weight_decay=0.05)
    np.testing.assert_allclose(p, t.detach().numpy(), rtol=1e-12, atol=1e-14)
