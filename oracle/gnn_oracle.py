"""CPU oracle (test infrastructure only) of the learned block preconditioner's network and
training loss: a float64 PyTorch restatement of the forward pass that ibem_gnn_loss_grad
and ibem_gnn_edge_weights run on the GPU, so that autograd gives the reference gradients.

The network has no counterpart in the reference (iBEMProject solves with Eigen's
fullPivLu, systemSolverElastic3D.h:44-60); this file restates the design documented at
ibem_gnn_param_count in include/ibem_gb300.h:

    h   = relu(x W_in + b_in)                                   node features x (10)
    for 3 layers:
        m_e = relu([h_i, h_j, f_e] W_m + b_m)                   edge e = (i <- j), f_e (7)
        h_i = h_i + relu([h_i, mean_e m_e] W_u + b_u)
    (w_e, alpha_e) = relu([h_i, h_j, f_e] W_o1 + b_o1) W_o2 + b_o2
    L   = sum_q sum_i || z_qi + sum_e (w_e u_qe0 + alpha_e u_qe1) ||^2

Missing neighbours (index -1) are left out of the mean and get w_e = alpha_e = 0.  Parameters are one
flat vector, every W row-major (fan-in x fan-out) followed by its bias, in the order above.
"""
from __future__ import annotations

import numpy as np

H, LAYERS, KNN, NODE_F, EDGE_F, NU, OUT = 64, 3, 16, 10, 7, 24, 2
EIN = 2 * H + EDGE_F
UIN = 2 * H


def layout():
    """(name, shape) of every parameter block, in storage order."""
    out = [("w_in", (NODE_F, H)), ("b_in", (H,))]
    for l in range(LAYERS):
        out += [(f"w_m{l}", (EIN, H)), (f"b_m{l}", (H,)), (f"w_u{l}", (UIN, H)), (f"b_u{l}", (H,))]
    out += [("w_o1", (EIN, H)), ("b_o1", (H,)), ("w_o2", (H, OUT)), ("b_o2", (OUT,))]
    return out


def param_count() -> int:
    return int(sum(np.prod(s) for _, s in layout()))


def unpack(p):
    out, o = {}, 0
    for name, shape in layout():
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def forward(p, nbr, xn, ef):
    """Edge weights (num * 16, 2) for parameters p (torch float64 vector)."""
    import torch
    P = unpack(p)
    num = xn.shape[0]
    nbr = nbr.reshape(num, KNN).long()
    valid = nbr >= 0
    src = torch.where(valid, nbr, torch.zeros_like(nbr))
    dst = torch.arange(num).unsqueeze(1).expand(num, KNN)
    ef = ef.reshape(num, KNN, EDGE_F)
    deg = valid.sum(1, keepdim=True).to(p.dtype)

    def edge_in(h):
        e = torch.cat([h[dst], h[src], ef], dim=2)
        return e * valid.unsqueeze(2).to(p.dtype)

    h = torch.relu(xn @ P["w_in"] + P["b_in"])
    for l in range(LAYERS):
        m = torch.relu(edge_in(h) @ P[f"w_m{l}"] + P[f"b_m{l}"])
        m = m * valid.unsqueeze(2).to(p.dtype)
        agg = m.sum(1) / torch.clamp(deg, min=1.0)
        h = h + torch.relu(torch.cat([h, agg], dim=1) @ P[f"w_u{l}"] + P[f"b_u{l}"])
    o1 = torch.relu(edge_in(h) @ P["w_o1"] + P["b_o1"])
    w = o1 @ P["w_o2"] + P["b_o2"]
    return (w * valid.unsqueeze(2).to(p.dtype)).reshape(-1, OUT)


def loss(p, nbr, xn, ef, z, u):
    """z: (nrhs, num, 24); u: (nrhs, num*16, 2, 24)."""
    w = forward(p, nbr, xn, ef)
    num = xn.shape[0]
    nrhs = z.shape[0]
    corr = (w.reshape(1, num, KNN, OUT, 1) * u.reshape(nrhs, num, KNN, OUT, NU)).sum((2, 3))
    return ((z + corr) ** 2).sum()


def loss_and_grad(p_np, nbr_np, xn_np, ef_np, z_np, u_np):
    """float64 loss and gradient (numpy) of the network at p_np."""
    import torch
    num = xn_np.size // NODE_F
    t = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64))
    p = t(p_np).requires_grad_(True)
    nrhs = z_np.size // (num * NU)
    L = loss(p, torch.from_numpy(np.asarray(nbr_np)), t(xn_np).reshape(num, NODE_F), t(ef_np),
             t(z_np).reshape(nrhs, num, NU), t(u_np).reshape(nrhs, num * KNN, OUT, NU))
    L.backward()
    return float(L.detach()), p.grad.numpy().copy()


def adamw_step(p, g, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
    """Decoupled-weight-decay Adam (Loshchilov & Hutter), bias-corrected moments; numpy."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    p = p - lr * weight_decay * p - lr * mh / (np.sqrt(vh) + eps)
    return p, m, v
