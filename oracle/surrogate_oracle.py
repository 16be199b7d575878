"""CPU reference of the learned surrogate potential (TEST INFRASTRUCTURE ONLY).

The surrogate has no counterpart in the reference; this file states its
mathematics in plain PyTorch (CPU, float64) so that the GPU kernels of
emdee_gb300/csrc/surrogate.cu can be checked:

- descriptors  G_i[c, k] = sum_{j: s_j = c, r_ij < rc} exp(-(r_ij - mu_k)^2 / (2 w^2)) fc(r_ij),
  fc(r) = (cos(pi r / rc) + 1) / 2;
- per-species networks E_i = w3 . silu(silu(G_i W1 + b1) W2 + b2) + b3;
- forces F = -dE/dR (autograd through the descriptors);
- the training loss  wE sum_c (E_c - Et_c)^2 / (N^2 C) + wF sum |F - Ft|^2 / (3 N C)
  and its parameter gradient (double backward).

``bf16=True`` rounds the network's GEMM operands to bfloat16 at the points where the
tensor-core kernels do (weights, layer inputs, back-propagated layer gradients),
with float32 arithmetic elsewhere, so kernel outputs can be compared tightly.
"""
import math

import torch

NG, NS, DIN, H = 16, 2, 32, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + DIN * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
PER_SPECIES = OFF_B3 + 1


def unpack(params, sp):
    p = params[sp * PER_SPECIES:(sp + 1) * PER_SPECIES]
    return dict(W1=p[OFF_W1:OFF_B1].reshape(DIN, H), b1=p[OFF_B1:OFF_W2], W2=p[OFF_W2:OFF_B2].reshape(H, H),
                b2=p[OFF_B2:OFF_W3], w3=p[OFF_W3:OFF_B3], b3=p[OFF_B3])


def pair_table(R, L, rc):
    """All pairs i != j within rc (minimum image): (i, j, r, unit vectors)."""
    N = R.shape[0]
    d = R[:, None, :] - R[None, :, :]
    d = d - L * torch.round(d / L)
    r = torch.sqrt((d * d).sum(-1) + torch.eye(N, dtype=R.dtype) * 1e6)
    i, j = torch.nonzero(r < rc, as_tuple=True)
    return i, j, r[i, j], d[i, j] / r[i, j][:, None]


def descriptors(R, L, species, rc, mu0, mu15, width):
    """R [N, 3] (float64, may require grad); species [N] in {0, 1}; returns G [N, 32]."""
    N = R.shape[0]
    i, j, r, _ = pair_table(R, L, rc)
    mu = mu0 + torch.arange(NG, dtype=R.dtype) * (mu15 - mu0) / 15.0
    fc = 0.5 * (torch.cos(math.pi * r / rc) + 1.0)
    g = torch.exp(-((r[:, None] - mu[None, :]) ** 2) / (2 * width * width)) * fc[:, None]
    cols = species[j][:, None] * NG + torch.arange(NG)[None, :]
    G = torch.zeros(N, DIN, dtype=R.dtype)
    G = G.index_put((i[:, None].expand(-1, NG), cols), g, accumulate=True)
    return G


def silu(x):
    return x * torch.sigmoid(x)


def _q(x, bf16):
    return x.to(torch.bfloat16).to(torch.float32) if bf16 else x


def network(G, species, params, bf16=False):
    """Per-atom energies E [N] and dE/dG [N, 32] by the explicit forward/backward
    passes of the kernel (float32 when bf16, else float64)."""
    dt = torch.float32 if bf16 else torch.float64
    E = torch.zeros(G.shape[0], dtype=dt)
    dG = torch.zeros(G.shape[0], DIN, dtype=dt)
    for sp in range(NS):
        idx = torch.nonzero(species == sp).flatten()
        if len(idx) == 0:
            continue
        w = {k: v.to(dt) for k, v in unpack(params, sp).items()}
        W1, W2 = _q(w["W1"], bf16), _q(w["W2"], bf16)
        x = _q(G[idx].to(dt), bf16)
        z1 = x @ W1 + w["b1"]
        a1 = silu(z1)
        z2 = _q(a1, bf16) @ W2 + w["b2"]
        s2 = torch.sigmoid(z2)
        E[idx] = silu(z2) @ w["w3"] + w["b3"]
        dz2 = w["w3"] * s2 * (1 + z2 * (1 - s2))
        da1 = _q(dz2, bf16) @ W2.T
        s1 = torch.sigmoid(z1)
        dz1 = da1 * s1 * (1 + z1 * (1 - s1))
        dG[idx] = _q(dz1, bf16) @ W1.T
    return E, dG


def energy(R, L, species, params, rc, mu0, mu15, width):
    """Total surrogate energy (float64, differentiable in R and params)."""
    G = descriptors(R, L, species, rc, mu0, mu15, width)
    E = torch.zeros((), dtype=R.dtype)
    for sp in range(NS):
        idx = torch.nonzero(species == sp).flatten()
        w = unpack(params, sp)
        E = E + (silu(silu(G[idx] @ w["W1"] + w["b1"]) @ w["W2"] + w["b2"]) @ w["w3"] + w["b3"]).sum()
    return E


def forces(R, L, species, params, rc, mu0, mu15, width):
    R = R.detach().clone().requires_grad_(True)
    E = energy(R, L, species, params, rc, mu0, mu15, width)
    (g,) = torch.autograd.grad(E, R)
    return E.detach(), -g


def loss_gradient(Rs, L, species, params, rc, mu0, mu15, width, Etrue, Ftrue, wE, wF):
    """Loss and its gradient in the parameters over configurations Rs [C, N, 3]."""
    params = params.detach().clone().requires_grad_(True)
    C, N = Rs.shape[0], Rs.shape[1]
    lossE = torch.zeros((), dtype=torch.float64)
    lossF = torch.zeros((), dtype=torch.float64)
    for c in range(C):
        R = Rs[c].detach().clone().requires_grad_(True)
        E = energy(R, L, species, params, rc, mu0, mu15, width)
        (g,) = torch.autograd.grad(E, R, create_graph=True)
        lossE = lossE + (E - Etrue[c]) ** 2
        lossF = lossF + ((-g - Ftrue[c]) ** 2).sum()
    loss = wE * lossE / (N * N * C) + wF * lossF / (3 * N * C)
    (grad,) = torch.autograd.grad(loss, params)
    return float(wE * lossE.detach() / (N * N * C)), float(wF * lossF.detach() / (3 * N * C)), grad
