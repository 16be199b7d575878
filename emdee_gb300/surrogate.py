"""Surrogate-proposal hybrid Monte Carlo on the GB300 library.

Pieces (device work in the CUDA library; PyTorch only holds device buffers and
draws random numbers):

- ``Surrogate``: the learned potential of ``csrc/surrogate.cu`` (radial
  descriptors, one 32-64-64-1 SiLU network per species on the BF16 tensor
  cores, adjoint forces, energy+force training with Adam);
- ``SurrogateEnergy``: a ``torch.autograd.Function`` whose backward is the
  adjoint force kernel;
- ``Chains``: many systems of the same shape run as one replica batch
  (``EmDee_replicas_*``), the exact Hamiltonian;
- ``plain_hmc`` / ``surrogate_hmc``: HMC whose trajectories use the exact forces
  or the surrogate forces, both accepted or rejected on the exact FP64
  Hamiltonian H = U + K, so both sample the exact Boltzmann distribution;
- ``integrated_autocorrelation`` / ``ess``: Sokal's automatic-window estimate of
  the integrated autocorrelation time (c = 5) and the effective sample size.
"""
import ctypes as C
import math
import time

import numpy as np
import torch

from .workloads import fcc  # noqa: F401  (re-exported for callers building systems)

# binary Lennard-Jones glass former (80:20), reduced units
BINARY = dict(eps=[[1.0, 1.5], [1.5, 0.5]], sig=[[1.0, 0.8], [0.8, 0.88]], rho=1.2, T=0.8, rc=2.5, skin=0.3)
DESCRIPTOR = dict(rc=2.5, mu0=0.8, mu15=2.5, width=0.15, skin=0.8)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def simple_cubic(N, L, seed, jitter=0.05):
    n = round(N ** (1.0 / 3.0))
    if n ** 3 != N:
        raise ValueError("N must be a cube")
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    R = (g + 0.5) * (L / n)
    return R + np.random.default_rng(seed).uniform(-jitter, jitter, size=R.shape)


def binary_system(lib, N, seed, precision=0, types=None):
    """One system of the mixture: types 1 (80 %) and 2 (20 %), simple-cubic start."""
    L = (N / BINARY["rho"]) ** (1.0 / 3.0)
    if types is None:
        types = np.where(np.random.default_rng(seed).permutation(N) < int(0.8 * N), 1, 2)
    md = lib.system(1, 1, BINARY["rc"], BINARY["skin"], N, types, [1.0, 1.0])
    lib.EmDee_set_precision(md, precision)
    for a, b in ((1, 1), (2, 2), (1, 2)):
        lib.EmDee_set_pair_model(md, a, b, lib.EmDee_pair_lj_cut(BINARY["eps"][a - 1][b - 1],
                                                                  BINARY["sig"][a - 1][b - 1]), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", simple_cubic(N, L, seed))
    return md, L, types


class Chains:
    """C systems of the mixture advanced together; exact energies and forces."""

    def __init__(self, lib, C_, N, seed, device="cuda"):
        self.lib, self.C, self.N = lib, C_, N
        self.mds, self.types = [], None
        for c in range(C_):
            md, self.L, t = binary_system(lib, N, seed + c, types=self.types)
            self.types = t
            self.mds.append(md)
        self.arr = (C.POINTER(type(self.mds[0])) * C_)(*[C.pointer(m) for m in self.mds])
        self.batch = lib.lib.EmDee_replicas_create(C_, C.cast(self.arr, C.c_void_p))
        self.device = device
        self.steps = 0

    def potential(self):
        return np.array([m.Energy.Potential for m in self.mds])

    def gather(self, which="R"):
        """[C, N, 3] FP64 device tensor copied from the systems."""
        out = torch.empty((self.C, self.N, 3), dtype=torch.float64, device=self.device)
        torch.cuda.synchronize()
        self.lib.lib.EmDee_replicas_gather(self.batch, _ITEM[which], _ptr(out))
        return out

    def scatter(self, t, which="R"):
        torch.cuda.synchronize()
        self.lib.lib.EmDee_replicas_scatter(self.batch, _ITEM[which], _ptr(t.contiguous()))

    def set_momenta(self, P):
        self.scatter(P, "P")

    def run(self, steps, dt, nprop):
        self.lib.lib.EmDee_replicas_run(self.batch, steps, dt, nprop)
        self.steps += steps

    def evaluate(self):
        self.lib.lib.EmDee_replicas_evaluate(self.batch)

    def checkpoint(self):
        self.lib.lib.EmDee_replicas_checkpoint(self.batch)

    def restore(self, mask):
        m = (C.c_int * self.C)(*[int(x) for x in mask])
        self.lib.lib.EmDee_replicas_restore(self.batch, m)

    def close(self):
        self.lib.lib.EmDee_replicas_destroy(self.batch)
        for m in self.mds:
            self.lib.lib.EmDee_destroy(C.byref(m))


_ITEM = {"R": b"coordinates", "P": b"momenta", "F": b"forces"}


class Surrogate:
    """The learned potential for C chains of N atoms (types shared by the chains)."""

    def __init__(self, lib, C_, N, L, types, device="cuda"):
        self.lib, self.C, self.N, self.L = lib, C_, N, L
        t = np.ascontiguousarray(types, dtype=np.int32)
        self.h = lib.lib.EmDee_surrogate_create(C_, N, L, t.ctypes.data_as(C.c_void_p), DESCRIPTOR["rc"],
                                                DESCRIPTOR["skin"], DESCRIPTOR["mu0"], DESCRIPTOR["mu15"],
                                                DESCRIPTOR["width"])
        self.nparam = lib.lib.EmDee_surrogate_param_count()
        self.device = device
        self.stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self.grad = torch.zeros(self.nparam, dtype=torch.float32, device=device)
        self.adam_step = 0

    def init_params(self, seed, e_atom):
        """Glorot-uniform weights, zero biases, b3 = mean energy per atom."""
        rng = np.random.default_rng(seed)
        p = np.zeros(self.nparam, dtype=np.float32)
        per = self.nparam // 2
        for s in range(2):
            o = s * per
            lim1, lim2 = math.sqrt(6 / (32 + 64)), math.sqrt(6 / (64 + 64))
            p[o:o + 2048] = rng.uniform(-lim1, lim1, 2048)
            p[o + 2048 + 64:o + 2048 + 64 + 4096] = rng.uniform(-lim2, lim2, 4096)
            p[o + per - 65:o + per - 1] = rng.uniform(-0.1, 0.1, 64)
            p[o + per - 1] = e_atom
        self.set_params(p)

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.lib.lib.EmDee_surrogate_set_params(self.h, p.ctypes.data_as(C.c_void_p))
        self.adam_step = 0

    def get_params(self):
        p = np.zeros(self.nparam, dtype=np.float32)
        self.lib.lib.EmDee_surrogate_get_params(self.h, p.ctypes.data_as(C.c_void_p))
        return p

    def descriptors(self, R, rebuild=True):
        G = torch.empty((self.C * self.N, 32), dtype=torch.float32, device=self.device)
        self.lib.lib.EmDee_surrogate_descriptors(self.h, _ptr(R), _ptr(G), int(rebuild), self.stream)
        return G

    def forces(self, R, rebuild=True):
        F = torch.empty_like(R)
        E = torch.empty(self.C, dtype=torch.float64, device=self.device)
        self.lib.lib.EmDee_surrogate_forces(self.h, _ptr(R), _ptr(F), _ptr(E), int(rebuild), self.stream)
        return E, F

    def atom_outputs(self):
        Ea = torch.empty(self.C * self.N, dtype=torch.float32, device=self.device)
        dG = torch.empty((self.C * self.N, 32), dtype=torch.float32, device=self.device)
        self.lib.lib.EmDee_surrogate_atom_outputs(self.h, _ptr(Ea), _ptr(dG), self.stream)
        return Ea, dG

    def gradient(self, R, Etrue, Ftrue, wE=1.0, wF=1.0):
        loss = (C.c_double * 2)()
        self.lib.lib.EmDee_surrogate_gradient(self.h, _ptr(R), _ptr(Etrue), _ptr(Ftrue), wE, wF, _ptr(self.grad),
                                              loss, self.stream)
        return loss[0], loss[1], self.grad

    def adam(self, lr):
        self.adam_step += 1
        self.lib.lib.EmDee_surrogate_adam(self.h, _ptr(self.grad), lr, self.adam_step, self.stream)

    def trajectory(self, R, P, F, steps, dt):
        E = torch.empty(self.C, dtype=torch.float64, device=self.device)
        self.lib.lib.EmDee_surrogate_trajectory(self.h, _ptr(R), _ptr(P), _ptr(F), _ptr(E), steps, dt, self.stream)
        return E

    def close(self):
        self.lib.lib.EmDee_surrogate_destroy(self.h)


class SurrogateEnergy(torch.autograd.Function):
    """E(R) summed over chains; backward through the adjoint force kernel."""

    @staticmethod
    def forward(ctx, R, model):
        E, F = model.forces(R.detach().contiguous())
        ctx.save_for_backward(F)
        return E.sum()

    @staticmethod
    def backward(ctx, gE):
        (F,) = ctx.saved_tensors
        return -gE * F, None


# ---- sampling ---------------------------------------------------------------------------


def integrated_autocorrelation(x, c=5.0):
    """Sokal's automatic windowing: tau = 1 + 2 sum_{t=1..W} rho(t), W the smallest t >= c tau(t)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    if n < 4 or np.var(x) == 0:
        return float("nan")
    y = x - x.mean()
    f = np.fft.rfft(y, n=2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n]
    acf /= acf[0]
    tau = 1.0
    for t in range(1, n):
        tau += 2.0 * acf[t]
        if t >= c * tau:
            return max(tau, 1.0)
    return max(tau, 1.0)


def ess(series):
    """Effective sample size summed over chains; series [chains, samples]."""
    total = 0.0
    for s in series:
        tau = integrated_autocorrelation(s)
        if np.isfinite(tau):
            total += len(s) / tau
    return total


def draw_momenta(C_, N, kT, gen, device="cuda"):
    return torch.randn((C_, N, 3), dtype=torch.float64, device=device, generator=gen) * math.sqrt(kT)


def plain_hmc(chains, iterations, steps, dt, kT, seed):
    """HMC with exact forces (replica batch); returns U samples [C, iterations], acceptance, seconds."""
    gen = torch.Generator(device="cuda").manual_seed(seed)
    rng = np.random.default_rng(seed)
    chains.evaluate()
    U = chains.potential()
    out, acc = [], 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(iterations):
        P = draw_momenta(chains.C, chains.N, kT, gen)
        K0 = 0.5 * (P * P).sum(dim=(1, 2)).cpu().numpy()
        chains.set_momenta(P)
        chains.checkpoint()
        chains.run(steps, dt, steps)   # energies at the last step of the trajectory
        U1 = chains.potential()
        K1 = np.array([m.Kinetic.Total for m in chains.mds])
        dH = (U1 + K1) - (U + K0)
        accept = rng.random(chains.C) < np.exp(np.minimum(0.0, -dH / kT))
        chains.restore(~accept)
        U = np.where(accept, U1, U)
        acc += int(accept.sum())
        out.append(U.copy())
    torch.cuda.synchronize()
    return np.array(out).T, acc / (iterations * chains.C), time.perf_counter() - t0


def surrogate_hmc(chains, model, iterations, steps, dt, kT, seed):
    """HMC whose trajectories run on the surrogate forces, accepted on the exact H."""
    gen = torch.Generator(device="cuda").manual_seed(seed)
    rng = np.random.default_rng(seed)
    chains.evaluate()
    U = chains.potential()
    out, acc, far = [], 0, 0
    limit = 0.5 * DESCRIPTOR["skin"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(iterations):
        R0 = chains.gather("R")
        P = draw_momenta(chains.C, chains.N, kT, gen)
        K0 = 0.5 * (P * P).sum(dim=(1, 2))
        R = R0.clone()
        _, F = model.forces(R, rebuild=True)
        model.trajectory(R, P, F, steps, dt)
        K1 = 0.5 * (P * P).sum(dim=(1, 2))
        moved = (R - R0).norm(dim=2).max(dim=1).values
        chains.checkpoint()
        chains.scatter(R, "R")
        chains.evaluate()
        U1 = chains.potential()
        dH = (U1 + K1.cpu().numpy()) - (U + K0.cpu().numpy())
        ok = (moved < limit).cpu().numpy()   # the surrogate lists stayed valid along the path
        far += int((~ok).sum())
        accept = ok & (rng.random(chains.C) < np.exp(np.minimum(0.0, -dH / kT)))
        chains.restore(~accept)
        U = np.where(accept, U1, U)
        acc += int(accept.sum())
        out.append(U.copy())
    torch.cuda.synchronize()
    return np.array(out).T, acc / (iterations * chains.C), time.perf_counter() - t0, far


# ---- training ---------------------------------------------------------------------------


def force_rmse(model, Rs, Fs, batch):
    """Root-mean-square force error of the model over configurations (one batch at a time)."""
    se, n = 0.0, 0
    for b in range(0, Rs.shape[0] - batch + 1, batch):
        _, F = model.forces(Rs[b:b + batch].double().contiguous())
        se += float(((F - Fs[b:b + batch].double()) ** 2).sum())
        n += F.numel()
    return math.sqrt(se / max(n, 1))


def generate_data(chains, snapshots, every, dt, kT, seed, burn=2000):
    """Configurations with exact energies and forces from plain MD of the chains, with the
    momenta redrawn at kT before every stretch of `every` steps (keeps the temperature).
    Returns R [S, N, 3] (FP64), E [S] (FP64), F [S, N, 3] (FP32 on the device, FP64 copies
    on demand)."""
    gen = torch.Generator(device="cuda").manual_seed(seed)
    for b in range(0, burn, every):
        chains.set_momenta(draw_momenta(chains.C, chains.N, kT, gen))
        chains.run(every, dt, every)
    Rs, Es, Fs = [], [], []
    rounds = (snapshots + chains.C - 1) // chains.C
    for r in range(rounds):
        chains.set_momenta(draw_momenta(chains.C, chains.N, kT, gen))
        chains.run(every, dt, every)
        chains.evaluate()
        Rs.append(chains.gather("R").float())
        Fs.append(_gather_forces(chains).float())
        Es.append(torch.tensor(chains.potential(), dtype=torch.float64, device="cuda"))
    return torch.cat(Rs)[:snapshots], torch.cat(Es)[:snapshots], torch.cat(Fs)[:snapshots]


def _gather_forces(chains):
    return chains.gather("F")


def train(model, Rs, Es, Fs, epochs, lr, batch, seed, wE=1.0, wF=1.0, log=None, lr_min=None):
    """Adam on energy + force matching.  The learning rate follows a cosine from lr to
    lr_min (default lr / 50) over all steps; the model's chain count is the batch size.
    Returns the mean (energy, force) loss of every epoch."""
    S = Rs.shape[0]
    g = torch.Generator(device="cuda").manual_seed(seed)
    lr_min = lr / 50.0 if lr_min is None else lr_min
    nb_epoch = S // batch
    total = max(1, epochs * nb_epoch)
    history = []
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(S, device="cuda", generator=g)
        lE = lF = 0.0
        nb = 0
        for b in range(0, S - batch + 1, batch):
            idx = perm[b:b + batch]
            R = Rs[idx].double().contiguous()
            E = Es[idx].contiguous()
            F = Fs[idx].double().contiguous()
            a, c, _ = model.gradient(R, E, F, wE, wF)
            model.adam(lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * step / total)))
            step += 1
            lE += a
            lF += c
            nb += 1
        history.append((lE / nb, lF / nb))
        if log:
            log(ep, lE / nb, lF / nb)
    return history
