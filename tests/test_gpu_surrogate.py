"""GPU checks of the learned surrogate potential (emdee_gb300/csrc/surrogate.cu)
against the CPU reference in oracle/surrogate_oracle.py (PyTorch, float64):

- descriptors (FP32 kernel vs FP64 reference);
- the tensor-core network: per-atom energies and dE/dG against the reference's
  explicit forward/backward with bfloat16 operands at the kernel's rounding points;
- the adjoint force kernel: against the reference adjoint for the same dE/dG, and
  against central finite differences of Phi(R) = sum_i dE/dG_i . G_i(R);
- the autograd.Function: its backward returns minus the kernel forces;
- the training gradient (forward-over-reverse kernels) against the reference's
  double-backward gradient of the energy + force loss (direction and size);
- a short training run lowers the loss; HMC with exact and with surrogate
  proposals accepts on the exact Hamiltonian."""
import os
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

pytestmark = pytest.mark.gpu

DESC = dict(rc=2.5, mu0=0.8, mu15=2.5, width=0.15)


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def so():
    import surrogate_oracle
    return surrogate_oracle


def config(N, C, seed):
    from emdee_gb300.surrogate import BINARY, simple_cubic
    L = (N / BINARY["rho"]) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    types = np.where(rng.permutation(N) < int(0.8 * N), 1, 2)
    R = np.stack([simple_cubic(N, L, seed + c, jitter=0.25) for c in range(C)])
    return R, L, types


def random_params(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.2 * scale, n).astype(np.float32)
    return p


def model(gpu, C, N, L, types):
    from emdee_gb300.surrogate import Surrogate
    return Surrogate(gpu, C, N, L, types)


@pytest.mark.parametrize("N", [512, 1728])
def test_descriptors(gpu, so, N):
    R, L, types = config(N, 2, 1)
    m = model(gpu, 2, N, L, types)
    G = m.descriptors(torch.tensor(R, device="cuda")).cpu().double().reshape(2, N, 32)
    for c in range(2):
        ref = so.descriptors(torch.tensor(R[c]), L, torch.tensor(types - 1), **DESC)
        assert torch.allclose(G[c], ref, rtol=1e-4, atol=1e-5), (G[c] - ref).abs().max()
    m.close()


@pytest.fixture(params=["tcgen05", "mma.sync"])
def engine(request):
    """The network on the tcgen05 tensor cores (default) or on mma.sync."""
    old = os.environ.get("EMDEE_SG_MMA")
    if request.param == "mma.sync":
        os.environ["EMDEE_SG_MMA"] = "sync"
    else:
        os.environ.pop("EMDEE_SG_MMA", None)
    yield request.param
    if old is None:
        os.environ.pop("EMDEE_SG_MMA", None)
    else:
        os.environ["EMDEE_SG_MMA"] = old


def test_network_engines_agree(gpu):
    """tcgen05 (M = 128 tiles, TMEM accumulators) and mma.sync (64-atom tiles) round
    the same BF16 operands; their FP32 sums differ only in order."""
    N = 1728
    R, L, types = config(N, 3, 12)
    m = model(gpu, 3, N, L, types)
    m.set_params(random_params(m.nparam, 13))
    Rt = torch.tensor(R, device="cuda")
    out = {}
    for eng in ("sync", None):
        if eng:
            os.environ["EMDEE_SG_MMA"] = eng
        else:
            os.environ.pop("EMDEE_SG_MMA", None)
        E, F = m.forces(Rt)
        Ea, dG = m.atom_outputs()
        out[eng] = (E.cpu(), F.cpu(), Ea.cpu(), dG.cpu())
    os.environ.pop("EMDEE_SG_MMA", None)
    a, b = out["sync"], out[None]
    ea = (a[2] - b[2]).abs().max().item()
    rg = ((a[3] - b[3]).norm() / a[3].norm()).item()
    rf = ((a[1] - b[1]).norm() / a[1].norm()).item()
    print("tcgen05 vs mma.sync: atom energies max %.2e, dE/dG rel %.2e, forces rel %.2e" % (ea, rg, rf))
    assert ea < 1e-4 and rg < 1e-4 and rf < 1e-4   # the same BF16 products, summed in another order
    m.close()


def test_network_energies_and_gradients(gpu, so, engine):
    N = 1728
    R, L, types = config(N, 2, 2)
    m = model(gpu, 2, N, L, types)
    p = random_params(m.nparam, 3)
    m.set_params(p)
    Rt = torch.tensor(R, device="cuda")
    E, F = m.forces(Rt)
    Ea, dG = m.atom_outputs()
    G = m.descriptors(Rt, rebuild=False).cpu()
    sp = torch.tensor(np.tile(types - 1, 2))
    Eref, dGref = so.network(G, sp, torch.tensor(p), bf16=True)
    assert torch.allclose(Ea.cpu(), Eref, rtol=2e-3, atol=2e-3), (Ea.cpu() - Eref).abs().max()
    rel = (dG.cpu() - dGref).norm() / dGref.norm()
    assert rel < 5e-3, rel
    assert np.allclose(E.cpu().numpy(), Eref.reshape(2, N).double().sum(1).numpy(), rtol=1e-5)
    m.close()


def test_adjoint_forces(gpu, so):
    N = 512
    R, L, types = config(N, 1, 4)
    m = model(gpu, 1, N, L, types)
    m.set_params(random_params(m.nparam, 5))
    Rt = torch.tensor(R, device="cuda")
    E, F = m.forces(Rt)
    _, dG = m.atom_outputs()
    # reference adjoint: F = -d/dR [sum_i dG_i . G_i(R)] with dG fixed
    Rr = torch.tensor(R[0]).requires_grad_(True)
    G = so.descriptors(Rr, L, torch.tensor(types - 1), **DESC)
    (g,) = torch.autograd.grad((G * dG.cpu().double()).sum(), Rr)
    rel = (F[0].cpu() + g).norm() / g.norm()
    assert rel < 1e-4, rel
    # central differences of Phi(R) = sum_i dG_i . G_i(R) on the GPU descriptors
    rng = np.random.default_rng(6)
    for a in rng.choice(N, 4, replace=False):
        for d in range(3):
            h = 1e-3
            Rp, Rm = R.copy(), R.copy()
            Rp[0, a, d] += h
            Rm[0, a, d] -= h
            Gp = m.descriptors(torch.tensor(Rp, device="cuda")).double()
            Gm = m.descriptors(torch.tensor(Rm, device="cuda")).double()
            fd = -((Gp - Gm) * dG.double()).sum() / (2 * h)
            assert abs(fd.item() - F[0, a, d].item()) < 2e-3 * max(1.0, abs(F[0, a, d].item()))
    m.close()


def test_autograd_function(gpu):
    from emdee_gb300.surrogate import SurrogateEnergy
    N = 512
    R, L, types = config(N, 1, 7)
    m = model(gpu, 1, N, L, types)
    m.set_params(random_params(m.nparam, 8))
    Rt = torch.tensor(R, device="cuda", requires_grad=True)
    E = SurrogateEnergy.apply(Rt, m)
    E.backward()
    _, F = m.forces(Rt.detach())
    assert torch.equal(Rt.grad, -F)
    m.close()


def test_training_gradient(gpu, so):
    from emdee_gb300.surrogate import Chains
    N, C = 512, 2
    ch = Chains(gpu, C, N, 11)
    ch.run(50, 0.004, 50)
    ch.evaluate()
    R = ch.gather("R")
    Et = torch.tensor(ch.potential(), dtype=torch.float64, device="cuda")
    Ft = ch.gather("F")
    m = model(gpu, C, N, ch.L, ch.types)
    p = random_params(m.nparam, 12, scale=0.5)
    p[m.nparam // 2 - 1] = p[m.nparam - 1] = -5.0
    m.set_params(p)
    lE, lF, grad = m.gradient(R, Et, Ft, 1.0, 1.0)
    oE, oF, ref = so.loss_gradient(R.cpu(), ch.L, torch.tensor(ch.types - 1), torch.tensor(p, dtype=torch.float64),
                                   DESC["rc"], DESC["mu0"], DESC["mu15"], DESC["width"], Et.cpu(), Ft.cpu(), 1.0, 1.0)
    print("loss (GPU, reference):", lE, lF, oE, oF)
    # BF16 operands on the tensor cores against FP64: observed 6e-4 (energy) and 5e-6 (force)
    assert abs(lE - oE) <= 5e-3 * oE and abs(lF - oF) <= 1e-4 * oF
    g = grad.cpu().double()
    cos = float((g * ref).sum() / (g.norm() * ref.norm()))
    ratio = float(g.norm() / ref.norm())
    print("gradient cosine %.5f, norm ratio %.4f" % (cos, ratio))
    assert cos > 0.9995 and 0.995 < ratio < 1.005
    m.close()
    ch.close()


def test_training_and_hmc(gpu):
    from emdee_gb300.surrogate import Chains, generate_data, plain_hmc, surrogate_hmc, train
    N, C = 512, 4
    ch = Chains(gpu, C, N, 21)
    Rs, Es, Fs = generate_data(ch, 64, 25, 0.004, 0.8, 22, burn=200)
    m = model(gpu, 8, N, ch.L, ch.types)
    m.init_params(23, float(Es.mean()) / N)
    hist = train(m, Rs, Es, Fs, 6, 2e-3, 8, 24)
    print("training losses (energy, force):", hist)
    assert hist[-1][1] < 0.75 * hist[0][1]
    U, acc, secs = plain_hmc(ch, 6, 10, 0.004, 0.8, 25)
    assert U.shape == (C, 6) and 0.0 < acc <= 1.0
    hm = model(gpu, C, N, ch.L, ch.types)
    hm.set_params(m.get_params())
    U2, acc2, secs2, far = surrogate_hmc(ch, hm, 6, 10, 0.004, 0.8, 26)
    print("acceptance plain %.3f surrogate %.3f, surrogate paths beyond the list skin: %d" % (acc, acc2, far))
    assert U2.shape == (C, 6) and far == 0
    m.close()
    hm.close()
    ch.close()


def test_trained_surrogate_accepts(gpu):
    """A surrogate trained on plain-MD data of a small mixture (512 atoms, 16
    chains) proposes trajectories that the exact Hamiltonian accepts: acceptance
    above zero for 2- and 5-step trajectories, held-out force error below 30 % of
    the RMS force.  Prints acceptance and ESS/s of surrogate and plain HMC."""
    from emdee_gb300.surrogate import (Chains, ess, force_rmse, generate_data, plain_hmc, surrogate_hmc,
                                       train)
    N, C, dt, kT = 512, 16, 0.004, 0.8
    ch = Chains(gpu, C, N, 41)
    Rs, Es, Fs = generate_data(ch, 1600, 25, dt, kT, 42, burn=400)
    m = model(gpu, 8, N, ch.L, ch.types)
    m.init_params(43, float(Es.mean()) / N)
    train(m, Rs[:1440], Es[:1440], Fs[:1440], 15, 3e-3, 8, 44)
    rmse = force_rmse(m, Rs[1440:], Fs[1440:], 8)
    rms = float(Fs[1440:].double().pow(2).mean().sqrt())
    print("held-out force RMSE %.3f of RMS force %.3f (%.1f %%)" % (rmse, rms, 100 * rmse / rms))
    assert rmse < 0.3 * rms
    hm = model(gpu, C, N, ch.L, ch.types)
    hm.set_params(m.get_params())
    for steps in (2, 5):
        U, acc, secs = plain_hmc(ch, 30, steps, dt, kT, 45 + steps)
        U2, acc2, secs2, far = surrogate_hmc(ch, hm, 30, steps, dt, kT, 46 + steps)
        print("%d-step trajectories: acceptance plain %.3f surrogate %.3f; ESS/s plain %.1f surrogate %.1f"
              % (steps, acc, acc2, ess(U[:, 6:]) / secs, ess(U2[:, 6:]) / secs2))
        assert acc2 > 0.0 and far == 0
    m.close()
    hm.close()
    ch.close()
