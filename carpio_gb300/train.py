"""Training data and training loop of the learned preconditioner.

Pairs (input, target) = (b / s, x / s): x a zero-mean pressure field, b = A x
with A the all-Neumann cell-centred 5-point operator the projection solves
(the reference's StencilPoisson_ with ghost folds on a uniform grid: the
graph Laplacian of the cell grid), s the RMS of b. Sampling x and applying A
gives the exact solution of A x = b without a solve; the random fields are
the pressure-like potentials of velocity fields u = curl psi + grad phi with
Gaussian random streamfunction and potential of spectral slope -3 (only the
potential part has a divergence), and cavity snapshots add the projection
solutions of a lid-driven cavity run (solved by the plain FP64 CG).

Generation runs on the GPU with torch (FFTs and elementwise shifts, the
data's plumbing); the network is trained by the library's own forward,
backward and Adam kernels.
"""
import math

import numpy as np


def neumann_laplacian(x):
    """(A x)[i, j] = sum over the existing neighbours of x[i, j] - x[nb]
    (the all-Neumann 5-point operator with unit face coefficients); x is a
    torch tensor (..., h, w)."""
    import torch
    b = torch.zeros_like(x)
    d = x[..., 1:, :] - x[..., :-1, :]
    b[..., 1:, :] += d
    b[..., :-1, :] -= d
    d = x[..., :, 1:] - x[..., :, :-1]
    b[..., :, 1:] += d
    b[..., :, :-1] -= d
    return b


def random_potentials(count, n, slope=-3.0, seed=0, device="cuda", rough=0.0):
    """zero-mean potentials phi (count, n, n), FP64. A fraction 1 - rough
    are the potentials of velocity fields with the power spectrum
    |u(k)|^2 ~ k^slope (so |phi(k)|^2 ~ k^(slope - 2)); the rest have
    |phi(k)|^2 ~ k^-beta with beta uniform in [1, 5], whose A phi reach the
    rough right-hand sides a Krylov iteration's residuals become."""
    import torch
    g = torch.Generator(device=device).manual_seed(int(seed))
    k = torch.fft.fftfreq(n, d=1.0 / n, device=device)
    kr = torch.fft.rfftfreq(n, d=1.0 / n, device=device)
    kk = torch.sqrt(k[:, None] ** 2 + kr[None, :] ** 2).clamp(min=1.0)
    zero = torch.zeros_like(kk)
    zero[0, 0] = 1.0
    out = torch.empty(count, n, n, dtype=torch.float64, device=device)
    n_rough = int(round(rough * count))
    betas = torch.full((count,), 2.0 - slope, dtype=torch.float64, device=device)
    if n_rough:
        betas[count - n_rough:] = 1.0 + 4.0 * torch.rand(n_rough, generator=g, device=device,
                                                          dtype=torch.float64)
    for i in range(0, count, 256):
        m = min(256, count - i)
        amp = kk[None] ** (-betas[i:i + m, None, None] / 2.0) * (1.0 - zero[None])
        re = torch.randn(m, n, n // 2 + 1, generator=g, device=device, dtype=torch.float64)
        im = torch.randn(m, n, n // 2 + 1, generator=g, device=device, dtype=torch.float64)
        phi = torch.fft.irfft2((re + 1j * im) * amp, s=(n, n))
        out[i:i + m] = phi - phi.mean(dim=(1, 2), keepdim=True)
    return out


def pairs_from_potentials(phi):
    """(input, target) float32 from FP64 zero-mean potentials"""
    import torch
    b = neumann_laplacian(phi)
    s = torch.sqrt((b * b).mean(dim=(1, 2), keepdim=True)).clamp(min=1e-300)
    return (b / s).float().contiguous(), (phi / s).float().contiguous()


def cavity_potentials(n=256, steps=2000, every=10, precision="fp64"):
    """projection solutions of a lid-driven cavity (Re 1000, van Leer), one
    every `every` steps, zero-mean, FP64 torch tensor (count, n, n)"""
    import torch
    from . import structure as S
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 2)
    ns = S.NS_explicit(g)
    for seg in range(4):
        bu, bv = S.BoundaryCondition(), S.BoundaryCondition()
        bu.set_default_1_bc(1.0 if seg == 3 else 0.0)
        bv.set_default_1_bc(0.0)
        ns.add_bc(0, seg, "u", bu)
        ns.add_bc(0, seg, "v", bv)
    ns.set_time(steps, 0.5 / n)
    ns.set_uniform_rho(1000.0)
    ns.set_uniform_mu(1.0)
    ns.set_CFL_number(0.5)
    ns.set_diffusion_number(0.25)
    ns.set_advection_scheme("VanLeer")
    ns.set_projection_solver("CG", max_iter=100000, tol=1e-10, precision=precision)
    ns.initial()
    snaps = []
    for _ in range(steps // every):
        ns.run(every)
        phi = g.interior(ns.state()["phi"]).copy()
        snaps.append(phi - phi.mean())
    return torch.from_numpy(np.stack(snaps)).cuda()


def make_dataset(count=20000, n=256, seed=0, cavity_steps=2000, cavity_every=10,
                 rough=0.5):
    """the training set: random potentials plus cavity snapshots (inputs,
    targets) as float32 CUDA tensors"""
    import torch
    parts_x, parts_t = [], []
    n_cav = 0
    if cavity_steps > 0:
        cav = cavity_potentials(n, cavity_steps, cavity_every)
        n_cav = cav.shape[0]
        x, t = pairs_from_potentials(cav)
        parts_x.append(x)
        parts_t.append(t)
    phi = random_potentials(count - n_cav, n, seed=seed, rough=rough)
    for i in range(0, phi.shape[0], 1024):
        x, t = pairs_from_potentials(phi[i:i + 1024])
        parts_x.append(x)
        parts_t.append(t)
    return torch.cat(parts_x), torch.cat(parts_t)


def train(net, inputs, targets, epochs=4, batch=16, lr=1e-3, seed=0, log=None,
          loss="energy"):
    """Adam over shuffled batches with a cosine learning-rate decay; returns
    the per-epoch mean losses"""
    import torch
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    n = inputs.shape[0]
    steps = epochs * (n // batch)
    hist, k = [], 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g)
        tot, cnt = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch].cuda()
            x = inputs.index_select(0, idx).contiguous()
            t = targets.index_select(0, idx).contiguous()
            a = lr * 0.5 * (1.0 + math.cos(math.pi * k / max(1, steps)))
            tot += net.train_step(x, t, a, loss=loss)
            cnt += 1
            k += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e}")
    return hist


def evaluate(net, sizes=(256, 512, 1024), seed=4242, cavity=True, log=print):
    """FCG iterations to 1e-8 with and without the network on held-out fields
    (and a 256^2 cavity projection), through the library's learned solve"""
    import torch
    from . import structure as S
    rows = []
    fields = [(f"random {n}^2", n, random_potentials(1, n, seed=seed + n)[0]) for n in sizes]
    if cavity:
        fields.append(("cavity 256^2", 256, cavity_potentials(256, 400, 400)[-1]))
    for name, n, phi in fields:
        b = neumann_laplacian(phi).cpu().numpy()
        res = {}
        for label, use_net, smooth in (("cg", None, 0), ("jacobi", False, 4),
                                       ("net", True, 4)):
            g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 1)
            P = S.Poisson(g)
            for seg in range(4):
                bc = S.BoundaryCondition()
                bc.set_default_2_bc(0.0)
                P.add_bc(0, seg, "phi", bc)
            src = g.zeros()
            src[1:-1, 1:-1] = -b * n * n
            P.set_depend(g.zeros(), None, src)
            P.set_solver("CG", None, 100000, 1e-8, mean_removal=True,
                         precision="fp64" if use_net is None else "mixed")
            if use_net is not None:
                P.set_learned(net if use_net else None, use_net=use_net, smooth=smooth,
                              fallback=False)
            P.run()
            res[label] = (P.stats.outer_iters if use_net is not None else P.stats.iters,
                          P.stats.ms, P.stats.tol_out)
        rows.append((name, res))
        log(f"{name}: " + "  ".join(f"{k} {v[0]} its {v[1]:.1f} ms (resid {v[2]:.1e})"
                                    for k, v in res.items()))
    return rows


def main(argv=None):
    import argparse
    import time
    import torch
    from .unet import UNet
    ap = argparse.ArgumentParser(description="train the learned preconditioner")
    ap.add_argument("--samples", type=int, default=20000)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cavity-steps", type=int, default=2000)
    ap.add_argument("--out", default=None, help="FP32 parameter file to write")
    ap.add_argument("--eval", action="store_true")
    ap.add_argument("--load", default=None, help="start from an FP32 parameter file")
    a = ap.parse_args(argv)
    net = UNet(seed=a.seed)
    if a.load:
        net.set_params(np.fromfile(a.load, dtype="<f4"))
    if a.samples <= 0:
        if a.eval:
            evaluate(net)
        return
    t0 = time.time()
    X, Y = make_dataset(a.samples, a.n, seed=a.seed, cavity_steps=a.cavity_steps)
    print(f"dataset {tuple(X.shape)} in {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    train(net, X, Y, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed,
          log=lambda s: print(s, flush=True))
    print(f"trained in {time.time() - t0:.1f} s", flush=True)
    del X, Y
    torch.cuda.empty_cache()
    if a.out:
        net.params().astype("<f4").tofile(a.out)
    if a.eval:
        evaluate(net)


if __name__ == "__main__":
    main()
