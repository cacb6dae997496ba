"""GPU checks of the learned preconditioner in use: flexible CG with the
U-Net on Poisson solves (converged to the reference's residual test and
agreeing with the oracle), what a briefly trained network gains over the
same iteration without it, the fallback to the plain CG after a stall, and
the NS projection with the learned solve."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def potential(n, seed, rough=0.0):
    from carpio_gb300 import train as T
    return T.random_potentials(1, n, seed=seed, rough=rough)[0].cpu().numpy()


def neumann_problem(n, phi):
    """a structure-level Poisson_ whose all-Neumann solution is phi (b = A phi)"""
    import torch
    from carpio_gb300 import structure as S, train as T
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 1)
    P = S.Poisson(g)
    for seg in range(4):
        bc = S.BoundaryCondition()
        bc.set_default_2_bc(0.0)
        P.add_bc(0, seg, "phi", bc)
    b = T.neumann_laplacian(torch.from_numpy(phi)).numpy()
    src = g.zeros()
    src[1:-1, 1:-1] = -b * n * n     # b = -vol f on unit square cells of size 1/n
    P.set_depend(g.zeros(), None, src)
    P.set_solver("CG", None, 20000, 1e-8, mean_removal=True, precision="mixed")
    return g, P


def solve(n, phi, net, **kw):
    g, P = neumann_problem(n, phi)
    P.set_learned(net, **kw)
    rc = P.run()
    return rc, P.stats, g.interior(P.phi)


def test_learned_solve_converges_to_the_solution(gpu_lib):
    from carpio_gb300.unet import UNet
    net = UNet(seed=0)     # untrained: the iteration must still converge
    phi = potential(128, 1)
    rc, st, x = solve(128, phi, net)
    assert rc == 0 and st.tol_out <= 1e-8
    assert rel_l2(x, phi) < 1e-4


def test_fallback_after_a_stall(gpu_lib):
    phi = potential(64, 2)
    # no network and no smoothing: the first direction is zero, the FCG stops
    # and the plain CG finishes
    rc, st, x = solve(64, phi, None, use_net=False, smooth=0)
    assert rc == 0 and st.tol_out <= 1e-8
    assert st.outer_iters == 0 and st.iters > 0
    assert rel_l2(x, phi) < 1e-4


def test_trained_network_cuts_iterations(gpu_lib):
    """a network trained briefly by the library's own kernels takes far fewer
    FCG iterations than the same iteration without it"""
    from carpio_gb300 import train as T
    from carpio_gb300.unet import UNet
    net = UNet(seed=0)
    X, Y = T.make_dataset(count=1536, n=128, seed=5, cavity_steps=0, rough=0.5)
    T.train(net, X, Y, epochs=2, batch=16, lr=1e-3, loss="energy")
    phi = potential(128, 77)     # held out
    rc0, st0, x0 = solve(128, phi, net, use_net=False, smooth=4, fallback=False)
    rc1, st1, x1 = solve(128, phi, net, use_net=True, smooth=4, fallback=False)
    assert rc0 == 0 and rc1 == 0
    assert st1.outer_iters * 3 < st0.outer_iters, (st1.outer_iters, st0.outer_iters)
    assert rel_l2(x1, x0) < 1e-4


def test_ns_projection_with_learned_solve(gpu_lib):
    from carpio_gb300 import structure as S
    from carpio_gb300.unet import UNet

    def cavity(learned):
        g = S.Grid((0.0, 0.0), (1.0, 1.0), (128, 128), 2)
        ns = S.NS_explicit(g)
        for seg in range(4):
            bu, bv = S.BoundaryCondition(), S.BoundaryCondition()
            bu.set_default_1_bc(1.0 if seg == 3 else 0.0)
            bv.set_default_1_bc(0.0)
            ns.add_bc(0, seg, "u", bu)
            ns.add_bc(0, seg, "v", bv)
        ns.set_time(10, 0.5 / 128)
        ns.set_uniform_rho(1000.0)
        ns.set_uniform_mu(1.0)
        ns.set_CFL_number(0.5)
        ns.set_diffusion_number(0.25)
        ns.set_advection_scheme("VanLeer")
        ns.set_projection_solver("CG", max_iter=20000, tol=1e-10)
        ns.initial()
        if learned is not None:
            ns.set_learned(learned)
        assert ns.run(6) == 0
        return ns.state()

    a = cavity(None)
    b = cavity(UNet(seed=1))
    for k in ("u", "v", "p"):
        assert rel_l2(b[k], a[k]) < 1e-6, (k, rel_l2(b[k], a[k]))
