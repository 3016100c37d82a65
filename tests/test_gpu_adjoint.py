"""Discrete adjoint and tangent-linear model (Euler2D, component-wise WENO5 +
Roe, periodic) through the C ABI and the torch.autograd.Function front ends.

Checks: the dual-number right-hand side against the solver's; dot-product
tests <J v, w> = <v, J^T w> of the hand-written adjoint kernel against the
independent dual-number kernel, for one right-hand side and for n Runge-Kutta
steps; checkpoint policies against each other; the gradient of the final-time
density misfit against central finite differences (h = 1e-6) on 16 random
smooth directions."""
import ctypes

import numpy as np
import pytest

from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.adjoint import Adjoint, density_misfit_gradient, rhs, trajectory
from hypar_gb300.solver import Inputs, Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DOT_RHS_TOL = 1e-12   # two exact derivatives of one operator: rounding only
DOT_TRAJ_TOL = 1e-10
FD_TOL = 1e-6         # central differences, h = 1e-6


def rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.fixture(scope="module")
def problem(tmp_path_factory):
    case, u_true = C.adjoint_problem(n=40, n_iter=24, seed=5)
    d = str(tmp_path_factory.mktemp("adj") / "deck")
    case.write(d)
    return case, u_true, d


def make(problem, ncheck=0, nsteps=None, wide_tape_max=-1):
    case, _, d = problem
    inp = Inputs(d)
    return Adjoint(inp.config, inp.dxinv, nsteps or case.n_iter, ncheck=ncheck, device=0,
                   wide_tape_max=wide_tape_max)


def state(adj, u_int, seed=None, scale=0.0):
    u = torch.from_numpy(np.asarray(u_int, dtype=np.float64).reshape(adj.dims[1], adj.dims[0], 4)).cuda()
    if seed is not None:
        g = torch.Generator(device="cpu").manual_seed(seed)
        u = u * (1.0 + scale * torch.randn(u.shape, generator=g, dtype=torch.float64).cuda())
    return adj.ghosted(u).contiguous()


def rand_interior(adj, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    v = torch.randn((adj.dims[1], adj.dims[0], 4), generator=g, dtype=torch.float64).cuda()
    return adj.ghosted(v).contiguous()


def smooth_direction(n, rng, modes=6, kmax=4):
    """A random periodic field of a few low Fourier modes on an n x n grid."""
    x = np.arange(n) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    v = np.zeros((n, n))
    for _ in range(modes):
        kx, ky = rng.integers(-kmax, kmax + 1, size=2)
        v += rng.normal() * np.sin(2 * np.pi * (kx * X + ky * Y) + rng.uniform(0, 2 * np.pi))
    return torch.from_numpy(v).cuda()


def idot(adj, a, b):
    return float((adj.interior(a) * adj.interior(b)).sum())


def test_create_rejects_outside_scope(built_lib, problem):
    case, _, d = problem
    inp = Inputs(d)
    cfg = inp.config
    cfg.interp = 1  # characteristic
    h = ctypes.c_void_p()
    rc = _lib.lib().gb_adjoint_create(ctypes.byref(cfg), inp.dxinv.ctypes.data_as(_lib.DP), 4, 0, 0, ctypes.byref(h))
    assert rc == 4  # GB_ERR_UNSUPPORTED


def test_dual_rhs_matches_solver_rhs(built_lib, problem):
    case, _, d = problem
    adj = make(problem)
    s = Solver.from_dir(d, device=0)
    u = state(adj, case.u, seed=1, scale=0.01)
    k, dk = adj.empty(), adj.empty()
    adj.rhs_jvp(u, torch.zeros_like(u), k, dk)
    ref = torch.zeros_like(u)
    s.rhs(ref, u.clone())
    a, b = adj.interior(k).cpu().numpy(), adj.interior(ref).cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-12
    assert float(adj.interior(dk).abs().max()) == 0.0
    s.close()


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_rhs_dot_product(built_lib, problem, seed):
    case, _, _ = problem
    adj = make(problem)
    u = state(adj, case.u, seed=seed, scale=0.02)
    v, w = rand_interior(adj, 100 + seed), rand_interior(adj, 200 + seed)
    k, Jv, JTw = adj.empty(), adj.empty(), adj.empty()
    adj.rhs_jvp(u, v, k, Jv)
    adj.rhs_vjp(u, w, JTw)
    lhs, rhs_ = idot(adj, Jv, w), idot(adj, v, JTw)
    assert rel(lhs, rhs_) <= DOT_RHS_TOL, (lhs, rhs_)


def test_rhs_vjp_vs_central_differences(built_lib, problem):
    case, _, _ = problem
    adj = make(problem)
    # A smooth state and smooth density directions.  Cell-by-cell noise of
    # size h = 1e-6 on a nearly uniform far field moves the WENO smoothness
    # indicators on the scale of their epsilon (1e-6) and the y-eigenvalue
    # (~0 there) across the edges of Harten's entropy-fix band |lambda| < 1e-6,
    # so central differences of the right-hand side would measure curvature
    # on those scales, not the slope.
    u = state(adj, case.u)
    w = rand_interior(adj, 7)
    JTw = adj.empty()
    adj.rhs_vjp(u, w, JTw)
    h = 1e-6
    rng = np.random.default_rng(300)
    for _ in range(4):
        v = adj.empty()
        adj.interior(v)[..., 0] = smooth_direction(adj.dims[0], rng)
        kp, km, dk = adj.empty(), adj.empty(), adj.empty()
        adj.rhs_jvp(u + h * v, torch.zeros_like(u), kp, dk)
        adj.rhs_jvp(u - h * v, torch.zeros_like(u), km, dk)
        fd = idot(adj, (kp - km) / (2 * h), w)
        assert rel(fd, idot(adj, v, JTw)) <= FD_TOL


def test_tlm_forward_matches_fused_forward(built_lib, problem):
    case, _, _ = problem
    adj = make(problem)
    u0 = state(adj, case.u)
    uT, uT2, duT = adj.empty(), adj.empty(), adj.empty()
    adj.forward(u0, uT)
    adj.tlm(u0, torch.zeros_like(u0), uT2, duT)
    a, b = adj.interior(uT2).cpu().numpy(), adj.interior(uT).cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-10


def test_trajectory_dot_product(built_lib, problem):
    case, _, _ = problem
    adj = make(problem)
    u0 = state(adj, case.u)
    v, w = rand_interior(adj, 41), rand_interior(adj, 42)
    uT, uT2, Mv, MTw = adj.empty(), adj.empty(), adj.empty(), adj.empty()
    adj.tlm(u0, v, uT2, Mv)
    adj.forward(u0, uT)
    adj.backward(w, MTw)
    lhs, rhs_ = idot(adj, Mv, w), idot(adj, v, MTw)
    assert rel(lhs, rhs_) <= DOT_TRAJ_TOL, (lhs, rhs_)
    info = adj.info()
    assert info["segments"] == 5 and info["segment_len"] == 5  # ceil(sqrt(24)) checkpoints
    assert info["recomputed_steps"] == 24 - 4


def test_checkpoint_policies_agree(built_lib, problem):
    case, _, _ = problem
    w = None
    grads = []
    held = {}
    # every checkpoint policy with the wide (72-double) interface tape, and two with the 8-double one
    for ncheck, wide in ((1, -1), (0, -1), (7, -1), (24, -1), (1, 0), (0, 0)):
        adj = make(problem, ncheck=ncheck, wide_tape_max=wide)
        held[(ncheck, wide)] = adj.info()["bytes"]
        u0 = state(adj, case.u)
        if w is None:
            w = rand_interior(adj, 9)
        uT, g = adj.empty(), adj.empty()
        adj.forward(u0, uT)
        adj.backward(w, g)
        grads.append(adj.interior(g).cpu().numpy())
        if ncheck == 1:
            assert adj.info()["recomputed_steps"] == 0
        adj.close()
    # the reverse kernel adds the stencil adjoints with atomics, whose order varies
    # from run to run: the same policy twice differs by ~5e-13 after 24 steps
    for g in grads[1:]:
        assert np.linalg.norm(g - grads[0]) / np.linalg.norm(grads[0]) <= 1e-11
    assert held[(1, 0)] < held[(1, -1)] and held[(0, 0)] < held[(0, -1)]  # the narrow tape is smaller


def test_misfit_gradient_vs_central_differences(built_lib, problem):
    case, u_true, _ = problem
    adj = make(problem)
    # target: density after n steps from the true initial state
    uT = adj.empty()
    adj.forward(state(adj, u_true), uT)
    rho_tgt = adj.interior(uT)[..., 0].clone()
    u0_int = torch.from_numpy(case.u.reshape(adj.dims[1], adj.dims[0], 4).copy()).cuda()
    loss, grad = density_misfit_gradient(adj, u0_int, rho_tgt)
    assert loss > 0 and float(grad.abs().max()) > 0

    def misfit(u_int):
        out = adj.empty()
        adj.forward(adj.ghosted(u_int).contiguous(), out)
        r = adj.interior(out)[..., 0] - rho_tgt
        return 0.5 * float((r * r).sum())

    # 16 random smooth directions (a few random low Fourier modes each): the
    # gradient must match to 1e-6.  Four directions of cell-by-cell N(0,1)
    # noise as well, to a looser bound: with h = 1e-6 such a perturbation moves
    # the WENO smoothness indicators on the scale of their epsilon (1e-6), so
    # the central difference itself carries a truncation error near 1e-6..1e-5
    # on this coarse grid, whatever the gradient.
    h = 1e-6
    rng = np.random.default_rng(2024)
    gen = torch.Generator(device="cpu").manual_seed(2024)

    def fd_err(v):
        up, um = u0_int.clone(), u0_int.clone()
        up[..., 0] += h * v
        um[..., 0] -= h * v
        fd = (misfit(up) - misfit(um)) / (2 * h)
        return rel(fd, float((grad * v).sum()))

    errs = [fd_err(smooth_direction(adj.dims[0], rng)) for _ in range(16)]
    assert max(errs) <= FD_TOL, errs
    noise = [fd_err(torch.randn((adj.dims[1], adj.dims[0]), generator=gen, dtype=torch.float64).cuda())
             for _ in range(4)]
    assert max(noise) <= 1e-4, noise


def test_autograd_functions(built_lib, problem):
    case, _, _ = problem
    adj = make(problem)
    u0 = state(adj, case.u, seed=4, scale=0.01)
    w = rand_interior(adj, 77)
    # reverse mode through Trajectory equals the C backward sweep
    x = u0.clone().requires_grad_(True)
    (trajectory(x, adj) * w).sum().backward()
    uT, g = adj.empty(), adj.empty()
    adj.forward(u0, uT)
    adj.backward(w, g)
    a, b = adj.interior(x.grad).cpu().numpy(), adj.interior(g).cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-12
    # forward mode through RHS equals the dual-number kernel; reverse mode its adjoint
    import torch.autograd.forward_ad as fwAD
    v = rand_interior(adj, 78)
    with fwAD.dual_level():
        k = rhs(fwAD.make_dual(u0, v), adj)
        Jv = fwAD.unpack_dual(k).tangent
    y = u0.clone().requires_grad_(True)
    (rhs(y, adj) * w).sum().backward()
    assert rel(idot(adj, Jv, w), idot(adj, v, y.grad)) <= DOT_RHS_TOL


@pytest.mark.parametrize("tile", [32, 64])
def test_tile_forms(built_lib, problem, tile):
    """The tile forms of the forward (gb_adjoint_set_launch seg = -tile for the two
    directions) and of the reverse kernel (seg = -tile for both directions): the RHS
    dot-product test, and the checkpointed gradient against the walker forms'."""
    case, _, _ = problem
    adj = make(problem)
    u = state(adj, case.u, seed=21, scale=0.02)
    v, w = rand_interior(adj, 121), rand_interior(adj, 221)
    k, Jv, JTw = adj.empty(), adj.empty(), adj.empty()
    adj.set_launch(2, -tile)
    adj.set_launch(3, -tile)
    assert adj.get_launch(2)[0] == -tile
    adj.rhs_jvp(u, v, k, Jv)
    adj.rhs_vjp(u, w, JTw)
    assert rel(idot(adj, Jv, w), idot(adj, v, JTw)) <= DOT_RHS_TOL
    grads = []
    for shapes in ((None, None), (-tile, -tile)):
        a = make(problem, ncheck=0)
        if shapes[0]:
            for which in range(4):
                a.set_launch(which, shapes[0])
        u0 = state(a, case.u)
        wt = rand_interior(a, 9)
        uT, g = a.empty(), a.empty()
        a.forward(u0, uT)
        a.backward(wt, g)
        grads.append(a.interior(g).cpu().numpy())
        a.close()
    assert np.linalg.norm(grads[1] - grads[0]) / np.linalg.norm(grads[0]) <= 1e-11


@pytest.mark.parametrize("tile", [32, 64])
def test_tile_reverse_is_deterministic(built_lib, problem, tile):
    """The tile form of the reverse kernel sums every cell's shares in a fixed order
    (per-tile shares, then a gather), so repeated gradients are bit-identical, in one
    adjoint object and across two."""
    case, _, _ = problem
    grads = []
    for _ in range(2):
        a = make(problem, ncheck=0)
        a.set_launch(2, -tile)
        a.set_launch(3, -tile)
        u0 = state(a, case.u)
        wt = rand_interior(a, 9)
        for _ in range(2):
            uT, g = a.empty(), a.empty()
            a.forward(u0, uT)
            a.backward(wt, g)
            grads.append(a.interior(g).cpu().numpy())
        a.close()
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])
