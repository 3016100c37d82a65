"""CRWENO5 (compact fifth-order WENO, component-wise and characteristic) on the GPU
against the oracle,
whose CRWENO5 is pinned bit-for-bit on the reference's golden decks (those decks
also run in test_gpu_parity.test_golden_reference).

Tolerances: relative L2 <= 1e-12 per right-hand side, <= 1e-10 after the steps."""
import numpy as np
import pytest

import oracle as O
from hypar_gb300 import cases as C
from hypar_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEP_TOL = 1e-10


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def crweno(case, weights="js"):
    case.hyp_scheme = "crweno5"
    case.weights = weights
    return case


def make(model, upw, n=None, interp="components", **kw):
    if model == "euler1d":
        return crweno(C.sod(n or 96, n_iter=kw.get("n_iter", 4), dt=1e-3, upwinding=upw, interp=interp,
                            scheme=kw.get("scheme", "44")), kw.get("weights", "js"))
    if model == "euler2d":
        return crweno(C.vortex(n or 40, n_iter=kw.get("n_iter", 3), dt=0.02, interp=interp, upwinding=upw,
                               scheme=kw.get("scheme", "ssprk3")), kw.get("weights", "js"))
    return crweno(C.tgv(n or 14, n_iter=kw.get("n_iter", 2), dt=0.02, upwinding=upw, perturb=0.05, interp=interp,
                        scheme=kw.get("scheme", "44")), kw.get("weights", "js"))


def solver_for(case, tmp_path):
    d = str(tmp_path / "deck")
    case.write(d)
    return Solver.from_dir(d, device=0)


def rhs_tol(case, u0, ref_full):
    """1e-12, or for the characteristic form within 4x the distance between the oracle
    and its own FMA-contracted build: the block-tridiagonal line solves of
    characteristic CRWENO5 amplify rounding (for the 2-D vortex that distance is
    3e-12 at 40^2 and 1e-9 at 512^2, growing with the line length), so the 1e-12 bar is
    below the noise of the reference's own arithmetic there."""
    if case.interp != "characteristic":
        return RHS_TOL
    Pf = O.Problem(case, fma=True)
    noise = relerr(O.interior(Pf.rhs(u0.copy()), case.size, case.nvars, 3),
                   O.interior(ref_full, case.size, case.nvars, 3))
    return max(RHS_TOL, 4.0 * noise)


def gpu_rhs(s, u0):
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    return out.cpu().numpy()


COMBOS = [(m, u) for m in ("euler1d", "euler2d", "navierstokes3d") for u in ("roe", "llf-char", "rf-char", "rusanov")
          if not (m == "euler2d" and u == "rusanov")]


@pytest.mark.parametrize("interp", ["components", "characteristic"])
@pytest.mark.parametrize("model,upw", COMBOS)
def test_crweno_rhs_matches_oracle(built_lib, oracle_lib, tmp_path, model, upw, interp):
    case = make(model, upw, interp=interp)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
    ref_full = P.rhs(u0.copy())
    ref = O.interior(ref_full, case.size, case.nvars, 3)
    assert relerr(got, ref) <= rhs_tol(case, u0, ref_full)


@pytest.mark.parametrize("interp", ["components", "characteristic"])
@pytest.mark.parametrize("weights", ["mapped", "borges", "yc", "none"])
@pytest.mark.parametrize("model", ["euler1d", "euler2d", "navierstokes3d"])
def test_crweno_weights_match_oracle(built_lib, oracle_lib, tmp_path, model, weights, interp):
    case = make(model, "roe", weights=weights, interp=interp)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
    ref_full = P.rhs(u0.copy())
    ref = O.interior(ref_full, case.size, case.nvars, 3)
    assert relerr(got, ref) <= rhs_tol(case, u0, ref_full)


@pytest.mark.parametrize("model,upw,interp", [("euler1d", "roe", "components"), ("euler2d", "roe", "components"),
                                              ("euler2d", "llf-char", "components"),
                                              ("navierstokes3d", "roe", "components"),
                                              ("navierstokes3d", "rusanov", "components"),
                                              ("euler1d", "roe", "characteristic"),
                                              ("euler2d", "roe", "characteristic"),
                                              ("navierstokes3d", "llf-char", "characteristic")])
def test_crweno_steps_match_oracle(built_lib, oracle_lib, tmp_path, model, upw, interp):
    case = make(model, upw, n_iter=10, interp=interp)
    s = solver_for(case, tmp_path)
    s.step(10)
    P = O.Problem(case)
    ref = O.interior(P.rk(P.u0(), 10), case.size, case.nvars, 3).reshape(-1)
    assert relerr(s.get_state(), ref) <= STEP_TOL


@pytest.mark.parametrize("seg,block", [(1, 32), (3, 64), (7, 128), (64, 128)])
def test_crweno_launch_shapes(built_lib, oracle_lib, tmp_path, seg, block):
    """The flux kernel's segments (ragged ends included) do not change the result."""
    case = make("euler2d", "roe", n=37)
    s = solver_for(case, tmp_path)
    for d in range(2):
        s.set_launch(d, seg, block)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
    ref_full = P.rhs(u0.copy())
    ref = O.interior(ref_full, case.size, case.nvars, 3)
    assert relerr(got, ref) <= rhs_tol(case, u0, ref_full)


@pytest.mark.parametrize("interp", ["components", "characteristic"])
def test_crweno_long_lines(built_lib, oracle_lib, tmp_path, interp):
    """A 2-D grid with 513-interface lines in both directions and the smallest grid."""
    for n in (512, 4):
        case = make("euler2d", "roe", n=n, interp=interp)
        s = solver_for(case, tmp_path / str(n))
        P = O.Problem(case)
        u0 = P.u0()
        got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
        ref_full = P.rhs(u0.copy())
        ref = O.interior(ref_full, case.size, case.nvars, 3)
        assert relerr(got, ref) <= rhs_tol(case, u0, ref_full), n


@pytest.mark.parametrize("interp", ["components", "characteristic"])
def test_crweno_function_pointers(built_lib, oracle_lib, tmp_path, interp):
    """gb_HyperbolicFunction with CRWENO5 (the hyperbolic term alone)."""
    case = make("navierstokes3d", "roe", interp=interp)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    s.apply_bc(u)
    hyp = torch.zeros_like(u)
    s.hyperbolic(hyp, u)
    assert relerr(hyp.cpu().numpy(), P.hyperbolic(u0)) <= rhs_tol(case, u0, P.rhs(u0.copy()))


# ---------------------------------------------------------------------------
# Gravity with CRWENO5 (Euler1DSource.c, NavierStokes3DSource.c): the source function
# [0, g e_d, g] solved for with the flux's weights (the same rows, another right-hand
# side), averaged, differenced and scaled per cell; the modified solution as the u
# values; the dissipation scaled by max(g_L, g_R).
# ---------------------------------------------------------------------------
GRAV = [("euler1d", "components", "roe", "js", 0), ("euler1d", "characteristic", "roe", "mapped", 1),
        ("euler1d", "characteristic", "llf-char", "yc", 0), ("euler1d", "components", "llf-char", "borges", 1),
        ("euler1d", "characteristic", "llf-char", "none", 1),
        ("navierstokes3d", "components", "rusanov", "yc", 2), ("navierstokes3d", "characteristic", "rusanov", "js", 3),
        ("navierstokes3d", "characteristic", "rusanov", "borges", 1),
        ("navierstokes3d", "components", "rusanov", "mapped", 3)]


def grav_case(model, interp, upw, weights, k, n_iter=1, stir=0.5):
    """Euler1D: the stratified atmosphere (gravity_type k), perturbed; NavierStokes3D: the
    rising-bubble deck (balance type HB k, gravity along z for k = 3), perturbed and
    stirred (at rest its energy right-hand side is rounding noise)."""
    if model == "euler1d":
        case = C.stratified_1d(96, n_iter=n_iter, grav_type=k, interp=interp, upwinding=upw, perturb=0.05)
    else:
        case = C.rising_thermal_bubble(14, n_iter=n_iter, dt=0.05, interp=interp, HB=k, perturb=0.02)
        if k == 3:
            case.gravity, case.N_bv = (0.0, 0.0, 9.8), 0.01
        if stir:
            rng = np.random.default_rng(11)
            case.u[:, 1:4] = stir * rng.standard_normal((case.u.shape[0], 3)) * case.u[:, :1]
    return crweno(case, weights)


@pytest.mark.parametrize("model,interp,upw,weights,k", GRAV)
def test_crweno_gravity_rhs_matches_oracle(built_lib, oracle_lib, tmp_path, model, interp, upw, weights, k):
    case = grav_case(model, interp, upw, weights, k)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
    ref_full = P.rhs(u0.copy())
    ref = O.interior(ref_full, case.size, case.nvars, 3)
    src = O.interior(P.source(u0), case.size, case.nvars, 3)
    tol = rhs_tol(case, u0, ref_full)
    assert relerr(ref - src, ref) > 1e6 * tol  # without the source the result would be far off
    assert relerr(got, ref) <= tol


@pytest.mark.parametrize("model,interp,upw,weights,k", [GRAV[0], GRAV[1], GRAV[5], GRAV[6]])
def test_crweno_gravity_steps_match_oracle(built_lib, oracle_lib, tmp_path, model, interp, upw, weights, k):
    case = grav_case(model, interp, upw, weights, k, n_iter=8)
    s = solver_for(case, tmp_path)
    s.step(8)
    P = O.Problem(case)
    ref = O.interior(P.rk(P.u0(), 8), case.size, case.nvars, 3).reshape(-1)
    assert relerr(s.get_state(), ref) <= STEP_TOL


@pytest.mark.parametrize("interp", ["components", "characteristic"])
@pytest.mark.parametrize("grav_type", [0, 1])
def test_crweno_euler1d_hydrostatic_state_is_preserved(built_lib, oracle_lib, tmp_path, interp, grav_type):
    """Well-balanced with the compact scheme too: the flux's pressure and the source
    function go through the same line solves, so the atmosphere at rest has a
    right-hand side of rounding noise while its gravity source alone is O(rho g)."""
    case = crweno(C.stratified_1d(200, n_iter=1, grav_type=grav_type, interp=interp, perturb=0.0))
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, 3, 3)
    src = O.interior(P.source(u0), case.size, 3, 3)
    assert np.abs(src[:, 1]).max() > 0.1
    assert np.abs(got).max() <= 1e-11, np.abs(got).max(axis=0)
    s.step(20)
    assert np.abs(s.get_state().reshape(-1, 3)[:, 1]).max() <= 1e-11


@pytest.mark.parametrize("model,interp,upw,weights,k", [GRAV[1], GRAV[5]])
def test_crweno_gravity_function_pointers(built_lib, oracle_lib, tmp_path, model, interp, upw, weights, k):
    """gb_HyperbolicFunction (the hyperbolic term alone) and gb_SourceFunction (the
    gravity source, the difference of the terms with and without it) with CRWENO5."""
    case = grav_case(model, interp, upw, weights, k)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    s.apply_bc(u)
    hyp = torch.zeros_like(u)
    s.hyperbolic(hyp, u)
    tol = rhs_tol(case, u0, P.rhs(u0.copy()))
    assert relerr(hyp.cpu().numpy(), P.hyperbolic(u0)) <= tol
    src = torch.full_like(u, 3.0)
    s.source(src, u)
    # the source is a difference of two hyperbolic terms: its error is relative to them
    ref = P.source(u0)
    assert np.linalg.norm(src.cpu().numpy() - ref) <= tol * np.linalg.norm(P.hyperbolic(u0)) + 1e-14
    assert np.linalg.norm(ref) > 0.0
