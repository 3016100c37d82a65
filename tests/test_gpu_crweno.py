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
