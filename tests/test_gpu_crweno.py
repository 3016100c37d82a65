"""CRWENO5 (compact fifth-order WENO, component-wise) on the GPU against the oracle,
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


def make(model, upw, n=None, **kw):
    if model == "euler1d":
        return crweno(C.sod(n or 96, n_iter=kw.get("n_iter", 4), dt=1e-3, upwinding=upw,
                            scheme=kw.get("scheme", "44")), kw.get("weights", "js"))
    if model == "euler2d":
        return crweno(C.vortex(n or 40, n_iter=kw.get("n_iter", 3), dt=0.02, interp="components", upwinding=upw,
                               scheme=kw.get("scheme", "ssprk3")), kw.get("weights", "js"))
    return crweno(C.tgv(n or 14, n_iter=kw.get("n_iter", 2), dt=0.02, upwinding=upw, perturb=0.05,
                        scheme=kw.get("scheme", "44")), kw.get("weights", "js"))


def solver_for(case, tmp_path):
    d = str(tmp_path / "deck")
    case.write(d)
    return Solver.from_dir(d, device=0)


def gpu_rhs(s, u0):
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    return out.cpu().numpy()


COMBOS = [(m, u) for m in ("euler1d", "euler2d", "navierstokes3d") for u in ("roe", "llf-char", "rf-char", "rusanov")
          if not (m == "euler2d" and u == "rusanov")]


@pytest.mark.parametrize("model,upw", COMBOS)
def test_crweno_rhs_matches_oracle(built_lib, oracle_lib, tmp_path, model, upw):
    case = make(model, upw)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
    ref = O.interior(P.rhs(u0.copy()), case.size, case.nvars, 3)
    assert relerr(got, ref) <= RHS_TOL


@pytest.mark.parametrize("weights", ["mapped", "borges", "yc", "none"])
@pytest.mark.parametrize("model", ["euler1d", "euler2d", "navierstokes3d"])
def test_crweno_weights_match_oracle(built_lib, oracle_lib, tmp_path, model, weights):
    case = make(model, "roe", weights=weights)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
    ref = O.interior(P.rhs(u0.copy()), case.size, case.nvars, 3)
    assert relerr(got, ref) <= RHS_TOL


@pytest.mark.parametrize("model,upw", [("euler1d", "roe"), ("euler2d", "roe"), ("euler2d", "llf-char"),
                                       ("navierstokes3d", "roe"), ("navierstokes3d", "rusanov")])
def test_crweno_steps_match_oracle(built_lib, oracle_lib, tmp_path, model, upw):
    case = make(model, upw, n_iter=10)
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
    ref = O.interior(P.rhs(u0.copy()), case.size, case.nvars, 3)
    assert relerr(got, ref) <= RHS_TOL


def test_crweno_long_lines(built_lib, oracle_lib, tmp_path):
    """A 2-D grid with 513-interface lines in both directions and the smallest grid."""
    for n in (512, 4):
        case = make("euler2d", "roe", n=n)
        s = solver_for(case, tmp_path / str(n))
        P = O.Problem(case)
        u0 = P.u0()
        got = O.interior(gpu_rhs(s, u0), case.size, case.nvars, 3)
        ref = O.interior(P.rhs(u0.copy()), case.size, case.nvars, 3)
        assert relerr(got, ref) <= RHS_TOL, n


def test_crweno_function_pointers(built_lib, oracle_lib, tmp_path):
    """gb_HyperbolicFunction with CRWENO5 (the hyperbolic term alone)."""
    case = make("navierstokes3d", "roe")
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    s.apply_bc(u)
    hyp = torch.zeros_like(u)
    s.hyperbolic(hyp, u)
    assert relerr(hyp.cpu().numpy(), P.hyperbolic(u0)) <= RHS_TOL
