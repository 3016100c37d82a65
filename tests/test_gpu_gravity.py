"""NavierStokes3D with gravity on the GPU: the well-balanced formulation of
NavierStokes3DModifiedSolution.c / NavierStokes3DSource.c / NavierStokes3DUpwind.c
(Rusanov) against the oracle, on rising-thermal-bubble decks.  The reference's
own golden vectors for these decks run in test_gpu_parity.test_golden_reference.

Tolerances: relative L2 <= 1e-12 per right-hand side, <= 1e-10 after the steps."""
import ctypes

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import _lib, cases as C
from hypar_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEP_TOL = 1e-10


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def solver_for(case, tmp_path):
    d = str(tmp_path / "deck")
    case.write(d)
    return Solver.from_dir(d, device=0)


def hydrostatic(case):
    """The bubble deck's ambient state alone: constant potential temperature at rest."""
    gamma, R, rho_ref, p_ref, g = case.gamma, case.R_gas, case.rho_ref, case.p_ref, case.gravity[1]
    x = case.x[0]
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    Cp = gamma * R / (gamma - 1.0)
    T = p_ref / (R * rho_ref)
    exner = 1.0 - g * Y / (Cp * T)
    rho = p_ref / (R * T) * np.exp(np.log(exner) / (gamma - 1.0))
    E = rho * (R / (gamma - 1.0)) * T * exner
    z = np.zeros_like(rho)
    return np.stack([rho, z, z, z, E], axis=-1).reshape(-1, 5)


# every WENO weight formulation with each interpolation, every balance type HB
VARIANTS = [("components", "yc", 2, "y"), ("characteristic", "js", 2, "y"), ("components", "none", 1, "y"),
            ("characteristic", "mapped", 3, "z"), ("components", "borges", 3, "z"), ("components", "js", 2, "y"),
            ("components", "mapped", 1, "y"), ("characteristic", "yc", 1, "y"), ("characteristic", "borges", 2, "y"),
            ("characteristic", "none", 3, "z")]


def bubble(n, interp, weights, hb, axis, stir=0.5, **kw):
    """The bubble deck with random velocities of about `stir` m/s: at rest the
    energy equation's right-hand side is pure rounding noise (the pressure work
    vanishes), which no tolerance relative to the state can compare."""
    case = C.rising_thermal_bubble(n, interp=interp, weights=weights, HB=hb, **kw)
    if axis == "z":
        case.gravity, case.N_bv = (0.0, 0.0, 9.8), 0.01
    if stir:
        rng = np.random.default_rng(11)
        case.u[:, 1:4] = stir * rng.standard_normal((case.u.shape[0], 3)) * case.u[:, :1]
    return case


@pytest.mark.parametrize("interp,weights,hb,axis", VARIANTS)
def test_bubble_rhs_matches_oracle(built_lib, oracle_lib, tmp_path, interp, weights, hb, axis):
    case = bubble(20, interp, weights, hb, axis, n_iter=1, perturb=0.02)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    got = O.interior(out.cpu().numpy(), case.size, 5, 3)
    ref = O.interior(P.rhs(u0.copy()), case.size, 5, 3)
    assert relerr(got, ref) <= RHS_TOL


@pytest.mark.parametrize("interp,weights,hb,axis", [VARIANTS[0], VARIANTS[1], VARIANTS[3]])
def test_bubble_steps_match_oracle(built_lib, oracle_lib, tmp_path, interp, weights, hb, axis):
    case = bubble(16, interp, weights, hb, axis, n_iter=10, dt=0.05, perturb=0.02)
    s = solver_for(case, tmp_path)
    s.step(10)
    P = O.Problem(case)
    ref = O.interior(P.rk(P.u0(), 10), case.size, 5, 3).reshape(-1)
    assert relerr(s.get_state(), ref) <= STEP_TOL


@pytest.mark.parametrize("interp", ["components", "characteristic"])
def test_hydrostatic_state_is_preserved(built_lib, oracle_lib, tmp_path, interp):
    """Well-balanced: the discrete right-hand side of the hydrostatic atmosphere is
    rounding noise (Ghosh & Constantinescu, AIAA J. 54(4), 2016), while the same
    state's gravity source alone is O(rho g)."""
    case = C.rising_thermal_bubble(40, n_iter=1, interp=interp)
    case.u = hydrostatic(case)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    got = O.interior(out.cpu().numpy(), case.size, 5, 3)
    src = O.interior(P.source(u0), case.size, 5, 3)
    dxinv = (len(case.x[0]) - 1) / 1000.0
    scale = np.abs(case.u[:, 4]).max() * dxinv
    assert np.abs(src[:, 2]).max() > 5.0
    assert np.abs(got).max() <= 1e-12 * scale, np.abs(got).max(axis=0)
    # and it stays at rest over steps
    s.step(5)
    v = s.get_state().reshape(-1, 5)
    assert np.abs(v[:, 1:4]).max() <= 1e-9


def test_function_pointer_surface_with_gravity(built_lib, oracle_lib, tmp_path):
    """HyperbolicFunction (modified solution, no source), SourceFunction,
    UFunction and Upwind (Rusanov scaled by max(g_L, g_R)) with gravity."""
    case = bubble(14, "components", "js", 2, "y", n_iter=1, perturb=0.02)
    rng = np.random.default_rng(3)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    ubc = P.apply_bc(u0)
    u = torch.from_numpy(u0).cuda()
    s.apply_bc(u)
    assert np.array_equal(u.cpu().numpy(), ubc)
    hyp = torch.zeros_like(u)
    s.hyperbolic(hyp, u)
    assert relerr(hyp.cpu().numpy(), P.hyperbolic(u0)) <= RHS_TOL
    src = torch.full_like(u, 7.0)
    s.source(src, u)
    ref_s = P.source(u0)
    assert relerr(src.cpu().numpy(), ref_s) <= RHS_TOL
    assert not src.cpu().numpy()[ref_s == 0.0].any()

    # UFunction: u* = (rho f, rho v f, P / ((gamma-1) g) + rho |v|^2 f / 2)
    fg = P.gravity_field()
    n = P.npts_wg
    f, g = fg[:n], fg[n:]
    U = ubc.reshape(-1, 5)
    rho = np.where(U[:, 0] != 0.0, U[:, 0], 1.0)  # the unfilled corner ghosts hold zeros
    vel = U[:, 1:4] / rho[:, None]
    vsq = (vel ** 2).sum(axis=1)
    Pr = (U[:, 4] - 0.5 * rho * vsq) * (case.gamma - 1.0)
    uc_ref = np.empty_like(U)
    uc_ref[:, :4] = U[:, :4] * f[:, None]
    uc_ref[:, 4] = Pr / (case.gamma - 1.0) / g + 0.5 * U[:, 0] * vsq * f
    uc = torch.zeros_like(u)
    s.ufunc(uc, u)
    filled = U[:, 0] != 0.0
    assert filled.sum() > 0.7 * len(U)
    assert relerr(uc.cpu().numpy().reshape(-1, 5)[filled], uc_ref[filled]) <= 1e-14

    # Upwind along y on random interface states
    dim, gh = case.size, 3
    nI = [dim[0], dim[1] + 1, dim[2]]
    m = int(np.prod(nI))
    fL, fR, uL, uR = (rng.standard_normal((m, 5)) for _ in range(4))
    fI = torch.zeros(m * 5, dtype=torch.float64, device="cuda")
    tens = [torch.from_numpy(np.ascontiguousarray(a).reshape(-1)).cuda() for a in (fL, fR, uL, uR)]
    s.upwind(fI, *tens, u, 1)
    k, j, i = np.meshgrid(np.arange(nI[2]), np.arange(nI[1]), np.arange(nI[0]), indexing="ij")
    NX, NY = dim[0] + 2 * gh, dim[1] + 2 * gh
    pR = ((i + gh) + NX * ((j + gh) + NY * (k + gh))).reshape(-1)
    pL = pR - NX

    def speed(Uc):
        r = Uc[:, 0]
        vv = Uc[:, 1:4] / r[:, None]
        p = (Uc[:, 4] - 0.5 * r * (vv ** 2).sum(axis=1)) * (case.gamma - 1.0)
        return np.sqrt(case.gamma * p / r) + np.abs(vv[:, 1]), r, vv, p

    aL, rL, vL, PL = speed(U[pL])
    aR, rR, vR, PR = speed(U[pR])
    gm = case.gamma
    HL = 0.5 * (vL ** 2).sum(1) + gm * PL / rL / (gm - 1.0)
    HR = 0.5 * (vR ** 2).sum(1) + gm * PR / rR / (gm - 1.0)
    tL, tR = np.sqrt(rL), np.sqrt(rR)
    ra = tL * tR
    va = (tL[:, None] * vL + tR[:, None] * vR) / (tL + tR)[:, None]
    Ha = (tL * HL + tR * HR) / (tL + tR)
    Pa = (Ha - 0.5 * (va ** 2).sum(1)) * (ra * (gm - 1.0)) / gm
    aA = np.sqrt(gm * Pa / ra) + np.abs(va[:, 1])
    alpha = np.maximum(g[pL], g[pR]) * np.maximum(np.maximum(aL, aR), aA)
    ref_fI = 0.5 * (fL + fR) - alpha[:, None] * 0.5 * (uR - uL)
    assert relerr(fI.cpu().numpy().reshape(-1, 5), ref_fI) <= 1e-13


def test_gravity_needs_the_field(built_lib, tmp_path):
    """A solver built from a gravity configuration refuses to evaluate the
    right-hand side before gb_solver_set_gravity_field."""
    case = C.rising_thermal_bubble(10, n_iter=1)
    d = str(tmp_path / "deck")
    case.write(d)
    from hypar_gb300.solver import Inputs
    inp = Inputs(d)
    s = Solver(inp.config, inp.dxinv)
    s.set_state(inp.u0)
    u = torch.zeros(s.npts_wg * 5, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(u)
    with pytest.raises(_lib.GbError) as e:
        s.rhs(out, u)
    assert e.value.code == 1 and "gravity" in str(e.value)
    with pytest.raises(_lib.GbError):
        s.step(1)
    s.set_gravity_field(inp.gravity_field)
    s.step(1)
    # the allocation-free entry point does not offer gravity
    dx = torch.from_numpy(inp.dxinv).cuda()
    rc = _lib.lib().gb_rhs_explicit_noalloc(ctypes.byref(inp.config), ctypes.c_void_p(dx.data_ptr()),
                                            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(u.data_ptr()), None)
    assert rc == 4


# ---------------------------------------------------------------------------
# Euler1D in a gravity field (Xing & Shu's well-balanced form; Euler1DSource.c,
# Euler1DModifiedSolution.c, Euler1DUpwind.c with kappa = max(S_L, S_R)).
# ---------------------------------------------------------------------------
E1_VARIANTS = [(0, "components", "roe", "js"), (0, "characteristic", "llf-char", "yc"),
               (1, "characteristic", "roe", "mapped"), (1, "components", "llf-char", "borges"),
               (0, "components", "llf-char", "none"), (1, "characteristic", "llf-char", "js")]


def strat(grav_type, interp, upw, weights, **kw):
    case = C.stratified_1d(kw.pop("n", 96), grav_type=grav_type, interp=interp, upwinding=upw, **kw)
    case.weights = weights
    return case


@pytest.mark.parametrize("grav_type,interp,upw,weights", E1_VARIANTS)
def test_euler1d_gravity_rhs_and_steps(built_lib, oracle_lib, tmp_path, grav_type, interp, upw, weights):
    case = strat(grav_type, interp, upw, weights, n_iter=10, perturb=0.05)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    got = O.interior(out.cpu().numpy(), case.size, 3, 3)
    assert relerr(got, O.interior(P.rhs(u0.copy()), case.size, 3, 3)) <= RHS_TOL
    s.step(10)
    ref = O.interior(P.rk(P.u0(), 10), case.size, 3, 3).reshape(-1)
    assert relerr(s.get_state(), ref) <= STEP_TOL


@pytest.mark.parametrize("grav_type", [0, 1])
def test_euler1d_hydrostatic_state_is_preserved(built_lib, oracle_lib, tmp_path, grav_type):
    """The isothermal atmosphere rho = p = S at rest: its right-hand side is rounding
    noise while its gravity source alone is O(rho g); it stays at rest over steps."""
    case = C.stratified_1d(200, n_iter=1, grav_type=grav_type, perturb=0.0)
    s = solver_for(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    got = O.interior(out.cpu().numpy(), case.size, 3, 3)
    src = O.interior(P.source(u0), case.size, 3, 3)
    assert np.abs(src[:, 1]).max() > 0.1
    assert np.abs(got).max() <= 1e-12, np.abs(got).max(axis=0)
    s.step(20)
    assert np.abs(s.get_state().reshape(-1, 3)[:, 1]).max() <= 1e-12


def test_euler1d_gravity_function_pointers(built_lib, oracle_lib, tmp_path):
    """HyperbolicFunction, SourceFunction, UFunction (u / S) and Upwind (Roe and LLF
    dissipation scaled by max(S_L, S_R)) with Euler1D gravity."""
    for upw in ("roe", "llf-char"):
        case = strat(0, "components", upw, "js", n=64, perturb=0.05)
        rng = np.random.default_rng(5)
        case.u[:, 1] = 0.3 * rng.standard_normal(64) * case.u[:, 0]
        s = solver_for(case, tmp_path / upw)
        P = O.Problem(case)
        u0 = P.u0()
        u = torch.from_numpy(u0).cuda()
        s.apply_bc(u)
        hyp = torch.zeros_like(u)
        s.hyperbolic(hyp, u)
        assert relerr(hyp.cpu().numpy(), P.hyperbolic(u0)) <= RHS_TOL
        src = torch.full_like(u, 3.0)
        s.source(src, u)
        assert relerr(src.cpu().numpy(), P.source(u0)) <= RHS_TOL
        fg = P.gravity_field()
        n = P.npts_wg
        uc = torch.zeros_like(u)
        s.ufunc(uc, u)
        U = P.apply_bc(u0).reshape(-1, 3)
        assert relerr(uc.cpu().numpy().reshape(-1, 3), U * fg[:n, None]) <= 1e-15
