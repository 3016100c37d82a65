"""Parity at the benchmark configurations' full sizes.

Sod 1024 (RK4, dt 1e-4, 1000 steps) is cheap enough for the oracle to run whole,
and so is the 1024^2 vortex over 100 SSPRK3 steps (about 30 s on 16 host cores):
both are held to relative L2 <= 1e-10 of the state.  The 256^3 Taylor-Green
vortex over 100 RK4 steps takes the oracle about 11 minutes on 16 cores; that
leg runs when HYPAR_LONG_VALIDATION=1 is set.
For the 1024^2 vortex and a perturbed 256^3 Taylor-Green vortex the oracle also
evaluates one right-hand side at full size: relative L2 <= 1e-12.  (A flux difference
over a fine grid cancels O(1) fluxes to O(h), so rounding is amplified by the grid
size; the kernels difference fluxes taken relative to each interface's left cell,
which keeps their own share of that rounding below the reference's: at 1024^2 the
oracle and its FMA-contracted build differ by 8e-13, the GPU and the oracle by
7.6e-13.)  A size-independent
property covers many steps: on a periodic grid the conservative flux difference
telescopes, so the domain sums of the conserved variables stay constant to
rounding.  (The viscous term does not telescope near the faces: on one rank the
reference forms no cross derivative at ghost points,
NavierStokes3DParabolicFunction.c:117-130, so the viscous fluxes there are not the
periodic images of the interior ones; for the Taylor-Green vortex only the mass,
which has no viscous flux, is conserved exactly.)"""
import os

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


def solver_for(case, tmp_path):
    d = str(tmp_path / "deck")
    case.write(d)
    return Solver.from_dir(d, device=0)


@pytest.fixture(scope="module", autouse=True)
def oracle_threads(oracle_lib):
    O.set_threads(os.cpu_count() or 1)


def test_sod_full_configuration(built_lib, tmp_path):
    """Sod shock tube, 1024 cells, comp-WENO5 + Roe, RK4, dt 1e-4, 1000 steps."""
    case = C.sod(1024, n_iter=1000, dt=1e-4)
    s = solver_for(case, tmp_path)
    s.step(1000)
    P = O.Problem(case)
    ref = O.interior(P.rk(P.u0(), 1000), case.size, case.nvars, 3).reshape(-1)
    assert relerr(s.get_state(), ref) <= STEP_TOL


def _rhs_vs_oracle(s, case):
    """(relative L2 distance GPU vs oracle, allowed distance)"""
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.zeros_like(u)
    s.rhs(out, u)
    got = O.interior(out.cpu().numpy(), case.size, case.nvars, 3)
    ref = O.interior(P.rhs(u0.copy()), case.size, case.nvars, 3)
    return relerr(got, ref), RHS_TOL


def _sums(s, case):
    u = s.get_state().reshape(-1, case.nvars)
    return u.sum(axis=0), np.abs(u).sum(axis=0)


def test_vortex_full_size(built_lib, tmp_path):
    """Isentropic vortex 1024^2, char-WENO5 + Roe, SSPRK3 at CFL 0.5: one RHS against
    the oracle; 20 steps conserve the domain sums of rho, rho u, rho v, e."""
    case = C.vortex(1024, n_iter=20)
    s = solver_for(case, tmp_path)
    err, tol = _rhs_vs_oracle(s, case)
    assert err <= tol, (err, tol)
    s.set_state(case.u)
    tot0, mag0 = _sums(s, case)
    s.step(20)
    tot, _ = _sums(s, case)
    assert np.all(np.abs(tot - tot0) <= 1e-12 * mag0), (tot - tot0) / mag0


def test_tgv_full_size(built_lib, tmp_path):
    """Taylor-Green vortex 256^3, comp-WENO5 + Roe + viscous, RK4: one RHS of the
    perturbed state against the oracle (the unperturbed t = 0 state's divergence is
    rounding noise); 4 steps of the benchmark state conserve the mass."""
    pert = C.tgv(256, n_iter=1, dt=2e-3, perturb=0.05)
    s = solver_for(pert, tmp_path / "p")
    err, tol = _rhs_vs_oracle(s, pert)
    assert err <= tol, (err, tol)
    s.close()
    case = C.tgv(256, n_iter=4, dt=2e-3)
    s = solver_for(case, tmp_path / "c")
    tot0, mag0 = _sums(s, case)
    s.step(4)
    tot, _ = _sums(s, case)
    assert abs(tot[0] - tot0[0]) <= 1e-12 * mag0[0], (tot[0] - tot0[0]) / mag0[0]


def test_vortex_full_size_100_steps(built_lib, tmp_path):
    """The benchmark configuration itself: isentropic vortex 1024^2, char-WENO5 + Roe,
    SSPRK3 at CFL 0.5, 100 steps on the GPU and in the oracle; the states agree to
    relative L2 <= 1e-10."""
    case = C.vortex(1024, n_iter=100)
    s = solver_for(case, tmp_path)
    s.step(100)
    got = s.get_state()
    P = O.Problem(case)
    ref = O.interior(P.rk(P.u0(), 100), case.size, case.nvars, 3).reshape(-1)
    err = relerr(got, ref)
    assert err <= STEP_TOL, err


@pytest.mark.skipif(os.environ.get("HYPAR_LONG_VALIDATION") != "1",
                    reason="about 11 minutes of oracle time on 16 cores: set HYPAR_LONG_VALIDATION=1")
def test_tgv_full_size_100_steps(built_lib, tmp_path):
    """Taylor-Green vortex 256^3, comp-WENO5 + Roe + viscous, RK4, dt 2e-3, 100 steps on
    the GPU and in the oracle; the states agree to relative L2 <= 1e-10."""
    case = C.tgv(256, n_iter=100, dt=2e-3)
    s = solver_for(case, tmp_path)
    s.step(100)
    got = s.get_state()
    s.close()
    P = O.Problem(case)
    ref = O.interior(P.rk(P.u0(), 100), case.size, case.nvars, 3).reshape(-1)
    err = relerr(got, ref)
    print(f"tgv 256^3 100 RK4 steps: relative L2 GPU vs oracle {err:.3e}")
    assert err <= STEP_TOL, err
