"""Three points along a dimension (the quasi-2-D NavierStokes3D decks of the reference
run with size N M 3): every ghost cell of such a line is a folded interior point, and
the walker segments, tiles, CRWENO5 line solves and boundary zones each see lines of
3 cells.  CPU: the reader takes such decks and refuses two points.  GPU: one
right-hand side against the oracle for every launch form, and a few steps.  The
rising-bubble slab is a near-cancellation (hydrostatic balance): there the bound is 4x
the distance between the oracle and its own FMA-contracted build, as for the other
well-balanced decks."""
import numpy as np
import pytest

import oracle as O
from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Inputs, Solver

RHS_TOL = 1e-12
STEP_TOL = 1e-10


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def slab(case, dim, n, start=0):
    shape = [s for s in reversed(case.size)] + [case.nvars]
    u = case.u.reshape(shape)
    sl = [slice(None)] * len(shape)
    sl[len(case.size) - 1 - dim] = slice(start, start + n)
    case.u = np.ascontiguousarray(u[tuple(sl)]).reshape(-1, case.nvars)
    case.size = list(case.size)
    case.size[dim] = n
    case.x = list(case.x)
    case.x[dim] = np.asarray(case.x[dim])[start:start + n]
    return case


def decks():
    # vortex slabs through the vortex core (rows 11-13 of 24)
    v = slab(C.vortex(24, n_iter=3, dt=0.02), 1, 3, 11)
    t = slab(C.tgv(12, n_iter=2, dt=0.02, perturb=0.05), 2, 3)
    w = slab(C.vortex(24, n_iter=3, dt=0.02, interp="components", upwinding="llf-char"), 1, 3, 11)
    w.bcs = {(1, 1): ("slip-wall", [0.0, 0.0]), (1, -1): ("slip-wall", [0.0, 0.0])}
    r = slab(C.rising_thermal_bubble(12, n_iter=2, dt=0.05, perturb=0.02), 2, 3)
    cr = slab(C.tgv(12, n_iter=2, dt=0.02, perturb=0.05), 2, 3)
    cr.hyp_scheme = "crweno5"
    return {"vortex_char": v, "vortex_walls": w, "tgv": t, "rtb_gravity": r, "tgv_crweno": cr}


def test_reader_three_and_two_points(built_lib, tmp_path):
    d = str(tmp_path / "three")
    decks()["tgv"].write(d)
    assert list(Inputs(d).config.dim) == [12, 12, 3]
    case = slab(C.tgv(12, n_iter=1, dt=0.02), 2, 2)
    d = str(tmp_path / "two")
    case.write(d)
    with pytest.raises(_lib.GbError) as e:
        Inputs(d)
    assert e.value.code == 3


SHAPES = [(1, 64), (2, 128), (32, 128), (-32, 0), (-64, 0), (-128, 0)]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["vortex_char", "vortex_walls", "tgv", "rtb_gravity", "tgv_crweno"])
@pytest.mark.parametrize("shape", SHAPES)
def test_three_point_lines_match_oracle(built_lib, oracle_lib, tmp_path, name, shape):
    torch = pytest.importorskip("torch")
    case = decks()[name]
    d = str(tmp_path / "deck")
    case.write(d)
    s = Solver.from_dir(d, device=0)
    for dd in range(case.ndims):
        s.set_launch(dd, shape[0], shape[1])
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.full_like(u, 7.0)
    s.rhs(out, u)
    got = O.interior(out.cpu().numpy(), case.size, case.nvars, 3)
    ref_full = P.rhs(u0)
    ref = O.interior(ref_full, case.size, case.nvars, 3)
    tol = RHS_TOL
    if name == "rtb_gravity":
        tol = max(RHS_TOL, 4.0 * relerr(O.Problem(case, fma=True).rhs(u0), ref_full))
    assert relerr(got, ref) <= tol
    s.step(case.n_iter)
    ref = O.interior(P.rk(P.u0(), case.n_iter), case.size, case.nvars, 3).reshape(-1)
    assert relerr(s.get_state(), ref) <= STEP_TOL
