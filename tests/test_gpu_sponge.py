"""Sponge zones (BCSponge.c) and the boundary fields a solver needs before a right-hand
side (the sponge's sigma, a thermal wall's temperature).

CPU: the reader's sigma against the reference's formula on the deck's coordinates, the
zone extents (interior points in every dimension, FindInterval), and the validation
of a sponge extent that reaches into the ghost points.  GPU: the source term of the
sponge alone is bit-identical to the oracle's (the same three roundings on both
sides); right-hand sides and Runge-Kutta steps with sponges inside the path's
tolerances; a solver whose sponge or thermal field was never uploaded refuses to
evaluate."""
import ctypes

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Inputs, Solver

GB_ERR_ARG, GB_ERR_UNSUPPORTED, GB_BC_SPONGE = 1, 4, 13
RHS_TOL = 1e-12
STEP_TOL = 1e-10


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def decks():
    return {
        "sod": _sp(C.sod(64, n_iter=6, dt=1e-3), [
            (0, -1, [(0.75, 1.5)], [0.2, 0.1, 0.3]), (0, 1, [(-0.5, 0.2)], [0.9, -0.1, 2.4])]),
        "vortex": _sp(C.vortex(32, n_iter=4, dt=0.02), [
            (0, -1, [(6.0, 9.9), (-1.0, 11.0)], [1.1, 0.4, 0.05, 2.7]),
            (1, 1, [(-1.0, 11.0), (0.0, 2.5)], [0.9, 0.55, -0.05, 2.5]),
            (1, -1, [(3.0, 7.0), (8.0, 9.9)], [1.0, 0.5, 0.0, 2.6])]),
        "tgv": _sp(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05), [
            (2, 1, [(-1.0, 7.0), (-1.0, 7.0), (0.0, 2.0)], [1.05, 0.1, 0.0, -0.1, 1.9]),
            (0, -1, [(4.0, 6.0), (1.0, 5.0), (-1.0, 7.0)], [0.95, 0.0, 0.1, 0.0, 1.7])]),
    }


def _sp(case, sponges):
    case.sponges = sponges
    return case


def _sigma_ref(case, row):
    """BCSponge.c:49-54 on the deck's coordinates over the zone's FindInterval range."""
    dim, face, box = row[0], row[1], row[2]
    x = np.asarray(case.x[dim], np.float64)
    lo, hi = O.find_interval(box[dim][0], box[dim][1], x)
    xs, xe = box[dim]
    xx = x[lo:hi]
    return (xx - xs) / (xe - xs) if face > 0 else (xx - xe) / (xs - xe), lo, hi


@pytest.mark.parametrize("name", ["sod", "vortex", "tgv"])
def test_reader_sponge_sigma_and_extent(built_lib, tmp_path, name):
    case = decks()[name]
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    c = inp.config
    nface = 2 * case.ndims
    assert c.nzones == nface + len(case.sponges)
    for k, row in enumerate(case.sponges):
        z = nface + k
        q = list(c.zones[z])
        assert q[0] == GB_BC_SPONGE and q[1] == row[0] and q[2] == row[1]
        for e in range(case.ndims):
            lo, hi = O.find_interval(row[2][e][0], row[2][e][1], np.asarray(case.x[e]))
            assert (q[3 + e], q[6 + e]) == (lo, hi), (z, e)
        assert list(c.zone_data[z])[:case.nvars] == list(row[3])
        ref, lo, hi = _sigma_ref(case, row)
        assert np.array_equal(inp.zone_sponge[z], ref)
    # the face zones carry no sigma
    assert set(inp.zone_sponge) == {nface + k for k in range(len(case.sponges))}


def test_sponge_extent_in_ghosts_rejected(built_lib, tmp_path):
    case = decks()["vortex"]
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    cfg = inp.config
    z = 2 * case.ndims
    cfg.zones[z][3] = -1  # into the ghost points along x
    with pytest.raises(_lib.GbError) as e:
        Solver(cfg, inp.dxinv, 0)
    assert e.value.code == GB_ERR_ARG


def test_sponge_not_in_ensemble_or_noalloc(built_lib, tmp_path):
    """The batched ensemble and the allocation-free right-hand side have no sigma: both
    refuse a sponge zone while checking the configuration, before any device work (the
    arrays passed here are host memory, so this runs on machines without a GPU only)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("host arrays stand in for device arrays here")
    case = decks()["vortex"]
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    cfg = inp.config
    buf = np.zeros(8)
    p = buf.ctypes.data_as(ctypes.c_void_p)
    rc = _lib.lib().gb_rhs_explicit_noalloc(ctypes.byref(cfg), p, p, p, None)
    assert rc == GB_ERR_UNSUPPORTED, _lib.lib().gb_last_error()
    dx = inp.dxinv.ctypes.data_as(_lib.DP)
    arr = (_lib.DP * 1)(dx)
    h = ctypes.c_void_p()
    rc = _lib.lib().gb_ensemble_create(ctypes.byref(cfg), arr, 1, 0, ctypes.byref(h))
    assert rc == GB_ERR_UNSUPPORTED, _lib.lib().gb_last_error()


# ---------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------

def _solver(case, tmp_path):
    d = str(tmp_path / "deck")
    case.write(d)
    return Solver.from_dir(d, device=0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sod", "vortex", "tgv"])
def test_sponge_source_bit_exact(built_lib, oracle_lib, tmp_path, name):
    torch = pytest.importorskip("torch")
    case = decks()[name]
    s = _solver(case, tmp_path)
    P = O.Problem(case)
    u0 = P.apply_bc(P.u0())
    u = torch.from_numpy(u0).cuda()
    src = torch.full_like(u, 5.0)
    s.source(src, u)
    got = src.cpu().numpy()
    ref = P.source(u0)
    assert np.array_equal(got, ref)
    assert np.count_nonzero(ref) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sod", "vortex", "tgv"])
def test_sponge_rhs_and_steps(built_lib, oracle_lib, tmp_path, name):
    torch = pytest.importorskip("torch")
    case = decks()[name]
    s = _solver(case, tmp_path)
    P = O.Problem(case)
    u0 = P.u0()
    u = torch.from_numpy(u0).cuda()
    out = torch.full_like(u, 7.0)
    s.rhs(out, u)
    ref = O.interior(P.rhs(u0), case.size, case.nvars, 3)
    got = O.interior(out.cpu().numpy(), case.size, case.nvars, 3)
    assert relerr(got, ref) <= RHS_TOL
    # the sponge changes the solution: compare with a run without it
    s.step(case.n_iter)
    got = s.get_state()
    ref = O.interior(P.rk(P.u0(), case.n_iter), case.size, case.nvars, 3).reshape(-1)
    assert relerr(got, ref) <= STEP_TOL
    case.sponges = None
    P0 = O.Problem(case)
    free = O.interior(P0.rk(P0.u0(), case.n_iter), case.size, case.nvars, 3).reshape(-1)
    assert relerr(free, ref) > 1e3 * STEP_TOL


@pytest.mark.gpu
def test_boundary_fields_required(built_lib, tmp_path):
    """A solver created from the configuration alone (no sigma, no wall temperature)
    refuses to evaluate, with GB_ERR_ARG, and works once the field is uploaded."""
    torch = pytest.importorskip("torch")
    case = decks()["vortex"]
    d = str(tmp_path / "a")
    case.write(d)
    inp = Inputs(d)
    s = Solver(inp.config, inp.dxinv, 0)
    s.set_state(inp.u0)
    u = torch.zeros(O.Problem(case).npts_wg * case.nvars, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(u)
    with pytest.raises(_lib.GbError) as e:
        s.rhs(out, u)
    assert e.value.code == GB_ERR_ARG
    for z, sg in inp.zone_sponge.items():
        s.set_zone_sponge(z, sg)
    s.step(1)
    tgv = C.tgv(12, n_iter=1, dt=0.02, perturb=0.05)
    tgv.bcs = {(2, 1): ("thermal-noslip-wall", [0.0, 0.0, 0.0], ([0.0], np.full(144, 0.7))),
               (2, -1): ("thermal-noslip-wall", [0.0, 0.0, 0.0], ([0.0], np.full(144, 0.7)))}
    d = str(tmp_path / "b")
    tgv.write(d)
    inp = Inputs(d)
    s = Solver(inp.config, inp.dxinv, 0)
    s.set_state(inp.u0)
    with pytest.raises(_lib.GbError) as e:
        s.step(1)
    assert e.value.code == GB_ERR_ARG
    for z, (times, field) in inp.zone_temperature.items():
        s.set_zone_temperature(z, times, field)
    s.step(1)
