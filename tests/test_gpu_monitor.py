"""The quantities around a time step, reduced on the device: the model's CFL
number (bit-identical to the reference's ComputeCFL), the norm of a step's
change, the error norms against an exact solution; and the driver's restart
runs, report lines and errors.dat."""
import importlib.util
import os

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import cases as C
from hypar_gb300.solver import Solver, run_case

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _golden_cases():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.CASES


GOLD = _golden_cases()


def rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


def deck(case, tmp_path, name="deck"):
    d = str(tmp_path / name)
    case.write(d)
    return d


@pytest.mark.parametrize("name", sorted(GOLD))
def test_cfl_matches_reference(built_lib, tmp_path, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    s = Solver.from_dir(deck(GOLD[name](), tmp_path))
    assert s.cfl() == float(g["cfl"])


@pytest.mark.parametrize("case", [C.sod(64, n_iter=3, dt=1e-3), C.vortex(32, n_iter=3, dt=0.02),
                                  C.tgv(12, n_iter=3, dt=0.02, perturb=0.05)], ids=["sod", "vortex", "tgv"])
def test_step_report(built_lib, oracle_lib, tmp_path, case):
    s = Solver.from_dir(deck(case, tmp_path))
    P = O.Problem(case)
    # the CFL of the device's own state, to the bit
    s.step(2)
    u2 = s.get_state(ghosted=True)
    assert s.cfl() == P.cfl(u2)
    cfl, norm = s.step_report(1)
    assert cfl == P.cfl(u2)
    u3 = s.get_state(ghosted=True)
    d = O.interior(u3, case.size, case.nvars, 3) - O.interior(u2, case.size, case.nvars, 3)
    ref = float(np.sqrt(np.sum(d * d) / np.prod(case.size)))
    assert rel(norm, ref) <= 1e-13
    # and against the oracle's trajectory
    o2 = P.rk(P.u0(), 2)
    o3 = P.rk(o2, 1)
    do = O.interior(o3, case.size, case.nvars, 3) - O.interior(o2, case.size, case.nvars, 3)
    assert rel(norm, float(np.sqrt(np.sum(do * do) / np.prod(case.size)))) <= 1e-9
    assert rel(cfl, P.cfl(o2)) <= 1e-13


def test_error_norms(built_lib, tmp_path):
    case = C.vortex(40, n_iter=2, dt=0.02)
    s = Solver.from_dir(deck(case, tmp_path))
    s.step(2)
    u = s.get_state()
    rng = np.random.default_rng(3)
    uex = u * (1.0 + 1e-3 * rng.standard_normal(u.shape))
    npts = np.prod(case.size)
    e = u - uex
    want = (np.abs(e).sum() / npts / (np.abs(uex).sum() / npts),
            np.sqrt((e * e).sum() / npts) / np.sqrt((uex * uex).sum() / npts),
            np.abs(e).max() / np.abs(uex).max())
    got = s.error(uex)
    for a, b in zip(got, want):
        assert rel(a, b) <= 1e-13
    assert s.error(torch.from_numpy(uex).cuda()) == got  # device input, same reduction


def test_restart_run_continues_the_run(built_lib, tmp_path):
    """A restart from op_00001 (iteration 4) reproduces the continuous run's later states
    bit for bit, with the reference's restart file numbering (the index is fast-forwarded
    over the outputs before restart_iter, InitializeSolvers.c:438-442)."""
    case = C.vortex(32, n_iter=12, dt=0.02)
    case.op_overwrite, case.file_op_iter, case.screen_op_iter = "no", 4, 2
    d = deck(case, tmp_path, "full")
    run_case(d)
    names = sorted(f for f in os.listdir(d) if f.startswith("op_"))
    assert names == ["op_00000.bin", "op_00001.bin", "op_00002.bin", "op_00003.bin"]
    full = {n: C.read_op_bin(os.path.join(d, n))["u"] for n in names}
    case.restart_iter = 4
    r = deck(case, tmp_path, "restart")
    from hypar_gb300 import _lib
    _lib.check(_lib.lib().gb_op_to_initial(os.path.join(d, "op_00001.bin").encode(),
                                           os.path.join(r, "initial.inp").encode()))
    run_case(r)
    rn = sorted(f for f in os.listdir(r) if f.startswith("op_"))
    assert rn == ["op_00001.bin", "op_00002.bin"]
    assert np.array_equal(C.read_op_bin(os.path.join(r, "op_00001.bin"))["u"], full["op_00002.bin"])
    assert np.array_equal(C.read_op_bin(os.path.join(r, "op_00002.bin"))["u"], full["op_00003.bin"])


def test_errors_dat(built_lib, tmp_path):
    """gb_run_case with exact.inp writes errors.dat (SimulationWriteErrors.c layout)."""
    case = C.vortex(32, n_iter=4, dt=0.02)
    d = deck(case, tmp_path)
    T = case.n_iter * case.dt
    _, uex = C.vortex_state(32, 5.0, 5.0 + 0.5 * T, 5.0)
    xs = np.concatenate([np.asarray(x, np.float64) for x in case.x])
    with open(os.path.join(d, "exact.inp"), "wb") as f:
        f.write(xs.tobytes() + np.ascontiguousarray(uex).tobytes())
    run_case(d)
    tok = open(os.path.join(d, "errors.dat")).read().split()
    assert [int(t) for t in tok[:4]] == [32, 32, 1, 1]
    assert float(tok[4]) == case.dt
    errs = [float(t) for t in tok[5:8]]
    s = Solver.from_dir(d)
    s.step(case.n_iter)
    got = s.error(uex)
    for a, b in zip(errs, got):
        assert rel(a, b) <= 1e-15
    assert 0 < errs[1] < 1e-2
    # no exact.inp: the reference's -1 errors
    os.remove(os.path.join(d, "exact.inp"))
    run_case(d)
    assert [float(t) for t in open(os.path.join(d, "errors.dat")).read().split()[5:8]] == [-1.0, -1.0, -1.0]


def test_conservation_check_api(built_lib, tmp_path):
    """gb_solver_conservation_*: a periodic vortex conserves to rounding, an
    extrapolate-bounded Sod tube once its boundary fluxes are counted; the launch-shape
    autotuner's trial steps add nothing; the ensemble gives each member's value."""
    from hypar_gb300.solver import Ensemble
    vort = C.vortex(32, n_iter=6, dt=0.02)
    d = str(tmp_path / "v")
    vort.write(d)
    s = Solver.from_dir(d)
    s.conservation_begin()
    s.autotune(1)
    s.step(6)
    ev = s.conservation_error()
    assert ev.shape == (4,) and np.all(ev < 1e-13), ev
    sod = C.sod(64, n_iter=30, dt=1e-3)
    d = str(tmp_path / "s")
    sod.write(d)
    s = Solver.from_dir(d)
    with pytest.raises(RuntimeError):
        s.conservation_error()  # no begin
    s.conservation_begin()
    s.step(30)
    es = s.conservation_error()
    assert np.all(es < 1e-13), es
    members = C.ensemble_vortex(3, sizes=[16, 24, 20], n_iter=4, seed=7)
    d = str(tmp_path / "e")
    C.write_ensemble(members, d)
    e = Ensemble.from_dir(d)
    e.conservation_begin()
    e.step(4)
    for k, m in enumerate(members):
        sd = str(tmp_path / f"m{k}")
        m.write(sd)
        one = Solver.from_dir(sd)
        one.conservation_begin()
        one.step(4)
        assert np.allclose(e.conservation_error(k), one.conservation_error(), rtol=0, atol=1e-14)
