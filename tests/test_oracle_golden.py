"""The CPU oracle against golden vectors produced by the reference HyPar itself
(tests/golden/make_golden.py).  On the machine that made them the agreement is
bit for bit; elsewhere (another libm or CPU) it must stay at rounding level."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import cases as C

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.CASES


CASES = _cases()


def relerr(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_rhs_matches_reference(oracle_lib, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = CASES[name]()
    assert np.array_equal(case.u, g["u0"]), "deck generator drifted from the golden inputs"
    P = O.Problem(case)
    rhs = O.interior(P.rhs(P.u0()), case.size, case.nvars, 3)
    assert relerr(rhs, g["rhs"]) <= 1e-13
    if not np.array_equal(rhs, g["rhs"]):
        pytest.skip("agreement at rounding level only (different libm/CPU than the golden run)")


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_cfl_matches_reference(oracle_lib, name):
    """<Model>ComputeCFL of the initial state, to the bit."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = CASES[name]()
    P = O.Problem(case)
    assert P.cfl(P.u0()) == float(g["cfl"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_steps_match_reference(oracle_lib, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = CASES[name]()
    P = O.Problem(case)
    u = O.interior(P.rk(P.u0(), int(g["n_iter"])), case.size, case.nvars, 3)
    assert relerr(u, g["uN"]) <= 1e-12


def test_oracle_threads_deterministic(oracle_lib):
    case = C.vortex(20, n_iter=1, dt=0.02)
    P = O.Problem(case)
    O.set_threads(1)
    a = P.rhs(P.u0())
    O.set_threads(4)
    b = P.rhs(P.u0())
    O.set_threads(0)
    assert np.array_equal(a, b)


@pytest.mark.skipif(not O.ref_available(), reason="reference build oracle/_ref not present")
def test_oracle_matches_live_reference(oracle_lib, tmp_path):
    import subprocess
    case = C.vortex(16, n_iter=2, dt=0.03, interp="characteristic", upwinding="llf-char", scheme="44")
    case.write(str(tmp_path))
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.check_call([os.path.join(O.REF_DIR, "HyPar")], cwd=str(tmp_path), stdout=subprocess.DEVNULL, env=env)
    ref = C.read_op_bin(str(tmp_path / "op.bin"))["u"]
    P = O.Problem(case)
    u = O.interior(P.rk(P.u0(), 2), case.size, case.nvars, 3)
    assert np.array_equal(u, ref)


def _ensembles():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.ENSEMBLES


ENSEMBLES = _ensembles()


@pytest.mark.parametrize("name", sorted(ENSEMBLES))
def test_ensemble_members_are_independent_runs(oracle_lib, name):
    """The reference's ensemble mode advances every member exactly as a single
    run with the common time step would (each member against the oracle)."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    members = ENSEMBLES[name]()
    for k, case in enumerate(members):
        P = O.Problem(case)
        u = O.interior(P.rk(P.u0(), int(g["n_iter"])), case.size, case.nvars, 3)
        assert relerr(u, g[f"uN_{k}"]) <= 1e-13
