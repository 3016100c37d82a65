"""Batched ensemble (gb_ensemble): members of mixed sizes advanced by one launch
per direction per stage inside a CUDA graph must equal single-grid runs (the
same device code on the same data: bit for bit) and the reference's own
ensemble output (tests/golden, within 1e-10)."""
import os

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import cases as C
from hypar_gb300.solver import Ensemble, Solver, run_case

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("interp,scheme", [("characteristic", "ssprk3"), ("components", "44")])
def test_ensemble_equals_single_runs(built_lib, tmp_path, interp, scheme):
    members = C.ensemble_vortex(5, sizes=[16, 40, 24, 64, 32], n_iter=3, seed=3, interp=interp, scheme=scheme)
    d = str(tmp_path / "ens")
    C.write_ensemble(members, d)
    e = Ensemble.from_dir(d)
    assert len(e) == 5
    e.step(3)
    for k, case in enumerate(members):
        sd = str(tmp_path / f"m{k}")
        case.write(sd)
        s = Solver.from_dir(sd)
        s.step(3)
        assert np.array_equal(e.get_state(k), s.get_state())


def test_ensemble_autotune_keeps_results(built_lib, tmp_path):
    members = C.ensemble_vortex(4, sizes=[24, 48, 32, 16], n_iter=2, seed=5)
    d = str(tmp_path / "ens")
    C.write_ensemble(members, d)
    a = Ensemble.from_dir(d)
    a.step(2)
    ref = [a.get_state(k) for k in range(4)]
    b = Ensemble.from_dir(d)
    tuned = b.autotune(1)
    assert all(s > 0 or s in (-32, -64, -128) for s, _ in tuned)
    assert all(b > 0 or (b == -1 and s < 0) for s, b in tuned)
    b.step(2)
    for k in range(4):
        assert np.array_equal(b.get_state(k), ref[k])


@pytest.mark.parametrize("tile", [32, 64, 128])
@pytest.mark.parametrize("interp,upw", [("characteristic", "roe"), ("components", "llf-char")])
def test_ensemble_tiles(built_lib, oracle_lib, tmp_path, tile, interp, upw):
    """The tile form of the batched kernel (gb_ensemble_set_launch seg = -tile): equal
    to single-grid runs in the same form (the same device code) and to the oracle."""
    members = C.ensemble_vortex(4, sizes=[16, 72, 40, 136], n_iter=3, seed=17, interp=interp, upwinding=upw,
                                scheme="ssprk3")
    d = str(tmp_path / "ens")
    C.write_ensemble(members, d)
    e = Ensemble.from_dir(d)
    for dd in range(2):
        e.set_launch(dd, -tile, 0)
        assert e.get_launch(dd)[0] == -tile
    e.step(3)
    for k, case in enumerate(members):
        sd = str(tmp_path / f"m{k}")
        case.write(sd)
        s = Solver.from_dir(sd)
        for dd in range(2):
            s.set_launch(dd, -tile, 0)
        s.step(3)
        assert np.array_equal(e.get_state(k), s.get_state())
        P = O.Problem(case)
        ref = O.interior(P.rk(P.u0(), 3), case.size, case.nvars, 3).reshape(-1)
        assert relerr(e.get_state(k), ref) <= 1e-10


@pytest.mark.parametrize("tile", [32, 128])
@pytest.mark.parametrize("interp,scheme", [("characteristic", "ssprk3"), ("components", "44")])
def test_ensemble_worklist(built_lib, oracle_lib, tmp_path, tile, interp, scheme):
    """The persistent work-list form (gb_ensemble_set_launch block = -1 with a tile
    form): one launch per stage and direction of as many blocks as the SMs hold,
    taking the members' tiles from a counter.  Each tile is computed by the same
    device code as in the one-block-per-tile launch, so the members equal
    single-grid runs in the tile form bit for bit, over many graph replays (the
    counters are cleared every step)."""
    members = C.ensemble_vortex(6, sizes=[16, 72, 40, 136, 24, 200], n_iter=5, seed=19, interp=interp,
                                scheme=scheme)
    d = str(tmp_path / "ens")
    C.write_ensemble(members, d)
    e = Ensemble.from_dir(d)
    for dd in range(2):
        e.set_launch(dd, -tile, -1)
        assert e.get_launch(dd) == (-tile, -1)
    e.step(5)
    for k, case in enumerate(members):
        sd = str(tmp_path / f"m{k}")
        case.write(sd)
        s = Solver.from_dir(sd)
        for dd in range(2):
            s.set_launch(dd, -tile, 0)
        s.step(5)
        assert np.array_equal(e.get_state(k), s.get_state())
    P = O.Problem(members[2])
    ref = O.interior(P.rk(P.u0(), 5), members[2].size, 4, 3).reshape(-1)
    assert relerr(e.get_state(2), ref) <= 1e-10
    # a walker shape cannot take the persistent form; back to one block per tile
    with pytest.raises(Exception):
        e.set_launch(0, 16, -1)
    e.set_launch(0, -tile, 128)
    assert e.get_launch(0) == (-tile, 128)


def test_ensemble_vs_oracle(built_lib, oracle_lib, tmp_path):
    members = C.ensemble_vortex(3, sizes=[20, 28, 36], n_iter=4, seed=11)
    d = str(tmp_path / "ens")
    C.write_ensemble(members, d)
    e = Ensemble.from_dir(d)
    e.step(4)
    for k, case in enumerate(members):
        P = O.Problem(case)
        ref = O.interior(P.rk(P.u0(), 4), case.size, case.nvars, 3).reshape(-1)
        assert relerr(e.get_state(k), ref) <= 1e-10


def test_ensemble_golden_run_case(built_lib, tmp_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    for name, mk in mod.ENSEMBLES.items():
        g = np.load(os.path.join(GOLDEN, name + ".npz"))
        members = mk()
        d = str(tmp_path / name)
        C.write_ensemble(members, d)
        run_case(d)
        for k in range(len(members)):
            op = C.read_op_bin(os.path.join(d, f"op_{k}.bin"))
            assert relerr(op["u"], g[f"uN_{k}"]) <= 1e-10


def test_ensemble_error_and_counts_files(built_lib, tmp_path):
    """An ensemble deck with exact_<k>.inp per member: errors_<k>.dat equals the
    single-grid run's errors.dat (CalculateError per member), and conservation_<k>.dat /
    function_counts_<k>.dat are written per member."""
    members = C.ensemble_vortex(3, sizes=[16, 24, 20], n_iter=3, seed=9)
    d = str(tmp_path / "ens")
    C.write_ensemble(members, d)

    def exact_bytes(c):
        xs = np.concatenate([np.asarray(x, np.float64) for x in c.x])
        return xs.tobytes() + np.ascontiguousarray(c.u * 1.01).tobytes()

    for k, c in enumerate(members):
        with open(os.path.join(d, f"exact_{k}.inp"), "wb") as f:
            f.write(exact_bytes(c))
    run_case(d)
    for k, c in enumerate(members):
        sd = str(tmp_path / f"m{k}")
        c.write(sd)
        with open(os.path.join(sd, "exact.inp"), "wb") as f:
            f.write(exact_bytes(c))
        run_case(sd)
        ens = open(os.path.join(d, f"errors_{k}.dat")).read().split()
        one = open(os.path.join(sd, "errors.dat")).read().split()
        # sizes, iproc, dt, L1, L2, Linf (the runtimes differ)
        assert ens[:2 * 2 + 4] == one[:2 * 2 + 4]
        assert float(ens[2 * 2 + 1]) > 0
        cons = open(os.path.join(d, f"conservation_{k}.dat")).read().split()[2 * 2 + 1:]
        assert [float(v) for v in cons] == [-1.0] * 4
        assert open(os.path.join(d, f"function_counts_{k}.dat")).read().split() == ["3", "9", "0", "0"]
