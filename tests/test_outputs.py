"""Solution files in op_file_format text / tecplot2d / tecplot3d, against files the
reference wrote (tests/golden/out_*.npz: header lines and the numeric table)."""
import ctypes
import importlib.util
import os

import numpy as np
import pytest

from hypar_gb300 import _lib

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
MG = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(MG)


def _write(fn, path, ndims, nvars, dim, x, u):
    L = _lib.lib()
    d = (ctypes.c_int * ndims)(*dim)
    x = np.ascontiguousarray(x, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    _lib.check(getattr(L, fn)(path.encode(), ndims, nvars, d, x.ctypes.data_as(_lib.DP), u.ctypes.data_as(_lib.DP)))


@pytest.mark.parametrize("name", sorted(MG.OUTPUTS))
def test_writers_reproduce_reference_files(built_lib, tmp_path, name):
    """gb_write_text / gb_write_tecplot given the reference's own solution write what
    the reference wrote (headers equal, every number equal)."""
    mk, files = MG.OUTPUTS[name]
    case = mk()
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    nd = case.ndims
    for k in range(len(files)):
        table = g[f"table_{k}"]
        x = np.concatenate([np.asarray(xx, dtype=np.float64) for xx in case.x])
        u = table[:, 2 * nd:]
        path = str(tmp_path / f"f{k}.dat")
        _write("gb_write_text" if case.op_format == "text" else "gb_write_tecplot", path, nd, case.nvars,
               case.size, x, u)
        header, got = MG.read_text_output(path)
        assert header == list(g[f"header_{k}"])
        assert np.array_equal(got, table)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MG.OUTPUTS))
def test_run_case_writes_the_reference_formats(built_lib, tmp_path, name):
    """gb_run_case with op_file_format text / tecplot2d / tecplot3d: the same files,
    indices and coordinates equal, the solution within 1e-10."""
    from hypar_gb300.solver import run_case
    mk, files = MG.OUTPUTS[name]
    case = mk()
    case.file_op_iter = case.n_iter if case.op_overwrite == "no" else None
    d = str(tmp_path / "deck")
    case.write(d)
    run_case(d)
    nd = case.ndims
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    for k, f in enumerate(files):
        header, got = MG.read_text_output(os.path.join(d, f))
        ref = g[f"table_{k}"]
        assert header == list(g[f"header_{k}"])
        assert np.array_equal(got[:, :2 * nd], ref[:, :2 * nd])
        err = np.linalg.norm(got[:, 2 * nd:] - ref[:, 2 * nd:]) / np.linalg.norm(ref[:, 2 * nd:])
        assert err <= 1e-10, err


def _bin(path, case, u):
    L = _lib.lib()
    d = (ctypes.c_int * case.ndims)(*case.size)
    x = np.concatenate([np.asarray(xx, dtype=np.float64) for xx in case.x])
    u = np.ascontiguousarray(u, dtype=np.float64)
    _lib.check(L.gb_write_binary(path.encode(), case.ndims, case.nvars, d, x.ctypes.data_as(_lib.DP),
                                 u.ctypes.data_as(_lib.DP)))


def test_diff_binary_is_hypardiff(built_lib, tmp_path):
    """gb_diff_binary / `gbhypar diff` against the norms of Extras/hyparDiff.c (restated
    here with numpy) and, where the reference was built here, against its own tool's
    output, line for line."""
    import subprocess
    from hypar_gb300 import cases as C
    from hypar_gb300.build import CLI
    case = C.vortex(12, n_iter=1, dt=0.01)
    rng = np.random.default_rng(5)
    ref = case.u.copy()
    sol = ref * (1.0 + 1e-9 * rng.standard_normal(ref.shape))
    a, b = str(tmp_path / "sol.bin"), str(tmp_path / "ref.bin")
    _bin(a, case, sol)
    _bin(b, case, ref)
    L = _lib.lib()
    ab, rl = (ctypes.c_double * 3)(), (ctypes.c_double * 3)()
    _lib.check(L.gb_diff_binary(a.encode(), b.encode(), ab, rl))
    d = (ref - sol).reshape(-1)
    npts = ref.shape[0]
    want_abs = [np.abs(d).sum() / npts, np.sqrt((d * d).sum() / npts), np.abs(d).max()]
    r = ref.reshape(-1)
    nrm = [np.abs(r).sum() / npts, np.sqrt((r * r).sum() / npts), np.abs(r).max()]
    assert np.allclose(list(ab), want_abs, rtol=1e-12, atol=0)
    assert np.allclose(list(rl), [x / y for x, y in zip(want_abs, nrm)], rtol=1e-12, atol=0)
    # a size mismatch is an input error
    small = C.vortex(8, n_iter=1, dt=0.01)
    c = str(tmp_path / "small.bin")
    _bin(c, small, small.u)
    assert L.gb_diff_binary(a.encode(), c.encode(), ab, rl) != 0
    out = subprocess.run([CLI, "diff", "-r", "1e-12", a, b], capture_output=True, text=True, check=True).stdout
    assert "differ." in out and "(rel)" in out
    same = subprocess.run([CLI, "diff", b, b], capture_output=True, text=True, check=True).stdout
    assert same == ""
    tool = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "hyparDiff")
    if os.path.exists(tool):
        theirs = subprocess.run([tool, "-r", "1e-12", a, b], capture_output=True, text=True, check=True).stdout
        assert out == theirs
