"""CPU-side checks of the C ABI: every declared symbol is exported, the input
reader reproduces the reference's set-up, and bad decks fail cleanly."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import _lib, cases as C
from hypar_gb300.solver import Inputs, rk_table

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gbhypar.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 30
    L = ctypes.CDLL(built_lib)
    for n in names:
        assert hasattr(L, n), n
    assert sorted(_lib.EXPORTS) == names


@pytest.mark.parametrize("mk", [
    lambda: C.sod(50, n_iter=3),
    lambda: C.vortex(20, n_iter=2, dt=0.01, interp="components", upwinding="llf-char"),
    lambda: C.tgv(10, n_iter=1, upwinding="rf-char", interp="characteristic", scheme="33"),
])
def test_reader_matches_reference_setup(built_lib, oracle_lib, tmp_path, mk):
    case = mk()
    case.write(str(tmp_path))
    inp = Inputs(str(tmp_path))
    c = inp.config
    P = O.Problem(case)
    assert np.array_equal(inp.dxinv, P.dxinv)
    zones = np.array([list(c.zones[z]) for z in range(c.nzones)], dtype=np.int32)
    assert np.array_equal(zones, P.zones)
    assert np.array_equal(inp.u0, case.u.reshape(-1))
    assert np.array_equal(inp.x, np.concatenate(case.x))
    assert c.model == _lib.MODEL[case.model]
    assert c.interp == _lib.INTERP[case.interp] and c.upwind == _lib.UPWIND[case.upwinding]
    assert c.dt == case.dt and c.n_iter == case.n_iter
    ns, A, b, cc = rk_table(case.time_scheme_type)
    ons, oA, ob = O.RK_TABLES[case.time_scheme_type]
    assert ns == ons and c.rk_nstages == ns
    for i in range(ns):
        assert b[i] == ob[i]
        for j in range(ns):
            assert A[4 * i + j] == oA[ns * i + j] == c.rk_A[4 * i + j]
    if case.model == "navierstokes3d":
        assert c.Re == case.Re and c.Minf == case.Minf and c.Pr == case.Pr


def test_ascii_initial_file(built_lib, tmp_path):
    case = C.sod(16, n_iter=1)
    case.write(str(tmp_path))
    txt = open(tmp_path / "solver.inp").read().replace("ip_file_type      binary", "ip_file_type      ascii")
    open(tmp_path / "solver.inp", "w").write(txt)
    with open(tmp_path / "initial.inp", "w") as f:
        f.write(" ".join(repr(float(v)) for v in case.x[0]) + "\n")
        for v in range(3):
            f.write(" ".join(repr(float(a)) for a in case.u[:, v]) + "\n")
    inp = Inputs(str(tmp_path))
    assert np.array_equal(inp.u0, case.u.reshape(-1))


def _expect(code, directory):
    with pytest.raises(_lib.GbError) as e:
        Inputs(directory)
    assert e.value.code == code, str(e.value)


def test_reader_errors(built_lib, tmp_path):
    _expect(3, str(tmp_path / "nowhere"))
    case = C.vortex(12, n_iter=1, dt=0.01)
    d = tmp_path / "b"
    case.write(str(d))
    t = open(d / "boundary.inp").read().replace("periodic", "numa-nfbc", 1)
    open(d / "boundary.inp", "w").write(t)
    _expect(4, str(d))
    d = tmp_path / "c"
    case.write(str(d))
    t = open(d / "solver.inp").read().replace("euler2d", "shallowwater2d")
    open(d / "solver.inp", "w").write(t)
    _expect(4, str(d))
    d = tmp_path / "e"
    case.write(str(d))
    t = open(d / "solver.inp").read().replace("weno5", "hcweno5")
    open(d / "solver.inp", "w").write(t)
    _expect(4, str(d))
    d = tmp_path / "f"
    case.write(str(d))
    with open(d / "initial.inp", "r+b") as f:
        f.truncate(100)
    _expect(3, str(d))
    d = tmp_path / "g"
    case.write(str(d))
    open(d / "physics.inp", "w").write("begin\n gamma 1.4\n upwinding ausm\nend\n")
    _expect(4, str(d))


@pytest.mark.parametrize("flags,expect", [
    ("", 0), ("mapped 1", 1), ("borges 1", 2), ("yc 1", 3), ("no_limiting 1", 4),
    ("mapped 1\n borges 1", 2), ("borges 1\n yc 1", 3), ("mapped 1\n no_limiting 1", 4)])
def test_reader_weno_weights(built_lib, tmp_path, flags, expect):
    """weno.inp flags -> gb_config.weno_weights with the reference's precedence
    (yc, borges, mapped; no_limiting keeps the optimal weights)."""
    case = C.vortex(12, n_iter=1, dt=0.01)
    d = str(tmp_path / "deck")
    case.write(d)
    open(os.path.join(d, "weno.inp"), "w").write(f"begin\n {flags}\n epsilon 1e-6\nend\n")
    assert Inputs(d).config.weno_weights == expect


def test_solver_create_rejects_bad_config(built_lib):
    cfg = _lib.GbConfig()
    cfg.model = 9
    dx = np.zeros(10)
    h = ctypes.c_void_p()
    rc = _lib.lib().gb_solver_create(ctypes.byref(cfg), dx.ctypes.data_as(_lib.DP), -1, ctypes.byref(h))
    assert rc == 1 and not h.value
    assert b"unknown model" in _lib.lib().gb_last_error()


def test_reader_restart_screen_and_exact(built_lib, tmp_path):
    """restart_iter / screen_op_iter from solver.inp, exact.inp in initial.inp's format."""
    case = C.vortex(12, n_iter=6, dt=0.01)
    case.restart_iter = 4
    case.screen_op_iter = 2
    d = str(tmp_path / "deck")
    case.write(d)
    inp_h = ctypes.c_void_p()
    L = _lib.lib()
    _lib.check(L.gb_inputs_read(d.encode(), ctypes.byref(inp_h)))
    c = L.gb_inputs_config(inp_h).contents
    assert (c.restart_iter, c.screen_op_iter, c.write_residual) == (4, 2, 0)
    assert not L.gb_inputs_exact(inp_h)
    L.gb_inputs_free(inp_h)
    ex = case.u * 1.5
    xs = np.concatenate([np.asarray(x, np.float64) for x in case.x])
    with open(os.path.join(d, "exact.inp"), "wb") as f:
        f.write(xs.tobytes() + np.ascontiguousarray(ex).tobytes())
    _lib.check(L.gb_inputs_read(d.encode(), ctypes.byref(inp_h)))
    p = L.gb_inputs_exact(inp_h)
    assert p
    got = np.ctypeslib.as_array(p, shape=(ex.size,)).copy()
    L.gb_inputs_free(inp_h)
    assert np.array_equal(got, ex.reshape(-1))


def test_reader_conservation_check(built_lib, tmp_path):
    """solver.inp conservation_check: "yes" turns it on, anything else (or absence) not."""
    L = _lib.lib()
    for flag, want in ((True, 1), (False, 0)):
        case = C.sod(16, n_iter=2, dt=1e-3)
        case.conservation_check = flag
        d = str(tmp_path / f"deck{want}")
        case.write(d)
        inp_h = ctypes.c_void_p()
        _lib.check(L.gb_inputs_read(d.encode(), ctypes.byref(inp_h)))
        assert L.gb_inputs_config(inp_h).contents.cons_check == want
        L.gb_inputs_free(inp_h)


@pytest.mark.parametrize("mode,fname", [("parallel", "initial_par.inp.0000"), ("mpi-io", "initial_mpi.inp")])
def test_reader_input_modes(built_lib, tmp_path, mode, fname):
    """solver.inp input_mode parallel / mpi-io: on one rank the initial solution comes from
    initial_par.inp.0000 / initial_mpi.inp (binary: grid, then solution), exact.inp likewise."""
    case = C.vortex(12, n_iter=1, dt=0.01)
    d = str(tmp_path / "deck")
    case.write(d)
    txt = open(os.path.join(d, "solver.inp")).read().replace("end", f"  input_mode {mode} 1\nend")
    open(os.path.join(d, "solver.inp"), "w").write(txt)
    os.rename(os.path.join(d, "initial.inp"), os.path.join(d, fname))
    xs = np.concatenate([np.asarray(x, np.float64) for x in case.x])
    with open(os.path.join(d, fname.replace("initial", "exact")), "wb") as f:
        f.write(xs.tobytes() + np.ascontiguousarray(case.u * 2.0).tobytes())
    L = _lib.lib()
    h = ctypes.c_void_p()
    _lib.check(L.gb_inputs_read(d.encode(), ctypes.byref(h)))
    n = case.u.size
    assert np.array_equal(np.ctypeslib.as_array(L.gb_inputs_u0(h), shape=(n,)), case.u.reshape(-1))
    assert np.array_equal(np.ctypeslib.as_array(L.gb_inputs_exact(h), shape=(n,)), 2.0 * case.u.reshape(-1))
    L.gb_inputs_free(h)
    # the serial file name is not read in these modes
    os.rename(os.path.join(d, fname), os.path.join(d, "initial.inp"))
    assert L.gb_inputs_read(d.encode(), ctypes.byref(h)) != 0


def test_op_to_initial_round_trip(built_lib, tmp_path):
    """gb_write_binary -> gb_op_to_initial -> the deck reader gives back x and u."""
    case = C.vortex(10, n_iter=1, dt=0.01)
    d = str(tmp_path / "deck")
    case.write(d)
    L = _lib.lib()
    xs = np.concatenate([np.asarray(x, np.float64) for x in case.x])
    u = np.ascontiguousarray(case.u * 0.75)
    dims = (ctypes.c_int * 2)(*case.size)
    op = os.path.join(d, "op_00003.bin")
    _lib.check(L.gb_write_binary(op.encode(), 2, 4, dims, xs.ctypes.data_as(_lib.DP), u.ctypes.data_as(_lib.DP)))
    _lib.check(L.gb_op_to_initial(op.encode(), os.path.join(d, "initial.inp").encode()))
    inp = Inputs(d)
    assert np.array_equal(inp.u0, u.reshape(-1))
    assert np.array_equal(inp.x, xs)
    assert L.gb_op_to_initial(os.path.join(d, "solver.inp").encode(), os.path.join(d, "junk").encode()) == 3


def test_reader_boundary_values(built_lib, tmp_path):
    """Wall / inflow / outflow / Dirichlet zones: type codes and the values after the extents."""
    case = C.vortex(12, n_iter=1, dt=0.01)
    case.bcs = {(0, 1): ("supersonic-inflow", [1.0, 0.5, 0.25, 1.0]), (0, -1): ("subsonic-outflow", [0.9]),
                (1, 1): ("slip-wall", [0.0, 0.125]), (1, -1): ("dirichlet", [1.0, 0.5, 0.0, 2.625])}
    d = str(tmp_path / "deck")
    case.write(d)
    c = Inputs(d).config
    codes = [c.zones[z][0] for z in range(c.nzones)]
    assert codes == [8, 7, 4, 3]
    assert list(c.zone_data[0])[:4] == [1.0, 0.5, 0.25, 1.0]
    assert c.zone_data[1][0] == 0.9
    assert list(c.zone_data[2])[:2] == [0.0, 0.125]
    assert list(c.zone_data[3])[:4] == [1.0, 0.5, 0.0, 2.625]
    # of the wall / inflow / outflow types only the slip wall has a 1-D branch
    # (BCSlipWall.c:38-76); the others are 2-D / 3-D only
    sod = C.sod(16, n_iter=1, dt=1e-3)
    sod.bcs = {(0, 1): ("slip-wall", [0.0]), (0, -1): ("slip-wall", [0.5])}
    d = str(tmp_path / "sod")
    sod.write(d)
    c = Inputs(d).config
    assert [c.zones[z][0] for z in range(2)] == [4, 4] and c.zone_data[1][0] == 0.5
    sod.bcs = {(0, 1): ("noslip-wall", [0.0])}
    d = str(tmp_path / "sod_noslip")
    sod.write(d)
    _expect(4, d)


@pytest.mark.parametrize("hb,axis", [(1, 1), (2, 1), (3, 2)])
def test_reader_gravity_fields(built_lib, oracle_lib, tmp_path, hb, axis):
    """physics.inp gravity / rho_ref / p_ref / R / HB (/ N_bv): the reader's hydrostatic
    fields f and g, ghost layers included, are bit-identical to the oracle's
    (NavierStokes3DGravityField.c:36-153)."""
    case = C.rising_thermal_bubble(10, n_iter=1, HB=hb)
    if axis == 2:
        case.gravity, case.N_bv = (0.0, 0.0, 9.8), 0.01
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    c = inp.config
    assert list(c.gravity) == list(case.gravity) and c.HB == hb
    assert (c.rho_ref, c.p_ref, c.R_gas) == (case.rho_ref, case.p_ref, case.R_gas)
    assert c.N_bv == (0.01 if hb == 3 else 0.0)
    ref = O.Problem(case).gravity_field()
    assert inp.gravity_field is not None and np.array_equal(inp.gravity_field, ref)
    assert Inputs(str(_deck(tmp_path / "plain", C.tgv(8, n_iter=1)))).gravity_field is None


def _deck(d, case):
    case.write(str(d))
    return d


def test_reader_gravity_errors(built_lib, tmp_path):
    """Gravity needs rusanov upwinding (NavierStokes3DInitialize.c:370-378); HB = 3 only
    along z (NavierStokes3DGravityField.c:98-106); Euler2D has none."""
    case = C.rising_thermal_bubble(8, n_iter=1)
    case.upwinding = "roe"
    _expect(3, str(_deck(tmp_path / "a", case)))
    case = C.rising_thermal_bubble(8, n_iter=1, HB=3)
    _expect(3, str(_deck(tmp_path / "b", case)))
    d = _deck(tmp_path / "c", C.vortex(12, n_iter=1, dt=0.01))
    open(d / "physics.inp", "w").write("begin\n gamma 1.4\n upwinding roe\n gravity 1.0\nend\n")
    _expect(4, str(d))  # Euler2D has no gravity


def test_solver_create_rejects_bad_gravity(built_lib):
    """gb_solver_create validates before touching a device: gravity outside
    NavierStokes3D and Euler1D, or with another upwinding than rusanov (NavierStokes3D), is refused."""
    L = _lib.lib()
    dx = np.zeros(64)
    for model, nd, upw, rc_want, msg in (("euler2d", 2, "roe", 4, b"Euler2D has none"),
                                         ("navierstokes3d", 3, "roe", 1, b"rusanov")):
        cfg = _lib.GbConfig()
        cfg.model, cfg.ndims, cfg.nvars, cfg.ghosts = _lib.MODEL[model], nd, nd + 2, 3
        for dd in range(nd):
            cfg.dim[dd] = 8
        cfg.upwind, cfg.rk_nstages, cfg.gamma, cfg.weno_eps = _lib.UPWIND[upw], 1, 1.4, 1e-6
        cfg.gravity[1], cfg.rho_ref, cfg.p_ref = 9.8, 1.0, 1.0
        h = ctypes.c_void_p()
        rc = L.gb_solver_create(ctypes.byref(cfg), dx.ctypes.data_as(_lib.DP), -1, ctypes.byref(h))
        assert not h.value
        assert rc == rc_want and msg in L.gb_last_error(), (rc, L.gb_last_error())


def test_reader_crweno(built_lib, tmp_path):
    """hyp_space_scheme crweno5 -> gb_config.hyp_scheme (component-wise and
    characteristic), with gravity too (both models that have it)."""
    case = C.sod(16, n_iter=1)
    case.hyp_scheme = "crweno5"
    assert Inputs(str(_deck(tmp_path / "a", case))).config.hyp_scheme == _lib.SCHEME["crweno5"]
    assert Inputs(str(_deck(tmp_path / "b", C.sod(16, n_iter=1)))).config.hyp_scheme == _lib.SCHEME["weno5"]
    case = C.vortex(12, n_iter=1, dt=0.01)  # characteristic
    case.hyp_scheme = "crweno5"
    c = Inputs(str(_deck(tmp_path / "c", case))).config
    assert c.hyp_scheme == _lib.SCHEME["crweno5"] and c.interp == _lib.INTERP["characteristic"]
    case = C.rising_thermal_bubble(8, n_iter=1)
    case.hyp_scheme = "crweno5"
    c = Inputs(str(_deck(tmp_path / "d", case))).config
    assert c.hyp_scheme == _lib.SCHEME["crweno5"] and c.gravity[1] == 9.8
    case = C.stratified_1d(16, n_iter=1, interp="characteristic")
    case.hyp_scheme = "crweno5"
    c = Inputs(str(_deck(tmp_path / "e", case))).config
    assert c.hyp_scheme == _lib.SCHEME["crweno5"] and c.gravity[0] == 1.0


@pytest.mark.parametrize("grav_type", [0, 1])
def test_reader_euler1d_gravity(built_lib, oracle_lib, tmp_path, grav_type):
    """physics.inp gravity / gravity_type for Euler1D: the field 1/S then S, bit-identical
    to the oracle's (Euler1DGravityField.c); gravity needs roe or llf-char upwinding."""
    case = C.stratified_1d(32, n_iter=1, grav_type=grav_type)
    inp = Inputs(str(_deck(tmp_path / "a", case)))
    assert inp.config.grav_type == grav_type and inp.config.gravity[0] == 1.0
    assert np.array_equal(inp.gravity_field, O.Problem(case).gravity_field())
    case.upwinding = "rusanov"
    _expect(3, str(_deck(tmp_path / "b", case)))


def _solver_inp_with(d, extra):
    t = open(d + "/solver.inp").read().replace("end\n", extra + "\nend\n")
    open(d + "/solver.inp", "w").write(t)


def test_solver_inp_keywords_outside_the_flux(built_lib, tmp_path):
    """hyp_flux_split yes changes nothing for explicit Runge-Kutta on Euler1D and
    NavierStokes3D and is refused for Euler2D (Euler2DInitialize.c:79-85);
    immersed_body and a size_exact other than size are refused; size_exact equal to
    size, plot_solution, use_gpu and gpu_device_no are read and change nothing."""
    for name, case in (("sod", C.sod(16, n_iter=1)), ("tgv", C.tgv(6, n_iter=1))):
        d = str(tmp_path / name)
        case.write(d)
        base = Inputs(d).config
        _solver_inp_with(d, "  hyp_flux_split yes\n  plot_solution no\n  use_gpu yes\n  gpu_device_no 0\n"
                            "  size_exact " + " ".join(str(s) for s in case.size))
        cfg = Inputs(d).config
        assert bytes(cfg) == bytes(base)
    d = str(tmp_path / "vortex")
    C.vortex(12, n_iter=1, dt=0.01).write(d)
    _solver_inp_with(d, "  hyp_flux_split yes")
    _expect(3, d)
    for extra in ("  immersed_body body.stl", "  size_exact 32 32"):
        d = str(tmp_path / ("v" + str(abs(hash(extra)))))
        C.vortex(12, n_iter=1, dt=0.01).write(d)
        _solver_inp_with(d, extra)
        _expect(4, d)
