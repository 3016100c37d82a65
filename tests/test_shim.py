"""The HyPar-side binding (hypar_gb300/shim/gbhypar_attach.c) compiled against the
reference's own headers and linked with the reference's objects (oracle/_ref, built
from the reference's sources) and libgbhypar.so.

For several decks, the reference's start-up sequence initialises its structs; the
gb_config that gbshim_config() reads from them must equal the one libgbhypar's own
reader (gb_inputs_read) makes from the same files.  gbshim_attach() runs up to the
device set-up (GB_ERR_CUDA without a GPU).  Needs the reference's source tree
(HYPAR_REF, or the build's default location) and oracle/_ref/libhypar_ref.a; skipped
where either is absent, e.g. on a GPU machine."""
import os
import subprocess

import numpy as np
import pytest

import __graft_entry__ as G
from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = G.REFERENCE
LIBREF = os.path.join(ROOT, "oracle", "_ref", "libhypar_ref.a")

pytestmark = pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "include")) and os.path.exists(LIBREF)),
                                reason="the reference's source tree and oracle/_ref build are not here")


@pytest.fixture(scope="module")
def shim_exe(built_lib, tmp_path_factory):
    d = tmp_path_factory.mktemp("shim")
    inc = ["-I", os.path.join(REF, "include"), "-I", os.path.join(REF, "include", "physicalmodels"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "hypar_gb300", "shim")]
    defs = ["-Dserial", "-Dwith_omp"]
    obj = str(d / "gbhypar_attach.o")
    subprocess.run(["gcc", "-O2", "-std=c99", "-Wall", "-Werror", "-fopenmp"] + defs + inc +
                   ["-c", os.path.join(ROOT, "hypar_gb300", "shim", "gbhypar_attach.c"), "-o", obj],
                   check=True, capture_output=True, text=True)
    exe = str(d / "shim_config")
    libdir = os.path.join(ROOT, "hypar_gb300")
    subprocess.run(["g++", "-O2", "-std=c++11", "-fopenmp"] + defs + inc +
                   [os.path.join(ROOT, "tests", "shim_config_main.cpp"), obj, "-Wl,--start-group", LIBREF,
                    "-Wl,--end-group", "-L", libdir, "-lgbhypar", "-Wl,-rpath," + libdir, "-lm", "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def _with(case, **kw):
    for k, v in kw.items():
        setattr(case, k, v)
    return case


DECKS = {
    "vortex_char_roe_ssprk3_slipwall": lambda: _with(C.vortex(24, n_iter=2, dt=0.02),
                                                     bcs={(1, 1): ("slip-wall", [0.0, 0.25]),
                                                          (1, -1): ("slip-wall", [0.0, 0.0])}),
    "vortex_comp_llf_mapped_subsonic_io": lambda: _with(C.vortex(20, n_iter=2, dt=0.02, interp="components",
                                                                 upwinding="llf-char", scheme="44"),
                                                        weights="mapped",
                                                        bcs={(0, 1): ("subsonic-inflow", [1.0, 0.5, 0.0]),
                                                             (0, -1): ("subsonic-outflow", [1.0])}),
    "vortex_dirichlet_supersonic_yc_rk22": lambda: _with(C.vortex(16, n_iter=2, dt=0.02, scheme="22"),
                                                         weights="yc",
                                                         bcs={(0, 1): ("supersonic-inflow", [1.0, 0.5, 0.0, 1.0]),
                                                              (0, -1): ("supersonic-outflow", []),
                                                              (1, 1): ("dirichlet", [1.0, 0.5, 0.0, 2.625]),
                                                              (1, -1): ("noslip-wall", [0.0, 0.0])}),
    "tgv_comp_roe_viscous_rk4": lambda: C.tgv(12, n_iter=2, dt=0.02),
    "tgv_char_rusanov_borges_inviscid": lambda: _with(C.tgv(12, n_iter=2, dt=0.02, interp="characteristic",
                                                            upwinding="rusanov"), weights="borges", Re=None),
    "sod_comp_roe_crweno": lambda: _with(C.sod(64, n_iter=2, dt=1e-3), hyp_scheme="crweno5"),
    "sod_no_limiting_rf": lambda: _with(C.sod(48, n_iter=2, dt=1e-3, upwinding="rf-char"), weights="none"),
    "rtb_gravity_hb2": lambda: C.rising_thermal_bubble(12, n_iter=2),
    "stratified_euler1d_gravity": lambda: C.stratified_1d(32, n_iter=2, g=1.0, grav_type=0),
    "sod_slip_walls_1d": lambda: _with(C.sod(48, n_iter=2, dt=1e-3),
                                       bcs={(0, 1): ("slip-wall", [0.0]), (0, -1): ("slip-wall", [0.2])}),
    "stratified_euler1d_gravity_crweno_char": lambda: _with(C.stratified_1d(32, n_iter=2, grav_type=1,
                                                                          interp="characteristic"),
                                                          hyp_scheme="crweno5"),
    "tgv_second_order_viscous": lambda: _with(C.tgv(12, n_iter=2, dt=0.02), par_scheme="2"),
    "vortex_steger_warming_char": lambda: C.vortex(20, n_iter=2, dt=0.02, upwinding="steger-warming"),
    "sod_forward_euler": lambda: C.sod(48, n_iter=2, dt=1e-3, scheme="euler"),
    "vortex_sponges": lambda: _with(C.vortex(24, n_iter=2, dt=0.02), sponges=[
        (0, -1, [(6.0, 9.6), (-1.0, 11.0)], [1.1, 0.4, 0.05, 2.7]),
        (1, 1, [(-1.0, 11.0), (0.0, 2.5)], [0.9, 0.55, -0.05, 2.5])]),
    "tgv_thermal_walls": lambda: _with(C.tgv(12, n_iter=2, dt=0.02), bcs={
        (2, 1): ("thermal-noslip-wall", [0.0, 0.0, 0.0], ([0.0, 0.03], np.full(2 * 144, 0.7))),
        (2, -1): ("thermal-slip-wall", [0.0, 0.1, 0.0], ([0.0], np.full(144, 0.75)))}),
}


def _parse(text):
    out = {}
    for ln in text.splitlines():
        parts = ln.split()
        if parts:
            out[parts[0]] = parts[1:]
    return out


@pytest.mark.parametrize("name", list(DECKS))
def test_shim_config_matches_reader(shim_exe, tmp_path, name):
    case = DECKS[name]()
    d = str(tmp_path / "deck")
    case.write(d)
    p = subprocess.run([shim_exe], cwd=d, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    got = _parse(p.stdout)
    assert got["config_rc"] == ["0"], p.stdout + p.stderr
    want = Inputs(d).config
    ints = ["model", "ndims", "nvars", "ghosts", "interp", "upwind", "hyp_scheme", "weno_weights", "nzones",
            "rk_nstages", "n_iter", "file_op_iter", "restart_iter", "screen_op_iter", "cons_check", "par_scheme"]
    for k in ints:
        assert int(got[k][0]) == getattr(want, k), k
    assert [int(v) for v in got["dim"]] == list(want.dim)
    exact = ["gamma", "weno_eps", "Pr", "Minf", "rho_ref", "p_ref", "dt"]
    for k in exact:
        assert float(got[k][0]) == getattr(want, k), k
    if want.model == 3:
        # NavierStokes3D keeps Re / Minf; the binding multiplies back (one rounding)
        assert float(got["Re"][0]) == pytest.approx(want.Re, rel=4e-16, abs=0.0) or (want.Re <= 0
                                                                                     and float(got["Re"][0]) <= 0)
    grav = [float(v) for v in got["gravity"]]
    assert grav == list(want.gravity)
    if any(grav):
        if want.model == 3:
            assert int(got["HB"][0]) == want.HB and float(got["R_gas"][0]) == want.R_gas
            assert float(got["N_bv"][0]) == want.N_bv
        else:
            assert int(got["grav_type"][0]) == want.grav_type
    for z in range(want.nzones):
        assert [int(v) for v in got[f"zone{z}"]] == list(want.zones[z]), z
        assert [float(v) for v in got[f"zone_data{z}"]] == list(want.zone_data[z]), z
    ns = want.rk_nstages
    A = np.array([float(v) for v in got["rk_A"]]).reshape(4, 4)
    assert np.array_equal(A[:ns, :ns], np.array(list(want.rk_A)).reshape(4, 4)[:ns, :ns])
    assert [float(v) for v in got["rk_b"]][:ns] == list(want.rk_b)[:ns]
    assert [float(v) for v in got["rk_c"]][:ns] == list(want.rk_c)[:ns]
    # without a GPU the device set-up fails cleanly; with one, the solver is created
    assert int(got["attach_rc"][0]) in (_lib.GB_OK, 2), p.stdout + p.stderr
