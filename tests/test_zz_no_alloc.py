"""gb_rhs_explicit_noalloc (the right-hand side computed with the library's
static scratch instead of any device allocation) against the solver entry point
gb_RHSFunctionExplicit and against the CPU oracle, through the C ABI, on
consecutive calls.  The cases cover every branch of the entry point: Jiang-Shu
and the other weight formulations (mapped, Yamaleev-Carpenter), boundaries
folded into the halo loads (periodic, extrapolate) and boundaries filled in
memory before the kernels (slip walls, subsonic inflow / outflow).

Runs last (file name) so that it also sees a device on which the rest of the
suite has already run; it also passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest

import oracle as O
from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Inputs, Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12  # relative L2 per right-hand-side evaluation, as the parity tests


def relerr(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _with(case, **kw):
    for k, v in kw.items():
        setattr(case, k, v)
    return case


CASES = {
    "euler2d_char_roe": lambda: C.vortex(40, n_iter=2, dt=0.02),
    "euler2d_comp_llf": lambda: C.vortex(36, n_iter=2, dt=0.02, interp="components", upwinding="llf-char"),
    "ns3d_inviscid_char_rf": lambda: _with(C.tgv(14, n_iter=2, dt=0.02, interp="characteristic",
                                                 upwinding="rf-char", perturb=0.05), Re=None),
    "euler1d_comp_roe": lambda: C.sod(72, n_iter=2, dt=1e-3),
    # weight formulations other than Jiang-Shu (the *_w kernels)
    "euler2d_char_roe_mapped": lambda: _with(C.vortex(32, n_iter=2, dt=0.02), weights="mapped"),
    "euler2d_comp_roe_yc": lambda: _with(C.vortex(28, n_iter=2, dt=0.02, interp="components"), weights="yc"),
    # boundary zones filled in memory before the kernels (bc_zone_kernel)
    "euler2d_char_roe_slipwall": lambda: _with(C.vortex(32, n_iter=2, dt=0.02),
                                               bcs={(1, 1): ("slip-wall", [0.0, 0.0]),
                                                    (1, -1): ("slip-wall", [0.0, 0.0])}),
    "euler2d_comp_llf_subsonic_io": lambda: _with(C.vortex(30, n_iter=2, dt=0.02, interp="components",
                                                           upwinding="llf-char"),
                                                  bcs={(0, 1): ("subsonic-inflow", [1.0, 0.5, 0.0]),
                                                       (0, -1): ("subsonic-outflow", [1.0])}),
}


def _interior(a, s):
    g = s.ghosts
    dims = s.dims
    arr = a.reshape(tuple(d + 2 * g for d in reversed(dims)) + (s.nvars,))
    sl = tuple(slice(g, g + d) for d in reversed(dims)) + (slice(None),)
    return arr[sl]


def _noalloc(cfg, dxinv_dev, rhs, u):
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.lib().gb_rhs_explicit_noalloc(ctypes.byref(cfg), dxinv_dev.data_ptr(), rhs.data_ptr(),
                                                  u.data_ptr(), stream))
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_matches_rhs_entry_point(built_lib, tmp_path, name):
    case = CASES[name]()
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    cfg = inp.config
    assert cfg.model != 3 or cfg.Re <= 0  # inviscid: the entry point has no viscous term
    s = Solver(cfg, inp.dxinv, device=0)
    dxinv_dev = torch.from_numpy(inp.dxinv).cuda()
    # two different states: the initial solution and the one after a step
    s.set_state(inp.u0)
    states = [s.get_state(ghosted=True)]
    s.step(1)
    states.append(s.get_state(ghosted=True))
    out = [torch.full((states[0].size,), 5.0, dtype=torch.float64, device="cuda") for _ in states]
    for k, st in enumerate(states):  # two calls in a row, nothing in between
        _noalloc(cfg, dxinv_dev, out[k], torch.from_numpy(st).cuda())
    P = O.Problem(case)
    for k, st in enumerate(states):
        ref = torch.full_like(out[k], 9.0)
        s.rhs(ref, torch.from_numpy(st).cuda())
        a = _interior(out[k].cpu().numpy(), s)
        b = _interior(ref.cpu().numpy(), s)
        c = _interior(P.rhs(st.copy()), s)
        assert np.isfinite(a).all()
        assert relerr(a, b) <= RHS_TOL, (name, k, relerr(a, b))
        assert relerr(a, c) <= RHS_TOL, (name, k, "oracle", relerr(a, c))
        # ghost entries of rhs are cleared, as by the solver entry point
        ga, gb = out[k].cpu().numpy().copy(), ref.cpu().numpy().copy()
        _interior(ga, s)[...] = 0.0
        _interior(gb, s)[...] = 0.0
        assert not ga.any() and not gb.any()
    s.close()


def test_noalloc_rejects_oversized_grid(built_lib):
    cfg = _lib.GbConfig()
    cfg.model, cfg.ndims, cfg.nvars, cfg.ghosts = 2, 2, 4, 3
    cfg.dim[0] = cfg.dim[1] = 2048  # 2054^2 points x 4 values x 8 bytes > 64 MiB
    cfg.interp, cfg.upwind = 1, 0
    cfg.gamma, cfg.weno_eps = 1.4, 1e-6  # Runge-Kutta fields left zero: the entry point ignores them
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = _lib.lib().gb_rhs_explicit_noalloc(ctypes.byref(cfg), dummy.data_ptr(), dummy.data_ptr(),
                                            dummy.data_ptr(), None)
    assert rc == 1  # GB_ERR_ARG
    assert b"scratch" in _lib.lib().gb_last_error()


def test_noalloc_largest_documented_grids_fit(built_lib):
    """The header's limits: 1442^2 Euler2D and 112^3 NavierStokes3D fit in the
    scratch, one more point per dimension does not (checked before any launch)."""
    L = _lib.lib()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    for model, nd, n_fit in ((2, 2, 1442), (3, 3, 112)):
        need = lambda n: (n + 6) ** nd * (nd + 2) * 8  # noqa: E731
        assert need(n_fit) <= 64 << 20 < need(n_fit + 1)
        cfg = _lib.GbConfig()
        cfg.model, cfg.ndims, cfg.nvars, cfg.ghosts = model, nd, nd + 2, 3
        for d in range(nd):
            cfg.dim[d] = n_fit + 1
        cfg.interp, cfg.upwind, cfg.gamma, cfg.weno_eps, cfg.Re = 1, 0, 1.4, 1e-6, -1.0
        assert L.gb_rhs_explicit_noalloc(ctypes.byref(cfg), dummy.data_ptr(), dummy.data_ptr(),
                                         dummy.data_ptr(), None) == 1
