"""HyPar's stage and step hooks (include/hypar.h:334-341) on the fused step.

gb_solver_set_hooks installs PreStep / PostStage / PostStep; the fused step calls
them as the reference's TimePreStep, TimeRK and TimePostStep do: PreStep(u, t)
before the step, PostStage(U_s, t + c_s dt) on every stage state before its
right-hand side (a copy where the stage's state is u itself), PostStep(u, t + dt,
iter) after it.  A PostStage hook that changes the stage state changes the step
exactly as TimeRK's Butcher form says: checked against the same form evaluated
with the library's own right-hand side (gb_RHSFunctionExplicit)."""
import ctypes
import glob
import os

import numpy as np
import pytest

from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Inputs, Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime (to read and write device memory from a hook)."""
    names = ["libcudart.so.13", "libcudart.so.12", "libcudart.so"]
    tl = os.path.join(os.path.dirname(torch.__file__), "lib")
    names += sorted(glob.glob(os.path.join(tl, "libcudart*.so*")))
    import site
    for sp in site.getsitepackages():
        names += sorted(glob.glob(os.path.join(sp, "nvidia", "cu*", "lib", "libcudart.so*")))
        names += sorted(glob.glob(os.path.join(sp, "nvidia", "cuda_runtime", "lib", "libcudart.so*")))
    names += ["/usr/local/cuda/lib64/libcudart.so"]
    for n in names:
        try:
            L = ctypes.CDLL(n)
        except OSError:
            continue
        L.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        return L
    pytest.skip("no CUDA runtime library to read device memory from a hook")


def _solver(tmp_path, scheme="ssprk3"):
    case = C.vortex(24, n_iter=3, dt=0.02, scheme=scheme)
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    s = Solver(inp.config, inp.dxinv, device=0)
    s.set_state(inp.u0)
    return s, inp


def test_hooks_called_in_reference_order(built_lib, tmp_path):
    s, inp = _solver(tmp_path, "44")
    cfg = inp.config
    L = _lib.lib()
    calls = []
    state_ptr = L.gb_solver_state(s._h)

    def pre_step(u, solver, mpi, t):
        calls.append(("pre", t, u == L.gb_solver_state(s._h), solver, mpi))
        return 0

    def post_stage(U, solver, mpi, t):
        calls.append(("stage", t, U == L.gb_solver_state(s._h), solver, mpi))
        return 0

    def post_step(u, solver, mpi, t, it):
        calls.append(("post", t, it, solver, mpi))
        return 0

    hooks = (_lib.PRESTAGE(), _lib.POSTSTAGE(post_stage), _lib.PRESTEP(pre_step), _lib.POSTSTEP(post_step))
    _lib.check(L.gb_solver_set_hooks(s._h, *hooks, 1234, 5678))
    s.autotune(1)  # trial steps call no hook
    assert calls == []
    s.step(2)
    s.sync()
    dt = cfg.dt
    cs = [cfg.rk_c[k] for k in range(cfg.rk_nstages)]
    want = []
    for n in range(2):
        t = n * dt
        want.append(("pre", t))
        want += [("stage", t + c * dt) for c in cs]
        want.append(("post", t + dt))
    assert [(c[0], pytest.approx(c[1], abs=1e-15)) for c in calls] == want
    assert all(c[-2:] == (1234, 5678) for c in calls)
    # PreStep sees the solution itself; PostStage never does (stage 0 gets a copy)
    assert all(c[2] for c in calls if c[0] == "pre")
    assert not any(c[2] for c in calls if c[0] == "stage")
    assert [c[2] for c in calls if c[0] == "post"] == [0, 1]
    assert state_ptr  # the solution array exists throughout
    # a PreStage hook is refused, as the reference's TimeRK refuses it
    prestage = _lib.PRESTAGE(lambda *a: 0)
    assert L.gb_solver_set_hooks(s._h, prestage, _lib.POSTSTAGE(), _lib.PRESTEP(), _lib.POSTSTEP(), None,
                                 None) == 4
    # a failing hook stops the step with GB_ERR_HOOK
    fail = _lib.POSTSTEP(lambda *a: 3)
    _lib.check(L.gb_solver_set_hooks(s._h, _lib.PRESTAGE(), _lib.POSTSTAGE(), _lib.PRESTEP(), fail, None, None))
    assert L.gb_solver_step(s._h, 1) == 7
    s.close()


@pytest.mark.parametrize("scheme", ["ssprk3", "44"])
def test_poststage_modifies_stage_state(built_lib, tmp_path, scheme):
    """PostStage scales every stage state's density by 1 + 1e-3: the step must equal
    TimeRK's Butcher form with that change, U_s = u + dt sum_i A_si k_i, then
    PostStage(U_s), k_s = rhs(U_s), u_new = u + dt sum_s b_s k_s."""
    rt = _cudart()
    s, inp = _solver(tmp_path, scheme)
    cfg = inp.config
    L = _lib.lib()
    nvals = s.npts_wg * s.nvars
    buf = np.empty(nvals)

    def post_stage(U, solver, mpi, t):
        assert rt.cudaMemcpy(buf.ctypes.data, U, nvals * 8, 2) == 0
        buf.reshape(-1, 4)[:, 0] *= 1.0 + 1e-3
        assert rt.cudaMemcpy(U, buf.ctypes.data, nvals * 8, 1) == 0
        return 0

    hook = _lib.POSTSTAGE(post_stage)
    u0 = s.get_state(ghosted=True)
    _lib.check(L.gb_solver_set_hooks(s._h, _lib.PRESTAGE(), hook, _lib.PRESTEP(), _lib.POSTSTEP(), None, None))
    s.step(1)
    got = s.get_state(ghosted=True)
    # the Butcher form with the library's right-hand side (no hooks on that path)
    ref_s, _ = _solver(tmp_path / "r", scheme)
    ns, dt = cfg.rk_nstages, cfg.dt
    u = torch.from_numpy(u0).cuda()
    ks = []
    for st in range(ns):
        U = u.clone()
        for i in range(st):
            U += dt * cfg.rk_A[4 * st + i] * ks[i]
        U.view(-1, 4)[:, 0] *= 1.0 + 1e-3
        k = torch.zeros_like(U)
        ref_s.rhs(k, U, t=cfg.rk_c[st] * dt)
        ks.append(k)
    unew = u.clone()
    for st in range(ns):
        unew += dt * cfg.rk_b[st] * ks[st]
    want = unew.cpu().numpy()
    g = s.ghosts
    n = s.dims[0]
    inner = lambda a: a.reshape(n + 2 * g, n + 2 * g, 4)[g:g + n, g:g + n]  # noqa: E731
    err = np.linalg.norm(inner(got) - inner(want)) / np.linalg.norm(inner(want))
    assert err <= 1e-13, err
    # and it differs from the step without the hook by far more than rounding
    plain_s, _ = _solver(tmp_path / "p", scheme)
    plain_s.step(1)
    plain = plain_s.get_state(ghosted=True)
    assert np.linalg.norm(inner(plain) - inner(want)) / np.linalg.norm(inner(want)) > 1e-6
    for x in (s, ref_s, plain_s):
        x.close()
