"""gb_solver_set_state / gb_solver_get_state with host buffers: pageable and pinned
host memory (the end-to-end benchmark's buffers) must give the same bits, in both
layouts."""
import numpy as np
import pytest

from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Solver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["vortex", "tgv"])
def test_pinned_and_pageable_state_io_agree(built_lib, tmp_path, name):
    case = C.vortex(48, n_iter=2, dt=0.02) if name == "vortex" else C.tgv(12, n_iter=2, dt=0.02, perturb=0.05)
    d = str(tmp_path / "deck")
    case.write(d)
    L = _lib.lib()
    a = Solver.from_dir(d, device=0)
    a.step(2)
    ref = a.get_state()  # pageable numpy buffer
    b = Solver.from_dir(d, device=0)
    pinned = torch.from_numpy(np.ascontiguousarray(case.u.reshape(-1), dtype=np.float64)).pin_memory()
    _lib.check(L.gb_solver_set_state(b._h, pinned.data_ptr(), _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))
    b.step(2)
    out = torch.full_like(pinned, np.nan).pin_memory()
    _lib.check(L.gb_solver_get_state(b._h, out.data_ptr(), _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))
    assert np.array_equal(out.numpy(), ref)
    # the ghosted layout with a pinned buffer (a plain copy)
    g = torch.empty(b.npts_wg * case.nvars, dtype=torch.float64).pin_memory()
    _lib.check(L.gb_solver_get_state(b._h, g.data_ptr(), _lib.LAYOUT_GHOSTED, _lib.MEM_HOST))
    assert np.array_equal(g.numpy(), b.get_state(ghosted=True))
