"""Turbulent supersonic inflow (BCTurbulentSupersonicInflow.c), reflect (BCReflect.c)
and 1-D slip-wall (BCSlipWall.c) boundaries.

CPU: the reader's inflow data and slice count against the file the deck wrote, the zone
codes, the validation of a turbulent inflow whose transverse extent leaves the grid.
GPU: ghost points bit-identical to the oracle's at times that select different slices
(including the wrap-around past the last one) and for reflect zones in every model;
a time at which the slice index would be negative is refused."""
import numpy as np
import pytest

import oracle as O
from hypar_gb300 import _lib
from hypar_gb300 import cases as C
from hypar_gb300.solver import Inputs, Solver

GB_ERR_ARG, GB_BC_TURBULENT_INFLOW, GB_BC_REFLECT = 1, 14, 15


def turbulent(dim=0, nslices=16, speed=2.0, seed=5, face=1):
    case = C.tgv(10, n_iter=2, dt=0.02, perturb=0.05)
    rng = np.random.default_rng(seed)
    size = [nslices if e == dim else case.size[e] for e in range(3)]
    data = rng.standard_normal((size[2], size[1], size[0], case.nvars))
    data[..., 1:4] *= 0.05
    vel = [0.0, 0.0, 0.0]
    vel[dim] = speed
    case.bcs = {(dim, face): ("turbulent-supersonic-inflow", [1.0] + vel + [1.0 / 1.4], (nslices, data.reshape(-1))),
                (dim, -face): ("supersonic-outflow", [])}
    return case


def reflect(model):
    if model == "euler1d":
        case = C.sod(40, n_iter=1, dt=1e-3)
    elif model == "euler2d":
        case = C.vortex(16, n_iter=1, dt=0.02)
    else:
        case = C.tgv(8, n_iter=1, dt=0.02, perturb=0.05)
    case.bcs = {(0, 1): ("reflect", []), (0, -1): ("reflect", [])}
    return case


@pytest.mark.parametrize("dim", [0, 1, 2])
def test_reader_inflow_data(built_lib, tmp_path, dim):
    case = turbulent(dim=dim, nslices=7)
    d = str(tmp_path / "deck")
    case.write(d)
    inp = Inputs(d)
    z = 2 * dim
    assert inp.config.zones[z][0] == GB_BC_TURBULENT_INFLOW
    assert list(inp.config.zone_data[z])[:5] == case.bcs[(dim, 1)][1]
    n, data = inp.zone_inflow[z]
    assert n == 7
    assert np.array_equal(data, case.bcs[(dim, 1)][2][1])
    assert set(inp.zone_inflow) == {z}


def test_reader_reflect_and_turbulent_limits(built_lib, tmp_path):
    case = reflect("euler1d")
    d = str(tmp_path / "a")
    case.write(d)
    assert [Inputs(d).config.zones[z][0] for z in range(2)] == [GB_BC_REFLECT, GB_BC_REFLECT]
    # a turbulent inflow's data spans the grid across its dimension: an extent beyond it
    # is refused before any device work
    case = turbulent(dim=0)
    d = str(tmp_path / "b")
    case.write(d)
    inp = Inputs(d)
    cfg = inp.config
    cfg.zones[0][7] = cfg.dim[1] + 2
    with pytest.raises(_lib.GbError) as e:
        Solver(cfg, inp.dxinv, 0)
    assert e.value.code == GB_ERR_ARG
    # Euler2D has no turbulent inflow (the reference's branch is 3-D only)
    v = C.vortex(12, n_iter=1, dt=0.01)
    v.bcs = {(0, 1): ("supersonic-outflow", [])}
    d = str(tmp_path / "c")
    v.write(d)
    t = open(d + "/boundary.inp").read().replace("supersonic-outflow 0 1", "turbulent-supersonic-inflow 0 1")
    lines = t.splitlines()
    lines[1] += " 1.0 2.0 0.0 0.7 inflow.bin"
    open(d + "/boundary.inp", "w").write("\n".join(lines) + "\n")
    with pytest.raises(_lib.GbError) as e:
        Inputs(d)
    assert e.value.code == 4


def _ghost_parity(case, tmp_path, times):
    torch = pytest.importorskip("torch")
    d = str(tmp_path / "deck")
    case.write(d)
    s = Solver.from_dir(d, device=0)
    P = O.Problem(case)
    rng = np.random.default_rng(3)
    u0 = P.u0() * (1.0 + 0.01 * rng.standard_normal(P.npts_wg * case.nvars))
    for t in times:
        u = torch.from_numpy(u0.copy()).cuda()
        s.apply_bc(u, t)
        ref = P.apply_bc(u0.copy(), t)
        assert np.array_equal(u.cpu().numpy(), ref), t
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [0, 1, 2])
def test_turbulent_inflow_ghosts_bit_exact(built_lib, oracle_lib, tmp_path, dim):
    # slice int(2 t / (2 pi) * 16) mod 16: 0 at t = 0, 5 at t = 1.0, 0 again and 3 past
    # the period (t = 2 pi + 0.6)
    case = turbulent(dim=dim)
    _ghost_parity(case, tmp_path, [0.0, 0.1, 1.0, 2 * np.pi + 0.01, 2 * np.pi + 0.6])


@pytest.mark.gpu
def test_turbulent_inflow_against_the_flow_refused(built_lib, tmp_path):
    """A mean velocity against the zone's dimension gives a negative slice index after
    t = 0, where the reference reads outside its data: the step is refused."""
    pytest.importorskip("torch")
    case = turbulent(dim=0, speed=-2.0, face=-1)
    d = str(tmp_path / "deck")
    case.write(d)
    s = Solver.from_dir(d, device=0)
    s.set_time(0.5)
    with pytest.raises(_lib.GbError) as e:
        s.step(1)
    assert e.value.code == GB_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["euler1d", "euler2d", "navierstokes3d"])
def test_reflect_ghosts_bit_exact(built_lib, oracle_lib, tmp_path, model):
    _ghost_parity(reflect(model), tmp_path, [0.0])


@pytest.mark.gpu
def test_euler1d_slip_wall_ghosts_bit_exact(built_lib, oracle_lib, tmp_path):
    """BCSlipWall.c's 1-D branch: density and pressure extrapolated, the velocity
    mirrored about the wall's (a moving wall on one face)."""
    case = C.sod(40, n_iter=1, dt=1e-3)
    rng = np.random.default_rng(2)
    case.u[:, 1] = 0.3 * rng.standard_normal(40) * case.u[:, 0]
    case.bcs = {(0, 1): ("slip-wall", [0.0]), (0, -1): ("slip-wall", [0.25])}
    _ghost_parity(case, tmp_path, [0.0])
