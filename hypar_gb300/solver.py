"""Python mirror of libgbhypar's C ABI.

``Solver`` wraps a gb_solver: HyPar's function-pointer surface
(``hyperbolic``, ``parabolic``, ``flux``, ``ufunc``, ``upwind``, ``apply_bc``,
``rhs``, ``time_rk``) on device arrays, and the fused fast path (``step``).
Device arrays are torch CUDA tensors (torch supplies device memory and
streams only); host arrays are numpy.  Arrays use HyPar's layout: ghost points
on every side, dimension 0 fastest, the nvars components of a point
contiguous.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GbConfig, check, lib


def _ptr(a) -> int:
    """Device or host address of a torch tensor / numpy array."""
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Inputs:
    """A HyPar input deck read by the library's C reader (gb_inputs_read)."""

    def __init__(self, directory: str):
        h = ctypes.c_void_p()
        check(lib().gb_inputs_read(directory.encode(), ctypes.byref(h)))
        self._h = h
        c = lib().gb_inputs_config(h).contents
        self.config = GbConfig()
        ctypes.pointer(self.config)[0] = c
        nd = c.ndims
        dims = [c.dim[d] for d in range(nd)]
        nx = sum(dims)
        nxg = sum(d + 2 * c.ghosts for d in dims)
        npts = int(np.prod(dims))
        self.x = np.ctypeslib.as_array(lib().gb_inputs_x(h), shape=(nx,)).copy()
        self.dxinv = np.ctypeslib.as_array(lib().gb_inputs_dxinv(h), shape=(nxg,)).copy()
        self.u0 = np.ctypeslib.as_array(lib().gb_inputs_u0(h), shape=(npts * c.nvars,)).copy()
        npts_wg = int(np.prod([d + 2 * c.ghosts for d in dims]))
        gp = lib().gb_inputs_gravity_field(h)
        # hydrostatic density and pressure fields f, g with ghost points (NavierStokes3D gravity)
        self.gravity_field = np.ctypeslib.as_array(gp, shape=(2 * npts_wg,)).copy() if gp else None
        # thermal walls: per zone (times, field) of the wall temperature
        self.zone_temperature = {}
        for z in range(c.nzones):
            n, tp, fp = ctypes.c_int(), _lib.DP(), _lib.DP()
            check(lib().gb_inputs_zone_temperature(h, z, ctypes.byref(n), ctypes.byref(tp), ctypes.byref(fp)))
            if n.value:
                q = c.zones[z]
                size = n.value
                for d in range(nd):
                    if d != q[1]:
                        size *= q[6 + d] - q[3 + d]
                self.zone_temperature[z] = (np.ctypeslib.as_array(tp, shape=(n.value,)).copy(),
                                            np.ctypeslib.as_array(fp, shape=(size,)).copy())
        # sponge zones: per zone sigma along the zone's dimension
        self.zone_sponge = {}
        for z in range(c.nzones):
            n, sp = ctypes.c_int(), _lib.DP()
            check(lib().gb_inputs_zone_sponge(h, z, ctypes.byref(n), ctypes.byref(sp)))
            if n.value:
                self.zone_sponge[z] = np.ctypeslib.as_array(sp, shape=(n.value,)).copy()
        # turbulent inflow zones: per zone (slices, data), nvars values per point
        self.zone_inflow = {}
        for z in range(c.nzones):
            n, dp = ctypes.c_int(), _lib.DP()
            check(lib().gb_inputs_zone_inflow(h, z, ctypes.byref(n), ctypes.byref(dp)))
            if n.value:
                cnt = n.value * c.nvars
                for d in range(nd):
                    if d != c.zones[z][1]:
                        cnt *= dims[d]
                self.zone_inflow[z] = (n.value, np.ctypeslib.as_array(dp, shape=(cnt,)).copy())
        lib().gb_inputs_free(h)
        self._h = None


def rk_table(name: str):
    ns = ctypes.c_int()
    A = (ctypes.c_double * 16)()
    b = (ctypes.c_double * 4)()
    c = (ctypes.c_double * 4)()
    check(lib().gb_rk_table(name.encode(), ctypes.byref(ns), A, b, c))
    return ns.value, list(A), list(b), list(c)


class Solver:
    def __init__(self, config: GbConfig, dxinv: np.ndarray, device: int = 0):
        self.config = config
        self.dxinv = np.ascontiguousarray(dxinv, dtype=np.float64)
        h = ctypes.c_void_p()
        check(lib().gb_solver_create(ctypes.byref(config), self.dxinv.ctypes.data_as(_lib.DP), device,
                                     ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_dir(cls, directory: str, device: int = 0) -> "Solver":
        inp = Inputs(directory)
        s = cls(inp.config, inp.dxinv, device)
        s.inputs = inp
        s.set_state(inp.u0)
        if inp.gravity_field is not None:
            s.set_gravity_field(inp.gravity_field)
        for z, (times, field) in inp.zone_temperature.items():
            s.set_zone_temperature(z, times, field)
        for z, sigma in inp.zone_sponge.items():
            s.set_zone_sponge(z, sigma)
        for z, (n, data) in inp.zone_inflow.items():
            s.set_zone_inflow(z, n, data)
        return s

    def set_zone_temperature(self, zone: int, times, field):
        """A thermal wall's temperature: time levels and the field over the zone's extent
        (the level along the zone's own dimension, dimension 0 fastest)."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        field = np.ascontiguousarray(field, dtype=np.float64).reshape(-1)
        check(lib().gb_solver_set_zone_temperature(self._h, int(zone), len(times), times.ctypes.data_as(_lib.DP),
                                                   field.ctypes.data_as(_lib.DP)))

    def set_zone_inflow(self, zone: int, n: int, data):
        """A turbulent inflow's data: n slices along the zone's dimension, the grid across,
        nvars values per point, dimension 0 fastest."""
        data = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
        check(lib().gb_solver_set_zone_inflow(self._h, int(zone), int(n), data.ctypes.data_as(_lib.DP)))

    def set_zone_sponge(self, zone: int, sigma):
        """A sponge zone's sigma, one value per index of the zone along its dimension."""
        sigma = np.ascontiguousarray(sigma, dtype=np.float64)
        check(lib().gb_solver_set_zone_sponge(self._h, int(zone), sigma.ctypes.data_as(_lib.DP)))

    def set_gravity_field(self, fg: np.ndarray):
        """Upload the hydrostatic fields f then g (ghosted layout, x fastest) that the
        well-balanced NavierStokes3D gravity formulation scales the state and the
        source with (NavierStokes3DGravityField.c:36-153)."""
        fg = np.ascontiguousarray(fg, dtype=np.float64)
        check(lib().gb_solver_set_gravity_field(self._h, fg.ctypes.data_as(_lib.DP)))

    def close(self):
        if getattr(self, "_h", None):
            lib().gb_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> int:
        return self._h.value

    @property
    def ndims(self) -> int:
        return self.config.ndims

    @property
    def nvars(self) -> int:
        return self.config.nvars

    @property
    def dims(self):
        return [self.config.dim[d] for d in range(self.config.ndims)]

    @property
    def ghosts(self) -> int:
        return self.config.ghosts

    @property
    def npts_wg(self) -> int:
        return int(np.prod([d + 2 * self.ghosts for d in self.dims]))

    @property
    def npts(self) -> int:
        return int(np.prod(self.dims))

    # ---- fused fast path ----
    def set_state(self, u, ghosted: bool = False):
        layout = _lib.LAYOUT_GHOSTED if ghosted else _lib.LAYOUT_INTERIOR
        if hasattr(u, "is_cuda") and u.is_cuda:
            import torch
            torch.cuda.synchronize()
            check(lib().gb_solver_set_state(self._h, _ptr(u), layout, _lib.MEM_DEVICE))
        else:
            arr = np.ascontiguousarray(u, dtype=np.float64)
            check(lib().gb_solver_set_state(self._h, arr.ctypes.data, layout, _lib.MEM_HOST))
            self.sync()

    def get_state(self, ghosted: bool = False) -> np.ndarray:
        n = (self.npts_wg if ghosted else self.npts) * self.nvars
        out = np.empty(n, dtype=np.float64)
        check(lib().gb_solver_get_state(self._h, out.ctypes.data,
                                        _lib.LAYOUT_GHOSTED if ghosted else _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))
        return out

    def step(self, nsteps: int = 1):
        check(lib().gb_solver_step(self._h, int(nsteps)))

    def sync(self):
        check(lib().gb_solver_sync(self._h))

    def set_stream(self, stream_handle: Optional[int]):
        check(lib().gb_solver_set_stream(self._h, stream_handle))

    def set_launch(self, dim: int, seg: int = 0, block: int = 0):
        check(lib().gb_solver_set_launch(self._h, dim, seg, block))

    def get_launch(self, dim: int):
        seg, blk = ctypes.c_int(), ctypes.c_int()
        check(lib().gb_solver_get_launch(self._h, dim, ctypes.byref(seg), ctypes.byref(blk)))
        return seg.value, blk.value

    def autotune(self, reps: int = 2):
        """Pick the launch shape per direction by timing (state restored)."""
        check(lib().gb_solver_autotune(self._h, int(reps)))
        return [self.get_launch(d) for d in range(self.ndims)]

    @property
    def time(self) -> float:
        return lib().gb_solver_time(self._h)

    def state_ptr(self) -> int:
        return lib().gb_solver_state(self._h)

    PROF_CLASSES = ("hyp_x", "hyp_y", "hyp_z", "viscous", "bc")

    def profile(self, enable: bool = True):
        check(lib().gb_solver_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        """{class: (milliseconds, launches)} accumulated since profiling was enabled."""
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_longlong * 5)()
        check(lib().gb_solver_profile_read(self._h, ms, n))
        return {k: (ms[i], n[i]) for i, k in enumerate(self.PROF_CLASSES)}

    def set_time(self, t: float):
        check(lib().gb_solver_set_time(self._h, float(t)))

    def cfl(self) -> float:
        """Maximum CFL of the resident solution for the configured dt (device reduction)."""
        c = ctypes.c_double()
        check(lib().gb_solver_cfl(self._h, ctypes.byref(c)))
        return c.value

    def step_report(self, nsteps: int = 1):
        """Advance nsteps steps; (CFL of the state the last step starts from, norm of its change)."""
        c, n = ctypes.c_double(), ctypes.c_double()
        check(lib().gb_solver_step_report(self._h, nsteps, ctypes.byref(c), ctypes.byref(n)))
        return c.value, n.value

    def error(self, uex, ghosted: bool = False):
        """(L1, L2, Linf) errors against an exact solution (host numpy array or device tensor)."""
        err = (ctypes.c_double * 3)()
        mem = _lib.MEM_DEVICE if hasattr(uex, "data_ptr") else _lib.MEM_HOST
        if mem == _lib.MEM_HOST:
            uex = np.ascontiguousarray(uex, dtype=np.float64)
        layout = _lib.LAYOUT_GHOSTED if ghosted else _lib.LAYOUT_INTERIOR
        check(lib().gb_solver_error(self._h, _ptr(uex), layout, mem, err))
        return tuple(err)

    def conservation_begin(self):
        """Start the conservation check from the current state (volume integral V0,
        boundary-flux integrals cleared)."""
        check(lib().gb_solver_conservation_begin(self._h))

    def conservation_error(self) -> np.ndarray:
        """|V + B - V0| / max(|V0|, 1) per variable (CalculateConservationError)."""
        err = (ctypes.c_double * self.config.nvars)()
        check(lib().gb_solver_conservation_error(self._h, err))
        return np.array(err[:])

    def check_finite(self) -> bool:
        f = ctypes.c_int()
        check(lib().gb_solver_check_finite(self._h, ctypes.byref(f)))
        return bool(f.value)

    # ---- HyPar function-pointer surface (device tensors) ----
    def _dev(self):
        import torch
        torch.cuda.synchronize()

    def hyperbolic(self, hyp, u, t: float = 0.0):
        self._dev()
        F = _lib.fn_address("gb_FFunction")
        U = _lib.fn_address("gb_Upwind")
        check(lib().gb_HyperbolicFunction(_ptr(hyp), _ptr(u), self._h, None, t, 1, F, U))
        self.sync()

    def parabolic(self, par, u, t: float = 0.0):
        self._dev()
        check(lib().gb_ParabolicFunction(_ptr(par), _ptr(u), self._h, None, t))
        self.sync()

    def source(self, src, u, t: float = 0.0):
        self._dev()
        check(lib().gb_SourceFunction(_ptr(src), _ptr(u), self._h, None, t))
        self.sync()

    def flux(self, f, u, dim: int, t: float = 0.0):
        self._dev()
        check(lib().gb_FFunction(_ptr(f), _ptr(u), dim, self._h, t))
        self.sync()

    def gflux(self, f, u, dim: int, t: float = 0.0):
        self._dev()
        check(lib().gb_GFunction(_ptr(f), _ptr(u), dim, self._h, t))
        self.sync()

    def ufunc(self, uC, u, dim: int = 0, t: float = 0.0):
        self._dev()
        check(lib().gb_UFunction(_ptr(uC), _ptr(u), dim, self._h, None, t))
        self.sync()

    def upwind(self, fI, fL, fR, uL, uR, u, dim: int, t: float = 0.0):
        self._dev()
        check(lib().gb_Upwind(_ptr(fI), _ptr(fL), _ptr(fR), _ptr(uL), _ptr(uR), _ptr(u), dim, self._h, t))
        self.sync()

    def set_interp_limiter_var(self, fC, u, dim: int):
        self._dev()
        check(lib().gb_SetInterpLimiterVar(_ptr(fC), _ptr(u), None, dim, self._h, None))

    def interpolate(self, fI, fC, u, upw: int, dim: int, uflag: int):
        """InterpolateInterfacesHyp: WENO5 interface values of fC along dim (upw > 0
        left-biased, < 0 right-biased; weights of fC for uflag 0, of u for uflag 1)."""
        self._dev()
        check(lib().gb_InterpolateInterfacesHyp(_ptr(fI), _ptr(fC), _ptr(u), None, int(upw), dim, self._h, None,
                                                int(uflag)))
        self.sync()

    def apply_bc(self, u, t: float = 0.0):
        self._dev()
        check(lib().gb_ApplyBoundaryConditions(self._h, None, _ptr(u), None, t))
        self.sync()

    def rhs(self, out, u, t: float = 0.0):
        self._dev()
        check(lib().gb_RHSFunctionExplicit(_ptr(out), _ptr(u), self._h, None, t))
        self.sync()

    def time_rk(self):
        check(lib().gb_TimeRK(self._h))


def run_case(directory: str, device: int = 0, verbose: bool = False) -> None:
    """gb_run_case: the HyPar driver for one deck directory (writes op*.bin)."""
    check(lib().gb_run_case(directory.encode(), device, 1 if verbose else 0))


def read_op(path: str):
    from .cases import read_op_bin
    return read_op_bin(path)


class Ensemble:
    """gb_ensemble: members of one HyPar ensemble deck advanced together."""

    def __init__(self, configs, dxinvs, device: int = 0):
        n = len(configs)
        self.configs = list(configs)
        arr = (GbConfig * n)(*configs)
        self._dx = [np.ascontiguousarray(d, dtype=np.float64) for d in dxinvs]
        ptrs = (_lib.DP * n)(*[d.ctypes.data_as(_lib.DP) for d in self._dx])
        h = ctypes.c_void_p()
        check(lib().gb_ensemble_create(arr, ptrs, n, device, ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_dir(cls, directory: str, device: int = 0) -> "Ensemble":
        n = lib().gb_inputs_nsims(directory.encode())
        if n < 1:
            raise _lib.GbError(3, "simulation.inp is malformed")
        inputs = []
        for m in range(n):
            h = ctypes.c_void_p()
            check(lib().gb_inputs_read_member(directory.encode(), m, n, ctypes.byref(h)))
            c = lib().gb_inputs_config(h).contents
            cfg = GbConfig()
            ctypes.pointer(cfg)[0] = c
            dims = [c.dim[d] for d in range(c.ndims)]
            nxg = sum(d + 2 * c.ghosts for d in dims)
            npts = int(np.prod(dims))
            dx = np.ctypeslib.as_array(lib().gb_inputs_dxinv(h), shape=(nxg,)).copy()
            u0 = np.ctypeslib.as_array(lib().gb_inputs_u0(h), shape=(npts * c.nvars,)).copy()
            lib().gb_inputs_free(h)
            inputs.append((cfg, dx, u0))
        e = cls([i[0] for i in inputs], [i[1] for i in inputs], device)
        for m, (_, _, u0) in enumerate(inputs):
            e.set_state(m, u0)
        return e

    def __len__(self):
        return lib().gb_ensemble_size(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().gb_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, m: int, u):
        arr = np.ascontiguousarray(u, dtype=np.float64)
        check(lib().gb_ensemble_set_state(self._h, m, arr.ctypes.data, _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))

    def get_state(self, m: int) -> np.ndarray:
        c = self.configs[m]
        n = int(np.prod([c.dim[d] for d in range(c.ndims)])) * c.nvars
        out = np.empty(n, dtype=np.float64)
        check(lib().gb_ensemble_get_state(self._h, m, out.ctypes.data, _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))
        return out

    def step(self, nsteps: int = 1):
        check(lib().gb_ensemble_step(self._h, int(nsteps)))

    def sync(self):
        check(lib().gb_ensemble_sync(self._h))

    def set_stream(self, stream_handle):
        check(lib().gb_ensemble_set_stream(self._h, stream_handle))

    def set_launch(self, dim: int, seg: int = 0, block: int = 0):
        check(lib().gb_ensemble_set_launch(self._h, dim, seg, block))

    def get_launch(self, dim: int):
        seg, blk = ctypes.c_int(), ctypes.c_int()
        check(lib().gb_ensemble_get_launch(self._h, dim, ctypes.byref(seg), ctypes.byref(blk)))
        return seg.value, blk.value

    def autotune(self, reps: int = 2):
        check(lib().gb_ensemble_autotune(self._h, int(reps)))
        return [self.get_launch(d) for d in range(self.configs[0].ndims)]

    def conservation_begin(self):
        check(lib().gb_ensemble_conservation_begin(self._h))

    def conservation_error(self, m: int) -> np.ndarray:
        err = (ctypes.c_double * self.configs[m].nvars)()
        check(lib().gb_ensemble_conservation_error(self._h, int(m), err))
        return np.array(err[:])

    @property
    def time(self) -> float:
        return lib().gb_ensemble_time(self._h)
