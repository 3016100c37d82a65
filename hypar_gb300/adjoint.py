"""Discrete adjoint and tangent-linear model of the Euler2D right-hand side
(component-wise WENO5 + Roe) and of n Runge-Kutta steps, over libgbhypar's
gb_adjoint_* C ABI, with torch.autograd.Function front ends.

Device arrays are torch CUDA tensors in HyPar's ghosted layout (flat, ghost
points on every side, dimension 0 fastest, 4 components per point contiguous);
``ghosted`` / ``interior`` convert from / to (ny, nx, 4) interior views with
torch indexing, so they take part in autograd.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from ._lib import GbConfig, check, lib


def _p(t) -> int:
    return t.data_ptr()


class Adjoint:
    """gb_adjoint: forward sweep with checkpoints, backward sweep, tangent-linear
    model, and the right-hand side's VJP / JVP."""

    def __init__(self, config: GbConfig, dxinv: np.ndarray, nsteps: int, ncheck: int = 0, device: int = 0,
                 wide_tape_max: int = -1):
        """wide_tape_max: bytes allowed for the 72-double interface tapes (< 0: 60 % of
        the free device memory; 0: always the 8-double tape)."""
        import torch
        self.config = config
        self.nsteps = nsteps
        self._dxinv = np.ascontiguousarray(dxinv, dtype=np.float64)
        h = ctypes.c_void_p()
        check(lib().gb_adjoint_create_ex(ctypes.byref(config), self._dxinv.ctypes.data_as(_lib.DP), nsteps, ncheck,
                                         device, int(wide_tape_max), ctypes.byref(h)))
        self._h = h
        self.dxinv_dev = torch.from_numpy(self._dxinv).to(f"cuda:{device}")
        g = config.ghosts
        self.dims = [config.dim[0], config.dim[1]]
        self.ghosts = g
        self.npts_wg = (self.dims[0] + 2 * g) * (self.dims[1] + 2 * g)
        self.nvals = self.npts_wg * 4

    @classmethod
    def from_case(cls, case, directory: str, nsteps: Optional[int] = None, ncheck: int = 0,
                  device: int = 0) -> "Adjoint":
        from .solver import Inputs
        case.write(directory)
        inp = Inputs(directory)
        return cls(inp.config, inp.dxinv, nsteps if nsteps is not None else case.n_iter, ncheck, device)

    def close(self):
        if getattr(self, "_h", None):
            lib().gb_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- layout helpers (torch, differentiable) ----
    def empty(self):
        import torch
        return torch.zeros(self.nvals, dtype=torch.float64, device=self.dxinv_dev.device)

    def ghosted(self, u_int):
        """(ny, nx, 4) or (npts, 4) interior -> flat ghosted tensor (ghosts zero)."""
        import torch
        g, (nx, ny) = self.ghosts, self.dims
        out = torch.zeros((ny + 2 * g, nx + 2 * g, 4), dtype=torch.float64, device=self.dxinv_dev.device)
        out = out.index_put((torch.arange(g, g + ny, device=out.device)[:, None],
                             torch.arange(g, g + nx, device=out.device)[None, :]),
                            u_int.reshape(ny, nx, 4))
        return out.reshape(-1)

    def interior(self, u_flat):
        """flat ghosted -> (ny, nx, 4) interior view."""
        g, (nx, ny) = self.ghosts, self.dims
        return u_flat.reshape(ny + 2 * g, nx + 2 * g, 4)[g:g + ny, g:g + nx, :]

    # ---- C ABI ----
    def sync(self):
        check(lib().gb_adjoint_sync(self._h))

    def set_stream(self, stream_handle):
        check(lib().gb_adjoint_set_stream(self._h, stream_handle))

    def set_launch(self, which: int, seg: int = 0, block: int = 0):
        check(lib().gb_adjoint_set_launch(self._h, which, seg, block))

    def get_launch(self, which: int):
        s, b = ctypes.c_int(), ctypes.c_int()
        check(lib().gb_adjoint_get_launch(self._h, which, ctypes.byref(s), ctypes.byref(b)))
        return s.value, b.value

    def info(self):
        L, n, r, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().gb_adjoint_info(self._h, ctypes.byref(L), ctypes.byref(n), ctypes.byref(r), ctypes.byref(b)))
        return {"segment_len": L.value, "segments": n.value, "recomputed_steps": r.value, "bytes": b.value}

    def autotune(self, u, reps: int = 3, candidates=(2, 3, 4, 6, 8, 12, 16, 24, 32), blocks=(32, 64, 128),
                 tiles=(32, 64)):
        """Choose the adjoint kernel's launch shape by timing right-hand-side
        VJPs of the state u: the block size (both directions share the launch),
        then the segment length per direction (one at a time, the other held),
        twice over, then the tile form.  Returns [seg_x, seg_y, block] (seg -t:
        tiles of t interfaces)."""
        import torch
        kb, ub = self.empty(), self.empty()
        kb.normal_()
        stream = torch.cuda.current_stream()

        def timed():
            self.rhs_vjp(u, kb, ub)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                check(lib().gb_adjoint_rhs_vjp(self._h, _p(u), _p(kb), _p(ub)))
            b.record(stream)
            self.sync()
            torch.cuda.synchronize()
            return a.elapsed_time(b)

        for _ in range(2):
            best = min((timed_with(self, 2, None, blk, timed), blk) for blk in blocks)
            self.set_launch(2, 0, best[1])
            for which in (2, 3):
                best = min((timed_with(self, which, seg, None, timed), seg) for seg in candidates)
                self.set_launch(which, best[1])
        # the tile form (one interface per thread, tiles of 32 or 64 interfaces) in both directions
        walker = [self.get_launch(2)[0], self.get_launch(3)[0]]
        t_best = timed()
        for tile in tiles:
            self.set_launch(2, -tile)
            self.set_launch(3, -tile)
            t = timed()
            if t < t_best:
                t_best, walker = t, [-tile, -tile]
        self.set_launch(2, walker[0])
        self.set_launch(3, walker[1])
        return [self.get_launch(2)[0], self.get_launch(3)[0], self.get_launch(2)[1]]

    def _pre(self):
        import torch
        torch.cuda.synchronize()

    def rhs_vjp(self, u, kbar, ubar):
        self._pre()
        check(lib().gb_adjoint_rhs_vjp(self._h, _p(u), _p(kbar), _p(ubar)))
        self.sync()

    def rhs_jvp(self, u, du, k, dk):
        self._pre()
        check(lib().gb_adjoint_rhs_jvp(self._h, _p(u), _p(du), _p(k), _p(dk)))
        self.sync()

    def forward(self, u0, uT):
        self._pre()
        check(lib().gb_adjoint_forward(self._h, _p(u0), _p(uT)))
        self.sync()

    def backward(self, ubarT, ubar0):
        self._pre()
        check(lib().gb_adjoint_backward(self._h, _p(ubarT), _p(ubar0)))
        self.sync()

    def tlm(self, u0, du0, uT, duT):
        self._pre()
        check(lib().gb_adjoint_tlm(self._h, _p(u0), _p(du0), _p(uT), _p(duT)))
        self.sync()


def timed_with(adj, which, seg, block, fn):
    adj.set_launch(which, seg or 0, block or 0)
    return fn()


def _functions():
    import torch

    class Trajectory(torch.autograd.Function):
        """u0 (flat ghosted) -> u after the Adjoint's nsteps steps; backward runs
        the checkpointed adjoint sweep."""

        @staticmethod
        def forward(ctx, u0, adj):
            uT = adj.empty()
            adj.forward(u0.detach().contiguous(), uT)
            ctx.adj = adj
            return uT

        @staticmethod
        def backward(ctx, g):
            ub0 = ctx.adj.empty()
            ctx.adj.backward(g.contiguous(), ub0)
            return ub0, None

    class RHS(torch.autograd.Function):
        """u (flat ghosted) -> right-hand side R(u); reverse mode through the
        hand-written adjoint kernel, forward mode through the dual-number kernel."""

        @staticmethod
        def forward(ctx, u, adj):
            k, dk = adj.empty(), adj.empty()
            u = u.detach().contiguous()
            adj.rhs_jvp(u, torch.zeros_like(u), k, dk)
            ctx.adj = adj
            ctx.save_for_backward(u)
            ctx.save_for_forward(u)
            return k

        @staticmethod
        def backward(ctx, g):
            (u,) = ctx.saved_tensors
            ub = ctx.adj.empty()
            ctx.adj.rhs_vjp(u, g.contiguous(), ub)
            return ub, None

        @staticmethod
        def jvp(ctx, du, _):
            (u,) = ctx.saved_tensors
            k, dk = ctx.adj.empty(), ctx.adj.empty()
            ctx.adj.rhs_jvp(u, du.contiguous(), k, dk)
            return dk

    return Trajectory, RHS


_FN = None


def trajectory(u0, adj: Adjoint):
    """Differentiable n-step solve (torch.autograd.Function over gb_adjoint_*)."""
    global _FN
    if _FN is None:
        _FN = _functions()
    return _FN[0].apply(u0, adj)


def rhs(u, adj: Adjoint):
    """Differentiable right-hand side (reverse and forward mode)."""
    global _FN
    if _FN is None:
        _FN = _functions()
    return _FN[1].apply(u, adj)


def density_misfit_gradient(adj: Adjoint, u0_int, rho_target):
    """Loss 0.5 ||rho(T) - rho_target||^2 over the interior and its gradient with
    respect to the initial density, through ``trajectory`` and torch autograd.
    u0_int: (ny, nx, 4) tensor; rho_target: (ny, nx) tensor."""
    u0 = adj.ghosted(u0_int.detach()).requires_grad_(True)
    uT = trajectory(u0, adj)
    rhoT = adj.interior(uT)[..., 0]
    loss = 0.5 * ((rhoT - rho_target) ** 2).sum()
    loss.backward()
    return float(loss.detach()), adj.interior(u0.grad)[..., 0].clone()
