"""Small, self-contained launches of single kernels, for profilers.

    python -m hypar_gb300.probe vjp  [--size N] [--calls K] [--seg SX SY]
    python -m hypar_gb300.probe jvp  [--size N] [--calls K]
    python -m hypar_gb300.probe step [--size N] [--calls K]

Each builds the adjoint test problem of `cases.adjoint_problem` on an N x N grid
(Euler2D, component-wise WENO5 + Roe, RK4), then makes K calls of one entry point:
the right-hand side's VJP (gb_adjoint_rhs_vjp), its dual-number JVP
(gb_adjoint_rhs_jvp), or one fused Runge-Kutta step (gb_solver_step).  Nothing
else is launched on the GPU besides the set-up copies, so a profiler can select
the launches by kernel name without skipping through unrelated work.
"""
from __future__ import annotations

import argparse
import tempfile


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["vjp", "jvp", "step"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--calls", type=int, default=3)
    ap.add_argument("--seg", type=int, nargs=2, default=None, help="adjoint kernel segment lengths x, y")
    args = ap.parse_args()
    import torch
    from . import cases as C
    from .adjoint import Adjoint
    from .solver import Inputs, Solver

    n = args.size
    case, _ = C.adjoint_problem(n, 4)
    d = tempfile.mkdtemp(prefix="gbh_probe_")
    case.write(d)
    inp = Inputs(d)
    if args.what == "step":
        s = Solver(inp.config, inp.dxinv, device=0)
        s.set_state(case.u)
        s.step(args.calls)
        s.sync()
        print("ok", args.what, n, args.calls)
        return
    adj = Adjoint(inp.config, inp.dxinv, 4, 0, 0)
    if args.seg:
        adj.set_launch(2, args.seg[0])
        adj.set_launch(3, args.seg[1])
    u = adj.ghosted(torch.from_numpy(case.u.reshape(n, n, 4).copy()).cuda()).contiguous()
    a, b = adj.empty(), adj.empty()
    a.normal_()
    for _ in range(args.calls):
        if args.what == "vjp":
            adj.rhs_vjp(u, a, b)
        else:
            adj.rhs_jvp(u, a, b, adj.empty())
    torch.cuda.synchronize()
    print("ok", args.what, n, args.calls)


if __name__ == "__main__":
    main()
