"""Input decks for the Euler1D / Euler2D / NavierStokes3D workloads.

Writes HyPar's own input files (``solver.inp``, ``physics.inp``,
``boundary.inp``, ``weno.inp`` and a binary ``initial.inp``) for the synthetic
workloads: the Sod shock tube, the isentropic vortex and the Taylor-Green
vortex.  The formats follow the reference readers: ``ReadInputs``
(src/Simulation/ReadInputs.c:94-440), ``InitializeBoundaries``
(src/Simulation/InitializeBoundaries.c:75-180), ``WENOInitialize``
(src/InterpolationFunctions/WENOInitialize.c:62-96) and the binary
``ReadArraySerial`` layout (src/IOFunctions/ReadArray.c:215-240: the grid
coordinates of every dimension, then the solution with the components of a
point contiguous and dimension 0 fastest).

The initial conditions restate the reference's example generators
(Examples/1D/Euler1D/SodShockTube/aux/init.c:38-60 and
Examples/2D/Euler2D/VortexConvection/aux/init.C:48-80, with the vortex
strength and centre as parameters) and the Taylor-Green vortex in acoustic
scaling (rho = 1, p = 1/gamma, Mach M).
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class Case:
    """A complete HyPar input deck held in memory."""

    model: str                      # "euler1d" | "euler2d" | "navierstokes3d"
    size: List[int]
    x: List[np.ndarray]             # grid coordinates per dimension
    u: np.ndarray                   # (prod(size), nvars), dimension 0 fastest
    dt: float
    n_iter: int
    time_scheme_type: str           # "44" | "ssprk3" | "22" | "33" | "1fe"
    interp: str = "components"      # "components" | "characteristic"
    upwinding: str = "roe"
    gamma: float = 1.4
    eps: float = 1e-6
    bc: str = "periodic"            # "periodic" | "extrapolate"
    Re: Optional[float] = None      # NavierStokes3D physics.inp values
    Pr: float = 0.72
    Minf: float = 1.0
    file_op_iter: Optional[int] = None
    weights: str = "js"             # WENO5 weights: "js" | "mapped" | "borges" | "yc" | "none" (no_limiting)
    hyp_scheme: str = "weno5"       # solver.inp hyp_space_scheme: "weno5" | "crweno5"
    op_overwrite: str = "yes"       # solver.inp op_overwrite ("no": op_NNNNN.bin every file_op_iter)
    restart_iter: int = 0           # solver.inp restart_iter
    screen_op_iter: Optional[int] = None
    # per-face boundary types: {(dim, face): (bctype, [values after the extents])};
    # faces not listed take `bc`.  Thermal walls add a third item, the wall
    # temperature (times, field): field has the face's size per transverse dimension
    # and len(times) along the wall's own dimension, dimension 0 fastest (the
    # reference's temperature file layout, written beside the deck by `write`).
    # turbulent-supersonic-inflow adds (n, data): n slices along the zone's dimension,
    # the grid across, nvars values per point, dimension 0 fastest (the reference's
    # inflow data file layout, also written by `write`)
    bcs: Optional[dict] = None
    # sponge zones after the face zones: [(dim, face, [(xmin, xmax) per dim], [nvars values])],
    # the state the sponge relaxes to over the box xmin..xmax (BCSponge.c)
    sponges: Optional[list] = None
    # gravity: NavierStokes3D (physics.inp gravity gx gy gz / rho_ref / p_ref / R / HB /
    # N_bv) or Euler1D (gravity g, gravity_type grav_type)
    gravity: Optional[Sequence[float]] = None
    grav_type: int = 0
    rho_ref: float = 1.0
    p_ref: float = 1.0
    R_gas: float = 1.0
    HB: int = 0
    N_bv: float = 0.0
    conservation_check: bool = False  # solver.inp conservation_check yes
    par_scheme: str = "4"             # NavierStokes3D solver.inp par_space_scheme: "4" or "2"
    op_format: str = "binary"         # solver.inp op_file_format: binary | text | tecplot2d | tecplot3d | none

    @property
    def ndims(self) -> int:
        return len(self.size)

    @property
    def nvars(self) -> int:
        return {"euler1d": 3, "euler2d": 4, "navierstokes3d": 5}[self.model]

    def solver_inp(self) -> str:
        nd = self.ndims
        lines = [
            "begin",
            f"  ndims             {nd}",
            f"  nvars             {self.nvars}",
            "  size              " + " ".join(str(s) for s in self.size),
            "  iproc             " + " ".join("1" for _ in self.size),
            "  ghost             3",
            f"  n_iter            {self.n_iter}",
        ]
        # "euler": forward Euler (time_scheme euler, HyPar's default), else an RK table
        if self.time_scheme_type == "euler":
            lines.append("  time_scheme       euler")
        else:
            lines += ["  time_scheme       rk", f"  time_scheme_type  {self.time_scheme_type}"]
        lines += [
            f"  hyp_space_scheme  {self.hyp_scheme}",
            f"  hyp_interp_type   {self.interp}",
        ]
        if self.model == "navierstokes3d":
            lines += ["  par_space_type    nonconservative-2stage", f"  par_space_scheme  {self.par_scheme}"]
        lines += [
            f"  dt                {float(self.dt)!r}",
            f"  screen_op_iter    {self.screen_op_iter or max(self.n_iter, 1)}",
            f"  file_op_iter      {self.file_op_iter or max(self.n_iter, 1)}",
            "  ip_file_type      binary",
            f"  op_file_format    {self.op_format}",
            f"  op_overwrite      {self.op_overwrite}",
            f"  model             {self.model}",
        ]
        if self.restart_iter:
            lines.append(f"  restart_iter      {self.restart_iter}")
        if self.conservation_check:
            lines.append("  conservation_check yes")
        lines.append("end")
        return "\n".join(lines) + "\n"

    def physics_inp(self) -> str:
        lines = ["begin", f"  gamma      {float(self.gamma)!r}", f"  upwinding  {self.upwinding}"]
        if self.model == "euler1d" and self.gravity is not None:
            lines += [f"  gravity    {float(self.gravity[0])!r}", f"  gravity_type {int(self.grav_type)}"]
        if self.model == "navierstokes3d":
            lines += [f"  Pr         {float(self.Pr)!r}", f"  Minf       {float(self.Minf)!r}"]
            if self.Re is not None:
                lines.append(f"  Re         {float(self.Re)!r}")
            if self.gravity is not None:
                gx, gy, gz = (float(v) for v in self.gravity)
                lines += [f"  gravity    {gx!r} {gy!r} {gz!r}", f"  rho_ref    {float(self.rho_ref)!r}",
                          f"  p_ref      {float(self.p_ref)!r}", f"  R          {float(self.R_gas)!r}"]
                lines.append(f"  HB         {int(self.HB)}" + (f" {float(self.N_bv)!r}" if self.HB == 3 else ""))
        lines.append("end")
        return "\n".join(lines) + "\n"

    def weno_inp(self) -> str:
        flags = {k: int(self.weights == k) for k in ("mapped", "borges", "yc")}
        flags["no_limiting"] = int(self.weights == "none")
        return ("begin\n" + "".join(f"  {k} {v}\n" for k, v in flags.items())
                + f"  epsilon {float(self.eps)!r}\n  p 2.0\nend\n")

    def boundary_inp(self) -> str:
        nd = self.ndims
        # transverse extents padded so that they cover the whole grid
        lo = [float(xx[0]) - 1.0 for xx in self.x]
        hi = [float(xx[-1]) + 1.0 for xx in self.x]
        rows = []
        for d in range(nd):
            for face in (1, -1):
                ext = []
                for e in range(nd):
                    ext += ["0", "0"] if e == d else [repr(lo[e]), repr(hi[e])]
                spec = (self.bcs or {}).get((d, face), (self.bc, []))
                bctype, vals = spec[0], spec[1]
                items = ext + [repr(float(v)) for v in vals]
                if bctype.startswith("thermal-"):
                    items.append(self.temperature_file(d, face))
                if bctype == "turbulent-supersonic-inflow":
                    items.append(self.inflow_file(d, face))
                rows.append(f"{bctype} {d} {face} " + " ".join(items))
        for d, face, box, vals in (self.sponges or []):
            items = [repr(float(v)) for lohi in box for v in lohi] + [repr(float(v)) for v in vals]
            rows.append(f"sponge {d} {face} " + " ".join(items))
        return f"{len(rows)}\n" + "\n".join(rows) + "\n"

    @staticmethod
    def temperature_file(d: int, face: int) -> str:
        return f"temperature_{d}_{'lo' if face == 1 else 'hi'}.bin"

    @staticmethod
    def inflow_file(d: int, face: int) -> str:
        return f"inflow_{d}_{'lo' if face == 1 else 'hi'}.bin"

    def inflow_bytes(self, d: int, face: int) -> bytes:
        """A turbulent inflow face's data in the reference's binary format
        (BCReadTurbulentInflowData, src/BoundaryConditions/BCIO.c:19-139, one rank): int
        rank[ndims], int size[ndims], double data[nvars * prod(size)]."""
        n, data = self.bcs[(d, face)][2]
        size = [int(n) if e == d else self.size[e] for e in range(self.ndims)]
        data = np.asarray(data, np.float64).reshape(-1)
        assert data.size == self.nvars * int(np.prod(size)), (data.size, size)
        rank = np.zeros(self.ndims, np.int32)
        return rank.tobytes() + np.asarray(size, np.int32).tobytes() + data.tobytes()

    def temperature_bytes(self, d: int, face: int) -> bytes:
        """The wall temperature of a thermal-wall face in the reference's binary format
        (BCReadTemperatureData, src/BoundaryConditions/BCIO.c:147-260, one rank): int
        rank[ndims], int size[ndims], double times[size[d]], double field[prod(size)]."""
        times, field = self.bcs[(d, face)][2]
        times = np.asarray(times, np.float64)
        size = [len(times) if e == d else self.size[e] for e in range(self.ndims)]
        field = np.asarray(field, np.float64).reshape(-1)
        assert field.size == int(np.prod(size)), (field.size, size)
        rank = np.zeros(self.ndims, np.int32)
        return rank.tobytes() + np.asarray(size, np.int32).tobytes() + times.tobytes() + field.tobytes()

    def initial_bytes(self) -> bytes:
        xs = np.concatenate([np.asarray(xx, dtype=np.float64) for xx in self.x])
        return xs.tobytes() + np.ascontiguousarray(self.u, dtype=np.float64).tobytes()

    def write(self, directory: str) -> str:
        os.makedirs(directory, exist_ok=True)
        files = {
            "solver.inp": self.solver_inp(),
            "physics.inp": self.physics_inp(),
            "boundary.inp": self.boundary_inp(),
            "weno.inp": self.weno_inp(),
        }
        for name, text in files.items():
            with open(os.path.join(directory, name), "w") as f:
                f.write(text)
        with open(os.path.join(directory, "initial.inp"), "wb") as f:
            f.write(self.initial_bytes())
        for (d, face), spec in (self.bcs or {}).items():
            if spec[0].startswith("thermal-"):
                with open(os.path.join(directory, self.temperature_file(d, face)), "wb") as f:
                    f.write(self.temperature_bytes(d, face))
            if spec[0] == "turbulent-supersonic-inflow":
                with open(os.path.join(directory, self.inflow_file(d, face)), "wb") as f:
                    f.write(self.inflow_bytes(d, face))
        return directory


def sod(n: int = 1024, n_iter: int = 1000, dt: float = 1e-4, interp: str = "components",
        upwinding: str = "roe", scheme: str = "44") -> Case:
    """Sod shock tube on x_i = i/(n-1) with mirror ("extrapolate") ends."""
    x = np.arange(n, dtype=np.float64) * (1.0 / float(n - 1))
    left = x < 0.5
    rho = np.where(left, 1.0, 0.125)
    P = np.where(left, 1.0, 0.1)
    U = np.zeros(n)
    e = P / 0.4 + 0.5 * rho * U * U
    u = np.stack([rho, rho * U, e], axis=1)
    return Case("euler1d", [n], [x], u, dt, n_iter, scheme, interp, upwinding, bc="extrapolate")


def vortex_state(n: int, b: float = 5.0, xc: float = 5.0, yc: float = 5.0, gamma: float = 1.4,
                 length: float = 10.0, uinf: float = 0.5, vinf: float = 0.0):
    """Isentropic vortex of strength b centred at (xc, yc) on an n x n periodic grid."""
    h = length / float(n)
    x = np.arange(n, dtype=np.float64) * h
    X, Y = np.meshgrid(x, x, indexing="xy")  # X[j, i] = x_i : dimension 0 fastest
    rsq = (X - xc) ** 2 + (Y - yc) ** 2
    pi = math.pi
    rho = np.power(1.0 - ((gamma - 1.0) * b * b) / (8.0 * gamma * pi * pi) * np.exp(1.0 - rsq),
                   1.0 / (gamma - 1.0))
    P = np.power(rho, gamma)
    du = -b / (2.0 * pi) * np.exp(0.5 * (1.0 - rsq)) * (Y - yc)
    dv = b / (2.0 * pi) * np.exp(0.5 * (1.0 - rsq)) * (X - xc)
    uu = uinf + du
    vv = vinf + dv
    e = P / (gamma - 1.0) + 0.5 * rho * (uu * uu + vv * vv)
    u = np.stack([rho, rho * uu, rho * vv, e], axis=-1).reshape(n * n, 4)
    return x, u


def vortex(n: int = 1024, n_iter: int = 200, dt: Optional[float] = None, b: float = 5.0,
           xc: float = 5.0, yc: float = 5.0, interp: str = "characteristic",
           upwinding: str = "roe", scheme: str = "ssprk3", cfl: float = 0.5) -> Case:
    """Isentropic vortex convection on [0,10)^2, periodic; dt from the CFL target if not given."""
    x, u = vortex_state(n, b, xc, yc)
    if dt is None:
        dt = cfl_dt(u, 4, [10.0 / n, 10.0 / n], cfl)
    return Case("euler2d", [n, n], [x, x.copy()], u, dt, n_iter, scheme, interp, upwinding)


def cfl_dt(u: np.ndarray, nvars: int, h: Sequence[float], cfl: float, gamma: float = 1.4) -> float:
    """Time step for a target CFL with the reference's CFL measure
    max_d (|v_d| + c) dt / h_d (Euler2DComputeCFL.c:21-39)."""
    rho = u[:, 0]
    vel = [u[:, 1 + d] / rho for d in range(len(h))]
    vsq = sum(v * v for v in vel)
    P = (u[:, nvars - 1] - 0.5 * rho * vsq) * (gamma - 1.0)
    c = np.sqrt(gamma * P / rho)
    rate = max(float(np.max((np.abs(v) + c) / hd)) for v, hd in zip(vel, h))
    return cfl / rate


def tgv(n: int = 256, n_iter: int = 100, dt: float = 2e-3, mach: float = 0.1, Re: float = 1600.0,
        Pr: float = 0.72, interp: str = "components", upwinding: str = "roe",
        scheme: str = "44", gamma: float = 1.4, perturb: float = 0.0, seed: int = 1) -> Case:
    """Taylor-Green vortex on [0, 2 pi)^3, periodic, acoustic scaling.

    perturb > 0 multiplies density and pressure pointwise by 1 + perturb*N(0,1)
    (seeded, clipped at 3 sigma): a state whose flux divergence is not the
    near-cancellation of the divergence-free t=0 vortex, for parity checks
    that should not be dominated by rounding noise."""
    h = 2.0 * math.pi / n
    x = np.arange(n, dtype=np.float64) * h
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")  # X[k, j, i] = x_i
    rho = np.ones_like(X)
    M = mach
    P = 1.0 / gamma + (M * M / 16.0) * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2.0)
    uu = M * np.sin(X) * np.cos(Y) * np.cos(Z)
    vv = -M * np.cos(X) * np.sin(Y) * np.cos(Z)
    ww = np.zeros_like(X)
    if perturb > 0.0:
        rng = np.random.default_rng(seed)
        rho = rho * (1.0 + perturb * np.clip(rng.standard_normal(rho.shape), -3, 3))
        P = P * (1.0 + perturb * np.clip(rng.standard_normal(P.shape), -3, 3))
    e = P / (gamma - 1.0) + 0.5 * rho * (uu * uu + vv * vv + ww * ww)
    u = np.stack([rho, rho * uu, rho * vv, rho * ww, e], axis=-1).reshape(n ** 3, 5)
    return Case("navierstokes3d", [n, n, n], [x, x.copy(), x.copy()], u, dt, n_iter, scheme,
                interp, upwinding, gamma=gamma, Re=Re, Pr=Pr, Minf=mach)


def stratified_1d(n: int = 64, n_iter: int = 10, dt: float = 2e-3, g: float = 1.0, grav_type: int = 0,
                  interp: str = "components", upwinding: str = "roe", scheme: str = "44", perturb: float = 0.01,
                  seed: int = 3) -> Case:
    """A 1-D atmosphere in the gravity field of physics.inp (Xing & Shu, J. Sci. Comput. 54,
    2013): isothermal hydrostatic rho = p = S with S = exp(-g x) (gravity_type 0, x_i =
    i/(n-1), mirror ends) or S = exp(sin(2 pi x)/(2 pi)) (gravity_type 1, x_i = i/n,
    periodic), at rest, with the pressure perturbed pointwise by 1 + perturb N(0,1)
    (seeded, clipped at 3 sigma; perturb = 0: the balanced state)."""
    gamma = 1.4
    if grav_type == 0:
        x = np.arange(n, dtype=np.float64) / float(n - 1)
        S = np.exp(-g * x)
        bc = "extrapolate"
    else:
        x = np.arange(n, dtype=np.float64) / float(n)
        S = np.exp(np.sin(2.0 * math.pi * x) / (2.0 * math.pi))
        bc = "periodic"
    rho, P = S.copy(), S.copy()
    if perturb > 0.0:
        rng = np.random.default_rng(seed)
        P = P * (1.0 + perturb * np.clip(rng.standard_normal(n), -3, 3))
    u = np.stack([rho, np.zeros(n), P / (gamma - 1.0)], axis=-1)
    return Case("euler1d", [n], [x], u, dt, n_iter, scheme, interp, upwinding, gamma=gamma, bc=bc,
                gravity=(g, 0.0, 0.0), grav_type=grav_type)


def rising_thermal_bubble(n: int = 64, n_iter: int = 100, dt: float = 0.01, interp: str = "components",
                          upwinding: str = "rusanov", weights: str = "yc", scheme: str = "ssprk3",
                          HB: int = 2, perturb: float = 0.0, seed: int = 1) -> Case:
    """Rising thermal bubble (Kelly & Giraldo, J. Comput. Phys. 231, 2012, sec. 5.1.2):
    a warm bubble in a hydrostatically balanced, neutrally stratified atmosphere on
    [0, 1000 m]^3 with n points per side (grid spacing 1000/(n-1)), gravity 9.8 m/s^2
    along y, slip walls on every face.  The ambient state has constant potential
    temperature T_ref = p_ref / (R rho_ref) and Exner pressure pi = 1 - g y / (Cp T_ref);
    a cosine bump of 0.5 K, radius 250 m, centred at (500, 260, 500), raises the
    potential temperature theta.  Then rho = p_ref / (R theta) pi^(1/(gamma-1)) and the
    energy is p / (gamma-1) with p = rho R theta pi (at rest).  perturb > 0 multiplies the
    density pointwise by 1 + perturb*N(0,1) (seeded, clipped at 3 sigma) for parity
    checks away from the balanced state."""
    gamma, R, rho_ref, p_ref, g = 1.4, 287.058, 1.1612055171196529, 100000.0, 9.8
    h = 1000.0 / (n - 1)
    x = np.arange(n, dtype=np.float64) * h
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")  # X[k, j, i] = x_i
    Cp = gamma * R / (gamma - 1.0)
    T_ref = p_ref / (R * rho_ref)
    r = np.sqrt((X - 500.0) ** 2 + (Y - 260.0) ** 2 + (Z - 500.0) ** 2)
    theta = T_ref + np.where(r > 250.0, 0.0, 0.5 * (1.0 + np.cos(math.pi * r / 250.0)))
    exner = 1.0 - g * Y / (Cp * T_ref)
    rho = p_ref / (R * theta) * np.exp(np.log(exner) / (gamma - 1.0))
    E = rho * (R / (gamma - 1.0)) * theta * exner
    if perturb > 0.0:
        rng = np.random.default_rng(seed)
        rho = rho * (1.0 + perturb * np.clip(rng.standard_normal(rho.shape), -3, 3))
    zero = np.zeros_like(rho)
    u = np.stack([rho, zero, zero, zero, E], axis=-1).reshape(n ** 3, 5)
    bcs = {(d, f): ("slip-wall", [0.0, 0.0, 0.0]) for d in range(3) for f in (1, -1)}
    return Case("navierstokes3d", [n, n, n], [x, x.copy(), x.copy()], u, dt, n_iter, scheme, interp,
                upwinding, gamma=gamma, weights=weights, bcs=bcs, gravity=(0.0, g, 0.0), rho_ref=rho_ref,
                p_ref=p_ref, R_gas=R, HB=HB)


def isotropic_turbulence(n: int = 256, n_iter: int = 100, dt: float = 0.005, u0: float = 0.3, kp: float = 4.0,
                         Re: float = 333.333333333333333, Pr: float = 0.72, weights: str = "mapped",
                         interp: str = "components", upwinding: str = "roe", scheme: str = "ssprk3",
                         seed: int = 1) -> Case:
    """Decaying isotropic turbulence on [0, 2 pi)^3, periodic: rho = 1, p = 1/gamma and a
    random solenoidal velocity field with the Passot-Pouquet energy spectrum
    E(k) ~ (k/kp)^4 exp(-2 (k/kp)^2), scaled to a component-wise rms velocity u0 (which is
    also the reference Mach number: c = 1).  Each Fourier mode gets a seeded random
    complex amplitude of magnitude sqrt(E(k) / (4 pi k^2)), projected on the plane normal
    to k (divergence free).  physics.inp: Minf = u0, Re as given."""
    gamma = 1.4
    h = 2.0 * math.pi / n
    x = np.arange(n, dtype=np.float64) * h
    rng = np.random.default_rng(seed)
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    kr = np.fft.rfftfreq(n, d=1.0 / n)
    KZ, KY, KX = np.meshgrid(k1, k1, kr, indexing="ij")  # field index [z, y, x]
    kk = np.sqrt(KX * KX + KY * KY + KZ * KZ)
    ks = np.where(kk > 0.0, kk, 1.0)
    E = (ks / kp) ** 4 * np.exp(-2.0 * (ks / kp) ** 2)
    amp = np.where(kk > 0.0, np.sqrt(E / (4.0 * math.pi * ks * ks)), 0.0)
    vel = []
    xi = [(rng.standard_normal(kk.shape) + 1j * rng.standard_normal(kk.shape)) * amp for _ in range(3)]
    kdotxi = (KX * xi[0] + KY * xi[1] + KZ * xi[2]) / (ks * ks)
    for comp, kc in zip(xi, (KX, KY, KZ)):
        vel.append(np.fft.irfftn(comp - kdotxi * kc, s=(n, n, n), axes=(0, 1, 2)))
    rms = math.sqrt(sum(float(np.mean(v * v)) for v in vel) / 3.0)
    uu, vv, ww = (v * (u0 / rms) for v in vel)
    rho = np.ones_like(uu)
    P = np.full_like(uu, 1.0 / gamma)
    e = P / (gamma - 1.0) + 0.5 * rho * (uu * uu + vv * vv + ww * ww)
    u = np.stack([rho, rho * uu, rho * vv, rho * ww, e], axis=-1).reshape(n ** 3, 5)
    return Case("navierstokes3d", [n, n, n], [x, x.copy(), x.copy()], u, dt, n_iter, scheme, interp, upwinding,
                gamma=gamma, Re=Re, Pr=Pr, Minf=u0, weights=weights)


def read_op_bin(path: str) -> Dict[str, np.ndarray]:
    """Read a HyPar binary solution file (src/IOFunctions/WriteBinary.c): int32
    ndims, nvars, dim[ndims], float64 grid, float64 solution."""
    with open(path, "rb") as f:
        buf = f.read()
    ndims, nvars = np.frombuffer(buf, np.int32, 2, 0)
    dims = np.frombuffer(buf, np.int32, ndims, 8)
    off = 8 + 4 * int(ndims)
    nx = int(dims.sum())
    x = np.frombuffer(buf, np.float64, nx, off)
    off += 8 * nx
    npts = int(np.prod(dims))
    u = np.frombuffer(buf, np.float64, npts * int(nvars), off).reshape(npts, int(nvars))
    return {"ndims": int(ndims), "nvars": int(nvars), "dims": dims.copy(), "x": x.copy(), "u": u.copy()}


def ensemble_sizes(nmembers: int = 64, seed: int = 20261203, lo: int = 128, hi: int = 1024, step: int = 64):
    """Square grid sizes drawn uniformly (seeded) from {lo, lo+step, ..., hi}."""
    rng = np.random.default_rng(seed)
    choices = np.arange(lo, hi + 1, step)
    return [int(v) for v in rng.choice(choices, size=nmembers)]


def ensemble_vortex(nmembers: int = 64, seed: int = 20261203, n_iter: int = 100, sizes=None,
                    interp: str = "characteristic", upwinding: str = "roe", scheme: str = "ssprk3",
                    cfl: float = 0.5):
    """Ensemble of isentropic vortices: sizes from ensemble_sizes, strength
    b ~ U[1,5], centre ~ U[3,7]^2 (seeded), one common dt = the CFL-0.5 step of
    the most restrictive member.  Returns a list of Cases sharing dt."""
    rng = np.random.default_rng(seed + 1)
    if sizes is None:
        sizes = ensemble_sizes(nmembers, seed)
    members = []
    dts = []
    for n in sizes:
        b = float(rng.uniform(1.0, 5.0))
        xc, yc = (float(v) for v in rng.uniform(3.0, 7.0, size=2))
        c = vortex(n, n_iter=n_iter, dt=1.0, b=b, xc=xc, yc=yc, interp=interp, upwinding=upwinding,
                   scheme=scheme)
        dts.append(cfl_dt(c.u, 4, [10.0 / n, 10.0 / n], cfl))
        members.append(c)
    dt = min(dts)
    for c in members:
        c.dt = dt
    return members


def write_ensemble(members, directory: str) -> str:
    """HyPar ensemble deck: simulation.inp, one solver.inp listing every size,
    initial_<k>.inp and boundary_<k>.inp (k zero-padded to log10(n)+1 digits)."""
    os.makedirs(directory, exist_ok=True)
    n = len(members)
    width = int(math.log10(n)) + 1
    c0 = members[0]
    # "size" and "iproc" list ndims values for every simulation (ReadInputs.c:189-230)
    txt = c0.solver_inp().replace("  size              " + " ".join(str(s) for s in c0.size),
                                  "  size              " + "  ".join(" ".join(str(s) for s in c.size)
                                                                     for c in members))
    txt = txt.replace("  iproc             " + " ".join("1" for _ in c0.size),
                      "  iproc             " + "  ".join(" ".join("1" for _ in c.size) for c in members))
    with open(os.path.join(directory, "simulation.inp"), "w") as f:
        f.write(f"begin\n  nsims {n}\nend\n")
    with open(os.path.join(directory, "solver.inp"), "w") as f:
        f.write(txt)
    with open(os.path.join(directory, "physics.inp"), "w") as f:
        f.write(c0.physics_inp())
    with open(os.path.join(directory, "weno.inp"), "w") as f:
        f.write(c0.weno_inp())
    for k, c in enumerate(members):
        idx = str(k).zfill(width)
        with open(os.path.join(directory, f"boundary_{idx}.inp"), "w") as f:
            f.write(c.boundary_inp())
        with open(os.path.join(directory, f"initial_{idx}.inp"), "wb") as f:
            f.write(c.initial_bytes())
    return directory


def adjoint_problem(n: int = 256, n_iter: int = 400, seed: int = 20261203, scheme: str = "44",
                    cfl: float = 0.5):
    """Initial-condition inversion for 2D Euler on [0,10)^2, periodic, component-wise
    WENO5 + Roe: the target is the density after n_iter steps from the b=5 vortex
    centred at (5, 5); the initial guess is a b=4 vortex whose centre is shifted by
    U[-0.5, 0.5]^2 (seeded).  One dt (CFL 0.5 of the more restrictive state) serves
    both runs.  Returns (case, u_true): the deck of the initial guess and the
    interior state whose run defines the target."""
    rng = np.random.default_rng(seed)
    sx, sy = (float(v) for v in rng.uniform(-0.5, 0.5, size=2))
    _, u_true = vortex_state(n, 5.0, 5.0, 5.0)
    case = vortex(n, n_iter=n_iter, dt=1.0, b=4.0, xc=5.0 + sx, yc=5.0 + sy, interp="components",
                  upwinding="roe", scheme=scheme)
    h = [10.0 / n, 10.0 / n]
    case.dt = min(cfl_dt(u_true, 4, h, cfl), cfl_dt(case.u, 4, h, cfl))
    return case, u_true
