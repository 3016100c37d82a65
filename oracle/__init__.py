"""Python access to the CPU oracle (test infrastructure only).

The oracle is a C restatement of HyPar's explicit WENO5 right-hand side and
Runge-Kutta step (``gbh_oracle.c``).  Only the tests, ``__graft_entry__.smoke``
and the CPU-baseline arm of ``bench.py`` use it -- always as the checker or the
timed CPU baseline, never as the product.

Grid set-up helpers restate the reference:
  * ghost grid coordinates extrapolated linearly (src/IOFunctions/ReadArray.c:68-88),
  * ``dxinv[i] = 2/(x[i+1]-x[i-1])`` per point, ghost values copied from the
    first/last interior value (src/Simulation/InitialSolution.c:69-99),
  * boundary-zone extents from ``FindInterval`` (src/MathFunctions/FindInterval.c:19-45,
    src/Simulation/InitializeBoundaries.c:365-420).
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
# The same restatement compiled with fused multiply-add contraction: it differs
# from the reference only by rounding, so its distance from liboracle.so
# measures how strongly a state amplifies rounding differences.
FMA_LIB_PATH = os.path.join(HERE, "liboracle_fma.so")
REF_DIR = os.path.join(HERE, "_ref")

MODELS = {"euler1d": 1, "euler2d": 2, "navierstokes3d": 3}
UPWIND = {"roe": 0, "llf-char": 1, "rf-char": 2, "rusanov": 3, "steger-warming": 4}
INTERP = {"components": 0, "characteristic": 1}
WEIGHTS = {"js": 0, "mapped": 1, "borges": 2, "yc": 3, "none": 4}
BCTYPE = {"periodic": 1, "extrapolate": 2, "dirichlet": 3, "slip-wall": 4, "noslip-wall": 5,
          "subsonic-inflow": 6, "subsonic-outflow": 7, "supersonic-inflow": 8, "supersonic-outflow": 9,
          "subsonic-ambivalent": 10, "thermal-slip-wall": 11, "thermal-noslip-wall": 12, "sponge": 13,
          "turbulent-supersonic-inflow": 14, "reflect": 15}


SCHEMES = {"weno5": 0, "crweno5": 1}


def bc_nvalues(bctype: str, ndims: int, nvars: int) -> int:
    """How many values boundary.inp gives after a zone's extents (InitializeBoundaries.c:109-188)."""
    return {"dirichlet": nvars, "slip-wall": ndims, "noslip-wall": ndims, "subsonic-inflow": 1 + ndims,
            "subsonic-outflow": 1, "supersonic-inflow": 2 + ndims,
            "subsonic-ambivalent": 2 + ndims, "thermal-slip-wall": ndims,
            "thermal-noslip-wall": ndims, "sponge": nvars,
            "turbulent-supersonic-inflow": 2 + ndims}.get(bctype, 0)

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so (gcc, OpenMP, no FMA contraction) and liboracle_fma.so."""
    src = os.path.join(HERE, "gbh_oracle.c")
    if (not force and all(os.path.exists(p) and os.path.getmtime(p) >= os.path.getmtime(src)
                          for p in (LIB_PATH, FMA_LIB_PATH))):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-std=c99", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB_PATH, src, "-lm"]
    subprocess.check_call(cmd)
    fma = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    subprocess.check_call(["gcc", "-O3", "-std=gnu99", "-ffp-contract=fast"] + fma +
                          ["-fopenmp", "-fPIC", "-shared", "-o", FMA_LIB_PATH, src, "-lm"])
    return LIB_PATH


def _bind(path):
    L = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    L.orc_problem_create.restype = ctypes.c_void_p
    L.orc_problem_create.argtypes = [ctypes.c_int, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_int, ip, dp]
    L.orc_problem_destroy.argtypes = [ctypes.c_void_p]
    L.orc_set_weights.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.orc_set_weights.restype = None
    L.orc_set_zone_data.argtypes = [ctypes.c_void_p, ctypes.c_int, dp]
    L.orc_set_zone_data.restype = None
    L.orc_set_zone_temperature.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp, dp]
    L.orc_set_zone_temperature.restype = ctypes.c_int
    L.orc_set_time.argtypes = [ctypes.c_void_p, ctypes.c_double]
    L.orc_set_time.restype = None
    L.orc_set_zone_sponge.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_double, ctypes.c_double]
    L.orc_set_zone_sponge.restype = ctypes.c_int
    L.orc_set_zone_inflow.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp]
    L.orc_set_zone_inflow.restype = ctypes.c_int
    L.orc_set_par_scheme.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.orc_set_par_scheme.restype = None
    L.orc_set_gravity.argtypes = [ctypes.c_void_p, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_double]
    L.orc_set_gravity.restype = ctypes.c_int
    L.orc_set_gravity_1d.argtypes = [ctypes.c_void_p, dp, ctypes.c_double, ctypes.c_int]
    L.orc_set_gravity_1d.restype = ctypes.c_int
    L.orc_get_gravity.argtypes = [ctypes.c_void_p, dp]
    L.orc_get_gravity.restype = None
    L.orc_cfl.argtypes = [ctypes.c_void_p, dp, ctypes.c_double]
    L.orc_cfl.restype = ctypes.c_double
    L.orc_apply_bc.argtypes = [ctypes.c_void_p, dp]
    for name in ("orc_hyperbolic", "orc_parabolic", "orc_rhs", "orc_source"):
        getattr(L, name).argtypes = [ctypes.c_void_p, dp, dp]
        getattr(L, name).restype = ctypes.c_int
    L.orc_set_scheme.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.orc_set_scheme.restype = None
    L.orc_rk.restype = ctypes.c_int
    L.orc_rk.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_int]
    L.orc_set_threads.argtypes = [ctypes.c_int]
    L.orc_get_threads.restype = ctypes.c_int
    return L


_fma_lib = None


def fma_lib():
    global _fma_lib
    if _fma_lib is None:
        build()
        _fma_lib = _bind(FMA_LIB_PATH)
    return _fma_lib


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = _bind(LIB_PATH)
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def grid_with_ghosts(x: np.ndarray, g: int) -> np.ndarray:
    """Interior coordinates -> coordinates with linearly extrapolated ghosts."""
    n = len(x)
    X = np.zeros(n + 2 * g)
    X[g:g + n] = x
    for i in range(g):
        delta = g - i
        X[i] = X[g] + float(delta) * (X[g] - X[g + 1])
    for i in range(n + g, n + 2 * g):
        delta = i - (n + g - 1)
        X[i] = X[n + g - 1] + float(delta) * (X[n + g - 1] - X[n + g - 2])
    return X


def dxinv_from_grid(xs: Sequence[np.ndarray], g: int) -> np.ndarray:
    out = []
    for x in xs:
        n = len(x)
        X = grid_with_ghosts(np.asarray(x, np.float64), g)
        D = np.zeros(n + 2 * g)
        for i in range(n):
            D[i + g] = 2.0 / (X[i + 1 + g] - X[i - 1 + g])
        D[:g] = D[g]
        D[n + g:] = D[n + g - 1]
        out.append(D)
    return np.concatenate(out)


def find_interval(a: float, b: float, x: np.ndarray):
    n = len(x)
    imax, imin = -1, n
    min_dx = x[1] - x[0]
    for i in range(2, n):
        min_dx = min(min_dx, x[i] - x[i - 1])
    tol = 1e-10 * min_dx
    for i in range(n):
        if x[i] <= b + tol:
            imax = i + 1
    for i in range(n - 1, -1, -1):
        if x[i] >= a - tol:
            imin = i
    return imin, imax


def zones_from_boundary(rows, xs: Sequence[np.ndarray], g: int) -> np.ndarray:
    """rows: [(bctype, dim, face, [(xmin, xmax) per dim])] -> nzones x 9 int array."""
    out = []
    nd = len(xs)
    for row in rows:
        bctype, dim, face, ext = row[:4]
        is_ = [0, 0, 0]
        ie = [1, 1, 1]
        for d in range(nd):
            if d == dim and bctype != "sponge":
                n = len(xs[d])
                is_[d], ie[d] = (-g, 0) if face == 1 else (n, n + g)
            else:
                is_[d], ie[d] = find_interval(ext[d][0], ext[d][1], np.asarray(xs[d]))
        out.append([BCTYPE[bctype], dim, face] + is_ + ie)
    return np.asarray(out, dtype=np.int32).reshape(-1, 9)


def parse_boundary_inp(text: str, ndims: int, nvars: int = 0):
    """rows (bctype, dim, face, extents, values) of a boundary.inp."""
    tok = text.split()
    nz = int(tok[0])
    k = 1
    rows = []
    for _ in range(nz):
        bctype, dim, face = tok[k], int(tok[k + 1]), int(tok[k + 2])
        k += 3
        ext = []
        for _d in range(ndims):
            ext.append((float(tok[k]), float(tok[k + 1])))
            k += 2
        nvals = bc_nvalues(bctype, ndims, nvars)
        vals = [float(t) for t in tok[k:k + nvals]]
        k += nvals
        if bctype.startswith("thermal-") or bctype == "turbulent-supersonic-inflow":
            k += 1  # the temperature or inflow data file's name
        rows.append((bctype, dim, face, ext, vals))
    return rows


def embed(u_interior: np.ndarray, size: Sequence[int], nvars: int, g: int) -> np.ndarray:
    """(prod(size), nvars) interior array -> flat array with zero ghosts."""
    nd = len(size)
    shp = [s + 2 * g for s in reversed(size)] + [nvars]
    U = np.zeros(shp)
    sl = tuple(slice(g, g + s) for s in reversed(size)) + (slice(None),)
    U[sl] = np.asarray(u_interior).reshape([s for s in reversed(size)] + [nvars])
    return U.reshape(-1)


def interior(u_wg: np.ndarray, size: Sequence[int], nvars: int, g: int) -> np.ndarray:
    shp = [s + 2 * g for s in reversed(size)] + [nvars]
    U = np.asarray(u_wg).reshape(shp)
    sl = tuple(slice(g, g + s) for s in reversed(size)) + (slice(None),)
    return np.ascontiguousarray(U[sl]).reshape(-1, nvars)


RK_TABLES = {
    "1fe": (1, [0.0], [1.0]),
    "22": (2, [0, 0, 1.0, 0], [0.5, 0.5]),
    "33": (3, [0, 0, 0, 2.0 / 3.0, 0, 0, 2.0 / 3.0 - 1.0 / 4.0, 1.0 / 4.0, 0], [1.0 / 4.0, -1.0 / 4.0, 1.0]),
    "44": (4, [0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 1.0, 0],
           [1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0]),
    "ssprk3": (3, [0, 0, 0, 1.0, 0, 0, 0.25, 0.25, 0], [1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0]),
    # time_scheme euler (TimeForwardEuler.c): u += dt RHS(u), the one-stage table
    "euler": (1, [0.0], [1.0]),
}
"""Butcher tables of TimeExplicitRKInitialize (src/TimeIntegration/TimeExplicitRKInitialize.c:28-80)."""


class Problem:
    """One oracle problem built from a case deck (hypar_gb300.cases.Case)."""

    def __init__(self, case, ghosts: int = 3, boundary_rows=None, fma: bool = False):
        self.case = case
        self.g = ghosts
        self.size = list(case.size)
        self.nvars = case.nvars
        xs = [np.asarray(x, np.float64) for x in case.x]
        self.dxinv = dxinv_from_grid(xs, ghosts)
        if boundary_rows is None:
            boundary_rows = parse_boundary_inp(case.boundary_inp(), case.ndims, case.nvars)
        self.zones = zones_from_boundary(boundary_rows, xs, ghosts)
        Re = -1.0
        if case.model == "navierstokes3d" and case.Re is not None:
            Re = case.Re / case.Minf
        dims = np.asarray(self.size, np.int32)
        L = fma_lib() if fma else lib()
        self._L = L
        self.h = L.orc_problem_create(MODELS[case.model], len(self.size), _ip(dims), ghosts,
                                      UPWIND[case.upwinding], INTERP[case.interp], case.gamma,
                                      case.eps, Re, case.Pr, len(self.zones),
                                      _ip(np.ascontiguousarray(self.zones)), _dp(self.dxinv))
        if not self.h:
            raise RuntimeError("orc_problem_create failed")
        L.orc_set_weights(self.h, WEIGHTS[getattr(case, "weights", "js")])
        L.orc_set_scheme(self.h, SCHEMES[getattr(case, "hyp_scheme", "weno5")])
        L.orc_set_par_scheme(self.h, int(getattr(case, "par_scheme", "4")))
        for z, row in enumerate(boundary_rows):
            vals = list(row[4]) if len(row) > 4 else []
            data = np.zeros(8)
            data[:len(vals)] = vals
            L.orc_set_zone_data(self.h, z, _dp(data))
            if row[0].startswith("thermal-"):
                times, field = case.bcs[(row[1], row[2])][2]
                times = np.ascontiguousarray(times, np.float64)
                field = np.ascontiguousarray(field, np.float64).reshape(-1)
                if L.orc_set_zone_temperature(self.h, z, len(times), _dp(times), _dp(field)):
                    raise RuntimeError("orc_set_zone_temperature failed")
            if row[0] == "turbulent-supersonic-inflow":
                n, data = case.bcs[(row[1], row[2])][2]
                data = np.ascontiguousarray(data, np.float64).reshape(-1)
                if L.orc_set_zone_inflow(self.h, z, int(n), _dp(data)):
                    raise RuntimeError("orc_set_zone_inflow failed")
            if row[0] == "sponge":
                dim = row[1]
                if L.orc_set_zone_sponge(self.h, z, _dp(np.ascontiguousarray(xs[dim])), float(row[3][dim][0]),
                                         float(row[3][dim][1])):
                    raise RuntimeError("orc_set_zone_sponge failed")
        grav = getattr(case, "gravity", None)
        if grav is not None and any(float(v) != 0.0 for v in grav):
            xg = np.concatenate([grid_with_ghosts(x, ghosts) for x in xs])
            if case.model == "euler1d":
                rc = L.orc_set_gravity_1d(self.h, _dp(xg), float(grav[0]), int(case.grav_type))
            else:
                rc = L.orc_set_gravity(self.h, _dp(xg), float(grav[0]), float(grav[1]), float(grav[2]),
                                       case.rho_ref, case.p_ref, case.R_gas, int(case.HB), case.N_bv)
            if rc:
                raise RuntimeError("setting the gravity field failed")

    def gravity_field(self) -> Optional[np.ndarray]:
        """The fields f then g with ghost points, as the reader computes them, or None."""
        grav = getattr(self.case, "gravity", None)
        if grav is None or not any(float(v) != 0.0 for v in grav):
            return None
        n = self.npts_wg
        out = np.empty(2 * n)
        self._L.orc_get_gravity(self.h, _dp(out))
        return out

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self._L.orc_problem_destroy(self.h)
        except Exception:
            pass

    @property
    def npts_wg(self) -> int:
        return int(np.prod([s + 2 * self.g for s in self.size]))

    def u0(self) -> np.ndarray:
        return embed(self.case.u, self.size, self.nvars, self.g)

    def rhs(self, u_wg: np.ndarray, t: float = 0.0) -> np.ndarray:
        """TimeRHSFunctionExplicit at time t (the time matters to time-dependent boundaries)."""
        u = np.ascontiguousarray(u_wg, np.float64).copy()
        out = np.zeros_like(u)
        self._L.orc_set_time(self.h, float(t))
        if self._L.orc_rhs(self.h, _dp(u), _dp(out)):
            raise RuntimeError("orc_rhs failed (a zero pivot, or a configuration the oracle does not restate)")
        return out

    def hyperbolic(self, u_wg: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_wg, np.float64).copy()
        self._L.orc_apply_bc(self.h, _dp(u))
        out = np.zeros_like(u)
        if self._L.orc_hyperbolic(self.h, _dp(u), _dp(out)):
            raise RuntimeError("orc_hyperbolic failed")
        return out

    def source(self, u_wg: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u_wg, np.float64).copy()
        self._L.orc_apply_bc(self.h, _dp(u))
        out = np.zeros_like(u)
        self._L.orc_source(self.h, _dp(u), _dp(out))
        return out

    def cfl(self, u_wg: np.ndarray, dt: Optional[float] = None) -> float:
        u = np.ascontiguousarray(u_wg, np.float64)
        return float(self._L.orc_cfl(self.h, _dp(u), float(self.case.dt if dt is None else dt)))

    def apply_bc(self, u_wg: np.ndarray, t: float = 0.0) -> np.ndarray:
        u = np.ascontiguousarray(u_wg, np.float64).copy()
        self._L.orc_set_time(self.h, float(t))
        self._L.orc_apply_bc(self.h, _dp(u))
        return u

    def rk(self, u_wg: np.ndarray, nsteps: int, dt: Optional[float] = None, scheme: Optional[str] = None,
           t0: float = 0.0):
        """nsteps steps of TimeRK from time t0 (stage times t + c_s dt)."""
        scheme = scheme or self.case.time_scheme_type
        ns, A, b = RK_TABLES[scheme]
        A = np.asarray(A, np.float64)
        b = np.asarray(b, np.float64)
        u = np.ascontiguousarray(u_wg, np.float64).copy()
        self._L.orc_set_time(self.h, float(t0))
        if self._L.orc_rk(self.h, ns, _dp(A), _dp(b), _dp(u), float(self.case.dt if dt is None else dt),
                          int(nsteps)):
            raise RuntimeError("orc_rk failed")
        return u


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def threads() -> int:
    return int(lib().orc_get_threads())


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "HyPar")) and os.path.exists(os.path.join(REF_DIR, "ref_rhs_harness"))


def read_harness_dump(path: str):
    with open(path, "rb") as f:
        buf = f.read()
    ndims, nvars, g = np.frombuffer(buf, np.int32, 3, 0)
    dims = np.frombuffer(buf, np.int32, ndims, 12)
    off = 12 + 4 * int(ndims)
    nx = int(sum(int(d) + 2 * int(g) for d in dims))
    dxinv = np.frombuffer(buf, np.float64, nx, off); off += 8 * nx
    n = int(np.prod([int(d) + 2 * int(g) for d in dims])) * int(nvars)
    u_in = np.frombuffer(buf, np.float64, n, off); off += 8 * n
    u_bc = np.frombuffer(buf, np.float64, n, off); off += 8 * n
    rhs = np.frombuffer(buf, np.float64, n, off); off += 8 * n
    cfl = float(np.frombuffer(buf, np.float64, 1, off)[0]) if len(buf) >= off + 8 else None
    return {"dims": dims.copy(), "nvars": int(nvars), "g": int(g), "dxinv": dxinv.copy(),
            "u_in": u_in.copy(), "u_bc": u_bc.copy(), "rhs": rhs.copy(), "cfl": cfl}
