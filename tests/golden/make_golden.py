"""Regenerate the golden fixtures in this directory from the REFERENCE HyPar.

Runs the reference CPU build (oracle/_ref/HyPar and oracle/_ref/ref_rhs_harness,
compiled from the reference sources by oracle/Makefile.ref) on small input
decks written by hypar_gb300.cases, single-threaded (OMP_NUM_THREADS=1: the
reference's OpenMP build races on shared scratch in
WENOFifthOrderCalculateWeightsCharJS), and stores, per case, the initial
interior solution, the reference right-hand side of that state (interior), the
reference solution after n_iter Runge-Kutta steps (op.bin), its CFL, and the
conservation errors and function counts it wrote (conservation.dat,
function_counts.dat); for OUTPUTS the header lines and numbers of its text and
Tecplot solution files; for ENSEMBLES every member's op_<k>.bin.

    make -f oracle/Makefile.ref REF=<hypar source tree> -j8
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hypar_gb300 import cases as C  # noqa: E402
import oracle as O  # noqa: E402

CASES = {
    "sod64_comp_roe": lambda: C.sod(64, n_iter=20, dt=1e-3),
    "sod64_char_llf_ssprk3": lambda: C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                           upwinding="llf-char", scheme="ssprk3"),
    "sod64_char_rf": lambda: C.sod(64, n_iter=20, dt=1e-3, interp="characteristic", upwinding="rf-char"),
    "vortex24_char_roe_ssprk3": lambda: C.vortex(24, n_iter=5, dt=0.02),
    "vortex24_comp_llf_rk4": lambda: C.vortex(24, n_iter=5, dt=0.02, interp="components",
                                              upwinding="llf-char", scheme="44"),
    "vortex24_char_rf_rk22": lambda: C.vortex(24, n_iter=5, dt=0.02, upwinding="rf-char", scheme="22"),
    "tgv12_comp_roe_rk4": lambda: C.tgv(12, n_iter=3, dt=0.02),
    "tgv12_char_llf_rk33": lambda: C.tgv(12, n_iter=3, dt=0.02, interp="characteristic",
                                         upwinding="llf-char", scheme="33"),
    # the other WENO5 weight formulations (weno.inp mapped / borges / yc / no_limiting)
    "sod64_comp_roe_mapped": lambda: _w(C.sod(64, n_iter=20, dt=1e-3), "mapped"),
    "sod64_char_llf_borges": lambda: _w(C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                              upwinding="llf-char"), "borges"),
    "vortex24_char_roe_yc_ssprk3": lambda: _w(C.vortex(24, n_iter=5, dt=0.02), "yc"),
    "vortex24_comp_llf_none_rk4": lambda: _w(C.vortex(24, n_iter=5, dt=0.02, interp="components",
                                                      upwinding="llf-char", scheme="44"), "none"),
    "tgv12_char_rf_mapped_rk4": lambda: _w(C.tgv(12, n_iter=3, dt=0.02, interp="characteristic",
                                                 upwinding="rf-char"), "mapped"),
    "tgv12_comp_roe_borges_rk4": lambda: _w(C.tgv(12, n_iter=3, dt=0.02), "borges"),
    # wall, inflow / outflow and Dirichlet boundaries (applied in memory before every stage)
    "vortex24_char_roe_slipwall": lambda: _b(C.vortex(24, n_iter=5, dt=0.02), {
        (1, 1): ("slip-wall", [0.0, 0.0]), (1, -1): ("slip-wall", [0.0, 0.0])}),
    "vortex24_comp_llf_subsonic_io_rk4": lambda: _b(C.vortex(24, n_iter=5, dt=0.02, interp="components",
                                                             upwinding="llf-char", scheme="44"), {
        (0, 1): ("subsonic-inflow", [1.0, 0.5, 0.0]), (0, -1): ("subsonic-outflow", [1.0])}),
    "vortex24_comp_roe_supersonic_dirichlet": lambda: _b(C.vortex(24, n_iter=5, dt=0.02, interp="components"), {
        (0, 1): ("supersonic-inflow", [1.0, 0.5, 0.0, 1.0]), (0, -1): ("supersonic-outflow", []),
        (1, 1): ("dirichlet", [1.0, 0.5, 0.0, 2.625]), (1, -1): ("dirichlet", [1.0, 0.5, 0.0, 2.625])}),
    "tgv12_comp_roe_noslip_rk4": lambda: _b(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05), {
        (2, 1): ("noslip-wall", [0.0, 0.0, 0.0]), (2, -1): ("noslip-wall", [0.0, 0.0, 0.0])}),
    "tgv12_char_llf_slipwall_io_rk4": lambda: _b(C.tgv(12, n_iter=3, dt=0.02, interp="characteristic",
                                                      upwinding="llf-char", perturb=0.05), {
        (0, 1): ("subsonic-inflow", [1.0, 0.1, 0.0, 0.0]), (0, -1): ("subsonic-outflow", [1.0 / 1.4]),
        (1, 1): ("slip-wall", [0.0, 0.0, 0.0]), (1, -1): ("slip-wall", [0.0, 0.0, 0.0])}),
    # Rusanov upwinding (Euler1D and NavierStokes3D offer it)
    "sod64_comp_rusanov": lambda: C.sod(64, n_iter=20, dt=1e-3, upwinding="rusanov"),
    "sod64_char_rusanov_ssprk3": lambda: C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                               upwinding="rusanov", scheme="ssprk3"),
    "tgv12_comp_rusanov_rk4": lambda: C.tgv(12, n_iter=3, dt=0.02, upwinding="rusanov", perturb=0.05),
    "tgv12_char_rusanov_rk4": lambda: C.tgv(12, n_iter=3, dt=0.02, interp="characteristic", upwinding="rusanov",
                                            perturb=0.05),
    "rtb12_comp_rusanov_yc_ssprk3": lambda: C.rising_thermal_bubble(12, n_iter=3, dt=0.05),
    "rtb12_char_rusanov_js_rk4": lambda: C.rising_thermal_bubble(12, n_iter=3, dt=0.05, interp="characteristic",
                                                                 weights="js", scheme="44", perturb=0.02),
    "rtb12_comp_rusanov_none_hb1": lambda: C.rising_thermal_bubble(12, n_iter=3, dt=0.05, weights="none", HB=1,
                                                                   perturb=0.02),
    "rtb12_char_rusanov_mapped_hb3z": lambda: _g(C.rising_thermal_bubble(12, n_iter=3, dt=0.05,
                                                                          interp="characteristic", weights="mapped",
                                                                          perturb=0.02),
                                                 (0.0, 0.0, 9.8), 3, 0.01),
    "rtb12_comp_rusanov_yc_stir": lambda: _stir(C.rising_thermal_bubble(12, n_iter=3, dt=0.05, perturb=0.02)),
    "rtb12_char_rusanov_js_stir_rk4": lambda: _stir(C.rising_thermal_bubble(12, n_iter=3, dt=0.05,
                                                                            interp="characteristic", weights="js",
                                                                            scheme="44", perturb=0.02)),
    "rtb12_char_rusanov_borges_hb3z_stir": lambda: _stir(_g(C.rising_thermal_bubble(12, n_iter=3, dt=0.05,
                                                                                     interp="characteristic",
                                                                                     weights="borges"),
                                                            (0.0, 0.0, 9.8), 3, 0.01)),
    "sod64_crweno_roe": lambda: _cr(C.sod(64, n_iter=20, dt=1e-3)),
    "sod64_crweno_llf_ssprk3": lambda: _cr(C.sod(64, n_iter=20, dt=1e-3, upwinding="llf-char", scheme="ssprk3")),
    "sod64_crweno_none_rusanov": lambda: _w(_cr(C.sod(64, n_iter=20, dt=1e-3, upwinding="rusanov")), "none"),
    "vortex24_crweno_roe": lambda: _cr(C.vortex(24, n_iter=4, dt=0.02, interp="components")),
    "vortex24_crweno_rf_mapped": lambda: _w(_cr(C.vortex(24, n_iter=4, dt=0.02, interp="components",
                                                          upwinding="rf-char")), "mapped"),
    "vortex24_crweno_llf_yc_slipwall": lambda: _w(_b(_cr(C.vortex(24, n_iter=4, dt=0.02, interp="components",
                                                                   upwinding="llf-char")),
                                                     {(1, 1): ("slip-wall", [0.0, 0.0]),
                                                      (1, -1): ("slip-wall", [0.0, 0.0])}), "yc"),
    "tgv12_crweno_roe_rk4": lambda: _cr(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05)),
    "tgv12_crweno_rusanov_borges": lambda: _w(_cr(C.tgv(12, n_iter=3, dt=0.02, upwinding="rusanov",
                                                         perturb=0.05)), "borges"),
    "sod64_crweno_char_roe": lambda: _cr(C.sod(64, n_iter=20, dt=1e-3, interp="characteristic")),
    "sod64_crweno_char_llf_yc": lambda: _w(_cr(C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                                      upwinding="llf-char", scheme="ssprk3")), "yc"),
    "vortex24_crweno_char_roe": lambda: _cr(C.vortex(24, n_iter=4, dt=0.02)),
    "vortex24_crweno_char_rf_mapped_slipwall": lambda: _w(_b(_cr(C.vortex(24, n_iter=4, dt=0.02,
                                                                          upwinding="rf-char")),
                                                             {(1, 1): ("slip-wall", [0.0, 0.0]),
                                                              (1, -1): ("slip-wall", [0.0, 0.0])}), "mapped"),
    "tgv12_crweno_char_roe_rk4": lambda: _cr(C.tgv(12, n_iter=3, dt=0.02, interp="characteristic", perturb=0.05)),
    "tgv12_crweno_char_rusanov_none": lambda: _w(_cr(C.tgv(12, n_iter=3, dt=0.02, interp="characteristic",
                                                            upwinding="rusanov", perturb=0.05)), "none"),
    "rtb12_comp_rusanov_visc_stir": lambda: _visc(_stir(C.rising_thermal_bubble(12, n_iter=3, dt=0.05,
                                                                                 perturb=0.02)), 100.0),
    "vortex24_crweno_char_roe_subsonic_io": lambda: _b(_cr(C.vortex(24, n_iter=4, dt=0.02)),
                                                       {(0, 1): ("subsonic-inflow", [1.0, 0.5, 0.0]),
                                                        (0, -1): ("subsonic-outflow", [1.0 / 1.4])}),
    "strat64_grav0_roe_comp": lambda: C.stratified_1d(64, n_iter=10),
    "strat64_grav0_llf_char_yc_ssprk3": lambda: _w(C.stratified_1d(64, n_iter=10, interp="characteristic",
                                                                    upwinding="llf-char", scheme="ssprk3"), "yc"),
    "strat64_grav1_roe_char": lambda: C.stratified_1d(64, n_iter=10, grav_type=1, interp="characteristic"),
    "strat64_grav1_llf_comp_mapped": lambda: _w(C.stratified_1d(64, n_iter=10, grav_type=1, upwinding="llf-char",
                                                                 g=2.0), "mapped"),
    "sod64_grav_roe_comp": lambda: _g1(C.sod(64, n_iter=20, dt=1e-3), 1.0),
    # gravity with CRWENO5: the source function solved with the flux's weights
    "strat64_crweno_grav0_roe_comp": lambda: _cr(C.stratified_1d(64, n_iter=10, perturb=0.05)),
    "strat64_crweno_grav1_roe_char_mapped": lambda: _w(_cr(C.stratified_1d(64, n_iter=10, grav_type=1,
                                                                           interp="characteristic",
                                                                           perturb=0.05)), "mapped"),
    "sod64_crweno_grav_llf_char": lambda: _g1(_cr(C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                                        upwinding="llf-char")), 1.0),
    # slip walls in 1-D (BCSlipWall.c's Euler1D branch), with and without gravity
    "sod64_slipwall_comp_roe": lambda: _b(C.sod(64, n_iter=20, dt=1e-3),
                                          {(0, 1): ("slip-wall", [0.0]), (0, -1): ("slip-wall", [0.1])}),
    "sod64_crweno_grav_slipwall_char_roe_mapped": lambda: _w(_b(_g1(_cr(C.sod(64, n_iter=20, dt=1e-3,
                                                                            interp="characteristic")), 1.0),
                                                                {(0, 1): ("slip-wall", [0.0]),
                                                                 (0, -1): ("slip-wall", [0.0])}), "mapped"),
    "rtb12_crweno_comp_rusanov_stir": lambda: _stir(_cr(C.rising_thermal_bubble(12, n_iter=3, dt=0.05,
                                                                                perturb=0.02))),
    "rtb12_crweno_char_rusanov_hb3z_stir": lambda: _stir(_g(_cr(C.rising_thermal_bubble(
        12, n_iter=3, dt=0.05, interp="characteristic", perturb=0.02)), (0.0, 0.0, 9.8), 3, 0.01)),
    # the conservation check (solver.inp conservation_check yes): boundary fluxes through
    # extrapolate / wall / inflow faces, a source (gravity), the viscous term
    "sod64_cons_comp_roe": lambda: _cons(C.sod(64, n_iter=20, dt=1e-3)),
    "sod64_cons_crweno_char_llf": lambda: _cons(_cr(C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                                         upwinding="llf-char"))),
    "strat64_cons_grav1_roe_char": lambda: _cons(C.stratified_1d(64, n_iter=10, grav_type=1,
                                                                 interp="characteristic")),
    "vortex24_cons_comp_roe_subsonic_io": lambda: _cons(_b(C.vortex(24, n_iter=5, dt=0.02, interp="components"), {
        (0, 1): ("subsonic-inflow", [1.0, 0.5, 0.0]), (0, -1): ("subsonic-outflow", [1.0])})),
    "vortex24_cons_char_roe_slipwall": lambda: _cons(_b(C.vortex(24, n_iter=5, dt=0.02), {
        (1, 1): ("slip-wall", [0.0, 0.0]), (1, -1): ("slip-wall", [0.0, 0.0])})),
    "tgv12_cons_comp_roe_noslip": lambda: _cons(_b(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05), {
        (2, 1): ("noslip-wall", [0.0, 0.0, 0.0]), (2, -1): ("noslip-wall", [0.0, 0.0, 0.0])})),
    "rtb12_cons_comp_rusanov_yc": lambda: _cons(C.rising_thermal_bubble(12, n_iter=3, dt=0.05, perturb=0.02)),
    # subsonic "ambivalent" faces: inflow or outflow point by point by the sign of the
    # extrapolated face velocity (random velocities make both occur on every face)
    "vortex24_char_roe_ambivalent": lambda: _b(_stir2(C.vortex(24, n_iter=4, dt=0.01)), {
        (0, 1): ("subsonic-ambivalent", [1.0, 0.5, 0.0, 1.0]), (0, -1): ("subsonic-ambivalent", [1.0, 0.5, 0.0, 1.0]),
        (1, 1): ("subsonic-ambivalent", [1.1, 0.0, 0.2, 0.9]), (1, -1): ("subsonic-ambivalent", [0.9, 0.1, 0.0, 1.1])}),
    # thermal walls (NavierStokes3D): the pressure from the extrapolated density and a wall
    # temperature read from file, at the time level of each stage's time
    "tgv12_comp_roe_thermal_noslip_rk4": lambda: _thermal(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05),
                                                          "thermal-noslip-wall", [0.0, 0.0, 0.0]),
    "tgv12_char_llf_thermal_slip_ssprk3": lambda: _thermal(C.tgv(12, n_iter=3, dt=0.02, interp="characteristic",
                                                                 upwinding="llf-char", scheme="ssprk3",
                                                                 perturb=0.05),
                                                           "thermal-slip-wall", [0.0, 0.05, 0.0], dim=1),
    "tgv12_comp_llf_ambivalent_rk4": lambda: _b(_stir(C.tgv(12, n_iter=3, dt=0.02, upwinding="llf-char",
                                                            perturb=0.05), speed=0.3), {
        (2, 1): ("subsonic-ambivalent", [1.0, 0.0, 0.0, 0.1, 1.0 / 1.4]),
        (2, -1): ("subsonic-ambivalent", [1.0, 0.0, 0.0, -0.1, 1.0 / 1.4])}),
    # sponge zones: a relaxation source over boxes of interior points (two overlapping
    # in the 2-D deck), beside periodic and extrapolate faces
    # NavierStokes3D viscous term with par_space_scheme 2 (first-order one-sided
    # derivatives, FirstDerivativeFirstOrder.c)
    "tgv12_comp_roe_par2_rk4": lambda: _par2(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05)),
    "rtb12_comp_rusanov_visc_par2": lambda: _par2(_visc(C.rising_thermal_bubble(12, n_iter=3, dt=0.05,
                                                                               perturb=0.02), 500.0)),
    # Steger-Warming flux vector splitting (Euler1D, Euler2D), component-wise and
    # characteristic; the Sod tube crosses Mach 1 nowhere, the stirred vortex does
    "sod64_comp_swfs": lambda: C.sod(64, n_iter=20, dt=1e-3, upwinding="steger-warming"),
    "sod64_char_swfs_ssprk3": lambda: C.sod(64, n_iter=20, dt=1e-3, interp="characteristic",
                                            upwinding="steger-warming", scheme="ssprk3"),
    "vortex24_comp_swfs_rk4": lambda: C.vortex(24, n_iter=5, dt=0.02, interp="components",
                                               upwinding="steger-warming", scheme="44"),
    "vortex24_char_swfs_ssprk3": lambda: _boost(C.vortex(24, n_iter=5, dt=0.01, upwinding="steger-warming"),
                                                1.0),
    # three points along one dimension (the quasi-2-D NavierStokes3D decks run with
    # size N M 3): ghost layers as deep as the line, every ghost a folded interior point
    "tgv12x12x3_comp_roe_rk4": lambda: _slab(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05), 2, 3),
    "rtb12x12x3_comp_rusanov_yc": lambda: _slab(C.rising_thermal_bubble(12, n_iter=3, dt=0.05, perturb=0.02), 2, 3),
    "vortex24x3_char_roe_ssprk3": lambda: _slab(C.vortex(24, n_iter=5, dt=0.02), 1, 3, start=11),
    # time_scheme euler (HyPar's default time integrator, TimeForwardEuler.c)
    "sod64_comp_roe_euler": lambda: C.sod(64, n_iter=20, dt=1e-3, scheme="euler"),
    "vortex24_char_llf_euler": lambda: C.vortex(24, n_iter=5, dt=0.01, upwinding="llf-char", scheme="euler"),
    "sod64_comp_roe_sponge": lambda: _sponge(C.sod(64, n_iter=20, dt=1e-3), [
        (0, -1, [(0.75, 1.5)], [0.2, 0.1, 0.3])]),
    "vortex24_char_roe_sponge_ssprk3": lambda: _sponge(C.vortex(24, n_iter=5, dt=0.02, scheme="ssprk3"), [
        (0, -1, [(6.0, 9.6), (-1.0, 11.0)], [1.1, 0.4, 0.05, 2.7]),
        (1, 1, [(-1.0, 11.0), (0.0, 2.5)], [0.9, 0.55, -0.05, 2.5])]),
    "tgv12_comp_roe_sponge_rk4": lambda: _sponge(C.tgv(12, n_iter=3, dt=0.02, perturb=0.05), [
        (2, 1, [(-1.0, 7.0), (-1.0, 7.0), (0.0, 2.0)], [1.05, 0.1, 0.0, -0.1, 1.9])]),
    # turbulent supersonic inflow (NavierStokes3D): a supersonic mean inflow with velocity
    # fluctuations from inflow data whose slice advances with the mean flow (slice 0 to 1
    # inside the run), supersonic outflow opposite
    "tgv12_comp_llf_turbulent_inflow_rk4": lambda: _turb(C.tgv(12, n_iter=3, dt=0.02, upwinding="llf-char",
                                                                perturb=0.05)),
    "tgv12_char_rusanov_turbulent_inflow_ssprk3": lambda: _turb(C.tgv(12, n_iter=3, dt=0.02,
                                                                       interp="characteristic",
                                                                       upwinding="rusanov", scheme="ssprk3",
                                                                       perturb=0.05), dim=1),
}


def _turb(case, dim=0, nslices=64, speed=2.0, seed=17):
    """Turbulent supersonic inflow on the low face along `dim` (mean velocity `speed`
    along it), supersonic outflow on the high face; random fluctuations of 0.05."""
    rng = np.random.default_rng(seed)
    size = [nslices if e == dim else case.size[e] for e in range(3)]
    data = np.zeros((size[2], size[1], size[0], case.nvars))
    data[..., 0] = 1.0 + 0.1 * rng.standard_normal(data.shape[:3])
    data[..., 1:4] = 0.05 * rng.standard_normal(data.shape[:3] + (3,))
    data[..., 4] = 2.0 + 0.1 * rng.standard_normal(data.shape[:3])
    vel = [0.0, 0.0, 0.0]
    vel[dim] = speed
    case.bcs = {(dim, 1): ("turbulent-supersonic-inflow", [1.0] + vel + [1.0 / 1.4], (nslices, data.reshape(-1))),
                (dim, -1): ("supersonic-outflow", [])}
    return case


def _slab(case, dim, n, start=0):
    """n grid planes of a deck along dimension dim, from plane `start`."""
    shape = [s for s in reversed(case.size)] + [case.nvars]
    u = case.u.reshape(shape)
    sl = [slice(None)] * len(shape)
    sl[len(case.size) - 1 - dim] = slice(start, start + n)
    case.u = np.ascontiguousarray(u[tuple(sl)]).reshape(-1, case.nvars)
    case.size = list(case.size)
    case.size[dim] = n
    case.x = list(case.x)
    case.x[dim] = np.asarray(case.x[dim])[start:start + n]
    return case


def _par2(case):
    """The deck with par_space_scheme 2."""
    case.par_scheme = "2"
    return case


def _sponge(case, sponges):
    """The deck with sponge zones [(dim, face, box per dim, reference state)]."""
    case.sponges = sponges
    return case


def _thermal(case, kind, vel, dim=2):
    """Thermal walls on both faces along `dim` of a 3-D deck: two time levels of the wall
    temperature (t = 0 and t = 0.03, so that a 3-step run with dt = 0.02 changes level
    inside a step), varying over the face."""
    n = case.size
    other = [e for e in range(3) if e != dim]
    a = np.arange(n[other[0]]) / n[other[0]]
    b = np.arange(n[other[1]]) / n[other[1]]
    B, A = np.meshgrid(b, a, indexing="ij")  # [index along other[1], index along other[0]]
    levels = [0.70 + 0.02 * np.sin(2 * np.pi * A) * np.cos(2 * np.pi * B),
              0.74 + 0.01 * np.cos(2 * np.pi * A)]
    bcs = {}
    for face, shift in ((1, 0.0), (-1, 0.01)):
        field = np.stack([lv + shift for lv in levels])  # [level, other[1], other[0]]
        # the reference's layout: dimension 0 fastest, the time level along `dim`
        if dim == 2:
            arr = field
        elif dim == 1:
            arr = np.transpose(field, (1, 0, 2))  # [z, level, x]
        else:
            arr = np.transpose(field, (1, 2, 0))  # [z, y, level]
        bcs[(dim, face)] = (kind, vel, ([0.0, 0.03], arr.reshape(-1)))
    case.bcs = bcs
    return case


def _boost(case, du):
    """A 2-D deck with du added to every x-velocity at the same pressure (the vortex
    then moves at Mach 0.5 to 2 across the grid)."""
    u = case.u
    rho = u[:, 0]
    vx, vy = u[:, 1] / rho, u[:, 2] / rho
    P = (u[:, 3] - 0.5 * rho * (vx * vx + vy * vy)) * (case.gamma - 1.0)
    vx = vx + du
    u[:, 1] = rho * vx
    u[:, 3] = P / (case.gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy)
    return case


def _stir2(case, speed=0.3, seed=13):
    """Random velocities of about `speed` on a 2-D deck's state, the energy kept."""
    rng = np.random.default_rng(seed)
    case.u[:, 1:3] = speed * rng.standard_normal((case.u.shape[0], 2)) * case.u[:, :1]
    return case


def _cons(case):
    """The deck with solver.inp conservation_check yes."""
    case.conservation_check = True
    return case


def _g1(case, g):
    """An Euler1D deck in the gravity field exp(-g x) (gravity_type 0)."""
    case.gravity, case.grav_type = (g, 0.0, 0.0), 0
    return case


def _visc(case, Re):
    """NavierStokes3D deck with the viscous term (Re, Pr 0.72, Minf 1)."""
    case.Re, case.Pr, case.Minf = Re, 0.72, 1.0
    return case


def _cr(case):
    """The deck with hyp_space_scheme crweno5 (compact WENO5)."""
    case.hyp_scheme = "crweno5"
    return case


def _stir(case, speed=0.5, seed=11):
    """Random velocities of about `speed` on the deck's state (density unchanged)."""
    rng = np.random.default_rng(seed)
    case.u[:, 1:4] = speed * rng.standard_normal((case.u.shape[0], 3)) * case.u[:, :1]
    return case


def _g(case, gravity, HB, N_bv):
    case.gravity, case.HB, case.N_bv = gravity, HB, N_bv
    return case


def _b(case, bcs):
    case.bcs = bcs
    return case


def _w(case, weights):
    case.weights = weights
    return case


def _fmt(case, fmt, overwrite="yes"):
    """The deck with solver.inp op_file_format fmt (and op_overwrite)."""
    case.op_format, case.op_overwrite = fmt, overwrite
    return case


# solution files in the text and Tecplot formats (op_file_format): file name -> deck
OUTPUTS = {
    "out_sod64_text": (lambda: _fmt(C.sod(64, n_iter=10, dt=1e-3), "text"), ["op.dat"]),
    "out_vortex24_tecplot2d": (lambda: _fmt(C.vortex(24, n_iter=3, dt=0.02), "tecplot2d", "no"),
                               ["op_00000.dat", "op_00001.dat"]),
    "out_tgv8_tecplot3d": (lambda: _fmt(C.tgv(8, n_iter=2, dt=0.02, perturb=0.05), "tecplot3d"), ["op.dat"]),
    "out_vortex16_text": (lambda: _fmt(C.vortex(16, n_iter=2, dt=0.02), "text"), ["op.dat"]),
}


def read_text_output(path):
    """(header lines, numeric table) of a text / Tecplot solution file."""
    header, rows = [], []
    for line in open(path):
        try:
            rows.append([float(t) for t in line.split()])
        except ValueError:
            header.append(line.rstrip("\n"))
    return header, np.array(rows, dtype=np.float64)


ENSEMBLES = {
    "ens3_vortex_char_roe_ssprk3": lambda: C.ensemble_vortex(3, sizes=[16, 24, 20], n_iter=4, seed=7),
}


def main() -> None:
    """python tests/golden/make_golden.py [name ...]: all fixtures, or the named ones."""
    if not O.ref_available():
        raise SystemExit("oracle/_ref is not built (make -f oracle/Makefile.ref)")
    only = set(sys.argv[1:])
    env = dict(os.environ, OMP_NUM_THREADS="1")
    for name, mk in CASES.items():
        if only and name not in only:
            continue
        case = mk()
        with tempfile.TemporaryDirectory() as d:
            case.write(d)
            subprocess.check_call([os.path.join(O.REF_DIR, "ref_rhs_harness"), "dump.bin"], cwd=d,
                                  stdout=subprocess.DEVNULL, env=env)
            dump = O.read_harness_dump(os.path.join(d, "dump.bin"))
            subprocess.check_call([os.path.join(O.REF_DIR, "HyPar")], cwd=d, stdout=subprocess.DEVNULL, env=env)
            op = C.read_op_bin(os.path.join(d, "op.bin"))
            # conservation.dat: sizes, iproc, dt, then the conservation error per variable
            cons = np.array(open(os.path.join(d, "conservation.dat")).read().split()[2 * case.ndims + 1:],
                            dtype=np.float64)
            counts = np.array(open(os.path.join(d, "function_counts.dat")).read().split()[:4], dtype=np.int64)
        rhs = O.interior(dump["rhs"], case.size, case.nvars, 3)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), u0=case.u, rhs=rhs, uN=op["u"],
                            n_iter=case.n_iter, dt=case.dt, cfl=dump["cfl"], cons=cons, counts=counts)
        print(name, rhs.shape, op["u"].shape)
    for name, (mk, files) in OUTPUTS.items():
        if only and name not in only:
            continue
        case = mk()
        case.file_op_iter = case.n_iter if case.op_overwrite == "no" else None
        with tempfile.TemporaryDirectory() as d:
            case.write(d)
            subprocess.check_call([os.path.join(O.REF_DIR, "HyPar")], cwd=d, stdout=subprocess.DEVNULL, env=env)
            out = {}
            for k, f in enumerate(files):
                header, table = read_text_output(os.path.join(d, f))
                out[f"header_{k}"] = np.array(header)
                out[f"table_{k}"] = table
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, [out[f"table_{k}"].shape for k in range(len(files))])
    for name, mk in ENSEMBLES.items():
        if only and name not in only:
            continue
        members = mk()
        with tempfile.TemporaryDirectory() as d:
            C.write_ensemble(members, d)
            subprocess.check_call([os.path.join(O.REF_DIR, "HyPar")], cwd=d, stdout=subprocess.DEVNULL, env=env)
            width = int(math.log10(len(members))) + 1
            outs = {f"uN_{k}": C.read_op_bin(os.path.join(d, f"op_{str(k).zfill(width)}.bin"))["u"]
                    for k in range(len(members))}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), n_iter=members[0].n_iter, dt=members[0].dt, **outs)
        print(name, [v.shape for v in outs.values()])


if __name__ == "__main__":
    main()
