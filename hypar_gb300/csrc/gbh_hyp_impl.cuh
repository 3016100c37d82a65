// gbh_hyp_impl.cuh -- the fused hyperbolic kernel, one launch per direction.
//
// Replaces, for one direction d, HyPar's FFunction -> SetInterpLimiterVar ->
// UFunction -> 4x InterpolateInterfacesHyp -> Upwind -> flux difference chain
// (src/HyParFunctions/HyperbolicFunction.c:75-117 with ReconstructHyperbolic
// :167-222), and, on the last direction of a Runge-Kutta stage, the
// right-hand-side assembly (TimeRHSFunctionExplicit.c:89-92) and the stage
// update of TimeRK (TimeRK.c:126-195).
//
// Each thread walks `seg` consecutive interfaces of one grid line along d,
// keeping a six-cell window (cells j-3..j+2 of interface j-1/2) in registers:
// a cell's flux, Roe-average ingredients and modified state are computed once,
// when the cell enters the window, and the flux difference of cell j-1 is
// formed from the previous interface's flux held in registers, so no interface
// array ever reaches memory.  Ghost cells outside the domain are read through
// the boundary fold (periodic wrap / mirror) or from memory.
#pragma once

#include "gbh_internal.h"

namespace gbh {

__device__ __forceinline__ int fold_index(int i, int N, int lo, int hi) {
  if (i < 0) {
    if (lo == FOLD_PERIODIC) return i + N;
    if (lo == FOLD_MIRROR) return -1 - i;
    return i;
  }
  if (i >= N) {
    if (hi == FOLD_PERIODIC) return i - N;
    if (hi == FOLD_MIRROR) return 2 * N - 1 - i;
    return i;
  }
  return i;
}

// Sound speed of a state (for LLF / RF eigenvalues at the left/right states).
template <int M>
__device__ __forceinline__ double sound_speed(const Prim<M>& q, const PhysParams& pp) {
  return nr_sqrt(pp.gamma * q.P * q.rinv);
}

template <int M>
struct CellAux {
  RoeSide rs;
  double c;
};

template <int M, bool CHAR, int UPW>
struct NeedCC {
  // cell-centre Roe average needed: characteristic WENO (WENOFifthOrderCalculateWeights.c:832),
  // Euler1D upwinding (Euler1DUpwind.c:74, :259), NavierStokes3D Roe (NavierStokes3DUpwind.c:90)
  static constexpr bool value = CHAR || (M == MODEL_EULER1D) || (M == MODEL_NS3D && UPW == UPW_ROE) ||
                                (UPW == UPW_RUS);
};

// Rusanov's wave speed |v_dir| + c of a cell-centre state (NavierStokes3DUpwind.c:392-403);
// Euler1DUpwindRusanov takes c = gamma P / rho, without the square root
// (Euler1DUpwind.c:394-404), which is kept.
template <int M, int DIR>
__device__ __forceinline__ double rusanov_speed(const Prim<M>& q, const PhysParams& pp) {
  const double c2 = pp.gamma * q.P * q.rinv;
  return (M == MODEL_EULER1D ? c2 : nr_sqrt(c2)) + fabs(q.vel[DIR]);
}

// The same for the Roe average of the two cell-centre states (eigen-system E).
template <int M>
__device__ __forceinline__ double rusanov_speed_avg(const Eig& E) {
  return (M == MODEL_EULER1D ? E.a * E.a : E.a) + fabs(E.un);
}

// Upwind flux at one interface from the reconstructed fL, fR, uL, uR and the
// two cell-centre neighbours (their Roe-average ingredients `cl`, `cr` and,
// when CC, the eigen-system `Ecc` of their Roe average).
// kappa: the Rusanov dissipation factor max(g_L, g_R) of the gravity field (1 without gravity).
// ush: when given, uL and uR are relative to ush (and fL, fR relative to some common
// value, which then carries over to fI): every scheme uses the values linearly
// except through the states' own Roe average and sound speeds, which take
// uL + ush and uR + ush.
template <int M, bool CHAR, int UPW, int DIR>
__device__ __forceinline__ void upwind_iface(const double* fL, const double* fR, const double* uL,
                                             const double* uR, const Eig& Ecc, const CellAux<M>& cl,
                                             const CellAux<M>& cr, const PhysParams& pp, double* fI,
                                             double kappa = 1.0, const double* ush = nullptr,
                                             const double* fsh = nullptr) {
  constexpr int NV = ModelTraits<M>::NV;
  auto actual = [&](const double* x, double* y) {
#pragma unroll
    for (int v = 0; v < NV; v++) y[v] = ush ? x[v] + ush[v] : x[v];
  };
  if (UPW == UPW_SWFS) {
    // Steger-Warming (Euler1DUpwind.c:293-362, Euler2DUpwind.c:211-291): by the Mach
    // number of the Roe average of the reconstructed states, fR (below -1), fL (1 and
    // above), or F+(uL) + F-(uR).  In the centre-relative form (ush, fsh: the centre
    // cell's state and flux) the split fluxes are taken of the actual states and the
    // centre flux is subtracted like the other fluxes.
    double aL[NV], aR[NV];
    actual(uL, aL);
    actual(uR, aR);
    const Eig Ea = roe_eig_cons<M, DIR>(aL, aR, pp);
    const double mach = Ea.un / Ea.a;
    if (mach < -1.0) {
#pragma unroll
      for (int v = 0; v < NV; v++) fI[v] = fR[v];
    } else if (mach < 1.0) {
      double fp[NV], fm[NV];
      swfs_half<M, DIR, true>(aL, pp, fp);
      swfs_half<M, DIR, false>(aR, pp, fm);
#pragma unroll
      for (int v = 0; v < NV; v++) fI[v] = fsh ? (fp[v] + fm[v]) - fsh[v] : fp[v] + fm[v];
    } else {
#pragma unroll
      for (int v = 0; v < NV; v++) fI[v] = fL[v];
    }
    return;
  }
  if (UPW == UPW_RUS) {
    // Rusanov (Euler1DUpwind.c:362-424, NavierStokes3DUpwind.c:349-428):
    // fI = (fL+fR)/2 - alpha (uR-uL)/2, alpha = max of |v|+c over the two
    // cell-centre states and their Roe average (times kappa = 1 without gravity)
    const double alpha = kappa * fmax(fmax(cl.c, cr.c), rusanov_speed_avg<M>(Ecc));
#pragma unroll
    for (int v = 0; v < NV; v++) fI[v] = fma(-alpha, 0.5 * (uR[v] - uL[v]), 0.5 * (fL[v] + fR[v]));
    return;
  }
  if (UPW == UPW_ROE) {
    // Roe: fI = (fL+fR)/2 - R|Lambda|L (uR-uL)/2, Roe average of the
    // reconstructed states for Euler2D (Euler2DUpwind.c:39) and of the
    // cell-centre states otherwise; Harten's fix except for Euler1D.
    Eig Eu;
    if (M == MODEL_EULER2D) {
      double aL[NV], aR[NV];
      actual(uL, aL);
      actual(uR, aR);
      Eu = roe_eig_cons<M, DIR>(aL, aR, pp);
    } else {
      Eu = Ecc;
    }
    double ud[NV], w[NV], lam[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) ud[v] = 0.5 * (uR[v] - uL[v]);
    projL<M, DIR>(Eu, pp, ud, w);
    eigvals<M>(Eu.un, Eu.a, lam);
#pragma unroll
    for (int k = 0; k < NV; k++) {
      // Harten's fix (Euler2D, NavierStokes3D); Euler1D: |lambda| times the gravity
      // field's factor (Euler1DUpwind.c:79-82; 1 without gravity)
      const double d = (M != MODEL_EULER1D) ? harten_abs(lam[k]) : kappa * fabs(lam[k]);
      w[k] *= d;
    }
    projR<M, DIR>(Eu, w, ud);
#pragma unroll
    for (int v = 0; v < NV; v++) fI[v] = 0.5 * (fL[v] + fR[v]) - ud[v];
  } else {
    // LLF / RF in the Roe eigenbasis (Euler2DUpwind.c:68-210 and the Euler1D /
    // NavierStokes3D counterparts): alpha = max |lambda| over left, average, right.
    Eig Eu;
    double unL, cL, unR, cR;
    if (M == MODEL_EULER1D) {
      Eu = Ecc;
      unL = cl.rs.vel[DIR];
      cL = cl.c;
      unR = cr.rs.vel[DIR];
      cR = cr.c;
    } else {
      double aL[NV], aR[NV];
      actual(uL, aL);
      actual(uR, aR);
      Prim<M> qL = to_prim<M>(aL, pp), qR = to_prim<M>(aR, pp);
      Eu = roe_eig<M, DIR>(roe_side<M>(qL), roe_side<M>(qR), pp);
      unL = qL.vel[DIR];
      cL = sound_speed<M>(qL, pp);
      unR = qR.vel[DIR];
      cR = sound_speed<M>(qR, pp);
    }
    double lamL[NV], lamC[NV], lamR[NV];
    eigvals<M>(unL, cL, lamL);
    eigvals<M>(Eu.un, Eu.a, lamC);
    eigvals<M>(unR, cR, lamR);
    double fc[NV];
    if (UPW == UPW_LLF) {
      double sf[NV], du[NV], ws[NV], wd[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) {
        sf[v] = fL[v] + fR[v];
        du[v] = uL[v] - uR[v];
      }
      projL<M, DIR>(Eu, pp, sf, ws);
      projL<M, DIR>(Eu, pp, du, wd);
#pragma unroll
      for (int k = 0; k < NV; k++) {
        double al = fmax(fmax(fabs(lamL[k]), fabs(lamC[k])), fabs(lamR[k]));
        if (M == MODEL_EULER1D) al = kappa * al;  // Euler1DUpwind.c:268
        fc[k] = 0.5 * fma(al, wd[k], ws[k]);
      }
    } else {
      double fcL[NV], fcR[NV], du[NV], wd[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) du[v] = uL[v] - uR[v];
      projL<M, DIR>(Eu, pp, fL, fcL);
      projL<M, DIR>(Eu, pp, fR, fcR);
      projL<M, DIR>(Eu, pp, du, wd);
#pragma unroll
      for (int k = 0; k < NV; k++) {
        if (lamL[k] > 0 && lamC[k] > 0 && lamR[k] > 0) {
          fc[k] = fcL[k];
        } else if (lamL[k] < 0 && lamC[k] < 0 && lamR[k] < 0) {
          fc[k] = fcR[k];
        } else {
          double al = fmax(fmax(fabs(lamL[k]), fabs(lamC[k])), fabs(lamR[k]));
          fc[k] = 0.5 * fma(al, wd[k], fcL[k] + fcR[k]);
        }
      }
    }
    projR<M, DIR>(Eu, fc, fI);
  }
}

// Upwinding from characteristic reconstructions xfL, xfR, xuL, xuR in the
// basis of the cell-centre Roe average Ecc (the characteristic-WENO basis).
// When the upwind scheme uses the same eigen-system (Roe for Euler1D and
// NavierStokes3D, which average the cell-centre states, NavierStokes3DUpwind.c:90,
// Euler1DUpwind.c:74; LLF/RF for Euler1D, Euler1DUpwind.c:259) the projections
// cancel (L R = I): fI = R ((xfL+xfR)/2 - |Lambda| (xuR-xuL)/2).  Otherwise the
// conserved interface values are rebuilt (fL+fR in one projection) and the
// conserved-variable upwinding applies.
// ush: as for upwind_iface, the characteristic u values are those of u - ush.
template <int M, int UPW, int DIR>
__device__ __forceinline__ void upwind_char(const double* xfL, const double* xfR, const double* xuL,
                                            const double* xuR, const Eig& Ecc, const CellAux<M>& cl,
                                            const CellAux<M>& cr, const PhysParams& pp, double* fI,
                                            double kappa = 1.0, const double* ush = nullptr,
                                            const double* fsh = nullptr) {
  constexpr int NV = ModelTraits<M>::NV;
  if (UPW == UPW_RUS) {
    // a scalar dissipation commutes with the basis: fI = R ((xfL+xfR)/2 - alpha (xuR-xuL)/2)
    const double alpha = kappa * fmax(fmax(cl.c, cr.c), rusanov_speed_avg<M>(Ecc));
    double fc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) fc[k] = fma(-alpha, 0.5 * (xuR[k] - xuL[k]), 0.5 * (xfL[k] + xfR[k]));
    projR<M, DIR>(Ecc, fc, fI);
    return;
  }
  constexpr bool SAME_BASIS = UPW != UPW_SWFS && ((M == MODEL_EULER1D) || (M == MODEL_NS3D && UPW == UPW_ROE));
  if (SAME_BASIS) {
    double lamC[NV], fc[NV];
    eigvals<M>(Ecc.un, Ecc.a, lamC);
    if (UPW == UPW_ROE) {
#pragma unroll
      for (int k = 0; k < NV; k++) {
        const double d = (M != MODEL_EULER1D) ? harten_abs(lamC[k]) : kappa * fabs(lamC[k]);
        fc[k] = 0.5 * fma(-d, xuR[k] - xuL[k], xfL[k] + xfR[k]);
      }
    } else {
      double lamL[NV], lamR[NV];
      eigvals<M>(cl.rs.vel[DIR], cl.c, lamL);
      eigvals<M>(cr.rs.vel[DIR], cr.c, lamR);
#pragma unroll
      for (int k = 0; k < NV; k++) {
        double al = fmax(fmax(fabs(lamL[k]), fabs(lamC[k])), fabs(lamR[k]));
        if (M == MODEL_EULER1D) al = kappa * al;
        double llf = 0.5 * fma(al, xuL[k] - xuR[k], xfL[k] + xfR[k]);
        if (UPW == UPW_RF) {
          if (lamL[k] > 0 && lamC[k] > 0 && lamR[k] > 0) llf = xfL[k];
          else if (lamL[k] < 0 && lamC[k] < 0 && lamR[k] < 0) llf = xfR[k];
        }
        fc[k] = llf;
      }
    }
    projR<M, DIR>(Ecc, fc, fI);
    return;
  }
  double uL[NV], uR[NV];
  projR<M, DIR>(Ecc, xuL, uL);
  projR<M, DIR>(Ecc, xuR, uR);
  if (UPW == UPW_ROE) {
    // Euler2D: Roe average of the reconstructed states (Euler2DUpwind.c:39)
    double xs[NV], fs[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) xs[k] = xfL[k] + xfR[k];
    projR<M, DIR>(Ecc, xs, fs);
    double aL[NV], aR[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      aL[v] = ush ? uL[v] + ush[v] : uL[v];
      aR[v] = ush ? uR[v] + ush[v] : uR[v];
    }
    Eig Eu = roe_eig_cons<M, DIR>(aL, aR, pp);
    double ud[NV], w[NV], lam[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) ud[v] = 0.5 * (uR[v] - uL[v]);
    projL<M, DIR>(Eu, pp, ud, w);
    eigvals<M>(Eu.un, Eu.a, lam);
#pragma unroll
    for (int k = 0; k < NV; k++) w[k] *= harten_abs(lam[k]);
    projR<M, DIR>(Eu, w, ud);
#pragma unroll
    for (int v = 0; v < NV; v++) fI[v] = fma(0.5, fs[v], -ud[v]);
  } else {
    double fL[NV], fR[NV];
    projR<M, DIR>(Ecc, xfL, fL);
    projR<M, DIR>(Ecc, xfR, fR);
    upwind_iface<M, true, UPW, DIR>(fL, fR, uL, uR, Ecc, cl, cr, pp, fI, 1.0, ush, fsh);
  }
}

// Jiang-Shu pair (the benchmark path) or, in the kernels instantiated with
// ALTW, the pair with the weight formulation selected at run time.
// C0: the window is relative to its centre cell (w[2] = v[2] = 0; the alternative
// formulations read the zeros, which the caller stores).
template <bool ALTW, bool C0 = false>
__device__ __forceinline__ void wpair(const double* w, const double* v, double eps4, int wtype, double& oL,
                                      double& oR) {
  if (ALTW) weno5_pair_alt(w, v, eps4, wtype, oL, oR);
  else if (C0) weno5_pair_c0(w, v, eps4, oL, oR);
  else weno5_pair(w, v, eps4, oL, oR);
}

// The conservation check's boundary fluxes: the flux leaving through face 0
// (-F at interface 0) and face N (+F at interface N) of grid line `line`, times the
// stage's dt b_s, added into that line's accumulators (one thread owns each).
template <int NV>
__device__ __forceinline__ void boundary_flux(const StageEpi& ep, int I, int N, long long line, long long ntrans,
                                              const double* fI) {
  if (!ep.bnd || (I != 0 && I != N)) return;
  double* b = ep.bnd + ((I == N ? ntrans : 0) + line) * NV;
  const double w = I == N ? ep.bw : -ep.bw;
#pragma unroll
  for (int v = 0; v < NV; v++) b[v] = fma(w, fI[v], b[v]);
}

// The upwind flux of one interface from the six-cell window (cells j-3 .. j+2 of
// interface j-1/2): the fused kernel's WENO5 reconstructions (component-wise or
// characteristic) and upwinding, with the gravity source function's interface value SI
// (GRAV, source direction) and the adjoint's tape at interface index tapeoff.
//
// Centre-relative form (every kernel but the gravity ones, `RelFlux`): the window's
// cells enter relative to the interface's left cell p[2] = j-1 (its flux, state and
// modified state subtracted), and fI returns F_{j-1/2} - f_{j-1}.  The reconstructions
// and the upwinding are linear in the values apart from the weights (invariant under
// the shift) and the Roe average and sound speeds of the reconstructed states (which
// take the states with p[2] added back), so the result is the same interface flux
// minus f_{j-1}; the caller differences it as
//   F_{i+1/2} - F_{i-1/2} = (f_i - f_{i-1}) + (fI_{i+1/2} - fI_{i-1/2})
// (HyperbolicFunction.c:94-101 in exact arithmetic).  Values of the size of the
// window's variation instead of O(1) ones keep the rounding of the reconstruction out
// of the flux difference, and a third of the WENO5 stencil terms vanish with p[2].
template <bool GRAV>
struct RelFlux {
  static constexpr bool value = !GRAV;
};

// CQ (component-wise, no gravity, no tape: the tile form): the smoothness terms come
// from the tile's per-cell table, `qt` pointing at the entry of window cell 0 in row 0,
// rows of `nc` cells; for quantity k (the NV flux components, then the NV state
// components) rows QR k + role: Jiang-Shu (QR = 3) q = B^2 for the places l, c, r
// (weno5_cell_q); the other formulations (QR = 4) B for l, c, r and the second
// difference (weno5_cell_b).
template <int M, bool CHAR, int UPW, int DIR, bool ALTW, bool GRAV, bool WT, bool CQ = false>
__device__ __forceinline__ void iface_flux(const double (&wu)[6][ModelTraits<M>::NV],
                                           const double (&wf)[6][ModelTraits<M>::NV], const double (&wuc)[6],
                                           const double (&wgf)[6], const double (&wgg)[6],
                                           const CellAux<M> (&ax)[6], const PhysParams& pp, const StageEpi& ep,
                                           double eps4, bool src_dir, long long tapeoff, double (&fI)[ModelTraits<M>::NV],
                                           double (&SI)[ModelTraits<M>::NV], const double* qt = nullptr,
                                           int nc = 0) {
  static_assert(!CQ || (!CHAR && !GRAV && !WT), "the per-cell table serves the plain component-wise form");
  constexpr int NV = ModelTraits<M>::NV;
  constexpr bool CC = NeedCC<M, CHAR, UPW>::value;
  constexpr bool REL = RelFlux<GRAV>::value;
  Eig Ecc;
  if (CC) Ecc = roe_eig<M, DIR>(ax[2].rs, ax[3].rs, pp);
  // the modified state of the centre cell (the u-reconstruction's values): u with the
  // UFunction energy (NavierStokes3D; the same as u for the Euler models)
  double uc2[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) uc2[v] = wu[2][v];
  uc2[NV - 1] = (M == MODEL_NS3D) ? wuc[2] : wu[2][NV - 1];
  if (!CHAR) {
    // Component-wise WENO5: weights of the u-reconstruction from u, values from uC.
    double fL[NV], fR[NV], uL[NV], uR[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double sf[6], su[6];
#pragma unroll
      for (int p = 0; p < 6; p++) {
        sf[p] = REL ? (p == 2 ? 0.0 : wf[p][v] - wf[2][v]) : wf[p][v];
        su[p] = REL ? (p == 2 ? 0.0 : wu[p][v] - wu[2][v]) : wu[p][v];
      }
      if (WT) {
        double* t = ep.tape + tapeoff * TAPE_WIDE + 8 + v * 16;
        weno5_pair_tape<REL>(sf, sf, eps4, fL[v], fR[v], t);
        weno5_pair_tape<REL>(su, su, eps4, uL[v], uR[v], t + 8);
        continue;
      }
      if (CQ) {
        // left (l[1], c[2], r[3]), right (r[4], c[3], l[2]) of the window cells
        constexpr int QR = ALTW ? 4 : 3;
        double sc[6];
#pragma unroll
        for (int p = 0; p < 6; p++) sc[p] = REL ? (p == 2 ? 0.0 : wuc[p] - wuc[2]) : wuc[p];
        const double* vu = (M == MODEL_NS3D && v == NV - 1) ? sc : su;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const double* q = qt + (QR * (h * NV + v)) * nc;
          const double* vals = h ? vu : sf;
          double& oL = h ? uL[v] : fL[v];
          double& oR = h ? uR[v] : fR[v];
          if (ALTW)
            weno5_pair_alt_finish(vals, pp.wtype, q[1], q[nc + 2], q[2 * nc + 3], q[2 * nc + 4], q[nc + 3], q[2],
                                  q[3 * nc + 1], q[3 * nc + 2], q[3 * nc + 3], q[3 * nc + 4], oL, oR);
          else
            weno5_pair_q<REL>(vals, q[1], q[nc + 2], q[2 * nc + 3], q[2 * nc + 4], q[nc + 3], q[2], oL, oR);
        }
        continue;
      }
      // the source function phi = g is reconstructed with this flux component's
      // weights: evaluate them once and apply them to both
      const bool srcv = src_dir && (v == 1 + DIR || v == NV - 1);
      double omL[3], omR[3];
      if (srcv) {
        weno5_weights<ALTW>(sf, eps4, pp.wtype, omL, omR);
        weno5_apply(omL, omR, sf, fL[v], fR[v]);
      } else {
        wpair<ALTW, REL>(sf, sf, eps4, pp.wtype, fL[v], fR[v]);
      }
      if (M == MODEL_NS3D && v == NV - 1) {
        double sc[6];
#pragma unroll
        for (int p = 0; p < 6; p++) sc[p] = REL ? (p == 2 ? 0.0 : wuc[p] - wuc[2]) : wuc[p];
        wpair<ALTW, REL>(su, sc, eps4, pp.wtype, uL[v], uR[v]);
      } else if (GRAV) {
        double sc[6];
#pragma unroll
        for (int p = 0; p < 6; p++) sc[p] = su[p] * wgf[p];
        wpair<ALTW>(su, sc, eps4, pp.wtype, uL[v], uR[v]);
      } else {
        wpair<ALTW, REL>(su, su, eps4, pp.wtype, uL[v], uR[v]);
      }
      if (srcv) {
        double sL, sR;
        weno5_apply(omL, omR, wgg, sL, sR);
        SI[v] = 0.5 * (sL + sR);
      }
    }
    if (M == MODEL_EULER2D && (WT || ep.tape)) {
      // the adjoint reads the reconstructed states themselves
      double* t = ep.tape + tapeoff * (WT ? TAPE_WIDE : 8);
#pragma unroll
      for (int v = 0; v < NV; v++) {
        t[v] = REL ? uL[v] + uc2[v] : uL[v];
        t[4 + v] = REL ? uR[v] + uc2[v] : uR[v];
      }
    }
    upwind_iface<M, false, UPW, DIR>(fL, fR, uL, uR, Ecc, ax[2], ax[3], pp, fI,
                                     GRAV ? fmax(wgg[2], wgg[3]) : 1.0, REL ? uc2 : nullptr, REL ? wf[2] : nullptr);
  } else {
    // Characteristic WENO5 (WENOFifthOrderCalculateWeightsCharJS :760-896 and
    // Interp1PrimFifthOrderWENOChar :86-198): one eigen-system per interface
    // from the Roe average of the two cell-centre states.
    double cf[6][NV], cu[6][NV], cuc[6][GRAV ? NV : 3];
#pragma unroll
    for (int p = 0; p < 6; p++) {
      if (REL && p == 2) {
#pragma unroll
        for (int k = 0; k < NV; k++) cf[p][k] = cu[p][k] = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) cuc[p][k] = 0.0;
        continue;
      }
      if (REL) {
        double df[NV], du[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) {
          df[v] = wf[p][v] - wf[2][v];
          du[v] = wu[p][v] - wu[2][v];
        }
        projL<M, DIR>(Ecc, pp, df, cf[p]);
        projL<M, DIR>(Ecc, pp, du, cu[p]);
        if (M == MODEL_NS3D) {
          // uC differs from u in the energy only: add that column of L.
          double de = (wuc[p] - wuc[2]) - du[NV - 1];
          cuc[p][0] = fma(de, Ecc.gh, cu[p][0]);
          cuc[p][1] = fma(de, Ecc.gh, cu[p][1]);
          cuc[p][2] = fma(-de, Ecc.gi, cu[p][2]);
        }
        continue;
      }
      projL<M, DIR>(Ecc, pp, wf[p], cf[p]);
      projL<M, DIR>(Ecc, pp, wu[p], cu[p]);
      if (GRAV) {
        // uC = f u + (uC_E - f u_E) e_E: f (L u) plus the energy column of L
        const double fp = wgf[p], de = fma(-fp, wu[p][NV - 1], wuc[p]);
        cuc[p][0] = fma(de, Ecc.gh, fp * cu[p][0]);
        cuc[p][1] = fma(de, Ecc.gh, fp * cu[p][1]);
        cuc[p][2] = fma(-de, Ecc.gi, fp * cu[p][2]);
#pragma unroll
        for (int k = 3; k < NV; k++) cuc[p][k] = fp * cu[p][k];
      } else if (M == MODEL_NS3D) {
        // uC differs from u in the energy only: add that column of L.
        double de = wuc[p] - wu[p][NV - 1];
        cuc[p][0] = fma(de, Ecc.gh, cu[p][0]);
        cuc[p][1] = fma(de, Ecc.gh, cu[p][1]);
        cuc[p][2] = fma(-de, Ecc.gi, cu[p][2]);
      }
    }
    double lcol[NV];  // L (e_{1+DIR} + e_E): the projection of the source function per unit phi
    if (src_dir) {
      double ev[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) ev[v] = (v == 1 + DIR || v == NV - 1) ? 1.0 : 0.0;
      projL<M, DIR>(Ecc, pp, ev, lcol);
    }
    double sch[NV];
    double xfL[NV], xfR[NV], xuL[NV], xuR[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double sf[6], su[6];
#pragma unroll
      for (int p = 0; p < 6; p++) {
        sf[p] = cf[p][v];
        su[p] = cu[p][v];
      }
      double omL[3], omR[3];
      if (src_dir) {
        // one evaluation of the flux weights for the flux and the source function
        weno5_weights<ALTW>(sf, eps4, pp.wtype, omL, omR);
        weno5_apply(omL, omR, sf, xfL[v], xfR[v]);
      } else {
        wpair<ALTW, REL>(sf, sf, eps4, pp.wtype, xfL[v], xfR[v]);
      }
      if ((M == MODEL_NS3D && v < 3) || GRAV) {
        double sc[6];
#pragma unroll
        for (int p = 0; p < 6; p++) sc[p] = cuc[p][v];
        wpair<ALTW, REL>(su, sc, eps4, pp.wtype, xuL[v], xuR[v]);
      } else {
        wpair<ALTW, REL>(su, su, eps4, pp.wtype, xuL[v], xuR[v]);
      }
      if (src_dir) {
        double sL, sR, ps[6];
#pragma unroll
        for (int p = 0; p < 6; p++) ps[p] = wgg[p] * lcol[v];
        weno5_apply(omL, omR, ps, sL, sR);
        sch[v] = 0.5 * (sL + sR);
      }
    }
    if (src_dir) projR<M, DIR>(Ecc, sch, SI);
    upwind_char<M, UPW, DIR>(xfL, xfR, xuL, xuR, Ecc, ax[2], ax[3], pp, fI, GRAV ? fmax(wgg[2], wgg[3]) : 1.0,
                             REL ? uc2 : nullptr, REL ? wf[2] : nullptr);
  }
}

// One thread's share of a launch: interfaces [sg*seg, min((sg+1)*seg, N)] of
// the grid line with transverse index `tr` (other dimensions ascending, first
// fastest), and the flux difference / epilogue of the cells in between.
// GRAV (NavierStokes3D with Rusanov): the well-balanced gravity treatment --
// the modified solution uC = [f u_{0..3}, P/(gamma-1)/g + f rho|v|^2/2]
// (NavierStokes3DModifiedSolution.c:52-66), the dissipation factor
// max(g_L, g_R) (NavierStokes3DUpwind.c:407) and, along a direction with
// gravity, the source term of NavierStokes3DSource.c:38-112 subtracted from
// the hyperbolic term of this direction (except when only that term is asked for).
// WT (Euler2D, component-wise, Jiang-Shu: the adjoint's configuration): the wide
// tape -- per interface uL, uR and, per component, the smoothness terms and
// normalisation reciprocals of the f and u pairs (TAPE_WIDE doubles).
template <int M, bool CHAR, int UPW, int DIR, bool ALTW = false, bool GRAV = false, bool WT = false>
__device__ __forceinline__ void hyp_segment(const double* __restrict__ U, double* __restrict__ H,
                                            const double* __restrict__ dxinv, const DevGeom& G,
                                            const PhysParams& pp, const StageEpi& ep, int seg, long long tr,
                                            int sg) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND;
  constexpr bool CC = NeedCC<M, CHAR, UPW>::value;
  constexpr bool REL = RelFlux<GRAV>::value;
  const long long line = tr;

  long long pbase = (long long)G.g * G.stride[DIR];
#pragma unroll
  for (int e = 0; e < ND; e++) {
    if (e == DIR) continue;
    int ie = (int)(tr % G.dim[e]);
    tr /= G.dim[e];
    pbase += (long long)(ie + G.g) * G.stride[e];
  }
  const int N = G.dim[DIR];
  const long long sd = G.stride[DIR];
  const int lo = G.bclo[DIR], hi = G.bchi[DIR];
  const int I0 = sg * seg;
  const int I1 = min(I0 + seg, N);
  const double eps4 = 4.0 * pp.eps;

  double wu[6][NV], wf[6][NV], wuc[6];
  double wgf[6], wgg[6];  // gravity fields f, g (GRAV)
  CellAux<M> ax[6];
  const bool src_dir = GRAV && pp.grav[DIR] != 0.0 && (ep.mode != EPI_HYP || ep.with_source);

  auto load = [&](int i) {
    const long long pt = pbase + (long long)fold_index(i, N, lo, hi) * sd;
    const double* src = U + pt * NV;
#pragma unroll
    for (int v = 0; v < NV; v++) wu[5][v] = src[v];
    Prim<M> q = to_prim<M>(wu[5], pp);
    cell_flux<M, DIR>(q, wf[5]);
    if (GRAV) {
      wgf[5] = pp.gf[pt];
      wgg[5] = pp.gg[pt];
      if (M == MODEL_EULER1D) {
        wuc[5] = wu[5][NV - 1] * wgf[5];  // u* = u / S (gf holds 1 / S)
      } else {
        double vsq = q.vel[0] * q.vel[0] + q.vel[1] * q.vel[1] + q.vel[2] * q.vel[2];
        wuc[5] = fma(q.P * pp.inv_gm1, nr_rcp(wgg[5]), (0.5 * q.rho * vsq) * wgf[5]);
      }
    } else {
      wuc[5] = ufunc_energy<M>(q, pp, wu[5][NV - 1]);
    }
    if (CC) ax[5].rs = roe_side<M>(q);
    if (UPW == UPW_RUS) ax[5].c = rusanov_speed<M, DIR>(q, pp);
    else if (M == MODEL_EULER1D && UPW != UPW_ROE) ax[5].c = sound_speed<M>(q, pp);
  };
  auto shift = [&]() {
#pragma unroll
    for (int p = 0; p < 5; p++) {
#pragma unroll
      for (int v = 0; v < NV; v++) {
        wu[p][v] = wu[p + 1][v];
        wf[p][v] = wf[p + 1][v];
      }
      wuc[p] = wuc[p + 1];
      if (GRAV) {
        wgf[p] = wgf[p + 1];
        wgg[p] = wgg[p + 1];
      }
      ax[p] = ax[p + 1];
    }
  };

  for (int k = 0; k < 5; k++) {
    load(I0 - 3 + k);
    shift();
  }

  double fIp[NV], SI[NV], SIp[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) fIp[v] = SI[v] = SIp[v] = 0.0;

  for (int I = I0; I <= I1; I++) {
    load(I + 2);
    double fI[NV];
    iface_flux<M, CHAR, UPW, DIR, ALTW, GRAV, WT>(wu, wf, wuc, wgf, wgg, ax, pp, ep, eps4, src_dir,
                                                   line * (N + 1) + I, fI, SI);
    if (ep.bnd && (I == 0 || I == N)) {
      long long ntr = 1;
#pragma unroll
      for (int e = 0; e < ND; e++)
        if (e != DIR) ntr *= G.dim[e];
      double Fb[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) Fb[v] = REL ? fI[v] + wf[2][v] : fI[v];
      boundary_flux<NV>(ep, I, N, line, ntr, Fb);
    }

    if (I > I0) {
      // Flux difference of cell I-1 and the stage epilogue.
      const int c = I - 1;
      const long long off = (pbase + (long long)c * sd) * NV;
      const double dxi = dxinv[G.g + c];
      const bool finish = ep.last && ep.mode != EPI_HYP;
      double kv[NV], term[NV];
      if (src_dir) {
        // [0, rho RT e_DIR, rho RT v_DIR] f of the cell (NavierStokes3DSource.c:92-97)
        const double rho = wu[2][0], rRT = rho * pp.RT, f = wgf[2];
        const double vd = rho == 0.0 ? 0.0 : wu[2][1 + DIR] * nr_rcp(rho);
#pragma unroll
        for (int v = 0; v < NV; v++) term[v] = 0.0;
        term[1 + DIR] = rRT * f;
        term[NV - 1] = (rRT * vd) * f;
      }
#pragma unroll
      for (int v = 0; v < NV; v++) {
        // centre-relative fluxes: F_I - F_{I-1} = (f_c - f_{c-1}) + (fI_I - fI_{I-1})
        double h = REL ? dxi * ((wf[2][v] - wf[1][v]) + (fI[v] - fIp[v])) : dxi * (fI[v] - fIp[v]);
        if (src_dir) h = fma(-term[v] * (SI[v] - SIp[v]), dxi, h);  // rhs = -hyp + source
        double hyp = ep.first ? h : H[off + v] + h;
        if (!finish) {
          H[off + v] = hyp;
        } else {
          kv[v] = (ep.par ? ep.par[off + v] : 0.0) - hyp;
        }
      }
      if (finish) {
        if (ep.mode == EPI_RHS) {
#pragma unroll
          for (int v = 0; v < NV; v++) ep.rhs[off + v] = kv[v];
        } else {
#pragma unroll
          for (int v = 0; v < NV; v++) {
            const double uv = ep.need_u ? ep.u[off + v] : 0.0;
            double av = fma(ep.cb, kv[v], ep.stage == 0 ? uv : ep.acc[off + v]);
            if (ep.stage == ep.nstages - 1) ep.uout[off + v] = av;
            else ep.acc[off + v] = av;
#pragma unroll
            for (int t = 1; t < 4; t++) {
              if (t > ep.stage && t < ep.nstages && ep.ca[t] != 0.0) {
                double base = ep.touched[t] ? ep.P[t][off + v] : uv;
                ep.P[t][off + v] = fma(ep.ca[t], kv[v], base);
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int v = 0; v < NV; v++) {
      fIp[v] = fI[v];
      SIp[v] = SI[v];
    }
    shift();
  }
}

// The stage epilogue of the fused kernel for one cell (hyp_segment's): h is
// this direction's dxinv (F_{j+1/2} - F_{j-1/2}).
template <int NV>
__device__ __forceinline__ void stage_epilogue(const StageEpi& ep, double* __restrict__ H, long long off,
                                            const double* h) {
  const bool finish = ep.last && ep.mode != EPI_HYP;
  double kv[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double hyp = ep.first ? h[v] : H[off + v] + h[v];
    if (!finish) H[off + v] = hyp;
    else kv[v] = (ep.par ? ep.par[off + v] : 0.0) - hyp;
  }
  if (!finish) return;
  if (ep.mode == EPI_RHS) {
#pragma unroll
    for (int v = 0; v < NV; v++) ep.rhs[off + v] = kv[v];
    return;
  }
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double uv = ep.need_u ? ep.u[off + v] : 0.0;
    const double av = fma(ep.cb, kv[v], ep.stage == 0 ? uv : ep.acc[off + v]);
    if (ep.stage == ep.nstages - 1) ep.uout[off + v] = av;
    else ep.acc[off + v] = av;
#pragma unroll
    for (int t = 1; t < 4; t++) {
      if (t > ep.stage && t < ep.nstages && ep.ca[t] != 0.0) {
        const double base = ep.touched[t] ? ep.P[t][off + v] : uv;
        ep.P[t][off + v] = fma(ep.ca[t], kv[v], base);
      }
    }
  }
}

// Small grids: a block takes a tile of TI interfaces of one grid line (TI - 1 cells):
// its threads compute the data of the tile's TI + 5 cells once into shared memory
// (flux, modified energy, Roe-average ingredients, wave speeds), then each thread the
// flux of one interface from its six-cell window there, then each thread the flux
// difference and stage epilogue of one cell.  The segment walker recomputes a
// window's cells for every segment and one interface per segment boundary; with the
// one-to-three-interface segments that small grids need to occupy the GPU that
// redundancy is most of the work.  No gravity; WT: the adjoint's wide tape.
// The tile of block `blk` of a grid (blocks ordered line-fastest, then tile index).
template <int M, bool CHAR, int UPW, int DIR, bool ALTW, int TI, bool WT>
__device__ __forceinline__ void hyp_tile_body(const double* __restrict__ U, double* __restrict__ H,
                                              const double* __restrict__ dxinv, const DevGeom& G,
                                              const PhysParams& pp, const StageEpi& ep, long long ntrans,
                                              long long blk) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND;
  constexpr bool CC = NeedCC<M, CHAR, UPW>::value;
  constexpr int TC = TI - 1, NCELL = TI + 5;
  // component-wise: the smoothness terms of every cell's sub-stencil, once per cell
  // instead of six times per interface pair (QR rows per quantity: q for l, c, r with
  // Jiang-Shu weights; B for l, c, r and the second difference otherwise), where the
  // table keeps the block's static shared memory within 48 KB
  constexpr int QR = ALTW ? 4 : 3;
  constexpr size_t SMEM0 = sizeof(double) * NCELL * (2 * NV + 1) + sizeof(CellAux<M>) * NCELL +
                           sizeof(double) * TI * NV;
  constexpr bool CQ = !CHAR && !WT && SMEM0 + sizeof(double) * QR * 2 * NV * NCELL <= 48 * 1024;
  __shared__ double su[NCELL][NV], sf[NCELL][NV], suc[NCELL];
  __shared__ CellAux<M> sax[NCELL];
  __shared__ double sfI[TI][NV];
  __shared__ double sq[CQ ? QR * 2 * NV : 1][CQ ? NCELL : 1];
  const long long line = blk % ntrans;
  const int I0 = (int)(blk / ntrans) * TC;
  long long tr = line, pbase = (long long)G.g * G.stride[DIR];
#pragma unroll
  for (int e = 0; e < ND; e++) {
    if (e == DIR) continue;
    const int ie = (int)(tr % G.dim[e]);
    tr /= G.dim[e];
    pbase += (long long)(ie + G.g) * G.stride[e];
  }
  const int N = G.dim[DIR];
  const long long sd = G.stride[DIR];
  const int lo = G.bclo[DIR], hi = G.bchi[DIR];
  const double eps4 = 4.0 * pp.eps;
  // cells I0-3 .. I0+TI+1 (those within the line's reach)
  for (int c = threadIdx.x; c < NCELL; c += TI) {
    const int i = I0 - 3 + c;
    if (i > N + 2) continue;
    const long long pt = pbase + (long long)fold_index(i, N, lo, hi) * sd;
    double uu[NV], ff[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uu[v] = U[pt * NV + v];
    Prim<M> q = to_prim<M>(uu, pp);
    cell_flux<M, DIR>(q, ff);
#pragma unroll
    for (int v = 0; v < NV; v++) {
      su[c][v] = uu[v];
      sf[c][v] = ff[v];
    }
    suc[c] = ufunc_energy<M>(q, pp, uu[NV - 1]);
    CellAux<M> a;
    if (CC) a.rs = roe_side<M>(q);
    if (UPW == UPW_RUS) a.c = rusanov_speed<M, DIR>(q, pp);
    else if (M == MODEL_EULER1D && UPW != UPW_ROE) a.c = sound_speed<M>(q, pp);
    sax[c] = a;
  }
  __syncthreads();
  if constexpr (CQ) {
    // cells 1 .. TI+3 (those whose terms the tile's interfaces read), each from its
    // two neighbours; cells past the line's reach hold terms no interface reads
    for (int c = 1 + threadIdx.x; c <= TI + 3; c += TI) {
#pragma unroll
      for (int k = 0; k < 2 * NV; k++) {
        const double a = k < NV ? sf[c - 1][k] : su[c - 1][k - NV];
        const double b = k < NV ? sf[c][k] : su[c][k - NV];
        const double e = k < NV ? sf[c + 1][k] : su[c + 1][k - NV];
        if (ALTW)
          weno5_cell_b(a, b, e, eps4, sq[QR * k][c], sq[QR * k + 1][c], sq[QR * k + 2][c], sq[QR * k + 3][c]);
        else
          weno5_cell_q(a, b, e, eps4, sq[QR * k][c], sq[QR * k + 1][c], sq[QR * k + 2][c]);
      }
    }
    __syncthreads();
  }
  const int t = threadIdx.x;
  const int I = I0 + t;
  if (I <= N) {
    double wu[6][NV], wf[6][NV], wuc[6], wgf[6], wgg[6];
    CellAux<M> ax[6];
#pragma unroll
    for (int p = 0; p < 6; p++) {
#pragma unroll
      for (int v = 0; v < NV; v++) {
        wu[p][v] = su[t + p][v];
        wf[p][v] = sf[t + p][v];
      }
      wuc[p] = suc[t + p];
      ax[p] = sax[t + p];
    }
    double fI[NV], SI[NV];
    iface_flux<M, CHAR, UPW, DIR, ALTW, false, WT, CQ>(wu, wf, wuc, wgf, wgg, ax, pp, ep, eps4, false,
                                                       line * (N + 1) + I, fI, SI, CQ ? &sq[0][t] : nullptr, NCELL);
    // fI is relative to the interface's left cell (window cell 2)
    if (ep.bnd && (I == 0 || I == N)) {
      double Fb[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) Fb[v] = fI[v] + wf[2][v];
      boundary_flux<NV>(ep, I, N, line, ntrans, Fb);
    }
#pragma unroll
    for (int v = 0; v < NV; v++) sfI[t][v] = fI[v];
  }
  __syncthreads();
  const int c = I0 + t;
  if (t < TC && c < N) {
    const long long off = (pbase + (long long)c * sd) * NV;
    const double dxi = dxinv[G.g + c];
    double h[NV];
    // cell c is tile cell t + 3; F_{c+1} - F_c = (f_c - f_{c-1}) + (fI_{t+1} - fI_t)
#pragma unroll
    for (int v = 0; v < NV; v++) h[v] = dxi * ((sf[t + 3][v] - sf[t + 2][v]) + (sfI[t + 1][v] - sfI[t][v]));
    stage_epilogue<NV>(ep, H, off, h);
  }
}

// Short 1-D lines (a Sod tube of 10^3 cells leaves one warp per SM, which then runs an
// interface's several hundred FP64 instructions back to back): the interface work
// split over lanes.  A block takes TI interfaces (TI - 1 cells) of the line in
// groups of 16 lanes; phase 1 computes the TI + 5 cells into shared memory, phase 2
// gives each side (left- or right-biased value) of each of the 2 NV reconstructions of
// an interface (the f or the u pair of one component) to its own lane, and the Roe
// average of the interface's two cells to the next lane, phase 3 upwinds each
// interface, phase 4 differences and updates each cell.  On GB300 an SM's FP64 unit
// takes a warp instruction every 16 cycles, so the time of a short line is the length
// of the longest dependent FP64 chain of a lane; splitting the pairs into sides and
// moving the Roe average off the upwinding lane shortens it.  Component-wise WENO5 of
// a model whose u-reconstruction reads u itself (Euler1D without gravity).
template <int M, int UPW, bool ALTW, int TI>
__global__ void __launch_bounds__(TI * 16)
hyp_lane_kernel(const double* __restrict__ U, double* __restrict__ H, const double* __restrict__ dxinv, DevGeom G,
                PhysParams pp, StageEpi ep) {
  constexpr int NV = ModelTraits<M>::NV;
  static_assert(4 * NV + 1 <= 16, "an interface's reconstruction sides fit a group of 16 lanes");
  constexpr bool CC = NeedCC<M, false, UPW>::value;
  constexpr int TC = TI - 1, NCELL = TI + 5, NT = TI * 16;
  __shared__ double su[NCELL][NV], sf[NCELL][NV];
  __shared__ CellAux<M> sax[NCELL];
  __shared__ double srec[TI][2 * NV][2];
  __shared__ double sfI[TI][NV];
  __shared__ Eig secc[TI];
  const int I0 = (int)blockIdx.x * TC;
  const int N = G.dim[0];
  const long long sd = G.stride[0];
  const long long pbase = (long long)G.g * sd;
  const int lo = G.bclo[0], hi = G.bchi[0];
  const double eps4 = 4.0 * pp.eps;
  const int t = threadIdx.x;
  for (int c = t; c < NCELL; c += NT) {
    const int i = I0 - 3 + c;
    if (i > N + 2) continue;
    const long long pt = pbase + (long long)fold_index(i, N, lo, hi) * sd;
    double uu[NV], ff[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uu[v] = U[pt * NV + v];
    Prim<M> q = to_prim<M>(uu, pp);
    cell_flux<M, 0>(q, ff);
#pragma unroll
    for (int v = 0; v < NV; v++) {
      su[c][v] = uu[v];
      sf[c][v] = ff[v];
    }
    CellAux<M> a;
    if (CC) a.rs = roe_side<M>(q);
    if (UPW == UPW_RUS) a.c = rusanov_speed<M, 0>(q, pp);
    else if (M == MODEL_EULER1D && UPW != UPW_ROE) a.c = sound_speed<M>(q, pp);
    sax[c] = a;
  }
  __syncthreads();
  {
    const int i = t >> 4, k = t & 15;
    if (k < 4 * NV && I0 + i <= N) {
      // lane k: component v, the u (bit 1) or f reconstruction, its right (bit 0) or
      // left side; the window relative to the interface's left cell (window cell 2),
      // mirrored for the right side
      const int v = k >> 2, isu = (k >> 1) & 1, right = k & 1;
      double m[5];
#pragma unroll
      for (int p = 0; p < 5; p++) {
        const int c = i + (right ? 5 - p : p);
        m[p] = c == i + 2 ? 0.0 : (isu ? su[c][v] - su[i + 2][v] : sf[c][v] - sf[i + 2][v]);
      }
      srec[i][2 * v + isu][right] = weno5_one_side<ALTW>(m, eps4, pp.wtype);
    } else if (CC && k == 4 * NV && I0 + i <= N) {
      secc[i] = roe_eig<M, 0>(sax[i + 2].rs, sax[i + 3].rs, pp);
    }
  }
  __syncthreads();
  if (t < TI && I0 + t <= N) {
    double fL[NV], fR[NV], uL[NV], uR[NV], fI[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      fL[v] = srec[t][2 * v][0];
      fR[v] = srec[t][2 * v][1];
      uL[v] = srec[t][2 * v + 1][0];
      uR[v] = srec[t][2 * v + 1][1];
    }
    Eig Ecc;
    if (CC) Ecc = secc[t];
    double uc2[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uc2[v] = su[t + 2][v];
    upwind_iface<M, false, UPW, 0>(fL, fR, uL, uR, Ecc, sax[t + 2], sax[t + 3], pp, fI, 1.0, uc2, sf[t + 2]);
    if (ep.bnd && (I0 + t == 0 || I0 + t == N)) {
      double Fb[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) Fb[v] = fI[v] + sf[t + 2][v];
      boundary_flux<NV>(ep, I0 + t, N, 0, 1, Fb);
    }
#pragma unroll
    for (int v = 0; v < NV; v++) sfI[t][v] = fI[v];
  }
  __syncthreads();
  const int c = I0 + t;
  if (t < TC && c < N) {
    const long long off = (pbase + (long long)c * sd) * NV;
    const double dxi = dxinv[G.g + c];
    double h[NV];
    // centre-relative fluxes, as in hyp_tile_body
#pragma unroll
    for (int v = 0; v < NV; v++) h[v] = dxi * ((sf[t + 3][v] - sf[t + 2][v]) + (sfI[t + 1][v] - sfI[t][v]));
    stage_epilogue<NV>(ep, H, off, h);
  }
}

// Resident blocks per SM the register allocation of the 128-interface tile kernels
// must allow: 4 (at most 128 registers a thread) keeps four 128-thread blocks on an
// SM, which the kernel needs to keep the FP64 pipe busy (1: as many registers as the
// compiler wants).
#ifndef GBH_TILE_MINB
#define GBH_TILE_MINB 4
#endif

template <int M, bool CHAR, int UPW, int DIR, bool ALTW, int TI, bool WT = false>
__global__ void __launch_bounds__(TI, (TI == 128 ? GBH_TILE_MINB : 1))
hyp_tile_kernel(const double* __restrict__ U, double* __restrict__ H, const double* __restrict__ dxinv, DevGeom G,
                PhysParams pp, StageEpi ep, long long ntrans) {
  hyp_tile_body<M, CHAR, UPW, DIR, ALTW, TI, WT>(U, H, dxinv, G, pp, ep, ntrans, blockIdx.x);
}

template <int M, bool CHAR, int UPW, int DIR, bool ALTW, bool GRAV = false, bool WT = false>
__global__ void __launch_bounds__(128)
hyp_dir_kernel(const double* __restrict__ U, double* __restrict__ H, const double* __restrict__ dxinv,
               DevGeom G, PhysParams pp, StageEpi ep, int seg, int nseg, long long ntrans) {
  long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= ntrans * (long long)nseg) return;
  hyp_segment<M, CHAR, UPW, DIR, ALTW, GRAV, WT>(U, H, dxinv, G, pp, ep, seg, tid % ntrans, (int)(tid / ntrans));
}

// All members of an ensemble advanced by one launch per direction: a thread
// finds its member by binary search over the start offsets, then walks its
// segment exactly as in the single-grid kernel.
// The member that owns work item `w` of direction DIR (members' first items
// ascending), with the stage pointers moved to its arrays.
template <int DIR>
__device__ __forceinline__ const MemberDev& batched_member(const MemberDev* __restrict__ mem, int nmem, long long w,
                                                           StageEpi& e) {
  int lo = 0, hi = nmem - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (mem[mid].start[DIR] <= w) lo = mid;
    else hi = mid - 1;
  }
  const MemberDev& m = mem[lo];
  const long long o = m.off;
  if (e.par) e.par += o;
  if (e.rhs) e.rhs += o;
  if (e.u) e.u += o;
  if (e.uout) e.uout += o;
  if (e.acc) e.acc += o;
#pragma unroll
  for (int t = 0; t < 4; t++)
    if (e.P[t]) e.P[t] += o;
  if (e.bnd) e.bnd += m.bnd_off[DIR];
  return m;
}

template <int M, bool CHAR, int UPW, int DIR>
__global__ void __launch_bounds__(128)
hyp_batched_kernel(const MemberDev* __restrict__ mem, int nmem, long long total, const double* __restrict__ U,
                   double* __restrict__ H, const double* __restrict__ dxinv, PhysParams pp, StageEpi ep) {
  long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= total) return;
  StageEpi e = ep;
  const MemberDev& m = batched_member<DIR>(mem, nmem, tid, e);
  long long lt = tid - m.start[DIR];
  long long ntr = m.ntrans[DIR];
  const long long o = m.off;
  hyp_segment<M, CHAR, UPW, DIR>(U + o, H ? H + o : nullptr, dxinv + m.dx_off[DIR], m.G, pp, e, m.seg[DIR],
                                 lt % ntr, (int)(lt / ntr));
}

// Tile form of the batched kernel: one block per tile of TI interfaces of one
// member's grid line; the members' tables count blocks instead of threads.
template <int M, bool CHAR, int UPW, int DIR, int TI>
__global__ void __launch_bounds__(TI)
hyp_batched_tile_kernel(const MemberDev* __restrict__ mem, int nmem, const double* __restrict__ U,
                        double* __restrict__ H, const double* __restrict__ dxinv, PhysParams pp, StageEpi ep) {
  StageEpi e = ep;
  const long long b = blockIdx.x;
  const MemberDev& m = batched_member<DIR>(mem, nmem, b, e);
  const long long o = m.off;
  hyp_tile_body<M, CHAR, UPW, DIR, false, TI, false>(U + o, H ? H + o : nullptr, dxinv + m.dx_off[DIR], m.G, pp,
                                                     e, m.ntrans[DIR], b - m.start[DIR]);
}

// Persistent work-list form of the batched tile kernel: a grid of as many blocks as
// the SMs hold at once pulls tile indices from a work counter (one atomicAdd per
// tile, by one thread of the block) until the launch's `total` tiles are taken.  The
// loop is bounded: every fetch takes a new index, so a block stops after at most
// total / gridDim + 1 fetches.  `counter` is zero when the launch starts.
template <int M, bool CHAR, int UPW, int DIR, int TI>
__global__ void __launch_bounds__(TI)
hyp_batched_worklist_kernel(const MemberDev* __restrict__ mem, int nmem, long long total,
                            unsigned long long* __restrict__ counter, const double* __restrict__ U,
                            double* __restrict__ H, const double* __restrict__ dxinv, PhysParams pp, StageEpi ep) {
  __shared__ long long s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = (long long)atomicAdd(counter, 1ULL);
    __syncthreads();
    const long long b = s_tile;
    __syncthreads();  // every thread holds b before thread 0 fetches the next one
    if (b >= total) return;
    StageEpi e = ep;
    const MemberDev& m = batched_member<DIR>(mem, nmem, b, e);
    const long long o = m.off;
    hyp_tile_body<M, CHAR, UPW, DIR, false, TI, false>(U + o, H ? H + o : nullptr, dxinv + m.dx_off[DIR], m.G, pp,
                                                       e, m.ntrans[DIR], b - m.start[DIR]);
  }
}

template <typename K>
unsigned worklist_grid(K kernel, int threads, long long total) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
  long long g = (long long)(per > 0 ? per : 1) * (sms > 0 ? sms : 1);
  return (unsigned)(g < total ? g : total);
}

// total = threads (walker, tile == 0) or blocks (tiles of `tile` interfaces).
// counter != nullptr with a tile form: the persistent work-list kernel.
template <int M, bool CHAR, int UPW, int DIR>
cudaError_t launch_batched_dir(const MemberDev* mem, int nmem, long long total, const double* U, double* H,
                               const double* dxinv, const PhysParams& pp, const StageEpi& ep, int block, int tile,
                               unsigned long long* counter, cudaStream_t s) {
  if (total <= 0) return cudaSuccess;
  if (counter && tile) {
#define GBH_WL(TI)                                                                                       \
  do {                                                                                                   \
    auto k = hyp_batched_worklist_kernel<M, CHAR, UPW, DIR, TI>;                                         \
    k<<<worklist_grid(k, TI, total), TI, 0, s>>>(mem, nmem, total, counter, U, H, dxinv, pp, ep);        \
  } while (0)
    if (tile == 32) GBH_WL(32);
    else if (tile == 64) GBH_WL(64);
    else if (tile == 128) GBH_WL(128);
    else return cudaErrorInvalidValue;
#undef GBH_WL
    return cudaGetLastError();
  }
  if (tile == 32)
    hyp_batched_tile_kernel<M, CHAR, UPW, DIR, 32><<<(unsigned)total, 32, 0, s>>>(mem, nmem, U, H, dxinv, pp, ep);
  else if (tile == 64)
    hyp_batched_tile_kernel<M, CHAR, UPW, DIR, 64><<<(unsigned)total, 64, 0, s>>>(mem, nmem, U, H, dxinv, pp, ep);
  else if (tile == 128)
    hyp_batched_tile_kernel<M, CHAR, UPW, DIR, 128><<<(unsigned)total, 128, 0, s>>>(mem, nmem, U, H, dxinv, pp, ep);
  else if (tile != 0)
    return cudaErrorInvalidValue;
  else {
    if (block <= 0) block = 128;
    long long grid = (total + block - 1) / block;
    hyp_batched_kernel<M, CHAR, UPW, DIR><<<(unsigned)grid, block, 0, s>>>(mem, nmem, total, U, H, dxinv, pp, ep);
  }
  return cudaGetLastError();
}

template <int M>
cudaError_t launch_batched_model(int dir, int chr, int upw, const MemberDev* mem, int nmem, long long total,
                                 const double* U, double* H, const double* dxinv, const PhysParams& pp,
                                 const StageEpi& ep, int block, int tile, unsigned long long* counter,
                                 cudaStream_t s) {
  constexpr int ND = ModelTraits<M>::ND;
#define GBH_B(C, W)                                                                                          \
  do {                                                                                                       \
    if (dir == 0)                                                                                            \
      return launch_batched_dir<M, C, W, 0>(mem, nmem, total, U, H, dxinv, pp, ep, block, tile, counter, s); \
    if (ND > 1 && dir == 1)                                                                                  \
      return launch_batched_dir<M, C, W, (ND > 1 ? 1 : 0)>(mem, nmem, total, U, H, dxinv, pp, ep, block, tile, \
                                                           counter, s);                                      \
    if (ND > 2 && dir == 2)                                                                                  \
      return launch_batched_dir<M, C, W, (ND > 2 ? 2 : 0)>(mem, nmem, total, U, H, dxinv, pp, ep, block, tile, \
                                                           counter, s);                                      \
    return cudaErrorInvalidValue;                                                                            \
  } while (0)
  // Rusanov: Euler1D and NavierStokes3D (Euler2D offers none); the template
  // argument falls back to RF for Euler2D only to keep that branch compilable.
  constexpr int RUS = (M != MODEL_EULER2D) ? UPW_RUS : UPW_RF;
  if (chr) {
    if (upw == UPW_ROE) GBH_B(true, UPW_ROE);
    if (upw == UPW_LLF) GBH_B(true, UPW_LLF);
    if (upw == UPW_RUS && M != MODEL_EULER2D) GBH_B(true, RUS);
    GBH_B(true, UPW_RF);
  } else {
    if (upw == UPW_ROE) GBH_B(false, UPW_ROE);
    if (upw == UPW_LLF) GBH_B(false, UPW_LLF);
    if (upw == UPW_RUS && M != MODEL_EULER2D) GBH_B(false, RUS);
    GBH_B(false, UPW_RF);
  }
#undef GBH_B
}

// Host launcher for one direction.
template <int M, bool CHAR, int UPW, int DIR, bool ALTW, bool GRAV = false, bool WT = false>
cudaError_t launch_dir(const double* U, double* H, const double* dxinv_dir, const DevGeom& G,
                       const PhysParams& pp, const StageEpi& ep, const HypLaunch& L, cudaStream_t s) {
  long long ntrans = 1;
  for (int e = 0; e < G.nd; e++)
    if (e != DIR) ntrans *= G.dim[e];
  int N = G.dim[DIR];
  if constexpr (M == MODEL_EULER1D && !CHAR && !GRAV && !WT) {
    if (L.seg == -8 || L.seg == -16) {
      // lane groups: TI interfaces of the one line per block, 16 lanes per interface
      const int ti = -L.seg;
      const unsigned nblk = (unsigned)((N + ti - 2) / (ti - 1));
      if (ti == 8) hyp_lane_kernel<M, UPW, ALTW, 8><<<nblk, 128, 0, s>>>(U, H, dxinv_dir, G, pp, ep);
      else hyp_lane_kernel<M, UPW, ALTW, 16><<<nblk, 256, 0, s>>>(U, H, dxinv_dir, G, pp, ep);
      return cudaGetLastError();
    }
  }
  if (L.seg < 0 && !GRAV) {
    // tiles of -seg interfaces (32, 64 or 128), one block each
    const int ti = -L.seg;
    const long long nblk = ntrans * ((N + ti - 2) / (ti - 1));
    if (ti == 32)
      hyp_tile_kernel<M, CHAR, UPW, DIR, ALTW, 32, WT><<<(unsigned)nblk, 32, 0, s>>>(U, H, dxinv_dir, G, pp, ep,
                                                                                   ntrans);
    else if (ti == 64)
      hyp_tile_kernel<M, CHAR, UPW, DIR, ALTW, 64, WT><<<(unsigned)nblk, 64, 0, s>>>(U, H, dxinv_dir, G, pp, ep,
                                                                                   ntrans);
    else
      hyp_tile_kernel<M, CHAR, UPW, DIR, ALTW, 128, WT><<<(unsigned)nblk, 128, 0, s>>>(U, H, dxinv_dir, G, pp, ep,
                                                                                     ntrans);
    return cudaGetLastError();
  }
  // a tile shape asked of a kernel without the tile form (gravity): segments that
  // spread the line over about four warps per SM
  int seg = L.seg > 0 ? L.seg : 32;
  if (L.seg < 0) {
    const long long want = 152LL * 4 * 32;
    seg = (int)((ntrans * N + want - 1) / want);
    seg = seg < 1 ? 1 : (seg > 64 ? 64 : seg);
  }
  int nseg = (N + seg - 1) / seg;
  long long nthr = ntrans * nseg;
  int block = L.block > 0 ? L.block : 128;
  long long grid = (nthr + block - 1) / block;
  hyp_dir_kernel<M, CHAR, UPW, DIR, ALTW, GRAV, WT><<<(unsigned)grid, block, 0, s>>>(U, H, dxinv_dir, G, pp, ep,
                                                                                  seg, nseg, ntrans);
  return cudaGetLastError();
}

template <int M, bool CHAR, int UPW, bool ALTW, bool GRAV = false>
cudaError_t launch_dir_any(int dir, const double* U, double* H, const double* dxinv_dir, const DevGeom& G,
                           const PhysParams& pp, const StageEpi& ep, const HypLaunch& L, cudaStream_t s) {
  constexpr int ND = ModelTraits<M>::ND;
  if (dir == 0) return launch_dir<M, CHAR, UPW, 0, ALTW, GRAV>(U, H, dxinv_dir, G, pp, ep, L, s);
  if (ND > 1 && dir == 1)
    return launch_dir<M, CHAR, UPW, (ND > 1 ? 1 : 0), ALTW, GRAV>(U, H, dxinv_dir, G, pp, ep, L, s);
  if (ND > 2 && dir == 2)
    return launch_dir<M, CHAR, UPW, (ND > 2 ? 2 : 0), ALTW, GRAV>(U, H, dxinv_dir, G, pp, ep, L, s);
  return cudaErrorInvalidValue;
}

// NavierStokes3D with gravity (Rusanov upwinding, as the reference requires):
// ALTW selects the weight formulation as in launch_hyp_model.
// Euler1D with gravity (Xing & Shu's well-balanced form): Roe or LLF, u* = u / S,
// the dissipation scaled by max(S_L, S_R), the source [0, rho, rho v] / S times the
// difference of the interface values of [0, S, S] (pp: gf = 1/S, gg = S, RT = 1).
template <bool ALTW>
cudaError_t launch_hyp_euler1d_gravity(int dir, int chr, int upw, const double* U, double* H,
                                       const double* dxinv_dir, const DevGeom& G, const PhysParams& pp,
                                       const StageEpi& ep, const HypLaunch& L, cudaStream_t s) {
  if (dir != 0) return cudaErrorInvalidValue;
  if (chr) {
    if (upw == UPW_LLF)
      return launch_dir<MODEL_EULER1D, true, UPW_LLF, 0, ALTW, true>(U, H, dxinv_dir, G, pp, ep, L, s);
    return launch_dir<MODEL_EULER1D, true, UPW_ROE, 0, ALTW, true>(U, H, dxinv_dir, G, pp, ep, L, s);
  }
  if (upw == UPW_LLF)
    return launch_dir<MODEL_EULER1D, false, UPW_LLF, 0, ALTW, true>(U, H, dxinv_dir, G, pp, ep, L, s);
  return launch_dir<MODEL_EULER1D, false, UPW_ROE, 0, ALTW, true>(U, H, dxinv_dir, G, pp, ep, L, s);
}

template <bool ALTW>
cudaError_t launch_hyp_ns3d_gravity(int dir, int chr, const double* U, double* H, const double* dxinv_dir,
                                    const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                                    cudaStream_t s) {
  if (chr) return launch_dir_any<MODEL_NS3D, true, UPW_RUS, ALTW, true>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
  return launch_dir_any<MODEL_NS3D, false, UPW_RUS, ALTW, true>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
}

// ALTW = false: Jiang-Shu weights (pp.wtype ignored); true: pp.wtype selects them.
template <int M, bool ALTW = false>
cudaError_t launch_hyp_model(int dir, int chr, int upw, const double* U, double* H, const double* dxinv_dir,
                             const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                             cudaStream_t s) {
  constexpr int RUS = (M != MODEL_EULER2D) ? UPW_RUS : UPW_RF;  // Euler2D offers no Rusanov
  constexpr int SW = (M != MODEL_NS3D) ? UPW_SWFS : UPW_RF;     // nor NavierStokes3D Steger-Warming
  if (upw == UPW_SWFS && M == MODEL_NS3D) return cudaErrorInvalidValue;
  if (chr) {
    if (upw == UPW_SWFS) return launch_dir_any<M, true, SW, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    if (upw == UPW_ROE) return launch_dir_any<M, true, UPW_ROE, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    if (upw == UPW_LLF) return launch_dir_any<M, true, UPW_LLF, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    if (upw == UPW_RUS && M != MODEL_EULER2D)
      return launch_dir_any<M, true, RUS, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    return launch_dir_any<M, true, UPW_RF, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
  } else {
    if (upw == UPW_SWFS) return launch_dir_any<M, false, SW, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    if (upw == UPW_ROE) return launch_dir_any<M, false, UPW_ROE, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    if (upw == UPW_LLF) return launch_dir_any<M, false, UPW_LLF, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    if (upw == UPW_RUS && M != MODEL_EULER2D)
      return launch_dir_any<M, false, RUS, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
    return launch_dir_any<M, false, UPW_RF, ALTW>(dir, U, H, dxinv_dir, G, pp, ep, L, s);
  }
}

// ---------------------------------------------------------------------------
// Unfused pieces of the HyPar function-pointer surface (FFunction, UFunction,
// Upwind), one thread per point / interface, on HyPar's own array layouts.
// ---------------------------------------------------------------------------
template <int M, int DIR>
__global__ void flux_kernel(double* __restrict__ f, const double* __restrict__ u, long long npts, PhysParams pp) {
  constexpr int NV = ModelTraits<M>::NV;
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  double uu[NV], ff[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) uu[v] = u[p * NV + v];
  Prim<M> q = to_prim<M>(uu, pp);
  cell_flux<M, DIR>(q, ff);
#pragma unroll
  for (int v = 0; v < NV; v++) f[p * NV + v] = ff[v];
}

template <int M>
__global__ void ufunc_kernel(double* __restrict__ uC, const double* __restrict__ u, long long npts, PhysParams pp) {
  constexpr int NV = ModelTraits<M>::NV;
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts) return;
  double uu[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) uu[v] = u[p * NV + v];
  Prim<M> q = to_prim<M>(uu, pp);
  if (M == MODEL_EULER1D && pp.gf) {
    // Euler1DModifiedSolution.c:48: u* = u / S (gf holds 1 / S)
  #pragma unroll
    for (int v = 0; v < NV; v++) uC[p * NV + v] = uu[v] * pp.gf[p];
    return;
  }
  if (M == MODEL_NS3D && pp.gf) {
    // NavierStokes3DModifiedSolution.c:55-66: u* scaled by the hydrostatic fields
    const double f = pp.gf[p], g = pp.gg[p];
    const double vsq = q.vel[0] * q.vel[0] + q.vel[1] * q.vel[1] + q.vel[2] * q.vel[2];
#pragma unroll
    for (int v = 0; v < NV - 1; v++) uC[p * NV + v] = uu[v] * f;
    uC[p * NV + NV - 1] = fma(q.P * pp.inv_gm1, nr_rcp(g), (0.5 * q.rho * vsq) * f);
    return;
  }
#pragma unroll
  for (int v = 0; v < NV - 1; v++) uC[p * NV + v] = uu[v];
  uC[p * NV + NV - 1] = ufunc_energy<M>(q, pp, uu[NV - 1]);
}

// Interface arrays have no ghost points and dim[DIR]+1 entries along DIR
// (include/hypar.h:133-145); u is the ghosted cell-centre solution.
template <int M, int UPW, int DIR>
__global__ void upwind_kernel(double* __restrict__ fI, const double* __restrict__ fL, const double* __restrict__ fR,
                              const double* __restrict__ uL, const double* __restrict__ uR,
                              const double* __restrict__ u, DevGeom G, PhysParams pp, long long nint) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND;
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nint) return;
  int idx[3] = {0, 0, 0};
  long long r = p;
#pragma unroll
  for (int e = 0; e < ND; e++) {
    int n = G.dim[e] + (e == DIR ? 1 : 0);
    idx[e] = (int)(r % n);
    r /= n;
  }
  long long pc = 0;
#pragma unroll
  for (int e = 0; e < ND; e++) pc += (long long)(idx[e] + G.g) * G.stride[e];
  long long pL = pc - G.stride[DIR], pR = pc;
  double a[NV], b[NV], c[NV], d[NV], ucl[NV], ucr[NV], out[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    a[v] = fL[p * NV + v];
    b[v] = fR[p * NV + v];
    c[v] = uL[p * NV + v];
    d[v] = uR[p * NV + v];
    ucl[v] = u[pL * NV + v];
    ucr[v] = u[pR * NV + v];
  }
  Prim<M> ql = to_prim<M>(ucl, pp), qr = to_prim<M>(ucr, pp);
  CellAux<M> cl, cr;
  cl.rs = roe_side<M>(ql);
  cr.rs = roe_side<M>(qr);
  cl.c = UPW == UPW_RUS ? rusanov_speed<M, DIR>(ql, pp) : sound_speed<M>(ql, pp);
  cr.c = UPW == UPW_RUS ? rusanov_speed<M, DIR>(qr, pp) : sound_speed<M>(qr, pp);
  Eig Ecc = roe_eig<M, DIR>(cl.rs, cr.rs, pp);
  // NavierStokes3DUpwind.c: Rusanov's dissipation scaled by max(g_L, g_R) of the gravity field
  const double kappa = ((UPW == UPW_RUS || M == MODEL_EULER1D) && pp.gg) ? fmax(pp.gg[pL], pp.gg[pR]) : 1.0;
  upwind_iface<M, true, UPW, DIR>(a, b, c, d, Ecc, cl, cr, pp, out, kappa);
#pragma unroll
  for (int v = 0; v < NV; v++) fI[p * NV + v] = out[v];
}

// InterpolateInterfacesHyp (Interp1PrimFifthOrderWENO.c:74-168 and
// Interp1PrimFifthOrderWENOChar.c:86-198): the WENO5 value at every interface of
// the ghosted cell array fC along DIR, left-biased (LEFT) or right-biased, with the
// nonlinear weights of the stencil of fC (!UF) or of u (UF), the weights the
// reference stores in SetInterpLimiterVar from the same arrays
// (WENOFifthOrderCalculateWeights.c).  CHAR: in the characteristic fields of the Roe
// average of u at the interface's two cells.  One thread per interface; ghost points
// are read as the caller left them.
template <int M, bool CHAR, int DIR>
__global__ void interp_kernel(double* __restrict__ fI, const double* __restrict__ fC, const double* __restrict__ u,
                              DevGeom G, PhysParams pp, int left, int uf, long long nint) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND;
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nint) return;
  int idx[3] = {0, 0, 0};
  long long r = p;
#pragma unroll
  for (int e = 0; e < ND; e++) {
    int n = G.dim[e] + (e == DIR ? 1 : 0);
    idx[e] = (int)(r % n);
    r /= n;
  }
  long long pc = 0;  // the cell right of the interface
#pragma unroll
  for (int e = 0; e < ND; e++) pc += (long long)(idx[e] + G.g) * G.stride[e];
  const long long sd = G.stride[DIR];
  const double eps4 = 4.0 * pp.eps;
  // window: cells I-3 .. I+2 of interface I (left cell I-1, right cell I)
  double wv[6][NV], ww[6][NV];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const long long q = (pc + (long long)(k - 3) * sd) * NV;
#pragma unroll
    for (int v = 0; v < NV; v++) {
      wv[k][v] = fC[q + v];
      ww[k][v] = uf ? u[q + v] : wv[k][v];
    }
  }
  double out[NV];
  if (!CHAR) {
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double sw[6], sv[6], omL[3], omR[3], oL, oR;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        sw[k] = ww[k][v];
        sv[k] = wv[k][v];
      }
      weno5_weights<true>(sw, eps4, pp.wtype, omL, omR);
      weno5_apply(omL, omR, sv, oL, oR);
      out[v] = left ? oL : oR;
    }
  } else {
    double uu[NV];
    RoeSide rs[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const long long q = (pc + (long long)(k - 1) * sd) * NV;
#pragma unroll
      for (int v = 0; v < NV; v++) uu[v] = u[q + v];
      rs[k] = roe_side<M>(to_prim<M>(uu, pp));
    }
    const Eig E = roe_eig<M, DIR>(rs[0], rs[1], pp);
    double cv[6][NV], cw[6][NV];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      projL<M, DIR>(E, pp, wv[k], cv[k]);
      if (uf) projL<M, DIR>(E, pp, ww[k], cw[k]);
    }
    double ch[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double sw[6], sv[6], omL[3], omR[3], oL, oR;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        sv[k] = cv[k][v];
        sw[k] = uf ? cw[k][v] : cv[k][v];
      }
      weno5_weights<true>(sw, eps4, pp.wtype, omL, omR);
      weno5_apply(omL, omR, sv, oL, oR);
      ch[v] = left ? oL : oR;
    }
    projR<M, DIR>(E, ch, out);
  }
#pragma unroll
  for (int v = 0; v < NV; v++) fI[p * NV + v] = out[v];
}

template <int M>
cudaError_t launch_interp_model(int dir, int chr, int left, int uf, double* fI, const double* fC, const double* u,
                                const DevGeom& G, const PhysParams& pp, cudaStream_t s) {
  constexpr int ND = ModelTraits<M>::ND;
  if (dir < 0 || dir >= ND) return cudaErrorInvalidValue;
  long long nint = 1;
  for (int e = 0; e < ND; e++) nint *= G.dim[e] + (e == dir ? 1 : 0);
  const unsigned grid = (unsigned)((nint + 127) / 128);
#define GBH_I(D)                                                                                          \
  do {                                                                                                    \
    if (chr) interp_kernel<M, true, D><<<grid, 128, 0, s>>>(fI, fC, u, G, pp, left, uf, nint);          \
    else interp_kernel<M, false, D><<<grid, 128, 0, s>>>(fI, fC, u, G, pp, left, uf, nint);             \
  } while (0)
  if (dir == 0) GBH_I(0);
  else if (dir == 1) GBH_I((ND > 1 ? 1 : 0));
  else GBH_I((ND > 2 ? 2 : 0));
#undef GBH_I
  return cudaGetLastError();
}

enum { UNFUSED_FLUX = 0, UNFUSED_UFUNC = 1, UNFUSED_UPWIND = 2 };

template <int M, int DIR>
cudaError_t launch_unfused_dir(int kind, int upw, double* out, const double* a, const double* b, const double* c,
                               const double* d, const double* u, const DevGeom& G, const PhysParams& pp,
                               cudaStream_t s) {
  long long npts = 1, nint = 1;
  for (int e = 0; e < G.nd; e++) {
    npts *= G.dim[e] + 2 * G.g;
    nint *= G.dim[e] + (e == DIR ? 1 : 0);
  }
  const int blk = 128;
  if (kind == UNFUSED_FLUX) {
    flux_kernel<M, DIR><<<(unsigned)((npts + blk - 1) / blk), blk, 0, s>>>(out, u, npts, pp);
  } else if (kind == UNFUSED_UFUNC) {
    ufunc_kernel<M><<<(unsigned)((npts + blk - 1) / blk), blk, 0, s>>>(out, u, npts, pp);
  } else {
    unsigned grid = (unsigned)((nint + blk - 1) / blk);
    if (upw == UPW_SWFS && M != MODEL_NS3D)
      upwind_kernel<M, (M != MODEL_NS3D ? UPW_SWFS : UPW_RF), DIR><<<grid, blk, 0, s>>>(out, a, b, c, d, u, G, pp, nint);
    else if (upw == UPW_ROE) upwind_kernel<M, UPW_ROE, DIR><<<grid, blk, 0, s>>>(out, a, b, c, d, u, G, pp, nint);
    else if (upw == UPW_LLF) upwind_kernel<M, UPW_LLF, DIR><<<grid, blk, 0, s>>>(out, a, b, c, d, u, G, pp, nint);
    else if (upw == UPW_RUS && M != MODEL_EULER2D)
      upwind_kernel<M, (M != MODEL_EULER2D ? UPW_RUS : UPW_RF), DIR><<<grid, blk, 0, s>>>(out, a, b, c, d, u, G, pp,
                                                                                       nint);
    else upwind_kernel<M, UPW_RF, DIR><<<grid, blk, 0, s>>>(out, a, b, c, d, u, G, pp, nint);
  }
  return cudaGetLastError();
}

template <int M>
cudaError_t launch_unfused_model(int kind, int dir, int upw, double* out, const double* a, const double* b,
                                 const double* c, const double* d, const double* u, const DevGeom& G,
                                 const PhysParams& pp, cudaStream_t s) {
  constexpr int ND = ModelTraits<M>::ND;
  if (dir == 0) return launch_unfused_dir<M, 0>(kind, upw, out, a, b, c, d, u, G, pp, s);
  if (ND > 1 && dir == 1) return launch_unfused_dir<M, (ND > 1 ? 1 : 0)>(kind, upw, out, a, b, c, d, u, G, pp, s);
  if (ND > 2 && dir == 2) return launch_unfused_dir<M, (ND > 2 ? 2 : 0)>(kind, upw, out, a, b, c, d, u, G, pp, s);
  return cudaErrorInvalidValue;
}

}  // namespace gbh
