// gbh_crweno.cu -- CRWENO5, the compact fifth-order WENO reconstruction
// (hyp_space_scheme crweno5, component-wise): Interp1PrimFifthOrderCRWENO
// (src/InterpolationFunctions/Interp1PrimFifthOrderCRWENO.c:124-237) with the
// weights of WENOFifthOrderCalculateWeights (.c:205-225) and the tridiagonal
// solve of tridiagLU (src/TridiagLU/tridiagLU.c).
//
// Per direction, two launches replace the fused WENO5 kernel:
//
//   cr_solve_kernel   one thread per (grid line, reconstruction, component):
//                     the reconstructions are fL, fR (values f, the cell fluxes of
//                     this direction computed once per point beforehand, weights
//                     from f), uL, uR (values u*, the modified solution, weights
//                     from u).  (Pairing the left and right systems of a quantity
//                     in one thread saved 3.5 % at 160^3 and lost 6 % at 64^3,
//                     where threads are scarce.)
//                     Walking the N+1 interfaces of its line with a six-cell
//                     window, the thread forms each interface's row
//                       (2 w1 + w2) F_{j-1/2} + (w1 + 2 (w2 + w3)) F_{j+1/2} + w3 F_{j+3/2}
//                         = [w1 (f_{j-1} + 5 f_j) + w2 (5 f_j + f_{j+1}) + w3 (f_j + 5 f_{j+1})] / 2
//                     (the reference's rows times 3; right-biased: mirrored), the
//                     weights taken with the CRWENO5 optimal weights (0.2, 0.5, 0.3),
//                     and eliminates the sub-diagonal as it goes (Thomas), storing
//                     the normalised super-diagonal and right-hand side; a backward
//                     sweep then leaves the interface values in place.  On one
//                     rank the first and last interfaces of a line take the explicit
//                     WENO5 value (identity rows, WENO5 optimal weights), as the
//                     reference's single-rank system does.
//   cr_flux_kernel    the fused kernel's back half: per segment of a line, the
//                     upwind flux of each interface from the solved values and the
//                     cell-centre states, the flux difference and the stage epilogue.
//
// With gravity two more reconstructions, sL and sR of the source function with the
// flux's weights, feed the well-balanced source term in cr_flux_kernel.
//
// Layout of the interface values (and of the elimination scratch):
// [interface I][reconstruction k][component v][line], so that the threads of a
// warp, which take consecutive lines, read and write consecutive addresses.
#include "gbh_hyp_impl.cuh"

// Threads per block of the component-wise solve launch (a multiple of 32, at most 128).
// The launch is one wave: small blocks spread its few systems evenly over the SMs
// (64^3: 81,920 systems in 2560 blocks of 32, at most 17 per SM where blocks of 128
// leave 5 on some SMs and 4 on others; 15.14 -> 13.72 ms per RK4 step, 128^3 unchanged).
#ifndef GBH_CR_SOLVE_BLOCK
#define GBH_CR_SOLVE_BLOCK 32
#endif

namespace gbh {

// Normalised weights from the smoothness terms B_k = 4 (beta_k + eps) of one biased
// stencil and, for Borges / Yamaleev-Carpenter, t = 4 tau, with optimal weights
// (c1, c2, c3): Jiang-Shu (ALT false), or the formulation wtype (mapped, Borges,
// Yamaleev-Carpenter, none) -- the formulas of weno5_weights with the optimal weights
// as arguments.
template <bool ALT>
__device__ __forceinline__ void cr_norm(double B1, double B2, double B3, double t, double c1, double c2, double c3,
                                        int wtype, double& w1, double& w2, double& w3) {
  if (ALT && wtype == WENO_W_NONE) {
    w1 = c1;
    w2 = c2;
    w3 = c3;
    return;
  }
  const double q1 = B1 * B1, q2 = B2 * B2, q3 = B3 * B3;
  double a1, a2, a3;
  if (ALT && (wtype == WENO_W_BORGES || wtype == WENO_W_YC)) {
    const double T = t * t;
    a1 = c1 * ((q1 + T) * (q2 * q3));
    a2 = c2 * ((q2 + T) * (q1 * q3));
    a3 = c3 * ((q3 + T) * (q1 * q2));
  } else {
    a1 = c1 * (q2 * q3);
    a2 = c2 * (q1 * q3);
    a3 = c3 * (q1 * q2);
  }
  const double r = nr_rcp(a1 + a2 + a3);
  w1 = a1 * r;
  w2 = a2 * r;
  w3 = a3 * r;
  if (ALT && wtype == WENO_W_MAPPED) {
    const double n1 = w1 * fma(w1, w1 - 3.0 * c1, c1 + c1 * c1);
    const double n2 = w2 * fma(w2, w2 - 3.0 * c2, c2 + c2 * c2);
    const double n3 = w3 * fma(w3, w3 - 3.0 * c3, c3 + c3 * c3);
    const double e1 = fma(w1, 1.0 - 2.0 * c1, c1 * c1);
    const double e2 = fma(w2, 1.0 - 2.0 * c2, c2 * c2);
    const double e3 = fma(w3, 1.0 - 2.0 * c3, c3 * c3);
    const double m1 = n1 * (e2 * e3), m2 = n2 * (e1 * e3), m3 = n3 * (e1 * e2);
    const double rm = nr_rcp(m1 + m2 + m3);
    w1 = m1 * rm;
    w2 = m2 * rm;
    w3 = m3 * rm;
  }
}

// Normalised weights of one biased stencil s = (f_{j-2}, f_{j-1}, f_j, f_{j+1}, f_{j+2}).
template <bool ALT>
__device__ __forceinline__ void cr_weights(const double* s, double c1, double c2, double c3, double eps4, int wtype,
                                           double& w1, double& w2, double& w3) {
  const double k13 = 13.0 / 3.0;
  const double d1 = fma(-2.0, s[1], s[0]) + s[2];
  const double d2 = fma(-2.0, s[2], s[1]) + s[3];
  const double d3 = fma(-2.0, s[3], s[2]) + s[4];
  const double g1 = fma(3.0, s[2], fma(-4.0, s[1], s[0]));
  const double g2 = s[1] - s[3];
  const double g3 = fma(3.0, s[2], fma(-4.0, s[3], s[4]));
  const double B1 = fma(k13 * d1, d1, fma(g1, g1, eps4));
  const double B2 = fma(k13 * d2, d2, fma(g2, g2, eps4));
  const double B3 = fma(k13 * d3, d3, fma(g3, g3, eps4));
  double t = 0.0;
  if (ALT && wtype == WENO_W_BORGES) {
    t = fabs(B1 - B3);
  } else if (ALT && wtype == WENO_W_YC) {
    const double e = d1 - 2.0 * d2 + d3;
    t = 4.0 * (e * e);
  }
  cr_norm<ALT>(B1, B2, B3, t, c1, c2, c3, wtype, w1, w2, w3);
}

// Grid line `tr` along DIR: offset (in points) of its cell 0.
template <int ND, int DIR>
__device__ __forceinline__ long long line_base(const DevGeom& G, long long tr) {
  long long pbase = (long long)G.g * G.stride[DIR];
#pragma unroll
  for (int e = 0; e < ND; e++) {
    if (e == DIR) continue;
    const int ie = (int)(tr % G.dim[e]);
    tr /= G.dim[e];
    pbase += (long long)(ie + G.g) * G.stride[e];
  }
  return pbase;
}

// The modified solution's last component at a point with gravity (the other components
// are u f): Euler1D u_E / S (Euler1DModifiedSolution.c:48, f = 1 / S), NavierStokes3D
// P / (gamma - 1) / g + f rho |v|^2 / 2 (NavierStokes3DModifiedSolution.c:52-66).
template <int M>
__device__ __forceinline__ double grav_ufunc_last(const double* uu, const Prim<M>& q, double f, double g,
                                                  const PhysParams& pp) {
  constexpr int NV = ModelTraits<M>::NV;
  if (M == MODEL_EULER1D) return uu[NV - 1] * f;
  const double vsq = q.vel[0] * q.vel[0] + q.vel[1] * q.vel[1] + q.vel[2] * q.vel[2];
  return fma(q.P * pp.inv_gm1, nr_rcp(g), (0.5 * q.rho * vsq) * f);
}

// The quantity thread (k, v) reconstructs at a cell, and the one its weights see:
// the cell flux component (read from F, the fluxes of this direction computed once
// per point), or the state component and, for the NavierStokes3D energy, the
// modified solution's energy.  GRAV: the u values are the modified solution with
// gravity, and k = 4, 5 reconstruct the source function [0, g e_DIR, g] (g the
// gravity field at the point) with the weights of the flux component.
template <int M, int DIR, bool GRAV>
__device__ __forceinline__ void cr_cell(const double* __restrict__ src, const double* __restrict__ fsrc, int k,
                                        int v, const PhysParams& pp, long long pt, double& val, double& wv) {
  constexpr int NV = ModelTraits<M>::NV;
  if (k < 2) {
    val = wv = fsrc[v];
  } else if (GRAV && k >= 4) {
    wv = fsrc[v];
    val = (v == 1 + DIR || v == NV - 1) ? pp.gg[pt] : 0.0;
  } else if (GRAV) {
    double uu[NV];
#pragma unroll
    for (int e = 0; e < NV; e++) uu[e] = src[e];
    double x = uu[0];
#pragma unroll
    for (int e = 1; e < NV; e++)
      if (v == e) x = uu[e];
    wv = x;
    const double f = pp.gf[pt];
    if (v == NV - 1) {
      Prim<M> q = to_prim<M>(uu, pp);
      val = grav_ufunc_last<M>(uu, q, f, pp.gg[pt], pp);
    } else {
      val = x * f;
    }
  } else {
    double uu[NV];
#pragma unroll
    for (int e = 0; e < NV; e++) uu[e] = src[e];
    double x = uu[0];
#pragma unroll
    for (int e = 1; e < NV; e++)
      if (v == e) x = uu[e];
    wv = x;
    if (M == MODEL_NS3D && v == NV - 1) {
      // the modified solution's energy (NavierStokes3DModifiedSolution.c:65)
      Prim<M> q = to_prim<M>(uu, pp);
      val = ufunc_energy<M>(q, pp, uu[NV - 1]);
    } else {
      val = x;
    }
  }
}

template <int M, int DIR, bool ALTW, bool GRAV>
__global__ void __launch_bounds__(128)
cr_solve_kernel(const double* __restrict__ U, const double* __restrict__ F, DevGeom G, PhysParams pp,
                double* __restrict__ X, double* __restrict__ Cp, long long ntrans) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND, R = GRAV ? 6 : 4;
  const long long nsys = ntrans * R * NV;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nsys) return;
  const long long line = tid % ntrans;
  const int kv = (int)(tid / ntrans);
  const int v = kv % NV, k = kv / NV;
  const bool left = (k % 2) == 0;
  const long long pbase = line_base<ND, DIR>(G, line);
  const int N = G.dim[DIR];
  const long long sd = G.stride[DIR];
  const int lo = G.bclo[DIR], hi = G.bchi[DIR];
  const double eps4 = 4.0 * pp.eps;
  const double s6 = 1.0 / 6.0;

  // window of cells I-3 .. I+2 for interface I
  double wval[6], wwv[6];
  auto load = [&](int i, int slot) {
    const long long pt = pbase + (long long)fold_index(i, N, lo, hi) * sd;
    cr_cell<M, DIR, GRAV>(U + pt * NV, F + pt * NV, k, v, pp, pt, wval[slot], wwv[slot]);
  };
#pragma unroll
  for (int p = 0; p < 5; p++) load(p - 3, p + 1);

  double cprev = 0.0, xprev = 0.0;
  for (int I = 0; I <= N; I++) {
#pragma unroll
    for (int p = 0; p < 5; p++) {
      wval[p] = wval[p + 1];
      wwv[p] = wwv[p + 1];
    }
    load(I + 2, 5);
    // the biased stencil (f_{j-2}, f_{j-1}, f_j, f_{j+1}, f_{j+2}) of this interface
    double sw[5], sv[5];
#pragma unroll
    for (int p = 0; p < 5; p++) {
      sw[p] = left ? wwv[p] : wwv[5 - p];
      sv[p] = left ? wval[p] : wval[5 - p];
    }
    const bool bnd = (I == 0) || (I == N);
    double w1, w2, w3;
    if (bnd) cr_weights<ALTW>(sw, 0.1, 0.6, 0.3, eps4, pp.wtype, w1, w2, w3);
    else cr_weights<ALTW>(sw, 0.2, 0.5, 0.3, eps4, pp.wtype, w1, w2, w3);
    double cI, xI;
    if (bnd) {
      // explicit WENO5 value: identity row
      const double f1 = fma(2.0, sv[0], fma(-7.0, sv[1], 11.0 * sv[2]));
      const double f2 = fma(5.0, sv[2], fma(2.0, sv[3], -sv[1]));
      const double f3 = fma(5.0, sv[3], fma(2.0, sv[2], -sv[4]));
      // b = 1, a = c = 0: the elimination leaves the value
      cI = 0.0;
      xI = fma(w1, f1, fma(w2, f2, w3 * f3)) * s6;
    } else {
      const double f1 = fma(5.0, sv[2], sv[1]);
      const double f2 = fma(5.0, sv[2], sv[3]);
      const double f3 = fma(5.0, sv[3], sv[2]);
      const double r = 0.5 * fma(w1, f1, fma(w2, f2, w3 * f3));
      const double a = left ? fma(2.0, w1, w2) : w3;
      const double c = left ? w3 : fma(2.0, w1, w2);
      const double b = fma(2.0, w2 + w3, w1);
      const double inv = nr_rcp(fma(-a, cprev, b));
      cI = c * inv;
      xI = fma(-a, xprev, r) * inv;
    }
    const long long o = (long long)I * nsys + tid;
    if (I < N) Cp[o] = cI;
    X[o] = xI;
    cprev = cI;
    xprev = xI;
  }
  // back-substitution: X[I] = X[I] - Cp[I] X[I+1]
  double x = xprev;
  for (int I = N - 1; I >= 0; I--) {
    const long long o = (long long)I * nsys + tid;
    x = fma(-Cp[o], x, X[o]);
    X[o] = x;
  }
}

// Characteristic CRWENO5 (Interp1PrimFifthOrderCRWENOChar.c:139-230): one thread per
// (grid line, reconstruction).  At interface I the rows of the nvars characteristic
// fields share the left eigenvectors L of the Roe average of the two cell-centre
// states: diag(a) L F_{I-1} + diag(b) L F_I + diag(c) L F_{I+1} = r, with per field
// the component-wise coefficients (here times 3) and r the weighted compact candidates
// of the characteristic stencil L f (weights of the characteristic stencils, CRWENO5 /
// WENO5 optimal weights); the first and last interfaces: L F = r (explicit WENO5).
// Block elimination, normalised: with F_{I-1} = y'_{I-1} - C'_{I-1} F_I,
//   D = diag(b) L - diag(a) (L C'_{I-1}),  D [C'_I | y'_I] = [diag(c) L | r - diag(a) L y'_{I-1}],
// solved by Gaussian elimination with partial pivoting, C'_I and y'_I stored per
// interface (nvars^2 + nvars doubles, [interface][entry][system] for coalescing),
// then F_I = y'_I - C'_I F_{I+1}
// backwards into X in the component-wise layout, which cr_flux_kernel reads.
// GRAV: the u values are the modified solution with gravity, and reconstructions
// k = 4, 5 solve for the source function [0, g e_DIR, g] with the flux's weights
// (the same blocks as k = 0, 1, another right-hand side).
template <int M, int DIR, bool ALTW, bool GRAV>
__global__ void __launch_bounds__(64)
cr_char_solve_kernel(const double* __restrict__ U, DevGeom G, PhysParams pp, double* __restrict__ X,
                     double* __restrict__ S, long long ntrans) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND, NE = NV * NV + NV, R = GRAV ? 6 : 4;
  const long long nsys = ntrans * R;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nsys) return;
  const long long line = tid % ntrans;
  const int k = (int)(tid / ntrans);
  const bool sx = GRAV && k >= 4;
  const bool left = (k % 2) == 0, fx = k < 2 || sx;
  const long long pbase = line_base<ND, DIR>(G, line);
  const int N = G.dim[DIR];
  const long long sd = G.stride[DIR];
  const int lo = G.bclo[DIR], hi = G.bchi[DIR];
  const double eps4 = 4.0 * pp.eps;
  const double s6 = 1.0 / 6.0;
  const long long nX = ntrans * R * NV;

  // window of cells I-3 .. I+2: the weights' quantity (f or u), the modified energy
  // (u reconstructions of NavierStokes3D; with GRAV of both models) or the gravity
  // field (source reconstructions), the modified solution's factor f (GRAV), and the
  // Roe-average ingredients
  double wq[6][NV], wE[6], wF[6];
  RoeSide rs[6];
  auto load = [&](int i, int slot) {
    const long long pt = pbase + (long long)fold_index(i, N, lo, hi) * sd;
    double uu[NV];
#pragma unroll
    for (int e = 0; e < NV; e++) uu[e] = U[pt * NV + e];
    Prim<M> q = to_prim<M>(uu, pp);
    rs[slot] = roe_side<M>(q);
    if (fx) {
      cell_flux<M, DIR>(q, wq[slot]);
    } else {
#pragma unroll
      for (int e = 0; e < NV; e++) wq[slot][e] = uu[e];
    }
    if (GRAV) {
      wF[slot] = pp.gf[pt];
      wE[slot] = sx ? pp.gg[pt] : (fx ? wq[slot][NV - 1] : grav_ufunc_last<M>(uu, q, wF[slot], pp.gg[pt], pp));
    } else {
      wE[slot] = (!fx && M == MODEL_NS3D) ? ufunc_energy<M>(q, pp, uu[NV - 1]) : wq[slot][NV - 1];
    }
  };
#pragma unroll
  for (int p = 0; p < 5; p++) load(p - 3, p + 1);

  double Cp[NV][NV], yp[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) {
    yp[i] = 0.0;
#pragma unroll
    for (int j = 0; j < NV; j++) Cp[i][j] = 0.0;
  }
  for (int I = 0; I <= N; I++) {
#pragma unroll
    for (int p = 0; p < 5; p++) {
#pragma unroll
      for (int e = 0; e < NV; e++) wq[p][e] = wq[p + 1][e];
      wE[p] = wE[p + 1];
      if (GRAV) wF[p] = wF[p + 1];
      rs[p] = rs[p + 1];
    }
    load(I + 2, 5);
    const Eig E = roe_eig<M, DIR>(rs[2], rs[3], pp);
    const bool bnd = (I == 0) || (I == N);
    // characteristic stencils (f_{j-2} .. f_{j+2} of this bias): weights' and values'
    double pw[5][NV], pv[5][NV];
#pragma unroll
    for (int m = 0; m < 5; m++) {
      const int slot = left ? m : 5 - m;
      projL<M, DIR>(E, pp, wq[slot], pw[m]);
      if (GRAV && sx) {
        double t[NV];
#pragma unroll
        for (int e = 0; e < NV; e++) t[e] = (e == 1 + DIR || e == NV - 1) ? wE[slot] : 0.0;
        projL<M, DIR>(E, pp, t, pv[m]);
      } else if (GRAV && !fx) {
        double t[NV];
#pragma unroll
        for (int e = 0; e < NV - 1; e++) t[e] = wq[slot][e] * wF[slot];
        t[NV - 1] = wE[slot];
        projL<M, DIR>(E, pp, t, pv[m]);
      } else if (!fx && M == MODEL_NS3D) {
        double t[NV];
#pragma unroll
        for (int e = 0; e < NV; e++) t[e] = wq[slot][e];
        t[NV - 1] = wE[slot];
        projL<M, DIR>(E, pp, t, pv[m]);
      } else {
#pragma unroll
        for (int e = 0; e < NV; e++) pv[m][e] = pw[m][e];
      }
    }
    double ca[NV], cb[NV], cc[NV], r[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double sw[5], sv[5];
#pragma unroll
      for (int m = 0; m < 5; m++) {
        sw[m] = pw[m][v];
        sv[m] = pv[m][v];
      }
      double w1, w2, w3;
      if (bnd) {
        cr_weights<ALTW>(sw, 0.1, 0.6, 0.3, eps4, pp.wtype, w1, w2, w3);
        const double f1 = fma(2.0, sv[0], fma(-7.0, sv[1], 11.0 * sv[2]));
        const double f2 = fma(5.0, sv[2], fma(2.0, sv[3], -sv[1]));
        const double f3 = fma(5.0, sv[3], fma(2.0, sv[2], -sv[4]));
        r[v] = fma(w1, f1, fma(w2, f2, w3 * f3)) * s6;
        ca[v] = cc[v] = 0.0;
        cb[v] = 1.0;
      } else {
        cr_weights<ALTW>(sw, 0.2, 0.5, 0.3, eps4, pp.wtype, w1, w2, w3);
        const double f1 = fma(5.0, sv[2], sv[1]);
        const double f2 = fma(5.0, sv[2], sv[3]);
        const double f3 = fma(5.0, sv[3], sv[2]);
        r[v] = 0.5 * fma(w1, f1, fma(w2, f2, w3 * f3));
        const double lo3 = fma(2.0, w1, w2);
        ca[v] = left ? lo3 : w3;
        cc[v] = left ? w3 : lo3;
        cb[v] = fma(2.0, w2 + w3, w1);
      }
    }
    double y[NV], Cn[NV][NV];
    if (bnd) {
      // L F = r: F = R r
      projR<M, DIR>(E, r, y);
#pragma unroll
      for (int i = 0; i < NV; i++)
#pragma unroll
        for (int j = 0; j < NV; j++) Cn[i][j] = 0.0;
    } else {
      // D = diag(b) L - diag(a) L C', right-hand sides diag(c) L and r - diag(a) L y'
      double D[NV][NV], Rh[NV][NV + 1];
#pragma unroll
      for (int j = 0; j < NV; j++) {
        double ej[NV], lj[NV], col[NV], mj[NV];
#pragma unroll
        for (int e = 0; e < NV; e++) {
          ej[e] = (e == j) ? 1.0 : 0.0;
          col[e] = Cp[e][j];
        }
        projL<M, DIR>(E, pp, ej, lj);   // column j of L
        projL<M, DIR>(E, pp, col, mj);  // column j of L C'
#pragma unroll
        for (int i = 0; i < NV; i++) {
          D[i][j] = fma(-ca[i], mj[i], cb[i] * lj[i]);
          Rh[i][j] = cc[i] * lj[i];
        }
      }
      double ly[NV];
      projL<M, DIR>(E, pp, yp, ly);
#pragma unroll
      for (int i = 0; i < NV; i++) Rh[i][NV] = fma(-ca[i], ly[i], r[i]);
      // Gaussian elimination with partial pivoting (the characteristic fields are
      // ordered differently from the reference's eigenvector rows, so the pivots the
      // reference meets without pivoting are not the leading ones here: at rest the
      // first field's row of L starts with a zero), then back-substitution
      double dinv[NV];
#pragma unroll
      for (int i = 0; i < NV; i++) {
#pragma unroll
        for (int p = i + 1; p < NV; p++) {
          const bool sw = fabs(D[p][i]) > fabs(D[i][i]);
#pragma unroll
          for (int q = i; q < NV; q++) {
            const double t = D[i][q];
            D[i][q] = sw ? D[p][q] : t;
            D[p][q] = sw ? t : D[p][q];
          }
#pragma unroll
          for (int q = 0; q <= NV; q++) {
            const double t = Rh[i][q];
            Rh[i][q] = sw ? Rh[p][q] : t;
            Rh[p][q] = sw ? t : Rh[p][q];
          }
        }
        dinv[i] = nr_rcp(D[i][i]);
#pragma unroll
        for (int j = i + 1; j < NV; j++) {
          const double f = D[j][i] * dinv[i];
#pragma unroll
          for (int q = i + 1; q < NV; q++) D[j][q] = fma(-f, D[i][q], D[j][q]);
#pragma unroll
          for (int q = 0; q <= NV; q++) Rh[j][q] = fma(-f, Rh[i][q], Rh[j][q]);
        }
      }
#pragma unroll
      for (int i = NV - 1; i >= 0; i--) {
#pragma unroll
        for (int q = 0; q <= NV; q++) {
          double t = Rh[i][q];
#pragma unroll
          for (int j = i + 1; j < NV; j++) t = fma(-D[i][j], Rh[j][q], t);
          Rh[i][q] = t * dinv[i];
        }
      }
#pragma unroll
      for (int i = 0; i < NV; i++) {
        y[i] = Rh[i][NV];
#pragma unroll
        for (int j = 0; j < NV; j++) Cn[i][j] = Rh[i][j];
      }
    }
    double* so = S + (long long)I * NE * nsys + tid;
#pragma unroll
    for (int i = 0; i < NV; i++) {
      so[(long long)i * nsys] = y[i];
#pragma unroll
      for (int j = 0; j < NV; j++) so[(long long)(NV + i * NV + j) * nsys] = Cn[i][j];
      yp[i] = y[i];
#pragma unroll
      for (int j = 0; j < NV; j++) Cp[i][j] = Cn[i][j];
    }
  }
  // back-substitution: F_N = y'_N, F_I = y'_I - C'_I F_{I+1}
  double x[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) x[i] = yp[i];
  {
    double* xo = X + (long long)N * nX + (long long)k * NV * ntrans + line;
#pragma unroll
    for (int i = 0; i < NV; i++) xo[(long long)i * ntrans] = x[i];
  }
  for (int I = N - 1; I >= 0; I--) {
    const double* so = S + (long long)I * NE * nsys + tid;
    double xn[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) {
      double t = so[(long long)i * nsys];
#pragma unroll
      for (int j = 0; j < NV; j++) t = fma(-so[(long long)(NV + i * NV + j) * nsys], x[j], t);
      xn[i] = t;
    }
    double* xo = X + (long long)I * nX + (long long)k * NV * ntrans + line;
#pragma unroll
    for (int i = 0; i < NV; i++) {
      x[i] = xn[i];
      xo[(long long)i * ntrans] = x[i];
    }
  }
}

// GRAV: the dissipation scaled by max(g_L, g_R) of the gravity field (Euler1DUpwind.c:79-82,
// NavierStokes3DUpwind.c:407) and, along a direction with gravity, the well-balanced
// source term (Euler1DSource.c:58-76, NavierStokes3DSource.c:73-101): the average of
// the source function's left and right values (SourceUpwind) differenced per cell and
// scaled by [0, rho RT e_DIR, rho RT v_DIR] f (RT = 1, f = 1 / S for Euler1D), subtracted
// from this direction's term.
template <int M, int UPW, int DIR, bool GRAV>
__global__ void __launch_bounds__(128)
cr_flux_kernel(const double* __restrict__ U, double* __restrict__ H, const double* __restrict__ dxinv, DevGeom G,
               PhysParams pp, StageEpi ep, const double* __restrict__ X, int seg, int nseg, long long ntrans) {
  constexpr int NV = ModelTraits<M>::NV, ND = ModelTraits<M>::ND, R = GRAV ? 6 : 4;
  constexpr bool CC = NeedCC<M, false, UPW>::value;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= ntrans * (long long)nseg) return;
  const long long line = tid % ntrans;
  const int sg = (int)(tid / ntrans);
  const long long pbase = line_base<ND, DIR>(G, line);
  const int N = G.dim[DIR];
  const long long sd = G.stride[DIR];
  const int lo = G.bclo[DIR], hi = G.bchi[DIR];
  const int I0 = sg * seg;
  const int I1 = min(I0 + seg, N);
  const long long nsys = ntrans * R * NV;
  const bool src_dir = GRAV && pp.grav[DIR] != 0.0 && (ep.mode != EPI_HYP || ep.with_source);

  // gL, gR: the gravity field at the interface's two cells (GRAV)
  auto aux = [&](int i, double& gv) {
    CellAux<M> a;
    const long long pt = pbase + (long long)fold_index(i, N, lo, hi) * sd;
    double uu[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uu[v] = U[pt * NV + v];
    Prim<M> q = to_prim<M>(uu, pp);
    if (CC) a.rs = roe_side<M>(q);
    if (UPW == UPW_RUS) a.c = rusanov_speed<M, DIR>(q, pp);
    else if (M == MODEL_EULER1D && UPW != UPW_ROE) a.c = sound_speed<M>(q, pp);
    if (GRAV) gv = pp.gg[pt];
    return a;
  };
  double gL = 1.0, gR = 1.0;
  CellAux<M> axL = aux(I0 - 1, gL);
  double fIp[NV], SI[NV], SIp[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) SI[v] = SIp[v] = 0.0;
  for (int I = I0; I <= I1; I++) {
    const CellAux<M> axR = aux(I, gR);
    double fL[NV], fR[NV], uL[NV], uR[NV];
    const double* q = X + (long long)I * nsys + line;
#pragma unroll
    for (int v = 0; v < NV; v++) {
      fL[v] = q[(0 * NV + v) * ntrans];
      fR[v] = q[(1 * NV + v) * ntrans];
      uL[v] = q[(2 * NV + v) * ntrans];
      uR[v] = q[(3 * NV + v) * ntrans];
      if (src_dir) SI[v] = 0.5 * (q[(4 * NV + v) * ntrans] + q[(5 * NV + v) * ntrans]);
    }
    Eig Ecc;
    if (CC) Ecc = roe_eig<M, DIR>(axL.rs, axR.rs, pp);
    double fI[NV];
    upwind_iface<M, false, UPW, DIR>(fL, fR, uL, uR, Ecc, axL, axR, pp, fI, GRAV ? fmax(gL, gR) : 1.0);
    boundary_flux<NV>(ep, I, N, line, ntrans, fI);
    if (I > I0) {
      const int c = I - 1;
      const long long pc = pbase + (long long)c * sd, off = pc * NV;
      const double dxi = dxinv[G.g + c];
      double h[NV];
#pragma unroll
      for (int v = 0; v < NV; v++) h[v] = dxi * (fI[v] - fIp[v]);
      if (src_dir) {
        // [0, rho RT e_DIR, rho RT v_DIR] f of the cell, as the fused WENO5 kernel
        const double rho = U[off], rRT = rho * pp.RT, f = pp.gf[pc];
        const double vd = rho == 0.0 ? 0.0 : U[off + 1 + DIR] * nr_rcp(rho);
        double term[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) term[v] = 0.0;
        term[1 + DIR] = rRT * f;
        term[NV - 1] = (rRT * vd) * f;
#pragma unroll
        for (int v = 0; v < NV; v++) h[v] = fma(-term[v] * (SI[v] - SIp[v]), dxi, h[v]);  // rhs = -hyp + source
      }
      stage_epilogue<NV>(ep, H, off, h);
    }
#pragma unroll
    for (int v = 0; v < NV; v++) {
      fIp[v] = fI[v];
      SIp[v] = SI[v];
    }
    axL = axR;
    gL = gR;
  }
}

template <int M, int DIR, bool ALTW, int UPW, bool GRAV = false>
static cudaError_t cr_dir(bool chr, const double* U, double* H, const double* dxinv_dir, const DevGeom& G,
                          const PhysParams& pp, const StageEpi& ep, const HypLaunch& L, double* X, double* Cp,
                          double* Fc, cudaStream_t s) {
  constexpr int NV = ModelTraits<M>::NV, R = GRAV ? 6 : 4;
  long long ntrans = 1;
  for (int e = 0; e < G.nd; e++)
    if (e != DIR) ntrans *= G.dim[e];
  const long long nsys = ntrans * R * NV;
  if (chr) {
    const long long nchr = ntrans * R;
    cr_char_solve_kernel<M, DIR, ALTW, GRAV><<<(unsigned)((nchr + 63) / 64), 64, 0, s>>>(U, G, pp, X, Cp, ntrans);
  } else {
    // the cell fluxes of this direction once per point, then the solves
    long long npts = 1;
    for (int e = 0; e < G.nd; e++) npts *= G.dim[e] + 2 * G.g;
    flux_kernel<M, DIR><<<(unsigned)((npts + 127) / 128), 128, 0, s>>>(Fc, U, npts, pp);
    cudaError_t e0 = cudaGetLastError();
    if (e0 != cudaSuccess) return e0;
    constexpr int SB = GBH_CR_SOLVE_BLOCK;
    static_assert(SB % 32 == 0 && SB <= 128, "the solve kernel's launch bounds are 128 threads");
    cr_solve_kernel<M, DIR, ALTW, GRAV><<<(unsigned)((nsys + SB - 1) / SB), SB, 0, s>>>(U, Fc, G, pp, X, Cp, ntrans);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int seg = L.seg > 0 ? L.seg : 32;
  const int nseg = (G.dim[DIR] + seg - 1) / seg;
  const long long nthr = ntrans * nseg;
  const int block = L.block > 0 ? L.block : 128;
  cr_flux_kernel<M, UPW, DIR, GRAV><<<(unsigned)((nthr + block - 1) / block), block, 0, s>>>(U, H, dxinv_dir, G, pp,
                                                                                           ep, X, seg, nseg, ntrans);
  return cudaGetLastError();
}

template <int M, int DIR, bool ALTW>
static cudaError_t cr_dir_upw(bool chr, int upw, const double* U, double* H, const double* dx, const DevGeom& G,
                              const PhysParams& pp, const StageEpi& ep, const HypLaunch& L, double* X, double* Cp,
                              double* Fc, cudaStream_t s) {
  switch (upw) {
    case UPW_ROE: return cr_dir<M, DIR, ALTW, UPW_ROE>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    case UPW_LLF: return cr_dir<M, DIR, ALTW, UPW_LLF>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    case UPW_RF: return cr_dir<M, DIR, ALTW, UPW_RF>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    case UPW_SWFS:
      if (M == MODEL_NS3D) return cudaErrorInvalidValue;  // NavierStokes3D has no Steger-Warming
      return cr_dir<M, DIR, ALTW, (M != MODEL_NS3D ? UPW_SWFS : UPW_RF)>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    default:
      if (M == MODEL_EULER2D) return cudaErrorInvalidValue;  // Euler2D has no Rusanov
      return cr_dir<M, DIR, ALTW, (M == MODEL_EULER2D ? UPW_ROE : UPW_RUS)>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
  }
}

template <int M, bool ALTW>
static cudaError_t cr_model(bool chr, int dir, int upw, const double* U, double* H, const double* dx,
                            const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L, double* X,
                            double* Cp, double* Fc, cudaStream_t s) {
  constexpr int ND = ModelTraits<M>::ND;
  if (dir == 0) return cr_dir_upw<M, 0, ALTW>(chr, upw, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
  if (ND > 1 && dir == 1) return cr_dir_upw<M, (ND > 1 ? 1 : 0), ALTW>(chr, upw, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
  if (ND > 2 && dir == 2) return cr_dir_upw<M, (ND > 2 ? 2 : 0), ALTW>(chr, upw, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
  return cudaErrorInvalidValue;
}

// With gravity: Euler1D (Roe, LLF) and NavierStokes3D (Rusanov, the only upwinding the
// reference allows with gravity), any direction.
template <int M, bool ALTW>
static cudaError_t cr_model_grav(bool chr, int dir, int upw, const double* U, double* H, const double* dx,
                                 const DevGeom& G, const PhysParams& pp, const StageEpi& ep, const HypLaunch& L,
                                 double* X, double* Cp, double* Fc, cudaStream_t s) {
  if constexpr (M == MODEL_EULER1D) {
    if (dir != 0) return cudaErrorInvalidValue;
    if (upw == UPW_LLF) return cr_dir<M, 0, ALTW, UPW_LLF, true>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    if (upw == UPW_ROE) return cr_dir<M, 0, ALTW, UPW_ROE, true>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    return cudaErrorInvalidValue;
  } else if constexpr (M == MODEL_NS3D) {
    if (upw != UPW_RUS) return cudaErrorInvalidValue;
    if (dir == 0) return cr_dir<M, 0, ALTW, UPW_RUS, true>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    if (dir == 1) return cr_dir<M, 1, ALTW, UPW_RUS, true>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    if (dir == 2) return cr_dir<M, 2, ALTW, UPW_RUS, true>(chr, U, H, dx, G, pp, ep, L, X, Cp, Fc, s);
    return cudaErrorInvalidValue;
  } else {
    return cudaErrorInvalidValue;  // Euler2D has no gravity
  }
}

// Scratch per direction (doubles), with R = 4 reconstructions (6 with gravity: the
// source function's two): X holds (N+1) * lines * R * nvars interface values; the
// second array the elimination: (N+1) * lines * R * nvars (component-wise) or
// (N+1) * lines * R * (nvars^2 + nvars) (characteristic).
size_t crweno_scratch_doubles(int nvars, int n_interfaces, long long lines, bool chr, bool second, bool grav) {
  const size_t R = grav ? 6 : 4;
  if (!second || !chr) return (size_t)n_interfaces * (size_t)lines * R * (size_t)nvars;
  return (size_t)n_interfaces * (size_t)lines * R * (size_t)(nvars * nvars + nvars);
}

// One direction of the hyperbolic term with CRWENO5, component-wise or characteristic,
// with gravity when `grav` (pp's gravity fields set).
// Fc: a ghosted state-sized array for the cell fluxes (component-wise form).
cudaError_t launch_hyp_crweno(int model, int dir, int upw, bool chr, bool grav, const double* U, double* H,
                              const double* dxinv_dir, const DevGeom& G, const PhysParams& pp, const StageEpi& ep,
                              const HypLaunch& L, double* X, double* Cp, double* Fc, cudaStream_t s) {
  const bool alt = pp.wtype != WENO_W_JS;
  if (grav) {
    if (!pp.gf || !pp.gg) return cudaErrorInvalidValue;
    if (model == MODEL_EULER1D)
      return alt ? cr_model_grav<MODEL_EULER1D, true>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s)
                 : cr_model_grav<MODEL_EULER1D, false>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s);
    if (model == MODEL_NS3D)
      return alt ? cr_model_grav<MODEL_NS3D, true>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s)
                 : cr_model_grav<MODEL_NS3D, false>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s);
    return cudaErrorInvalidValue;
  }
  if (model == MODEL_EULER1D)
    return alt ? cr_model<MODEL_EULER1D, true>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s)
               : cr_model<MODEL_EULER1D, false>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s);
  if (model == MODEL_EULER2D)
    return alt ? cr_model<MODEL_EULER2D, true>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s)
               : cr_model<MODEL_EULER2D, false>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s);
  return alt ? cr_model<MODEL_NS3D, true>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s)
             : cr_model<MODEL_NS3D, false>(chr, dir, upw, U, H, dxinv_dir, G, pp, ep, L, X, Cp, Fc, s);
}

}  // namespace gbh
