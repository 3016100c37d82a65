// gbh_adjoint.cu -- derivatives of the Euler2D right-hand side (component-wise
// WENO5 with Jiang-Shu weights + Roe upwinding, periodic / extrapolate
// boundaries folded into the halo) and of the explicit Runge-Kutta step.
//
//  * rhs_vjp_kernel: reverse mode (k_bar -> u_bar += (dF/du)^T k_bar), written
//    by hand from the forward formulas of gbh_device.cuh: the flux difference,
//    the Roe flux (through the Roe average, the eigen-structure and Harten's
//    entropy fix), the left/right WENO5 pair (through the nonlinear weights)
//    and the cell flux.  Each thread walks a segment of a grid line like the
//    forward kernel, recomputing the forward values of each interface, and
//    scatters the stencil adjoints with atomic adds (ghost cells fold onto the
//    interior cells they copy).  Its tile form (rhs_vjp_tile_kernel, small grids)
//    stores per-tile shares instead, summed in a fixed order by
//    vjp_slot_gather_kernel: bit-identical results from run to run.
//  * rhs_jvp_kernel: forward mode (du -> (F(u), dF/du du)) in dual numbers,
//    written independently in the reference's own form (per-side Jiang-Shu
//    weights, dense eigenvector matrices and R |Lambda| L of the Roe flux,
//    Euler2DUpwind.c:10-66, include/physicalmodels/euler2d.h:70-230), so that
//    <J v, w> = <v, J^T w> tests the adjoint against an independent derivative.
// The reference has no derivative code; these follow its discrete operator.
#include <cstring>
#include <vector>

#include "gbh_internal.h"

namespace gbh {
cudaError_t launch_hyp_euler2d_wide_tape(int, const double*, double*, const double*, const DevGeom&,
                                         const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);
cudaError_t launch_hyp_euler2d(int, int, int, const double*, double*, const double*, const DevGeom&,
                               const PhysParams&, const StageEpi&, const HypLaunch&, cudaStream_t);

constexpr int NV2 = 4;

__device__ __forceinline__ int fold2(int i, int N, int lo, int hi) {
  if (i < 0) return lo == FOLD_PERIODIC ? i + N : (lo == FOLD_MIRROR ? -1 - i : i);
  if (i >= N) return hi == FOLD_PERIODIC ? i - N : (hi == FOLD_MIRROR ? 2 * N - 1 - i : i);
  return i;
}

// ---------------------------------------------------------------------------
// Reverse of the WENO5 left/right pair (forward: weno5_pair in gbh_device.cuh).
// gL, gR: adjoints of the two outputs; wb, vb: adjoint accumulators of the
// weight stencil and of the value stencil (the same array when w == v).
// ---------------------------------------------------------------------------
// TP: the smoothness terms B and the normalisation reciprocals come from the
// forward kernel's wide tape tp[0..7] (weno5_pair_tape) instead of being recomputed
// (bit-identical values: the same expressions).
template <bool TP>
__device__ __forceinline__ void weno5_pair_vjp_impl(const double* w, const double* v, double eps4, double gL,
                                                    double gR, double* wb, double* vb, const double* tp) {
  const double k13 = 13.0 / 3.0;
  double d1 = fma(-2.0, w[1], w[0]) + w[2];
  double d2 = fma(-2.0, w[2], w[1]) + w[3];
  double d3 = fma(-2.0, w[3], w[2]) + w[4];
  double d4 = fma(-2.0, w[4], w[3]) + w[5];
  double gL1 = fma(3.0, w[2], fma(-4.0, w[1], w[0]));
  double gL2 = w[1] - w[3];
  double gL3 = fma(3.0, w[2], fma(-4.0, w[3], w[4]));
  double gR1 = fma(3.0, w[3], fma(-4.0, w[4], w[5]));
  double gR2 = w[4] - w[2];
  double gR3 = fma(3.0, w[3], fma(-4.0, w[2], w[1]));
  double BL1, BL2, BL3, BR1, BR2, BR3;
  if (TP) {
    BL1 = tp[0];
    BL2 = tp[1];
    BL3 = tp[2];
    BR1 = tp[3];
    BR2 = tp[4];
    BR3 = tp[5];
  } else {
    BL1 = fma(k13 * d1, d1, fma(gL1, gL1, eps4));
    BL2 = fma(k13 * d2, d2, fma(gL2, gL2, eps4));
    BL3 = fma(k13 * d3, d3, fma(gL3, gL3, eps4));
    BR1 = fma(k13 * d4, d4, fma(gR1, gR1, eps4));
    BR2 = fma(k13 * d3, d3, fma(gR2, gR2, eps4));
    BR3 = fma(k13 * d2, d2, fma(gR3, gR3, eps4));
  }
  double qL1 = BL1 * BL1, qL2 = BL2 * BL2, qL3 = BL3 * BL3;
  double qR1 = BR1 * BR1, qR2 = BR2 * BR2, qR3 = BR3 * BR3;
  double aL1 = qL2 * qL3, aL2 = qL1 * qL3, aL3 = qL1 * qL2;
  double aR1 = qR2 * qR3, aR2 = qR1 * qR3, aR3 = qR1 * qR2;
  double cL1 = fma(2.0, v[0], fma(-7.0, v[1], 11.0 * v[2]));
  double cR1 = fma(2.0, v[5], fma(-7.0, v[4], 11.0 * v[3]));
  double cA = fma(5.0, v[2], fma(2.0, v[3], -v[1]));
  double cB = fma(5.0, v[3], fma(2.0, v[2], -v[4]));
  double nL = fma(aL1, cL1, fma(6.0 * aL2, cA, (3.0 * aL3) * cB));
  double nR = fma(aR1, cR1, fma(6.0 * aR2, cB, (3.0 * aR3) * cA));
  double rL, rR;
  if (TP) {
    rL = tp[6];
    rR = tp[7];
  } else {
    double DL = fma(36.0, aL2, fma(18.0, aL3, 6.0 * aL1));
    double DR = fma(36.0, aR2, fma(18.0, aR3, 6.0 * aR1));
    rL = nr_rcp(DL);
    rR = nr_rcp(DR);
  }
  double oL = nL * rL, oR = nR * rR;
  // reverse
  double nLb = gL * rL, DLb = -gL * oL * rL;
  double nRb = gR * rR, DRb = -gR * oR * rR;
  double aL1b = fma(nLb, cL1, 6.0 * DLb), aL2b = fma(6.0 * nLb, cA, 36.0 * DLb), aL3b = fma(3.0 * nLb, cB, 18.0 * DLb);
  double aR1b = fma(nRb, cR1, 6.0 * DRb), aR2b = fma(6.0 * nRb, cB, 36.0 * DRb), aR3b = fma(3.0 * nRb, cA, 18.0 * DRb);
  double cL1b = nLb * aL1, cR1b = nRb * aR1;
  double cAb = fma(6.0 * nLb, aL2, 3.0 * nRb * aR3);
  double cBb = fma(3.0 * nLb, aL3, 6.0 * nRb * aR2);
  double qL1b = fma(aL2b, qL3, aL3b * qL2), qL2b = fma(aL1b, qL3, aL3b * qL1), qL3b = fma(aL1b, qL2, aL2b * qL1);
  double qR1b = fma(aR2b, qR3, aR3b * qR2), qR2b = fma(aR1b, qR3, aR3b * qR1), qR3b = fma(aR1b, qR2, aR2b * qR1);
  double BL1b = 2.0 * BL1 * qL1b, BL2b = 2.0 * BL2 * qL2b, BL3b = 2.0 * BL3 * qL3b;
  double BR1b = 2.0 * BR1 * qR1b, BR2b = 2.0 * BR2 * qR2b, BR3b = 2.0 * BR3 * qR3b;
  double d1b = 2.0 * k13 * d1 * BL1b;
  double d2b = 2.0 * k13 * d2 * (BL2b + BR3b);
  double d3b = 2.0 * k13 * d3 * (BL3b + BR2b);
  double d4b = 2.0 * k13 * d4 * BR1b;
  double gL1b = 2.0 * gL1 * BL1b, gL2b = 2.0 * gL2 * BL2b, gL3b = 2.0 * gL3 * BL3b;
  double gR1b = 2.0 * gR1 * BR1b, gR2b = 2.0 * gR2 * BR2b, gR3b = 2.0 * gR3 * BR3b;
  wb[0] += d1b + gL1b;
  wb[1] += -2.0 * d1b + d2b - 4.0 * gL1b + gL2b + gR3b;
  wb[2] += d1b - 2.0 * d2b + d3b + 3.0 * gL1b + 3.0 * gL3b - gR2b - 4.0 * gR3b;
  wb[3] += d2b - 2.0 * d3b + d4b - gL2b - 4.0 * gL3b + 3.0 * gR1b + 3.0 * gR3b;
  wb[4] += d3b - 2.0 * d4b + gL3b - 4.0 * gR1b + gR2b;
  wb[5] += d4b + gR1b;
  vb[0] += 2.0 * cL1b;
  vb[1] += -7.0 * cL1b - cAb;
  vb[2] += 11.0 * cL1b + 5.0 * cAb + 2.0 * cBb;
  vb[3] += 11.0 * cR1b + 2.0 * cAb + 5.0 * cBb;
  vb[4] += -7.0 * cR1b - cBb;
  vb[5] += 2.0 * cR1b;
}

__device__ __forceinline__ void weno5_pair_vjp(const double* w, const double* v, double eps4, double gL, double gR,
                                               double* wb, double* vb) {
  weno5_pair_vjp_impl<false>(w, v, eps4, gL, gR, wb, vb, nullptr);
}

// ---------------------------------------------------------------------------
// Reverse of the Euler2D cell flux along D: u_bar += (df/du)^T f_bar.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void flux_vjp(const double* u, const double* fb, double* ub, const PhysParams& pp) {
  double rho = u[0], ri = nr_rcp(rho);
  double v[2] = {u[1] * ri, u[2] * ri};
  double e = u[3];
  double vsq = fma(v[1], v[1], v[0] * v[0]);
  double P = (e - 0.5 * rho * vsq) * pp.gm1;
  double mn = rho * v[D];
  double mnb = fb[0], vb[2] = {0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 2; k++) {
    mnb = fma(fb[1 + k], v[k], mnb);
    vb[k] += fb[1 + k] * mn;
  }
  double Pb = fma(fb[3], v[D], fb[1 + D]);
  double eb = fb[3] * v[D];
  vb[D] = fma(fb[3], e + P, vb[D]);
  double rhob = mnb * v[D];
  vb[D] = fma(mnb, rho, vb[D]);
  eb = fma(pp.gm1, Pb, eb);
  rhob = fma(-0.5 * pp.gm1 * vsq, Pb, rhob);
  double vsqb = -0.5 * pp.gm1 * rho * Pb;
  double rib = 0.0;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    vb[k] = fma(2.0 * v[k], vsqb, vb[k]);
    ub[1 + k] = fma(vb[k], ri, ub[1 + k]);
    rib = fma(vb[k], u[1 + k], rib);
  }
  rhob = fma(-rib, ri * ri, rhob);
  ub[0] += rhob;
  ub[3] += eb;
}

// ---------------------------------------------------------------------------
// Roe flux of Euler2D along D (the forward of upwind_iface for component-wise
// WENO, Euler2DUpwind.c:10-66) and its reverse.
// ---------------------------------------------------------------------------
struct SideRev {
  double r, ri, v[2], E, P, t, H, vsq;
};
__device__ __forceinline__ SideRev side_fwd(const double* u, const PhysParams& pp) {
  SideRev s;
  s.r = u[0];
  s.ri = nr_rcp(s.r);
  s.v[0] = u[1] * s.ri;
  s.v[1] = u[2] * s.ri;
  s.E = u[3];
  s.vsq = fma(s.v[1], s.v[1], s.v[0] * s.v[0]);
  s.P = (s.E - 0.5 * s.r * s.vsq) * pp.gm1;
  s.t = nr_sqrt(s.r);
  s.H = (s.E + s.P) * s.ri;
  return s;
}
__device__ __forceinline__ void side_rev(const SideRev& s, const double* u, double tb, const double* vb_in, double Hb,
                                         double* ub, const PhysParams& pp) {
  double vb[2] = {vb_in[0], vb_in[1]};
  double rb = tb * 0.5 * nr_rcp(s.t);
  double Eb = Hb * s.ri, Pb = Hb * s.ri, rib = Hb * (s.E + s.P);
  Eb = fma(pp.gm1, Pb, Eb);
  rb = fma(-0.5 * pp.gm1 * s.vsq, Pb, rb);
  double vsqb = -0.5 * pp.gm1 * s.r * Pb;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    vb[k] = fma(2.0 * s.v[k], vsqb, vb[k]);
    ub[1 + k] = fma(vb[k], s.ri, ub[1 + k]);
    rib = fma(vb[k], u[1 + k], rib);
  }
  rb = fma(-rib, s.ri * s.ri, rb);
  ub[0] += rb;
  ub[3] += Eb;
}

__device__ __forceinline__ double harten(double lam, double& dlam) {
  const double delta = 0.000001, delta2 = delta * delta;
  double d = fabs(lam);
  if (d < delta) {
    dlam = lam * (1.0 / delta);
    return (lam * lam + delta2) * (0.5 / delta);
  }
  dlam = lam < 0.0 ? -1.0 : 1.0;
  return d;
}

// Forward Roe flux and, given Fb, the adjoints of fL, fR (0.5 Fb each, added
// by the caller) and of uL, uR.
template <int D>
__device__ __forceinline__ void roe_vjp(const double* uL, const double* uR, const double* Fb, double* uLb,
                                        double* uRb, const PhysParams& pp) {
  constexpr int T = 1 - D;
  SideRev L = side_fwd(uL, pp), R = side_fwd(uR, pp);
  double inv = nr_rcp(L.t + R.t);
  double numv[2], vel[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    numv[k] = fma(L.t, L.v[k], R.t * R.v[k]);
    vel[k] = numv[k] * inv;
  }
  double numH = fma(L.t, L.H, R.t * R.H);
  double H = numH * inv;
  double ek = 0.5 * fma(vel[1], vel[1], vel[0] * vel[0]);
  double a2 = pp.gm1 * (H - ek);
  double ia = nr_rsqrt(a2);
  double a = a2 * ia, inv_a2 = ia * ia;
  double hac = 0.5 * inv_a2, gh = pp.gm1 * hac, gi = pp.gm1 * inv_a2, ah = a * hac;
  double un = vel[D], aun = a * un;
  double ud[4];
#pragma unroll
  for (int k = 0; k < 4; k++) ud[k] = 0.5 * (uR[k] - uL[k]);
  double s = fma(-vel[1], ud[2], fma(-vel[0], ud[1], fma(ek, ud[0], ud[3])));
  double m = fma(un, ud[0], -ud[1 + D]);
  double th = ah * m;
  double w[4] = {fma(s, gh, th), fma(s, gh, -th), fma(-s, gi, ud[0]), fma(vel[T], ud[0], -ud[1 + T])};
  double lam[4] = {un - a, un + a, un, un}, Dk[4], dD[4], z[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    Dk[k] = harten(lam[k], dD[k]);
    z[k] = Dk[k] * w[k];
  }
  double sa = z[0] + z[1], da = z[1] - z[0], y0 = sa + z[2];
  // reverse: y = R z, F = (fL + fR)/2 - y
  double yb[4] = {-Fb[0], -Fb[1], -Fb[2], -Fb[3]};
  double unb = 0.0, ab = 0.0, velb[2] = {0.0, 0.0}, Hb = 0.0, ekb = 0.0, aunb = 0.0;
  double zb[4] = {0.0, 0.0, 0.0, 0.0}, sab = 0.0, dab = 0.0;
  double y0b = yb[0];
  // y_{1+D} = un y0 + a da
  unb = fma(yb[1 + D], y0, unb);
  y0b = fma(un, yb[1 + D], y0b);
  ab = fma(yb[1 + D], da, ab);
  dab = fma(a, yb[1 + D], dab);
  // y_{1+T} = v_T y0 - z3
  velb[T] = fma(yb[1 + T], y0, velb[T]);
  y0b = fma(vel[T], yb[1 + T], y0b);
  zb[3] -= yb[1 + T];
  // yE = H sa + aun da + ek z2 - v_T z3
  Hb = fma(yb[3], sa, Hb);
  sab = fma(yb[3], H, sab);
  aunb = fma(yb[3], da, aunb);
  dab = fma(yb[3], aun, dab);
  ekb = fma(yb[3], z[2], ekb);
  zb[2] = fma(yb[3], ek, zb[2]);
  velb[T] = fma(-yb[3], z[3], velb[T]);
  zb[3] = fma(-yb[3], vel[T], zb[3]);
  // y0 = sa + z2; sa = z0 + z1; da = z1 - z0
  sab += y0b;
  zb[2] += y0b;
  zb[0] += sab - dab;
  zb[1] += sab + dab;
  // z = D w
  double wb[4], lamb[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    wb[k] = Dk[k] * zb[k];
    lamb[k] = w[k] * zb[k] * dD[k];
  }
  unb += lamb[0] + lamb[1] + lamb[2] + lamb[3];
  ab += lamb[1] - lamb[0];
  // w3 = v_T ud0 - ud_{1+T}; w2 = ud0 - s gi; w0,1 = s gh +- th
  double udb[4] = {0.0, 0.0, 0.0, 0.0};
  velb[T] = fma(wb[3], ud[0], velb[T]);
  udb[0] = fma(wb[3], vel[T], udb[0]);
  udb[1 + T] -= wb[3];
  udb[0] += wb[2];
  double sb = -wb[2] * gi;
  double gib = -wb[2] * s;
  sb = fma(wb[0] + wb[1], gh, sb);
  double ghb = (wb[0] + wb[1]) * s;
  double thb = wb[0] - wb[1];
  double ahb = thb * m;
  double mb = thb * ah;
  unb = fma(mb, ud[0], unb);
  udb[0] = fma(mb, un, udb[0]);
  udb[1 + D] -= mb;
  // s = ek ud0 + ud3 - vx ud1 - vy ud2
  ekb = fma(sb, ud[0], ekb);
  udb[0] = fma(sb, ek, udb[0]);
  udb[3] += sb;
  velb[0] = fma(-sb, ud[1], velb[0]);
  udb[1] = fma(-sb, vel[0], udb[1]);
  velb[1] = fma(-sb, ud[2], velb[1]);
  udb[2] = fma(-sb, vel[1], udb[2]);
  // aun = a un; ah = a hac; gh = gm1 hac; gi = gm1 inv_a2; hac = inv_a2 / 2
  ab = fma(aunb, un, ab);
  unb = fma(aunb, a, unb);
  ab = fma(ahb, hac, ab);
  double hacb = ahb * a;
  hacb = fma(pp.gm1, ghb, hacb);
  double inv_a2b = pp.gm1 * gib;
  inv_a2b = fma(0.5, hacb, inv_a2b);
  // a = sqrt(a2), inv_a2 = 1/a2
  double a2b = fma(ab, 0.5 * ia, -inv_a2b * inv_a2 * inv_a2);
  Hb = fma(pp.gm1, a2b, Hb);
  ekb = fma(-pp.gm1, a2b, ekb);
  velb[D] += unb;
  velb[0] = fma(ekb, vel[0], velb[0]);
  velb[1] = fma(ekb, vel[1], velb[1]);
  // vel_k = numv_k inv; H = numH inv; inv = 1/(tL + tR)
  double invb = fma(velb[0], numv[0], fma(velb[1], numv[1], Hb * numH));
  double nvb[2] = {velb[0] * inv, velb[1] * inv};
  double nHb = Hb * inv;
  double tsb = -invb * inv * inv;
  double tLb = tsb + fma(nvb[0], L.v[0], fma(nvb[1], L.v[1], nHb * L.H));
  double tRb = tsb + fma(nvb[0], R.v[0], fma(nvb[1], R.v[1], nHb * R.H));
  double vLb[2] = {nvb[0] * L.t, nvb[1] * L.t}, vRb[2] = {nvb[0] * R.t, nvb[1] * R.t};
  side_rev(L, uL, tLb, vLb, nHb * L.t, uLb, pp);
  side_rev(R, uR, tRb, vRb, nHb * R.t, uRb, pp);
  // ud = (uR - uL)/2
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uRb[k] = fma(0.5, udb[k], uRb[k]);
    uLb[k] = fma(-0.5, udb[k], uLb[k]);
  }
}

// ---------------------------------------------------------------------------
// Adjoint right-hand side: k_bar is a linear combination of up to four arrays
// (the Runge-Kutta stage adjoints are formed on the fly).
// ---------------------------------------------------------------------------
struct AdjTerms {
  const double* p[4];
  double c[4];
  int n;
};

__device__ __forceinline__ void terms_at(const AdjTerms& t, long long off, double* out) {
#pragma unroll
  for (int v = 0; v < NV2; v++) out[v] = 0.0;
  for (int j = 0; j < t.n; j++) {
#pragma unroll
    for (int v = 0; v < NV2; v++) out[v] = fma(t.c[j], t.p[j][off + v], out[v]);
  }
}

// One thread's share along direction D: interfaces [sg*seg, min((sg+1)*seg, N)]
// of grid line `tr`, owning the adjoints of cells [sg*seg, min((sg+1)*seg, N)).
// The six-cell window of the forward kernel is kept with, per cell, the
// adjoint of its state (ab) and of its flux (fbb); a cell leaving the window
// is finished: u_bar += ab + (df/du)^T fbb, added atomically at the folded
// index (neighbouring segments and the other direction add to the same cells).
// tape: the forward kernel's reconstructed states uL, uR of this direction
// (StageEpi::tape layout), read instead of recomputed when present.
// WT: the tape is the wide one (TAPE_WIDE doubles per interface), whose smoothness
// terms and normalisation reciprocals spare the pairs' forward recomputation.
template <int D, bool WT>
__device__ __forceinline__ void vjp_segment(const double* __restrict__ U, const AdjTerms& kt, double* Ub,
                                            const double* __restrict__ dxinv, const DevGeom& G,
                                            const PhysParams& pp, int seg, long long tr, int sg,
                                            const double* __restrict__ tape) {
  constexpr int T = 1 - D;
  const long long pbase = (long long)(tr + G.g) * G.stride[T] + (long long)G.g * G.stride[D];
  const int N = G.dim[D];
  const long long sd = G.stride[D];
  const int lo = G.bclo[D], hi = G.bchi[D];
  const int I0 = sg * seg, I1 = min(I0 + seg, N);
  const double eps4 = 4.0 * pp.eps;
  double wu[6][NV2], wf[6][NV2], ab[6][NV2], fbb[6][NV2];
  int widx[6];
  auto load = [&](int i) {
    const int fi = fold2(i, N, lo, hi);
    widx[5] = fi;
    const double* src = U + (pbase + (long long)fi * sd) * NV2;
#pragma unroll
    for (int v = 0; v < NV2; v++) {
      wu[5][v] = src[v];
      ab[5][v] = 0.0;
      fbb[5][v] = 0.0;
    }
    Prim<MODEL_EULER2D> q = to_prim<MODEL_EULER2D>(wu[5], pp);
    cell_flux<MODEL_EULER2D, D>(q, wf[5]);
  };
  auto flush = [&](int p) {
    flux_vjp<D>(wu[p], fbb[p], ab[p], pp);
    double* dst = Ub + (pbase + (long long)widx[p] * sd) * NV2;
#pragma unroll
    for (int v = 0; v < NV2; v++) atomicAdd(dst + v, ab[p][v]);
  };
  auto shift = [&]() {
#pragma unroll
    for (int p = 0; p < 5; p++) {
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        wu[p][v] = wu[p + 1][v];
        wf[p][v] = wf[p + 1][v];
        ab[p][v] = ab[p + 1][v];
        fbb[p][v] = fbb[p + 1][v];
      }
      widx[p] = widx[p + 1];
    }
  };
  for (int k = 0; k < 5; k++) {
    load(I0 - 3 + k);
    shift();
  }
  // rhs_c = -dxinv_c (F_{c+1/2} - F_{c-1/2}): interface I feeds cells I-1 (-) and I (+)
  double kprev[NV2] = {0.0, 0.0, 0.0, 0.0};
  for (int I = I0; I <= I1; I++) {
    load(I + 2);
    double Fb[NV2];
#pragma unroll
    for (int v = 0; v < NV2; v++) Fb[v] = -kprev[v];
    if (I < I1) {
      double kb[NV2];
      terms_at(kt, (pbase + (long long)I * sd) * NV2, kb);
      const double dx = dxinv[G.g + I];
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        kprev[v] = dx * kb[v];
        Fb[v] += kprev[v];
      }
    }
    double uL[NV2], uR[NV2];
    const double* t = tape ? tape + (tr * (N + 1) + I) * (WT ? TAPE_WIDE : 8) : nullptr;
    if (tape) {
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        uL[v] = t[v];
        uR[v] = t[4 + v];
      }
    } else {
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        double su[6];
#pragma unroll
        for (int p = 0; p < 6; p++) su[p] = wu[p][v];
        weno5_pair(su, su, eps4, uL[v], uR[v]);
      }
    }
    double uLb[NV2] = {0.0, 0.0, 0.0, 0.0}, uRb[NV2] = {0.0, 0.0, 0.0, 0.0};
    roe_vjp<D>(uL, uR, Fb, uLb, uRb, pp);
#pragma unroll
    for (int v = 0; v < NV2; v++) {
      double sf[6], su[6], gf[6] = {0, 0, 0, 0, 0, 0}, gu[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int p = 0; p < 6; p++) {
        sf[p] = wf[p][v];
        su[p] = wu[p][v];
      }
      if (WT) {
        weno5_pair_vjp_impl<true>(sf, sf, eps4, 0.5 * Fb[v], 0.5 * Fb[v], gf, gf, t + 8 + v * 16);
        weno5_pair_vjp_impl<true>(su, su, eps4, uLb[v], uRb[v], gu, gu, t + 16 + v * 16);
      } else {
        weno5_pair_vjp(sf, sf, eps4, 0.5 * Fb[v], 0.5 * Fb[v], gf, gf);
        weno5_pair_vjp(su, su, eps4, uLb[v], uRb[v], gu, gu);
      }
#pragma unroll
      for (int p = 0; p < 6; p++) {
        fbb[p][v] += gf[p];
        ab[p][v] += gu[p];
      }
    }
    flush(0);  // cell I-3: no later interface of this segment reads it
    shift();
  }
#pragma unroll
  for (int p = 0; p < 5; p++) flush(p);  // cells I1-2 .. I1+2
}

// The tile form of the reverse kernel (small grids): a block takes TI interfaces of
// one grid line and the TI + 5 cells their windows touch.  The cells' states and
// fluxes go to shared memory once; each thread reverses one interface (its flux
// adjoint from both neighbouring cells' k_bar, so no interface is reversed twice as
// at the walker's segment boundaries) and stores its six cells' stencil adjoints in
// shared memory; after a barrier each cell sums the contributions of the interfaces
// that touch it, in a fixed order (no shared-memory atomics, and the same sum on
// every run), is finished (u_bar += a + (df/du)^T f_bar) and stored as this tile's
// share of the cell; vjp_slot_gather_kernel then adds the shares of all tiles and both
// directions into u_bar in a fixed order, so the result does not depend on the order
// in which blocks run.
// Shared memory of the tile reverse (both directions use the same block of it): the
// tile's cell states and fluxes, and per interface t the adjoints of its window cells
// t .. t+5, of the flux (gf) and of the state (gu).
template <int TI>
struct VjpTileSmem {
  double su[TI + 5][NV2], sf[TI + 5][NV2];
  double sgf[TI][6][NV2], sgu[TI][6][NV2];
};

template <int D, bool WT, int TI>
__device__ __forceinline__ void vjp_tile(const double* __restrict__ U, const AdjTerms& kt, double* __restrict__ slot,
                                         int ntile, const double* __restrict__ dxinv, const DevGeom& G,
                                         const PhysParams& pp, long long tr, int tile,
                                         const double* __restrict__ tape, VjpTileSmem<TI>& sm) {
  constexpr int T = 1 - D, NCELL = TI + 5;
  auto& su = sm.su;
  auto& sf = sm.sf;
  auto& sgf = sm.sgf;
  auto& sgu = sm.sgu;
  const long long pbase = (long long)(tr + G.g) * G.stride[T] + (long long)G.g * G.stride[D];
  const int N = G.dim[D];
  const long long sd = G.stride[D];
  const int lo = G.bclo[D], hi = G.bchi[D];
  const int I0 = tile * TI;
  const double eps4 = 4.0 * pp.eps;
  for (int c = threadIdx.x; c < NCELL; c += TI) {
    const int i = I0 - 3 + c;
    const double* src = U + (pbase + (long long)fold2(i, N, lo, hi) * sd) * NV2;
    double uu[NV2], ff[NV2];
#pragma unroll
    for (int v = 0; v < NV2; v++) uu[v] = src[v];
    Prim<MODEL_EULER2D> q = to_prim<MODEL_EULER2D>(uu, pp);
    cell_flux<MODEL_EULER2D, D>(q, ff);
#pragma unroll
    for (int v = 0; v < NV2; v++) {
      su[c][v] = uu[v];
      sf[c][v] = ff[v];
    }
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int I = I0 + t;
  if (I <= N) {
    // rhs_c = -dxinv_c (F_{c+1/2} - F_{c-1/2}): interface I feeds cells I-1 (-) and I (+)
    double Fb[NV2] = {0.0, 0.0, 0.0, 0.0};
    double kb[NV2];
    if (I > 0) {
      terms_at(kt, (pbase + (long long)(I - 1) * sd) * NV2, kb);
      const double dx = dxinv[G.g + I - 1];
#pragma unroll
      for (int v = 0; v < NV2; v++) Fb[v] = -dx * kb[v];
    }
    if (I < N) {
      terms_at(kt, (pbase + (long long)I * sd) * NV2, kb);
      const double dx = dxinv[G.g + I];
#pragma unroll
      for (int v = 0; v < NV2; v++) Fb[v] = fma(dx, kb[v], Fb[v]);
    }
    const double* tp = tape ? tape + (tr * (N + 1) + I) * (WT ? TAPE_WIDE : 8) : nullptr;
    double uL[NV2], uR[NV2];
    if (tp) {
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        uL[v] = tp[v];
        uR[v] = tp[4 + v];
      }
    } else {
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        double w6[6];
#pragma unroll
        for (int p = 0; p < 6; p++) w6[p] = su[t + p][v];
        weno5_pair(w6, w6, eps4, uL[v], uR[v]);
      }
    }
    double uLb[NV2] = {0.0, 0.0, 0.0, 0.0}, uRb[NV2] = {0.0, 0.0, 0.0, 0.0};
    roe_vjp<D>(uL, uR, Fb, uLb, uRb, pp);
#pragma unroll
    for (int v = 0; v < NV2; v++) {
      double wf6[6], wu6[6], gf[6] = {0, 0, 0, 0, 0, 0}, gu[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int p = 0; p < 6; p++) {
        wf6[p] = sf[t + p][v];
        wu6[p] = su[t + p][v];
      }
      if (WT) {
        weno5_pair_vjp_impl<true>(wf6, wf6, eps4, 0.5 * Fb[v], 0.5 * Fb[v], gf, gf, tp + 8 + v * 16);
        weno5_pair_vjp_impl<true>(wu6, wu6, eps4, uLb[v], uRb[v], gu, gu, tp + 16 + v * 16);
      } else {
        weno5_pair_vjp(wf6, wf6, eps4, 0.5 * Fb[v], 0.5 * Fb[v], gf, gf);
        weno5_pair_vjp(wu6, wu6, eps4, uLb[v], uRb[v], gu, gu);
      }
#pragma unroll
      for (int p = 0; p < 6; p++) {
        sgf[t][p][v] = gf[p];
        sgu[t][p][v] = gu[p];
      }
    }
  }
  __syncthreads();
  // interfaces of this tile that exist (I <= N); cell c is window cell c - t of interface t
  const int nI = min(TI, N + 1 - I0);
  for (int c = threadIdx.x; c < NCELL; c += TI) {
    const int i = I0 - 3 + c;
    if (i > N + 2) continue;
    double ab[NV2] = {0.0, 0.0, 0.0, 0.0}, fb[NV2] = {0.0, 0.0, 0.0, 0.0}, uu[NV2];
    const int t0 = max(0, c - 5), t1 = min(c, nI - 1);
    for (int tt = t0; tt <= t1; tt++) {
#pragma unroll
      for (int v = 0; v < NV2; v++) {
        fb[v] += sgf[tt][c - tt][v];
        ab[v] += sgu[tt][c - tt][v];
      }
    }
#pragma unroll
    for (int v = 0; v < NV2; v++) uu[v] = su[c][v];
    flux_vjp<D>(uu, fb, ab, pp);
    // this tile's share of the cell, summed with the other tiles' by vjp_slot_gather_kernel
    double* dst = slot + (((long long)tr * ntile + tile) * NCELL + c) * NV2;
#pragma unroll
    for (int v = 0; v < NV2; v++) dst[v] = ab[v];
  }
}

template <bool WT, int TI>
__global__ void __launch_bounds__(TI)
rhs_vjp_tile_kernel(const double* __restrict__ U, AdjTerms kt, double* __restrict__ slot0,
                    double* __restrict__ slot1, const double* __restrict__ dx0, const double* __restrict__ dx1,
                    DevGeom G, PhysParams pp, int nt0, int nt1, const double* __restrict__ tape0,
                    const double* __restrict__ tape1) {
  __shared__ VjpTileSmem<TI> sm;
  const long long b = blockIdx.x;
  const long long n0 = (long long)G.dim[1] * nt0;
  if (b < n0) {
    vjp_tile<0, WT, TI>(U, kt, slot0, nt0, dx0, G, pp, b % G.dim[1], (int)(b / G.dim[1]), tape0, sm);
  } else {
    const long long t = b - n0;
    vjp_tile<1, WT, TI>(U, kt, slot1, nt1, dx1, G, pp, t % G.dim[0], (int)(t / G.dim[0]), tape1, sm);
  }
}

// The tile reverse's cells summed in a fixed order, so that repeated gradients are
// bit-identical.  Along direction D, interior cell i of a line receives the shares of
// every tile whose window holds one of its images: i itself and, through the folded
// boundaries, the ghost cell that copies it (periodic: i - N, i + N; mirror: -1 - i,
// 2N - 1 - i).  Tile T's window is cells T TI - 3 .. T TI + TI + 1 (at most N + 2).
template <int TI>
__device__ __forceinline__ void slot_sum(const double* __restrict__ slot, long long line, int ntile, int i, int N,
                                         int lo, int hi, double* acc) {
  constexpr int NCELL = TI + 5;
  int img[3] = {i, INT_MIN, INT_MIN};
  if (lo == FOLD_PERIODIC && i >= N - 3) img[1] = i - N;
  if (lo == FOLD_MIRROR && i <= 2) img[1] = -1 - i;
  if (hi == FOLD_PERIODIC && i <= 2) img[2] = i + N;
  if (hi == FOLD_MIRROR && i >= N - 3) img[2] = 2 * N - 1 - i;
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const int ip = img[m];
    if (ip == INT_MIN || ip < -3 || ip > N + 2) continue;
    // tiles T with T TI - 3 <= ip <= T TI + TI + 1
    const int tmax = min(ntile - 1, (ip + 3) / TI);
    for (int T = max(0, (ip - TI - 1 + TI - 1) / TI); T <= tmax; T++) {
      const int c = ip - T * TI + 3;
      if (c < 0 || c >= NCELL) continue;
      const double* src = slot + ((line * ntile + T) * NCELL + c) * NV2;
#pragma unroll
      for (int v = 0; v < NV2; v++) acc[v] += src[v];
    }
  }
}


// Both directions in one launch (they only add into Ub): threads
// [0, n0) walk x-lines, [n0, n0 + n1) y-lines.
template <bool WT>
__global__ void __launch_bounds__(128)
rhs_vjp_kernel(const double* __restrict__ U, AdjTerms kt, double* Ub, const double* __restrict__ dx0,
               const double* __restrict__ dx1, DevGeom G, PhysParams pp, int seg0, int nseg0, int seg1, int nseg1,
               const double* __restrict__ tape0, const double* __restrict__ tape1) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n0 = (long long)G.dim[1] * nseg0, n1 = (long long)G.dim[0] * nseg1;
  if (tid < n0) {
    vjp_segment<0, WT>(U, kt, Ub, dx0, G, pp, seg0, tid % G.dim[1], (int)(tid / G.dim[1]), tape0);
  } else if (tid < n0 + n1) {
    const long long t = tid - n0;
    vjp_segment<1, WT>(U, kt, Ub, dx1, G, pp, seg1, t % G.dim[0], (int)(t / G.dim[0]), tape1);
  }
}

// ---------------------------------------------------------------------------
// JVP kernel in dual numbers, one thread per interior cell and direction,
// reference formulation.
// ---------------------------------------------------------------------------
struct Dual {
  double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator*(double c, Dual a) { return {c * a.v, c * a.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual dsqrt(Dual a) {
  double s = sqrt(a.v);
  return {s, a.d / (2.0 * s)};
}
__device__ __forceinline__ Dual dabs(Dual a) { return a.v < 0 ? -a : a; }
__device__ __forceinline__ Dual C(double c) { return {c, 0.0}; }

// _WENOWeights_v_JS_ + Interp1PrimFifthOrderWENO for one biased stencil.
__device__ Dual weno_js_dual(Dual m3, Dual m2, Dual m1, Dual p1, Dual p2, double eps) {
  const double k13 = 13.0 / 12.0, k14 = 0.25, s6 = 1.0 / 6.0;
  Dual t1 = m3 - 2.0 * m2 + m1, t2 = m3 - 4.0 * m2 + 3.0 * m1;
  Dual b1 = k13 * (t1 * t1) + k14 * (t2 * t2);
  Dual t3 = m2 - 2.0 * m1 + p1, t4 = m2 - p1;
  Dual b2 = k13 * (t3 * t3) + k14 * (t4 * t4);
  Dual t5 = m1 - 2.0 * p1 + p2, t6 = 3.0 * m1 - 4.0 * p1 + p2;
  Dual b3 = k13 * (t5 * t5) + k14 * (t6 * t6);
  Dual e1 = b1 + C(eps), e2 = b2 + C(eps), e3 = b3 + C(eps);
  Dual a1 = C(0.1) / (e1 * e1), a2 = C(0.6) / (e2 * e2), a3 = C(0.3) / (e3 * e3);
  Dual sum = a1 + a2 + a3;
  Dual f1 = (2.0 * s6) * m3 + (-7.0 * s6) * m2 + (11.0 * s6) * m1;
  Dual f2 = (-s6) * m2 + (5.0 * s6) * m1 + (2.0 * s6) * p1;
  Dual f3 = (2.0 * s6) * m1 + (5.0 * s6) * p1 + (-s6) * p2;
  return (a1 * f1 + a2 * f2 + a3 * f3) / sum;
}

template <int D>
__device__ void flux_dual(const Dual* u, Dual* f, double gamma) {
  Dual rho = u[0], vx = u[1] / rho, vy = u[2] / rho, e = u[3];
  Dual P = (e - 0.5 * (rho * (vx * vx + vy * vy))) * C(gamma - 1.0);
  Dual vn = D == 0 ? vx : vy;
  f[0] = rho * vn;
  f[1] = rho * vn * vx + (D == 0 ? P : C(0.0));
  f[2] = rho * vn * vy + (D == 1 ? P : C(0.0));
  f[3] = (e + P) * vn;
}

// Euler2DUpwindRoe in the reference's dense form: the Roe-averaged conserved
// state (_Euler2DRoeAverage_), eigenvalues, L and R from that state
// (euler2d.h:108-230), Harten's fix, then R (D (L udiff)).
template <int D>
__device__ void roe_dual(const Dual* fL, const Dual* fR, const Dual* uL, const Dual* uR, Dual* fI, double gamma) {
  Dual g = C(gamma), gm1 = C(gamma - 1.0);
  Dual rL = uL[0], vxL = uL[1] / rL, vyL = uL[2] / rL, EL = uL[3];
  Dual PL = (EL - 0.5 * (rL * (vxL * vxL + vyL * vyL))) * gm1;
  Dual HL = 0.5 * (vxL * vxL + vyL * vyL) + (g * PL / rL) / gm1;
  Dual rR = uR[0], vxR = uR[1] / rR, vyR = uR[2] / rR, ER = uR[3];
  Dual PR = (ER - 0.5 * (rR * (vxR * vxR + vyR * vyR))) * gm1;
  Dual HR = 0.5 * (vxR * vxR + vyR * vyR) + (g * PR / rR) / gm1;
  Dual tL = dsqrt(rL), tR = dsqrt(rR);
  Dual ra = tL * tR;
  Dual vxa = (tL * vxL + tR * vxR) / (tL + tR), vya = (tL * vyL + tR * vyR) / (tL + tR);
  Dual Ha = (tL * HL + tR * HR) / (tL + tR);
  Dual vsqa = vxa * vxa + vya * vya;
  Dual csq = gm1 * (Ha - 0.5 * vsqa);
  Dual Pa = csq * ra / g;
  Dual ea = Pa / gm1 + 0.5 * (ra * vsqa);
  Dual uavg[4] = {ra, ra * vxa, ra * vya, ea};
  // eigen-structure of uavg
  Dual rho = uavg[0], vx = uavg[1] / rho, vy = uavg[2] / rho, e = uavg[3];
  Dual vsq = vx * vx + vy * vy;
  Dual P = (e - 0.5 * (rho * vsq)) * gm1;
  Dual ek = 0.5 * vsq;
  Dual a = dsqrt(g * P / rho);
  Dual un = D == 0 ? vx : vy;
  double nx = D == 0 ? 1.0 : 0.0, ny = D == 0 ? 0.0 : 1.0;
  Dual a2x2 = 2.0 * (a * a), a2 = a * a;
  Dual Lm[4][4], Rm[4][4], Dg[4];
  // rows: acoustic -, acoustic +, shear, entropy (euler2d.h:128-230)
  Lm[0][0] = (gm1 * ek + a * un) / a2x2;
  Lm[0][1] = (-(gm1 * vx) - a * C(nx)) / a2x2;
  Lm[0][2] = (-(gm1 * vy) - a * C(ny)) / a2x2;
  Lm[0][3] = gm1 / a2x2;
  Lm[1][0] = (gm1 * ek - a * un) / a2x2;
  Lm[1][1] = (-(gm1 * vx) + a * C(nx)) / a2x2;
  Lm[1][2] = (-(gm1 * vy) + a * C(ny)) / a2x2;
  Lm[1][3] = gm1 / a2x2;
  if (D == 0) {
    Lm[2][0] = vy; Lm[2][1] = C(0.0); Lm[2][2] = C(-1.0); Lm[2][3] = C(0.0);
  } else {
    Lm[2][0] = -vx; Lm[2][1] = C(1.0); Lm[2][2] = C(0.0); Lm[2][3] = C(0.0);
  }
  Lm[3][0] = (a2 - gm1 * ek) / a2;
  Lm[3][1] = gm1 * vx / a2;
  Lm[3][2] = gm1 * vy / a2;
  Lm[3][3] = -gm1 / a2;
  Dual h0 = a2 / gm1 + ek;
  Rm[0][0] = C(1.0); Rm[1][0] = vx - a * C(nx); Rm[2][0] = vy - a * C(ny); Rm[3][0] = h0 - a * un;
  Rm[0][1] = C(1.0); Rm[1][1] = vx + a * C(nx); Rm[2][1] = vy + a * C(ny); Rm[3][1] = h0 + a * un;
  if (D == 0) {
    Rm[0][2] = C(0.0); Rm[1][2] = C(0.0); Rm[2][2] = C(-1.0); Rm[3][2] = -vy;
  } else {
    Rm[0][2] = C(0.0); Rm[1][2] = C(1.0); Rm[2][2] = C(0.0); Rm[3][2] = vx;
  }
  Rm[0][3] = C(1.0); Rm[1][3] = vx; Rm[2][3] = vy; Rm[3][3] = ek;
  Dual lam[4] = {un - a, un + a, un, un};
  const double delta = 0.000001, delta2 = delta * delta;
  for (int k = 0; k < 4; k++) {
    Dual l = lam[k];
    Dg[k] = (fabs(l.v) < delta) ? (l * l + C(delta2)) / C(2.0 * delta) : dabs(l);
  }
  Dual ud[4], w[4];
  for (int k = 0; k < 4; k++) ud[k] = 0.5 * (uR[k] - uL[k]);
  for (int i = 0; i < 4; i++) {
    Dual s = C(0.0);
    for (int j = 0; j < 4; j++) s = s + Lm[i][j] * ud[j];
    w[i] = Dg[i] * s;
  }
  for (int i = 0; i < 4; i++) {
    Dual s = C(0.0);
    for (int j = 0; j < 4; j++) s = s + Rm[i][j] * w[j];
    fI[i] = 0.5 * (fL[i] + fR[i]) - s;
  }
}

template <int D>
__device__ void iface_dual(const double* U, const double* dU, long long pbase, long long sd, int I, int N, int lo,
                           int hi, double eps, double gamma, Dual* F) {
  Dual su[6][NV2], sf[6][NV2];
  for (int p = 0; p < 6; p++) {
    int fi = fold2(I - 3 + p, N, lo, hi);
    long long q = (pbase + (long long)fi * sd) * NV2;
    for (int v = 0; v < NV2; v++) su[p][v] = {U[q + v], dU[q + v]};
    flux_dual<D>(su[p], sf[p], gamma);
  }
  Dual fL[4], fR[4], uL[4], uR[4];
  for (int v = 0; v < NV2; v++) {
    fL[v] = weno_js_dual(sf[0][v], sf[1][v], sf[2][v], sf[3][v], sf[4][v], eps);
    fR[v] = weno_js_dual(sf[5][v], sf[4][v], sf[3][v], sf[2][v], sf[1][v], eps);
    uL[v] = weno_js_dual(su[0][v], su[1][v], su[2][v], su[3][v], su[4][v], eps);
    uR[v] = weno_js_dual(su[5][v], su[4][v], su[3][v], su[2][v], su[1][v], eps);
  }
  roe_dual<D>(fL, fR, uL, uR, F, gamma);
}

// k = F(U) and dk = dF/dU dU; the first direction writes, later ones add.
template <int D>
__global__ void rhs_jvp_kernel(const double* __restrict__ U, const double* __restrict__ dU, double* K, double* dK,
                               const double* __restrict__ dxinv, DevGeom G, PhysParams pp, int first) {
  long long n = (long long)G.dim[0] * G.dim[1];
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int idx[2] = {(int)(t % G.dim[0]), (int)(t / G.dim[0])};
  constexpr int T = 1 - D;
  long long pbase = (long long)(idx[T] + G.g) * G.stride[T] + (long long)G.g * G.stride[D];
  const long long sd = G.stride[D];
  int c = idx[D];
  Dual Fp[4], Fm[4];
  iface_dual<D>(U, dU, pbase, sd, c + 1, G.dim[D], G.bclo[D], G.bchi[D], pp.eps, pp.gamma, Fp);
  iface_dual<D>(U, dU, pbase, sd, c, G.dim[D], G.bclo[D], G.bchi[D], pp.eps, pp.gamma, Fm);
  double dx = dxinv[G.g + c];
  long long q = (pbase + (long long)c * sd) * NV2;
  for (int v = 0; v < NV2; v++) {
    double kv = -dx * (Fp[v].v - Fm[v].v), dkv = -dx * (Fp[v].d - Fm[v].d);
    if (first) {
      K[q + v] = kv;
      dK[q + v] = dkv;
    } else {
      K[q + v] += kv;
      dK[q + v] += dkv;
    }
  }
}

// ---------------------------------------------------------------------------
// Interior-point kernels of the Runge-Kutta tangent and adjoint.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool interior_offset(const DevGeom& G, long long p, long long& q) {
  const long long n = (long long)G.dim[0] * G.dim[1];
  if (p >= n) return false;
  const int i = (int)(p % G.dim[0]), j = (int)(p / G.dim[0]);
  q = ((long long)(i + G.g) * G.stride[0] + (long long)(j + G.g) * G.stride[1]) * NV2;
  return true;
}

template <int TI>
__global__ void vjp_slot_gather_kernel(double* Ub, const double* __restrict__ slot0, const double* __restrict__ slot1,
                                       DevGeom G, int nt0, int nt1) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long q;
  if (!interior_offset(G, p, q)) return;
  const int i = (int)(p % G.dim[0]), j = (int)(p / G.dim[0]);
  double ax[NV2] = {0.0, 0.0, 0.0, 0.0}, ay[NV2] = {0.0, 0.0, 0.0, 0.0};
  slot_sum<TI>(slot0, j, nt0, i, G.dim[0], G.bclo[0], G.bchi[0], ax);  // x-line j
  slot_sum<TI>(slot1, i, nt1, j, G.dim[1], G.bclo[1], G.bchi[1], ay);  // y-line i
#pragma unroll
  for (int v = 0; v < NV2; v++) Ub[q + v] += ax[v] + ay[v];
}

// out = base + sum_j c_j X_j at interior points (out may be base).
__global__ void lincomb_kernel(double* out, const double* base, AdjTerms t, DevGeom G) {
  long long q;
  if (!interior_offset(G, (long long)blockIdx.x * blockDim.x + threadIdx.x, q)) return;
  double acc[NV2];
#pragma unroll
  for (int v = 0; v < NV2; v++) acc[v] = base[q + v];
  for (int j = 0; j < t.n; j++) {
#pragma unroll
    for (int v = 0; v < NV2; v++) acc[v] = fma(t.c[j], t.p[j][q + v], acc[v]);
  }
#pragma unroll
  for (int v = 0; v < NV2; v++) out[q + v] = acc[v];
}

// End of an adjoint step: ubar += sum_s Ub[s], and Ub[s] cleared for the next step.
__global__ void adj_gather_kernel(double* ubar, double* Ub0, double* Ub1, double* Ub2, double* Ub3, int ns,
                                  DevGeom G) {
  long long q;
  if (!interior_offset(G, (long long)blockIdx.x * blockDim.x + threadIdx.x, q)) return;
  double* Ub[4] = {Ub0, Ub1, Ub2, Ub3};
#pragma unroll
  for (int v = 0; v < NV2; v++) {
    double a = ubar[q + v];
    for (int s = 0; s < ns; s++) {
      a += Ub[s][q + v];
      Ub[s][q + v] = 0.0;
    }
    ubar[q + v] = a;
  }
}

}  // namespace gbh

using namespace gbh;

// ---------------------------------------------------------------------------
// gb_adjoint: the discrete adjoint of n Runge-Kutta steps with two-level
// checkpointing, and the tangent-linear model.
// ---------------------------------------------------------------------------
struct gb_adjoint {
  gb_config cfg;
  DevGeom G;
  PhysParams pp;
  HypLaunch hl[2];
  int vjp_seg[2] = {8, 8};
  int vjp_block = 128;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t nvals = 0;
  long long dx_off[2] = {0, 0};
  double* d_dxinv = nullptr;
  int nsteps = 0, seglen = 0, nseg = 0, lastlen = 0;
  int touched[4] = {0, 0, 0, 0};  // stage t reads its own stage array (else u_n)
  double* block = nullptr;        // one allocation carved into the arrays below
  std::vector<double*> ck;        // checkpoint of u at the start of every segment
  // Two segment buffers: u at steps 1..seglen of a segment (su) and the stage
  // states of each of its steps (sP, [i*4 + t]).  The backward sweep reverses
  // one segment from one buffer while the next earlier segment is recomputed
  // into the other on a second stream.
  std::vector<double*> su[2];
  std::vector<double*> sP[2];
  std::vector<double*> sT[2];     // interface tapes of every stage of every step, [(i*4 + s)*2 + d]
  int tape_w = 8;                 // doubles per interface in the tapes (8 or TAPE_WIDE)
  double* tblock2 = nullptr;      // their allocation
  int nbuf = 1;
  cudaStream_t aux = nullptr;     // recomputation stream
  cudaEvent_t ev_start = nullptr;
  std::vector<cudaEvent_t> ev_rec, ev_back;
  double* acc = nullptr;          // Runge-Kutta accumulator of the fused step
  double* H = nullptr;            // x-direction hyperbolic term of the fused step
  double* Ub[4] = {nullptr, nullptr, nullptr, nullptr};
  double* ubar = nullptr;
  // the tile reverse's per-tile cell shares, x and y (sized for tiles of 32 or 64)
  double* slot[2] = {nullptr, nullptr};
  // tangent-linear model arrays (allocated on first use)
  double* tblock = nullptr;
  double *tu = nullptr, *tdu = nullptr, *tU = nullptr, *tdU = nullptr, *tK[4] = {}, *tdK[4] = {};
  bool forward_done = false;
  long long recomputed = 0;
  size_t bytes = 0;
};

#define AK(x)                                                                         \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess) {                                                          \
      gbh_set_error("%s:%d: %s", __FILE__, __LINE__, cudaGetErrorString(e_));         \
      return e_ == cudaErrorMemoryAllocation ? GB_ERR_NOMEM : GB_ERR_CUDA;            \
    }                                                                                 \
  } while (0)

static unsigned interior_grid(const gb_adjoint* a) {
  long long n = (long long)a->G.dim[0] * a->G.dim[1];
  return (unsigned)((n + 255) / 256);
}

static AdjTerms terms0() {
  AdjTerms t;
  memset(&t, 0, sizeof(t));
  return t;
}

// y = y_base + sum c_j X_j (interior).
static int adj_lincomb(gb_adjoint* a, double* out, const double* base, const AdjTerms& t) {
  lincomb_kernel<<<interior_grid(a), 256, 0, a->stream>>>(out, base, t, a->G);
  AK(cudaGetLastError());
  return GB_OK;
}

static int adj_vjp(gb_adjoint* a, const double* U, const AdjTerms& kt, double* Ub, double* const* tape = nullptr) {
  const DevGeom& G = a->G;
  int s0 = a->vjp_seg[0], s1 = a->vjp_seg[1];
  int n0s = (G.dim[0] + s0 - 1) / s0, n1s = (G.dim[1] + s1 - 1) / s1;
  long long nthr = (long long)G.dim[1] * n0s + (long long)G.dim[0] * n1s;
  const int blk = a->vjp_block;
  if (s0 < 0) {
    // tiles of -s0 interfaces (32 or 64) in both directions
    const int ti = -s0;
    const int nt0 = (G.dim[0] + 1 + ti - 1) / ti, nt1 = (G.dim[1] + 1 + ti - 1) / ti;
    const unsigned nblk = (unsigned)((long long)G.dim[1] * nt0 + (long long)G.dim[0] * nt1);
    const bool wide = tape && a->tape_w == TAPE_WIDE;
    const double* t0 = tape ? tape[0] : nullptr;
    const double* t1 = tape ? tape[1] : nullptr;
    const double* dx0 = a->d_dxinv + a->dx_off[0];
    const double* dx1 = a->d_dxinv + a->dx_off[1];
    double *s0 = a->slot[0], *s1 = a->slot[1];
    if (ti == 32) {
      if (wide) rhs_vjp_tile_kernel<true, 32><<<nblk, 32, 0, a->stream>>>(U, kt, s0, s1, dx0, dx1, G, a->pp, nt0, nt1, t0, t1);
      else rhs_vjp_tile_kernel<false, 32><<<nblk, 32, 0, a->stream>>>(U, kt, s0, s1, dx0, dx1, G, a->pp, nt0, nt1, t0, t1);
      AK(cudaGetLastError());
      vjp_slot_gather_kernel<32><<<interior_grid(a), 256, 0, a->stream>>>(Ub, s0, s1, G, nt0, nt1);
    } else {
      if (wide) rhs_vjp_tile_kernel<true, 64><<<nblk, 64, 0, a->stream>>>(U, kt, s0, s1, dx0, dx1, G, a->pp, nt0, nt1, t0, t1);
      else rhs_vjp_tile_kernel<false, 64><<<nblk, 64, 0, a->stream>>>(U, kt, s0, s1, dx0, dx1, G, a->pp, nt0, nt1, t0, t1);
      AK(cudaGetLastError());
      vjp_slot_gather_kernel<64><<<interior_grid(a), 256, 0, a->stream>>>(Ub, s0, s1, G, nt0, nt1);
    }
    AK(cudaGetLastError());
    return GB_OK;
  }
  if (tape && a->tape_w == TAPE_WIDE)
    rhs_vjp_kernel<true><<<(unsigned)((nthr + blk - 1) / blk), blk, 0, a->stream>>>(
        U, kt, Ub, a->d_dxinv + a->dx_off[0], a->d_dxinv + a->dx_off[1], G, a->pp, s0, n0s, s1, n1s, tape[0],
        tape[1]);
  else
    rhs_vjp_kernel<false><<<(unsigned)((nthr + blk - 1) / blk), blk, 0, a->stream>>>(
        U, kt, Ub, a->d_dxinv + a->dx_off[0], a->d_dxinv + a->dx_off[1], G, a->pp, s0, n0s, s1, n1s,
        tape ? tape[0] : nullptr, tape ? tape[1] : nullptr);
  AK(cudaGetLastError());
  return GB_OK;
}

static int adj_jvp(gb_adjoint* a, const double* U, const double* dU, double* K, double* dK) {
  const DevGeom& G = a->G;
  unsigned grid = interior_grid(a) * 2;  // 128-thread blocks
  rhs_jvp_kernel<0><<<grid, 128, 0, a->stream>>>(U, dU, K, dK, a->d_dxinv + a->dx_off[0], G, a->pp, 1);
  rhs_jvp_kernel<1><<<grid, 128, 0, a->stream>>>(U, dU, K, dK, a->d_dxinv + a->dx_off[1], G, a->pp, 0);
  AK(cudaGetLastError());
  return GB_OK;
}

// One fused Runge-Kutta step uin -> uout (distinct arrays) keeping the stage
// states in P[1..ns-1] (the same launches as the solver's step).
// tapes (optional): per stage s and direction d, tapes[2 s + d] receives the
// reconstructed interface states for the adjoint kernel.
static int adj_step(gb_adjoint* a, cudaStream_t strm, const double* uin, double* uout, double* const* P,
                    double* const* tapes = nullptr) {
  const gb_config& c = a->cfg;
  const int ns = c.rk_nstages;
  const double dt = c.dt;
  int touched[4] = {0, 0, 0, 0};
  for (int st = 0; st < ns; st++) {
    const double* U = (st == 0 || !touched[st]) ? uin : P[st];
    StageEpi ep;
    memset(&ep, 0, sizeof(ep));
    ep.mode = EPI_RK;
    ep.stage = st;
    ep.nstages = ns;
    ep.cb = dt * c.rk_b[st];
    ep.need_u = (st == 0);
    for (int t = 0; t < 4; t++) {
      ep.ca[t] = 0.0;
      ep.touched[t] = touched[t];
      ep.P[t] = P[t];
      if (t > st && t < ns) {
        ep.ca[t] = dt * c.rk_A[4 * t + st];
        if (ep.ca[t] != 0.0 && !touched[t]) ep.need_u = 1;
      }
    }
    ep.u = const_cast<double*>(uin);
    ep.acc = a->acc;
    ep.uout = uout;
    for (int d = 0; d < 2; d++) {
      StageEpi e = ep;
      e.first = (d == 0);
      e.last = (d == 1);
      e.tape = tapes ? tapes[2 * st + d] : nullptr;
      if (e.tape && a->tape_w == TAPE_WIDE)
        AK(launch_hyp_euler2d_wide_tape(d, U, a->H, a->d_dxinv + a->dx_off[d], a->G, a->pp, e, a->hl[d], strm));
      else
        AK(launch_hyp_euler2d(d, c.interp, c.upwind, U, a->H, a->d_dxinv + a->dx_off[d], a->G, a->pp, e, a->hl[d],
                              strm));
    }
    for (int t = st + 1; t < ns; t++)
      if (ep.ca[t] != 0.0) touched[t] = 1;
  }
  return GB_OK;
}

// The adjoint of one step: given the step's stage states U[0..ns-1] and, in
// a->ubar, the adjoint of its result, leaves the adjoint of its input in a->ubar:
//   kbar_s = dt b_s ubar + sum_{t>s} dt A_ts Ubar_t,  Ubar_s = J(U_s)^T kbar_s,
//   ubar  += sum_s Ubar_s.
static int adj_back_step(gb_adjoint* a, const double* const* U, double* const* tapes) {
  const gb_config& c = a->cfg;
  const int ns = c.rk_nstages;
  const double dt = c.dt;
  for (int s = ns - 1; s >= 0; s--) {
    AdjTerms kt = terms0();
    if (c.rk_b[s] != 0.0) {
      kt.p[kt.n] = a->ubar;
      kt.c[kt.n++] = dt * c.rk_b[s];
    }
    for (int t = s + 1; t < ns; t++)
      if (c.rk_A[4 * t + s] != 0.0) {
        kt.p[kt.n] = a->Ub[t];
        kt.c[kt.n++] = dt * c.rk_A[4 * t + s];
      }
    if (kt.n == 0) continue;
    int rc = adj_vjp(a, U[s], kt, a->Ub[s], tapes ? tapes + 2 * s : nullptr);
    if (rc) return rc;
  }
  adj_gather_kernel<<<interior_grid(a), 256, 0, a->stream>>>(a->ubar, a->Ub[0], a->Ub[1], a->Ub[2], a->Ub[3], ns,
                                                              a->G);
  AK(cudaGetLastError());
  return GB_OK;
}

// Buffer of segment j: the last segment (kept by the forward sweep) uses 0,
// earlier ones alternate.
static int segbuf(const gb_adjoint* a, int j) { return (a->nseg - 1 - j) & (a->nbuf - 1); }
static double* ustate(gb_adjoint* a, int j, int i) { return i == 0 ? a->ck[j] : a->su[segbuf(a, j)][i]; }
static double* const* stages(gb_adjoint* a, int b, int i) { return &a->sP[b][(size_t)i * 4]; }
static double* const* tapes(gb_adjoint* a, int b, int i) { return &a->sT[b][(size_t)i * 8]; }

extern "C" int gb_adjoint_create(const gb_config* cfg, const double* dxinv, int nsteps, int ncheck, int device,
                                 gb_adjoint** out) {
  return gb_adjoint_create_ex(cfg, dxinv, nsteps, ncheck, device, -1, out);
}

extern "C" int gb_adjoint_create_ex(const gb_config* cfg, const double* dxinv, int nsteps, int ncheck, int device,
                                    long long wide_tape_max, gb_adjoint** out) {
  if (!out || !dxinv || nsteps < 1) { gbh_set_error("gb_adjoint_create: bad argument"); return GB_ERR_ARG; }
  *out = nullptr;
  int rc = gbh_validate(cfg);
  if (rc) return rc;
  if (cfg->model != GB_MODEL_EULER2D || cfg->interp != GB_INTERP_COMPONENTS || cfg->upwind != GB_UPWIND_ROE ||
      cfg->weno_weights != GB_WENO_JS || cfg->hyp_scheme != GB_SCHEME_WENO5) {
    gbh_set_error("gb_adjoint_create: the adjoint covers Euler2D with component-wise Jiang-Shu WENO5 and Roe "
                  "upwinding");
    return GB_ERR_UNSUPPORTED;
  }
  DevGeom G;
  std::vector<int> mem;
  long long npts = gbh_geometry(*cfg, G, &mem);
  for (int z = 0; z < cfg->nzones; z++)
    if (cfg->zones[z][0] == GB_BC_SPONGE) mem.push_back(z);
  if (!mem.empty()) {
    gbh_set_error("gb_adjoint_create: every boundary face must be one whole-face periodic or extrapolate zone, "
                  "with no sponge zone");
    return GB_ERR_UNSUPPORTED;
  }
  gb_adjoint* a = new gb_adjoint();
  a->cfg = *cfg;
  a->G = G;
  a->nvals = (size_t)npts * NV2;
  a->pp.gamma = cfg->gamma;
  a->pp.gm1 = cfg->gamma - 1.0;
  a->pp.inv_gm1 = 1.0 / (cfg->gamma - 1.0);
  a->pp.eps = cfg->weno_eps;
  a->pp.wtype = WENO_W_JS;
  a->pp.gf = a->pp.gg = nullptr;
  for (int d = 0; d < 2; d++) {
    a->hl[d].seg = 32;
    a->hl[d].block = 128;
  }
  a->dx_off[0] = 0;
  a->dx_off[1] = cfg->dim[0] + 2 * cfg->ghosts;
  const long long ndx = a->dx_off[1] + cfg->dim[1] + 2 * cfg->ghosts;
  a->nsteps = nsteps;
  if (ncheck <= 0) {
    ncheck = 1;
    while ((long long)ncheck * ncheck < nsteps) ncheck++;
  }
  if (ncheck > nsteps) ncheck = nsteps;
  a->seglen = (nsteps + ncheck - 1) / ncheck;
  a->nseg = (nsteps + a->seglen - 1) / a->seglen;
  a->lastlen = nsteps - (a->nseg - 1) * a->seglen;
  const int ns = cfg->rk_nstages;
  // arrays: checkpoints, per segment buffer seglen+1 states and seglen*(ns-1)
  // stage states, acc, hyperbolic accumulator, 4 stage adjoints, ubar
  a->nbuf = a->nseg > 1 ? 2 : 1;
  size_t narr = (size_t)a->nseg + (size_t)a->nbuf * ((a->seglen + 1) + (size_t)a->seglen * (ns - 1)) + 1 + 1 + 4 + 1;
  a->bytes = narr * a->nvals * sizeof(double);
  if (device >= 0) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { gbh_set_error("cudaSetDevice(%d): %s", device, cudaGetErrorString(e)); delete a; return GB_ERR_CUDA; }
  }
  cudaGetDevice(&a->device);
  // interface tapes: per buffer, step and stage, at every interface of both
  // directions uL and uR (8 values), widened to TAPE_WIDE values (the WENO pairs'
  // smoothness terms and normalisations) when the wide tapes take at most 60 % of
  // the device memory left free by the state arrays (a 256^2 RK4 run of 400 steps
  // keeping every state: 121 GB of wide tapes, within a GB300's 280 GB)
  const size_t nif = (size_t)cfg->dim[1] * (cfg->dim[0] + 1) + (size_t)cfg->dim[0] * (cfg->dim[1] + 1);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
  const size_t room = free_b > a->bytes ? free_b - a->bytes : 0;
  const size_t wide_bytes = (size_t)a->nbuf * a->seglen * ns * nif * TAPE_WIDE * sizeof(double);
  const size_t cap = wide_tape_max < 0 ? room / 10 * 6 : (size_t)wide_tape_max;
  a->tape_w = wide_bytes <= cap ? TAPE_WIDE : 8;
  const size_t tape_x = (size_t)cfg->dim[1] * (cfg->dim[0] + 1) * a->tape_w;
  const size_t tape_y = (size_t)cfg->dim[0] * (cfg->dim[1] + 1) * a->tape_w;
  const size_t tape_bytes = (size_t)a->nbuf * a->seglen * ns * (tape_x + tape_y) * sizeof(double);
  a->bytes += tape_bytes;
  const size_t block_bytes = a->bytes - tape_bytes;
  cudaError_t e = cudaMalloc((void**)&a->block, block_bytes);
  if (e == cudaSuccess) e = cudaMemset(a->block, 0, block_bytes);
  // tile shares: per line, tiles x (TI + 5) cells x 4, the larger of tiles of 32 and 64
  for (int d = 0; d < 2 && e == cudaSuccess; d++) {
    const long long n = a->G.dim[d] + 1, lines = a->G.dim[1 - d];
    const long long c32 = (n + 31) / 32 * 37, c64 = (n + 63) / 64 * 69;
    const size_t sb = (size_t)(lines * (c32 > c64 ? c32 : c64) * NV2) * sizeof(double);
    e = cudaMalloc((void**)&a->slot[d], sb);
    a->bytes += sb;
  }
  if (e == cudaSuccess) e = cudaMalloc((void**)&a->tblock2, tape_bytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&a->d_dxinv, ndx * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpy(a->d_dxinv, dxinv, ndx * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a->ev_start, cudaEventDisableTiming);
  a->ev_rec.assign(a->nseg, nullptr);
  a->ev_back.assign(a->nseg, nullptr);
  for (int j = 0; j < a->nseg && e == cudaSuccess; j++) {
    e = cudaEventCreateWithFlags(&a->ev_rec[j], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a->ev_back[j], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    gbh_set_error("gb_adjoint_create: %s", cudaGetErrorString(e));
    a->own_stream = a->stream != nullptr;
    gb_adjoint_destroy(a);
    return e == cudaErrorMemoryAllocation ? GB_ERR_NOMEM : GB_ERR_CUDA;
  }
  a->own_stream = true;
  double* p = a->block;
  auto take = [&]() { double* r = p; p += a->nvals; return r; };
  for (int j = 0; j < a->nseg; j++) a->ck.push_back(take());
  for (int b = 0; b < a->nbuf; b++) {
    for (int i = 0; i <= a->seglen; i++) a->su[b].push_back(take());
    a->sP[b].assign((size_t)a->seglen * 4, nullptr);
    for (int i = 0; i < a->seglen; i++)
      for (int t = 1; t < ns; t++) a->sP[b][(size_t)i * 4 + t] = take();
  }
  double* tp = a->tblock2;
  for (int b = 0; b < a->nbuf; b++) {
    a->sT[b].assign((size_t)a->seglen * 8, nullptr);
    for (int i = 0; i < a->seglen; i++)
      for (int t = 0; t < ns; t++) {
        a->sT[b][((size_t)i * 4 + t) * 2 + 0] = tp;
        tp += tape_x;
        a->sT[b][((size_t)i * 4 + t) * 2 + 1] = tp;
        tp += tape_y;
      }
  }
  a->acc = take();
  a->H = take();
  for (int s = 0; s < 4; s++) a->Ub[s] = take();
  a->ubar = take();
  // which stages read their stage array (A row not all zero)
  for (int t = 1; t < ns; t++)
    for (int s = 0; s < t; s++)
      if (cfg->rk_A[4 * t + s] != 0.0) a->touched[t] = 1;
  *out = a;
  return GB_OK;
}

extern "C" void gb_adjoint_destroy(gb_adjoint* a) {
  if (!a) return;
  if (a->stream) cudaStreamSynchronize(a->stream);
  if (a->aux) cudaStreamSynchronize(a->aux);
  for (cudaEvent_t ev : a->ev_rec)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : a->ev_back)
    if (ev) cudaEventDestroy(ev);
  if (a->ev_start) cudaEventDestroy(a->ev_start);
  if (a->aux) cudaStreamDestroy(a->aux);
  cudaFree(a->block);
  cudaFree(a->slot[0]);
  cudaFree(a->slot[1]);
  cudaFree(a->tblock);
  cudaFree(a->tblock2);
  cudaFree(a->d_dxinv);
  if (a->own_stream) cudaStreamDestroy(a->stream);
  delete a;
}

extern "C" int gb_adjoint_set_stream(gb_adjoint* a, void* stream) {
  if (!a) { gbh_set_error("null adjoint"); return GB_ERR_ARG; }
  if (a->own_stream) {
    cudaStreamSynchronize(a->stream);
    cudaStreamDestroy(a->stream);
    a->own_stream = false;
  }
  if (stream) {
    a->stream = (cudaStream_t)stream;
  } else {
    AK(cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking));
    a->own_stream = true;
  }
  return GB_OK;
}

extern "C" int gb_adjoint_sync(gb_adjoint* a) {
  if (!a) { gbh_set_error("null adjoint"); return GB_ERR_ARG; }
  AK(cudaStreamSynchronize(a->stream));
  return GB_OK;
}

extern "C" int gb_adjoint_set_launch(gb_adjoint* a, int which, int seg, int block) {
  if (!a || which < 0 || which > 3) { gbh_set_error("gb_adjoint_set_launch: bad argument"); return GB_ERR_ARG; }
  if (which < 2) {
    if (seg > 0 || seg == -32 || seg == -64 || seg == -128) a->hl[which].seg = seg;  // -t: tiles of t interfaces
    if (block > 0) {
      if (block % 32 || block > 128) { gbh_set_error("block must be a multiple of 32, at most 128"); return GB_ERR_ARG; }
      a->hl[which].block = block;
    }
  } else {
    if (seg > 0 || seg == -32 || seg == -64) a->vjp_seg[which - 2] = seg;  // -t: tiles of t interfaces
    if (block > 0) {  // one block size for the adjoint kernel's single launch
      if (block % 32 || block > 128) { gbh_set_error("block must be a multiple of 32, at most 128"); return GB_ERR_ARG; }
      a->vjp_block = block;
    }
  }
  return GB_OK;
}

extern "C" int gb_adjoint_get_launch(const gb_adjoint* a, int which, int* seg, int* block) {
  if (!a || which < 0 || which > 3 || !seg || !block) { gbh_set_error("gb_adjoint_get_launch: bad argument"); return GB_ERR_ARG; }
  if (which < 2) {
    *seg = a->hl[which].seg;
    *block = a->hl[which].block;
  } else {
    *seg = a->vjp_seg[which - 2];
    *block = a->vjp_block;
  }
  return GB_OK;
}

extern "C" int gb_adjoint_info(const gb_adjoint* a, int* seglen, int* nseg, long long* recomputed, long long* bytes) {
  if (!a) { gbh_set_error("null adjoint"); return GB_ERR_ARG; }
  if (seglen) *seglen = a->seglen;
  if (nseg) *nseg = a->nseg;
  if (recomputed) *recomputed = a->recomputed;
  if (bytes) *bytes = (long long)a->bytes;
  return GB_OK;
}

extern "C" int gb_adjoint_rhs_vjp(gb_adjoint* a, const double* u, const double* kbar, double* ubar) {
  if (!a || !u || !kbar || !ubar) { gbh_set_error("gb_adjoint_rhs_vjp: null argument"); return GB_ERR_ARG; }
  AK(cudaMemsetAsync(ubar, 0, a->nvals * sizeof(double), a->stream));
  AdjTerms kt = terms0();
  kt.p[0] = kbar;
  kt.c[0] = 1.0;
  kt.n = 1;
  return adj_vjp(a, u, kt, ubar);
}

extern "C" int gb_adjoint_rhs_jvp(gb_adjoint* a, const double* u, const double* du, double* k, double* dk) {
  if (!a || !u || !du || !k || !dk) { gbh_set_error("gb_adjoint_rhs_jvp: null argument"); return GB_ERR_ARG; }
  AK(cudaMemsetAsync(k, 0, a->nvals * sizeof(double), a->stream));
  AK(cudaMemsetAsync(dk, 0, a->nvals * sizeof(double), a->stream));
  return adj_jvp(a, u, du, k, dk);
}

extern "C" int gb_adjoint_forward(gb_adjoint* a, const double* u0, double* uT) {
  if (!a || !u0 || !uT) { gbh_set_error("gb_adjoint_forward: null argument"); return GB_ERR_ARG; }
  const size_t bytes = a->nvals * sizeof(double);
  AK(cudaMemcpyAsync(a->ck[0], u0, bytes, cudaMemcpyDeviceToDevice, a->stream));
  const int L = a->seglen;
  const int bl = segbuf(a, a->nseg - 1), bt = a->nbuf - 1 - bl;  // last segment's buffer, the other
  for (int j = 0; j < a->nseg; j++) {
    const bool last = (j == a->nseg - 1);
    const int len = last ? a->lastlen : L;
    for (int i = 0; i < len; i++) {
      const double* uin;
      double* uout;
      double* const* P;
      double* const* T = nullptr;
      if (last) {
        // the last segment keeps every state (and interface tape) for the backward sweep
        uin = ustate(a, j, i);
        uout = a->su[bl][i + 1];
        P = stages(a, bl, i);
        T = tapes(a, bl, i);
      } else {
        uin = i == 0 ? a->ck[j] : a->su[bt][1 + (i & 1)];
        uout = (i + 1 == len) ? a->ck[j + 1] : a->su[bt][1 + ((i + 1) & 1)];
        P = stages(a, bt, 0);
      }
      int rc = adj_step(a, a->stream, uin, uout, P, T);
      if (rc) return rc;
    }
  }
  AK(cudaMemcpyAsync(uT, a->su[bl][a->lastlen], bytes, cudaMemcpyDeviceToDevice, a->stream));
  a->forward_done = true;
  a->recomputed = 0;
  return GB_OK;
}

// Backward sweep.  Segment j is reversed on the main stream from its buffer
// while segment j-1 is recomputed from its checkpoint into the other buffer
// on the second stream; reversing j-1 waits for that recomputation, and
// recomputing j-2 waits until the reversal of j has released the buffer.
extern "C" int gb_adjoint_backward(gb_adjoint* a, const double* ubarT, double* ubar0) {
  if (!a || !ubarT || !ubar0) { gbh_set_error("gb_adjoint_backward: null argument"); return GB_ERR_ARG; }
  if (!a->forward_done) { gbh_set_error("gb_adjoint_backward: no forward sweep to reverse"); return GB_ERR_ARG; }
  const size_t bytes = a->nvals * sizeof(double);
  const int ns = a->cfg.rk_nstages;
  AK(cudaMemcpyAsync(a->ubar, ubarT, bytes, cudaMemcpyDeviceToDevice, a->stream));
  for (int s = 0; s < 4; s++) AK(cudaMemsetAsync(a->Ub[s], 0, bytes, a->stream));
  AK(cudaEventRecord(a->ev_start, a->stream));
  AK(cudaStreamWaitEvent(a->aux, a->ev_start, 0));
  for (int j = a->nseg - 1; j >= 0; j--) {
    if (j >= 1) {
      const int jr = j - 1, b = segbuf(a, jr);
      if (jr + 2 <= a->nseg - 1) AK(cudaStreamWaitEvent(a->aux, a->ev_back[jr + 2], 0));
      for (int i = 0; i < a->seglen; i++) {
        int rc = adj_step(a, a->aux, ustate(a, jr, i), a->su[b][i + 1], stages(a, b, i), tapes(a, b, i));
        if (rc) return rc;
      }
      AK(cudaEventRecord(a->ev_rec[jr], a->aux));
      a->recomputed += a->seglen;
    }
    if (j < a->nseg - 1) AK(cudaStreamWaitEvent(a->stream, a->ev_rec[j], 0));
    const int len = (j == a->nseg - 1) ? a->lastlen : a->seglen;
    const int b = segbuf(a, j);
    for (int i = len - 1; i >= 0; i--) {
      const double* U[4];
      for (int t = 0; t < ns; t++) U[t] = (t == 0 || !a->touched[t]) ? ustate(a, j, i) : a->sP[b][(size_t)i * 4 + t];
      int rc = adj_back_step(a, U, tapes(a, b, i));
      if (rc) return rc;
    }
    AK(cudaEventRecord(a->ev_back[j], a->stream));
  }
  AK(cudaMemcpyAsync(ubar0, a->ubar, bytes, cudaMemcpyDeviceToDevice, a->stream));
  return GB_OK;
}

// Tangent-linear model of nsteps Runge-Kutta steps with the dual-number
// right-hand side: (u, du) advanced together.
extern "C" int gb_adjoint_tlm(gb_adjoint* a, const double* u0, const double* du0, double* uT, double* duT) {
  if (!a || !u0 || !du0 || !uT || !duT) { gbh_set_error("gb_adjoint_tlm: null argument"); return GB_ERR_ARG; }
  const size_t bytes = a->nvals * sizeof(double);
  const gb_config& c = a->cfg;
  const int ns = c.rk_nstages;
  const double dt = c.dt;
  if (!a->tblock) {
    AK(cudaMalloc((void**)&a->tblock, 12 * bytes));
    AK(cudaMemsetAsync(a->tblock, 0, 12 * bytes, a->stream));
    double* p = a->tblock;
    a->tu = p; p += a->nvals;
    a->tdu = p; p += a->nvals;
    a->tU = p; p += a->nvals;
    a->tdU = p; p += a->nvals;
    for (int s = 0; s < 4; s++) { a->tK[s] = p; p += a->nvals; a->tdK[s] = p; p += a->nvals; }
  }
  AK(cudaMemcpyAsync(a->tu, u0, bytes, cudaMemcpyDeviceToDevice, a->stream));
  AK(cudaMemcpyAsync(a->tdu, du0, bytes, cudaMemcpyDeviceToDevice, a->stream));
  for (int n = 0; n < a->nsteps; n++) {
    for (int s = 0; s < ns; s++) {
      const double *U = a->tu, *dU = a->tdu;
      AdjTerms t = terms0(), dtm = terms0();
      for (int j = 0; j < s; j++)
        if (c.rk_A[4 * s + j] != 0.0) {
          t.p[t.n] = a->tK[j];
          t.c[t.n++] = dt * c.rk_A[4 * s + j];
          dtm.p[dtm.n] = a->tdK[j];
          dtm.c[dtm.n++] = dt * c.rk_A[4 * s + j];
        }
      if (t.n) {
        int rc = adj_lincomb(a, a->tU, a->tu, t);
        if (!rc) rc = adj_lincomb(a, a->tdU, a->tdu, dtm);
        if (rc) return rc;
        U = a->tU;
        dU = a->tdU;
      }
      int rc = adj_jvp(a, U, dU, a->tK[s], a->tdK[s]);
      if (rc) return rc;
    }
    AdjTerms t = terms0(), dtm = terms0();
    for (int s = 0; s < ns; s++)
      if (c.rk_b[s] != 0.0) {
        t.p[t.n] = a->tK[s];
        t.c[t.n++] = dt * c.rk_b[s];
        dtm.p[dtm.n] = a->tdK[s];
        dtm.c[dtm.n++] = dt * c.rk_b[s];
      }
    int rc = adj_lincomb(a, a->tu, a->tu, t);
    if (!rc) rc = adj_lincomb(a, a->tdu, a->tdu, dtm);
    if (rc) return rc;
  }
  AK(cudaMemcpyAsync(uT, a->tu, bytes, cudaMemcpyDeviceToDevice, a->stream));
  AK(cudaMemcpyAsync(duT, a->tdu, bytes, cudaMemcpyDeviceToDevice, a->stream));
  return GB_OK;
}
