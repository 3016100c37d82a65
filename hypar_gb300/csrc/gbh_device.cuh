// gbh_device.cuh -- FP64 device math for the fused WENO5 right-hand side.
//
// Physics (Euler1D, Euler2D, NavierStokes3D), Jiang-Shu WENO5 and Roe / LLF /
// RF upwinding, written for the GB300 FP64 pipe: every formula is the
// reference's (file:line cited per routine) rearranged so that one interface
// costs as few FP64 instructions as possible.  Results agree with the
// reference to rounding (the parity tests hold them to a relative L2 of 1e-12
// per right-hand side); nothing here is bit-for-bit by design.
#pragma once

#include <cstdint>

namespace gbh {

enum { MODEL_EULER1D = 1, MODEL_EULER2D = 2, MODEL_NS3D = 3 };
enum { UPW_ROE = 0, UPW_LLF = 1, UPW_RF = 2, UPW_RUS = 3, UPW_SWFS = 4 };

template <int M> struct ModelTraits;
template <> struct ModelTraits<MODEL_EULER1D> { static constexpr int NV = 3, ND = 1; };
template <> struct ModelTraits<MODEL_EULER2D> { static constexpr int NV = 4, ND = 2; };
template <> struct ModelTraits<MODEL_NS3D>    { static constexpr int NV = 5, ND = 3; };

struct PhysParams {
  double gamma, gm1, inv_gm1, eps;
  int wtype;  // WENO weights: WENO_W_* (the kernels take Jiang-Shu unless instantiated for the others)
  // NavierStokes3D gravity (kernels instantiated with GRAV): the hydrostatic density and
  // pressure variations f, g at every point with ghosts, the acceleration and RT = p0 / rho0
  const double* gf;
  const double* gg;
  double grav[3], RT;
};

// WENO5 nonlinear weight formulations (weno.inp flags, WENOFifthOrderCalculateWeights.c:40-64;
// no_limiting keeps the optimal weights, InitializeSolvers.c:219 / HyperbolicFunction.c:62).
enum { WENO_W_JS = 0, WENO_W_MAPPED = 1, WENO_W_BORGES = 2, WENO_W_YC = 3, WENO_W_NONE = 4 };

// ---------------------------------------------------------------------------
// Reciprocal and square root.
//
// The FP64 pipe of a GB300 SM retires only two operations per clock, so a
// correctly rounded IEEE division (a multi-instruction sequence) is replaced by
// refinement of the hardware reciprocal / reciprocal-square-root estimates
// (rcp.approx.ftz.f64 / rsqrt.approx.ftz.f64, PTX ISA).  With e = 1 - x r the
// relative error of an estimate r of 1/x, 1/x = r / (1 - e) = r (1 + e + e^2 + ...):
// the third-order step r' = r + r (e + e^2) (Householder's method of order 3 for
// the reciprocal) leaves a relative error of order e^3, far below 2^-53 from the
// hardware estimate, in three FMAs.  For 1/sqrt(x), with e = 1 - x y^2,
// 1/sqrt(x) = y (1 - e)^(-1/2) = y (1 + e/2 + 3 e^2 / 8 + ...) likewise.  Results are
// within one unit in the last place of the correctly rounded value: the GPU test
// test_gpu_math.py checks that bound over 1e6 inputs from each range the path
// feeds (1e-30 .. 1e30 for the reciprocals, 1e-6 .. 1e6 for the square roots).
// Inputs are positive normal numbers on this path (densities, squared sound
// speeds, WENO denominators >= eps^2).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rcp_approx(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ double rsqrt_approx(double x) {
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ double nr_rcp(double x) {
  const double r = rcp_approx(x);
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
// sqrt(x) via y ~ 1/sqrt(x):  y' = y + y(1 - x y^2)/2, then s = x y refined once
// with s' = s + y (x - s^2)/2 (Newton on s^2 = x).
__device__ __forceinline__ double nr_sqrt(double x) {
  double y = rsqrt_approx(x);
  double e = fma(-x * y, y, 1.0);
  y = fma(y, 0.5 * e, y);
  double s = x * y;
  double h = 0.5 * y;
  double d = fma(-s, s, x);
  s = fma(d, h, s);
  return s;
}

// ---------------------------------------------------------------------------
// Conserved -> primitive.  Euler1D: include/physicalmodels/euler1d.h:81-89,
// Euler2D: euler2d.h:44-54, NavierStokes3D (with its rho == 0 guard):
// navierstokes3d.h:98-108.
// ---------------------------------------------------------------------------
template <int M>
struct Prim {
  double rho, rinv, vel[3], P, e;
};

template <int M>
__device__ __forceinline__ Prim<M> to_prim(const double* u, const PhysParams& pp) {
  constexpr int ND = ModelTraits<M>::ND, NV = ModelTraits<M>::NV;
  Prim<M> q;
  q.rho = u[0];
  q.rinv = nr_rcp(q.rho);
  double vsq = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) q.vel[k] = 0.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    double v = u[1 + k] * q.rinv;
    if (M == MODEL_NS3D) v = (q.rho == 0.0) ? 0.0 : v;
    q.vel[k] = v;
    vsq = fma(v, v, vsq);
  }
  q.e = u[NV - 1];
  q.P = (q.e - 0.5 * q.rho * vsq) * pp.gm1;
  return q;
}

// Cell flux along DIR (Euler1DFlux.c:16-45, Euler2DFlux.c:7-36, NavierStokes3DFlux.c:23-60).
template <int M, int DIR>
__device__ __forceinline__ void cell_flux(const Prim<M>& q, double* f) {
  constexpr int ND = ModelTraits<M>::ND, NV = ModelTraits<M>::NV;
  double vn = q.vel[DIR];
  double mn = q.rho * vn;
  f[0] = mn;
#pragma unroll
  for (int k = 0; k < ND; k++) f[1 + k] = mn * q.vel[k];
  f[1 + DIR] += q.P;
  f[NV - 1] = (q.e + q.P) * vn;
}

// UFunction value of the energy component: NavierStokes3D recomputes it
// (NavierStokes3DModifiedSolution.c:56-65, gravity fields = 1); Euler1D
// (gravity field exp(0) = 1) and Euler2D (no UFunction) leave u unchanged.
template <int M>
__device__ __forceinline__ double ufunc_energy(const Prim<M>& q, const PhysParams& pp, double e) {
  if (M == MODEL_NS3D) {
    double vsq = q.vel[0] * q.vel[0] + q.vel[1] * q.vel[1] + q.vel[2] * q.vel[2];
    return q.P * pp.inv_gm1 + 0.5 * q.rho * vsq;
  }
  return e;
}

// Roe-average ingredients of a state: sqrt(rho), velocity, total enthalpy.
struct RoeSide {
  double t, vel[3], H;
};
template <int M>
__device__ __forceinline__ RoeSide roe_side(const Prim<M>& q) {
  RoeSide s;
  s.t = nr_sqrt(q.rho);
#pragma unroll
  for (int k = 0; k < 3; k++) s.vel[k] = q.vel[k];
  s.H = (q.e + q.P) * q.rinv;
  return s;
}

// ---------------------------------------------------------------------------
// Eigen-structure at a Roe-averaged state (_Euler1DRoeAverage_ euler1d.h:134-160,
// _Euler2DRoeAverage_ euler2d.h:70-108, _NavierStokes3DRoeAverage_
// navierstokes3d.h:147-180) in factored form.  With
//   s = (gamma-1) (ek q0 - v.q_mom + q_E),  t = a (u_n q0 - q_{1+d}),
// the reference's left eigenvectors (euler1d.h:209-228, euler2d.h:128-175,
// navierstokes3d.h:317-408) are, row by row,
//   acoustic u_n-a :  (s + t) * hac      acoustic u_n+a :  (s - t) * hac
//   entropy        :  q0 - s / a^2       shear (each transverse e): v_e q0 - q_{1+e}
// with hac = 1/(2a^2) (Euler2D, NavierStokes3D) or 1/(rho a) (Euler1D), up to
// row signs, which neither the WENO weights (squares) nor the interpolation
// (linear) see.  The matching right eigenvectors (columns) are
//   (1, v -+ a e_d, H -+ a u_n) * rs,  (1, v, ek),  -(e_{1+e} + v_e e_E)
// with rs = 1/(2 a^2 hac).
// ---------------------------------------------------------------------------
struct Eig {
  double vel[3], un, a, ek, H, hac, rs, inv_a2, rho;
  double gh, gi, ah, aun;  // (gamma-1) hac, (gamma-1)/a^2, a hac, a u_n
};

// 1/sqrt(x): the hardware estimate y refined by the third-order step
// y' = y + y (e/2 + 3 e^2/8), e = 1 - x y^2 (same error bound as nr_rcp).
__device__ __forceinline__ double nr_rsqrt(double x) {
  const double y = rsqrt_approx(x);
  const double e = fma(-x * y, y, 1.0);
  return fma(y, e * fma(0.375, e, 0.5), y);
}

// The eigen-system's remaining quantities once the Roe-averaged velocity, enthalpy
// and density (E.vel, E.H, E.rho) and |v|^2 are set.
template <int M, int DIR>
__device__ __forceinline__ void roe_eig_finish(Eig& E, double vsq, const PhysParams& pp);

template <int M, int DIR>
__device__ __forceinline__ Eig roe_eig(const RoeSide& L, const RoeSide& R, const PhysParams& pp) {
  constexpr int ND = ModelTraits<M>::ND;
  Eig E;
  double inv = nr_rcp(L.t + R.t);
  double vsq = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) E.vel[k] = 0.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    E.vel[k] = fma(L.t, L.vel[k], R.t * R.vel[k]) * inv;
    vsq = fma(E.vel[k], E.vel[k], vsq);
  }
  E.H = fma(L.t, L.H, R.t * R.H) * inv;
  E.rho = L.t * R.t;
  roe_eig_finish<M, DIR>(E, vsq, pp);
  return E;
}

// Roe average of two conserved states in one pass (the reconstructed states of
// Euler2D's Roe upwinding, Euler2DUpwind.c:39): with r = 1/sqrt(rho) of each state,
// sqrt(rho) = rho r, sqrt(rho) v = m r and sqrt(rho) H = (e + P) r, where
// P = (e - |m r|^2 / 2) (gamma - 1); so neither 1/rho nor the velocities are formed.
template <int M, int DIR>
__device__ __forceinline__ Eig roe_eig_cons(const double* a, const double* b, const PhysParams& pp) {
  constexpr int ND = ModelTraits<M>::ND, NV = ModelTraits<M>::NV;
  const double ra = nr_rsqrt(a[0]), rb = nr_rsqrt(b[0]);
  const double ta = a[0] * ra, tb = b[0] * rb;
  double wa[3], wb[3], qa = 0.0, qb = 0.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    wa[k] = a[1 + k] * ra;
    wb[k] = b[1 + k] * rb;
    qa = fma(wa[k], wa[k], qa);
    qb = fma(wb[k], wb[k], qb);
  }
  const double Pa = fma(-0.5, qa, a[NV - 1]) * pp.gm1, Pb = fma(-0.5, qb, b[NV - 1]) * pp.gm1;
  Eig E;
  const double inv = nr_rcp(ta + tb);
  double vsq = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) E.vel[k] = 0.0;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    E.vel[k] = (wa[k] + wb[k]) * inv;
    vsq = fma(E.vel[k], E.vel[k], vsq);
  }
  E.H = fma(a[NV - 1] + Pa, ra, (b[NV - 1] + Pb) * rb) * inv;
  E.rho = ta * tb;
  roe_eig_finish<M, DIR>(E, vsq, pp);
  return E;
}

// Steger-Warming flux vector splitting of one conserved state along DIR (PLUS: the
// part of the non-negative eigenvalues, else of the non-positive ones), in the
// reference's expressions: Euler1DUpwind.c:336-350 (Euler1D, whose split takes v + c
// for the plus part and v - c for the minus part) and Euler2DUpwind.c:244-276.
template <int M, int DIR, bool PLUS>
__device__ __forceinline__ void swfs_half(const double* u, const PhysParams& pp, double* f) {
  const double gamma = pp.gamma;
  const double rho = u[0];
  if (M == MODEL_EULER1D) {
    const double v = u[1] / rho, e = u[2];
    const double P = (e - 0.5 * rho * v * v) * (gamma - 1.0);
    const double c = sqrt(gamma * P / rho);
    const double term = rho / (2.0 * gamma);
    if (PLUS) {
      f[0] = term * (2 * gamma * v + c - v);
      f[1] = term * (2 * (gamma - 1.0) * v * v + (v + c) * (v + c));
      f[2] = term * ((gamma - 1.0) * v * v * v + 0.5 * (v + c) * (v + c) * (v + c) +
                     ((3.0 - gamma) * (v + c) * c * c) / (2.0 * (gamma - 1.0)));
    } else {
      f[0] = term * (v - c);
      f[1] = term * (v - c) * (v - c);
      f[2] = term * (0.5 * (v - c) * (v - c) * (v - c) + ((3.0 - gamma) * (v - c) * c * c) / (2.0 * (gamma - 1.0)));
    }
  } else {
    const double vx = u[1] / rho, vy = u[2] / rho, e = u[3];
    const double P = (e - 0.5 * rho * ((vx * vx) + (vy * vy))) * (gamma - 1.0);
    const double c = sqrt(gamma * P / rho);
    const double term = rho / (2.0 * gamma);
    const double kx = DIR == 0 ? 1.0 : 0.0, ky = DIR == 1 ? 1.0 : 0.0;
    double l0 = kx * vx + ky * vy, l2 = l0 + c, l3 = l0 - c;
    if (PLUS) {
      l0 = l0 < 0.0 ? 0.0 : l0;
      l2 = l2 < 0.0 ? 0.0 : l2;
      l3 = l3 < 0.0 ? 0.0 : l3;
    } else {
      l0 = l0 > 0.0 ? 0.0 : l0;
      l2 = l2 > 0.0 ? 0.0 : l2;
      l3 = l3 > 0.0 ? 0.0 : l3;
    }
    f[0] = term * (2.0 * (gamma - 1.0) * l0 + l2 + l3);
    f[1] = term * (2.0 * (gamma - 1.0) * l0 * vx + l2 * (vx + c * kx) + l3 * (vx - c * kx));
    f[2] = term * (2.0 * (gamma - 1.0) * l0 * vy + l2 * (vy + c * ky) + l3 * (vy - c * ky));
    f[3] = term * ((gamma - 1.0) * l0 * (vx * vx + vy * vy) +
                   0.5 * l2 * ((vx + c * kx) * (vx + c * kx) + (vy + c * ky) * (vy + c * ky)) +
                   0.5 * l3 * ((vx - c * kx) * (vx - c * kx) + (vy - c * ky) * (vy - c * ky)) +
                   ((3.0 - gamma) * (l2 + l3) * c * c) / (2.0 * (gamma - 1.0)));
  }
}

template <int M, int DIR>
__device__ __forceinline__ void roe_eig_finish(Eig& E, double vsq, const PhysParams& pp) {
  E.ek = 0.5 * vsq;
  double a2 = pp.gm1 * (E.H - E.ek);
  double ia = nr_rsqrt(a2);  // 1/a
  E.a = a2 * ia;
  E.inv_a2 = ia * ia;
  E.un = E.vel[DIR];
  if (M == MODEL_EULER1D) {
    // hac = 1/(rho a), rs = rho/(2a) = 1/(2 a^2 hac)
    E.hac = nr_rcp(E.rho) * ia;
    E.rs = 0.5 * E.rho * ia;
  } else {
    E.hac = 0.5 * E.inv_a2;
    E.rs = 1.0;
  }
  E.gh = pp.gm1 * E.hac;
  E.gi = pp.gm1 * E.inv_a2;
  E.ah = E.a * E.hac;
  E.aun = E.a * E.un;
}

// Harten's entropy fix of |lambda| with delta = 1e-6 (Euler2DUpwind.c:45-51,
// NavierStokes3DUpwind.c:97-102): (lambda^2 + delta^2) / (2 delta) inside |lambda| < delta.
// The comparison is made on the bit patterns (non-negative doubles order as their
// integers do; a NaN compares above), which keeps it off the FP64 pipe.
__device__ __forceinline__ double harten_abs(double lam) {
  const double delta = 0.000001, delta2 = delta * delta;
  const double d = fabs(lam);
  return (__double_as_longlong(d) < __double_as_longlong(delta)) ? fma(lam, lam, delta2) * (0.5 / delta) : d;
}

// Characteristic fields, in this order: 0 acoustic (u_n - a), 1 acoustic
// (u_n + a), 2 entropy, 3.. shear components (transverse directions ascending).
template <int M, int DIR>
__device__ __forceinline__ void projL(const Eig& E, const PhysParams& pp, const double* q, double* w) {
  constexpr int ND = ModelTraits<M>::ND, NV = ModelTraits<M>::NV;
  (void)pp;
  double s = fma(E.ek, q[0], q[NV - 1]);  // s / (gamma-1)
#pragma unroll
  for (int k = 0; k < ND; k++) s = fma(-E.vel[k], q[1 + k], s);
  double th = E.ah * fma(E.un, q[0], -q[1 + DIR]);  // t hac
  w[0] = fma(s, E.gh, th);
  w[1] = fma(s, E.gh, -th);
  w[2] = fma(-s, E.gi, q[0]);
  int j = 3;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    if (k == DIR) continue;
    w[j++] = fma(E.vel[k], q[0], -q[1 + k]);
  }
}

template <int M, int DIR>
__device__ __forceinline__ void projR(const Eig& E, const double* w, double* y) {
  constexpr int ND = ModelTraits<M>::ND, NV = ModelTraits<M>::NV;
  double Wm = w[0], Wp = w[1];
  if (M == MODEL_EULER1D) {
    Wm *= E.rs;
    Wp *= E.rs;
  }
  double sa = Wm + Wp;
  double da = Wp - Wm;
  double y0 = sa + w[2];
  double yE = fma(E.H, sa, fma(E.aun, da, E.ek * w[2]));
  int j = 3;
#pragma unroll
  for (int k = 0; k < ND; k++) {
    if (k == DIR) {
      y[1 + k] = fma(E.un, y0, E.a * da);
    } else {
      y[1 + k] = fma(E.vel[k], y0, -w[j]);
      yE = fma(-E.vel[k], w[j], yE);
      j++;
    }
  }
  y[0] = y0;
  y[NV - 1] = yE;
}

// Eigenvalues in the same field order.
template <int M>
__device__ __forceinline__ void eigvals(double un, double a, double* lam) {
  constexpr int NV = ModelTraits<M>::NV;
  lam[0] = un - a;
  lam[1] = un + a;
#pragma unroll
  for (int k = 2; k < NV; k++) lam[k] = un;
}

// ---------------------------------------------------------------------------
// WENO5 with Jiang-Shu weights (_WENOWeights_v_JS_, include/interpolation.h:265-285,
// optimal weights 0.1/0.6/0.3 at :228-232) and the fifth-order interpolant
// (Interp1PrimFifthOrderWENO.c:143-158), evaluated for the left- AND the
// right-biased reconstruction of one interface together.
//
// p[0..5] are the six cells j-2..j+3 of interface j+1/2; the left-biased
// stencil (m3..p2) is p[0..4], the right-biased one p[5..1].  The two share
// the second differences of the sub-stencils centred at p[2] and p[3] and two
// of their candidate polynomials.  Per side, with beta_k the smoothness
// indicators and q_k = (beta_k + eps)^2,
//   w_k = c_k/q_k / sum_j c_j/q_j = c_k prod_{j!=k} q_j / sum_j c_j prod_{i!=j} q_i,
// and because the weights are ratios, every beta_k + eps may be scaled by the
// same factor: B_k = 4 (beta_k + eps) = (13/3) d_k^2 + g_k^2 + 4 eps.  The
// candidates are kept unnormalised (f = (2 m3 - 7 m2 + 11 m1)/6, ...): the 1/6
// and the optimal weights (0.1, 0.6, 0.3) = 0.1 (1, 6, 3) fold into the final
// normalisation.  The weights come from `w`, the interpolated values from `v`
// (they differ for the u-reconstruction, whose weights are computed from u
// while the values are uC = UFunction(u), HyperbolicFunction.c:201-215).
// ---------------------------------------------------------------------------
//
// C0: the window is given relative to its centre cell p[2] (w[2] = v[2] = 0, not
// read).  The weights depend on differences only and the interpolant reproduces
// constants, so the pair of the shifted window is the pair of the original one minus
// p[2]'s value; with a zero centre a third of the stencil terms drop out, and the
// values stay of the size of the window's variation, so their rounding is far
// smaller than that of reconstructions of O(1) values.
//
// The second half of a pair, from the squared smoothness terms q = B^2 of its six
// sub-stencils: the unnormalised weights (products of the other two q's), the
// candidates of the values v and the two normalisations (rL, rR: their reciprocals).
template <bool C0>
__device__ __forceinline__ void weno5_pair_finish(const double* v, double qL1, double qL2, double qL3, double qR1,
                                                  double qR2, double qR3, double& outL, double& outR, double& rL,
                                                  double& rR) {
  double aL1 = qL2 * qL3, aL2 = qL1 * qL3, aL3 = qL1 * qL2;  // x (1, 1/6, 1/3) of the weights
  double aR1 = qR2 * qR3, aR2 = qR1 * qR3, aR3 = qR1 * qR2;
  // candidates (times 6): two of them shared between the sides
  double cL1 = C0 ? fma(2.0, v[0], -7.0 * v[1]) : fma(2.0, v[0], fma(-7.0, v[1], 11.0 * v[2]));
  double cR1 = fma(2.0, v[5], fma(-7.0, v[4], 11.0 * v[3]));
  double cA = C0 ? fma(2.0, v[3], -v[1]) : fma(5.0, v[2], fma(2.0, v[3], -v[1]));  // left #2, right #3
  double cB = C0 ? fma(5.0, v[3], -v[4]) : fma(5.0, v[3], fma(2.0, v[2], -v[4]));  // left #3, right #2
  double nL = fma(aL1, cL1, fma(6.0 * aL2, cA, (3.0 * aL3) * cB));
  double nR = fma(aR1, cR1, fma(6.0 * aR2, cB, (3.0 * aR3) * cA));
  double DL = fma(36.0, aL2, fma(18.0, aL3, 6.0 * aL1));
  double DR = fma(36.0, aR2, fma(18.0, aR3, 6.0 * aR1));
  rL = nr_rcp(DL);
  rR = nr_rcp(DR);
  outL = nL * rL;
  outR = nR * rR;
}

template <bool TP, bool C0 = false>
__device__ __forceinline__ void weno5_pair_impl(const double* w, const double* v, double eps4, double& outL,
                                                double& outR, double* tp) {
  const double k13 = 13.0 / 3.0;
  // second differences, sub-stencils centred at p1..p4
  double d1 = C0 ? fma(-2.0, w[1], w[0]) : fma(-2.0, w[1], w[0]) + w[2];
  double d2 = C0 ? w[1] + w[3] : fma(-2.0, w[2], w[1]) + w[3];
  double d3 = C0 ? fma(-2.0, w[3], w[4]) : fma(-2.0, w[3], w[2]) + w[4];
  double d4 = fma(-2.0, w[4], w[3]) + w[5];
  double kd1 = k13 * d1, kd2 = k13 * d2, kd3 = k13 * d3, kd4 = k13 * d4;
  // first-difference terms
  double gL1 = C0 ? fma(-4.0, w[1], w[0]) : fma(3.0, w[2], fma(-4.0, w[1], w[0]));
  double gL2 = w[1] - w[3];
  double gL3 = C0 ? fma(-4.0, w[3], w[4]) : fma(3.0, w[2], fma(-4.0, w[3], w[4]));
  double gR1 = fma(3.0, w[3], fma(-4.0, w[4], w[5]));
  double gR2 = C0 ? w[4] : w[4] - w[2];
  double gR3 = C0 ? fma(3.0, w[3], w[1]) : fma(3.0, w[3], fma(-4.0, w[2], w[1]));
  double BL1 = fma(kd1, d1, fma(gL1, gL1, eps4));
  double BL2 = fma(kd2, d2, fma(gL2, gL2, eps4));
  double BL3 = fma(kd3, d3, fma(gL3, gL3, eps4));
  double BR1 = fma(kd4, d4, fma(gR1, gR1, eps4));
  double BR2 = fma(kd3, d3, fma(gR2, gR2, eps4));
  double BR3 = fma(kd2, d2, fma(gR3, gR3, eps4));
  double qL1 = BL1 * BL1, qL2 = BL2 * BL2, qL3 = BL3 * BL3;
  double qR1 = BR1 * BR1, qR2 = BR2 * BR2, qR3 = BR3 * BR3;
  double rL, rR;
  weno5_pair_finish<C0>(v, qL1, qL2, qL3, qR1, qR2, qR3, outL, outR, rL, rR);
  if (TP) {
    // the values the reverse pass would otherwise recompute first
    tp[0] = BL1;
    tp[1] = BL2;
    tp[2] = BL3;
    tp[3] = BR1;
    tp[4] = BR2;
    tp[5] = BR3;
    tp[6] = rL;
    tp[7] = rR;
  }
}

__device__ __forceinline__ void weno5_pair(const double* w, const double* v, double eps4, double& outL,
                                           double& outR) {
  weno5_pair_impl<false>(w, v, eps4, outL, outR, nullptr);
}

// The squared smoothness terms of the three-point sub-stencil (a, b, c) centred at a
// cell, for each of the three places it takes in the pairs around it:
//   ql, g = a - 4b + 3c: the left sub-stencil of a left-biased stencil (BL1 of the
//       interface two cells to its right) and the right-biased stencil's third (BR3 of
//       the interface to its right);
//   qc, g = a - c: the central one (BL2 of the interface to its right, BR2 of the one
//       to its left);
//   qr, g = 3a - 4b + c: BL3 of the interface to its left, BR1 of the one two cells to
//       its left;
// each q = B^2 with B = (13/3) d^2 + g^2 + 4 eps and d = a - 2b + c, as in the pair.
// Interface j+1/2 (window cells j-2 .. j+3) then takes
//   qL = (ql[j-1], qc[j], qr[j+1]),  qR = (qr[j+2], qc[j+1], ql[j]).
__device__ __forceinline__ void weno5_cell_q(double a, double b, double c, double eps4, double& ql, double& qc,
                                             double& qr) {
  const double d = fma(-2.0, b, a) + c;
  const double kde = fma((13.0 / 3.0) * d, d, eps4);
  const double gl = fma(3.0, c, fma(-4.0, b, a));
  const double gc = a - c;
  const double gr = fma(3.0, a, fma(-4.0, b, c));
  const double Bl = fma(gl, gl, kde), Bc = fma(gc, gc, kde), Br = fma(gr, gr, kde);
  ql = Bl * Bl;
  qc = Bc * Bc;
  qr = Br * Br;
}

// A pair from the per-cell table of weno5_cell_q (q's given) and the values v.
template <bool C0>
__device__ __forceinline__ void weno5_pair_q(const double* v, double qL1, double qL2, double qL3, double qR1,
                                             double qR2, double qR3, double& outL, double& outR) {
  double rL, rR;
  weno5_pair_finish<C0>(v, qL1, qL2, qL3, qR1, qR2, qR3, outL, outR, rL, rR);
}

// The pair of a window given relative to its centre cell (w[2] = v[2] = 0).
__device__ __forceinline__ void weno5_pair_c0(const double* w, const double* v, double eps4, double& outL,
                                              double& outR) {
  weno5_pair_impl<false, true>(w, v, eps4, outL, outR, nullptr);
}

// weno5_pair(_c0) that also stores its smoothness terms B (left 1-3, right 1-3) and
// the reciprocals of the two normalisations in tp[0..7] (the adjoint's tape).
template <bool C0 = false>
__device__ __forceinline__ void weno5_pair_tape(const double* w, const double* v, double eps4, double& outL,
                                                double& outR, double* tp) {
  weno5_pair_impl<true, C0>(w, v, eps4, outL, outR, tp);
}

// Left/right WENO5 pair with the other weight formulations (runtime `wtype`).
// B_k = 4 (beta_k + eps) as in weno5_pair; per side, with optimal weights
// c = (0.1, 0.6, 0.3) and candidates p_k:
//   Borges (WENO-Z, _WENOWeights_v_Z_, include/interpolation.h:417-437):
//     a_k = c_k (1 + (tau/(beta_k+eps))^2), tau = |beta_1 - beta_3|, i.e. 4 tau = |B_1 - B_3|;
//   Yamaleev-Carpenter (_WENOWeights_v_YC_, :474-494): the same with
//     tau = (f_{j-2} - 4 f_{j-1} + 6 f_j - 4 f_{j+1} + f_{j+2})^2;
//   both evaluated as a_k = c_k (B_k^2 + T) prod_{j != k} B_j^2, T = (4 tau)^2, so that one
//   reciprocal normalises them;
//   mapped (Henrick et al., _WENOWeights_v_M_, :319-345): JS weights w~ (one reciprocal),
//     then a_k = w~_k (c_k + c_k^2 - 3 c_k w~_k + w~_k^2) / (c_k^2 + w~_k (1 - 2 c_k)),
//     normalised as num_k prod_{j != k} den_j (one more reciprocal);
//   none: the optimal weights.
// out = sum_k a_k p_k / sum_k a_k.
__device__ __forceinline__ void weno5_side_alt(int wtype, double B1, double B2, double B3, double tau4,
                                               double p1, double p2, double p3, double& out) {
  const double c1 = 0.1, c2 = 0.6, c3 = 0.3;
  if (wtype == WENO_W_NONE) {
    out = fma(c1, p1, fma(c2, p2, c3 * p3));
    return;
  }
  const double q1 = B1 * B1, q2 = B2 * B2, q3 = B3 * B3;
  double a1, a2, a3;
  if (wtype == WENO_W_MAPPED) {
    double j1 = c1 * (q2 * q3), j2 = c2 * (q1 * q3), j3 = c3 * (q1 * q2);
    double r = nr_rcp(j1 + j2 + j3);
    double w1 = j1 * r, w2 = j2 * r, w3 = j3 * r;
    double n1 = w1 * fma(w1, w1 - 3.0 * c1, c1 + c1 * c1);
    double n2 = w2 * fma(w2, w2 - 3.0 * c2, c2 + c2 * c2);
    double n3 = w3 * fma(w3, w3 - 3.0 * c3, c3 + c3 * c3);
    double e1 = fma(w1, 1.0 - 2.0 * c1, c1 * c1);
    double e2 = fma(w2, 1.0 - 2.0 * c2, c2 * c2);
    double e3 = fma(w3, 1.0 - 2.0 * c3, c3 * c3);
    a1 = n1 * (e2 * e3);
    a2 = n2 * (e1 * e3);
    a3 = n3 * (e1 * e2);
  } else {
    // Borges / YC (tau4 = 4 tau); Jiang-Shu would be T = 0
    const double T = tau4 * tau4;
    a1 = c1 * ((q1 + T) * (q2 * q3));
    a2 = c2 * ((q2 + T) * (q1 * q3));
    a3 = c3 * ((q3 + T) * (q1 * q2));
  }
  out = fma(a1, p1, fma(a2, p2, a3 * p3)) * nr_rcp(a1 + a2 + a3);
}

// The second half of weno5_pair_alt: from the six smoothness terms B, the second
// differences d1..d4 centred at window cells 1..4 (Yamaleev-Carpenter's tau), and the
// values v.
__device__ __forceinline__ void weno5_pair_alt_finish(const double* v, int wtype, double BL1, double BL2,
                                                      double BL3, double BR1, double BR2, double BR3, double d1,
                                                      double d2, double d3, double d4, double& outL,
                                                      double& outR) {
  const double s6 = 1.0 / 6.0;
  double tL = 0.0, tR = 0.0;
  if (wtype == WENO_W_BORGES) {
    tL = fabs(BL1 - BL3);
    tR = fabs(BR1 - BR3);
  } else if (wtype == WENO_W_YC) {
    // fourth differences of the left stencil (w0..w4) and of the right one (w5..w1)
    double eL = d1 - 2.0 * d2 + d3, eR = d4 - 2.0 * d3 + d2;
    tL = 4.0 * (eL * eL);
    tR = 4.0 * (eR * eR);
  }
  double cL1 = fma(2.0, v[0], fma(-7.0, v[1], 11.0 * v[2])) * s6;
  double cR1 = fma(2.0, v[5], fma(-7.0, v[4], 11.0 * v[3])) * s6;
  double cA = fma(5.0, v[2], fma(2.0, v[3], -v[1])) * s6;
  double cB = fma(5.0, v[3], fma(2.0, v[2], -v[4])) * s6;
  weno5_side_alt(wtype, BL1, BL2, BL3, tL, cL1, cA, cB, outL);
  weno5_side_alt(wtype, BR1, BR2, BR3, tR, cR1, cB, cA, outR);
}

// The per-cell table of the alternative formulations: B (not squared) for the three
// places of the sub-stencil (a, b, c), as weno5_cell_q, and its second difference d.
__device__ __forceinline__ void weno5_cell_b(double a, double b, double c, double eps4, double& Bl, double& Bc,
                                             double& Br, double& d) {
  d = fma(-2.0, b, a) + c;
  const double kde = fma((13.0 / 3.0) * d, d, eps4);
  const double gl = fma(3.0, c, fma(-4.0, b, a));
  const double gc = a - c;
  const double gr = fma(3.0, a, fma(-4.0, b, c));
  Bl = fma(gl, gl, kde);
  Bc = fma(gc, gc, kde);
  Br = fma(gr, gr, kde);
}

__device__ __forceinline__ void weno5_pair_alt(const double* w, const double* v, double eps4, int wtype,
                                               double& outL, double& outR) {
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
  double BL1 = fma(k13 * d1, d1, fma(gL1, gL1, eps4));
  double BL2 = fma(k13 * d2, d2, fma(gL2, gL2, eps4));
  double BL3 = fma(k13 * d3, d3, fma(gL3, gL3, eps4));
  double BR1 = fma(k13 * d4, d4, fma(gR1, gR1, eps4));
  double BR2 = fma(k13 * d3, d3, fma(gR2, gR2, eps4));
  double BR3 = fma(k13 * d2, d2, fma(gR3, gR3, eps4));
  weno5_pair_alt_finish(v, wtype, BL1, BL2, BL3, BR1, BR2, BR3, d1, d2, d3, d4, outL, outR);
}

// One side of weno5_pair / weno5_pair_alt: the left-biased value on the five-point
// stencil m0..m4 (the right-biased value of a window w0..w5 is this of the mirrored
// stencil w5..w1), with Jiang-Shu weights or, when ALT, the formulation `wtype`.
template <bool ALT>
__device__ __forceinline__ double weno5_one_side(const double* m, double eps4, int wtype) {
  const double k13 = 13.0 / 3.0;
  const double d1 = fma(-2.0, m[1], m[0]) + m[2];
  const double d2 = fma(-2.0, m[2], m[1]) + m[3];
  const double d3 = fma(-2.0, m[3], m[2]) + m[4];
  const double g1 = fma(3.0, m[2], fma(-4.0, m[1], m[0]));
  const double g2 = m[1] - m[3];
  const double g3 = fma(3.0, m[2], fma(-4.0, m[3], m[4]));
  const double B1 = fma(k13 * d1, d1, fma(g1, g1, eps4));
  const double B2 = fma(k13 * d2, d2, fma(g2, g2, eps4));
  const double B3 = fma(k13 * d3, d3, fma(g3, g3, eps4));
  const double c1 = fma(2.0, m[0], fma(-7.0, m[1], 11.0 * m[2]));
  const double cA = fma(5.0, m[2], fma(2.0, m[3], -m[1]));
  const double cB = fma(5.0, m[3], fma(2.0, m[2], -m[4]));
  if (ALT) {
    double t = 0.0;
    if (wtype == WENO_W_BORGES) {
      t = fabs(B1 - B3);
    } else if (wtype == WENO_W_YC) {
      const double e = d1 - 2.0 * d2 + d3;
      t = 4.0 * (e * e);
    }
    const double s6 = 1.0 / 6.0;
    double out;
    weno5_side_alt(wtype, B1, B2, B3, t, c1 * s6, cA * s6, cB * s6, out);
    return out;
  }
  const double q1 = B1 * B1, q2 = B2 * B2, q3 = B3 * B3;
  const double a1 = q2 * q3, a2 = q1 * q3, a3 = q1 * q2;
  const double n = fma(a1, c1, fma(6.0 * a2, cA, (3.0 * a3) * cB));
  const double D = fma(36.0, a2, fma(18.0, a3, 6.0 * a1));
  return n * nr_rcp(D);
}

// Normalised WENO5 weights of the left- and right-biased stencils of a six-point
// window (Jiang-Shu, or the formulation `wtype` when ALT), for reconstructing other
// values with the weights of this stencil (InterpolateInterfacesHyp with stored weights).
template <bool ALT>
__device__ __forceinline__ void weno5_weights(const double* w, double eps4, int wtype, double* omL, double* omR) {
  const double k13 = 13.0 / 3.0, c[3] = {0.1, 0.6, 0.3};
  double d1 = fma(-2.0, w[1], w[0]) + w[2];
  double d2 = fma(-2.0, w[2], w[1]) + w[3];
  double d3 = fma(-2.0, w[3], w[2]) + w[4];
  double d4 = fma(-2.0, w[4], w[3]) + w[5];
  double gL1 = fma(3.0, w[2], fma(-4.0, w[1], w[0])), gL2 = w[1] - w[3], gL3 = fma(3.0, w[2], fma(-4.0, w[3], w[4]));
  double gR1 = fma(3.0, w[3], fma(-4.0, w[4], w[5])), gR2 = w[4] - w[2], gR3 = fma(3.0, w[3], fma(-4.0, w[2], w[1]));
  double BL[3] = {fma(k13 * d1, d1, fma(gL1, gL1, eps4)), fma(k13 * d2, d2, fma(gL2, gL2, eps4)),
                  fma(k13 * d3, d3, fma(gL3, gL3, eps4))};
  double BR[3] = {fma(k13 * d4, d4, fma(gR1, gR1, eps4)), fma(k13 * d3, d3, fma(gR2, gR2, eps4)),
                  fma(k13 * d2, d2, fma(gR3, gR3, eps4))};
  double T[2] = {0.0, 0.0};
  if (ALT && wtype == WENO_W_BORGES) {
    T[0] = (BL[0] - BL[2]) * (BL[0] - BL[2]);
    T[1] = (BR[0] - BR[2]) * (BR[0] - BR[2]);
  } else if (ALT && wtype == WENO_W_YC) {
    double eL = d1 - 2.0 * d2 + d3, eR = d4 - 2.0 * d3 + d2;
    T[0] = 16.0 * (eL * eL) * (eL * eL);
    T[1] = 16.0 * (eR * eR) * (eR * eR);
  }
  for (int side = 0; side < 2; side++) {
    const double* B = side ? BR : BL;
    double* om = side ? omR : omL;
    if (ALT && wtype == WENO_W_NONE) {
      for (int k = 0; k < 3; k++) om[k] = c[k];
      continue;
    }
    double q[3] = {B[0] * B[0], B[1] * B[1], B[2] * B[2]};
    // a_k = c_k prod_{j != k} q_j (Jiang-Shu, and mapped's first stage);
    // Borges / YC: c_k (q_k + T) prod_{j != k} q_j, as in weno5_side_alt
    const bool z = ALT && (wtype == WENO_W_BORGES || wtype == WENO_W_YC);
    double a[3] = {c[0] * ((z ? q[0] + T[side] : 1.0) * (q[1] * q[2])),
                   c[1] * ((z ? q[1] + T[side] : 1.0) * (q[0] * q[2])),
                   c[2] * ((z ? q[2] + T[side] : 1.0) * (q[0] * q[1]))};
    double r = nr_rcp(a[0] + a[1] + a[2]);
    for (int k = 0; k < 3; k++) om[k] = a[k] * r;
    if (ALT && wtype == WENO_W_MAPPED) {
      double n[3], e[3];
      for (int k = 0; k < 3; k++) {
        n[k] = om[k] * fma(om[k], om[k] - 3.0 * c[k], c[k] + c[k] * c[k]);
        e[k] = fma(om[k], 1.0 - 2.0 * c[k], c[k] * c[k]);
      }
      double m[3] = {n[0] * (e[1] * e[2]), n[1] * (e[0] * e[2]), n[2] * (e[0] * e[1])};
      double rm = nr_rcp(m[0] + m[1] + m[2]);
      for (int k = 0; k < 3; k++) om[k] = m[k] * rm;
    }
  }
}

// Reconstruction of the values v with given weights (left-biased at omL, right at omR).
__device__ __forceinline__ void weno5_apply(const double* omL, const double* omR, const double* v, double& outL,
                                            double& outR) {
  const double s6 = 1.0 / 6.0;
  double cL1 = fma(2.0, v[0], fma(-7.0, v[1], 11.0 * v[2])) * s6;
  double cR1 = fma(2.0, v[5], fma(-7.0, v[4], 11.0 * v[3])) * s6;
  double cA = fma(5.0, v[2], fma(2.0, v[3], -v[1])) * s6;
  double cB = fma(5.0, v[3], fma(2.0, v[2], -v[4])) * s6;
  outL = fma(omL[0], cL1, fma(omL[1], cA, omL[2] * cB));
  outR = fma(omR[0], cR1, fma(omR[1], cB, omR[2] * cA));
}

__device__ __forceinline__ double dabs(double x) { return fabs(x); }

}  // namespace gbh
