// gbh_visc.cu -- NavierStokes3D viscous term and the boundary / pointwise kernels.
//
// The viscous term follows NavierStokes3DParabolicFunction
// (src/PhysicalModels/NavierStokes3D/NavierStokes3DParabolicFunction.c:50-325)
// with the fourth-order central first derivative of
// FirstDerivativeFourthOrderCentral (src/FirstDerivative/FirstDerivativeFourthOrder.c:36-129),
// including its single-rank behaviour: a derivative along d is formed only on
// lines whose other indices are interior, so at a ghost point the derivatives
// across the ghost direction are zero.  Three passes:
//   visc_q      : Q = (rho, u, v, w, T = gamma P / rho) and mu = T^0.76 at every point
//   visc_grad   : dQ/dx_d * dxinv_d for the velocity and temperature, with the rule above
//   visc_dir<d> : viscous flux along d on each line (window of five points) and
//                 par += dxinv_d * d/dx_d (flux) at interior points.
#include "gbh_internal.h"

namespace gbh {

__device__ __forceinline__ int fold1(int i, int N, int lo, int hi) {
  if (i < 0) return lo == FOLD_PERIODIC ? i + N : (lo == FOLD_MIRROR ? -1 - i : i);
  if (i >= N) return hi == FOLD_PERIODIC ? i - N : (hi == FOLD_MIRROR ? 2 * N - 1 - i : i);
  return i;
}


// Q (5) and mu at all points including ghosts; ghost points read through the fold.
__global__ void visc_q_kernel(const double* __restrict__ u, double* __restrict__ Q, DevGeom G, ViscParams vp) {
  long long n = (long long)(G.dim[0] + 2 * G.g) * (G.dim[1] + 2 * G.g) * (G.dim[2] + 2 * G.g);
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int ng0 = G.dim[0] + 2 * G.g, ng1 = G.dim[1] + 2 * G.g;
  int i = (int)(p % ng0) - G.g;
  int j = (int)((p / ng0) % ng1) - G.g;
  int k = (int)(p / ((long long)ng0 * ng1)) - G.g;
  int si = fold1(i, G.dim[0], G.bclo[0], G.bchi[0]);
  int sj = fold1(j, G.dim[1], G.bclo[1], G.bchi[1]);
  int sk = fold1(k, G.dim[2], G.bclo[2], G.bchi[2]);
  long long q = (long long)(si + G.g) * G.stride[0] + (long long)(sj + G.g) * G.stride[1] +
                (long long)(sk + G.g) * G.stride[2];
  const double* uu = u + q * 5;
  double rho = uu[0];
  double ri = nr_rcp(rho);
  double vx = rho == 0.0 ? 0.0 : uu[1] * ri;
  double vy = rho == 0.0 ? 0.0 : uu[2] * ri;
  double vz = rho == 0.0 ? 0.0 : uu[3] * ri;
  double vsq = vx * vx + vy * vy + vz * vz;
  double P = (uu[4] - 0.5 * rho * vsq) * vp.gm1;
  double T = vp.gamma * P * ri;
  double* out = Q + p * 6;
  out[0] = rho;
  out[1] = vx;
  out[2] = vy;
  out[3] = vz;
  out[4] = T;
  out[5] = exp(0.76 * log(T));  // raiseto(T, 0.76), include/math_ops.h:37
}

// Fourth-order first derivative of one Q component at position i of a line of
// length N with g ghost points on each side, f(k) = value at position i+k.
template <class F>
__device__ __forceinline__ double d4(int i, int N, int g, F f) {
  const double one_twelve = 1.0 / 12.0;
  if (i == -g) return (-25.0 * f(0) + 48.0 * f(1) - 36.0 * f(2) + 16.0 * f(3) - 3.0 * f(4)) * one_twelve;
  if (i == -g + 1) return (-3.0 * f(-1) - 10.0 * f(0) + 18.0 * f(1) - 6.0 * f(2) + f(3)) * one_twelve;
  if (i < N + g - 2) return (f(-2) - 8.0 * f(-1) + 8.0 * f(1) - f(2)) * one_twelve;
  if (i == N + g - 2) return (-f(-3) + 6.0 * f(-2) - 18.0 * f(-1) + 10.0 * f(0) + 3.0 * f(1)) * one_twelve;
  return (3.0 * f(-4) - 16.0 * f(-3) + 36.0 * f(-2) - 48.0 * f(-1) + 25.0 * f(0)) * one_twelve;
}

// First-order one-sided first derivative (FirstDerivativeFirstOrder.c:50-84): bias 1
// forward, -1 backward in the interior of the ghost-extended line, forward at its first
// point and backward at its last, in the reference's expression
// max(bias,0) f(1) - bias f(0) + min(bias,0) f(-1).
template <class F>
__device__ __forceinline__ double d1(int i, int N, int g, int bias, F f) {
  if (i == -g) return f(1) - f(0);
  if (i == N + g - 1) return f(0) - f(-1);
  return (bias > 0) ? __dadd_rn(__dsub_rn(f(1), f(0)), __dmul_rn(0.0, f(-1)))
                    : __dsub_rn(__dadd_rn(__dmul_rn(0.0, f(1)), f(0)), f(-1));
}

// Scaled gradients of (u, v, w, T): Gr[p*12 + d*4 + c].
__global__ void visc_grad_kernel(const double* __restrict__ Q, double* __restrict__ Gr, const double* __restrict__ dxinv,
                                 DevGeom G, int order) {
  int ng[3] = {G.dim[0] + 2 * G.g, G.dim[1] + 2 * G.g, G.dim[2] + 2 * G.g};
  long long n = (long long)ng[0] * ng[1] * ng[2];
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int idx[3];
  idx[0] = (int)(p % ng[0]) - G.g;
  idx[1] = (int)((p / ng[0]) % ng[1]) - G.g;
  idx[2] = (int)(p / ((long long)ng[0] * ng[1])) - G.g;
  int off = 0;
  for (int d = 0; d < 3; d++) {
    bool line = true;
    for (int e = 0; e < 3; e++)
      if (e != d && (idx[e] < 0 || idx[e] >= G.dim[e])) line = false;
    double* out = Gr + p * 12 + d * 4;
    if (!line) {
      out[0] = out[1] = out[2] = out[3] = 0.0;
    } else {
      long long sd = G.stride[d];
      double di = dxinv[off + G.g + idx[d]];
      for (int c = 0; c < 4; c++) {
        const double* base = Q + p * 6 + 1 + c;
        auto fk = [&](int k) { return base[(long long)k * sd * 6]; };
        double v = order == 2 ? d1(idx[d], G.dim[d], G.g, 1, fk) : d4(idx[d], G.dim[d], G.g, fk);
        out[c] = v * di;
      }
    }
    off += ng[d];
  }
}

// Viscous flux along DIR at one point (NavierStokes3DParabolicFunction.c:151-314).
template <int DIR>
__device__ __forceinline__ void visc_flux(const double* Qp, const double* Gp, const ViscParams& vp, double* F) {
  const double two_third = 2.0 / 3.0;
  double uvel = Qp[1], vvel = Qp[2], wvel = Qp[3], mu = Qp[5];
  double mr = mu * vp.inv_Re;
  double kq = mr * vp.inv_gm1 * vp.inv_Pr;
  const double* X = Gp;      // d/dx of (u, v, w, T)
  const double* Y = Gp + 4;  // d/dy
  const double* Z = Gp + 8;  // d/dz
  double t1, t2, t3, q;
  if (DIR == 0) {
    t1 = two_third * mr * (2.0 * X[0] - Y[1] - Z[2]);
    t2 = mr * (Y[0] + X[1]);
    t3 = mr * (Z[0] + X[2]);
    q = kq * X[3];
  } else if (DIR == 1) {
    t1 = mr * (Y[0] + X[1]);
    t2 = two_third * mr * (-X[0] + 2.0 * Y[1] - Z[2]);
    t3 = mr * (Z[1] + Y[2]);
    q = kq * Y[3];
  } else {
    t1 = mr * (Z[0] + X[2]);
    t2 = mr * (Z[1] + Y[2]);
    t3 = two_third * mr * (-X[0] - Y[1] + 2.0 * Z[2]);
    q = kq * Z[3];
  }
  F[0] = t1;
  F[1] = t2;
  F[2] = t3;
  F[3] = uvel * t1 + vvel * t2 + wvel * t3 + q;
}

// One thread per (interior line along DIR, segment of `seg` interior points).
template <int DIR>
__global__ void visc_dir_kernel(const double* __restrict__ Q, const double* __restrict__ Gr,
                                const double* __restrict__ dxinv_dir, double* __restrict__ par, DevGeom G,
                                ViscParams vp, int seg, int nseg, int first) {
  long long ntrans = 1;
  for (int e = 0; e < 3; e++)
    if (e != DIR) ntrans *= G.dim[e];
  long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= ntrans * nseg) return;
  long long tr = tid % ntrans;
  int sg = (int)(tid / ntrans);
  long long pb = (long long)G.g * G.stride[DIR];
  for (int e = 0; e < 3; e++) {
    if (e == DIR) continue;
    int ie = (int)(tr % G.dim[e]);
    tr /= G.dim[e];
    pb += (long long)(ie + G.g) * G.stride[e];
  }
  const long long sd = G.stride[DIR];
  const int N = G.dim[DIR];
  const int c0 = sg * seg, c1 = min(c0 + seg, N);
  const double one_twelve = 1.0 / 12.0;
  double W[5][4];
  auto flux_at = [&](int i, double* F) {
    long long p = pb + (long long)i * sd;
    visc_flux<DIR>(Q + p * 6, Gr + p * 12, vp, F);
  };
#pragma unroll
  for (int k = 0; k < 4; k++) flux_at(c0 - 2 + k, W[k + 1]);
  for (int c = c0; c < c1; c++) {
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int v = 0; v < 4; v++) W[k][v] = W[k + 1][v];
    flux_at(c + 2, W[4]);
    long long p = pb + (long long)c * sd;
    double di = dxinv_dir[G.g + c];
    double* out = par + p * 5;
    if (first) out[0] = 0.0;
#pragma unroll
    for (int v = 0; v < 4; v++) {
      // interior points: the central fourth-order difference, or the backward
      // first-order one of the second-order scheme
      double fd = vp.order == 2 ? __dsub_rn(__dadd_rn(__dmul_rn(0.0, W[3][v]), W[2][v]), W[1][v])
                                : (W[0][v] - 8.0 * W[1][v] + 8.0 * W[3][v] - W[4][v]) * one_twelve;
      double val = di * fd;
      out[1 + v] = first ? val : out[1 + v] + val;
    }
  }
}

cudaError_t launch_visc(const double* u, double* Q, double* Gr, double* par, const double* dxinv, const DevGeom& G,
                        const ViscParams& vp, int seg, cudaStream_t s) {
  long long n = (long long)(G.dim[0] + 2 * G.g) * (G.dim[1] + 2 * G.g) * (G.dim[2] + 2 * G.g);
  int blk = 256;
  visc_q_kernel<<<(unsigned)((n + blk - 1) / blk), blk, 0, s>>>(u, Q, G, vp);
  visc_grad_kernel<<<(unsigned)((n + blk - 1) / blk), blk, 0, s>>>(Q, Gr, dxinv, G, vp.order);
  int off = 0;
  for (int d = 0; d < 3; d++) {
    long long ntrans = 1;
    for (int e = 0; e < 3; e++)
      if (e != d) ntrans *= G.dim[e];
    int nseg = (G.dim[d] + seg - 1) / seg;
    long long nthr = ntrans * nseg;
    unsigned grid = (unsigned)((nthr + 127) / 128);
    const double* dxd = dxinv + off;
    if (d == 0) visc_dir_kernel<0><<<grid, 128, 0, s>>>(Q, Gr, dxd, par, G, vp, seg, nseg, 1);
    if (d == 1) visc_dir_kernel<1><<<grid, 128, 0, s>>>(Q, Gr, dxd, par, G, vp, seg, nseg, 0);
    if (d == 2) visc_dir_kernel<2><<<grid, 128, 0, s>>>(Q, Gr, dxd, par, G, vp, seg, nseg, 0);
    off += G.dim[d] + 2 * G.g;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Boundary zones applied to the array in memory (ApplyBoundaryConditions ->
// BCPeriodicU / BCExtrapolateU, src/BoundaryConditions/BCPeriodic.c:36-56,
// BCExtrapolate.c:29-46) for faces whose zone does not cover the whole face.
// ---------------------------------------------------------------------------
struct ZoneDev {
  int type, dim, face, is[3], ie[3];
  double data[8];
  double gamma;
  // thermal walls: the wall temperature field (all time levels) and the level in use;
  // turbulent inflow: the inflow data (all slices), their number and the slice in use
  const double* tfield;
  int tn, it;
};

// Ghost state from the mirror interior state w, for the wall and inflow /
// outflow types (BCSlipWall.c, BCNoslipWall.c, BCSubsonicInflow.c,
// BCSubsonicOutflow.c, BCSupersonicInflow.c, BCSupersonicOutflow.c; 2-D and 3-D
// branches), in their operation order without contraction.
template <int ND>
__device__ __forceinline__ void bc_ghost(const ZoneDev& z, const double* w, double* out, bool inflow = false,
                                         double Tb = 0.0, const double* fluct = nullptr) {
  constexpr int NV = ND + 2;
  const double gm1 = z.gamma - 1.0;
  const double inv_gm1 = __ddiv_rn(1.0, gm1);
  double rho = 0.0, vel[3] = {0.0, 0.0, 0.0}, P = 0.0;
  if (z.type != GB_BC_SUPERSONIC_INFLOW && z.type != GB_BC_TURBULENT_INFLOW) {
    rho = w[0];
    for (int d = 0; d < ND; d++) vel[d] = (ND == 3 && rho == 0.0) ? 0.0 : __ddiv_rn(w[1 + d], rho);
    double vsq = __dadd_rn(__dmul_rn(vel[0], vel[0]), __dmul_rn(vel[1], vel[1]));
    if (ND == 3) vsq = __dadd_rn(vsq, __dmul_rn(vel[2], vel[2]));
    P = __dmul_rn(__dsub_rn(w[NV - 1], __dmul_rn(__dmul_rn(0.5, rho), vsq)), gm1);
  }
  double rg = rho, vg[3] = {vel[0], vel[1], vel[2]}, Pg = P;
  switch (z.type) {
    case GB_BC_SLIP_WALL: vg[z.dim] = __dsub_rn(__dmul_rn(2.0, z.data[z.dim]), vel[z.dim]); break;
    case GB_BC_NOSLIP_WALL:
      for (int d = 0; d < ND; d++) vg[d] = __dsub_rn(__dmul_rn(2.0, z.data[d]), vel[d]);
      break;
    case GB_BC_SUBSONIC_INFLOW:
      rg = z.data[0];
      for (int d = 0; d < ND; d++) vg[d] = z.data[1 + d];
      break;
    case GB_BC_SUBSONIC_OUTFLOW: Pg = z.data[0]; break;
    case GB_BC_SUPERSONIC_INFLOW:
      rg = z.data[0];
      for (int d = 0; d < ND; d++) vg[d] = z.data[1 + d];
      Pg = z.data[1 + ND];
      break;
    case GB_BC_THERMAL_SLIP_WALL:
      // BCThermalSlipWall.c:86-105: the normal velocity mirrored about the wall's, the
      // pressure from the extrapolated density and the wall temperature
      vg[z.dim] = __dsub_rn(__dmul_rn(2.0, z.data[z.dim]), vel[z.dim]);
      Pg = __dmul_rn(rg, Tb);
      break;
    case GB_BC_THERMAL_NOSLIP_WALL:
      // BCThermalNoslipWall.c:86-105: every velocity component mirrored
      for (int d = 0; d < ND; d++) vg[d] = __dsub_rn(__dmul_rn(2.0, z.data[d]), vel[d]);
      Pg = __dmul_rn(rg, Tb);
      break;
    case GB_BC_TURBULENT_INFLOW:
      // BCTurbulentSupersonicInflow.c:54-85: the supersonic inflow state with the data's
      // velocity fluctuations added
      rg = z.data[0];
      for (int d = 0; d < ND; d++) vg[d] = __dadd_rn(z.data[1 + d], fluct[d]);
      Pg = z.data[1 + ND];
      break;
    case GB_BC_SUBSONIC_AMBIVALENT:
      // BCSubsonicAmbivalent.c:105-117: inflow's rule (density, velocity given) or
      // outflow's (pressure given) by the sign of the extrapolated face velocity
      if (inflow) {
        rg = z.data[0];
        for (int d = 0; d < ND; d++) vg[d] = z.data[1 + d];
      } else {
        Pg = z.data[1 + ND];
      }
      break;
    default: break;  // supersonic outflow: the interior state, energy recomputed
  }
  double vsq = __dadd_rn(__dmul_rn(vg[0], vg[0]), __dmul_rn(vg[1], vg[1]));
  if (ND == 3) vsq = __dadd_rn(vsq, __dmul_rn(vg[2], vg[2]));
  out[0] = rg;
  for (int d = 0; d < ND; d++) out[1 + d] = __dmul_rn(rg, vg[d]);
  out[NV - 1] = __dadd_rn(__dmul_rn(inv_gm1, Pg), __dmul_rn(__dmul_rn(0.5, rg), vsq));
}

__global__ void bc_zone_kernel(double* u, DevGeom G, int nv, ZoneDev z) {
  int b[3] = {1, 1, 1};
  for (int d = 0; d < G.nd; d++) b[d] = z.ie[d] - z.is[d];
  long long n = (long long)b[0] * b[1] * b[2];
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int ib[3] = {(int)(t % b[0]), (int)((t / b[0]) % b[1]), (int)(t / ((long long)b[0] * b[1]))};
  int ig[3] = {0, 0, 0}, is[3] = {0, 0, 0};
  for (int d = 0; d < G.nd; d++) {
    ig[d] = ib[d] + z.is[d];
    is[d] = ig[d];
  }
  int dd = z.dim, N = G.dim[dd];
  if (z.type == GB_BC_PERIODIC) is[dd] = (z.face == 1) ? ib[dd] + N - G.g : ib[dd];
  else is[dd] = (z.face == 1) ? G.g - 1 - ib[dd] : N - ib[dd] - 1;  // the mirror interior point
  long long p1 = 0, p2 = 0;
  for (int d = 0; d < G.nd; d++) {
    p1 += (long long)(ig[d] + G.g) * G.stride[d];
    p2 += (long long)(is[d] + G.g) * G.stride[d];
  }
  if (z.type == GB_BC_PERIODIC || z.type == GB_BC_EXTRAPOLATE) {
    for (int v = 0; v < nv; v++) u[p1 * nv + v] = u[p2 * nv + v];
  } else if (z.type == GB_BC_REFLECT) {
    for (int v = 0; v < nv; v++) u[p1 * nv + v] = -u[p2 * nv + v];
  } else if (z.type == GB_BC_DIRICHLET) {
    for (int v = 0; v < nv; v++) u[p1 * nv + v] = z.data[v];
  } else {
    bool inflow = false;
    if (z.type == GB_BC_SUBSONIC_AMBIVALENT) {
      // BCSubsonicAmbivalent.c:70-92: the face velocity extrapolated from the boundary
      // cell and its neighbour at this transverse position, 1.5 v_1 - 0.5 v_2, on the
      // inward normal face * e_dim (only interior points are read: no ordering with the
      // ghost writes of other threads)
      long long q1 = 0, q2 = 0;
      for (int d = 0; d < G.nd; d++) {
        const int i1 = d == dd ? (z.face == 1 ? 0 : N - 1) : ig[d];
        const int i2 = d == dd ? (z.face == 1 ? 1 : N - 2) : ig[d];
        q1 += (long long)(i1 + G.g) * G.stride[d];
        q2 += (long long)(i2 + G.g) * G.stride[d];
      }
      const double *w1 = u + q1 * nv, *w2 = u + q2 * nv;
      const double r1 = w1[0], r2 = w2[0];
      const double m1 = w1[1 + dd], m2 = w2[1 + dd];
      const double v1 = (G.nd == 3 && r1 == 0.0) ? 0.0 : __ddiv_rn(m1, r1);
      const double v2 = (G.nd == 3 && r2 == 0.0) ? 0.0 : __ddiv_rn(m2, r2);
      const double vb = __dsub_rn(__dmul_rn(1.5, v1), __dmul_rn(0.5, v2));
      inflow = (z.face == 1) ? vb > 0.0 : vb < 0.0;
    }
    double Tb = 0.0;
    if (z.type == GB_BC_THERMAL_SLIP_WALL || z.type == GB_BC_THERMAL_NOSLIP_WALL) {
      // the temperature at this point: zone-relative index, the time level along dim
      // (BCThermalNoslipWall.c:80-84)
      long long q = 0, stride = 1;
      for (int d = 0; d < G.nd; d++) {
        q += stride * (d == dd ? z.it : ib[d]);
        stride *= (d == dd ? z.tn : b[d]);
      }
      Tb = z.tfield[q];
    }
    const double* fl = nullptr;
    if (z.type == GB_BC_TURBULENT_INFLOW) {
      // the slice in use along dim, the zone-relative indices across it (the data spans
      // the grid across, BCTurbulentSupersonicInflow.c:66-72)
      long long q = 0, stride = 1;
      for (int d = 0; d < G.nd; d++) {
        q += stride * (d == dd ? z.it : ib[d]);
        stride *= (d == dd ? z.tn : G.dim[d]);
      }
      fl = z.tfield + q * nv + 1;
    }
    double g[5];
    if (G.nd == 1) {
      // BCSlipWall.c:38-76 (Euler1D, the one wall type with a 1-D branch): density and
      // pressure extrapolated, the velocity mirrored about the wall's, in the 1-D flow
      // variables' operation order
      const double* w = u + p2 * nv;
      const double gm1 = z.gamma - 1.0, inv_gm1 = __ddiv_rn(1.0, gm1);
      const double rho = w[0], vel = __ddiv_rn(w[1], rho);
      const double P = __dmul_rn(__dsub_rn(w[2], __dmul_rn(__dmul_rn(__dmul_rn(0.5, rho), vel), vel)), gm1);
      const double vg = __dsub_rn(__dmul_rn(2.0, z.data[0]), vel);
      g[0] = rho;
      g[1] = __dmul_rn(rho, vg);
      g[2] = __dadd_rn(__dmul_rn(inv_gm1, P), __dmul_rn(__dmul_rn(__dmul_rn(0.5, rho), vg), vg));
    } else if (G.nd == 2) {
      bc_ghost<2>(z, u + p2 * nv, g, inflow, Tb, fl);
    } else {
      bc_ghost<3>(z, u + p2 * nv, g, inflow, Tb, fl);
    }
    for (int v = 0; v < nv; v++) u[p1 * nv + v] = g[v];
  }
}

cudaError_t launch_bc_zone_t(double* u, const DevGeom& G, int nv, const int* zone9, const double* data8,
                             double gamma, const double* tfield, int tn, int it, cudaStream_t s);

cudaError_t launch_bc_zone(double* u, const DevGeom& G, int nv, const int* zone9, const double* data8, double gamma,
                           cudaStream_t s) {
  return launch_bc_zone_t(u, G, nv, zone9, data8, gamma, nullptr, 0, 0, s);
}

// As launch_bc_zone, with a thermal wall's temperature field (tn time levels, device
// array) and the level `it` in use.
cudaError_t launch_bc_zone_t(double* u, const DevGeom& G, int nv, const int* zone9, const double* data8,
                             double gamma, const double* tfield, int tn, int it, cudaStream_t s) {
  if (zone9[0] == GB_BC_SPONGE) return cudaSuccess;  // a source term, no ghost points (BCSpongeUDummy)
  ZoneDev z;
  z.tfield = tfield;
  z.tn = tn;
  z.it = it;
  if ((zone9[0] == GB_BC_THERMAL_SLIP_WALL || zone9[0] == GB_BC_THERMAL_NOSLIP_WALL ||
       zone9[0] == GB_BC_TURBULENT_INFLOW) && (!tfield || tn < 1 || it < 0 || it >= tn))
    return cudaErrorInvalidValue;  // a thermal wall or turbulent inflow without its field
  z.type = zone9[0];
  z.dim = zone9[1];
  z.face = zone9[2];
  z.gamma = gamma;
  for (int k = 0; k < 8; k++) z.data[k] = data8 ? data8[k] : 0.0;
  long long n = 1;
  for (int d = 0; d < 3; d++) {
    z.is[d] = zone9[3 + d];
    z.ie[d] = zone9[6 + d];
    if (d < G.nd) n *= (z.ie[d] - z.is[d] > 0 ? z.ie[d] - z.is[d] : 0);
  }
  if (n <= 0) return cudaSuccess;
  bc_zone_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(u, G, nv, z);
  return cudaGetLastError();
}

// The sponge zone's source (BCSponge.c:34-61): src -= sigma_i (u - u_ref) at every
// interior point of the zone's extent, sigma indexed along the zone's dimension.  The
// three roundings of the reference's expression are kept (no contraction).  Zones may
// overlap: one launch per zone, in zone order, on one stream.
__global__ void sponge_kernel(double* __restrict__ src, const double* __restrict__ u, DevGeom G, int nv,
                              ZoneDev z, const double* __restrict__ sigma) {
  int b[3] = {1, 1, 1};
  for (int d = 0; d < G.nd; d++) b[d] = z.ie[d] - z.is[d];
  const long long n = (long long)b[0] * b[1] * b[2];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int ib[3] = {(int)(t % b[0]), (int)((t / b[0]) % b[1]), (int)(t / ((long long)b[0] * b[1]))};
  long long p = 0;
  for (int d = 0; d < G.nd; d++) p += (long long)(ib[d] + z.is[d] + G.g) * G.stride[d];
  const double sg = sigma[ib[z.dim]];
  for (int v = 0; v < nv; v++)
    src[p * nv + v] = __dsub_rn(src[p * nv + v], __dmul_rn(sg, __dsub_rn(u[p * nv + v], z.data[v])));
}

cudaError_t launch_sponge(double* src, const double* u, const DevGeom& G, int nv, const int* zone9,
                          const double* uref8, const double* sigma, cudaStream_t s) {
  if (zone9[0] != GB_BC_SPONGE) return cudaErrorInvalidValue;
  ZoneDev z;
  z.tfield = nullptr;
  z.tn = z.it = 0;
  z.type = zone9[0];
  z.dim = zone9[1];
  z.face = zone9[2];
  z.gamma = 0.0;
  for (int k = 0; k < 8; k++) z.data[k] = uref8[k];
  long long n = 1;
  for (int d = 0; d < 3; d++) {
    z.is[d] = zone9[3 + d];
    z.ie[d] = zone9[6 + d];
    if (d < G.nd) n *= (z.ie[d] - z.is[d] > 0 ? z.ie[d] - z.is[d] : 0);
  }
  if (n <= 0) return cudaSuccess;
  if (!sigma) return cudaErrorInvalidValue;
  sponge_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, u, G, nv, z, sigma);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Layout copies between interior-only and ghosted arrays, and a finite check.
// ---------------------------------------------------------------------------
__global__ void pack_kernel(double* dst, const double* src, DevGeom G, int nv, int to_interior) {
  long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int i = (int)(p % G.dim[0]);
  int j = (int)((p / G.dim[0]) % G.dim[1]);
  int k = (int)(p / ((long long)G.dim[0] * G.dim[1]));
  long long q = (long long)(i + G.g) * G.stride[0];
  if (G.nd > 1) q += (long long)(j + G.g) * G.stride[1];
  if (G.nd > 2) q += (long long)(k + G.g) * G.stride[2];
  for (int v = 0; v < nv; v++) {
    if (to_interior) dst[p * nv + v] = src[q * nv + v];
    else dst[q * nv + v] = src[p * nv + v];
  }
}

cudaError_t launch_pack(double* dst, const double* src, const DevGeom& G, int nv, int to_interior, cudaStream_t s) {
  long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  pack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dst, src, G, nv, to_interior);
  return cudaGetLastError();
}

__global__ void finite_kernel(const double* u, DevGeom G, int nv, int* flag) {
  long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int i = (int)(p % G.dim[0]);
  int j = (int)((p / G.dim[0]) % G.dim[1]);
  int k = (int)(p / ((long long)G.dim[0] * G.dim[1]));
  long long q = (long long)(i + G.g) * G.stride[0];
  if (G.nd > 1) q += (long long)(j + G.g) * G.stride[1];
  if (G.nd > 2) q += (long long)(k + G.g) * G.stride[2];
  bool bad = false;
  for (int v = 0; v < nv; v++) bad |= !isfinite(u[q * nv + v]);
  if (bad) atomicOr(flag, 1);
}

cudaError_t launch_finite_check(const double* u, const DevGeom& G, int nv, int* flag, cudaStream_t s) {
  long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  finite_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(u, G, nv, flag);
  return cudaGetLastError();
}

}  // namespace gbh
