// gbh_monitor.cu -- the quantities the reference computes around a time step,
// as device reductions over the resident solution:
//   * the maximum CFL number (<Model>ComputeCFL: Euler1DComputeCFL.c:16-44,
//     Euler2DComputeCFL.c:14-39, NavierStokes3DComputeCFL.c:18-49), computed in
//     the reference's operation order without contraction, so the result is
//     the reference's to the bit;
//   * the norm of a step's change, sqrt(sum (u_new - u_old)^2 / npoints) over
//     the interior (TimePostStep.c:38-60);
//   * the relative L1 / L2 / Linf errors against an exact solution
//     (CalculateError.c:27-110).
//   * the conservation check: the volume integral sum u dV (VolumeIntegral.c) and
//     the sums over the grid lines of the boundary-flux time integrals that the
//     fused kernels accumulate per line (BoundaryIntegral.c,
//     CalculateConservationError.c).
// Sums are reduced in two passes in a fixed order (per-block partials, then
// one block), so every result is deterministic.
#include <cmath>
#include <cstring>

#include "gbh_internal.h"
#include "gbh_solver.h"

namespace gbh {
cudaError_t launch_pack(double*, const double*, const DevGeom&, int, int, cudaStream_t);

constexpr int RED_BLOCK = 256;
constexpr int RED_MAX_BLOCKS = 1024;

// Interior point p (dimension 0 fastest) -> point index with ghosts.
__device__ __forceinline__ long long interior_point(const DevGeom& G, long long p, int idx[3]) {
  idx[0] = (int)(p % G.dim[0]);
  long long r = p / G.dim[0];
  idx[1] = (int)(r % G.dim[1]);
  idx[2] = (int)(r / G.dim[1]);
  long long q = 0;
  for (int d = 0; d < G.nd; d++) q += (long long)(idx[d] + G.g) * G.stride[d];
  return q;
}

// Block reduction of (sum, sum, max) triples into partials[blockIdx.x].
__device__ void block_reduce3(double a, double b, double c, double* out) {
  __shared__ double sa[RED_BLOCK], sb[RED_BLOCK], sc[RED_BLOCK];
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int w = RED_BLOCK / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sa[threadIdx.x] += sa[threadIdx.x + w];
      sb[threadIdx.x] += sb[threadIdx.x + w];
      sc[threadIdx.x] = fmax(sc[threadIdx.x], sc[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[3 * blockIdx.x + 0] = sa[0];
    out[3 * blockIdx.x + 1] = sb[0];
    out[3 * blockIdx.x + 2] = sc[0];
  }
}

// Over the interior: sum |x|, sum x^2, max |x| with x = a - b (b may be null).
// Each thread strides through the points in a fixed order.
__global__ void __launch_bounds__(RED_BLOCK) norms_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                          DevGeom G, int nv, double* partials) {
  const long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  double s1 = 0.0, s2 = 0.0, mx = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    int idx[3];
    const long long q = interior_point(G, p, idx) * nv;
    for (int v = 0; v < nv; v++) {
      double x = b ? a[q + v] - b[q + v] : a[q + v];
      double ax = fabs(x);
      s1 += ax;
      s2 = fma(x, x, s2);
      mx = fmax(mx, ax);
    }
  }
  block_reduce3(s1, s2, mx, partials);
}

// Maximum local CFL of the model, (|v_d| + c) dt dxinv_d, in the reference's
// order: v_d = u_{1+d}/rho, P = (e - 0.5 rho |v|^2)(gamma-1), c = sqrt(gamma P / rho).
template <int ND>
__global__ void __launch_bounds__(RED_BLOCK) cfl_kernel(const double* __restrict__ u, const double* __restrict__ dxinv,
                                                        DevGeom G, double gamma, double dt, long long dxo1,
                                                        long long dxo2, double* partials) {
  const long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  constexpr int NV = ND + 2;
  double mx = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    int idx[3];
    const long long q = interior_point(G, p, idx) * NV;
    const double rho = u[q];
    double vel[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < ND; d++) vel[d] = __ddiv_rn(u[q + 1 + d], rho);
    const double e = u[q + NV - 1];
    double vsq = __dmul_rn(vel[0], vel[0]);
    if (ND > 1) vsq = __dadd_rn(vsq, __dmul_rn(vel[1], vel[1]));
    if (ND > 2) vsq = __dadd_rn(vsq, __dmul_rn(vel[2], vel[2]));
    const double P = __dmul_rn(__dsub_rn(e, __dmul_rn(__dmul_rn(0.5, rho), vsq)), gamma - 1.0);
    const double c = __dsqrt_rn(__ddiv_rn(__dmul_rn(gamma, P), rho));
    const long long off[3] = {0, dxo1, dxo2};
    for (int d = 0; d < ND; d++) {
      const double dxi = dxinv[off[d] + idx[d] + G.g];
      const double l = __dmul_rn(__dmul_rn(__dadd_rn(fabs(vel[d]), c), dt), dxi);
      if (l > mx) mx = l;
    }
  }
  block_reduce3(0.0, 0.0, mx, partials);
}

// Second pass: one block folds the partials in index order.
__global__ void __launch_bounds__(RED_BLOCK) finish_kernel(double* partials, int nblocks) {
  double a = 0.0, b = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += RED_BLOCK) {
    a += partials[3 * i + 0];
    b += partials[3 * i + 1];
    c = fmax(c, partials[3 * i + 2]);
  }
  __syncthreads();  // every thread has read its partials before block 0's slot is overwritten
  block_reduce3(a, b, c, partials);
}

// Block sums of NV values per thread into out[NV * blockIdx.x + v].
template <int NV>
__device__ void block_reduce_n(const double* x, double* out) {
  __shared__ double sm[NV][RED_BLOCK];
#pragma unroll
  for (int v = 0; v < NV; v++) sm[v][threadIdx.x] = x[v];
  __syncthreads();
  for (int w = RED_BLOCK / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int v = 0; v < NV; v++) sm[v][threadIdx.x] += sm[v][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int v = 0; v < NV; v++) out[NV * blockIdx.x + v] = sm[v][0];
}

// Volume integral partials: sum over the interior of u dV, dV = prod_d 1/dxinv_d
// (VolumeIntegral.c: dV *= 1/dxinv per dimension, then u dV).
template <int NV>
__global__ void __launch_bounds__(RED_BLOCK) volume_kernel(const double* __restrict__ u,
                                                           const double* __restrict__ dxinv, DevGeom G,
                                                           long long dxo1, long long dxo2, double* partials) {
  const long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  const long long off[3] = {0, dxo1, dxo2};
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) acc[v] = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    int idx[3];
    const long long q = interior_point(G, p, idx) * NV;
    double dV = 1.0;
    for (int d = 0; d < G.nd; d++) dV = __dmul_rn(dV, __ddiv_rn(1.0, dxinv[off[d] + idx[d] + G.g]));
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] += __dmul_rn(u[q + v], dV);
  }
  block_reduce_n<NV>(acc, partials);
}

// Second pass of volume_kernel: one block folds the partials in index order.
template <int NV>
__global__ void __launch_bounds__(RED_BLOCK) volume_finish_kernel(double* partials, int nblocks) {
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) acc[v] = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += RED_BLOCK)
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] += partials[NV * i + v];
  __syncthreads();  // all partials read before block 0's slot is overwritten
  block_reduce_n<NV>(acc, partials);
}

// Boundary-flux integrals: block b = 2 d + face sums its face's lines
// (bnd + off[d] + face * nlines[d] * NV) into out[NV * b + v].
template <int NV>
__global__ void __launch_bounds__(RED_BLOCK) boundary_sum_kernel(const double* __restrict__ bnd, long long off0,
                                                                 long long off1, long long off2, long long n0,
                                                                 long long n1, long long n2, double* out) {
  const int d = blockIdx.x / 2, face = blockIdx.x % 2;
  const long long nl = d == 0 ? n0 : (d == 1 ? n1 : n2);
  const double* b = bnd + (d == 0 ? off0 : (d == 1 ? off1 : off2)) + (long long)face * nl * NV;
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) acc[v] = 0.0;
  for (long long l = threadIdx.x; l < nl; l += RED_BLOCK)
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] += b[l * NV + v];
  block_reduce_n<NV>(acc, out);
}

}  // namespace gbh

using namespace gbh;

#define MK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      gbh_set_error("%s:%d: %s", __FILE__, __LINE__, cudaGetErrorString(e_));                      \
      return e_ == cudaErrorMemoryAllocation ? GB_ERR_NOMEM : GB_ERR_CUDA;                         \
    }                                                                                              \
  } while (0)

static int red_buffer(gb_solver* s) {
  if (!s->d_red) MK(cudaMalloc((void**)&s->d_red, sizeof(double) * 3 * RED_MAX_BLOCKS));
  return GB_OK;
}

static int red_blocks(const gb_solver* s) {
  long long n = (long long)s->G.dim[0] * s->G.dim[1] * s->G.dim[2];
  long long b = (n + RED_BLOCK - 1) / RED_BLOCK;
  return (int)(b < RED_MAX_BLOCKS ? (b < 1 ? 1 : b) : RED_MAX_BLOCKS);
}

// Reads the three folded results back (synchronises the solver's stream).
static int red_read(gb_solver* s, int nb, double out[3]) {
  finish_kernel<<<1, RED_BLOCK, 0, s->stream>>>(s->d_red, nb);
  MK(cudaGetLastError());
  MK(cudaMemcpyAsync(out, s->d_red, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  MK(cudaStreamSynchronize(s->stream));
  return GB_OK;
}

static int cfl_launch(gb_solver* s, const double* u, double* cfl) {
  int rc = red_buffer(s);
  if (rc) return rc;
  const int nb = red_blocks(s);
  const gb_config& c = s->cfg;
  if (c.ndims == 1)
    cfl_kernel<1><<<nb, RED_BLOCK, 0, s->stream>>>(u, s->d_dxinv, s->G, c.gamma, c.dt, s->dx_off[1], s->dx_off[2],
                                                   s->d_red);
  else if (c.ndims == 2)
    cfl_kernel<2><<<nb, RED_BLOCK, 0, s->stream>>>(u, s->d_dxinv, s->G, c.gamma, c.dt, s->dx_off[1], s->dx_off[2],
                                                   s->d_red);
  else
    cfl_kernel<3><<<nb, RED_BLOCK, 0, s->stream>>>(u, s->d_dxinv, s->G, c.gamma, c.dt, s->dx_off[1], s->dx_off[2],
                                                   s->d_red);
  MK(cudaGetLastError());
  double r[3];
  rc = red_read(s, nb, r);
  if (rc) return rc;
  *cfl = r[2];
  return GB_OK;
}

static int norms_launch(gb_solver* s, const double* a, const double* b, double out[3]) {
  int rc = red_buffer(s);
  if (rc) return rc;
  const int nb = red_blocks(s);
  norms_kernel<<<nb, RED_BLOCK, 0, s->stream>>>(a, b, s->G, s->cfg.nvars, s->d_red);
  MK(cudaGetLastError());
  return red_read(s, nb, out);
}

static double npoints(const gb_solver* s) {
  double n = 1.0;
  for (int d = 0; d < s->cfg.ndims; d++) n *= (double)s->cfg.dim[d];
  return n;
}

extern "C" int gb_solver_cfl(gb_solver* s, double* cfl) {
  if (!s || !cfl) { gbh_set_error("gb_solver_cfl: null argument"); return GB_ERR_ARG; }
  return cfl_launch(s, s->d_u, cfl);
}

extern "C" int gb_solver_step_report(gb_solver* s, int nsteps, double* cfl, double* norm) {
  if (!s || nsteps < 1) { gbh_set_error("gb_solver_step_report: bad argument"); return GB_ERR_ARG; }
  for (int n = 0; n < nsteps - 1; n++) {
    int rc = gbh_rk_step(s);
    if (rc) return rc;
  }
  int rc = GB_OK;
  if (cfl) {
    rc = cfl_launch(s, s->d_u, cfl);  // TimePreStep: the state the last step starts from
    if (rc) return rc;
  }
  if (norm) {
    if (!s->d_snap) MK(cudaMalloc((void**)&s->d_snap, s->nvals * sizeof(double)));
    MK(cudaMemcpyAsync(s->d_snap, s->d_u, s->nvals * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
  }
  rc = gbh_rk_step(s);
  if (rc) return rc;
  MK(cudaGetLastError());
  if (norm) {
    double r[3];
    rc = norms_launch(s, s->d_u, s->d_snap, r);
    if (rc) return rc;
    *norm = std::sqrt(r[1] / npoints(s));
  }
  return GB_OK;
}

namespace gbh {
// CalculateError.c:27-110 on one grid: relative L1 / L2 / Linf of u - uex (both
// ghosted device arrays; relative when the exact solution's norms exceed 1e-15).
int grid_error(const double* u, const double* uex, const DevGeom& G, int nv, double* red, cudaStream_t st,
               double* err) {
  long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  long long b = (n + RED_BLOCK - 1) / RED_BLOCK;
  const int nb = (int)(b < RED_MAX_BLOCKS ? (b < 1 ? 1 : b) : RED_MAX_BLOCKS);
  double ex[3], df[3];
  for (int pass = 0; pass < 2; pass++) {
    norms_kernel<<<nb, RED_BLOCK, 0, st>>>(pass ? u : uex, pass ? uex : nullptr, G, nv, red);
    finish_kernel<<<1, RED_BLOCK, 0, st>>>(red, nb);
    MK(cudaGetLastError());
    MK(cudaMemcpyAsync(pass ? df : ex, red, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    MK(cudaStreamSynchronize(st));
  }
  double np = 1.0;
  for (int d = 0; d < G.nd; d++) np *= (double)G.dim[d];
  const double nrm[3] = {ex[0] / np, std::sqrt(ex[1] / np), ex[2]};
  err[0] = df[0] / np;
  err[1] = std::sqrt(df[1] / np);
  err[2] = df[2];
  const double tol = 1e-15;  // CalculateError.c:48
  if (nrm[0] > tol && nrm[1] > tol && nrm[2] > tol) {
    err[0] /= nrm[0];
    err[1] /= nrm[1];
    err[2] /= nrm[2];
  }
  return GB_OK;
}
}  // namespace gbh

extern "C" int gb_solver_error(gb_solver* s, const double* uex, int layout, int mem, double* err) {
  if (!s || !uex || !err) { gbh_set_error("gb_solver_error: null argument"); return GB_ERR_ARG; }
  if (!s->d_snap) MK(cudaMalloc((void**)&s->d_snap, s->nvals * sizeof(double)));
  // the exact solution, ghosted, into the snapshot array
  if (layout == GB_LAYOUT_GHOSTED) {
    MK(cudaMemcpyAsync(s->d_snap, uex, s->nvals * sizeof(double),
                       mem == GB_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s->stream));
  } else {
    const size_t nint = (size_t)npoints(s) * s->cfg.nvars;
    const double* src = uex;
    double* tmp = nullptr;
    if (mem == GB_MEM_HOST) {
      MK(cudaMallocAsync((void**)&tmp, nint * sizeof(double), s->stream));
      MK(cudaMemcpyAsync(tmp, uex, nint * sizeof(double), cudaMemcpyHostToDevice, s->stream));
      src = tmp;
    }
    MK(launch_pack(s->d_snap, src, s->G, s->cfg.nvars, 0, s->stream));
    if (tmp) MK(cudaFreeAsync(tmp, s->stream));
  }
  int rc = red_buffer(s);
  if (rc) return rc;
  return grid_error(s->d_u, s->d_snap, s->G, s->cfg.nvars, s->d_red, s->stream, err);
}

// ---------------------------------------------------------------------------
// Conservation check (shared by the solver and the ensemble)
// ---------------------------------------------------------------------------
namespace gbh {

long long cons_lines(const gb_config& c, int d) {
  long long n = 1;
  for (int e = 0; e < c.ndims; e++)
    if (e != d) n *= c.dim[e];
  return n;
}

// sum u dV over the interior of one grid, per variable; `red` holds
// 3 * RED_MAX_BLOCKS doubles (synchronises `st`).
int cons_volume(const double* u, const double* dxinv, const DevGeom& G, long long dxo1, long long dxo2, int nv,
                double* red, cudaStream_t st, double* V) {
  long long n = (long long)G.dim[0] * G.dim[1] * G.dim[2];
  long long b = (n + RED_BLOCK - 1) / RED_BLOCK;
  // at most RED_MAX_BLOCKS / 2 blocks: their nv <= 5 partials fit the buffer
  const int nb = (int)(b < RED_MAX_BLOCKS / 2 ? (b < 1 ? 1 : b) : RED_MAX_BLOCKS / 2);
  if (nv == 3) {
    volume_kernel<3><<<nb, RED_BLOCK, 0, st>>>(u, dxinv, G, dxo1, dxo2, red);
    volume_finish_kernel<3><<<1, RED_BLOCK, 0, st>>>(red, nb);
  } else if (nv == 4) {
    volume_kernel<4><<<nb, RED_BLOCK, 0, st>>>(u, dxinv, G, dxo1, dxo2, red);
    volume_finish_kernel<4><<<1, RED_BLOCK, 0, st>>>(red, nb);
  } else {
    volume_kernel<5><<<nb, RED_BLOCK, 0, st>>>(u, dxinv, G, dxo1, dxo2, red);
    volume_finish_kernel<5><<<1, RED_BLOCK, 0, st>>>(red, nb);
  }
  MK(cudaGetLastError());
  MK(cudaMemcpyAsync(V, red, nv * sizeof(double), cudaMemcpyDeviceToHost, st));
  MK(cudaStreamSynchronize(st));
  return GB_OK;
}

// The conservation error per variable, |V + B - V0| / max(|V0|, 1), with B the
// boundary-flux time integrals of the accumulators `bnd` (per direction d at
// off[d]: face 0 then face N, lines x nv) summed over lines and times the face
// areas dS_d = prod_{k != d} 1 / dxinv_k at the middle of dimension k
// (BoundaryIntegral.c; CalculateConservationError.c).  `dxmid[k]` is that dxinv.
int cons_error(const gb_config& c, const double* bnd, const long long* off, const double* V, const double* V0,
               const double* dxmid, double* red, cudaStream_t st, double* err) {
  const int nv = c.nvars;
  const long long n0 = cons_lines(c, 0), n1 = c.ndims > 1 ? cons_lines(c, 1) : 0,
                  n2 = c.ndims > 2 ? cons_lines(c, 2) : 0;
  const long long o1 = c.ndims > 1 ? off[1] : 0, o2 = c.ndims > 2 ? off[2] : 0;
  const int nblk = 2 * c.ndims;
  if (nv == 3)
    boundary_sum_kernel<3><<<nblk, RED_BLOCK, 0, st>>>(bnd, off[0], o1, o2, n0, n1, n2, red);
  else if (nv == 4)
    boundary_sum_kernel<4><<<nblk, RED_BLOCK, 0, st>>>(bnd, off[0], o1, o2, n0, n1, n2, red);
  else
    boundary_sum_kernel<5><<<nblk, RED_BLOCK, 0, st>>>(bnd, off[0], o1, o2, n0, n1, n2, red);
  MK(cudaGetLastError());
  double F[6 * 5];
  MK(cudaMemcpyAsync(F, red, nblk * nv * sizeof(double), cudaMemcpyDeviceToHost, st));
  MK(cudaStreamSynchronize(st));
  double B[5] = {0, 0, 0, 0, 0};
  for (int d = 0; d < c.ndims; d++) {
    double dS = 1.0;
    for (int k = 0; k < c.ndims; k++)
      if (k != d) dS *= (1.0 / dxmid[k]);
    for (int v = 0; v < nv; v++) {
      B[v] += F[(2 * d + 0) * nv + v] * dS;
      B[v] += F[(2 * d + 1) * nv + v] * dS;
    }
  }
  for (int v = 0; v < nv; v++) {
    const double base = std::fabs(V0[v]) > 1.0 ? std::fabs(V0[v]) : 1.0;
    const double e = V[v] + B[v] - V0[v];
    err[v] = std::sqrt(e * e) / base;
  }
  return GB_OK;
}

}  // namespace gbh

extern "C" int gb_solver_conservation_begin(gb_solver* s) {
  if (!s) { gbh_set_error("gb_solver_conservation_begin: null solver"); return GB_ERR_ARG; }
  const gb_config& c = s->cfg;
  int rc = red_buffer(s);
  if (rc) return rc;
  if (!s->d_bnd) {
    long long n = 0;
    for (int d = 0; d < c.ndims; d++) {
      s->bnd_off[d] = n;
      n += 2 * cons_lines(c, d) * c.nvars;
    }
    s->bnd_n = n;
    MK(cudaMalloc((void**)&s->d_bnd, n * sizeof(double)));
  }
  MK(cudaMemsetAsync(s->d_bnd, 0, s->bnd_n * sizeof(double), s->stream));
  rc = cons_volume(s->d_u, s->d_dxinv, s->G, s->dx_off[1], s->dx_off[2], c.nvars, s->d_red, s->stream, s->V0);
  if (rc) return rc;
  s->cons_on = true;
  return GB_OK;
}

extern "C" int gb_solver_conservation_error(gb_solver* s, double* err) {
  if (!s || !err) { gbh_set_error("gb_solver_conservation_error: null argument"); return GB_ERR_ARG; }
  if (!s->cons_on) { gbh_set_error("gb_solver_conservation_error: no gb_solver_conservation_begin"); return GB_ERR_ARG; }
  const gb_config& c = s->cfg;
  double V[5];
  int rc = cons_volume(s->d_u, s->d_dxinv, s->G, s->dx_off[1], s->dx_off[2], c.nvars, s->d_red, s->stream, V);
  if (rc) return rc;
  double mid[3] = {1.0, 1.0, 1.0};
  for (int k = 0; k < c.ndims; k++)
    MK(cudaMemcpyAsync(&mid[k], s->d_dxinv + s->dx_off[k] + c.ghosts + c.dim[k] / 2, sizeof(double),
                       cudaMemcpyDeviceToHost, s->stream));
  return cons_error(c, s->d_bnd, s->bnd_off, V, s->V0, mid, s->d_red, s->stream, err);
}
