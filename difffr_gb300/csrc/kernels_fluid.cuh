// kernels_fluid.cuh — fluid-side kernels of the DiffDFSPH step, templated on the
// fluid scalar T (float or double).
//
// Data layout (HBM, structure of arrays, particles kept in cell order and re-sorted
// every step by a stable counting sort):
//   x[i]  : V4<T> (x, y, z, -)        v[i] : V4<T> (vx, vy, vz, -)
//   kk[i] : stiffness read by the next velocity-correction pass
//   rho, alpha (DFSPH factor), kappa, kappaV, rhoAdv : T
//   sumgrad[i] : V4<T> (sum_grad_p_k, -)
//   fluid neighbours of i: flist[k * n + i], k < fcount[i]   (neighbour-major: coalesced)
//   boundary neighbours of i: blist[k * n + i], k < bcount[i]
// Boundary samples: static ones sorted once; dynamic ones in body order (xd, vd, x0d)
// plus a per-step cell-sorted copy appended after the static ones (bx, bv: x,y,z,psi).
#pragma once
#include "common.cuh"

namespace dfsph {

template <class T>
struct FluidConsts {
  int n;
  T h2, rho0, V, m, dt, invH, invH2, eps, visc, gx, gy, gz;
  Cubic<T> kc;
  Grid<T> grid;
  int kf, kb;  // list capacities
};

// ------------------------------------------------------------------ sorting

template <class T>
static __global__ void k_cell_keys(int n, const V4<T> *__restrict__ x, Grid<T> g, int *__restrict__ key,
                            int *__restrict__ rank, int *__restrict__ count, int *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V4<T> p = x[i];
  if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(err, ERR_NONFINITE_POSITION);
  int cx, cy, cz;
  grid_cell(g, p.x, p.y, p.z, cx, cy, cz);
  const int k = grid_key(g, cx, cy, cz);
  key[i] = k;
  rank[i] = atomicAdd(&count[k], 1);
}

static __global__ void k_scatter_order(int n, const int *__restrict__ key, const int *__restrict__ rank,
                                const int *__restrict__ start, int *__restrict__ order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  order[start[key[i]] + rank[i]] = i;
}

// Makes the order inside each cell ascending in the previous index, so that the
// sort (and every neighbour sum after it) is deterministic.
static __global__ void k_cell_insertion_sort(int ncell, const int *__restrict__ start, int *__restrict__ order) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int b = start[c], e = start[c + 1];
  for (int a = b + 1; a < e; a++) {
    const int v = order[a];
    int j = a - 1;
    while (j >= b && order[j] > v) { order[j + 1] = order[j]; j--; }
    order[j + 1] = v;
  }
}

template <class T>
static __global__ void k_gather_fluid(int n, const int *__restrict__ order, const V4<T> *__restrict__ x,
                               const V4<T> *__restrict__ v, const T *__restrict__ kappa,
                               const T *__restrict__ kappaV, const int *__restrict__ perm, V4<T> *__restrict__ x2,
                               V4<T> *__restrict__ v2, T *__restrict__ kappa2, T *__restrict__ kappaV2,
                               int *__restrict__ perm2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = order[i];
  x2[i] = x[o];
  v2[i] = v[o];
  kappa2[i] = kappa[o];
  kappaV2[i] = kappaV[o];
  perm2[i] = perm[o];
}

// dynamic boundary: body order -> cell order copy behind the static samples
template <class T>
static __global__ void k_gather_dynamic(int nd, int ns, const int *__restrict__ order, const V4<T> *__restrict__ xd,
                                 const V4<T> *__restrict__ vd, V4<T> *__restrict__ bx, V4<T> *__restrict__ bv,
                                 int *__restrict__ dyn_sorted_to_body) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nd) return;
  const int o = order[j];
  bx[ns + j] = xd[o];
  bv[ns + j] = vd[o];
  dyn_sorted_to_body[j] = o;
}

// ------------------------------------------------------------------ neighbour rows
// The 3 x 3 rows of cells around (cx, cy, cz); each row of 3 cells is one contiguous
// range of the cell-sorted array.
template <class T, class F>
static __device__ __forceinline__ void for_each_row(const Grid<T> &g, const int *__restrict__ cstart, int cx, int cy,
                                             int cz, F &&f) {
  const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx < g.nx - 1 ? cx + 1 : g.nx - 1;
  for (int dz = -1; dz <= 1; dz++) {
    const int z = cz + dz;
    if (z < 0 || z >= g.nz) continue;
    for (int dy = -1; dy <= 1; dy++) {
      const int y = cy + dy;
      if (y < 0 || y >= g.ny) continue;
      const int rb = (z * g.ny + y) * g.nx;
      f(cstart[rb + x0], cstart[rb + x1 + 1]);
    }
  }
}

// Neighbour lists (fluid and boundary), density (TimeStep.cpp:147-200) and the
// DFSPH factor with sum_grad_p_k (TimeStepDiffDFSPH.cpp:883-962), fused in one pass.
template <class T>
static __global__ void __launch_bounds__(256) k_lists_density_factor(
    FluidConsts<T> c, const V4<T> *__restrict__ x, const int *__restrict__ cstartF, const V4<T> *__restrict__ bx,
    const int *__restrict__ cstartS, const int *__restrict__ cstartD, int ns, int *__restrict__ flist,
    int *__restrict__ fcount, int *__restrict__ blist, int *__restrict__ bcount, T *__restrict__ rho,
    T *__restrict__ alpha, V4<T> *__restrict__ sumgrad, int *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const V4<T> xi = x[i];
  int cx, cy, cz;
  grid_cell(c.grid, xi.x, xi.y, xi.z, cx, cy, cz);
  T dens = c.V * c.kc.w0;
  T sgk = T(0);
  V3<T> gpi = {T(0), T(0), T(0)};
  int cnt = 0;
  for_each_row(c.grid, cstartF, cx, cy, cz, [&](int b, int e) {
    for (int j = b; j < e; j++) {
      if (j == i) continue;
      const V4<T> xj = x[j];
      const T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const T d2 = dist2_rn(dx, dy, dz);
      if (d2 < c.h2) {
        if (cnt < c.kf) flist[(size_t)cnt * c.n + i] = j;
        cnt++;
        const T rl = sqrt(d2);
        dens += c.V * cubic_W(rl, c.kc);
        const V3<T> gw = cubic_gradW(mk3(dx, dy, dz), rl, c.kc);
        const V3<T> gpj = (-c.V) * gw;
        sgk += dot(gpj, gpj);
        gpi = gpi - gpj;
      }
    }
  });
  if (cnt > c.kf) { atomicOr(err, ERR_FLUID_LIST_OVERFLOW); cnt = c.kf; }
  fcount[i] = cnt;
  int bc = 0;
  auto visit_boundary = [&](int b, int e, int off) {
    for (int j = b; j < e; j++) {
      const V4<T> xj = bx[off + j];
      const T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const T d2 = dist2_rn(dx, dy, dz);
      if (d2 < c.h2) {
        if (bc < c.kb) blist[(size_t)bc * c.n + i] = off + j;
        bc++;
        const T rl = sqrt(d2);
        dens += xj.w * cubic_W(rl, c.kc);
        const V3<T> gw = cubic_gradW(mk3(dx, dy, dz), rl, c.kc);
        const V3<T> gpj = (-xj.w) * gw;
        gpi = gpi - gpj;
      }
    }
  };
  for_each_row(c.grid, cstartS, cx, cy, cz, [&](int b, int e) { visit_boundary(b, e, 0); });
  if (cstartD) for_each_row(c.grid, cstartD, cx, cy, cz, [&](int b, int e) { visit_boundary(b, e, ns); });
  if (bc > c.kb) { atomicOr(err, ERR_BOUNDARY_LIST_OVERFLOW); bc = c.kb; }
  bcount[i] = bc;
  rho[i] = dens * c.rho0;
  sumgrad[i] = V4<T>{-gpi.x, -gpi.y, -gpi.z, T(0)};
  sgk += dot(gpi, gpi);
  alpha[i] = (sgk > c.eps) ? -T(1) / sgk : T(0);
}

// Fluid neighbours of each dynamic boundary sample (body order).
template <class T>
static __global__ void k_bf_lists(FluidConsts<T> c, int nd, const V4<T> *__restrict__ xd, const V4<T> *__restrict__ x,
                           const int *__restrict__ cstartF, int kbf, int *__restrict__ bflist,
                           int *__restrict__ bfcount, int *__restrict__ err) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd) return;
  const V4<T> xj = xd[d];
  int cx, cy, cz;
  grid_cell(c.grid, xj.x, xj.y, xj.z, cx, cy, cz);
  int cnt = 0;
  for_each_row(c.grid, cstartF, cx, cy, cz, [&](int b, int e) {
    for (int i = b; i < e; i++) {
      const V4<T> xi = x[i];
      const T dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      if (dist2_rn(dx, dy, dz) < c.h2) {
        if (cnt < kbf) bflist[(size_t)cnt * nd + d] = i;
        cnt++;
      }
    }
  });
  if (cnt > kbf) { atomicOr(err, ERR_BF_LIST_OVERFLOW); cnt = kbf; }
  bfcount[d] = cnt;
}

// psi of every boundary sample: 1 / (W0 + sum_k W over boundary neighbours of any body)
// (BoundaryModel_Akinci2012.cpp:257-284 via Simulation::updateBoundaryVolume).
// Samples p < ns are static (cell-sorted), p >= ns dynamic (sorted copy).
template <class T>
static __global__ void k_boundary_psi(FluidConsts<T> c, int ns, int nd, const V4<T> *__restrict__ bx,
                               const int *__restrict__ cstartS, const int *__restrict__ cstartD,
                               T *__restrict__ psi_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ns + nd) return;
  const V4<T> xp = bx[p];
  int cx, cy, cz;
  grid_cell(c.grid, xp.x, xp.y, xp.z, cx, cy, cz);
  T delta = c.kc.w0;
  auto visit = [&](int b, int e, int off) {
    for (int j = b; j < e; j++) {
      if (off + j == p) continue;
      const V4<T> xj = bx[off + j];
      const T dx = xp.x - xj.x, dy = xp.y - xj.y, dz = xp.z - xj.z;
      const T d2 = dist2_rn(dx, dy, dz);
      if (d2 < c.h2) delta += cubic_W(sqrt(d2), c.kc);
    }
  };
  if (ns > 0) for_each_row(c.grid, cstartS, cx, cy, cz, [&](int b, int e) { visit(b, e, 0); });
  if (nd > 0) for_each_row(c.grid, cstartD, cx, cy, cz, [&](int b, int e) { visit(b, e, ns); });
  psi_out[p] = T(1) / delta;
}

template <class T>
static __global__ void k_set_psi(int ns, int nd, const T *__restrict__ psi, V4<T> *__restrict__ bx, V4<T> *__restrict__ xd,
                          const int *__restrict__ dyn_sorted_to_body) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ns + nd) return;
  bx[p].w = psi[p];
  if (p >= ns) xd[dyn_sorted_to_body[p - ns]].w = psi[p];
}

// ------------------------------------------------------------------ solver passes

// Block reduction of a double to one partial per block (fixed order).
static __device__ __forceinline__ void block_partial_sum(double v, double *__restrict__ partials) {
  __shared__ double ws[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    double s = lane < nw ? ws[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) partials[blockIdx.x] = s;
  }
}

enum PassMode : int {
  PASS_PRESSURE = 0,         // rho_adv, k = (rho_adv - 1) alpha / h^2          (:1926-1975, :1110-1111)
  PASS_DIVERGENCE = 1,       // rho_dot, k = rho_dot alpha / h                   (:1977-2041, :1834-1835)
  PASS_PRESSURE_WARM = 2,    // rho_adv, kappa = rho_adv > 1 ? .5 max(kappa, -2.5e-4)/h^2 : 0  (:988-999)
  PASS_DIVERGENCE_WARM = 3,  // rho_dot, kappaV = rho_dot > 0 ? .5 max(kappaV, -.5)/h : 0      (:1721-1732)
};

// Density advection / density change of every particle, the stiffness for the next
// velocity correction, and the block partials of the solver residual.
template <class T, int MODE>
static __global__ void __launch_bounds__(256) k_density_pass(
    FluidConsts<T> c, const V4<T> *__restrict__ x, const V4<T> *__restrict__ v, const V4<T> *__restrict__ bx,
    const V4<T> *__restrict__ bv, const int *__restrict__ flist, const int *__restrict__ fcount,
    const int *__restrict__ blist, const int *__restrict__ bcount, const T *__restrict__ rho,
    const T *__restrict__ alpha, T *__restrict__ rhoAdv, T *__restrict__ kk, T *__restrict__ kappa_io,
    double *__restrict__ partials) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < c.n) {
    const V4<T> xi = x[i], vi4 = v[i];
    const V3<T> vi = xyz(vi4);
    T delta = T(0);
    const int nf = fcount[i];
    for (int k = 0; k < nf; k++) {
      const int j = flist[(size_t)k * c.n + i];
      const V4<T> xj = x[j], vj = v[j];
      const V3<T> r = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
      const T rl = sqrt(dot(r, r));
      delta += c.V * dot(vi - xyz(vj), cubic_gradW(r, rl, c.kc));
    }
    const int nb = bcount[i];
    for (int k = 0; k < nb; k++) {
      const int j = blist[(size_t)k * c.n + i];
      const V4<T> xj = bx[j], vj = bv[j];
      const V3<T> r = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
      const T rl = sqrt(dot(r, r));
      delta += xj.w * dot(vi - xyz(vj), cubic_gradW(r, rl, c.kc));
    }
    T ra;
    if (MODE == PASS_PRESSURE || MODE == PASS_PRESSURE_WARM) {
      ra = rho[i] / c.rho0 + c.dt * delta;
      ra = ra > T(1) ? ra : T(1);
    } else {
      ra = delta > T(0) ? delta : T(0);
      if (nf + nb < 20) ra = T(0);
    }
    rhoAdv[i] = ra;
    if (MODE == PASS_PRESSURE) {
      kk[i] = (ra - T(1)) * alpha[i] * c.invH2;
      e = (double)(c.rho0 * ra - c.rho0);
    } else if (MODE == PASS_DIVERGENCE) {
      kk[i] = ra * alpha[i] * c.invH;
      e = (double)(c.rho0 * ra);
    } else if (MODE == PASS_PRESSURE_WARM) {
      const T kp = kappa_io[i];
      const T kn = (ra > T(1)) ? T(0.5) * (kp > T(-0.00025) ? kp : T(-0.00025)) * c.invH2 : T(0);
      kappa_io[i] = kn;
      kk[i] = kn;
    } else {
      const T kp = kappa_io[i];
      const T kn = (ra > T(0)) ? T(0.5) * (kp > T(-0.5) ? kp : T(-0.5)) * c.invH : T(0);
      kappa_io[i] = kn;
      kk[i] = kn;
    }
  }
  if (partials) block_partial_sum(e, partials);
}

// Velocity correction with stiffness kk (warm start or Jacobi sweep):
// v_i -= dt sum_f (k_i + k_j)(-V grad W) [if |k_i + k_j| > eps];
// v_i += -dt k_i (-psi grad W) over boundary neighbours [if |k_i| > eps].
// ACC = 1 adds k_i to kappa_acc (the solver's running stiffness).
template <class T, int ACC>
static __global__ void __launch_bounds__(256) k_velocity_pass(
    FluidConsts<T> c, const V4<T> *__restrict__ x, V4<T> *__restrict__ v, const V4<T> *__restrict__ bx,
    const int *__restrict__ flist, const int *__restrict__ fcount, const int *__restrict__ blist,
    const int *__restrict__ bcount, const T *__restrict__ kk, T *__restrict__ kappa_acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const T ki = kk[i];
  if (ACC) kappa_acc[i] += ki;
  const V4<T> xi = x[i];
  V4<T> vi = v[i];
  const int nf = fcount[i];
  for (int k = 0; k < nf; k++) {
    const int j = flist[(size_t)k * c.n + i];
    const T kSum = ki + kk[j];
    if (fabs(kSum) > c.eps) {
      const V4<T> xj = x[j];
      const V3<T> r = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
      const T rl = sqrt(dot(r, r));
      const V3<T> gpj = (-c.V) * cubic_gradW(r, rl, c.kc);
      const T s = c.dt * kSum;
      vi.x -= s * gpj.x; vi.y -= s * gpj.y; vi.z -= s * gpj.z;
    }
  }
  if (fabs(ki) > c.eps) {
    const int nb = bcount[i];
    const T s = -c.dt * T(1) * ki;
    for (int k = 0; k < nb; k++) {
      const int j = blist[(size_t)k * c.n + i];
      const V4<T> xj = bx[j];
      const V3<T> r = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
      const T rl = sqrt(dot(r, r));
      const V3<T> gpj = (-xj.w) * cubic_gradW(r, rl, c.kc);
      vi.x += s * gpj.x; vi.y += s * gpj.y; vi.z += s * gpj.z;
    }
  }
  v[i] = vi;
}

// clearAccelerations + XSPH viscosity + v += dt a (TimeStep.cpp:66-81,
// Viscosity_XSPH.cpp:35-110, TimeStepDiffDFSPH.cpp:588-605); also kappaV *= dt
// (end of the divergence solve, :870-880) when scale_kappaV is set.
template <class T>
static __global__ void __launch_bounds__(256) k_xsph_advect(FluidConsts<T> c, const V4<T> *__restrict__ x,
                                                     const V4<T> *__restrict__ v, V4<T> *__restrict__ v_out,
                                                     const int *__restrict__ flist, const int *__restrict__ fcount,
                                                     const T *__restrict__ rho, T *__restrict__ kappaV,
                                                     int scale_kappaV) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const V4<T> xi = x[i], vi = v[i];
  V3<T> a = {c.gx, c.gy, c.gz};
  const int nf = fcount[i];
  const T cvis = c.invH * c.visc;
  for (int k = 0; k < nf; k++) {
    const int j = flist[(size_t)k * c.n + i];
    const V4<T> xj = x[j], vj = v[j];
    const V3<T> r = {xi.x - xj.x, xi.y - xj.y, xi.z - xj.z};
    const T w = cubic_W(sqrt(dot(r, r)), c.kc);
    const T s = cvis * (c.m / rho[j]);
    a.x -= s * (vi.x - vj.x) * w;
    a.y -= s * (vi.y - vj.y) * w;
    a.z -= s * (vi.z - vj.z) * w;
  }
  v_out[i] = V4<T>{vi.x + c.dt * a.x, vi.y + c.dt * a.y, vi.z + c.dt * a.z, T(0)};
  if (scale_kappaV) kappaV[i] *= c.dt;
}

// x += dt v (TimeStepDiffDFSPH.cpp:613-635); kappa *= dt^2 (:752-767) when requested.
template <class T>
static __global__ void k_integrate(FluidConsts<T> c, V4<T> *__restrict__ x, const V4<T> *__restrict__ v,
                            T *__restrict__ kappa, int scale_kappa) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  V4<T> p = x[i];
  const V4<T> u = v[i];
  p.x += c.dt * u.x; p.y += c.dt * u.y; p.z += c.dt * u.z;
  x[i] = p;
  if (scale_kappa) kappa[i] *= c.dt * c.dt;
}

// Final residual sum (one warp, fixed order); also publishes the device error word
// next to it in mapped host memory, so one stream synchronisation reads both.
static __global__ void k_final_sum(int nparts, const double *__restrict__ partials, double scale,
                                   double *__restrict__ out, double *__restrict__ out_host,
                                   const int *__restrict__ err) {
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += 32) s += partials[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) {
    *out = s * scale;
    if (out_host) {
      out_host[0] = s * scale;
      out_host[1] = (double)(*err);
    }
  }
}

}  // namespace dfsph
