// kernels_fluid.cuh — fluid-side kernels of the DiffDFSPH step, templated on the
// fluid scalar T (float or double).
//
// Data layout (HBM; particles kept in cell order and re-sorted every step by a
// stable counting sort):
//   R[i]  : Rec<T> = { x, y, z, - | vx, vy, vz, m_i / rho_i }   (32 bytes in FP32: one
//           256-bit load gives a neighbour's position and velocity)
//   Q[i]  : V4<T> (x, y, z, k) during a solve: the stiffness each density pass produces
//           for the next velocity-correction pass
//   rho, alpha (DFSPH factor), kappa, kappaV, rhoAdv : T;  sumgrad[i] : V4<T>
//   fluid neighbours of i: flist[k * n + i], k < fcount[i]   (neighbour-major)
//   boundary neighbours of i: blist[k * n + i], k < bcount[i]
// The neighbour passes run L lanes per particle, a template argument (sub-lane s visits
// list entries k = s, s + L, ...; the partial sums are combined with xor-shuffles in a
// fixed order). The context picks L from the particle count: 1 when one lane per particle
// fills the GPU (measured fastest on GB300 at 250k and 1M particles: the passes are bound
// by L1 data wavefronts, about one per distinct 32-byte record a warp gathers, which more
// lanes do not reduce), more for small scenes, whose one-lane grids would leave most SMs
// idle (L = LPP_MAX = 8: the 8,000-particle FP64 tank's passes run twice as fast).
// Boundary samples: static ones sorted once; dynamic ones in body order (xd, vd, x0d)
// plus a per-step cell-sorted copy after the static ones, both in BR[j] =
// { x, y, z, psi | vx, vy, vz, - }.
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
  int nbr;     // boundary records (static and dynamic samples): the bound of boundary indices
  int lpp;  // lanes per particle of the neighbour passes: 1 or LPP_MAX (the passes' template argument)
  // Akinci2013 surface tension: coefficients, cohesion kernel k and c, adhesion kernel k
  T st_k, st_kb, coh_k, coh_c, adh_k;
  T visc_b;  // XSPH coefficient against boundary samples (viscosityBoundary)
};

// |r|^2 summed as Eigen's squaredNorm sums a 3-vector (float: x^2 + (y^2 + z^2); double:
// (x^2 + y^2) + z^2), without contraction: the surface-tension kernels branch on |r|
// against h/2, and the reference's cohesion kernel is discontinuous there (its constant
// term h^6/64 is not scaled by k), so the branch has to be decided as the reference does.
template <class T> static __device__ __forceinline__ T sqnorm_ref(T x, T y, T z);
template <> __device__ __forceinline__ float sqnorm_ref<float>(float x, float y, float z) {
  return __fadd_rn(__fmul_rn(x, x), __fadd_rn(__fmul_rn(y, y), __fmul_rn(z, z)));
}
template <> __device__ __forceinline__ double sqnorm_ref<double>(double x, double y, double z) {
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// CohesionKernel (SPHKernels.h:437-506) and AdhesionKernel (:508-559) with support h,
// evaluated at r1 = |r| (IEEE square root of r2), r2 = |r|^2 <= h^2; the comparison with
// 0.5 h is made in double, as the reference's mixed-type expression does.
template <class T>
static __device__ __forceinline__ T cohesion_W(T r1, T r2, const FluidConsts<T> &c) {
  const T d = c.kc.h - r1;
  const T d3 = d * d * d;
  return ((double)r1 > 0.5 * (double)c.kc.h) ? c.coh_k * d3 * (r2 * r1) : c.coh_k * T(2) * d3 * (r2 * r1) - c.coh_c;
}
template <class T>
static __device__ __forceinline__ T adhesion_W(T r1, T r2, const FluidConsts<T> &c) {
  if (!((double)r1 > 0.5 * (double)c.kc.h)) return T(0);
  T a = -T(4) * r2 / c.kc.h + T(6) * r1 - T(2) * c.kc.h;
  a = a > T(0) ? a : T(0);  // rounding can take the argument below 0 at |r| = h
  return c.adh_k * sqrt(sqrt(a));
}

template <class T>
struct alignas(8 * sizeof(T)) Rec {
  V4<T> x, v;
};

// Whole-record load through the read-only path (the record is not written by the
// kernel that calls this): one 256-bit request in FP32.
template <class T> static __device__ __forceinline__ Rec<T> ld_rec(const Rec<T> *p) { return *p; }
template <> __device__ __forceinline__ Rec<float> ld_rec<float>(const Rec<float> *p) {
  Rec<float> r;
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(r.x.x), "=f"(r.x.y), "=f"(r.x.z), "=f"(r.x.w), "=f"(r.v.x), "=f"(r.v.y), "=f"(r.v.z), "=f"(r.v.w)
      : "l"(p));
  return r;
}

// ------------------------------------------------------------------ sorting

// pts[i * stride] is the position of point i (stride 2 for Rec arrays, 1 for V4 arrays)
template <class T>
static __global__ void k_cell_keys(int n, const V4<T> *__restrict__ pts, int stride, Grid<T> g,
                                   int *__restrict__ key, int *__restrict__ rank, int *__restrict__ count,
                                   int *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V4<T> p = pts[(size_t)i * stride];
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
static __global__ void k_gather_fluid(int n, const int *__restrict__ order, const Rec<T> *__restrict__ R,
                                      const T *__restrict__ kappa, const T *__restrict__ kappaV,
                                      const int *__restrict__ perm, Rec<T> *__restrict__ R2, T *__restrict__ kappa2,
                                      T *__restrict__ kappaV2, int *__restrict__ perm2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = order[i];
  R2[i] = ld_rec(R + o);
  kappa2[i] = kappa[o];
  kappaV2[i] = kappaV[o];
  perm2[i] = perm[o];
}

// Dynamic samples, few of them: one block sorts (cell key, body-order index) pairs with a
// bitonic network in shared memory (the order the counting sort plus per-cell insertion
// sort gives: by cell, then by index), writes the sorted records behind the static ones and
// the sorted keys; k_cstart_from_keys then fills the cell-start table by binary search.
constexpr int SMALL_SORT_MAX = 4096;
template <class T>
static __global__ void __launch_bounds__(1024) k_sort_dynamic_small(int nd, int ns, Grid<T> g,
                                                                    const V4<T> *__restrict__ xd,
                                                                    const V4<T> *__restrict__ vd, Rec<T> *__restrict__ BR,
                                                                    int *__restrict__ dyn_sorted_to_body,
                                                                    int *__restrict__ skeys, int *__restrict__ err) {
  __shared__ unsigned long long kv[SMALL_SORT_MAX];
  int m = 1;
  while (m < nd) m <<= 1;
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    unsigned long long v = ~0ull;
    if (j < nd) {
      const V4<T> p = xd[j];
      if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(err, ERR_NONFINITE_POSITION);
      int cx, cy, cz;
      grid_cell(g, p.x, p.y, p.z, cx, cy, cz);
      v = ((unsigned long long)(unsigned)grid_key(g, cx, cy, cz) << 32) | (unsigned)j;
    }
    kv[j] = v;
  }
  __syncthreads();
  for (int k = 2; k <= m; k <<= 1)
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int a = threadIdx.x; a < m; a += blockDim.x) {
        const int b = a ^ jj;
        if (b > a) {
          const unsigned long long x = kv[a], y = kv[b];
          const bool up = (a & k) == 0;
          if ((x > y) == up) { kv[a] = y; kv[b] = x; }
        }
      }
      __syncthreads();
    }
  for (int j = threadIdx.x; j < nd; j += blockDim.x) {
    const int o = (int)(kv[j] & 0xffffffffu);
    BR[ns + j] = Rec<T>{xd[o], vd[o]};
    dyn_sorted_to_body[j] = o;
    skeys[j] = (int)(kv[j] >> 32);
  }
}
static __global__ void k_cstart_from_keys(int ncell, int nd, const int *__restrict__ skeys, int *__restrict__ cstart) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncell) return;
  int lo = 0, hi = nd;  // first sorted key >= c
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (skeys[mid] < c) lo = mid + 1; else hi = mid;
  }
  cstart[c] = lo;
}

// dynamic boundary: body order -> cell order copy behind the static samples
template <class T>
static __global__ void k_gather_dynamic(int nd, int ns, const int *__restrict__ order, const V4<T> *__restrict__ xd,
                                        const V4<T> *__restrict__ vd, Rec<T> *__restrict__ BR,
                                        int *__restrict__ dyn_sorted_to_body) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nd) return;
  const int o = order[j];
  BR[ns + j] = Rec<T>{xd[o], vd[o]};
  dyn_sorted_to_body[j] = o;
}

// ------------------------------------------------------------------ neighbour rows
// The 3 x 3 rows of cells around (cx, cy, cz); each row of 3 cells is one contiguous
// range of the cell-sorted array.
template <class T, class F>
static __device__ __forceinline__ void for_each_row(const Grid<T> &g, const int *__restrict__ cstart, int cx, int cy,
                                             int cz, F &&f, int npts = 0x7fffffff) {
  const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx < g.nx - 1 ? cx + 1 : g.nx - 1;
  for (int dz = -1; dz <= 1; dz++) {
    const int z = cz + dz;
    if (z < 0 || z >= g.nz) continue;
    for (int dy = -1; dy <= 1; dy++) {
      const int y = cy + dy;
      if (y < 0 || y >= g.ny) continue;
      const int rb = (z * g.ny + y) * g.nx;
#ifdef DFSPH_BOUNDS_CHECK
      int b = cstart[rb + x0], e = cstart[rb + x1 + 1];
      if (b < 0 || e < b || e > npts) {
        atomicOr(&g_dfsph_bounds_err, BOUNDS_CELL_RANGE);
        b = e = 0;
      }
      f(b, e);
#else
      (void)npts;
      f(cstart[rb + x0], cstart[rb + x1 + 1]);
#endif
    }
  }
}

// The list build's arithmetic, shared by k_lists_density_factor and the small scenes'
// k_density_factor_from_lists: the neighbour terms in list order, then the outputs.
template <class T> struct ListSums {
  T dens, sgk, delta;
  V3<T> gpi;
};
template <class T, bool DIVWARM>
static __device__ __forceinline__ void list_fluid_terms(const FluidConsts<T> &c, const Rec<T> *__restrict__ R,
                                                        const int *__restrict__ flist, int i, int cnt, V4<T> xi,
                                                        V4<T> vi, ListSums<T> &S) {
  for (int k0 = 0; k0 < cnt; k0 += 4) {
    int js[4];
    V4<T> xs[4];
#pragma unroll
    for (int u = 0; u < 4; u++) js[u] = (k0 + u < cnt) ? DF_INDEX(flist[(size_t)(k0 + u) * c.n + i], c.n, BOUNDS_FLUID_LIST) : i;
#pragma unroll
    for (int u = 0; u < 4; u++) xs[u] = R[js[u]].x;
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (k0 + u >= cnt) break;
      const T dx = xi.x - xs[u].x, dy = xi.y - xs[u].y, dz = xi.z - xs[u].z;
      const T d2 = dist2_rn(dx, dy, dz);
      S.dens += c.V * KEval<T>::W(d2, c.kc);
      const T g = KEval<T>::G(d2, c.kc);
      const V3<T> gpj = (-c.V) * V3<T>{g * dx, g * dy, g * dz};
      S.sgk += dot(gpj, gpj);
      S.gpi = S.gpi - gpj;
      if (DIVWARM) {
        const V4<T> vj = R[js[u]].v;
        S.delta += c.V * (g * ((vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz));
      }
    }
  }
}
template <class T, bool DIVWARM>
static __device__ __forceinline__ void list_boundary_terms(const FluidConsts<T> &c, const Rec<T> *__restrict__ BR,
                                                           const int *__restrict__ blist, int i, int bc, V4<T> xi,
                                                           V4<T> vi, ListSums<T> &S) {
  for (int k = 0; k < bc; k++) {
    const int j = DF_INDEX(blist[(size_t)k * c.n + i], c.nbr, BOUNDS_BOUNDARY_LIST);
    const V4<T> xj = BR[j].x;
    const T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    const T d2 = dist2_rn(dx, dy, dz);
    S.dens += xj.w * KEval<T>::W(d2, c.kc);
    const T g = KEval<T>::G(d2, c.kc);
    const V3<T> gpj = (-xj.w) * V3<T>{g * dx, g * dy, g * dz};
    S.gpi = S.gpi - gpj;
    if (DIVWARM) {
      const V4<T> vj = BR[j].v;
      S.delta += xj.w * (g * ((vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz));
    }
  }
}
template <class T, bool DIVWARM>
static __device__ __forceinline__ void list_outputs(const FluidConsts<T> &c, Rec<T> *__restrict__ R, int i, int cnt,
                                                    int bc, V4<T> xi, const ListSums<T> &S, T *__restrict__ rho,
                                                    T *__restrict__ alpha, V4<T> *__restrict__ sumgrad,
                                                    V4<T> *__restrict__ Q, T *__restrict__ rhoAdv,
                                                    T *__restrict__ kappaV) {
  const T rh = S.dens * c.rho0;
  rho[i] = rh;
  R[i].v.w = c.m / rh;
  sumgrad[i] = V4<T>{-S.gpi.x, -S.gpi.y, -S.gpi.z, T(0)};
  const T sgk = S.sgk + dot(S.gpi, S.gpi);
  alpha[i] = (sgk > c.eps) ? -T(1) / sgk : T(0);
  if (DIVWARM) {
    T ra = S.delta > T(0) ? S.delta : T(0);
    if (cnt + bc < 20) ra = T(0);
    rhoAdv[i] = ra;
    const T kp = kappaV[i];
    const T kq = (ra > T(0)) ? T(0.5) * (kp > T(-0.5) ? kp : T(-0.5)) * c.invH : T(0);
    kappaV[i] = kq;
    Q[i] = V4<T>{xi.x, xi.y, xi.z, kq};
  }
}

// Neighbour lists (fluid and boundary), density (TimeStep.cpp:147-200) and the
// DFSPH factor with sum_grad_p_k (TimeStepDiffDFSPH.cpp:883-962), fused in one pass.
// Also stores the XSPH weight m_i / rho_i in v[i].w for the viscosity pass.
// DIVWARM: also the divergence solve's warm start (what k_density_pass does in
// PASS_DIVERGENCE_WARM, :1698-1788 with :1977-2041): the density change over the same
// neighbours in the same order, rho_dot = 0 below 20 neighbours, kappaV = 0.5 max(kappaV,
// -0.5) / h where rho_dot > 0, and Q[i] = (x_i, kappaV) for the warm-start correction.
constexpr int LIST_THREADS = 128;
#ifndef DFSPH_LIST_SCAN_BATCH
#define DFSPH_LIST_SCAN_BATCH 4  // candidate loads in flight per lane in the list build's scan
#endif
template <class T, bool DIVWARM>
static __global__ void __launch_bounds__(LIST_THREADS) k_lists_density_factor(
    FluidConsts<T> c, Rec<T> *__restrict__ R, const int *__restrict__ cstartF,
    const Rec<T> *__restrict__ BR, const int *__restrict__ cstartS, const int *__restrict__ cstartD, int ns,
    int *__restrict__ flist, int *__restrict__ fcount, int *__restrict__ blist, int *__restrict__ bcount,
    T *__restrict__ rho, T *__restrict__ alpha, V4<T> *__restrict__ sumgrad, int *__restrict__ err,
    V4<T> *__restrict__ Q, T *__restrict__ rhoAdv, T *__restrict__ kappaV) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const Rec<T> ri = ld_rec(R + i);
  const V4<T> xi = ri.x, vi = ri.v;
  int cx, cy, cz;
  grid_cell(c.grid, xi.x, xi.y, xi.z, cx, cy, cz);
  ListSums<T> S{c.V * c.kc.w0, T(0), T(0), {T(0), T(0), T(0)}};
  // Two phases, so that the kernel arithmetic runs once per neighbour: the lane's candidate
  // scan only appends accepted indices (about one candidate in eight is accepted, so a
  // fused accept branch would be taken by some lane of the warp nearly every iteration),
  // then the lane walks its own list in order. Same neighbours, same order, same formulas.
  int cnt = 0;
  for_each_row(c.grid, cstartF, cx, cy, cz, [&](int b, int e) {
    for (int j0 = b; j0 < e; j0 += DFSPH_LIST_SCAN_BATCH) {
      V4<T> xs[DFSPH_LIST_SCAN_BATCH];
#pragma unroll
      for (int u = 0; u < DFSPH_LIST_SCAN_BATCH; u++)
        if (j0 + u < e) xs[u] = R[j0 + u].x;
#pragma unroll
      for (int u = 0; u < DFSPH_LIST_SCAN_BATCH; u++) {
        const int j = j0 + u;
        if (j >= e || j == i) continue;
        const T dx = xi.x - xs[u].x, dy = xi.y - xs[u].y, dz = xi.z - xs[u].z;
        if (dist2_rn(dx, dy, dz) < c.h2) {
          if (cnt < c.kf) flist[(size_t)cnt * c.n + i] = j;
          cnt++;
        }
      }
    }
  }, c.n);
  if (cnt > c.kf) { atomicOr(err, ERR_FLUID_LIST_OVERFLOW); cnt = c.kf; }
  fcount[i] = cnt;
  list_fluid_terms<T, DIVWARM>(c, R, flist, i, cnt, xi, vi, S);
  int bc = 0;
  auto scan_boundary = [&](int b, int e, int off) {
    for (int j = b; j < e; j++) {
      const V4<T> xj = BR[off + j].x;
      const T dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      if (dist2_rn(dx, dy, dz) < c.h2) {
        if (bc < c.kb) blist[(size_t)bc * c.n + i] = off + j;
        bc++;
      }
    }
  };
  for_each_row(c.grid, cstartS, cx, cy, cz, [&](int b, int e) { scan_boundary(b, e, 0); }, ns);
  if (cstartD) for_each_row(c.grid, cstartD, cx, cy, cz, [&](int b, int e) { scan_boundary(b, e, ns); }, c.nbr - ns);
  if (bc > c.kb) { atomicOr(err, ERR_BOUNDARY_LIST_OVERFLOW); bc = c.kb; }
  bcount[i] = bc;
  list_boundary_terms<T, DIVWARM>(c, BR, blist, i, bc, xi, vi, S);
  list_outputs<T, DIVWARM>(c, R, i, cnt, bc, xi, S, rho, alpha, sumgrad, Q, rhoAdv, kappaV);
}

// One warp's scan of the 3 x 3 cell rows around (cx, cy, cz) in a cell-start array, for
// particle i: lanes 0-8 read the rows' bounds together, the rows' candidates are numbered
// in row order, and the lanes test 32 consecutive candidate numbers at a time (accept(j));
// the accepted ones are appended in candidate order (ballot and prefix count) to
// list[k * n + i] for k < cap, after cnt0 earlier entries, each as off + j: the list the
// serial scan of k_lists_density_factor makes, entry for entry. Returns the count (in every
// lane), which may exceed cap.
template <class T, class AcceptF>
static __device__ __forceinline__ int warp_scan_rows(const Grid<T> &g, const int *__restrict__ cstart, int cx, int cy,
                                                     int cz, int npts, int off, int *__restrict__ list, int n, int i,
                                                     int cap, int cnt0, AcceptF &&accept) {
  (void)npts;
  const int lane = threadIdx.x & 31;
  int rb = 0, re = 0;
  if (lane < 9) {
    const int z = cz + lane / 3 - 1, y = cy + lane % 3 - 1;
    if (z >= 0 && z < g.nz && y >= 0 && y < g.ny) {
      const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx < g.nx - 1 ? cx + 1 : g.nx - 1;
      const int base = (z * g.ny + y) * g.nx;
      rb = cstart[base + x0];
      re = cstart[base + x1 + 1];
#ifdef DFSPH_BOUNDS_CHECK
      if (rb < 0 || re < rb || re > npts) {
        atomicOr(&g_dfsph_bounds_err, BOUNDS_CELL_RANGE);
        rb = re = 0;
      }
#endif
    }
  }
  const int len = re - rb;
  int incl = len;
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 8);
  int rowb[9], rowoff[9];
#pragma unroll
  for (int r = 0; r < 9; r++) {
    rowb[r] = __shfl_sync(0xffffffffu, rb, r);
    rowoff[r] = __shfl_sync(0xffffffffu, incl - len, r);
  }
  int cnt = cnt0;
  for (int c0 = 0; c0 < total; c0 += 32) {
    const int q = c0 + lane;
    bool acc = false;
    int j = 0;
    if (q < total) {
      // the row holding candidate q (empty rows share their successor's offset)
      int bb = rowb[0], oo = rowoff[0];
#pragma unroll
      for (int k = 1; k < 9; k++)
        if (q >= rowoff[k]) { bb = rowb[k]; oo = rowoff[k]; }
      j = bb + (q - oo);
      acc = accept(j);
    }
    const unsigned m = __ballot_sync(0xffffffffu, acc);
    if (acc) {
      const int k = cnt + __popc(m & ((1u << lane) - 1u));
      if (k < cap) list[(size_t)k * n + i] = off + j;
    }
    cnt += __popc(m);
  }
  return cnt;
}

// Small scenes (where the neighbour passes run several lanes per particle): the lists of
// k_lists_density_factor, built one warp per particle (warp_scan_rows; same entries, same
// order, same counts and overflow bits), so that the candidate scan spreads over the GPU.
// k_density_factor_from_lists then runs the list build's arithmetic, one thread per
// particle, with the same code: the results are those of k_lists_density_factor.
template <class T>
static __global__ void __launch_bounds__(LIST_THREADS) k_lists_scan_warp(
    FluidConsts<T> c, const Rec<T> *__restrict__ R, const int *__restrict__ cstartF, const Rec<T> *__restrict__ BR,
    const int *__restrict__ cstartS, const int *__restrict__ cstartD, int ns, int *__restrict__ flist,
    int *__restrict__ fcount, int *__restrict__ blist, int *__restrict__ bcount, int *__restrict__ err) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= c.n) return;  // whole warps
  const V4<T> xi = R[i].x;
  int cx, cy, cz;
  grid_cell(c.grid, xi.x, xi.y, xi.z, cx, cy, cz);
  int cnt = warp_scan_rows(c.grid, cstartF, cx, cy, cz, c.n, 0, flist, c.n, i, c.kf, 0, [&](int j) {
    if (j == i) return false;
    const V4<T> xj = R[j].x;
    return dist2_rn(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z) < c.h2;
  });
  auto near_boundary = [&](int j) {
    const V4<T> xj = BR[j].x;
    return dist2_rn(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z) < c.h2;
  };
  int bc = warp_scan_rows(c.grid, cstartS, cx, cy, cz, ns, 0, blist, c.n, i, c.kb, 0, near_boundary);
  if (cstartD)
    bc = warp_scan_rows(c.grid, cstartD, cx, cy, cz, c.nbr - ns, ns, blist, c.n, i, c.kb, bc,
                        [&](int j) { return near_boundary(ns + j); });
  if ((threadIdx.x & 31) != 0) return;
  if (cnt > c.kf) { atomicOr(err, ERR_FLUID_LIST_OVERFLOW); cnt = c.kf; }
  if (bc > c.kb) { atomicOr(err, ERR_BOUNDARY_LIST_OVERFLOW); bc = c.kb; }
  fcount[i] = cnt;
  bcount[i] = bc;
}
template <class T, bool DIVWARM>
static __global__ void __launch_bounds__(LIST_THREADS) k_density_factor_from_lists(
    FluidConsts<T> c, Rec<T> *__restrict__ R, const Rec<T> *__restrict__ BR, const int *__restrict__ flist,
    const int *__restrict__ fcount, const int *__restrict__ blist, const int *__restrict__ bcount,
    T *__restrict__ rho, T *__restrict__ alpha, V4<T> *__restrict__ sumgrad, V4<T> *__restrict__ Q,
    T *__restrict__ rhoAdv, T *__restrict__ kappaV) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const Rec<T> ri = ld_rec(R + i);
  const V4<T> xi = ri.x, vi = ri.v;
  ListSums<T> S{c.V * c.kc.w0, T(0), T(0), {T(0), T(0), T(0)}};
  const int cnt = fcount[i], bc = bcount[i];
  list_fluid_terms<T, DIVWARM>(c, R, flist, i, cnt, xi, vi, S);
  list_boundary_terms<T, DIVWARM>(c, BR, blist, i, bc, xi, vi, S);
  list_outputs<T, DIVWARM>(c, R, i, cnt, bc, xi, S, rho, alpha, sumgrad, Q, rhoAdv, kappaV);
}

// Fluid neighbours of each dynamic boundary sample (body order), one warp per sample. The
// candidates of the 9 cell rows are numbered in row order; lanes 0-8 read the rows' bounds
// together, then the lanes test 32 consecutive candidate numbers at a time, across row
// ends, and append the accepted ones in candidate order (ballot and prefix count): the
// list a serial scan of the rows in order makes.
template <class T>
static __global__ void k_bf_lists(FluidConsts<T> c, int nd, const V4<T> *__restrict__ xd, const Rec<T> *__restrict__ R,
                           const int *__restrict__ cstartF, int kbf, int *__restrict__ bflist,
                           int *__restrict__ bfcount, int *__restrict__ err) {
  const int d = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (d >= nd) return;  // whole warps
  const V4<T> xj = xd[d];
  int cx, cy, cz;
  grid_cell(c.grid, xj.x, xj.y, xj.z, cx, cy, cz);
  // row r = 3 (dz + 1) + (dy + 1): [rb, re) of the cells x-1..x+1 (empty outside the grid)
  int rb = 0, re = 0;
  if (lane < 9) {
    const int z = cz + lane / 3 - 1, y = cy + lane % 3 - 1;
    if (z >= 0 && z < c.grid.nz && y >= 0 && y < c.grid.ny) {
      const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx < c.grid.nx - 1 ? cx + 1 : c.grid.nx - 1;
      const int base = (z * c.grid.ny + y) * c.grid.nx;
      rb = cstartF[base + x0];
      re = cstartF[base + x1 + 1];
    }
  }
  // exclusive prefix of the row lengths over lanes 0-8
  const int len = re - rb;
  int incl = len;
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 8);
  int rowb[9], rowoff[9];
#pragma unroll
  for (int r = 0; r < 9; r++) {
    rowb[r] = __shfl_sync(0xffffffffu, rb, r);
    rowoff[r] = __shfl_sync(0xffffffffu, incl - len, r);
  }
  int cnt = 0;
  for (int c0 = 0; c0 < total; c0 += 32) {
    const int q = c0 + lane;
    bool acc = false;
    int i = 0;
    if (q < total) {
      int r = 0;
#pragma unroll
      for (int k = 1; k < 9; k++)
        if (q >= rowoff[k]) r = k;
      // rows are numbered in order and empty rows share their successor's offset
      int bb = rowb[0], oo = rowoff[0];
#pragma unroll
      for (int k = 1; k < 9; k++)
        if (k == r) { bb = rowb[k]; oo = rowoff[k]; }
      i = bb + (q - oo);
      const V4<T> xi = R[i].x;
      const T dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      acc = dist2_rn(dx, dy, dz) < c.h2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, acc);
    if (acc) {
      const int k = cnt + __popc(m & ((1u << lane) - 1u));
      if (k < kbf) bflist[(size_t)k * nd + d] = i;
    }
    cnt += __popc(m);
  }
  if (lane == 0) {
    if (cnt > kbf) { atomicOr(err, ERR_BF_LIST_OVERFLOW); cnt = kbf; }
    bfcount[d] = cnt;
  }
}

// psi of every boundary sample: 1 / (W0 + sum_k W over boundary neighbours of any body)
// (BoundaryModel_Akinci2012.cpp:257-284 via Simulation::updateBoundaryVolume).
// Samples p < ns are static (cell-sorted), p >= ns dynamic (sorted copy).
template <class T>
static __global__ void k_boundary_psi(FluidConsts<T> c, int ns, int nd, const Rec<T> *__restrict__ BR,
                               const int *__restrict__ cstartS, const int *__restrict__ cstartD,
                               T *__restrict__ psi_out, int p0) {
  const int p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ns + nd) return;
  const V4<T> xp = BR[p].x;
  int cx, cy, cz;
  grid_cell(c.grid, xp.x, xp.y, xp.z, cx, cy, cz);
  T delta = c.kc.w0;
  auto visit = [&](int b, int e, int off) {
    for (int j = b; j < e; j++) {
      if (off + j == p) continue;
      const V4<T> xj = BR[off + j].x;
      const T dx = xp.x - xj.x, dy = xp.y - xj.y, dz = xp.z - xj.z;
      const T d2 = dist2_rn(dx, dy, dz);
      if (d2 < c.h2) delta += KEval<T>::W(d2, c.kc);
    }
  };
  if (ns > 0) for_each_row(c.grid, cstartS, cx, cy, cz, [&](int b, int e) { visit(b, e, 0); }, ns);
  if (nd > 0) for_each_row(c.grid, cstartD, cx, cy, cz, [&](int b, int e) { visit(b, e, ns); }, nd);
  psi_out[p] = T(1) / delta;
}

template <class T>
static __global__ void k_set_psi(int ns, int nd, const T *__restrict__ psi, Rec<T> *__restrict__ BR,
                                 V4<T> *__restrict__ xd, const int *__restrict__ dyn_sorted_to_body, int p0) {
  const int p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ns + nd) return;
  BR[p].x.w = psi[p];
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

constexpr int LPP_MAX = 8;  // most lanes per particle in the neighbour passes

// Visits the entries k = s, s + lpp, ... < cnt of the neighbour-major list of particle i
// for sub-lane s of lpp, U at a time, as a software pipeline: the U list indices of the next
// batch are requested before the U gathers (load(j)) of the current batch are consumed,
// so the list's DRAM latency overlaps the gathers. Bodies run in ascending k.
// lim, bit: the bound of the list's indices and its bit in the bounds-checked build.
template <int U, class D, class LoadF, class BodyF>
static __device__ __forceinline__ void for_neighbors_sub(int cnt, const int *__restrict__ list, int n, int i, int s,
                                                         int lpp, LoadF &&load, BodyF &&body, int lim, int bit) {
  (void)lim;
  (void)bit;
  int js[U];
#pragma unroll
  for (int u = 0; u < U; u++)
    js[u] = (s + u * lpp < cnt) ? DF_INDEX(__ldcs(list + (size_t)(s + u * lpp) * n + i), lim, bit) : 0;
  for (int k0 = s; k0 < cnt; k0 += U * lpp) {
    D d[U];
#pragma unroll
    for (int u = 0; u < U; u++)
      if (k0 + u * lpp < cnt) d[u] = load(js[u]);
    const int k1 = k0 + U * lpp;
#pragma unroll
    for (int u = 0; u < U; u++)
      js[u] = (k1 + u * lpp < cnt) ? DF_INDEX(__ldcs(list + (size_t)(k1 + u * lpp) * n + i), lim, bit) : 0;
#pragma unroll
    for (int u = 0; u < U; u++)
      if (k0 + u * lpp < cnt) body(d[u]);
  }
}

// Batch sizes of the neighbour passes and their minimum resident blocks per SM
// (register budget); build-time tuning constants.
#ifndef DFSPH_DENSITY_BATCH
#define DFSPH_DENSITY_BATCH 2
#endif
#ifndef DFSPH_VELOCITY_BATCH
#define DFSPH_VELOCITY_BATCH 4
#endif
#ifndef DFSPH_XSPH_BATCH
#define DFSPH_XSPH_BATCH 4
#endif
// Threads per block of the density and velocity passes; the minimum resident blocks below
// are given for 256 threads and scaled, so that the register budget stays the same.
#ifndef DFSPH_PASS_THREADS
#define DFSPH_PASS_THREADS 128
#endif
constexpr int PASS_THREADS = DFSPH_PASS_THREADS;
#ifndef DFSPH_DENSITY_MIN_BLOCKS
#define DFSPH_DENSITY_MIN_BLOCKS 6
#endif
#ifndef DFSPH_DENSITY_XS_MIN_BLOCKS
#define DFSPH_DENSITY_XS_MIN_BLOCKS 5
#endif
#ifndef DFSPH_VELOCITY_MIN_BLOCKS
#define DFSPH_VELOCITY_MIN_BLOCKS 5
#endif
#ifndef DFSPH_XSPH_MIN_BLOCKS
#define DFSPH_XSPH_MIN_BLOCKS 4
#endif

// Minimum resident blocks of a pass for the fluid type: the FP32 figures above; FP64 passes
// need about twice the registers, so they ask for half the blocks (instead of spilling).
template <class T> constexpr int pass_min_blocks(int fp32_blocks) {
  return sizeof(T) == 8 ? (fp32_blocks + 1) / 2 : fp32_blocks;
}

// Sum over the L sub-lanes of a particle (all lanes of the warp take part), in a fixed
// order for a given L.
template <int L, class T> static __device__ __forceinline__ T sub_sum(T v) {
#pragma unroll
  for (int o = 1; o < L; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Density advection / density change of every particle, the stiffness for the next
// velocity correction, and the block partials of the solver residual.
// Reads R (positions, velocities); writes Q[i] = (x_i, k_i): the next velocity pass
// gathers position and stiffness of a neighbour with one 16-byte load.
// XS (divergence passes only): the same neighbour records also give the XSPH viscosity
// and gravity of the next phase (k_xsph_advect's arithmetic, in its order); the advected
// records go to R_out. Once the divergence solve's last check passes, R_out holds the
// state the separate XSPH pass would have produced.
template <class T, int MODE, bool XS, int L>
static __global__ void __launch_bounds__(PASS_THREADS, pass_min_blocks<T>((XS ? DFSPH_DENSITY_XS_MIN_BLOCKS : DFSPH_DENSITY_MIN_BLOCKS) * 256 / PASS_THREADS)) k_density_pass(
    FluidConsts<T> c, const Rec<T> *__restrict__ R, V4<T> *__restrict__ Q, const Rec<T> *__restrict__ BR,
    const int *__restrict__ flist, const int *__restrict__ fcount, const int *__restrict__ blist,
    const int *__restrict__ bcount, const T *__restrict__ rho, const T *__restrict__ alpha, T *__restrict__ rhoAdv,
    T *__restrict__ kappa_io, double *__restrict__ partials, float4 *__restrict__ feat, Rec<T> *__restrict__ R_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / L, s = t % L;
  const bool live = i < c.n;
  double e = 0.0;
  T delta = T(0);
  T ax = T(0), ay = T(0), az = T(0);
  int nf = 0, nb = 0;
  Rec<T> ri;
  if (live) {
    ri = ld_rec(R + i);
    const V4<T> xi = ri.x, vi4 = ri.v;
    const T cvis = c.invH * c.visc;
    nf = fcount[i];
    for_neighbors_sub<DFSPH_DENSITY_BATCH, Rec<T>>(nf, flist, c.n, i, s, L, [&](int j) { return ld_rec(R + j); }, [&](const Rec<T> &d) {
      const T rx = xi.x - d.x.x, ry = xi.y - d.x.y, rz = xi.z - d.x.z;
      const T g = KEval<T>::G(rx * rx + ry * ry + rz * rz, c.kc);
      delta += c.V * (g * ((vi4.x - d.v.x) * rx + (vi4.y - d.v.y) * ry + (vi4.z - d.v.z) * rz));
      if (XS) {
        const T w = KEval<T>::W(rx * rx + ry * ry + rz * rz, c.kc);
        const T f = cvis * d.v.w;
        ax -= f * (vi4.x - d.v.x) * w;
        ay -= f * (vi4.y - d.v.y) * w;
        az -= f * (vi4.z - d.v.z) * w;
      }
    }, c.n, BOUNDS_FLUID_LIST);
    nb = bcount[i];
    for_neighbors_sub<DFSPH_DENSITY_BATCH, Rec<T>>(nb, blist, c.n, i, s, L, [&](int j) { return ld_rec(BR + j); }, [&](const Rec<T> &d) {
      const T rx = xi.x - d.x.x, ry = xi.y - d.x.y, rz = xi.z - d.x.z;
      const T g = KEval<T>::G(rx * rx + ry * ry + rz * rz, c.kc);
      delta += d.x.w * (g * ((vi4.x - d.v.x) * rx + (vi4.y - d.v.y) * ry + (vi4.z - d.v.z) * rz));
    }, c.nbr, BOUNDS_BOUNDARY_LIST);
  }
  delta = sub_sum<L>(delta);
  if (XS) { ax = sub_sum<L>(ax); ay = sub_sum<L>(ay); az = sub_sum<L>(az); }
  if (live && s == 0) {
    T ra;
    if (MODE == PASS_PRESSURE || MODE == PASS_PRESSURE_WARM) {
      ra = rho[i] / c.rho0 + c.dt * delta;
      ra = ra > T(1) ? ra : T(1);
    } else {
      ra = delta > T(0) ? delta : T(0);
      if (nf + nb < 20) ra = T(0);
    }
    rhoAdv[i] = ra;
    T kq;
    if (MODE == PASS_PRESSURE) {
      kq = (ra - T(1)) * alpha[i] * c.invH2;
      e = (double)(c.rho0 * ra - c.rho0);
    } else if (MODE == PASS_DIVERGENCE) {
      kq = ra * alpha[i] * c.invH;
      e = (double)(c.rho0 * ra);
    } else if (MODE == PASS_PRESSURE_WARM) {
      const T kp = kappa_io[i];
      kq = (ra > T(1)) ? T(0.5) * (kp > T(-0.00025) ? kp : T(-0.00025)) * c.invH2 : T(0);
      kappa_io[i] = kq;
      // learned warm start: its features (density error, neighbour count, previous
      // stiffness in pass units, speed)
      if (feat)
        feat[i] = make_float4((float)(ra - T(1)), (float)(nf + nb), (float)(kp * c.invH2),
                              (float)sqrt(ri.v.x * ri.v.x + ri.v.y * ri.v.y + ri.v.z * ri.v.z));
    } else {
      const T kp = kappa_io[i];
      kq = (ra > T(0)) ? T(0.5) * (kp > T(-0.5) ? kp : T(-0.5)) * c.invH : T(0);
      kappa_io[i] = kq;
    }
    Q[i] = V4<T>{ri.x.x, ri.x.y, ri.x.z, kq};
    if (XS) {
      const V4<T> vi = ri.v;
      ax += c.gx; ay += c.gy; az += c.gz;
      R_out[i] = Rec<T>{ri.x, V4<T>{vi.x + c.dt * ax, vi.y + c.dt * ay, vi.z + c.dt * az, vi.w}};
    }
  }
  if (partials) block_partial_sum(e, partials);
}

// Velocity correction with the stiffness k held in Q[.].w (warm start or Jacobi sweep):
// v_i -= dt sum_f (k_i + k_j)(-V grad W) [if |k_i + k_j| > eps];
// v_i += -dt k_i (-psi grad W) over boundary neighbours [if |k_i| > eps].
// ACC = 1 adds k_i to kappa_acc (the solver's running stiffness). v[i].w is kept.
template <class T, int ACC, int L>
static __global__ void __launch_bounds__(PASS_THREADS, pass_min_blocks<T>(DFSPH_VELOCITY_MIN_BLOCKS * 256 / PASS_THREADS)) k_velocity_pass(
    FluidConsts<T> c, const V4<T> *__restrict__ Q, Rec<T> *__restrict__ R, const Rec<T> *__restrict__ BR,
    const int *__restrict__ flist, const int *__restrict__ fcount, const int *__restrict__ blist,
    const int *__restrict__ bcount, T *__restrict__ kappa_acc) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / L, s = t % L;
  const bool live = i < c.n;
  T dvx = T(0), dvy = T(0), dvz = T(0);
  T ki = T(0);
  if (live) {
    const V4<T> qi = Q[i];
    ki = qi.w;
    const T sV = c.dt * c.V;
    for_neighbors_sub<DFSPH_VELOCITY_BATCH, V4<T>>(fcount[i], flist, c.n, i, s, L, [&](int j) { return Q[j]; }, [&](const V4<T> &qj) {
      const T kSum = ki + qj.w;
      if (fabs(kSum) > c.eps) {
        const T rx = qi.x - qj.x, ry = qi.y - qj.y, rz = qi.z - qj.z;
        const T f = sV * kSum * KEval<T>::G(rx * rx + ry * ry + rz * rz, c.kc);
        dvx += f * rx; dvy += f * ry; dvz += f * rz;
      }
    }, c.n, BOUNDS_FLUID_LIST);
    if (fabs(ki) > c.eps) {
      const T sk = c.dt * ki;
      for_neighbors_sub<DFSPH_VELOCITY_BATCH, V4<T>>(bcount[i], blist, c.n, i, s, L, [&](int j) { return BR[j].x; }, [&](const V4<T> &xj) {
        const T rx = qi.x - xj.x, ry = qi.y - xj.y, rz = qi.z - xj.z;
        const T f = sk * xj.w * KEval<T>::G(rx * rx + ry * ry + rz * rz, c.kc);
        dvx += f * rx; dvy += f * ry; dvz += f * rz;
      }, c.nbr, BOUNDS_BOUNDARY_LIST);
    }
  }
  dvx = sub_sum<L>(dvx); dvy = sub_sum<L>(dvy); dvz = sub_sum<L>(dvz);
  if (live && s == 0) {
    if (ACC) kappa_acc[i] += ki;
    V4<T> vi = R[i].v;
    vi.x += dvx; vi.y += dvy; vi.z += dvz;
    R[i].v = vi;
  }
}

// clearAccelerations + XSPH viscosity + v += dt a (TimeStep.cpp:66-81,
// Viscosity_XSPH.cpp:35-110, TimeStepDiffDFSPH.cpp:588-605); also kappaV *= dt
// (end of the divergence solve, :870-880) when scale_kappaV is set.
// v[j].w holds m_j / rho_j.
// ST: Akinci2013 surface tension first (SurfaceTension_Akinci2013.cpp:60-148; it runs before
// the viscosity, Simulation.cpp:618-631): cohesion and curvature over fluid neighbours with
// K_ij = 2 rho0 / (rho_i + rho_j), adhesion over boundary neighbours; N[j] = (n_j, rho_j).
// With visc_b != 0 the boundary term of Viscosity_XSPH::step (:72-82):
// a_i += -(1/h) visc_b (rho0 psi_j / rho_i) (v_i - v_j) W_ij over boundary neighbours (the
// bodies' reaction is summed per sample by k_visc_boundary_force).
template <class T, bool ST, int L>
static __global__ void __launch_bounds__(256, pass_min_blocks<T>(DFSPH_XSPH_MIN_BLOCKS)) k_xsph_advect(FluidConsts<T> c, const Rec<T> *__restrict__ R,
                                                            Rec<T> *__restrict__ R_out, const int *__restrict__ flist,
                                                            const int *__restrict__ fcount, T *__restrict__ kappaV,
                                                            int scale_kappaV, const V4<T> *__restrict__ N,
                                                            const Rec<T> *__restrict__ BR, const int *__restrict__ blist,
                                                            const int *__restrict__ bcount, const T *__restrict__ rho) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / L, s = t % L;
  const bool live = i < c.n;
  T ax = T(0), ay = T(0), az = T(0);
  Rec<T> ri;
  if (live) {
    ri = ld_rec(R + i);
    const V4<T> xi = ri.x, vi = ri.v;
    if (ST) {
      const V4<T> ni = N[i];
      for_neighbors_sub<DFSPH_XSPH_BATCH, Rec<T>>(fcount[i], flist, c.n, i, s, L,
                                                  [&](int j) { return Rec<T>{R[j].x, N[j]}; }, [&](const Rec<T> &d) {
        const V4<T> xj = d.x, nj = d.v;
        const T Kij = T(2) * c.rho0 / (ni.w + nj.w);
        const T rx = xi.x - xj.x, ry = xi.y - xj.y, rz = xi.z - xj.z;
        const T r2 = sqnorm_ref(rx, ry, rz);
        T cx = T(0), cy = T(0), cz = T(0);
        if (r2 > T(1.0e-9)) {
          const T r1 = sqrt(r2);
          const T f = c.st_k * c.m * cohesion_W(r1, r2, c) / r1;
          cx = -f * rx; cy = -f * ry; cz = -f * rz;
        }
        cx -= c.st_k * (ni.x - nj.x); cy -= c.st_k * (ni.y - nj.y); cz -= c.st_k * (ni.z - nj.z);
        ax += Kij * cx; ay += Kij * cy; az += Kij * cz;
      }, c.n, BOUNDS_FLUID_LIST);
      for_neighbors_sub<DFSPH_XSPH_BATCH, V4<T>>(bcount[i], blist, c.n, i, s, L, [&](int j) { return BR[j].x; },
                                                 [&](const V4<T> &xj) {
        const T rx = xi.x - xj.x, ry = xi.y - xj.y, rz = xi.z - xj.z;
        const T r2 = sqnorm_ref(rx, ry, rz);
        if (r2 > T(1.0e-9)) {
          const T r1 = sqrt(r2);
          const T f = c.st_kb * c.rho0 * xj.w * adhesion_W(r1, r2, c) / r1;
          ax -= f * rx; ay -= f * ry; az -= f * rz;
        }
      }, c.nbr, BOUNDS_BOUNDARY_LIST);
    }
    const T cvis = c.invH * c.visc;
    for_neighbors_sub<DFSPH_XSPH_BATCH, Rec<T>>(fcount[i], flist, c.n, i, s, L, [&](int j) { return ld_rec(R + j); },
                                 [&](const Rec<T> &d) {
      const T rx = xi.x - d.x.x, ry = xi.y - d.x.y, rz = xi.z - d.x.z;
      const T w = KEval<T>::W(rx * rx + ry * ry + rz * rz, c.kc);
      const T f = cvis * d.v.w;
      ax -= f * (vi.x - d.v.x) * w;
      ay -= f * (vi.y - d.v.y) * w;
      az -= f * (vi.z - d.v.z) * w;
    }, c.n, BOUNDS_FLUID_LIST);
    if (c.visc_b != T(0)) {
      const T fb = -c.invH * c.visc_b;
      const T rho_i = rho[i];
      for_neighbors_sub<DFSPH_XSPH_BATCH, Rec<T>>(bcount[i], blist, c.n, i, s, L, [&](int j) { return ld_rec(BR + j); },
                                                  [&](const Rec<T> &d) {
        const T rx = xi.x - d.x.x, ry = xi.y - d.x.y, rz = xi.z - d.x.z;
        const T w = KEval<T>::W(rx * rx + ry * ry + rz * rz, c.kc);
        const T f = fb * (c.rho0 * d.x.w / rho_i);
        ax += f * (vi.x - d.v.x) * w;
        ay += f * (vi.y - d.v.y) * w;
        az += f * (vi.z - d.v.z) * w;
      }, c.nbr, BOUNDS_BOUNDARY_LIST);
    }
  }
  ax = sub_sum<L>(ax); ay = sub_sum<L>(ay); az = sub_sum<L>(az);
  if (live && s == 0) {
    const V4<T> vi = ri.v;
    ax += c.gx; ay += c.gy; az += c.gz;
    R_out[i] = Rec<T>{ri.x, V4<T>{vi.x + c.dt * ax, vi.y + c.dt * ay, vi.z + c.dt * az, vi.w}};
    if (scale_kappaV) kappaV[i] *= c.dt;
  }
}

// Surface-tension normals (SurfaceTension_Akinci2013.cpp:28-58): n_i = h sum_j (m_j/rho_j)
// grad W_ij over fluid neighbours; N[i] = (n_i, rho_i) for the force part of the XSPH pass.
template <class T>
static __global__ void __launch_bounds__(256) k_normals(FluidConsts<T> c, const Rec<T> *__restrict__ R,
                                                        const int *__restrict__ flist, const int *__restrict__ fcount,
                                                        const T *__restrict__ rho, V4<T> *__restrict__ N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const V4<T> xi = R[i].x;
  T nx = T(0), ny = T(0), nz = T(0);
  for_neighbors_sub<DFSPH_XSPH_BATCH, Rec<T>>(fcount[i], flist, c.n, i, 0, 1, [&](int j) { return ld_rec(R + j); },
                                              [&](const Rec<T> &d) {
    const T rx = xi.x - d.x.x, ry = xi.y - d.x.y, rz = xi.z - d.x.z;
    const T g = d.v.w * KEval<T>::G(rx * rx + ry * ry + rz * rz, c.kc);
    nx += g * rx; ny += g * ry; nz += g * rz;
  }, c.n, BOUNDS_FLUID_LIST);
  N[i] = V4<T>{c.kc.h * nx, c.kc.h * ny, c.kc.h * nz, rho[i]};
}

// x += h v with the step's initial size h (TimeStepDiffDFSPH.cpp:613-635); kappa *= dt^2
// with the current size (:752-767) when requested.
// kappaV *= h_div (the end of the divergence solve, :870-880) when the XSPH pass was
// fused into the divergence solve's last density pass (kappaV is next read by the next
// step's warm start).
template <class T>
static __global__ void k_integrate(FluidConsts<T> c, Rec<T> *__restrict__ R, T *__restrict__ kappa, int scale_kappa,
                                   T h, T *__restrict__ kappaV, T h_div) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  if (kappaV) kappaV[i] *= h_div;
  Rec<T> r = R[i];
  r.x.x += h * r.v.x; r.x.y += h * r.v.y; r.x.z += h * r.v.z;
  R[i].x = r.x;
  if (scale_kappa) kappa[i] *= c.dt * c.dt;
}

// Final residual sum (one block of FINAL_SUM_THREADS threads, fixed order); also publishes
// the device error word next to it in mapped host memory, so one stream synchronisation
// reads both. Thread t adds partials t, t + 1024, t + 2048, ... in index order, with eight
// loads in flight at a time (one memory latency per 8192 partials instead of one per
// partial); then a shuffle tree per warp and the 32 warp sums in warp order.
constexpr int FINAL_SUM_THREADS = 1024;
static __global__ void __launch_bounds__(FINAL_SUM_THREADS) k_final_sum(int nparts, const double *__restrict__ partials,
                                                                        double scale, double *__restrict__ out,
                                                                        double *__restrict__ out_host,
                                                                        const int *__restrict__ err) {
  __shared__ double ws[FINAL_SUM_THREADS / 32];
  double s = 0.0;
  for (int k0 = threadIdx.x; k0 < nparts; k0 += 8 * FINAL_SUM_THREADS) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int k = k0 + u * FINAL_SUM_THREADS;
      v[u] = k < nparts ? partials[k] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) s += v[u];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < FINAL_SUM_THREADS / 32; w++) t += ws[w];
    *out = t * scale;
    if (out_host) {
      out_host[0] = t * scale;
      out_host[1] = (double)(*err);
    }
  }
}

}  // namespace dfsph
