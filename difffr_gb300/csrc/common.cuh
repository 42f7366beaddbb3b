// common.cuh — device-side types and math shared by the DFSPH kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef DFSPH_MAX_BODIES_DEV
#define DFSPH_MAX_BODIES_DEV 16
#endif

namespace dfsph {

// Device error word bits (read by the host after each step; no trap, no assert).
enum : int {
  ERR_FLUID_LIST_OVERFLOW = 1 << 0,
  ERR_BOUNDARY_LIST_OVERFLOW = 1 << 1,
  ERR_BF_LIST_OVERFLOW = 1 << 2,
  ERR_NONFINITE_POSITION = 1 << 3,
  ERR_MLP_TIMEOUT = 1 << 4,
};

// Bounds-checked build (-DDFSPH_BOUNDS_CHECK, libdfsph_boundscheck.so): every neighbour index
// read from a list, and every cell-row range, is checked against its array before use. A bad
// index sets a bit of this translation unit's g_dfsph_bounds_err and is replaced by index 0,
// so the access stays in bounds; the engine reads the word after each step and reports it as
// a device error. In the regular build the checks compile to nothing.
enum : int {
  BOUNDS_FLUID_LIST = 1 << 0,     // fluid neighbour index outside [0, n)
  BOUNDS_BOUNDARY_LIST = 1 << 1,  // boundary neighbour index outside [0, boundary samples)
  BOUNDS_SAMPLE_LIST = 1 << 2,    // a dynamic sample's fluid neighbour outside [0, n)
  BOUNDS_CELL_RANGE = 1 << 3,     // a cell row's [start, end) outside [0, points]
};
#ifdef DFSPH_BOUNDS_CHECK
static __device__ int g_dfsph_bounds_err;
__device__ __forceinline__ int checked_index(int j, int lim, int bit) {
  if ((unsigned)j >= (unsigned)lim) {
    atomicOr(&g_dfsph_bounds_err, bit);
    return 0;
  }
  return j;
}
#define DF_INDEX(j, lim, bit) ::dfsph::checked_index((j), (lim), (bit))
#else
#define DF_INDEX(j, lim, bit) (j)
#endif

template <class T>
struct alignas(4 * sizeof(T)) V4 {
  T x, y, z, w;
};

template <class T>
struct V3 {
  T x, y, z;
};

template <class T> __host__ __device__ __forceinline__ V3<T> mk3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> __device__ __forceinline__ V3<T> xyz(const V4<T> &a) { return V3<T>{a.x, a.y, a.z}; }
template <class T> __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __device__ __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> __device__ __forceinline__ V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> __device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Products without FMA contraction: the neighbour predicate must give the same
// answer as the CPU oracle's ((dx*dx + dy*dy) + dz*dz) < h*h.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <class T> __device__ __forceinline__ T dist2_rn(T dx, T dy, T dz) {
  return add_rn(add_rn(mul_rn(dx, dx), mul_rn(dy, dy)), mul_rn(dz, dz));
}

// Cubic spline kernel with support h: W, gradW, gradGradW of the reference's
// CubicKernel (SPlisHSPlasH/SPHKernels.h:16-176). k = 8/(pi h^3), l = 48/(pi h^3).
template <class T>
struct Cubic {
  T h, k, l, w0, invh;
};

template <class T> __device__ __forceinline__ T cubic_W(T rl, const Cubic<T> &c) {
  const T q = rl / c.h;
  T res = T(0);
  if (q <= T(1)) {
    if (q <= T(0.5)) {
      const T q2 = q * q, q3 = q2 * q;
      res = c.k * (T(6) * q3 - T(6) * q2 + T(1));
    } else {
      const T f = T(1) - q;
      res = c.k * (T(2) * (f * f * f));
    }
  }
  return res;
}

// gradW(r) = s * (r * inv) with inv = 1/(|r| h); returns the vector.
template <class T> __device__ __forceinline__ V3<T> cubic_gradW(V3<T> r, T rl, const Cubic<T> &c) {
  const T q = rl / c.h;
  if ((rl > T(1.0e-5)) && (q <= T(1))) {
    const T inv = T(1) / (rl * c.h);
    T s;
    if (q <= T(0.5)) s = c.l * q * (T(3) * q - T(2));
    else { const T f = T(1) - q; s = c.l * (-f * f); }
    return {s * (r.x * inv), s * (r.y * inv), s * (r.z * inv)};
  }
  return {T(0), T(0), T(0)};
}

// Kernel terms from the squared distance d2 of a neighbour pair (d2 < h^2):
//   KEval<T>::W(d2) = W(|r|),  KEval<T>::G(d2) = g with gradW(r) = g r.
// double: IEEE sqrt and divisions in the reference's order (SPHKernels.h:37-102).
// float:  one rsqrt and multiplications by 1/h; differs from the IEEE form by a few ulp.
template <class T> struct KEval;
template <> struct KEval<double> {
  static __device__ __forceinline__ double W(double d2, const Cubic<double> &c) { return cubic_W(sqrt(d2), c); }
  static __device__ __forceinline__ double G(double d2, const Cubic<double> &c) {
    const double rl = sqrt(d2);
    const double q = rl / c.h;
    if ((rl > 1.0e-5) && (q <= 1.0)) {
      const double inv = 1.0 / (rl * c.h);
      double s;
      if (q <= 0.5) s = c.l * q * (3.0 * q - 2.0);
      else { const double f = 1.0 - q; s = c.l * (-f * f); }
      return s * inv;
    }
    return 0.0;
  }
};
template <> struct KEval<float> {
  static __device__ __forceinline__ float W(float d2, const Cubic<float> &c) {
    const float rl = d2 * rsqrtf(d2);  // d2 = 0 gives NaN -> q <= 1 false; handled below
    const float q = d2 > 0.f ? rl * c.invh : 0.f;
    float res = 0.f;
    if (q <= 1.f) {
      if (q <= 0.5f) { const float q2 = q * q; res = c.k * (6.f * q2 * q - 6.f * q2 + 1.f); }
      else { const float f = 1.f - q; res = c.k * (2.f * (f * f * f)); }
    }
    return res;
  }
  static __device__ __forceinline__ float G(float d2, const Cubic<float> &c) {
    const float rinv = rsqrtf(d2);
    const float rl = d2 * rinv;
    const float q = rl * c.invh;
    if ((rl > 1.0e-5f) && (q <= 1.f)) {
      float s;
      if (q <= 0.5f) s = c.l * q * (3.f * q - 2.f);
      else { const float f = 1.f - q; s = c.l * (-f * f); }
      return s * rinv * c.invh;
    }
    return 0.f;
  }
};

// Symmetric 3x3 Hessian stored as xx, xy, xz, yy, yz, zz.
template <class T> struct Sym3 { T xx, xy, xz, yy, yz, zz; };

template <class T> __device__ __forceinline__ Sym3<T> cubic_gradGradW(V3<T> r, T rl, const Cubic<T> &c) {
  const T q = rl / c.h;
  Sym3<T> H{T(0), T(0), T(0), T(0), T(0), T(0)};
  if ((rl > T(1.0e-5)) && (q <= T(1))) {
    const T inv = T(1) / (rl * c.h);
    const V3<T> g = {r.x * inv, r.y * inv, r.z * inv};   // grad q
    const T ir2 = T(1) / (rl * rl);
    T a, b;
    if (q <= T(0.5)) { a = c.l * q * (T(3) * q - T(2)); b = c.l * (T(6) * q - T(2)); }
    else { const T f = T(1) - q; a = c.l * (-f * f); b = c.l * T(2) * f; }
    // a * inv * (I - r r^T / |r|^2) + b * g g^T
    const T ai = a * inv;
    H.xx = ai * (T(1) - r.x * r.x * ir2) + b * g.x * g.x;
    H.yy = ai * (T(1) - r.y * r.y * ir2) + b * g.y * g.y;
    H.zz = ai * (T(1) - r.z * r.z * ir2) + b * g.z * g.z;
    H.xy = ai * (-r.x * r.y * ir2) + b * g.x * g.y;
    H.xz = ai * (-r.x * r.z * ir2) + b * g.x * g.z;
    H.yz = ai * (-r.y * r.z * ir2) + b * g.y * g.z;
  }
  return H;
}

template <class T> __device__ __forceinline__ V3<T> symmul(const Sym3<T> &H, V3<T> v) {
  return {H.xx * v.x + H.xy * v.y + H.xz * v.z, H.xy * v.x + H.yy * v.y + H.yz * v.z,
          H.xz * v.x + H.yz * v.y + H.zz * v.z};
}

// Uniform grid over the simulation domain. Cell size is h * (1 + 1e-4) so that a
// rounding error in the cell coordinate can never hide a neighbour at distance < h;
// positions outside the box clamp to the border cells (still a conservative search).
template <class T>
struct Grid {
  T ox, oy, oz, inv_cell;
  int nx, ny, nz;
};

template <class T> __device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <class T> __device__ __forceinline__ void grid_cell(const Grid<T> &g, T x, T y, T z, int &cx, int &cy, int &cz) {
  // floor in the scalar type; NaN maps to cell 0 (the caller flags it)
  T fx = floor((x - g.ox) * g.inv_cell), fy = floor((y - g.oy) * g.inv_cell), fz = floor((z - g.oz) * g.inv_cell);
  fx = fx < T(0) ? T(0) : (fx > T(g.nx - 1) ? T(g.nx - 1) : fx);
  fy = fy < T(0) ? T(0) : (fy > T(g.ny - 1) ? T(g.ny - 1) : fy);
  fz = fz < T(0) ? T(0) : (fz > T(g.nz - 1) ? T(g.nz - 1) : fz);
  cx = (fx == fx) ? (int)fx : 0;
  cy = (fy == fy) ? (int)fy : 0;
  cz = (fz == fz) ? (int)fz : 0;
}

template <class T> __device__ __forceinline__ int grid_key(const Grid<T> &g, int cx, int cy, int cz) {
  return (cz * g.ny + cy) * g.nx + cx;
}

}  // namespace dfsph
