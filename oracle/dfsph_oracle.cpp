// dfsph_oracle.cpp — CPU ORACLE (test infrastructure only).
//
// A line-by-line restatement, in plain C++17 + OpenMP, of DiffFR's DiffDFSPH time
// step with Akinci2012 rigid coupling and the forward-mode rigid gradient chain.
// It exists to check the GPU library (tests, the smoke check, and the CPU-baseline leg
// of the benchmark); nothing in the product links or calls it.
//
// Parity status: partially pinned. The reference cannot be built in full without
// three git-fetched dependencies (CompactNSearch, GenericParameters, Discregrid), so
// this file restates the reference's arithmetic. The cubic kernel (W, gradW,
// gradGradW) and the quaternion Jacobians used below are pinned bit-for-bit against
// the reference's own SPHKernels.h / GradientUtils.cpp compiled from source (golden
// vectors under tests/golden/, generator beside them). Step-level arithmetic is
// checked by finite differences and invariants, not by a reference run.
//
// Citations are paths relative to the DiffFR repository root.
//
// Templates: F = fluid scalar, R = rigid/chain scalar.
//   <float,float>   the reference's default float build
//   <float,double>  the GPU library's split (FP32 fluid, FP64 rigid)
//   <double,double> the reference's USE_DOUBLE build

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <memory>
#include <omp.h>
#include "../include/dfsph.h"

namespace orc {

// ---------------------------------------------------------------- small linear algebra
template <class T, int RR, int CC>
struct Mat {
  T a[RR][CC];
  static Mat zero() { Mat m; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) m.a[i][j] = T(0); return m; }
  static Mat eye() { Mat m = zero(); for (int i = 0; i < RR && i < CC; i++) m.a[i][i] = T(1); return m; }
  T &operator()(int i, int j) { return a[i][j]; }
  const T &operator()(int i, int j) const { return a[i][j]; }
  T &operator[](int i) { return a[i][0]; }
  const T &operator[](int i) const { return a[i][0]; }
  Mat &operator+=(const Mat &o) { for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) a[i][j] += o.a[i][j]; return *this; }
  Mat &operator-=(const Mat &o) { for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) a[i][j] -= o.a[i][j]; return *this; }
  Mat operator+(const Mat &o) const { Mat m = *this; m += o; return m; }
  Mat operator-(const Mat &o) const { Mat m = *this; m -= o; return m; }
  Mat operator-() const { Mat m; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) m.a[i][j] = -a[i][j]; return m; }
  Mat<T, CC, RR> T_() const { Mat<T, CC, RR> m; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) m.a[j][i] = a[i][j]; return m; }
  template <class U> Mat<U, RR, CC> cast() const { Mat<U, RR, CC> m; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) m.a[i][j] = U(a[i][j]); return m; }
};
template <class T, int RR, int CC> Mat<T, RR, CC> operator*(T s, const Mat<T, RR, CC> &m) { Mat<T, RR, CC> r; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) r.a[i][j] = s * m.a[i][j]; return r; }
template <class T, int RR, int CC> Mat<T, RR, CC> operator*(const Mat<T, RR, CC> &m, T s) { Mat<T, RR, CC> r; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) r.a[i][j] = m.a[i][j] * s; return r; }
template <class T, int RR, int CC> Mat<T, RR, CC> operator/(const Mat<T, RR, CC> &m, T s) { Mat<T, RR, CC> r; for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) r.a[i][j] = m.a[i][j] / s; return r; }
// Sums the terms p[0..n) with Eigen's unrolled reduction order (recursive halving:
// x0 + (x1 + x2) for 3 terms, (x0 + x1) + (x2 + x3) for 4), so that dot products,
// norms and small matrix products round exactly as the reference's Eigen code does.
// Float vectors of 3 or 4 are shorter than or equal to one 4-wide packet and reduce by
// recursive halving; double reductions run over 2-wide packets, ((x0 + x1) + x2) for 3
// terms and ((x0 + x2) + (x1 + x3)) for 4.
template <class T> inline T redux(const T *p, int n) {
  if (n == 1) return p[0];
  const int half = n / 2;
  return redux(p, half) + redux(p + half, n - half);
}
template <> inline double redux<double>(const double *p, int n) {
  if (n == 1) return p[0];
  if (n == 2) return p[0] + p[1];
  if (n == 3) return (p[0] + p[1]) + p[2];
  if (n == 4) return (p[0] + p[2]) + (p[1] + p[3]);
  double s = p[0];
  for (int k = 1; k < n; k++) s += p[k];
  return s;
}
template <class T, int RR, int K, int CC>
Mat<T, RR, CC> operator*(const Mat<T, RR, K> &x, const Mat<T, K, CC> &y) {
  Mat<T, RR, CC> r;
  for (int i = 0; i < RR; i++)
    for (int j = 0; j < CC; j++) {
      T t[K];
      for (int k = 0; k < K; k++) t[k] = x.a[i][k] * y.a[k][j];
      r.a[i][j] = redux(t, K);
    }
  return r;
}

template <class T> using V3 = Mat<T, 3, 1>;
template <class T> using M3 = Mat<T, 3, 3>;
template <class T> using M34 = Mat<T, 3, 4>;
template <class T> using M43 = Mat<T, 4, 3>;
template <class T> using M4 = Mat<T, 4, 4>;
template <class T> using V4 = Mat<T, 4, 1>;

template <class T> V3<T> v3(T x, T y, T z) { V3<T> v; v[0] = x; v[1] = y; v[2] = z; return v; }
template <class T> T dot(const V3<T> &a, const V3<T> &b) { const T t[3] = {a[0] * b[0], a[1] * b[1], a[2] * b[2]}; return redux(t, 3); }
template <class T> T sqnorm(const V3<T> &a) { return dot(a, a); }
template <class T> T norm(const V3<T> &a) { return std::sqrt(sqnorm(a)); }
template <class T> V3<T> cross(const V3<T> &a, const V3<T> &b) {
  return v3<T>(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
template <class T> M3<T> outer(const V3<T> &a, const V3<T> &b) { return a * b.T_(); }
// GradientUtils.cpp:4-6
template <class T> M3<T> skew(const V3<T> &v) {
  M3<T> m;
  m(0, 0) = 0; m(0, 1) = -v[2]; m(0, 2) = v[1];
  m(1, 0) = v[2]; m(1, 1) = 0; m(1, 2) = -v[0];
  m(2, 0) = -v[1]; m(2, 1) = v[0]; m(2, 2) = 0;
  return m;
}
template <class T> M3<T> inverse3(const M3<T> &m) {
  const T c00 = m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1);
  const T c01 = m(1, 2) * m(2, 0) - m(1, 0) * m(2, 2);
  const T c02 = m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0);
  const T det = m(0, 0) * c00 + m(0, 1) * c01 + m(0, 2) * c02;
  const T id = T(1) / det;
  M3<T> r;
  r(0, 0) = c00 * id; r(0, 1) = (m(0, 2) * m(2, 1) - m(0, 1) * m(2, 2)) * id; r(0, 2) = (m(0, 1) * m(1, 2) - m(0, 2) * m(1, 1)) * id;
  r(1, 0) = c01 * id; r(1, 1) = (m(0, 0) * m(2, 2) - m(0, 2) * m(2, 0)) * id; r(1, 2) = (m(1, 0) * m(0, 2) - m(0, 0) * m(1, 2)) * id;
  r(2, 0) = c02 * id; r(2, 1) = (m(2, 0) * m(0, 1) - m(0, 0) * m(2, 1)) * id; r(2, 2) = (m(0, 0) * m(1, 1) - m(1, 0) * m(0, 1)) * id;
  return r;
}

// Quaternion (w, x, y, z), Hamilton product.
template <class T> struct Quat {
  T w, x, y, z;
  Quat operator*(const Quat &b) const {
    return {w * b.w - x * b.x - y * b.y - z * b.z, w * b.x + x * b.w + y * b.z - z * b.y,
            w * b.y + y * b.w + z * b.x - x * b.z, w * b.z + z * b.w + x * b.y - y * b.x};
  }
  T norm() const { return std::sqrt(w * w + x * x + y * y + z * z); }
  void normalize() { T n = norm(); w /= n; x /= n; y /= n; z /= n; }
  M3<T> R() const {  // rotation matrix of a unit quaternion
    const T tx = T(2) * x, ty = T(2) * y, tz = T(2) * z;
    const T twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
    const T tyy = ty * y, tyz = tz * y, tzz = tz * z;
    M3<T> m;
    m(0, 0) = T(1) - (tyy + tzz); m(0, 1) = txy - twz; m(0, 2) = txz + twy;
    m(1, 0) = txy + twz; m(1, 1) = T(1) - (txx + tzz); m(1, 2) = tyz - twx;
    m(2, 0) = txz - twy; m(2, 1) = tyz + twx; m(2, 2) = T(1) - (txx + tyy);
    return m;
  }
  V3<T> rotate(const V3<T> &v) const {  // q v q^-1 for a unit quaternion
    V3<T> u = v3(x, y, z);
    V3<T> uv = cross(u, v);
    uv += uv;
    return v + w * uv + cross(u, uv);
  }
  V4<T> vec4() const { V4<T> r; r[0] = w; r[1] = x; r[2] = y; r[3] = z; return r; }
};

// GradientUtils.cpp:9-20  d(R(q) p)/dq, columns (w, x, y, z)
template <class T> M34<T> grad_Rqp_to_q(const Quat<T> &q, const V3<T> &p) {
  V3<T> qv = v3(q.x, q.y, q.z);
  V3<T> t1 = T(2) * (q.w * p - cross(p, qv));
  M3<T> t2 = T(2) * (dot(qv, p) * M3<T>::eye() + outer(qv, p) - outer(p, qv) - q.w * skew(p));
  M34<T> r;
  for (int i = 0; i < 3; i++) { r(i, 0) = t1[i]; for (int j = 0; j < 3; j++) r(i, j + 1) = t2(i, j); }
  return r;
}
// GradientUtils.cpp:23-35  d(R(q)^T p)/dq
template <class T> M34<T> grad_RqTp_to_q(const Quat<T> &q, const V3<T> &p) {
  V3<T> qv = v3(q.x, q.y, q.z);
  V3<T> t1 = T(2) * (q.w * p + cross(p, qv));
  M3<T> t2 = T(2) * (dot(qv, p) * M3<T>::eye() + outer(qv, p) - outer(p, qv) + q.w * skew(p));
  M34<T> r;
  for (int i = 0; i < 3; i++) { r(i, 0) = t1[i]; for (int j = 0; j < 3; j++) r(i, j + 1) = t2(i, j); }
  return r;
}
// GradientUtils.cpp:37-44  d(p * q)/dq
template <class T> M4<T> grad_p_q_product_to_q(const Quat<T> &p) {
  M4<T> m;
  T r[4][4] = {{p.w, -p.x, -p.y, -p.z}, {p.x, p.w, -p.z, p.y}, {p.y, p.z, p.w, -p.x}, {p.z, -p.y, p.x, p.w}};
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) m(i, j) = r[i][j];
  return m;
}
// GradientUtils.cpp:46-53  d((0,omega) * q)/domega
template <class T> M43<T> grad_omega_q_product_to_omega(const Quat<T> &q) {
  M43<T> m;
  T r[4][3] = {{-q.x, -q.y, -q.z}, {q.w, q.z, -q.y}, {-q.z, q.w, q.x}, {q.y, -q.x, q.w}};
  for (int i = 0; i < 4; i++) for (int j = 0; j < 3; j++) m(i, j) = r[i][j];
  return m;
}

// ---------------------------------------------------------------- cubic spline kernel
// SPlisHSPlasH/SPHKernels.h:16-176 (CubicKernel)
template <class T> struct Cubic {
  T radius, k, l, w0;
  void set(T h) {
    radius = h;
    const T pi = static_cast<T>(M_PI);
    const T h3 = radius * radius * radius;
    k = static_cast<T>(8.0) / (pi * h3);
    l = static_cast<T>(48.0) / (pi * h3);
    w0 = W(T(0));
  }
  T W(T r) const {  // SPHKernels.h:37-55
    T res = 0;
    const T q = r / radius;
    if (q <= T(1)) {
      if (q <= T(0.5)) {
        const T q2 = q * q, q3 = q2 * q;
        res = k * (T(6) * q3 - T(6) * q2 + T(1));
      } else {
        res = k * (T(2) * std::pow(T(1) - q, T(3)));
      }
    }
    return res;
  }
  T W(const V3<T> &r) const { return W(norm(r)); }
  V3<T> gradW(const V3<T> &r) const {  // SPHKernels.h:80-102
    V3<T> res;
    const T rl = norm(r);
    const T q = rl / radius;
    if ((rl > T(1.0e-5)) && (q <= T(1))) {
      const V3<T> gradq = r * (T(1) / (rl * radius));
      if (q <= T(0.5)) res = l * q * (T(3) * q - T(2)) * gradq;
      else { const T f = T(1) - q; res = l * (-f * f) * gradq; }
    } else res = V3<T>::zero();
    return res;
  }
  M3<T> gradGradW(const V3<T> &r) const {  // SPHKernels.h:123-150
    M3<T> res;
    const T rl = norm(r);
    const T q = rl / radius;
    if ((rl > T(1.0e-5)) && (q <= T(1))) {
      const V3<T> gradq = r * (T(1) / (rl * radius));
      const M3<T> ggq = (T(1) / (rl * radius)) * (M3<T>::eye() - outer(r, r) / (rl * rl));
      if (q <= T(0.5)) res = l * q * (T(3) * q - T(2)) * ggq + outer(V3<T>(l * (T(6) * q - T(2)) * gradq), gradq);
      else { const T f = T(1) - q; res = l * (-f * f) * ggq + outer(V3<T>(l * T(2) * f * gradq), gradq); }
    } else res = M3<T>::zero();
    return res;
  }
};

// ---------------------------------------------------------------- surface-tension kernels
// SPlisHSPlasH/SPHKernels.h:437-506 (CohesionKernel) and :508-559 (AdhesionKernel), both
// with the support radius h; the mixed float/double comparisons against 0.5 * radius are
// kept as in the reference.
template <class T> struct CohesionK {
  T radius, k, c;
  void set(T h) {
    radius = h;
    const T pi = static_cast<T>(M_PI);
    k = static_cast<T>(32.0) / (pi * std::pow(radius, static_cast<T>(9.0)));
    c = std::pow(radius, static_cast<T>(6.0)) / static_cast<T>(64.0);
  }
  T W(const V3<T> &r) const {
    T res = 0;
    const T r2 = dot(r, r);
    if (r2 <= radius * radius) {
      const T r1 = std::sqrt(r2);
      const T r3 = r2 * r1;
      if (r1 > 0.5 * radius) res = k * std::pow(radius - r1, static_cast<T>(3.0)) * r3;
      else res = k * static_cast<T>(2.0) * std::pow(radius - r1, static_cast<T>(3.0)) * r3 - c;
    }
    return res;
  }
};
template <class T> struct AdhesionK {
  T radius, k;
  void set(T h) {
    radius = h;
    k = static_cast<T>(0.007) / std::pow(radius, static_cast<T>(3.25));
  }
  T W(const V3<T> &r) const {
    T res = 0;
    const T r2 = dot(r, r);
    if (r2 <= radius * radius) {
      const T rl = std::sqrt(r2);
      if (rl > 0.5 * radius)
        res = k * std::pow(-static_cast<T>(4.0) * r2 / radius + static_cast<T>(6.0) * rl - static_cast<T>(2.0) * radius,
                           static_cast<T>(0.25));
    }
    return res;
  }
};

// ---------------------------------------------------------------- neighbour search
// Fixed-radius search with the predicate |xi - xj|^2 < h^2, evaluated as
// ((dx*dx + dy*dy) + dz*dz) < h*h in the fluid scalar type. Rows are sorted ascending.
// (Stands in for CompactNSearch, Simulation.cpp:743-748; see the header note.)
template <class F>
void neighbor_search(const std::vector<V3<F>> &q, const std::vector<V3<F>> &d, F h, bool same_set,
                     std::vector<int64_t> &start, std::vector<int32_t> &idx,
                     const std::vector<char> *query_mask = nullptr) {
  const int64_t nq = (int64_t)q.size(), nd = (int64_t)d.size();
  start.assign(nq + 1, 0);
  idx.clear();
  if (nq == 0 || nd == 0) return;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (const auto &p : d) for (int c = 0; c < 3; c++) { lo[c] = std::min(lo[c], (double)p[c]); hi[c] = std::max(hi[c], (double)p[c]); }
  int64_t dim[3];
  for (int c = 0; c < 3; c++) dim[c] = std::min<int64_t>(std::max<int64_t>((int64_t)std::floor((hi[c] - lo[c]) / (double)h) + 1, 1), 1024);
  auto cell = [&](const V3<F> &p, int64_t *cc) {
    for (int c = 0; c < 3; c++) {
      int64_t v = (int64_t)std::floor(((double)p[c] - lo[c]) / (double)h);
      cc[c] = std::min<int64_t>(std::max<int64_t>(v, 0), dim[c] - 1);
    }
  };
  const int64_t ncell = dim[0] * dim[1] * dim[2];
  std::vector<int64_t> cstart(ncell + 1, 0);
  std::vector<int64_t> key(nd);
  for (int64_t j = 0; j < nd; j++) { int64_t cc[3]; cell(d[j], cc); key[j] = (cc[2] * dim[1] + cc[1]) * dim[0] + cc[0]; cstart[key[j] + 1]++; }
  for (int64_t c = 0; c < ncell; c++) cstart[c + 1] += cstart[c];
  std::vector<int32_t> sorted(nd);
  { std::vector<int64_t> fill(cstart.begin(), cstart.end() - 1); for (int64_t j = 0; j < nd; j++) sorted[fill[key[j]]++] = (int32_t)j; }
  const F h2 = h * h;
  std::vector<std::vector<int32_t>> rows(nq);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < nq; i++) {
    if (query_mask && !(*query_mask)[i]) continue;
    int64_t cc[3]; cell(q[i], cc);
    // q may lie outside d's box: clamp the searched range conservatively.
    auto &row = rows[i];
    for (int64_t z = std::max<int64_t>(cc[2] - 1, 0); z <= std::min<int64_t>(cc[2] + 1, dim[2] - 1); z++)
      for (int64_t y = std::max<int64_t>(cc[1] - 1, 0); y <= std::min<int64_t>(cc[1] + 1, dim[1] - 1); y++)
        for (int64_t x = std::max<int64_t>(cc[0] - 1, 0); x <= std::min<int64_t>(cc[0] + 1, dim[0] - 1); x++) {
          int64_t c = (z * dim[1] + y) * dim[0] + x;
          for (int64_t s = cstart[c]; s < cstart[c + 1]; s++) {
            int32_t j = sorted[s];
            if (same_set && j == i) continue;
            const F dx = q[i][0] - d[j][0], dy = q[i][1] - d[j][1], dz = q[i][2] - d[j][2];
            const F d2 = (dx * dx + dy * dy) + dz * dz;
            if (d2 < h2) row.push_back(j);
          }
        }
    std::sort(row.begin(), row.end());
  }
  for (int64_t i = 0; i < nq; i++) start[i + 1] = start[i] + (int64_t)rows[i].size();
  idx.resize(start[nq]);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nq; i++) std::copy(rows[i].begin(), rows[i].end(), idx.begin() + start[i]);
}

// ---------------------------------------------------------------- simulation
struct Base {
  virtual ~Base() {}
  virtual int step(int n, dfsph_step_stats *st) = 0;
  virtual int copy_field(int f, double *dst) = 0;
  virtual int set_field(int f, const double *src) = 0;
  virtual int rigid_state(int b, double *x, double *q, double *v, double *w) = 0;
  virtual int rigid_force(int b, double *F, double *T) = 0;
  virtual int rigid_mass(int b, double *m, double *I) = 0;
  virtual int rigid_grad(int b, double *out) = 0;
  virtual int net_jac(int b, double *out) = 0;
  virtual int set_init(int b, const double *v, const double *w) = 0;
  virtual int set_velocity(int b, const double *v, const double *w) = 0;
  virtual int set_rigid_state(int b, const double *x, const double *q, const double *v, const double *w) = 0;
  virtual int set_time(double t, int64_t step_count) = 0;
  virtual int neighbors(int which, int64_t *start, int32_t *idx, int64_t *total) = 0;
  virtual int reset() = 0;
  virtual int reset_gradient() = 0;
  virtual int counts(int64_t *nf, int64_t *nb) = 0;
  virtual double time() = 0;
  virtual int mgr_grad(int b, int b2, double *out) = 0;
  virtual int mgr_jac(int b, int b2, double *out) = 0;
  virtual int contact_count(int64_t *nc, int64_t *na) = 0;
};

template <class F, class R>
struct Sim : Base {
  using V3F = V3<F>; using M3F = M3<F>; using M34F = M34<F>;
  using V3R = V3<R>; using M3R = M3<R>; using M34R = M34<R>; using M43R = M43<R>; using QR = Quat<R>;

  dfsph_params P;
  F r, h, rho0, Vf, mf, visc, dt, invH, invH2, eps;
  V3F grav;
  Cubic<F> K;
  CohesionK<F> KC;
  AdhesionK<F> KA;
  int64_t nf = 0, nbp = 0;
  std::vector<V3F> x, v, a, x_init, v_init;
  std::vector<V3F> normals;  // surface-tension normals (SurfaceTension_Akinci2013.cpp:28-58)
  std::vector<F> rho, factor, kappa, kappaV, rhoAdv;
  std::vector<V3F> sumgrad;
  std::vector<V3F> bx, bv, bx0;
  std::vector<F> psi;
  std::vector<int> bbody;

  struct Body {
    bool dyn = false, anim = false, anim0 = false;
    int64_t start = 0, count = 0;
    R mass = 0, invMass = 0;
    M3R I0, I, Iinv;
    V3R x, v, w, x0;
    QR q, q0;
    V3R initV, initW, targetX;
    std::vector<V3R> fth, tth, fbak, tbak;  // per-thread force/torque buckets (BoundaryModel.h:25-28)
    std::vector<M3R> gFv, gFx, gFw, gTw, gTv, gTx;  // per-particle accumulators (BoundaryModel_Akinci2012.h:42-50)
    std::vector<M34R> gFq, gTq;
    M3R nFv, nFx, nFw, nTw, nTv, nTx;  // per-step nets
    M34R nFq, nTq;
    M3R Gx_v, Gx_w, Gv_v, Gv_w, Gw_v, Gw_w;  // chain state
    M43R Gq_v, Gq_w, partial_qn_w;
  };
  std::vector<Body> bodies;
  // RigidContactSolver (InterlinkedSPH/RigidContactSolver.h:140-224): per boundary sample rest
  // volume and rest density from its own body, the contact kernel with the contact support
  // radius, and the last step's contact counts
  Cubic<R> KCt, KHr;
  std::vector<R> cvol0, cdens0;
  int64_t n_contact = 0, n_active = 0;
  // RigidBodyGradientManager (RigidBodyGradientManager.h:20-93): Jacobian blocks [R][RR]
  // (the contact solver's of this step in mgrMc) and the chain state [R][RR]
  struct MgrBlk { M3R Fv, Fx, Fw, Tw, Tv, Tx; M34R Fq, Tq; };
  struct MgrState { M3R Gx_v, Gx_w, Gv_v, Gv_w, Gw_v, Gw_w; M43R Gq_v, Gq_w; };
  std::vector<MgrBlk> mgrM, mgrMc;
  std::vector<MgrState> mgrS;
  std::vector<M3R> mFv0, mFw0, mTv0, mTw0;  // grad_net_{force,torque}_to_{v0,omega0}[R][RR]
  std::vector<int64_t> ffS, fbS, bfS;
  std::vector<int32_t> ff, fb, bf;
  R t = 0;
  int64_t step_count = 0;
  int iters = 0, itersV = 0;
  double lastErr = 0, lastErrV = 0;
  bool finished = false;
  int nthreads = 1;

  explicit Sim(const dfsph_scene *sc) {
    P = sc->params;
    r = (F)P.particle_radius;
    h = F(4) * r;  // Simulation.cpp:385
    K.set(h);
    KC.set(h);
    KA.set(h);
    rho0 = (F)P.density0;
    const F diam = F(2) * r;
    Vf = F(0.8) * diam * diam * diam;  // FluidModel.cpp:255-272
    mf = Vf * rho0;
    visc = (F)P.viscosity;
    set_dt((F)P.time_step);
    eps = F(1.0e-5);  // TimeStepDiffDFSPH.h:26
    grav = v3<F>((F)P.gravity[0], (F)P.gravity[1], (F)P.gravity[2]);
    nf = sc->n_fluid;
    x.resize(nf); v.resize(nf); a.resize(nf);
    for (int64_t i = 0; i < nf; i++) {
      x[i] = v3<F>((F)sc->fluid_x[3 * i], (F)sc->fluid_x[3 * i + 1], (F)sc->fluid_x[3 * i + 2]);
      v[i] = sc->fluid_v ? v3<F>((F)sc->fluid_v[3 * i], (F)sc->fluid_v[3 * i + 1], (F)sc->fluid_v[3 * i + 2]) : V3F::zero();
    }
    x_init = x; v_init = v;
    rho.assign(nf, 0); factor.assign(nf, 0); kappa.assign(nf, 0); kappaV.assign(nf, 0); rhoAdv.assign(nf, 0);
    sumgrad.assign(nf, V3F::zero());
    nthreads = omp_get_max_threads();
    for (int b = 0; b < sc->n_bodies; b++) {
      const dfsph_body_desc &d = sc->bodies[b];
      Body B;
      B.dyn = d.is_dynamic != 0; B.anim = B.anim0 = d.is_animated != 0;
      B.start = nbp; B.count = d.n_samples;
      B.x0 = v3<R>((R)d.translation[0], (R)d.translation[1], (R)d.translation[2]);
      B.q0 = {(R)d.rotation[0], (R)d.rotation[1], (R)d.rotation[2], (R)d.rotation[3]};
      B.q0.normalize();
      B.initV = v3<R>((R)d.init_velocity[0], (R)d.init_velocity[1], (R)d.init_velocity[2]);
      B.initW = v3<R>((R)d.init_angular_velocity[0], (R)d.init_angular_velocity[1], (R)d.init_angular_velocity[2]);
      B.targetX = v3<R>((R)d.target_x[0], (R)d.target_x[1], (R)d.target_x[2]);
      // Dynamic3dRigidBody::determineMassProperties (Dynamic3dRigidBody.h:184-213)
      const R vol = static_cast<R>(4.0 / 3.0 * M_PI) * (R)r * (R)r * (R)r;
      const R dm = vol * (R)d.density;
      B.mass = 0; B.I0 = M3R::zero();
      for (int64_t s = 0; s < d.n_samples; s++) {
        V3R p = v3<R>((R)d.samples[3 * s], (R)d.samples[3 * s + 1], (R)d.samples[3 * s + 2]);
        B.mass += dm;
        B.I0 += dm * (dot(p, p) * M3R::eye() - outer(p, p));
        bx0.push_back(v3<F>((F)d.samples[3 * s], (F)d.samples[3 * s + 1], (F)d.samples[3 * s + 2]));
        bbody.push_back(b);
      }
      B.invMass = R(1) / B.mass;
      B.fth.assign(nthreads, V3R::zero()); B.tth = B.fth; B.fbak = B.fth; B.tbak = B.fth;
      B.gFv.assign(B.count, M3R::zero()); B.gFx = B.gFv; B.gFw = B.gFv; B.gTw = B.gFv; B.gTv = B.gFv; B.gTx = B.gFv;
      B.gFq.assign(B.count, M34R::zero()); B.gTq = B.gFq;
      nbp += d.n_samples;
      bodies.push_back(B);
    }
    bx.assign(nbp, V3F::zero()); bv.assign(nbp, V3F::zero()); psi.assign(nbp, 0);
    const size_t nb2 = bodies.size() * bodies.size();
    mgrM.resize(nb2); mgrMc.resize(nb2); mgrS.resize(nb2);
    mFv0.resize(nb2); mFw0.resize(nb2); mTv0.resize(nb2); mTw0.resize(nb2);
    reset();
    if (P.use_rigid_contact_solver) init_contact();
  }

  // RigidContactSolver::RigidContactSolver (RigidContactSolver.cpp:23-262): every boundary
  // sample's rest volume gamma / (W0 + sum over its own body's neighbours of W) and rest
  // density, with the contact kernel of support factor * r, from the samples' world positions
  // once (own-body distances do not change as the bodies move).
  void init_contact() {
    KCt.set((R)P.rigid_contact_support_radius_factor * (R)P.particle_radius);
    KHr.set((R)h);
    std::vector<int64_t> S; std::vector<int32_t> I;
    neighbor_search(bx, bx, h, true, S, I);
    cvol0.assign(nbp, R(0)); cdens0.assign(nbp, R(0));
    const R gamma = (R)P.rigid_contact_gamma;
    for (int64_t j = 0; j < nbp; j++) {
      R sumW = KCt.w0;
      for (int64_t s = S[j]; s < S[j + 1]; s++)
        if (bbody[I[s]] == bbody[j]) sumW += KCt.W(V3R(bx[j].template cast<R>() - bx[I[s]].template cast<R>()));
      cvol0[j] = gamma / sumW;
    }
    for (int64_t j = 0; j < nbp; j++) {
      R d = cvol0[j] * KCt.w0;
      for (int64_t s = S[j]; s < S[j + 1]; s++)
        if (bbody[I[s]] == bbody[j]) d += cvol0[I[s]] * KCt.W(V3R(bx[j].template cast<R>() - bx[I[s]].template cast<R>()));
      cdens0[j] = d;
    }
  }

  void update_inertia(Body &B) {  // Dynamic3dRigidBody.h:215-219
    M3R Rm = B.q.R();
    B.I = Rm * B.I0 * Rm.T_();
    B.Iinv = inverse3(B.I);
  }
  // SimulatorBase::updateBoundaryParticles (SimulatorBase.cpp:1827-1857)
  void update_boundary_particles(bool force) {
    for (auto &B : bodies) {
      if (!(B.dyn || B.anim || force)) continue;
      for (int64_t j = B.start; j < B.start + B.count; j++) {
        V3R p = B.q.rotate(bx0[j].template cast<R>()) + B.x;
        bx[j] = p.template cast<F>();
        if (B.dyn || B.anim) bv[j] = (cross(B.w, bx[j].template cast<R>() - B.x) + B.v).template cast<F>();
        else bv[j] = V3F::zero();
      }
    }
  }
  // Simulation::updateBoundaryVolume + BoundaryModel_Akinci2012::computeBoundaryVolume
  // (Simulation.cpp:831-900, BoundaryModel_Akinci2012.cpp:257-284): psi_j = 1 / (W0 + sum over
  // boundary neighbours of any body). Static bodies are activated together and each dynamic body
  // alone, but every activation searches all point sets, so all boundary neighbours count.
  void update_boundary_volume() {
    std::vector<int64_t> S; std::vector<int32_t> I;
    neighbor_search(bx, bx, h, true, S, I);
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < nbp; j++) {
      F delta = K.w0;
      for (int64_t s = S[j]; s < S[j + 1]; s++) delta += K.W(bx[j] - bx[I[s]]);
      psi[j] = F(1) / delta;
    }
  }
  int reset() override {  // SimulatorBase::reset (SimulatorBase.cpp:887-934)
    x = x_init; v = v_init;
    std::fill(kappa.begin(), kappa.end(), F(0)); std::fill(kappaV.begin(), kappaV.end(), F(0));
    std::fill(sumgrad.begin(), sumgrad.end(), V3F::zero());
    for (auto &B : bodies) {  // Dynamic3dRigidBody::reset (Dynamic3dRigidBody.h:163-175)
      B.x = B.x0; B.q = B.q0; B.v = V3R::zero(); B.w = V3R::zero(); B.anim = B.anim0;
      update_inertia(B);
      std::fill(B.fth.begin(), B.fth.end(), V3R::zero()); std::fill(B.tth.begin(), B.tth.end(), V3R::zero());
    }
    update_boundary_particles(true);
    update_boundary_volume();
    t = 0; step_count = 0; finished = false;
    set_dt((F)P.time_step);
    reset_gradient();
    clear_manager_blocks();
    return 0;
  }
  int reset_gradient() override {  // BoundaryModel_Akinci2012::reset_gradient (:61-108)
    for (auto &B : bodies) {
      for (int64_t j = 0; j < B.count; j++) {
        B.gFv[j] = M3R::zero(); B.gFx[j] = M3R::zero(); B.gFw[j] = M3R::zero(); B.gTw[j] = M3R::zero();
        B.gTv[j] = M3R::zero(); B.gTx[j] = M3R::zero(); B.gFq[j] = M34R::zero(); B.gTq[j] = M34R::zero();
      }
      B.nFv = B.nFx = B.nFw = B.nTw = B.nTv = B.nTx = M3R::zero(); B.nFq = B.nTq = M34R::zero();
      B.Gv_v = M3R::eye(); B.Gv_w = M3R::zero(); B.Gw_w = M3R::eye(); B.Gw_v = M3R::zero();
      B.Gq_w = M43R::zero(); B.partial_qn_w = M43R::zero(); B.Gq_v = M43R::zero();
      B.Gx_v = M3R::zero(); B.Gx_w = M3R::zero();
    }
    // RigidBodyGradientManager::reset (RigidBodyGradientManager.cpp:477-524) of the chain
    // state; the blocks are cleared by reset() only (the GPU library keeps them across
    // dfsph_reset_gradient so that checkpointed replays map as the first run did)
    const int nb = (int)bodies.size();
    for (int a = 0; a < nb; a++)
      for (int c = 0; c < nb; c++) {
        MgrState &S = mgrS[a * nb + c];
        S.Gx_v = S.Gx_w = S.Gv_w = S.Gw_v = M3R::zero();
        S.Gq_v = S.Gq_w = M43R::zero();
        S.Gv_v = S.Gw_w = (a == c) ? M3R::eye() : M3R::zero();
        mFv0[a * nb + c] = mFw0[a * nb + c] = mTv0[a * nb + c] = mTw0[a * nb + c] = M3R::zero();
      }
    return 0;
  }
  void clear_manager_blocks() {
    for (size_t k = 0; k < mgrM.size(); k++) {
      MgrBlk &M = mgrM[k];
      M.Fv = M.Fx = M.Fw = M.Tw = M.Tv = M.Tx = M3R::zero(); M.Fq = M.Tq = M34R::zero();
      mgrMc[k] = M;
    }
  }

  // BoundaryModel::addForce (BoundaryModel.h:46-58)
  void add_force(int b, const V3F &pos, const V3F &f) {
    Body &B = bodies[b];
    if (!B.dyn) return;
    const int tid = omp_get_thread_num();
    V3R fr = f.template cast<R>();
    B.fth[tid] += fr;
    B.tth[tid] += cross(pos.template cast<R>() - B.x, fr);
  }
  void force_and_torque(Body &B, V3R &F_, V3R &T_) {  // BoundaryModel.cpp:38-54
    F_ = V3R::zero(); T_ = V3R::zero();
    for (int j = 0; j < nthreads; j++) { F_ += B.fth[j]; T_ += B.tth[j]; B.fbak[j] = B.fth[j]; B.tbak[j] = B.tth[j]; }
  }

  // ---- fluid passes
  void compute_densities() {  // TimeStep.cpp:147-200
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) {
      F d = Vf * K.w0;
      for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) d += Vf * K.W(x[i] - x[ff[s]]);
      for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) d += psi[fb[s]] * K.W(x[i] - bx[fb[s]]);
      rho[i] = d * rho0;
    }
  }
  void compute_factor() {  // TimeStepDiffDFSPH.cpp:883-962
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) {
      F sum_grad_p_k = 0;
      V3F gpi = V3F::zero();
      for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) {
        const V3F gpj = -Vf * K.gradW(x[i] - x[ff[s]]);
        sum_grad_p_k += sqnorm(gpj);
        gpi -= gpj;
      }
      for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) {
        const V3F gpj = -psi[fb[s]] * K.gradW(x[i] - bx[fb[s]]);
        gpi -= gpj;
      }
      sumgrad[i] = -gpi;
      sum_grad_p_k += sqnorm(gpi);
      factor[i] = (sum_grad_p_k > eps) ? -F(1) / sum_grad_p_k : F(0);
    }
  }
  void density_adv(int64_t i) {  // TimeStepDiffDFSPH.cpp:1926-1975
    F delta = 0;
    for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) { const int j = ff[s]; delta += Vf * dot(v[i] - v[j], K.gradW(x[i] - x[j])); }
    for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) { const int j = fb[s]; delta += psi[j] * dot(v[i] - bv[j], K.gradW(x[i] - bx[j])); }
    F da = rho[i] / rho0 + dt * delta;
    rhoAdv[i] = std::max(da, F(1));
  }
  void density_change(int64_t i) {  // TimeStepDiffDFSPH.cpp:1977-2041
    F da = 0;
    for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) { const int j = ff[s]; da += Vf * dot(v[i] - v[j], K.gradW(x[i] - x[j])); }
    for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) { const int j = fb[s]; da += psi[j] * dot(v[i] - bv[j], K.gradW(x[i] - bx[j])); }
    da = std::max(da, F(0));
    const int64_t nn = (ffS[i + 1] - ffS[i]) + (fbS[i + 1] - fbS[i]);
    if (nn < 20) da = 0;
    rhoAdv[i] = da;
  }
  // velocity correction shared by the warm starts and the Jacobi sweeps
  // (TimeStepDiffDFSPH.cpp:1016-1055, 1117-1196, 1745-1785, 1840-1901)
  template <class KFn>
  void velocity_correction(int64_t i, F ki, KFn kj_of) {
    V3F vi = v[i];
    for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) {
      const int j = ff[s];
      const F kSum = ki + (rho0 / rho0) * kj_of(j);
      if (std::fabs(kSum) > eps) {
        const V3F gpj = -Vf * K.gradW(x[i] - x[j]);
        vi -= dt * kSum * gpj;
      }
    }
    if (std::fabs(ki) > eps) {
      for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) {
        const int j = fb[s];
        const V3F gpj = -psi[j] * K.gradW(x[i] - bx[j]);
        const V3F velChange = -dt * F(1) * ki * gpj;
        vi += velChange;
        const V3F force = -mf * velChange * invH;
        add_force(bbody[j], bx[j], force);
      }
    }
    v[i] = vi;
  }

  // ---- gradient: TimeStepDiffDFSPH.cpp:1226-1482 (+ helpers :1485-1694)
  void compute_rigid_body_gradient(int mode) {
    const F invH2_g = F(1) / dt / dt, invH_g = F(1) / dt;  // :1231-1232, :1293-1294
    const F cReal = (mode == 0) ? invH2_g : invH_g;          // :1320-1322
    unsigned int cu = (mode == 0) ? (unsigned int)invH2_g : (unsigned int)invH_g;  // :1266
    const F cTrunc = P.truncate_gradient_coeff ? (F)cu : ((mode == 0) ? invH2_g : invH_g);
    for (size_t b = 0; b < bodies.size(); b++) {
      Body &B = bodies[b];
      if (!(B.dyn && !B.anim)) continue;
      const QR q = B.q;
      const V3R om = B.w;
#pragma omp parallel for schedule(static)
      for (int64_t jj = 0; jj < B.count; jj++) {
        const int64_t j = B.start + jj;
        const V3F xj = bx[j];
        for (int64_t s = bfS[j]; s < bfS[j + 1]; s++) {
          const int64_t i = bf[s];
          const F b_i = (mode == 0) ? rhoAdv[i] - F(1) : rhoAdv[i];
          const F ki = b_i * factor[i] * cTrunc;
          const V3F gpj = -psi[j] * K.gradW(x[i] - xj);
          const V3F velChange = -dt * F(1) * ki * gpj;
          const V3F force = -mf * velChange * invH;
          // computeGradient
          const M3F g2 = psi[j] * K.gradGradW(x[i] - xj);
          const F fac = factor[i];
          V3F gbx;
          if (mode == 0) {  // :1518-1549
            if (rhoAdv[i] <= F(1)) gbx = V3F::zero();
            else gbx = (-psi[j] * K.gradW(x[i] - xj)) / rho0 - dt * psi[j] * K.gradGradW(x[i] - xj) * (v[i] - bv[j]);
          } else {  // :1552-1577
            if (rhoAdv[i] <= F(0)) gbx = V3F::zero();
            else gbx = -psi[j] * K.gradGradW(x[i] - xj) * (v[i] - bv[j]);
          }
          V3F gfx = V3F::zero();  // :1485-1516
          if (!(fac >= F(0))) gfx = F(2) * fac * fac * (g2 * sumgrad[i]);
          const V3F gkx = (gbx * fac + b_i * gfx) * cReal;
          const M3F gvcx = -F(1) * (outer(gpj, gkx) + ki * g2);
          V3F gbv;  // :1579-1628
          if (mode == 0) gbv = (rhoAdv[i] <= F(1)) ? V3F::zero() : V3F(-dt * psi[j] * K.gradW(x[i] - xj));
          else gbv = (rhoAdv[i] <= F(0)) ? V3F::zero() : V3F(-psi[j] * K.gradW(x[i] - xj));
          const V3F gkv = gbv * fac * cReal;
          const M3F gvcv = -F(1) * outer(gpj, gkv);
          // :1632-1694 (all neighbours of i, fluid then boundary)
          V3F gbvi = V3F::zero();
          const bool act = (mode == 0) ? (rhoAdv[i] > F(1)) : (rhoAdv[i] > F(0));
          if (act) {
            for (int64_t t2 = ffS[i]; t2 < ffS[i + 1]; t2++) gbvi += Vf * K.gradW(x[i] - x[ff[t2]]);
            for (int64_t t2 = fbS[i]; t2 < fbS[i + 1]; t2++) gbvi += psi[fb[t2]] * K.gradW(x[i] - bx[fb[t2]]);
            if (mode == 0) gbvi = gbvi * dt;
          }
          const V3F gkvi = gbvi * fac * cReal;
          const M3F gvcvi = -outer(gpj, gkvi);
          const M3F Fx = -mf * gvcx;
          const M3F Fv = inverse3(M3F(M3F::eye() - dt * gvcvi)) * (-mf * gvcv);
          const M3R Fxr = Fx.template cast<R>(), Fvr = Fv.template cast<R>();
          B.gFx[jj] += Fxr;
          B.gFv[jj] += Fvr;
          if (P.optimize_rotation) {  // :1425-1480
            const V3R rj = xj.template cast<R>() - B.x;
            const V3R r0 = bx0[j].template cast<R>();
            const M34R Grq = grad_Rqp_to_q(q, r0);
            const M34R Fq = Fxr * Grq + Fvr * skew(om) * Grq;
            const M3R Fw = Fvr * skew(rj).T_();
            const M34R Tq = skew(rj) * Fq + skew(force.template cast<R>()).T_() * Grq;
            const M3R Tw = skew(rj) * Fw;
            B.gFw[jj] += Fw; B.gFq[jj] += Fq; B.gTw[jj] += Tw; B.gTq[jj] += Tq;
            B.gTv[jj] += skew(rj) * Fvr;
            B.gTx[jj] += skew(rj) * Fxr;
          }
        }
      }
    }
  }

  // ---- solvers
  void divergence_solve() {  // TimeStepDiffDFSPH.cpp:770-881
    if (P.use_divergence_warmstart) {  // :1698-1788
#pragma omp parallel
      {
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nf; i++) {
          density_change(i);
          kappaV[i] = (rhoAdv[i] > F(0)) ? F(0.5) * std::max(kappaV[i], F(-0.5)) * invH : F(0);
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nf; i++) velocity_correction(i, kappaV[i], [&](int j) { return kappaV[j]; });
      }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) density_change(i);
    itersV = 0;
    bool chk = false;
    double avg = 0;
    const int maxIter = P.max_iterations_v;
    while ((!chk || itersV < 1) && itersV < maxIter) {
      chk = true;
      // divergenceSolveIteration :1790-1922
      if (P.enable_gradient) compute_rigid_body_gradient(1);
      std::vector<F> kv(nf);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nf; i++) kv[i] = rhoAdv[i] * factor[i] * invH;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nf; i++) {
        const F ki = kv[i];
        if (P.use_divergence_warmstart) kappaV[i] += ki;
        velocity_correction(i, ki, [&](int j) { return kv[j]; });
      }
      F err = 0;
#pragma omp parallel for reduction(+ : err) schedule(static)
      for (int64_t i = 0; i < nf; i++) { density_change(i); err += rho0 * rhoAdv[i]; }
      avg = (double)(err / (F)nf);
      const F eta = (F(1) / dt) * (F)P.max_error_v * F(0.01) * rho0;
      chk = chk && ((F)avg <= eta);
      itersV++;
    }
    lastErrV = avg;
    if (P.use_divergence_warmstart)
      for (int64_t i = 0; i < nf; i++) kappaV[i] *= dt;
  }
  void pressure_solve() {  // TimeStepDiffDFSPH.cpp:654-768
    if (P.use_pressure_warmstart) {  // :964-1059
#pragma omp parallel
      {
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nf; i++) {
          density_adv(i);
          kappa[i] = (rhoAdv[i] > F(1)) ? F(0.5) * std::max(kappa[i], F(-0.00025)) * invH2 : F(0);
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nf; i++) velocity_correction(i, kappa[i], [&](int j) { return kappa[j]; });
      }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) density_adv(i);
    iters = 0;
    bool chk = false;
    double avg = 0;
    while ((!chk || iters < P.min_iterations) && iters < P.max_iterations) {
      chk = true;
      // pressureSolveIteration :1061-1220
      if (P.enable_gradient) compute_rigid_body_gradient(0);
      std::vector<F> kp(nf);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nf; i++) kp[i] = (rhoAdv[i] - F(1)) * factor[i] * invH2;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nf; i++) {
        const F ki = kp[i];
        if (P.use_pressure_warmstart) kappa[i] += ki;
        velocity_correction(i, ki, [&](int j) { return kp[j]; });
      }
      F err = 0;
#pragma omp parallel for reduction(+ : err) schedule(static)
      for (int64_t i = 0; i < nf; i++) { density_adv(i); err += rho0 * rhoAdv[i] - rho0; }
      avg = (double)(err / (F)nf);
      const F eta = (F)P.max_error * F(0.01) * rho0;
      chk = chk && ((F)avg <= eta);
      iters++;
    }
    lastErr = avg;
    if (P.use_pressure_warmstart)
      for (int64_t i = 0; i < nf; i++) kappa[i] *= dt * dt;
  }

  // ---- chain rule: BoundaryModel_Akinci2012.cpp:543-889
  M3R grad_inertia_v(const Body &B, const V3R &vv, const M43R &Gq) {  // :513-533
    const M3R Rm = B.q.R();
    return grad_Rqp_to_q(B.q, V3R(B.I0 * Rm.T_() * vv)) * Gq + Rm * B.I0 * (grad_RqTp_to_q(B.q, vv) * Gq);
  }
  void chain_rule(Body &B) {
    const int mode = P.gradient_mode;
    const bool gyro = P.rigid_body_mode == DFSPH_RB_GYROSCOPIC;
    const R mass = B.mass;
    const R invMass = R(1) / (mass + R(1e-10));
    const M3R &inertia = B.I, &inv_inertia = B.Iinv;
    const V3R om = B.w;
    const R h_ = (R)dt;
    V3R temp_v = V3R::zero();
    V3R force, torque;
    if (mode == DFSPH_GRAD_COMPLETE || mode == DFSPH_GRAD_INCOMPLETE) {
      M3R gF_v0, gF_w0, gT_v0, gT_w0;
      if (mode == DFSPH_GRAD_COMPLETE) {  // :569-672
        gF_v0 = B.nFx * B.Gx_v + B.nFv * B.Gv_v + B.nFq * B.Gq_v + B.nFw * B.Gw_v;
        gF_w0 = B.nFx * B.Gx_w + B.nFv * B.Gv_w + B.nFq * B.Gq_w + B.nFw * B.Gw_w;
      } else {  // :711-824
        gF_v0 = B.nFv * B.Gv_v + B.nFw * B.Gw_v;
        gF_w0 = B.nFv * B.Gv_w + B.nFw * B.Gw_w;
      }
      B.Gv_v = B.Gv_v + h_ * invMass * gF_v0;
      B.Gv_w = B.Gv_w + h_ * invMass * gF_w0;
      B.Gx_v = B.Gx_v + h_ * B.Gv_v;
      B.Gx_w = B.Gx_w + h_ * B.Gv_w;
      force_and_torque(B, force, torque);
      if (mode == DFSPH_GRAD_COMPLETE) {
        gT_w0 = B.nTx * B.Gx_w + B.nTv * B.Gv_w + B.nTq * B.Gq_w + B.nTw * B.Gw_w;
        gT_v0 = B.nTx * B.Gx_v + B.nTv * B.Gv_v + B.nTq * B.Gq_v + B.nTw * B.Gw_v;
      } else {
        gT_w0 = B.nTv * B.Gv_w + B.nTw * B.Gw_w;
        gT_v0 = B.nTv * B.Gv_v + B.nTw * B.Gw_v;
      }
      M3R gTau_w0, gTau_v0;
      if (gyro) {
        temp_v = cross(V3R(inertia * om), om) + torque;
        const M3R gL_w0 = skew(V3R(inertia * om)) * B.Gw_w + skew(om).T_() * (inertia * B.Gw_w + grad_inertia_v(B, om, B.Gq_w));
        const M3R gL_v0 = skew(V3R(inertia * om)) * B.Gw_v + skew(om).T_() * (inertia * B.Gw_v + grad_inertia_v(B, om, B.Gq_v));
        gTau_w0 = gL_w0 + gT_w0;
        gTau_v0 = gL_v0 + gT_v0;
      } else {
        temp_v = torque;
        gTau_w0 = gT_w0;
        gTau_v0 = gT_v0;
      }
      const M3R gII_w0 = inv_inertia * grad_inertia_v(B, V3R(inv_inertia * temp_v), B.Gq_w);
      const M3R gII_v0 = inv_inertia * grad_inertia_v(B, V3R(inv_inertia * temp_v), B.Gq_v);
      B.Gw_w = B.Gw_w + h_ * (gII_w0 + inv_inertia * gTau_w0);
      B.Gw_v = B.Gw_v + h_ * (gII_v0 + inv_inertia * gTau_v0);
    } else {  // RigidGradOnly :674-709
      B.Gx_v = B.Gx_v + h_ * B.Gv_v;
      B.Gx_w = B.Gx_w + h_ * B.Gv_w;
      if (gyro) {
        temp_v = cross(V3R(inertia * om), om);
        const M3R gII_w0 = inv_inertia * grad_inertia_v(B, V3R(inv_inertia * temp_v), B.Gq_w);
        const M3R gII_v0 = inv_inertia * grad_inertia_v(B, V3R(inv_inertia * temp_v), B.Gq_v);
        const M3R gL_w0 = skew(V3R(inertia * om)) * B.Gw_w + skew(om).T_() * (inertia * B.Gw_w + grad_inertia_v(B, om, B.Gq_w));
        const M3R gL_v0 = skew(V3R(inertia * om)) * B.Gw_v + skew(om).T_() * (inertia * B.Gw_v + grad_inertia_v(B, om, B.Gq_v));
        B.Gw_w = B.Gw_w + h_ * (gII_w0 + inv_inertia * gL_w0);
        B.Gw_v = B.Gw_v + h_ * (gII_v0 + inv_inertia * gL_v0);
      }
    }
    if (P.optimize_rotation) {  // :827-888
      const QR q = B.q;
      const V3R new_om = om + h_ * (inv_inertia * temp_v);
      const QR p = {R(0), new_om[0], new_om[1], new_om[2]};
      QR nq = q;
      const QR pq = p * nq;
      nq.w += h_ * R(0.5) * pq.w; nq.x += h_ * R(0.5) * pq.x; nq.y += h_ * R(0.5) * pq.y; nq.z += h_ * R(0.5) * pq.z;
      QR nqn = nq; nqn.normalize();
      const V4<R> nv = nqn.vec4();
      const M4<R> Gpq = grad_p_q_product_to_q(p);
      const M43R Gpw = grad_omega_q_product_to_omega(q);
      const M4<R> Gn = (M4<R>::eye() - nv * nv.T_()) / nq.norm();
      B.partial_qn_w = Gn * ((h_ / R(2)) * Gpw);
      B.Gq_w = Gn * (B.Gq_w + (h_ / R(2)) * (Gpw * B.Gw_w + Gpq * B.Gq_w));
      B.Gq_v = Gn * (B.Gq_v + (h_ / R(2)) * (Gpw * B.Gw_v + Gpq * B.Gq_v));
    }
  }
  // BoundaryModel_Akinci2012::accumulate_and_reset_gradient (:453-497)
  void accumulate_and_reset(Body &B) {
    B.nFv = B.nFx = B.nFw = B.nTw = B.nTv = B.nTx = M3R::zero(); B.nFq = B.nTq = M34R::zero();
    for (int64_t j = 0; j < B.count; j++) {
      B.nFv += B.gFv[j]; B.nFx += B.gFx[j]; B.nFw += B.gFw[j]; B.nFq += B.gFq[j];
      B.nTw += B.gTw[j]; B.nTq += B.gTq[j]; B.nTv += B.gTv[j]; B.nTx += B.gTx[j];
      B.gFv[j] = B.gFx[j] = B.gFw[j] = B.gTw[j] = B.gTv[j] = B.gTx[j] = M3R::zero();
      B.gFq[j] = B.gTq[j] = M34R::zero();
    }
  }

  // Dynamic3dRigidBody::addForce / addTorque (Dynamic3dRigidBody.h:113-142): each call moves
  // the body's velocities at once; in the gyroscopic mode every addTorque adds (I w) x w with
  // the angular velocity of that moment.
  void add_force_now(Body &B, const V3R &f) { B.v += B.invMass * f * (R)dt; }
  void add_torque_now(Body &B, const V3R &tq) {
    if (P.rigid_body_mode == DFSPH_RB_GYROSCOPIC) {
      const V3R L = B.I * B.w;
      B.w += B.Iinv * (cross(L, B.w) + tq) * (R)dt;
    } else B.w += B.Iinv * tq * (R)dt;
  }
  static V3R normalized_or_self(const V3R &a) {  // Eigen 3.4 MatrixBase::normalized()
    const R z = sqnorm(a);
    return z > R(0) ? V3R(a / std::sqrt(z)) : a;
  }
  // RigidContactSolver::beforePenaltyInitialize + solveRigidContactPenalty
  // (RigidContactSolver.cpp:307-345, 419-555), for the samples of dynamic bodies (a static
  // body's force moves nothing and the manager skips its blocks). Neighbours over all boundary
  // point sets within h; the contact density uses the contact kernel, its gradient the
  // simulation's kernel (sim->gradW, :456-460).
  void contact_forces(bool grad) {
    const int nb = (int)bodies.size();
    for (auto &M : mgrMc) { M.Fv = M.Fx = M.Fw = M.Tw = M.Tv = M.Tx = M3R::zero(); M.Fq = M.Tq = M34R::zero(); }
    n_contact = n_active = 0;
    std::vector<char> mask(nbp, 0);
    for (auto &B : bodies) if (B.dyn) for (int64_t j = B.start; j < B.start + B.count; j++) mask[j] = 1;
    std::vector<int64_t> S; std::vector<int32_t> I;
    neighbor_search(bx, bx, h, true, S, I, &mask);
    auto svel = [&](int64_t k) -> V3R {  // vel[R][r] (:313-316): the bodies' velocities after gravity
      const Body &C = bodies[bbody[k]];
      if (!(C.dyn || C.anim)) return V3R::zero();
      return V3R(C.v + cross(C.w, V3R(bx[k].template cast<R>() - C.x)));
    };
    const R beta = (R)P.rigid_contact_beta, mu = (R)P.rigid_contact_friction_coeff;
    for (int b = 0; b < nb; b++) {
      Body &B = bodies[b];
      if (!B.dyn) continue;
      for (int64_t j = B.start; j < B.start + B.count; j++) {
        bool has = false;
        for (int64_t s = S[j]; s < S[j + 1]; s++) if (bbody[I[s]] != b) has = true;
        if (!has) continue;
        n_contact++;
        const V3R xr = bx[j].template cast<R>();
        const V3R rr = xr - B.x;
        const V3R r0 = bx0[j].template cast<R>();
        R dens = cvol0[j] * KCt.w0;
        V3R sum_x = V3R::zero(), sum_vk = V3R::zero(), avg_rk = V3R::zero(), gdx = V3R::zero();
        V4<R> gdq = V4<R>::zero(), gdqk = V4<R>::zero();
        R sum_w = 0;
        int RR = b;
        const M34R GqB = grad_Rqp_to_q(B.q, r0);
        for (int64_t s = S[j]; s < S[j + 1]; s++) {
          const int64_t k = I[s];
          const V3R xk = bx[k].template cast<R>();
          const V3R d = xr - xk;
          const R w = KCt.W(d);
          dens += cvol0[k] * w;
          if (bbody[k] == b) { sum_x += xk * w; sum_w += w; }
          else {
            RR = bbody[k];
            const Body &C = bodies[RR];
            sum_vk += svel(k) * w;
            avg_rk += V3R(xk - C.x) * w;
            const V3R gw = KHr.gradW(d);
            gdx += cvol0[k] * gw;
            gdq += (cvol0[k] * gw.T_() * GqB).T_();
            gdqk += (cvol0[k] * gw.T_() * R(-1) * grad_Rqp_to_q(C.q, V3R(bx0[k].template cast<R>()))).T_();
          }
        }
        const R ratio = dens / cdens0[j];
        if (!(ratio > R(1))) continue;
        n_active++;
        const V3R normal = xr - sum_x / sum_w;
        const V3R vrel = svel(j) - sum_vk / sum_w;
        avg_rk = avg_rk / sum_w;
        const V3R Fn = -beta * std::max(ratio - R(1), R(0)) * normal;
        const V3R u = normalized_or_self(vrel);
        const V3R Ff = -mu * norm(Fn) * u;
        const V3R f = Fn + Ff;
        add_force_now(B, f);
        add_torque_now(B, cross(rr, f));
        if (!grad) continue;
        const V3R gFn_d = -beta * normal;
        const M3R gFn_x = gFn_d * gdx.T_();
        const M34R gFn_q = gFn_d * gdq.T_();
        const M34R gFn_qk = gFn_d * gdqk.T_();
        const V3R gFf_d = ((-mu * u) * Fn.T_() / norm(Fn)) * gFn_d;
        const M3R gFf_vr = (-mu * norm(Fn) / norm(vrel)) * (M3R::eye() - u * u.T_());
        const M3R gFf_w = gFf_vr * skew(rr).T_();
        const M3R gFf_wk = -gFf_vr * skew(avg_rk).T_();
        const M3R gFf_x = gFf_d * gdx.T_();
        const M34R gFf_q = gFf_d * gdq.T_();
        const M34R gFf_qk = gFf_d * gdqk.T_();
        MgrBlk &D = mgrMc[b * nb + b];
        const M3R gf_x = gFn_x + gFf_x;
        D.Fx += gf_x;
        D.Tx += skew(rr) * gf_x;
        const M34R gf_q = gFn_q + gFf_q;
        D.Fq += gf_q;
        D.Tq += skew(rr) * gf_q + skew(f).T_() * GqB;
        D.Fv += gFf_vr;
        D.Fw += gFf_w;
        if (RR != b) {
          MgrBlk &X = mgrMc[b * nb + RR];
          X.Fv += -gFf_vr;
          X.Fw += gFf_wk;
          X.Fx += -gf_x;
          X.Tx += -skew(rr) * gf_x;
          const M34R gf_qk = gFn_qk + gFf_qk;
          X.Fq += gf_qk;
          X.Tq += skew(rr) * gf_qk;
        }
      }
    }
  }

  // ---- RigidBodyGradientManager (RigidBodyGradientManager.cpp:96-468)
  // perform_force_and_torque_chain_rule (:96-156) and its _Rigid form (:158-290), which adds
  // the x and q terms; its v0 columns lose the q term to a statement that ends early (:196-205).
  void mgr_force_chain(bool rigid) {
    const int nb = (int)bodies.size();
    for (int a = 0; a < nb; a++)
      for (int c = 0; c < nb; c++) mFv0[a * nb + c] = mFw0[a * nb + c] = mTv0[a * nb + c] = mTw0[a * nb + c] = M3R::zero();
    for (int a = 0; a < nb; a++) {
      if (!bodies[a].dyn) continue;
      for (int c = 0; c < nb; c++) {
        if (!bodies[c].dyn) continue;
        for (int k = 0; k < nb; k++) {
          if (!bodies[k].dyn) continue;
          const MgrBlk &M = mgrM[a * nb + k];
          const MgrState &S = mgrS[k * nb + c];
          if (!rigid) {
            mFv0[a * nb + c] += M.Fv * S.Gv_v + M.Fw * S.Gw_v;
            mTv0[a * nb + c] += M.Tv * S.Gv_v + M.Tw * S.Gw_v;
            mFw0[a * nb + c] += M.Fv * S.Gv_w + M.Fw * S.Gw_w;
            mTw0[a * nb + c] += M.Tv * S.Gv_w + M.Tw * S.Gw_w;
          } else {
            mFv0[a * nb + c] += M.Fv * S.Gv_v + M.Fw * S.Gw_v + M.Fx * S.Gx_v;
            mTv0[a * nb + c] += M.Tv * S.Gv_v + M.Tw * S.Gw_v + M.Tx * S.Gx_v;
            mFw0[a * nb + c] += M.Fv * S.Gv_w + M.Fw * S.Gw_w + M.Fx * S.Gx_w + M.Fq * S.Gq_w;
            mTw0[a * nb + c] += M.Tv * S.Gv_w + M.Tw * S.Gw_w + M.Tx * S.Gx_w + M.Tq * S.Gq_w;
          }
        }
      }
    }
  }
  // perform_velocity_chain_rule (:292-393); F and T are the fluid force and torque still held by
  // the boundary model (zero once updateBoundaryForces has cleared them)
  void mgr_velocity_chain(bool fluid_ft) {
    const int nb = (int)bodies.size();
    const bool gyro = P.rigid_body_mode == DFSPH_RB_GYROSCOPIC;
    const R dt_ = (R)dt;
    for (int a = 0; a < nb; a++) {
      Body &B = bodies[a];
      if (!B.dyn) continue;
      const M3R &inertia = B.I, &inv_inertia = B.Iinv;
      const V3R om = B.w;
      V3R force = V3R::zero(), torque = V3R::zero();
      if (fluid_ft) force_and_torque(B, force, torque);
      for (int c = 0; c < nb; c++) {
        if (!bodies[c].dyn) continue;
        MgrState &S = mgrS[a * nb + c];
        S.Gv_v = S.Gv_v + dt_ * B.invMass * mFv0[a * nb + c];
        S.Gv_w = S.Gv_w + dt_ * B.invMass * mFw0[a * nb + c];
        V3R temp_v;
        M3R gTau_w0, gTau_v0;
        if (gyro) {
          temp_v = cross(V3R(inertia * om), om) + torque;
          const M3R gL_w0 = skew(V3R(inertia * om)) * S.Gw_w + skew(om).T_() * (inertia * S.Gw_w + grad_inertia_v(B, om, S.Gq_w));
          const M3R gL_v0 = skew(V3R(inertia * om)) * S.Gw_v + skew(om).T_() * (inertia * S.Gw_v + grad_inertia_v(B, om, S.Gq_v));
          gTau_w0 = gL_w0 + mTw0[a * nb + c];
          gTau_v0 = gL_v0 + mTv0[a * nb + c];
        } else {
          temp_v = torque;
          gTau_w0 = mTw0[a * nb + c];
          gTau_v0 = mTv0[a * nb + c];
        }
        const M3R gII_w0 = inv_inertia * grad_inertia_v(B, V3R(inv_inertia * temp_v), S.Gq_w);
        const M3R gII_v0 = inv_inertia * grad_inertia_v(B, V3R(inv_inertia * temp_v), S.Gq_v);
        S.Gw_w = S.Gw_w + dt_ * (gII_w0 + B.Iinv * gTau_w0);
        S.Gw_v = S.Gw_v + dt_ * (gII_v0 + B.Iinv * gTau_v0);
      }
    }
  }
  // perform_position_and_rotation_chain_rule (:395-453), with the angular velocity the
  // velocity step left and the rotation before the position step
  void mgr_position_rotation() {
    const int nb = (int)bodies.size();
    const R dt_ = (R)dt;
    for (int a = 0; a < nb; a++) {
      const Body &B = bodies[a];
      if (!B.dyn) continue;
      const QR q = B.q;
      const QR p = {R(0), B.w[0], B.w[1], B.w[2]};
      QR nq = q;
      const QR pq = p * nq;
      nq.w += dt_ * R(0.5) * pq.w; nq.x += dt_ * R(0.5) * pq.x; nq.y += dt_ * R(0.5) * pq.y; nq.z += dt_ * R(0.5) * pq.z;
      QR nqn = nq; nqn.normalize();
      const V4<R> nv = nqn.vec4();
      const M4<R> Gpq = grad_p_q_product_to_q(p);
      const M43R Gpw = grad_omega_q_product_to_omega(q);
      const M4<R> Gn = (M4<R>::eye() - nv * nv.T_()) / nq.norm();
      for (int c = 0; c < nb; c++) {
        if (!bodies[c].dyn) continue;
        MgrState &S = mgrS[a * nb + c];
        S.Gx_v += dt_ * S.Gv_v;
        S.Gx_w += dt_ * S.Gv_w;
        S.Gq_v = Gn * (S.Gq_v + dt_ / R(2) * (Gpw * S.Gw_v + Gpq * S.Gq_v));
        S.Gq_w = Gn * (S.Gq_w + dt_ / R(2) * (Gpw * S.Gw_w + Gpq * S.Gq_w));
      }
    }
  }

  void neighborhood_search() {
    neighbor_search(x, x, h, true, ffS, ff);
    neighbor_search(x, bx, h, false, fbS, fb);
    std::vector<char> dynmask(nbp, 0);
    for (auto &B : bodies) if (B.dyn) for (int64_t j = B.start; j < B.start + B.count; j++) dynmask[j] = 1;
    neighbor_search(bx, x, h, false, bfS, bf, &dynmask);
  }

  // TimeStepDiffDFSPH::beginStep (:353-430)
  void begin_step() {
    step_count++;
    const R uat = (R)P.uniform_accelerate_rb_time;
    for (size_t b = 0; b < bodies.size(); b++) {
      Body &B = bodies[b];
      if (!B.dyn) continue;
      if (P.release_rigid_body_mode) {
        if (b == 1) {
          if (t <= uat + (R)dt) {
            if (uat > R(1e-3)) B.anim = true;
            B.v = V3R::zero(); B.w = V3R::zero();
          } else {
            B.v = B.initV; B.w = B.initW; B.anim = false;
          }
        }
      } else {
        if (t <= uat + (R)dt) {
          R fac = 1.;
          if (uat > R(1e-3)) { fac = (t / uat) > R(1) ? R(1) : (t / uat); B.anim = true; }
          B.v = fac * B.initV; B.w = fac * B.initW;
        } else B.anim = false;
      }
    }
  }

  void set_dt(F h) {
    dt = h;
    invH = F(1) / dt;
    invH2 = F(1) / (dt * dt);
  }

  // Simulation::updateTimeStepSizeCFL (Simulation.cpp:541-616)
  F cfl_time_step(F h) const {
    F maxVel = F(0.1);
    const F diameter = F(2.0) * r;
    for (int64_t i = 0; i < nf; i++) {
      const F velMag = sqnorm(V3F(v[i] + a[i] * h));
      if (velMag > maxVel) maxVel = velMag;
    }
    for (const auto &B : bodies) {
      if (!(B.dyn || B.anim)) continue;
      for (int64_t j = B.start; j < B.start + B.count; j++) {
        const F velMag = sqnorm(bv[j]);
        if (velMag > maxVel) maxVel = velMag;
      }
    }
    F hn = (F)P.cfl_factor * F(0.4) * (diameter / std::sqrt(maxVel));
    hn = std::min(hn, (F)P.cfl_max_time_step);
    hn = std::max(hn, (F)P.cfl_min_time_step);
    return hn;
  }

  void one_step() {
    begin_step();
    neighborhood_search();
    compute_densities();
    compute_factor();
    if (P.enable_divergence_solver) divergence_solve(); else { itersV = 0; lastErrV = 0; }
    // clearAccelerations (TimeStep.cpp:66-81), SurfaceTension_Akinci2013::step when enabled
    // (SurfaceTension_Akinci2013.cpp:28-148; Simulation::computeNonPressureForces runs it
    // before the viscosity, Simulation.cpp:618-631), Viscosity_XSPH::step (Viscosity_XSPH.cpp:35-110)
    const bool st = P.surface_tension_method == 2;
    if (st) {
      normals.assign(nf, V3F::zero());
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < nf; i++) {  // computeNormals (:28-58)
        V3F ni = V3F::zero();
        for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) {
          const int j = ff[s];
          ni += (mf / rho[j]) * K.gradW(x[i] - x[j]);
        }
        normals[i] = h * ni;
      }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) {
      V3F ai = grav;
      if (st) {
        const F kst = (F)P.surface_tension, kb = (F)P.surface_tension_boundary;
        for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) {  // cohesion and curvature (:84-107)
          const int j = ff[s];
          const F Kij = F(2.0) * rho0 / (rho[i] + rho[j]);
          V3F accel = V3F::zero();
          V3F xixj = x[i] - x[j];
          const F length2 = dot(xixj, xixj);
          if (length2 > F(1.0e-9)) {
            xixj = (F(1.0) / std::sqrt(length2)) * xixj;
            accel -= kst * mf * xixj * KC.W(x[i] - x[j]);
          }
          accel -= kst * (normals[i] - normals[j]);
          ai += Kij * accel;
        }
        for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) {  // adhesion (:112-124)
          const int j = fb[s];
          V3F xixj = x[i] - bx[j];
          const F length2 = dot(xixj, xixj);
          if (length2 > F(1.0e-9)) {
            xixj = (F(1.0) / std::sqrt(length2)) * xixj;
            ai -= kb * rho0 * psi[j] * xixj * KA.W(x[i] - bx[j]);
          }
        }
      }
      for (int64_t s = ffS[i]; s < ffS[i + 1]; s++) {
        const int j = ff[s];
        ai -= invH * visc * (mf / rho[j]) * (v[i] - v[j]) * K.W(x[i] - x[j]);
      }
      // boundary term and the bodies' reaction (Viscosity_XSPH.cpp:72-82)
      if (P.viscosity_boundary != 0.0) {
        const F vb = (F)P.viscosity_boundary;
        for (int64_t s = fbS[i]; s < fbS[i + 1]; s++) {
          const int j = fb[s];
          const V3F aa = -invH * vb * (rho0 * psi[j] / rho[i]) * (v[i] - bv[j]) * K.W(x[i] - bx[j]);
          ai += aa;
          add_force(bbody[j], bx[j], V3F(-mf * aa));
        }
      }
      a[i] = ai;
    }
    // Simulation::updateTimeStepSize (Simulation.cpp:524-616, called at
    // TimeStepDiffDFSPH.cpp:583): the new size applies to the pressure solve and the rigid
    // step; the advection, position update and time advance keep the step's size h_step
    const F h_step = dt;
    if (P.cfl_method == 1) set_dt(cfl_time_step(h_step));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) v[i] += h_step * a[i];  // :588-605
    pressure_solve();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) x[i] += h_step * v[i];  // :613-635
    t += (R)h_step;
    // backwardPerStep (:493-524): the per-body chain, or with the gradient manager the body's
    // net blocks become the manager's diagonal blocks (BoundaryModel_Akinci2012.cpp:952-967)
    const bool mgr = P.use_rigid_gradient_manager != 0;
    const int nbod = (int)bodies.size();
    for (int b = 0; b < nbod; b++) {
      Body &B = bodies[b];
      if (!B.dyn || B.anim) continue;
      accumulate_and_reset(B);
      if (mgr) {
        MgrBlk &M = mgrM[b * nbod + b];
        M.Fv = B.nFv; M.Fx = B.nFx; M.Fw = B.nFw; M.Fq = B.nFq;
        M.Tv = B.nTv; M.Tx = B.nTx; M.Tw = B.nTw; M.Tq = B.nTq;
      } else chain_rule(B);
    }
    // endStep (:432-490)
    finished = t >= (R)P.target_time + (R)P.uniform_accelerate_rb_time;
    // SimulatorBase::timeStep (SimulatorBase.cpp:999-1016): the manager's fluid stage, the
    // boundary simulator's velocity step, the manager's rigid stage, the position step
    if (mgr && nf > 0) { mgr_force_chain(false); mgr_velocity_chain(true); }
    if (P.use_rigid_contact_solver) {
      // RigidBody3dBoundarySimulator::velocityTimeStep with the contact solver (:284-298):
      // gravity on every dynamic body, the penalty forces, then updateBoundaryForces once per
      // boundary model (RigidContactSolver.cpp:355-358); after the first call the fluid force
      // is cleared, but each later addTorque(0) still adds the gyroscopic term
      for (auto &B : bodies) if (B.dyn) add_force_now(B, V3R(grav.template cast<R>() * B.mass));
      contact_forces(mgr);
      for (int rep = 0; rep < nbod; rep++)
        for (auto &B : bodies) {
          if (!B.dyn) continue;
          if (!B.anim) {
            V3R Fo, To;
            force_and_torque(B, Fo, To);
            add_force_now(B, Fo);
            add_torque_now(B, To);
          }
          if (rep == 0)
            for (int th = 0; th < nthreads; th++) { B.fbak[th] = B.fth[th]; B.tbak[th] = B.tth[th]; }
          for (int th = 0; th < nthreads; th++) { B.fth[th] = V3R::zero(); B.tth[th] = V3R::zero(); }
        }
    } else {
      // RigidBody3dBoundarySimulator::velocityTimeStep (:278-320) + BoundarySimulator::updateBoundaryForces
      for (auto &B : bodies) {
        if (!B.dyn) continue;
        if (!B.anim) {
          V3R Fo, To;
          force_and_torque(B, Fo, To);
          B.v += B.invMass * Fo * (R)dt;  // Dynamic3dRigidBody::addForce (:113-124)
          if (P.rigid_body_mode == DFSPH_RB_GYROSCOPIC) {  // addTorque (:125-142)
            const V3R L = B.I * B.w;
            B.w += B.Iinv * (cross(L, B.w) + To) * (R)dt;
          } else B.w += B.Iinv * To * (R)dt;
        }
        for (int th = 0; th < nthreads; th++) { B.fbak[th] = B.fth[th]; B.tbak[th] = B.tth[th]; B.fth[th] = V3R::zero(); B.tth[th] = V3R::zero(); }
        if (!B.anim) B.v += B.invMass * (grav.template cast<R>() * B.mass) * (R)dt;  // addGravity (:230-235)
      }
    }
    if (mgr) {
      if (P.use_rigid_contact_solver) {
        // RigidContactSolver::update_rigid_body_gradient_manager (:1341-1369): every dynamic pair
        for (int a = 0; a < nbod; a++)
          for (int c = 0; c < nbod; c++)
            if (bodies[a].dyn && bodies[c].dyn) mgrM[a * nbod + c] = mgrMc[a * nbod + c];
        mgr_force_chain(true);
        mgr_velocity_chain(false);
      }
      mgr_position_rotation();
    }
    // positionTimeStep (:322-344) -> Dynamic3dRigidBody::animate (:143-154)
    for (auto &B : bodies) {
      if (!B.dyn) continue;
      B.x += B.v * (R)dt;
      const QR wq = {R(0), B.w[0], B.w[1], B.w[2]};
      const QR d = wq * B.q;
      B.q.w += (R)dt * R(0.5) * d.w; B.q.x += (R)dt * R(0.5) * d.x; B.q.y += (R)dt * R(0.5) * d.y; B.q.z += (R)dt * R(0.5) * d.z;
      B.q.normalize();
      update_inertia(B);
    }
    update_boundary_particles(false);
  }

  int step(int n, dfsph_step_stats *st) override {
    int64_t ti = 0, tv = 0;
    int rc = 0;
    for (int k = 0; k < n; k++) {
      one_step();
      ti += iters; tv += itersV;
      if (iters >= P.max_iterations || (P.enable_divergence_solver && itersV >= P.max_iterations_v)) rc = DFSPH_ERR_NOT_CONVERGED;
    }
    if (st) {
      st->steps_done = n; st->pressure_iterations = iters; st->divergence_iterations = itersV;
      st->trajectory_finished = finished; st->pressure_avg_error = lastErr; st->divergence_avg_error = lastErrV;
      st->total_pressure_iterations = ti; st->total_divergence_iterations = tv; st->time = (double)t;
    }
    return rc;
  }

  // ---- accessors
  static void put3(double *d, const V3F &v) { d[0] = v[0]; d[1] = v[1]; d[2] = v[2]; }
  int copy_field(int f, double *dst) override {
    switch (f) {
      case DFSPH_FIELD_X: for (int64_t i = 0; i < nf; i++) put3(dst + 3 * i, x[i]); return 0;
      case DFSPH_FIELD_V: for (int64_t i = 0; i < nf; i++) put3(dst + 3 * i, v[i]); return 0;
      case DFSPH_FIELD_DENSITY: for (int64_t i = 0; i < nf; i++) dst[i] = rho[i]; return 0;
      case DFSPH_FIELD_FACTOR: for (int64_t i = 0; i < nf; i++) dst[i] = factor[i]; return 0;
      case DFSPH_FIELD_KAPPA: for (int64_t i = 0; i < nf; i++) dst[i] = kappa[i]; return 0;
      case DFSPH_FIELD_KAPPA_V: for (int64_t i = 0; i < nf; i++) dst[i] = kappaV[i]; return 0;
      case DFSPH_FIELD_DENSITY_ADV: for (int64_t i = 0; i < nf; i++) dst[i] = rhoAdv[i]; return 0;
      case DFSPH_FIELD_SUM_GRAD_P: for (int64_t i = 0; i < nf; i++) put3(dst + 3 * i, sumgrad[i]); return 0;
      case DFSPH_FIELD_BOUNDARY_X: for (int64_t i = 0; i < nbp; i++) put3(dst + 3 * i, bx[i]); return 0;
      case DFSPH_FIELD_BOUNDARY_V: for (int64_t i = 0; i < nbp; i++) put3(dst + 3 * i, bv[i]); return 0;
      case DFSPH_FIELD_BOUNDARY_PSI: for (int64_t i = 0; i < nbp; i++) dst[i] = psi[i]; return 0;
    }
    return DFSPH_ERR_INVALID_ARG;
  }
  int set_field(int f, const double *src) override {
    auto get3 = [&](int64_t i) { return v3<F>((F)src[3 * i], (F)src[3 * i + 1], (F)src[3 * i + 2]); };
    switch (f) {
      case DFSPH_FIELD_X: for (int64_t i = 0; i < nf; i++) x[i] = get3(i); return 0;
      case DFSPH_FIELD_V: for (int64_t i = 0; i < nf; i++) v[i] = get3(i); return 0;
      case DFSPH_FIELD_KAPPA: for (int64_t i = 0; i < nf; i++) kappa[i] = (F)src[i]; return 0;
      case DFSPH_FIELD_KAPPA_V: for (int64_t i = 0; i < nf; i++) kappaV[i] = (F)src[i]; return 0;
    }
    return DFSPH_ERR_INVALID_ARG;
  }
  int rigid_state(int b, double *xo, double *qo, double *vo, double *wo) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    const Body &B = bodies[b];
    for (int c = 0; c < 3; c++) { if (xo) xo[c] = B.x[c]; if (vo) vo[c] = B.v[c]; if (wo) wo[c] = B.w[c]; }
    if (qo) { qo[0] = B.q.w; qo[1] = B.q.x; qo[2] = B.q.y; qo[3] = B.q.z; }
    return 0;
  }
  int rigid_force(int b, double *Fo, double *To) override {  // BoundaryModel::getForce/getTorque
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    const Body &B = bodies[b];
    V3R f = V3R::zero(), tq = V3R::zero();
    for (int j = 0; j < nthreads; j++) { f += B.fbak[j]; tq += B.tbak[j]; }
    for (int c = 0; c < 3; c++) { Fo[c] = f[c]; To[c] = tq[c]; }
    return 0;
  }
  int rigid_mass(int b, double *m, double *I) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    *m = bodies[b].mass;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) I[3 * i + j] = bodies[b].I(i, j);
    return 0;
  }
  template <int RR, int CC> static double *put(double *o, const Mat<R, RR, CC> &m) {
    for (int i = 0; i < RR; i++) for (int j = 0; j < CC; j++) *o++ = m(i, j);
    return o;
  }
  int rigid_grad(int b, double *out) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    const Body &B = bodies[b];
    double *o = out;
    o = put(o, B.Gx_v); o = put(o, B.Gx_w); o = put(o, B.Gq_v); o = put(o, B.Gq_w);
    o = put(o, B.Gv_v); o = put(o, B.Gv_w); o = put(o, B.Gw_v); o = put(o, B.Gw_w);
    return 0;
  }
  int net_jac(int b, double *out) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    const Body &B = bodies[b];
    double *o = out;
    o = put(o, B.nFv); o = put(o, B.nFx); o = put(o, B.nFw); o = put(o, B.nFq);
    o = put(o, B.nTw); o = put(o, B.nTv); o = put(o, B.nTx); o = put(o, B.nTq);
    return 0;
  }
  int set_init(int b, const double *vv, const double *ww) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    bodies[b].initV = v3<R>((R)vv[0], (R)vv[1], (R)vv[2]);
    bodies[b].initW = v3<R>((R)ww[0], (R)ww[1], (R)ww[2]);
    return 0;
  }
  int set_velocity(int b, const double *vv, const double *ww) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    Body &B = bodies[b];
    B.v = v3<R>((R)vv[0], (R)vv[1], (R)vv[2]);
    B.w = v3<R>((R)ww[0], (R)ww[1], (R)ww[2]);
    for (int64_t j = B.start; j < B.start + B.count; j++)
      bv[j] = (B.dyn || B.anim) ? (cross(B.w, bx[j].template cast<R>() - B.x) + B.v).template cast<F>() : V3F::zero();
    return 0;
  }
  // A body's whole state (x, q as w x y z, v, omega), e.g. taken from another run at some step,
  // with the world inertia and the samples moved as Dynamic3dRigidBody::setPosition /
  // setRotation and SimulatorBase::updateBoundaryParticles do (Dynamic3dRigidBody.h:215-219).
  int set_rigid_state(int b, const double *xx, const double *qq, const double *vv, const double *ww) override {
    if (b < 0 || b >= (int)bodies.size()) return DFSPH_ERR_INVALID_ARG;
    const double qn = std::sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
    if (!(qn > 0)) return DFSPH_ERR_INVALID_ARG;
    Body &B = bodies[b];
    B.x = v3<R>((R)xx[0], (R)xx[1], (R)xx[2]);
    B.q = QR{(R)(qq[0] / qn), (R)(qq[1] / qn), (R)(qq[2] / qn), (R)(qq[3] / qn)};
    B.v = v3<R>((R)vv[0], (R)vv[1], (R)vv[2]);
    B.w = v3<R>((R)ww[0], (R)ww[1], (R)ww[2]);
    update_inertia(B);
    for (int64_t j = B.start; j < B.start + B.count; j++) {
      bx[j] = (B.q.rotate(bx0[j].template cast<R>()) + B.x).template cast<F>();
      bv[j] = (B.dyn || B.anim) ? (cross(B.w, bx[j].template cast<R>() - B.x) + B.v).template cast<F>() : V3F::zero();
    }
    return 0;
  }
  int set_time(double tt, int64_t sc) override {
    t = (R)tt;
    step_count = sc;
    return 0;
  }
  int neighbors(int which, int64_t *start, int32_t *idx, int64_t *total) override {
    const std::vector<int64_t> *S; const std::vector<int32_t> *I;
    if (which == DFSPH_NB_FLUID_FLUID) { S = &ffS; I = &ff; }
    else if (which == DFSPH_NB_FLUID_BOUNDARY) { S = &fbS; I = &fb; }
    else if (which == DFSPH_NB_BOUNDARY_FLUID) { S = &bfS; I = &bf; }
    else return DFSPH_ERR_INVALID_ARG;
    if (S->empty()) return DFSPH_ERR_STATE;
    *total = (int64_t)I->size();
    if (start) std::copy(S->begin(), S->end(), start);
    if (idx) std::copy(I->begin(), I->end(), idx);
    return 0;
  }
  int counts(int64_t *a_, int64_t *b_) override { *a_ = nf; *b_ = nbp; return 0; }
  int mgr_grad(int b, int b2, double *out) override {
    const int nb = (int)bodies.size();
    if (b < 0 || b >= nb || b2 < 0 || b2 >= nb) return DFSPH_ERR_INVALID_ARG;
    const MgrState &S = mgrS[b * nb + b2];
    double *o = out;
    o = put(o, S.Gx_v); o = put(o, S.Gx_w); o = put(o, S.Gq_v); o = put(o, S.Gq_w);
    o = put(o, S.Gv_v); o = put(o, S.Gv_w); o = put(o, S.Gw_v); o = put(o, S.Gw_w);
    return 0;
  }
  int mgr_jac(int b, int b2, double *out) override {
    const int nb = (int)bodies.size();
    if (b < 0 || b >= nb || b2 < 0 || b2 >= nb) return DFSPH_ERR_INVALID_ARG;
    const MgrBlk &M = mgrM[b * nb + b2];
    double *o = out;
    o = put(o, M.Fv); o = put(o, M.Fx); o = put(o, M.Fw); o = put(o, M.Fq);
    o = put(o, M.Tw); o = put(o, M.Tv); o = put(o, M.Tx); o = put(o, M.Tq);
    return 0;
  }
  int contact_count(int64_t *nc, int64_t *na) override { *nc = n_contact; *na = n_active; return 0; }
  double time() override { return (double)t; }
};

}  // namespace orc

extern "C" {
// mode: 0 = <float,float>, 1 = <float,double>, 2 = <double,double>
void *orc_create(const dfsph_scene *sc, int mode) {
  try {
    if (mode == 0) return new orc::Sim<float, float>(sc);
    if (mode == 1) return new orc::Sim<float, double>(sc);
    if (mode == 2) return new orc::Sim<double, double>(sc);
  } catch (...) {}
  return nullptr;
}
void orc_destroy(void *s) { delete (orc::Base *)s; }
int orc_set_threads(int n) { if (n > 0) omp_set_num_threads(n); return omp_get_max_threads(); }
int orc_step(void *s, int n, dfsph_step_stats *st) { return ((orc::Base *)s)->step(n, st); }
int orc_copy_field(void *s, int f, double *d) { return ((orc::Base *)s)->copy_field(f, d); }
int orc_set_field(void *s, int f, const double *d) { return ((orc::Base *)s)->set_field(f, d); }
int orc_get_rigid_state(void *s, int b, double *x, double *q, double *v, double *w) { return ((orc::Base *)s)->rigid_state(b, x, q, v, w); }
int orc_get_rigid_force(void *s, int b, double *F, double *T) { return ((orc::Base *)s)->rigid_force(b, F, T); }
int orc_get_rigid_mass(void *s, int b, double *m, double *I) { return ((orc::Base *)s)->rigid_mass(b, m, I); }
int orc_get_rigid_grad(void *s, int b, double *o) { return ((orc::Base *)s)->rigid_grad(b, o); }
int orc_get_net_jacobians(void *s, int b, double *o) { return ((orc::Base *)s)->net_jac(b, o); }
int orc_set_rigid_init(void *s, int b, const double *v, const double *w) { return ((orc::Base *)s)->set_init(b, v, w); }
int orc_set_rigid_velocity(void *s, int b, const double *v, const double *w) { return ((orc::Base *)s)->set_velocity(b, v, w); }
int orc_set_rigid_state(void *s, int b, const double *x, const double *q, const double *v, const double *w) {
  return ((orc::Base *)s)->set_rigid_state(b, x, q, v, w);
}
int orc_set_time(void *s, double t, int64_t sc) { return ((orc::Base *)s)->set_time(t, sc); }
int orc_get_neighbors(void *s, int which, int64_t *st, int32_t *idx, int64_t *tot) { return ((orc::Base *)s)->neighbors(which, st, idx, tot); }
int orc_reset(void *s) { return ((orc::Base *)s)->reset(); }
int orc_reset_gradient(void *s) { return ((orc::Base *)s)->reset_gradient(); }
int orc_num_particles(void *s, int64_t *nf, int64_t *nb) { return ((orc::Base *)s)->counts(nf, nb); }
double orc_get_time(void *s) { return ((orc::Base *)s)->time(); }
int orc_get_manager_grad(void *s, int b, int b2, double *o) { return ((orc::Base *)s)->mgr_grad(b, b2, o); }
int orc_get_manager_jacobians(void *s, int b, int b2, double *o) { return ((orc::Base *)s)->mgr_jac(b, b2, o); }
int orc_get_contact_count(void *s, int64_t *nc, int64_t *na) { return ((orc::Base *)s)->contact_count(nc, na); }

// Kernel probes for the golden-vector pin (double precision kernel with support h).
void orc_kernel_eval(double h, int n, const double *r, double *W, double *gradW, double *gradGradW) {
  orc::Cubic<double> K; K.set(h);
  for (int i = 0; i < n; i++) {
    orc::V3<double> v = orc::v3<double>(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
    W[i] = K.W(v);
    orc::V3<double> g = K.gradW(v);
    for (int c = 0; c < 3; c++) gradW[3 * i + c] = g[c];
    orc::M3<double> H = K.gradGradW(v);
    for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) gradGradW[9 * i + 3 * a + b] = H(a, b);
  }
}
void orc_kernel_eval_f(float h, int n, const float *r, float *W, float *gradW, float *gradGradW) {
  orc::Cubic<float> K; K.set(h);
  for (int i = 0; i < n; i++) {
    orc::V3<float> v = orc::v3<float>(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
    W[i] = K.W(v);
    orc::V3<float> g = K.gradW(v);
    for (int c = 0; c < 3; c++) gradW[3 * i + c] = g[c];
    orc::M3<float> H = K.gradGradW(v);
    for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) gradGradW[9 * i + 3 * a + b] = H(a, b);
  }
}
// Surface-tension kernel probes (cohesion and adhesion, support h) for the golden-vector pin.
void orc_st_kernel_eval(double h, int n, const double *r, double *C, double *A) {
  orc::CohesionK<double> KC; KC.set(h);
  orc::AdhesionK<double> KA; KA.set(h);
  for (int i = 0; i < n; i++) {
    orc::V3<double> v = orc::v3<double>(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
    C[i] = KC.W(v);
    A[i] = KA.W(v);
  }
}
void orc_st_kernel_eval_f(float h, int n, const float *r, float *C, float *A) {
  orc::CohesionK<float> KC; KC.set(h);
  orc::AdhesionK<float> KA; KA.set(h);
  for (int i = 0; i < n; i++) {
    orc::V3<float> v = orc::v3<float>(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
    C[i] = KC.W(v);
    A[i] = KA.W(v);
  }
}
// Quaternion Jacobian probes: q (w,x,y,z), p (3) -> RqP(12), RqTp(12), pq(16) for p=(0,p), wq(12)
void orc_quat_eval(int n, const double *q, const double *p, double *Rqp, double *RqTp, double *pq, double *wq) {
  for (int i = 0; i < n; i++) {
    orc::Quat<double> Q{q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]};
    orc::V3<double> P = orc::v3<double>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    orc::M34<double> a = orc::grad_Rqp_to_q(Q, P), b = orc::grad_RqTp_to_q(Q, P);
    orc::Quat<double> Pq{0.0, P[0], P[1], P[2]};
    orc::M4<double> c = orc::grad_p_q_product_to_q(Pq);
    orc::M43<double> d = orc::grad_omega_q_product_to_omega(Q);
    for (int r = 0; r < 3; r++) for (int s = 0; s < 4; s++) { Rqp[12 * i + 4 * r + s] = a(r, s); RqTp[12 * i + 4 * r + s] = b(r, s); }
    for (int r = 0; r < 4; r++) for (int s = 0; s < 4; s++) pq[16 * i + 4 * r + s] = c(r, s);
    for (int r = 0; r < 4; r++) for (int s = 0; s < 3; s++) wq[12 * i + 3 * r + s] = d(r, s);
  }
}
}
