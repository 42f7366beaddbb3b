// kernels_rigid.cuh — rigid-body side of the step: Akinci2012 pair forces and the
// reference's per-pair gradient Jacobians (boundary-centric, one warp per dynamic
// boundary sample), FP64 per-body reductions, the forward-mode chain rule expressed as
// a 13x13 step matrix, FP64 rigid integration, boundary-sample update and the
// reverse-mode adjoint sweep over the recorded step matrices.
#pragma once
#include "common.cuh"
#include "kernels_fluid.cuh"

namespace dfsph {

// per-dynamic-sample accumulator row: force[3], then the 78 Jacobian entries in the
// order Fv Fx Fw (3x3) Fq (3x4) Tw Tv Tx (3x3) Tq (3x4), row-major; padded to 84.
constexpr int ACC_STRIDE = 84;
constexpr int ACC_FORCE = 0;
constexpr int ACC_JAC = 3;
constexpr int NJAC = 78;
constexpr int NSTATE = 13;  // x(3) q(4: w,x,y,z) v(3) omega(3)

struct BodyState {
  double x[3], q[4], v[3], w[3];
  double mass, invMass;
  double I0[9], I[9], Iinv[9];
  double F[3], T[3];      // net fluid force / torque of the last step (BoundaryModel::getForce/getTorque)
  double nets[NJAC];      // per-step net Jacobians (grad_net_force_to_* / grad_net_torque_to_*)
  double G[NSTATE * 6];   // forward-mode chain state: rows x q v omega, columns v0 (3) omega0 (3)
  // the last velocity step's angular velocity before and after it, and the rotation and
  // world inertia before the position step (the gradient manager's stages read these)
  double wpre[3], wmid[3], qpre[4], Ipre[9], Iipre[9];
  int dyn, anim, dstart, dcount;  // dynamic samples [dstart, dstart + dcount) in body order
  int chain_ran;          // 1 if the last step applied the chain rule
  int pad_;
};

struct RigidConsts {
  double dt, gx, gy, gz;
  int gradient_mode, gyroscopic, optimize_rotation, enable_gradient;
  int manager;  // the gradient manager's multi-body chain replaces the per-body chain
  int nbodies;
};

// ------------------------------------------------------------------ small matrices (T)
template <class T> struct M3 { T a[9]; };
template <class T> struct M34 { T a[12]; };

template <class T> __device__ __forceinline__ void skew3(V3<T> v, T *m) {
  m[0] = T(0); m[1] = -v.z; m[2] = v.y;
  m[3] = v.z; m[4] = T(0); m[5] = -v.x;
  m[6] = -v.y; m[7] = v.x; m[8] = T(0);
}
template <int R, int K, int C, class T> __device__ __forceinline__ void mm(const T *A, const T *B, T *out) {
#pragma unroll
  for (int i = 0; i < R; i++)
#pragma unroll
    for (int j = 0; j < C; j++) {
      T s = A[i * K] * B[j];
#pragma unroll
      for (int k = 1; k < K; k++) s += A[i * K + k] * B[k * C + j];
      out[i * C + j] = s;
    }
}
// out = A * B^T for 3x3
template <class T> __device__ __forceinline__ void mmT3(const T *A, const T *B, T *out) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) out[i * 3 + j] = A[i * 3] * B[j * 3] + A[i * 3 + 1] * B[j * 3 + 1] + A[i * 3 + 2] * B[j * 3 + 2];
}
template <class T> __device__ __forceinline__ void inv3(const T *m, T *r) {
  const T c00 = m[4] * m[8] - m[5] * m[7];
  const T c01 = m[5] * m[6] - m[3] * m[8];
  const T c02 = m[3] * m[7] - m[4] * m[6];
  const T det = m[0] * c00 + m[1] * c01 + m[2] * c02;
  const T id = T(1) / det;
  r[0] = c00 * id; r[1] = (m[2] * m[7] - m[1] * m[8]) * id; r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  r[3] = c01 * id; r[4] = (m[0] * m[8] - m[2] * m[6]) * id; r[5] = (m[3] * m[2] - m[0] * m[5]) * id;
  r[6] = c02 * id; r[7] = (m[6] * m[1] - m[0] * m[7]) * id; r[8] = (m[0] * m[4] - m[3] * m[1]) * id;
}
// d(R(q) p)/dq, columns (w, x, y, z) (GradientUtils.cpp:9-20)
template <class T> __device__ __forceinline__ void grad_Rqp(T qw, T qx, T qy, T qz, V3<T> p, T *out) {
  const V3<T> qv = {qx, qy, qz};
  const V3<T> pc = cross(p, qv);
  const T d = dot(qv, p);
  const T t1[3] = {T(2) * (qw * p.x - pc.x), T(2) * (qw * p.y - pc.y), T(2) * (qw * p.z - pc.z)};
  const T pv[3] = {p.x, p.y, p.z}, qq[3] = {qx, qy, qz};
  T sk[9];
  skew3(p, sk);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    out[i * 4] = t1[i];
#pragma unroll
    for (int j = 0; j < 3; j++)
      out[i * 4 + 1 + j] = T(2) * ((i == j ? d : T(0)) + qq[i] * pv[j] - pv[i] * qq[j] - qw * sk[i * 3 + j]);
  }
}
// d(R(q)^T p)/dq (GradientUtils.cpp:23-35)
template <class T> __device__ __forceinline__ void grad_RqTp(T qw, T qx, T qy, T qz, V3<T> p, T *out) {
  const V3<T> qv = {qx, qy, qz};
  const V3<T> pc = cross(p, qv);
  const T d = dot(qv, p);
  const T t1[3] = {T(2) * (qw * p.x + pc.x), T(2) * (qw * p.y + pc.y), T(2) * (qw * p.z + pc.z)};
  const T pv[3] = {p.x, p.y, p.z}, qq[3] = {qx, qy, qz};
  T sk[9];
  skew3(p, sk);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    out[i * 4] = t1[i];
#pragma unroll
    for (int j = 0; j < 3; j++)
      out[i * 4 + 1 + j] = T(2) * ((i == j ? d : T(0)) + qq[i] * pv[j] - pv[i] * qq[j] + qw * sk[i * 3 + j]);
  }
}

// ------------------------------------------------------------------ pair kernel
template <class T>
struct PairConsts {
  T cReal;    // 1/dt^2 (pressure) or 1/dt (divergence)
  T cTrunc;   // the same, truncated to unsigned as at TimeStepDiffDFSPH.cpp:1266 (or not)
  int optimize_rotation;
  int grad;   // accumulate the pair Jacobians in this launch
};

// One warp per dynamic boundary sample j, lanes over its fluid neighbours i; x[i].w
// carries the stiffness k_i of the current pass.
// Force: the Akinci reaction f_ij = -m_i (-dt k_i (-psi_j grad W_ij)) / dt that the
// fluid-side velocity correction applies (TimeStepDiffDFSPH.cpp:1038-1053, 1139-1196,
// 1767-1784, 1862-1901), only where |k_i| > eps, k_i the pass's stiffness.
// Gradient (GRAD): computeRigidBodyGradient + computeGradient (:1226-1482) with the
// helper derivatives (:1485-1694); the nested neighbour sum of :1632-1694 equals
// -h sum_grad_p_k (pressure) or -sum_grad_p_k (divergence) exactly, because particle
// positions do not change between the factor pass and the solver sweeps.
//
// The Jacobian switch is a launch constant, not a template parameter: one compiled body
// serves both, so the force sums (and hence the forward trajectory) are bit-identical
// whether or not gradients are recorded.
#ifndef DFSPH_PAIR_THREADS
#define DFSPH_PAIR_THREADS 128
#endif
constexpr int PAIR_THREADS = DFSPH_PAIR_THREADS;  // k_pairs: one warp per dynamic sample
template <class T, int MODE>
static __global__ void __launch_bounds__(PAIR_THREADS) k_pairs(FluidConsts<T> c, PairConsts<T> pc, int nd,
                                               const V4<T> *__restrict__ xd, const V4<T> *__restrict__ vd,
                                               const V4<T> *__restrict__ x0d, const int *__restrict__ bodyd,
                                               const BodyState *__restrict__ bs, const int *__restrict__ bflist,
                                               const int *__restrict__ bfcount, const V4<T> *__restrict__ x,
                                               const Rec<T> *__restrict__ R, const T *__restrict__ alpha,
                                               const T *__restrict__ rhoAdv, const V4<T> *__restrict__ sumgrad,
                                               double *__restrict__ acc) {
  const int d = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (d >= nd) return;
  const int b = bodyd[d];
  const BodyState &B = bs[b];
  if (!B.dyn) return;
  const bool grad = pc.grad && !B.anim;
  const V4<T> xj4 = xd[d];
  const V3<T> xj = xyz(xj4);
  const T psi = xj4.w;
  const V3<T> vj = xyz(vd[d]);
  const int cnt = bfcount[d];

  T facc[3] = {T(0), T(0), T(0)};
  T J[NJAC];
#pragma unroll
  for (int k = 0; k < NJAC; k++) J[k] = T(0);

  // per-sample constants of the rotation terms
  T Grq[12], SoG[12], Srj[9];
  V3<T> rj = {T(0), T(0), T(0)};
  if (grad && pc.optimize_rotation) {
    const T qw = (T)B.q[0], qx = (T)B.q[1], qy = (T)B.q[2], qz = (T)B.q[3];
    grad_Rqp(qw, qx, qy, qz, xyz(x0d[d]), Grq);
    T So[9];
    skew3(V3<T>{(T)B.w[0], (T)B.w[1], (T)B.w[2]}, So);
    mm<3, 3, 4>(So, Grq, SoG);
    rj = {xj.x - (T)B.x[0], xj.y - (T)B.x[1], xj.z - (T)B.x[2]};
    skew3(rj, Srj);
  }

  for (int k = lane; k < cnt; k += 32) {
    const int i = DF_INDEX(bflist[(size_t)k * nd + d], c.n, BOUNDS_SAMPLE_LIST);
    const V4<T> xi4 = x[i];  // position and the pass's stiffness k_i
    const V3<T> r = {xi4.x - xj.x, xi4.y - xj.y, xi4.z - xj.z};
    const T rl = sqrt(dot(r, r));
    const V3<T> g = cubic_gradW(r, rl, c.kc);
    const V3<T> gpj = (-psi) * g;
    {
      const T kF = xi4.w;
      if (fabs(kF) > c.eps) {
        const T s = -c.dt * T(1) * kF;
        facc[0] += (-c.m * (s * gpj.x)) * c.invH;
        facc[1] += (-c.m * (s * gpj.y)) * c.invH;
        facc[2] += (-c.m * (s * gpj.z)) * c.invH;
      }
    }
    if (!grad) continue;
    const T ai = alpha[i], ra = rhoAdv[i];
    const T b_i = (MODE == 0) ? ra - T(1) : ra;
    const T ki = b_i * ai * pc.cTrunc;
    const T sT = -c.dt * T(1) * ki;
    const V3<T> fT = {(-c.m * (sT * gpj.x)) * c.invH, (-c.m * (sT * gpj.y)) * c.invH, (-c.m * (sT * gpj.z)) * c.invH};
    const Sym3<T> Hs = cubic_gradGradW(r, rl, c.kc);
    const V3<T> sg = xyz(sumgrad[i]);
    const V3<T> dv = xyz(R[i].v) - vj;
    const bool act = (MODE == 0) ? (ra > T(1)) : (ra > T(0));
    V3<T> gbx = {T(0), T(0), T(0)}, gbv = {T(0), T(0), T(0)}, gbvi = {T(0), T(0), T(0)};
    if (act) {
      const V3<T> Hdv = symmul(Hs, dv);
      if (MODE == 0) {
        gbx = (T(1) / c.rho0) * gpj - (c.dt * psi) * Hdv;
        gbv = (-c.dt * psi) * g;
        gbvi = c.dt * (-sg);
      } else {
        gbx = (-psi) * Hdv;
        gbv = (-psi) * g;
        gbvi = -sg;
      }
    }
    V3<T> gfx = {T(0), T(0), T(0)};
    if (!(ai >= T(0))) gfx = (T(2) * ai * ai) * (psi * symmul(Hs, sg));
    const V3<T> gkx = pc.cReal * (ai * gbx + b_i * gfx);
    const V3<T> gkv = (ai * pc.cReal) * gbv;
    const V3<T> gkvi = (ai * pc.cReal) * gbvi;
    const T gp[3] = {gpj.x, gpj.y, gpj.z};
    const T kx[3] = {gkx.x, gkx.y, gkx.z}, kv[3] = {gkv.x, gkv.y, gkv.z}, kvi[3] = {gkvi.x, gkvi.y, gkvi.z};
    const T g2[9] = {psi * Hs.xx, psi * Hs.xy, psi * Hs.xz, psi * Hs.xy, psi * Hs.yy,
                     psi * Hs.yz, psi * Hs.xz, psi * Hs.yz, psi * Hs.zz};
    T Fx[9], Mv[9], A[9], Ai[9], Fv[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int e = 0; e < 3; e++) {
        const T gvcx = -(gp[a] * kx[e] + ki * g2[a * 3 + e]);
        const T gvcv = -(gp[a] * kv[e]);
        const T gvcvi = -(gp[a] * kvi[e]);
        Fx[a * 3 + e] = -c.m * gvcx;
        Mv[a * 3 + e] = -c.m * gvcv;
        A[a * 3 + e] = (a == e ? T(1) : T(0)) - c.dt * gvcvi;
      }
    inv3(A, Ai);
    mm<3, 3, 3>(Ai, Mv, Fv);
#pragma unroll
    for (int k2 = 0; k2 < 9; k2++) { J[k2] += Fv[k2]; J[9 + k2] += Fx[k2]; }
    if (pc.optimize_rotation) {
      T Fq[12], t12[12], Fw[9], Tw[9], Sf[9], t12b[12];
      mm<3, 3, 4>(Fx, Grq, Fq);
      mm<3, 3, 4>(Fv, SoG, t12);
#pragma unroll
      for (int k2 = 0; k2 < 12; k2++) Fq[k2] += t12[k2];
      mmT3(Fv, Srj, Fw);                       // Fv * skew(rj)^T
      mm<3, 3, 4>(Srj, Fq, t12);               // skew(rj) * Fq
      skew3(fT, Sf);
      T SfT[9] = {Sf[0], Sf[3], Sf[6], Sf[1], Sf[4], Sf[7], Sf[2], Sf[5], Sf[8]};
      mm<3, 3, 4>(SfT, Grq, t12b);             // skew(force)^T * Grq
      mm<3, 3, 3>(Srj, Fw, Tw);
#pragma unroll
      for (int k2 = 0; k2 < 9; k2++) { J[18 + k2] += Fw[k2]; J[39 + k2] += Tw[k2]; }
#pragma unroll
      for (int k2 = 0; k2 < 12; k2++) { J[27 + k2] += Fq[k2]; J[66 + k2] += t12[k2] + t12b[k2]; }
      T Tv[9], Tx[9];
      mm<3, 3, 3>(Srj, Fv, Tv);
      mm<3, 3, 3>(Srj, Fx, Tx);
#pragma unroll
      for (int k2 = 0; k2 < 9; k2++) { J[48 + k2] += Tv[k2]; J[57 + k2] += Tx[k2]; }
    }
  }
  // warp reductions (fixed butterfly order); the sums go through shared memory so that the
  // lanes add them into the FP64 row together (an FP64 warp instruction costs about the same
  // for one active lane as for 32)
  static_assert(ACC_FORCE == 0 && ACC_JAC == 3, "row layout: force, then the Jacobian terms");
  __shared__ T wsum[PAIR_THREADS / 32][3 + NJAC];
  T *ws = wsum[threadIdx.x >> 5];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) facc[k] += __shfl_xor_sync(0xffffffffu, facc[k], o);
    if (lane == 0) ws[ACC_FORCE + k] = facc[k];
  }
  if (grad) {
#pragma unroll
    for (int k = 0; k < NJAC; k++) {
      T s = J[k];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) ws[ACC_JAC + k] = s;
    }
  }
  __syncwarp();
  double *row = acc + (size_t)d * ACC_STRIDE;
  const int nvals = grad ? 3 + NJAC : 3;
  for (int k = lane; k < nvals; k += 32) row[k] += (double)ws[k];
}

// CFL: max squared speed over the fluid records and the samples of dynamic or animated
// bodies, folded into *out as the bits of a non-negative double (ordered like integers).
template <class T>
static __global__ void __launch_bounds__(256) k_max_speed2(int n, const Rec<T> *__restrict__ R, int nd,
                                                           const V4<T> *__restrict__ vd, const int *__restrict__ bodyd,
                                                           const BodyState *__restrict__ bs,
                                                           unsigned long long *__restrict__ out) {
  T m = T(0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V4<T> v = R[i].v;
    const T s = sqnorm_ref(v.x, v.y, v.z);
    m = s > m ? s : m;
  }
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
    const BodyState &B = bs[bodyd[d]];
    if (!(B.dyn || B.anim)) continue;
    const V4<T> v = vd[d];
    const T s = sqnorm_ref(v.x, v.y, v.z);
    m = s > m ? s : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const T q = __shfl_xor_sync(0xffffffffu, m, o);
    m = q > m ? q : m;
  }
  if ((threadIdx.x & 31) == 0) {
    const double md = (double)m;
    atomicMax(out, (unsigned long long)__double_as_longlong(md));
  }
}

// ------------------------------------------------------------------ per-body reduction
// Sums the accumulator rows of every dynamic body's samples in a fixed order, forms the
// torque sum (x_j - x_b) x F_j, stores F, T and the net Jacobians, and zeroes the rows
// (BoundaryModel_Akinci2012::accumulate_and_reset_gradient, :453-497;
// BoundaryModel::getForceAndTorque / clearForceAndTorque, BoundaryModel.cpp:38-85).
// The bodies' reaction to the boundary XSPH term (Viscosity_XSPH.cpp:72-82:
// bm->addForce(x_j, -m_i a_ij)), summed per dynamic sample over its fluid neighbours in
// list order from the velocities before the XSPH update, into the sample's force row.
template <class T>
static __global__ void k_visc_boundary_force(FluidConsts<T> c, int nd, const V4<T> *__restrict__ xd,
                                             const V4<T> *__restrict__ vd, const Rec<T> *__restrict__ R,
                                             const T *__restrict__ rho, const int *__restrict__ bflist,
                                             const int *__restrict__ bfcount, double *__restrict__ acc) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd) return;
  const V4<T> xj = xd[d], vj = vd[d];
  const T fb = -c.invH * c.visc_b;
  T f[3] = {T(0), T(0), T(0)};
  const int cnt = bfcount[d];
  for (int k = 0; k < cnt; k++) {
    const int i = DF_INDEX(bflist[(size_t)k * nd + d], c.n, BOUNDS_SAMPLE_LIST);
    const Rec<T> ri = R[i];
    const T rx = ri.x.x - xj.x, ry = ri.x.y - xj.y, rz = ri.x.z - xj.z;
    const T w = KEval<T>::W(rx * rx + ry * ry + rz * rz, c.kc);
    const T s = fb * (c.rho0 * xj.w / rho[i]);
    f[0] -= c.m * (s * (ri.v.x - vj.x) * w);
    f[1] -= c.m * (s * (ri.v.y - vj.y) * w);
    f[2] -= c.m * (s * (ri.v.z - vj.z) * w);
  }
  double *row = acc + (size_t)d * ACC_STRIDE;
  for (int k = 0; k < 3; k++) row[ACC_FORCE + k] += (double)f[k];
}

// Two stages so that many SMs share the reads: k_body_partials sums each chunk of
// RED_CHUNK consecutive samples of one body in sample order; k_rigid_step then sums a
// body's chunk partials in chunk order.
constexpr int RED_VALUES = 3 + NJAC + 3;  // force, jacobians, torque
constexpr int RED_CHUNK = 16;
constexpr int RED_THREADS = 128;
constexpr int RIGID_THREADS = 384;  // k_rigid_step: one block per body (samples updated in one round up to this count)
static_assert(RED_VALUES <= RED_THREADS, "one thread per reduced value");
struct RedChunk {
  int body, start, count;
};

template <class T>
static __global__ void __launch_bounds__(RED_THREADS) k_body_partials(const BodyState *__restrict__ bs,
                                                                      const RedChunk *__restrict__ chunks,
                                                                      const V4<T> *__restrict__ xd,
                                                                      double *__restrict__ acc,
                                                                      double *__restrict__ part) {
  const RedChunk ch = chunks[blockIdx.x];
  const BodyState &B = bs[ch.body];
  const int v = threadIdx.x;
  // the loads of a batch are issued together, then summed in sample order (FP64 adds have a
  // long dependent latency on this part; the loads should not add theirs to each add)
  constexpr int BATCH = 8;
  static_assert(RED_CHUNK % BATCH == 0, "whole batches per chunk");
  // the torque of each sample's force about the body's position, one sample per thread of
  // the last warp (the FP64 cost is per warp instruction: the lanes share it)
  __shared__ double tq[RED_CHUNK][3];
  static_assert(RED_THREADS - 32 >= RED_VALUES && RED_CHUNK <= 32, "the last warp is free");
  if (v >= RED_THREADS - 32 && v - (RED_THREADS - 32) < ch.count) {
    const int d = ch.start + v - (RED_THREADS - 32);
    const double *row = acc + (size_t)d * ACC_STRIDE;
    const V4<T> xj = xd[d];
    const double rx = (double)xj.x - B.x[0], ry = (double)xj.y - B.x[1], rz = (double)xj.z - B.x[2];
    const double fx = row[0], fy = row[1], fz = row[2];
    double *o = tq[v - (RED_THREADS - 32)];
    o[0] = ry * fz - rz * fy;
    o[1] = rz * fx - rx * fz;
    o[2] = rx * fy - ry * fx;
  }
  __syncthreads();
  if (v < RED_VALUES) {
    double s = 0.0;
    if (v < 3 + NJAC) {
      for (int k0 = 0; k0 < RED_CHUNK; k0 += BATCH) {
        double a[BATCH];
#pragma unroll
        for (int k = 0; k < BATCH; k++)
          a[k] = k0 + k < ch.count ? acc[(size_t)(ch.start + k0 + k) * ACC_STRIDE + v] : 0.0;
#pragma unroll
        for (int k = 0; k < BATCH; k++)
          if (k0 + k < ch.count) s += a[k];
      }
    } else {
      const int comp = v - 3 - NJAC;
      for (int k = 0; k < ch.count; k++) s += tq[k][comp];
    }
    part[(size_t)blockIdx.x * RED_VALUES + v] = s;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < ch.count * ACC_STRIDE; k += blockDim.x) acc[(size_t)ch.start * ACC_STRIDE + k] = 0.0;
}


// ------------------------------------------------------------------ chain rule + integration (FP64)
static __device__ __forceinline__ void q_mul(const double *a, const double *b, double *o) {  // Hamilton, (w,x,y,z)
  o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  o[2] = a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3];
  o[3] = a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1];
}
static __device__ __forceinline__ void q_to_R(const double *q, double *R) {
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = 1 - (tyy + tzz); R[1] = txy - twz; R[2] = txz + twy;
  R[3] = txy + twz; R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
  R[6] = txz - twy; R[7] = tyz + twx; R[8] = 1 - (txx + tyy);
}
static __device__ __forceinline__ void mv3(const double *M, const double *v, double *o) {
  for (int i = 0; i < 3; i++) o[i] = M[3 * i] * v[0] + M[3 * i + 1] * v[1] + M[3 * i + 2] * v[2];
}
static __device__ __forceinline__ void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1]; o[1] = a[2] * b[0] - a[0] * b[2]; o[2] = a[0] * b[1] - a[1] * b[0];
}

// Coefficients of one step's chain update (BoundaryModel_Akinci2012::perform_chain_rule,
// :543-889), shared by the 13 columns.
struct ChainCoef {
  double R[9], I0[9], I[9], Iinv[9], om[3], Iom[3], temp_v[3];
  double gRq_a[12], gRTq_a[12];  // for grad_inertia_v(omega, .)
  double gRq_b[12], gRTq_b[12];  // for grad_inertia_v(Iinv temp_v, .)
  double Gn[16], Gpq[16], Gpw[12];
  double invMass;
};

// gIv(v, Q) = grad_Rqp(q, I0 R^T v) Q + R I0 grad_RqTp(q, v) Q (:513-533) for one column Q.
static __device__ __forceinline__ void gIv_col(const double *gRq, const double *gRTq, const ChainCoef &C, const double *Q,
                                        double *o) {
  double a[3], bq[3], t[3];
  for (int i = 0; i < 3; i++) {
    a[i] = gRq[4 * i] * Q[0] + gRq[4 * i + 1] * Q[1] + gRq[4 * i + 2] * Q[2] + gRq[4 * i + 3] * Q[3];
    bq[i] = gRTq[4 * i] * Q[0] + gRTq[4 * i + 1] * Q[1] + gRTq[4 * i + 2] * Q[2] + gRTq[4 * i + 3] * Q[3];
  }
  mv3(C.I0, bq, t);
  double u[3];
  mv3(C.R, t, u);
  for (int i = 0; i < 3; i++) o[i] = a[i] + u[i];
}

// Applies the chain update to one column s (13) -> o (13).
static __device__ void chain_column(const BodyState &B, const ChainCoef &C, const RigidConsts &rc, const double *s,
                             double *o) {
  const double dt = rc.dt;
  const double *X = s, *Q = s + 3, *Vv = s + 7, *W = s + 10;
  double Xn[3], Vn[3], Wn[3], Qn[4];
  const double *nFv = B.nets, *nFx = B.nets + 9, *nFw = B.nets + 18, *nFq = B.nets + 27;
  const double *nTw = B.nets + 39, *nTv = B.nets + 48, *nTx = B.nets + 57, *nTq = B.nets + 66;
  auto m3v = [](const double *M, const double *v, double *out) { mv3(M, v, out); };
  auto m34v = [](const double *M, const double *v, double *out) {
    for (int i = 0; i < 3; i++) out[i] = M[4 * i] * v[0] + M[4 * i + 1] * v[1] + M[4 * i + 2] * v[2] + M[4 * i + 3] * v[3];
  };
  const bool complete = rc.gradient_mode == 0, rigid_only = rc.gradient_mode == 2;
  if (!rigid_only) {
    double gF[3], t1[3], t2[3];
    m3v(nFv, Vv, gF);
    m3v(nFw, W, t1);
    for (int i = 0; i < 3; i++) gF[i] += t1[i];
    if (complete) {
      m3v(nFx, X, t1); m34v(nFq, Q, t2);
      for (int i = 0; i < 3; i++) gF[i] += t1[i] + t2[i];
    }
    for (int i = 0; i < 3; i++) Vn[i] = Vv[i] + dt * C.invMass * gF[i];
    for (int i = 0; i < 3; i++) Xn[i] = X[i] + dt * Vn[i];
    double gT[3];
    m3v(nTv, Vn, gT);
    m3v(nTw, W, t1);
    for (int i = 0; i < 3; i++) gT[i] += t1[i];
    if (complete) {
      m3v(nTx, Xn, t1); m34v(nTq, Q, t2);
      for (int i = 0; i < 3; i++) gT[i] += t1[i] + t2[i];
    }
    double gTau[3];
    if (rc.gyroscopic) {
      double g1[3], IW[3], gi[3], sum[3], t3[3];
      cross3(C.Iom, W, g1);            // skew(I om) W
      mv3(C.I, W, IW);
      gIv_col(C.gRq_a, C.gRTq_a, C, Q, gi);
      for (int i = 0; i < 3; i++) sum[i] = IW[i] + gi[i];
      cross3(sum, C.om, t3);           // skew(om)^T y = -om x y = y x om
      for (int i = 0; i < 3; i++) gTau[i] = g1[i] + t3[i] + gT[i];
    } else {
      for (int i = 0; i < 3; i++) gTau[i] = gT[i];
    }
    double gII[3], tmp[3], iT[3];
    gIv_col(C.gRq_b, C.gRTq_b, C, Q, tmp);
    mv3(C.Iinv, tmp, gII);
    mv3(C.Iinv, gTau, iT);
    for (int i = 0; i < 3; i++) Wn[i] = W[i] + dt * (gII[i] + iT[i]);
  } else {
    for (int i = 0; i < 3; i++) { Vn[i] = Vv[i]; Xn[i] = X[i] + dt * Vv[i]; }
    if (rc.gyroscopic) {
      double gII[3], tmp[3], g1[3], IW[3], gi[3], sum[3], t3[3], gL[3], iL[3];
      gIv_col(C.gRq_b, C.gRTq_b, C, Q, tmp);
      mv3(C.Iinv, tmp, gII);
      cross3(C.Iom, W, g1);
      mv3(C.I, W, IW);
      gIv_col(C.gRq_a, C.gRTq_a, C, Q, gi);
      for (int i = 0; i < 3; i++) sum[i] = IW[i] + gi[i];
      cross3(sum, C.om, t3);
      for (int i = 0; i < 3; i++) gL[i] = g1[i] + t3[i];
      mv3(C.Iinv, gL, iL);
      for (int i = 0; i < 3; i++) Wn[i] = W[i] + dt * (gII[i] + iL[i]);
    } else {
      for (int i = 0; i < 3; i++) Wn[i] = W[i];
    }
  }
  if (rc.optimize_rotation) {
    double inner[4];
    for (int i = 0; i < 4; i++) {
      double a = C.Gpw[3 * i] * Wn[0] + C.Gpw[3 * i + 1] * Wn[1] + C.Gpw[3 * i + 2] * Wn[2];
      double bq = C.Gpq[4 * i] * Q[0] + C.Gpq[4 * i + 1] * Q[1] + C.Gpq[4 * i + 2] * Q[2] + C.Gpq[4 * i + 3] * Q[3];
      inner[i] = Q[i] + dt / 2.0 * (a + bq);
    }
    for (int i = 0; i < 4; i++)
      Qn[i] = C.Gn[4 * i] * inner[0] + C.Gn[4 * i + 1] * inner[1] + C.Gn[4 * i + 2] * inner[2] + C.Gn[4 * i + 3] * inner[3];
  } else {
    for (int i = 0; i < 4; i++) Qn[i] = Q[i];
  }
  for (int i = 0; i < 3; i++) { o[i] = Xn[i]; o[7 + i] = Vn[i]; o[10 + i] = Wn[i]; }
  for (int i = 0; i < 4; i++) o[3 + i] = Qn[i];
}

static __device__ void grad_Rqp_d(const double *q, const double *p, double *out) {
  grad_Rqp<double>(q[0], q[1], q[2], q[3], V3<double>{p[0], p[1], p[2]}, out);
}
static __device__ void grad_RqTp_d(const double *q, const double *p, double *out) {
  grad_RqTp<double>(q[0], q[1], q[2], q[3], V3<double>{p[0], p[1], p[2]}, out);
}

// SimulatorBase::updateBoundaryParticles (SimulatorBase.cpp:1827-1857) for dynamic
// samples: x_j = R(q) x0_j + x_b, v_j = omega x (x_j - x_b) + v_b, in FP64 then stored in T.
template <class T>
static __device__ __forceinline__ void sample_update(const BodyState &B, int d, const V4<T> *__restrict__ x0d,
                                                     V4<T> *__restrict__ xd, V4<T> *__restrict__ vd) {
  const V4<T> p0 = x0d[d];
  // Quaternion rotation v + w (2 u x v) + u x (2 u x v)
  const double u[3] = {B.q[1], B.q[2], B.q[3]}, pv[3] = {(double)p0.x, (double)p0.y, (double)p0.z};
  double uv[3], uuv[3];
  cross3(u, pv, uv);
  for (int k = 0; k < 3; k++) uv[k] += uv[k];
  cross3(u, uv, uuv);
  double pw[3];
  for (int k = 0; k < 3; k++) pw[k] = pv[k] + B.q[0] * uv[k] + uuv[k] + B.x[k];
  const T xs[3] = {(T)pw[0], (T)pw[1], (T)pw[2]};
  xd[d] = V4<T>{xs[0], xs[1], xs[2], xd[d].w};
  double rr[3] = {(double)xs[0] - B.x[0], (double)xs[1] - B.x[1], (double)xs[2] - B.x[2]}, vv[3];
  cross3(B.w, rr, vv);
  vd[d] = (B.dyn || B.anim) ? V4<T>{(T)(vv[0] + B.v[0]), (T)(vv[1] + B.v[1]), (T)(vv[2] + B.v[2]), T(0)}
                            : V4<T>{T(0), T(0), T(0), T(0)};
}
// Dynamic3dRigidBody::addForce / addTorque (Dynamic3dRigidBody.h:113-142) on a state
// (v, w) with the world inertia I and its inverse.
static __device__ __forceinline__ void body_add_force(double *v, double invMass, const double *f, double dt) {
  for (int k = 0; k < 3; k++) v[k] += invMass * f[k] * dt;
}
static __device__ __forceinline__ void body_add_torque(double *w, const double *I, const double *Iinv,
                                                       const double *tq, bool gyro, double dt) {
  double d[3], L[3], cr[3];
  if (gyro) {
    mv3(I, w, L);
    cross3(L, w, cr);
    for (int k = 0; k < 3; k++) cr[k] += tq[k];
  } else for (int k = 0; k < 3; k++) cr[k] = tq[k];
  mv3(Iinv, cr, d);
  for (int k = 0; k < 3; k++) w[k] += d[k] * dt;
}
// The contact samples' forces and torques of one body applied in sample order (per sample
// body_add_force, then body_add_torque), one vector component per lane of the calling warp
// (lanes 0-2; the others repeat component 0 and write nothing): the same expressions,
// component by component, with the other components fetched by shuffles. FP64 costs about
// the same per warp instruction whatever the number of active lanes, so the lanes cut this
// sequential part's FP64 work to about a third. All 32 lanes of the warp call it.
static __device__ __forceinline__ void body_apply_samples_lanes(double *bv, double *bw, const double *I,
                                                                const double *Iinv, double invMass,
                                                                const double (*ft)[6], int m, bool gyro, double dt) {
  const int lane = threadIdx.x & 31;
  const int r = lane < 3 ? lane : 0;
  double v = bv[r], w = bw[r];
  const double I0 = I[3 * r], I1 = I[3 * r + 1], I2 = I[3 * r + 2];
  const double J0 = Iinv[3 * r], J1 = Iinv[3 * r + 1], J2 = Iinv[3 * r + 2];
  for (int k = 0; k < m; k++) {
    v += invMass * ft[k][r] * dt;
    const double w0 = __shfl_sync(0xffffffffu, w, 0), w1 = __shfl_sync(0xffffffffu, w, 1),
                 w2 = __shfl_sync(0xffffffffu, w, 2);
    double c;
    if (gyro) {
      // cross3(I w, w)[r] = L[r+1] w[r+2] - L[r+2] w[r+1] (indices mod 3)
      const double L = I0 * w0 + I1 * w1 + I2 * w2;
      const double L0 = __shfl_sync(0xffffffffu, L, 0), L1 = __shfl_sync(0xffffffffu, L, 1),
                   L2 = __shfl_sync(0xffffffffu, L, 2);
      const double La = r == 0 ? L1 : (r == 1 ? L2 : L0), Lb = r == 0 ? L2 : (r == 1 ? L0 : L1);
      const double wa = r == 0 ? w1 : (r == 1 ? w2 : w0), wb = r == 0 ? w2 : (r == 1 ? w0 : w1);
      c = La * wb - Lb * wa;
      c += ft[k][3 + r];
    } else {
      c = ft[k][3 + r];
    }
    const double c0 = __shfl_sync(0xffffffffu, c, 0), c1 = __shfl_sync(0xffffffffu, c, 1),
                 c2 = __shfl_sync(0xffffffffu, c, 2);
    const double d = J0 * c0 + J1 * c1 + J2 * c2;
    w += d * dt;
  }
  if (lane < 3) { bv[r] = v; bw[r] = w; }
}

// Dynamic3dRigidBody::animate + updateInertia (Dynamic3dRigidBody.h:143-154, 215-219)
static __device__ __forceinline__ void body_animate(double *x, double *q, double *I, double *Iinv, const double *v,
                                                    const double *w, const double *I0, double dt) {
  for (int k = 0; k < 3; k++) x[k] += v[k] * dt;
  const double wq[4] = {0.0, w[0], w[1], w[2]};
  double dq[4];
  q_mul(wq, q, dq);
  for (int k = 0; k < 4; k++) q[k] += dt * 0.5 * dq[k];
  const double nn = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int k = 0; k < 4; k++) q[k] /= nn;
  double R[9], RI[9], RT[9];
  q_to_R(q, R);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { RT[3 * i + j] = R[3 * j + i]; }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) RI[3 * i + j] = R[3 * i] * I0[j] + R[3 * i + 1] * I0[3 + j] + R[3 * i + 2] * I0[6 + j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) I[3 * i + j] = RI[3 * i] * RT[j] + RI[3 * i + 1] * RT[3 + j] + RI[3 * i + 2] * RT[6 + j];
  inv3<double>(I, Iinv);
}

// Rigid contact of one sample of a dynamic body (kernels_contact.cuh writes these).
constexpr int CONTACT_BLK = 2 * NJAC;  // per force-carrying sample: own-body blocks, other-body blocks
struct ContactRec {
  double f[3], tau[3];  // penalty + friction force and r x f on the sample's body
  int flag;             // 0: no neighbour of another body, 1: contact without force, 2: force
  int RR;               // the other body the cross blocks refer to (the last in point-set order)
};
struct ContactStep {
  const ContactRec *rec;  // per dynamic sample (body order), or null without the contact solver
  const double *blk;      // per dynamic sample CONTACT_BLK Jacobian terms, or null
  int *list;              // scratch: each body's force-carrying samples in order
  int *counts;            // per body: samples in contact, samples with a force
  double *Mc;             // [body][body][NJAC] contact blocks of this step, or null
  double *Mf;             // the gradient manager's blocks: the fluid's diagonal block of each
                          // dynamic, non-animated body goes to [b][b] (null: manager chain off)
};

// exclusive prefix over the block's threads (blockDim.x a multiple of 32, at most 1024)
static __device__ __forceinline__ int block_exclusive_scan(int v, int *warp_tot, int &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int inc = v;
  for (int o = 1; o < 32; o <<= 1) { const int u = __shfl_up_sync(0xffffffffu, inc, o); if (lane >= o) inc += u; }
  __syncthreads();
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  int before = 0;
  total = 0;
  for (int k = 0; k < nw; k++) { if (k < w) before += warp_tot[k]; total += warp_tot[k]; }
  return before + inc - v;
}

// One block per body: RigidBody3dBoundarySimulator::velocityTimeStep (forces,
// gyroscopic torque, gravity; :278-320) and positionTimeStep -> animate (:322-344,
// Dynamic3dRigidBody.h:113-154, 215-235). With the contact solver the velocity step is
// gravity, then each force-carrying contact sample's force and torque in sample order, then
// updateBoundaryForces once per boundary model (RigidBody3dBoundarySimulator.cpp:284-298,
// RigidContactSolver.cpp:347-362); every addForce / addTorque moves the velocities at once and
// every gyroscopic addTorque adds (I w) x w (Dynamic3dRigidBody.h:113-142).
// The body's fluid force, torque and net Jacobians come first: the sums of its chunk
// partials in chunk order (the second stage of the body reduction); the body's samples are
// moved last (SimulatorBase::updateBoundaryParticles). The state before the velocity step is
// kept (wpre, qpre, Ipre, Iipre) and chain_ran marks the bodies whose chain rule
// k_rigid_chain then runs.
template <class T>
static __global__ void __launch_bounds__(RIGID_THREADS) k_rigid_step(BodyState *__restrict__ bs, int nbodies, RigidConsts rc,
                                                    ContactStep cs,
                                                    const int2 *__restrict__ body_chunks,
                                                    const double *__restrict__ red_part,
                                                    const V4<T> *__restrict__ x0d, V4<T> *__restrict__ xd,
                                                    V4<T> *__restrict__ vd) {
  // the body record is worked on in shared memory (the single-thread parts read it
  // many times) and written back at the end
  __shared__ BodyState sB;
  static_assert(sizeof(BodyState) % 8 == 0, "BodyState copies as 8-byte words");
  const int b = blockIdx.x;
  if (b >= nbodies) return;
  const int t = threadIdx.x;
  {
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(bs + b);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(&sB);
    for (int k = t; k < (int)(sizeof(BodyState) / 8); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  BodyState &B = sB;
  if (B.dyn && t < RED_VALUES) {
    const int2 r = body_chunks[b];
    double tot = 0.0;
    for (int c = r.x; c < r.y; c++) tot += red_part[(size_t)c * RED_VALUES + t];
    if (t < 3) B.F[t] = tot;
    else if (t < 3 + NJAC) B.nets[t - 3] = tot;
    else B.T[t - 3 - NJAC] = tot;
  }
  __syncthreads();
  const bool chain = B.dyn && !B.anim && rc.enable_gradient && !rc.manager;
  if (t == 0) B.chain_ran = chain ? 1 : 0;
  // the body's force-carrying contact samples, in sample order (the first CH also in
  // shared memory, with the body each one's cross blocks refer to)
  constexpr int CH = 256;
  __shared__ int warp_tot[32];
  __shared__ int s_con, s_act;
  __shared__ int s_list[CH], s_rr[CH];
  const bool contact = cs.rec != nullptr && B.dyn;
  if (t == 0) { s_con = 0; s_act = 0; }
  __syncthreads();
  if (contact) {
    for (int base = 0; base < B.dcount; base += blockDim.x) {
      const int i = base + t;
      const int flag = i < B.dcount ? cs.rec[B.dstart + i].flag : 0;
      int tot;
      const int pos = block_exclusive_scan(flag == 2 ? 1 : 0, warp_tot, tot);
      if (flag == 2) {
        cs.list[B.dstart + s_act + pos] = B.dstart + i;
        if (s_act + pos < CH) s_list[s_act + pos] = B.dstart + i;
      }
      const int ncon = __syncthreads_count(flag >= 1);
      if (t == 0) { s_act += tot; s_con += ncon; }
      __syncthreads();
    }
  }
  if (t == 0 && cs.counts) { cs.counts[2 * b] = s_con; cs.counts[2 * b + 1] = s_act; }
  const double dt = rc.dt;
  auto add_force = [&](const double *f) { body_add_force(B.v, B.invMass, f, dt); };
  auto add_torque = [&](const double *tq) { body_add_torque(B.w, B.I, B.Iinv, tq, rc.gyroscopic, dt); };
  if (t == 0 && B.dyn) {
    for (int k = 0; k < 3; k++) { B.wpre[k] = B.w[k]; }
    for (int k = 0; k < 4; k++) B.qpre[k] = B.q[k];
    for (int k = 0; k < 9; k++) { B.Ipre[k] = B.I[k]; B.Iipre[k] = B.Iinv[k]; }
    if (cs.rec) {
      const double gm[3] = {rc.gx * B.mass, rc.gy * B.mass, rc.gz * B.mass};
      add_force(gm);
    }
  }
  if (contact) {
    // the force-carrying samples' forces and torques, in sample order; staged in shared
    // memory by all threads so that the sequential part reads no global memory
    __shared__ double sft[CH][6];
    for (int base = 0; base < s_act; base += CH) {
      const int m = min(CH, s_act - base);
      for (int k = t; k < m; k += blockDim.x) {
        const ContactRec &cr = cs.rec[cs.list[B.dstart + base + k]];
        for (int e = 0; e < 3; e++) { sft[k][e] = cr.f[e]; sft[k][3 + e] = cr.tau[e]; }
        if (base == 0) s_rr[k] = cr.RR;
      }
      __syncthreads();
      if (t < 32) body_apply_samples_lanes(B.v, B.w, B.I, B.Iinv, B.invMass, sft, m, rc.gyroscopic, dt);
      __syncthreads();
    }
  }
  if (t == 0 && B.dyn) {
    {
      if (cs.rec) {
        const double zero[3] = {0.0, 0.0, 0.0};
        if (!B.anim)
          for (int rep = 0; rep < rc.nbodies; rep++) {
            add_force(rep == 0 ? B.F : zero);
            add_torque(rep == 0 ? B.T : zero);
          }
      } else if (!B.anim) {
        const double gm[3] = {rc.gx * B.mass, rc.gy * B.mass, rc.gz * B.mass};
        add_force(B.F);
        add_torque(B.T);
        add_force(gm);
      }
      for (int k = 0; k < 3; k++) B.wmid[k] = B.w[k];
      body_animate(B.x, B.q, B.I, B.Iinv, B.v, B.w, B.I0, dt);
    }
  }
  // the contact solver's Jacobian blocks of this body, summed in sample order
  if (cs.Mc) {
    const int nb = rc.nbodies;
    for (int e = t; e < nb * NJAC; e += blockDim.x) {
      const int c = e / NJAC, k = e % NJAC;
      double acc = 0.0;
      if (contact)
        for (int m = 0; m < s_act; m++) {
          const int smp = m < CH ? s_list[m] : cs.list[B.dstart + m];
          if (c == b) acc += cs.blk[(size_t)smp * CONTACT_BLK + k];
          else if ((m < CH ? s_rr[m] : cs.rec[smp].RR) == c) acc += cs.blk[(size_t)smp * CONTACT_BLK + NJAC + k];
        }
      cs.Mc[((size_t)b * nb + c) * NJAC + k] = acc;
    }
  }
  // BoundaryModel_Akinci2012::update_rigid_body_gradient_manager (:952-967): the fluid's
  // net blocks of this body for the manager's fluid stage
  if (cs.Mf && B.dyn && !B.anim)
    for (int e = t; e < NJAC; e += blockDim.x) cs.Mf[((size_t)b * rc.nbodies + b) * NJAC + e] = B.nets[e];
  __syncthreads();
  if (B.dyn || B.anim)
    for (int d = B.dstart + t; d < B.dstart + B.dcount; d += blockDim.x) sample_update(B, d, x0d, xd, vd);
  {
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&sB);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(bs + b);
    for (int k = t; k < (int)(sizeof(BodyState) / 8); k += blockDim.x) dst[k] = src[k];
  }
}

// The chain rule of one step (perform_chain_rule, BoundaryModel_Akinci2012.cpp:543-889) for
// the bodies k_rigid_step marked (chain_ran), from the state the step started from (wpre,
// qpre, Ipre, Iipre) and its reduced net force and torque blocks: the step map A of the
// body's 13 states goes to the tape, G = A G. It runs on its own stream after k_rigid_step:
// the bodies' new states do not wait for it, and it writes only G and the tape. Other
// bodies get an identity tape block.
// FP64 on this part costs about the same per warp instruction whatever the number of
// active lanes, and each of the SM's four sub-partitions issues its own warps' FP64 work:
// independent single-thread pieces run in separate warps between block barriers, and
// lane-parallel work shares a warp:
//   phase 1: coefficients, part A (warp 0)
//   phase 2: coefficients, part B (warps 0-3)
//   phase 3: the 13 columns in the lanes of warp 0
constexpr int CHAIN_THREADS = 128;
static __global__ void __launch_bounds__(CHAIN_THREADS) k_rigid_chain(BodyState *__restrict__ bs, int nbodies,
                                                                      RigidConsts rc, double *__restrict__ tape_step) {
  __shared__ ChainCoef C;
  __shared__ double A[NSTATE * NSTATE];
  __shared__ double Gold[NSTATE * 6];
  __shared__ BodyState sB;
  static_assert(sizeof(BodyState) % 8 == 0, "BodyState copies as 8-byte words");
  const int b = blockIdx.x;
  if (b >= nbodies) return;
  const int t = threadIdx.x;
  {
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(bs + b);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(&sB);
    for (int k = t; k < (int)(sizeof(BodyState) / 8); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  BodyState &B = sB;
  if (!B.chain_ran) {
    if (tape_step)
      for (int k = t; k < NSTATE * NSTATE; k += blockDim.x)
        tape_step[(size_t)b * NSTATE * NSTATE + k] = (k / NSTATE == k % NSTATE) ? 1.0 : 0.0;
    return;
  }
  // the state the step started from
  if (t < 9) { B.I[t] = B.Ipre[t]; B.Iinv[t] = B.Iipre[t]; }
  if (t < 4) B.q[t] = B.qpre[t];
  if (t < 3) B.w[t] = B.wpre[t];
  __syncthreads();
  __shared__ double sVb[3];  // Iinv temp_v
  const int wid = t >> 5, lane = t & 31;
  // ---- phase 1
  {
    if (t == 0) {
      q_to_R(B.q, C.R);
      for (int k = 0; k < 3; k++) C.om[k] = B.w[k];
      mv3(B.I, C.om, C.Iom);
      C.invMass = 1.0 / (B.mass + 1e-10);
      // temp_v (:601, :679, :743)
      if (rc.gradient_mode != 2) {
        if (rc.gyroscopic) { double cr[3]; cross3(C.Iom, C.om, cr); for (int k = 0; k < 3; k++) C.temp_v[k] = cr[k] + B.T[k]; }
        else for (int k = 0; k < 3; k++) C.temp_v[k] = B.T[k];
      } else {
        if (rc.gyroscopic) cross3(C.Iom, C.om, C.temp_v);
        else for (int k = 0; k < 3; k++) C.temp_v[k] = 0.0;
      }
      mv3(B.Iinv, C.temp_v, sVb);
    } else if (wid == 1 && lane < 9) {
      C.I0[lane] = B.I0[lane]; C.I[lane] = B.I[lane]; C.Iinv[lane] = B.Iinv[lane];
    }
    for (int k = t; k < NSTATE * 6; k += blockDim.x) Gold[k] = B.G[k];
  }
  __syncthreads();
  // ---- phase 2
  if (lane == 0 && wid < 4) {
    // grad_inertia_v operands: v = omega (a) and v = Iinv temp_v (b)
    const double RT[9] = {C.R[0], C.R[3], C.R[6], C.R[1], C.R[4], C.R[7], C.R[2], C.R[5], C.R[8]};
    const double *va = C.om, *vb = sVb;
    double tmp[3], tmp2[3];
    if (wid == 0) {
      mv3(RT, va, tmp); mv3(B.I0, tmp, tmp2); grad_Rqp_d(B.q, tmp2, C.gRq_a);
    } else if (wid == 1) {
      grad_RqTp_d(B.q, va, C.gRTq_a); grad_RqTp_d(B.q, vb, C.gRTq_b);
    } else if (wid == 2) {
      mv3(RT, vb, tmp); mv3(B.I0, tmp, tmp2); grad_Rqp_d(B.q, tmp2, C.gRq_b);
    } else {
      // rotation block (:827-888)
      double nom[3];
      for (int k = 0; k < 3; k++) nom[k] = C.om[k] + rc.dt * vb[k];
      const double p[4] = {0.0, nom[0], nom[1], nom[2]};
      double pq[4], nq[4];
      q_mul(p, B.q, pq);
      for (int k = 0; k < 4; k++) nq[k] = B.q[k] + rc.dt * 0.5 * pq[k];
      const double nn = sqrt(nq[0] * nq[0] + nq[1] * nq[1] + nq[2] * nq[2] + nq[3] * nq[3]);
      double nv[4];
      for (int k = 0; k < 4; k++) nv[k] = nq[k] / nn;
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) C.Gn[4 * i + j] = ((i == j ? 1.0 : 0.0) - nv[i] * nv[j]) / nn;
      const double Gpq[16] = {p[0], -p[1], -p[2], -p[3], p[1], p[0], -p[3], p[2],
                              p[2], p[3], p[0], -p[1], p[3], -p[2], p[1], p[0]};
      for (int k = 0; k < 16; k++) C.Gpq[k] = Gpq[k];
      const double *q = B.q;
      const double Gpw[12] = {-q[1], -q[2], -q[3], q[0], q[3], -q[2], -q[3], q[0], q[1], q[2], -q[1], q[0]};
      for (int k = 0; k < 12; k++) C.Gpw[k] = Gpw[k];
    }
  }
  __syncthreads();
  // ---- phase 3
  {
    // the columns in the lanes of one warp: an FP64 warp instruction costs the same with 13
    // active lanes as with one, so more warps would only queue on the FP64 units
    if (t < NSTATE) {
      double e[NSTATE], col[NSTATE];
      for (int k = 0; k < NSTATE; k++) e[k] = (k == t) ? 1.0 : 0.0;
      chain_column(B, C, rc, e, col);
      for (int k = 0; k < NSTATE; k++) A[k * NSTATE + t] = col[k];
    }
    __syncthreads();
    for (int k = t; k < NSTATE * 6; k += blockDim.x) {
      const int r = k / 6, cc = k % 6;
      double s = 0.0;
      for (int m = 0; m < NSTATE; m++) s += A[r * NSTATE + m] * Gold[m * 6 + cc];
      B.G[k] = s;
    }
    if (tape_step)
      for (int k = t; k < NSTATE * NSTATE; k += blockDim.x) tape_step[(size_t)b * NSTATE * NSTATE + k] = A[k];
    __syncthreads();
  }
  for (int k = t; k < NSTATE * 6; k += blockDim.x) bs[b].G[k] = B.G[k];
}

// TimeStepDiffDFSPH::beginStep velocity overrides (:379-429), decided on the host.
struct BeginCmd {
  int n;
  int set[DFSPH_MAX_BODIES_DEV];
  int anim[DFSPH_MAX_BODIES_DEV];
  double v[DFSPH_MAX_BODIES_DEV][3];
  double w[DFSPH_MAX_BODIES_DEV][3];
};

static __global__ void k_rigid_begin(BodyState *__restrict__ bs, BeginCmd cmd) {
  const int b = threadIdx.x;
  if (b >= cmd.n) return;
  BodyState &B = bs[b];
  if (!B.dyn) return;
  B.anim = cmd.anim[b];
  if (cmd.set[b]) {
    for (int k = 0; k < 3; k++) { B.v[k] = cmd.v[b][k]; B.w[k] = cmd.w[b][k]; }
  }
}

template <class T>
static __global__ void k_boundary_update(const BodyState *__restrict__ bs, int nd, const V4<T> *__restrict__ x0d,
                                  const int *__restrict__ bodyd, V4<T> *__restrict__ xd, V4<T> *__restrict__ vd,
                                  int only_moving) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd) return;
  const BodyState &B = bs[bodyd[d]];
  if (only_moving && !(B.dyn || B.anim)) return;
  sample_update(B, d, x0d, xd, vd);
}

// Reverse sweep: lambda <- A_n^T lambda for n = last..first, one block per body.
static __global__ void k_backward(const double *__restrict__ tape, int nsteps, int nbodies, const double *__restrict__ lam_in,
                           double *__restrict__ lam_out) {
  __shared__ double lam[NSTATE], nl[NSTATE];
  const int b = blockIdx.x, t = threadIdx.x;
  if (b >= nbodies) return;
  if (t < NSTATE) lam[t] = lam_in[b * NSTATE + t];
  __syncthreads();
  for (int n = nsteps - 1; n >= 0; n--) {
    const double *A = tape + ((size_t)n * nbodies + b) * NSTATE * NSTATE;
    if (t < NSTATE) {
      double s = 0.0;
      for (int k = 0; k < NSTATE; k++) s += A[k * NSTATE + t] * lam[k];
      nl[t] = s;
    }
    __syncthreads();
    if (t < NSTATE) lam[t] = nl[t];
    __syncthreads();
  }
  if (t < NSTATE) lam_out[b * NSTATE + t] = lam[t];
}

}  // namespace dfsph
