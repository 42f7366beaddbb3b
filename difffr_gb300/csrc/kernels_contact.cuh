// kernels_contact.cuh — rigid-rigid contact and the multi-body gradient chain, FP64.
//
//  - k_contact_rest / k_contact_samples: the InterlinkedSPH RigidContactSolver in the penalty
//    form the reference runs (use_penalty_force is fixed on, RigidContactSolver.cpp:28):
//    rest volume and rest density of every boundary sample from its own body (:216-258), and
//    per sample of a dynamic body with a neighbour of another body its contact density,
//    penalty normal force, Coulomb friction and the Jacobian blocks of that force
//    (beforePenaltyInitialize :307-345, solveRigidContactPenalty :419-555).
//  - k_manager_coef / k_manager_columns / k_manager_blocks: RigidBodyGradientManager's
//    forward chain over body pairs [R][RR] (RigidBodyGradientManager.cpp:96-468), its step
//    maps for the reverse sweep, and the blocks carried into the next step.
#pragma once
#include "kernels_fluid.cuh"
#include "kernels_rigid.cuh"

namespace dfsph {

struct ContactConsts {
  Cubic<double> kc;  // contact kernel, support rigidContactSupportRadiusFactor * r
  Cubic<double> kh;  // the simulation's kernel (support h), used for the density gradient (:456-460)
  double beta, mu, dt, gx, gy, gz;
  int grad;
};

// vel[R][r] of a sample (RigidContactSolver.cpp:313-316): the body's velocities after the
// velocity step's gravity (added before the contact solver, RigidBody3dBoundarySimulator.cpp:
// 286-295); samples of static bodies keep zero.
static __device__ __forceinline__ void sample_velocity(const BodyState &B, const ContactConsts &c, const double *x,
                                                       double *out) {
  if (!(B.dyn || B.anim)) { out[0] = out[1] = out[2] = 0.0; return; }
  double v[3] = {B.v[0], B.v[1], B.v[2]};
  if (B.dyn) {
    const double g[3] = {c.gx, c.gy, c.gz};
    for (int k = 0; k < 3; k++) v[k] += B.invMass * (g[k] * B.mass) * c.dt;
  }
  const double r[3] = {x[0] - B.x[0], x[1] - B.x[1], x[2] - B.x[2]};
  double wr[3];
  cross3(B.w, r, wr);
  for (int k = 0; k < 3; k++) out[k] = v[k] + wr[k];
}

// Rest volume (phase 0) and rest density (phase 1) of every boundary sample p (static in
// their sorted order, then the dynamic ones in the current cell-sorted order) from the
// neighbours of its own body (RigidContactSolver.cpp:216-258); dynamic results are stored
// by body-order index so they survive later sorts.
template <class T>
static __global__ void k_contact_rest(ContactConsts c, Grid<T> g, T h2, int ns, int nd, const Rec<T> *__restrict__ BR,
                                      const int *__restrict__ cstartS, const int *__restrict__ cstartD,
                                      const int *__restrict__ bodyS, const int *__restrict__ bodyd,
                                      const int *__restrict__ dynSortedToBody, double gamma, int phase,
                                      double *__restrict__ vol0S, double *__restrict__ vol0D,
                                      double *__restrict__ dens0S, double *__restrict__ dens0D) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ns + nd) return;
  const V4<T> xp = BR[p].x;
  const int bp = p < ns ? bodyS[p] : bodyd[dynSortedToBody[p - ns]];
  int cx, cy, cz;
  grid_cell(g, xp.x, xp.y, xp.z, cx, cy, cz);
  double acc = phase == 0 ? c.kc.w0 : 0.0;
  auto visit = [&](int b, int e, int off) {
    for (int j = b; j < e; j++) {
      if (off + j == p) continue;
      const V4<T> xj = BR[off + j].x;
      if (!(dist2_rn(xp.x - xj.x, xp.y - xj.y, xp.z - xj.z) < h2)) continue;
      const int bj = off == 0 ? bodyS[j] : bodyd[dynSortedToBody[j]];
      if (bj != bp) continue;
      const double dx = (double)xp.x - (double)xj.x, dy = (double)xp.y - (double)xj.y, dz = (double)xp.z - (double)xj.z;
      const double w = cubic_W(sqrt(dist2_rn(dx, dy, dz)), c.kc);
      if (phase == 0) acc += w;
      else acc += (off == 0 ? vol0S[j] : vol0D[dynSortedToBody[j]]) * w;
    }
  };
  if (ns > 0) for_each_row(g, cstartS, cx, cy, cz, [&](int b, int e) { visit(b, e, 0); }, ns);
  if (nd > 0) for_each_row(g, cstartD, cx, cy, cz, [&](int b, int e) { visit(b, e, ns); }, nd);
  if (phase == 0) {
    const double v0 = gamma / acc;
    if (p < ns) vol0S[p] = v0; else vol0D[dynSortedToBody[p - ns]] = v0;
  } else {
    const double v0 = p < ns ? vol0S[p] : vol0D[dynSortedToBody[p - ns]];
    const double d0 = v0 * c.kc.w0 + acc;
    if (p < ns) dens0S[p] = d0; else dens0D[dynSortedToBody[p - ns]] = d0;
  }
}

// CONTACT_LANES lanes per sample of a dynamic body (body order): they split the candidate
// rows and combine their sums with shuffles, then split the Jacobian blocks of the sample's
// force between them; the result is the sample's contact record and, when gradients are on,
// the blocks for its own body [R][R] and the other body [R][RR], in the
// dfsph_get_net_jacobians layout (Fv Fx Fw Fq Tw Tv Tx Tq). FP64 runs at a low rate on this
// part, so the work is spread over many SMs rather than one thread per sample.
constexpr int CONTACT_LANES = 8;
template <class T>
static __global__ void __launch_bounds__(128) k_contact_samples(
    ContactConsts c, Grid<T> g, T h2, int ns, int nd, const BodyState *__restrict__ bs, const Rec<T> *__restrict__ BR,
    const int *__restrict__ cstartS, const int *__restrict__ cstartD, const int *__restrict__ bodyS,
    const V4<T> *__restrict__ x0S, const int *__restrict__ bodyd, const int *__restrict__ dynSortedToBody,
    const V4<T> *__restrict__ xd, const V4<T> *__restrict__ x0d, const double *__restrict__ vol0S,
    const double *__restrict__ vol0D, const double *__restrict__ dens0D, ContactRec *__restrict__ rec,
    double *__restrict__ blk) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int d = gt / CONTACT_LANES, sub = gt % CONTACT_LANES;
  const bool live = d < nd;
  const int dd = live ? d : 0;
  const int b = bodyd[dd];
  const BodyState &B = bs[b];
  const V4<T> xT = xd[dd];
  const double xr[3] = {(double)xT.x, (double)xT.y, (double)xT.z};
  double dens = 0.0;
  double sum_x[3] = {0, 0, 0}, sum_vk[3] = {0, 0, 0}, avg_rk[3] = {0, 0, 0}, gdx[3] = {0, 0, 0};
  double gdqk[4] = {0, 0, 0, 0};
  double sum_w = 0.0;
  int has = 0, RR = -1;
  if (live && B.dyn) {
    int cx, cy, cz;
    grid_cell(g, xT.x, xT.y, xT.z, cx, cy, cz);
    auto visit = [&](int jb, int je, int off) {
      for (int j = jb + sub; j < je; j += CONTACT_LANES) {
        int o = -1, bk;
        if (off == 0) bk = bodyS[j];
        else { o = dynSortedToBody[j]; if (o == dd) continue; bk = bodyd[o]; }
        const V4<T> xkT = BR[off + j].x;
        if (!(dist2_rn(xT.x - xkT.x, xT.y - xkT.y, xT.z - xkT.z) < h2)) continue;
        const double xk[3] = {(double)xkT.x, (double)xkT.y, (double)xkT.z};
        const double rv[3] = {xr[0] - xk[0], xr[1] - xk[1], xr[2] - xk[2]};
        const double rl = sqrt(dist2_rn(rv[0], rv[1], rv[2]));
        const double w = cubic_W(rl, c.kc);
        const double vol = off == 0 ? vol0S[j] : vol0D[o];
        dens += vol * w;
        if (bk == b) {
          for (int k = 0; k < 3; k++) sum_x[k] += xk[k] * w;
          sum_w += w;
        } else {
          has = 1;
          RR = bk > RR ? bk : RR;
          const BodyState &C = bs[bk];
          double vk[3];
          sample_velocity(C, c, xk, vk);
          for (int k = 0; k < 3; k++) { sum_vk[k] += vk[k] * w; avg_rk[k] += (xk[k] - C.x[k]) * w; }
          const V3<double> gw = cubic_gradW(V3<double>{rv[0], rv[1], rv[2]}, rl, c.kh);
          const double gv[3] = {vol * gw.x, vol * gw.y, vol * gw.z};
          for (int k = 0; k < 3; k++) gdx[k] += gv[k];
          if (c.grad) {
            const V4<T> p0 = off == 0 ? x0S[j] : x0d[o];
            double Gk[12];
            grad_Rqp<double>(C.q[0], C.q[1], C.q[2], C.q[3], V3<double>{(double)p0.x, (double)p0.y, (double)p0.z}, Gk);
            for (int q = 0; q < 4; q++) gdqk[q] -= gv[0] * Gk[q] + gv[1] * Gk[4 + q] + gv[2] * Gk[8 + q];
          }
        }
      }
    };
    if (ns > 0) for_each_row(g, cstartS, cx, cy, cz, [&](int jb, int je) { visit(jb, je, 0); }, ns);
    for_each_row(g, cstartD, cx, cy, cz, [&](int jb, int je) { visit(jb, je, ns); }, nd);
  }
  // combine the lanes' sums (fixed butterfly order)
  auto red = [](double &v) {
#pragma unroll
    for (int o = CONTACT_LANES / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  };
  red(dens); red(sum_w);
  for (int k = 0; k < 3; k++) { red(sum_x[k]); red(sum_vk[k]); red(avg_rk[k]); red(gdx[k]); }
  for (int k = 0; k < 4; k++) red(gdqk[k]);
#pragma unroll
  for (int o = CONTACT_LANES / 2; o > 0; o >>= 1) {
    has |= __shfl_xor_sync(0xffffffffu, has, o);
    const int r2 = __shfl_xor_sync(0xffffffffu, RR, o);
    RR = r2 > RR ? r2 : RR;
  }
  if (!live) return;
  ContactRec out;
  out.flag = 0;
  out.RR = b;
  for (int k = 0; k < 3; k++) out.f[k] = out.tau[k] = 0.0;
  if (!B.dyn || !has) { if (sub == 0) rec[dd] = out; return; }
  dens += vol0D[dd] * c.kc.w0;
  out.flag = 1;
  out.RR = RR;
  const double ratio = dens / dens0D[dd];
  if (!(ratio > 1.0)) { if (sub == 0) rec[dd] = out; return; }
  out.flag = 2;
  double normal[3], vrel[3], vr[3];
  sample_velocity(B, c, xr, vr);
  for (int k = 0; k < 3; k++) {
    normal[k] = xr[k] - sum_x[k] / sum_w;
    vrel[k] = vr[k] - sum_vk[k] / sum_w;
    avg_rk[k] = avg_rk[k] / sum_w;
  }
  const double mag = fmax(ratio - 1.0, 0.0);
  double Fn[3], u[3], f[3];
  for (int k = 0; k < 3; k++) Fn[k] = -c.beta * mag * normal[k];
  const double vz = vrel[0] * vrel[0] + vrel[1] * vrel[1] + vrel[2] * vrel[2];
  const double vn = sqrt(vz);
  for (int k = 0; k < 3; k++) u[k] = vz > 0.0 ? vrel[k] / vn : vrel[k];  // Eigen's normalized()
  const double fnn = sqrt(Fn[0] * Fn[0] + Fn[1] * Fn[1] + Fn[2] * Fn[2]);
  for (int k = 0; k < 3; k++) f[k] = Fn[k] + (-c.mu * fnn) * u[k];
  const double rr[3] = {xr[0] - B.x[0], xr[1] - B.x[1], xr[2] - B.x[2]};
  double tau[3];
  cross3(rr, f, tau);
  for (int k = 0; k < 3; k++) { out.f[k] = f[k]; out.tau[k] = tau[k]; }
  if (sub == 0) rec[dd] = out;
  if (!c.grad) return;
  // ---- Jacobian blocks (RigidContactSolver.cpp:467-552), split between the lanes
  double *D = blk + (size_t)dd * CONTACT_BLK, *X = D + NJAC;
  double gFn_d[3], gFf_d[3], gd[3];
  for (int k = 0; k < 3; k++) gFn_d[k] = -c.beta * normal[k];
  {
    const double fd = Fn[0] * gFn_d[0] + Fn[1] * gFn_d[1] + Fn[2] * gFn_d[2];
    for (int k = 0; k < 3; k++) gFf_d[k] = (-c.mu * u[k]) * fd / fnn;
  }
  for (int k = 0; k < 3; k++) gd[k] = gFn_d[k] + gFf_d[k];  // d(normal + friction force) / d(density)
  double gFf_vr[9];
  {
    const double sc = (-c.mu * fnn) / vn;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) gFf_vr[3 * i + j] = sc * ((i == j ? 1.0 : 0.0) - u[i] * u[j]);
  }
  double Sr[9];
  skew3(V3<double>{rr[0], rr[1], rr[2]}, Sr);
  double gfx[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) gfx[3 * i + j] = gd[i] * gdx[j];
  double *DFv = D, *DFx = D + 9, *DFw = D + 18, *DFq = D + 27, *DTw = D + 39, *DTv = D + 48, *DTx = D + 57,
         *DTq = D + 66;
  double *XFv = X, *XFx = X + 9, *XFw = X + 18, *XFq = X + 27, *XTw = X + 39, *XTv = X + 48, *XTx = X + 57,
         *XTq = X + 66;
  switch (sub) {
    case 0:
      for (int k = 0; k < 9; k++) { DFx[k] = gfx[k]; DFv[k] = gFf_vr[k]; XFv[k] = -gFf_vr[k]; XFx[k] = -gfx[k]; }
      break;
    case 1: {
      mm<3, 3, 3>(Sr, gfx, DTx);
      for (int k = 0; k < 9; k++) XTx[k] = -DTx[k];
      break;
    }
    case 2:
    case 3:
    case 4: {
      const V4<T> p0 = x0d[dd];
      double GqB[12], gdq[4];
      grad_Rqp<double>(B.q[0], B.q[1], B.q[2], B.q[3], V3<double>{(double)p0.x, (double)p0.y, (double)p0.z}, GqB);
      for (int q = 0; q < 4; q++) gdq[q] = gdx[0] * GqB[q] + gdx[1] * GqB[4 + q] + gdx[2] * GqB[8 + q];
      if (sub == 2) {
        for (int i = 0; i < 3; i++)
          for (int q = 0; q < 4; q++) { DFq[4 * i + q] = gd[i] * gdq[q]; XFq[4 * i + q] = gd[i] * gdqk[q]; }
      } else if (sub == 3) {  // Tq = skew(r) gfq + skew(f)^T GqB
        double gfq[12], a[12], Sf[9], SfT[9], b2[12];
        for (int i = 0; i < 3; i++)
          for (int q = 0; q < 4; q++) gfq[4 * i + q] = gd[i] * gdq[q];
        mm<3, 3, 4>(Sr, gfq, a);
        skew3(V3<double>{f[0], f[1], f[2]}, Sf);
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) SfT[3 * i + j] = Sf[3 * j + i];
        mm<3, 3, 4>(SfT, GqB, b2);
        for (int k = 0; k < 12; k++) DTq[k] = a[k] + b2[k];
      } else {  // cross Tq = skew(r) gfqk
        double gfqk[12];
        for (int i = 0; i < 3; i++)
          for (int q = 0; q < 4; q++) gfqk[4 * i + q] = gd[i] * gdqk[q];
        mm<3, 3, 4>(Sr, gfqk, XTq);
      }
      break;
    }
    case 5: {  // Fw = gFf_vr skew(r)^T, cross Fw = -gFf_vr skew(avg_rk)^T
      double Sa[9], t9[9];
      skew3(V3<double>{avg_rk[0], avg_rk[1], avg_rk[2]}, Sa);
      mmT3(gFf_vr, Sr, DFw);
      mmT3(gFf_vr, Sa, t9);
      for (int k = 0; k < 9; k++) XFw[k] = -t9[k];
      break;
    }
    default:  // the torque-to-v / omega blocks of the contact force are zero
      for (int k = 0; k < 9; k++) { DTw[k] = 0.0; DTv[k] = 0.0; XTw[k] = 0.0; XTv[k] = 0.0; }
      break;
  }
}

// ------------------------------------------------------------------ gradient manager
// Per-body coefficients of one step's manager chain: the fluid stage with the angular
// velocity before the velocity step and the fluid torque, the contact stage with the
// angular velocity after it and no torque, the rotation stage with the angular velocity
// after it and the rotation before the position step.
struct MgrCoef {
  double invMass;
  double I[9], Iinv[9], R[9], I0[9];
  double Iom2[3], om2[3], gRq_a2[12], gRTq_a2[12], gRq_b2[12], gRTq_b2[12];
  double Iom3[3], om3[3], gRq_a3[12], gRTq_a3[12], gRq_b3[12], gRTq_b3[12];
  double Gn[16], Gpq[16], Gpw[12];
  int dyn;
};

struct MgrConsts {
  double dt;
  int nb, gyroscopic, fluid_stage, contact_stage;
  int chain;  // 0: only carry the contact blocks forward (gradients off), 1: advance the chain too
};

static __device__ __forceinline__ void gIv_mgr(const double *gRq, const double *gRTq, const MgrCoef &C,
                                               const double *Q, double *o) {
  double a[3], bq[3], t[3], u[3];
  for (int i = 0; i < 3; i++) {
    a[i] = gRq[4 * i] * Q[0] + gRq[4 * i + 1] * Q[1] + gRq[4 * i + 2] * Q[2] + gRq[4 * i + 3] * Q[3];
    bq[i] = gRTq[4 * i] * Q[0] + gRTq[4 * i + 1] * Q[1] + gRTq[4 * i + 2] * Q[2] + gRTq[4 * i + 3] * Q[3];
  }
  mv3(C.I0, bq, t);
  mv3(C.R, t, u);
  for (int i = 0; i < 3; i++) o[i] = a[i] + u[i];
}

// perform_velocity_chain_rule (:292-393) on body a's part of a column
static __device__ void mgr_velocity(const MgrCoef &C, bool gyro, double dt, const double *dF, const double *dT,
                                    double *s, bool contact_stage) {
  double *Q = s + 3, *Vv = s + 7, *W = s + 10;
  for (int i = 0; i < 3; i++) Vv[i] += dt * C.invMass * dF[i];
  const double *Iom = contact_stage ? C.Iom3 : C.Iom2, *om = contact_stage ? C.om3 : C.om2;
  const double *gRq_a = contact_stage ? C.gRq_a3 : C.gRq_a2, *gRTq_a = contact_stage ? C.gRTq_a3 : C.gRTq_a2;
  const double *gRq_b = contact_stage ? C.gRq_b3 : C.gRq_b2, *gRTq_b = contact_stage ? C.gRTq_b3 : C.gRTq_b2;
  double gTau[3];
  if (gyro) {
    double g1[3], IW[3], gi[3], sum[3], t3[3];
    cross3(Iom, W, g1);  // skew(I om) W
    mv3(C.I, W, IW);
    gIv_mgr(gRq_a, gRTq_a, C, Q, gi);
    for (int i = 0; i < 3; i++) sum[i] = IW[i] + gi[i];
    cross3(sum, om, t3);  // skew(om)^T y = y x om
    for (int i = 0; i < 3; i++) gTau[i] = g1[i] + t3[i] + dT[i];
  } else {
    for (int i = 0; i < 3; i++) gTau[i] = dT[i];
  }
  double tmp[3], gII[3], iT[3];
  gIv_mgr(gRq_b, gRTq_b, C, Q, tmp);
  mv3(C.Iinv, tmp, gII);
  mv3(C.Iinv, gTau, iT);
  for (int i = 0; i < 3; i++) W[i] += dt * (gII[i] + iT[i]);
}

// One column (13 per body) through the step: the fluid stage (force chain :96-156 with the
// v / omega blocks, velocity chain), the contact stage (force chain with the x / q blocks
// too, the q blocks only in the omega0 columns, :158-290; velocity chain), then the position
// and rotation chain (:395-453).
static __device__ void mgr_apply(const MgrCoef *Cs, const MgrConsts &mc, const double *M, const double *Mc,
                                 double *s, bool wcol) {
  const int nb = mc.nb;
  double dF[3 * DFSPH_MAX_BODIES_DEV], dT[3 * DFSPH_MAX_BODIES_DEV];
  auto mv3x = [](const double *A, const double *v, double *o) {
    for (int i = 0; i < 3; i++) o[i] += A[3 * i] * v[0] + A[3 * i + 1] * v[1] + A[3 * i + 2] * v[2];
  };
  auto mv34x = [](const double *A, const double *v, double *o) {
    for (int i = 0; i < 3; i++) o[i] += A[4 * i] * v[0] + A[4 * i + 1] * v[1] + A[4 * i + 2] * v[2] + A[4 * i + 3] * v[3];
  };
  for (int stage = 0; stage < 2; stage++) {
    if (stage == 0 && !mc.fluid_stage) continue;
    if (stage == 1 && !mc.contact_stage) continue;
    const double *B = stage == 0 ? M : Mc;
    for (int a = 0; a < nb; a++) {
      for (int i = 0; i < 3; i++) dF[3 * a + i] = dT[3 * a + i] = 0.0;
      if (!Cs[a].dyn) continue;
      for (int k = 0; k < nb; k++) {
        if (!Cs[k].dyn) continue;
        const double *J = B + ((size_t)a * nb + k) * NJAC;
        const double *sk = s + NSTATE * k;
        const double *Fv = J, *Fx = J + 9, *Fw = J + 18, *Fq = J + 27, *Tw = J + 39, *Tv = J + 48, *Tx = J + 57,
                     *Tq = J + 66;
        mv3x(Fv, sk + 7, dF + 3 * a); mv3x(Fw, sk + 10, dF + 3 * a);
        mv3x(Tv, sk + 7, dT + 3 * a); mv3x(Tw, sk + 10, dT + 3 * a);
        if (stage == 1) {
          mv3x(Fx, sk, dF + 3 * a); mv3x(Tx, sk, dT + 3 * a);
          if (wcol) { mv34x(Fq, sk + 3, dF + 3 * a); mv34x(Tq, sk + 3, dT + 3 * a); }
        }
      }
    }
    for (int a = 0; a < nb; a++)
      if (Cs[a].dyn) mgr_velocity(Cs[a], mc.gyroscopic, mc.dt, dF + 3 * a, dT + 3 * a, s + NSTATE * a, stage == 1);
  }
  for (int a = 0; a < nb; a++) {
    if (!Cs[a].dyn) continue;
    const MgrCoef &C = Cs[a];
    double *X = s + NSTATE * a, *Q = X + 3, *Vv = X + 7, *W = X + 10;
    for (int i = 0; i < 3; i++) X[i] += mc.dt * Vv[i];
    double inner[4], Qn[4];
    for (int i = 0; i < 4; i++) {
      const double aw = C.Gpw[3 * i] * W[0] + C.Gpw[3 * i + 1] * W[1] + C.Gpw[3 * i + 2] * W[2];
      const double bq = C.Gpq[4 * i] * Q[0] + C.Gpq[4 * i + 1] * Q[1] + C.Gpq[4 * i + 2] * Q[2] + C.Gpq[4 * i + 3] * Q[3];
      inner[i] = Q[i] + mc.dt / 2.0 * (aw + bq);
    }
    for (int i = 0; i < 4; i++)
      Qn[i] = C.Gn[4 * i] * inner[0] + C.Gn[4 * i + 1] * inner[1] + C.Gn[4 * i + 2] * inner[2] + C.Gn[4 * i + 3] * inner[3];
    for (int i = 0; i < 4; i++) Q[i] = Qn[i];
  }
}

static __device__ void mgr_stage_coef(const double *q, const double *I0, const double *I, const double *Iinv,
                                      const double *om, const double *torque, bool gyro, double *Iom, double *omo,
                                      double *gRq_a, double *gRTq_a, double *gRq_b, double *gRTq_b) {
  double R[9];
  q_to_R(q, R);
  const double RT[9] = {R[0], R[3], R[6], R[1], R[4], R[7], R[2], R[5], R[8]};
  mv3(I, om, Iom);
  for (int k = 0; k < 3; k++) omo[k] = om[k];
  double temp_v[3];
  if (gyro) { cross3(Iom, om, temp_v); for (int k = 0; k < 3; k++) temp_v[k] += torque[k]; }
  else for (int k = 0; k < 3; k++) temp_v[k] = torque[k];
  double vb[3], tmp[3], tmp2[3];
  mv3(Iinv, temp_v, vb);
  mv3(RT, om, tmp); mv3(I0, tmp, tmp2); grad_Rqp_d(q, tmp2, gRq_a); grad_RqTp_d(q, om, gRTq_a);
  mv3(RT, vb, tmp); mv3(I0, tmp, tmp2); grad_Rqp_d(q, tmp2, gRq_b); grad_RqTp_d(q, vb, gRTq_b);
}

// The manager's step runs as three kernels after k_rigid_step (which writes the fluid's
// diagonal blocks into M): the per-body coefficients (two threads per body, one per stage);
// then one block
// per column of the state S (13 nb x 6 nb, row-major: row = 13 body + component, column =
// 6 body + j, j < 3 the v0 columns) and per column of the step maps A (two 13 nb x 13 nb
// maps, v0 then omega0 columns, row-major, A[r][c] = component r of the column that starts
// as unit vector c; written when tape_step is set), spread over the SMs because FP64 runs
// at a low rate on this part; then the contact solver's blocks of this step replace M's
// for every dynamic pair (RigidContactSolver::update_rigid_body_gradient_manager,
// :1341-1369).
static __global__ void k_manager_coef(const BodyState *__restrict__ bs, MgrConsts mc, MgrCoef *__restrict__ coefs) {
  const int nb = mc.nb, t = threadIdx.x;
  if (nb > DFSPH_MAX_BODIES_DEV) return;
  const bool gyro = mc.gyroscopic != 0;
  if (t < 2 * nb) {
    const int a = t >> 1;
    const BodyState &B = bs[a];
    MgrCoef &C = coefs[a];
    if ((t & 1) == 0) {
      C.dyn = B.dyn;
      C.invMass = B.invMass;
      for (int k = 0; k < 9; k++) { C.I[k] = B.Ipre[k]; C.Iinv[k] = B.Iipre[k]; C.I0[k] = B.I0[k]; }
      q_to_R(B.qpre, C.R);
      mgr_stage_coef(B.qpre, B.I0, B.Ipre, B.Iipre, B.wpre, B.T, gyro, C.Iom2, C.om2, C.gRq_a2, C.gRTq_a2, C.gRq_b2,
                     C.gRTq_b2);
    } else {
      const double zero[3] = {0.0, 0.0, 0.0};
      mgr_stage_coef(B.qpre, B.I0, B.Ipre, B.Iipre, B.wmid, zero, gyro, C.Iom3, C.om3, C.gRq_a3, C.gRTq_a3, C.gRq_b3,
                     C.gRTq_b3);
      const double p[4] = {0.0, B.wmid[0], B.wmid[1], B.wmid[2]};
      double pq[4], nq[4];
      q_mul(p, B.qpre, pq);
      for (int k = 0; k < 4; k++) nq[k] = B.qpre[k] + mc.dt * 0.5 * pq[k];
      const double nn = sqrt(nq[0] * nq[0] + nq[1] * nq[1] + nq[2] * nq[2] + nq[3] * nq[3]);
      double nv[4];
      for (int k = 0; k < 4; k++) nv[k] = nq[k] / nn;
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) C.Gn[4 * i + j] = ((i == j ? 1.0 : 0.0) - nv[i] * nv[j]) / nn;
      const double Gpq[16] = {p[0], -p[1], -p[2], -p[3], p[1], p[0], -p[3], p[2],
                              p[2], p[3], p[0], -p[1], p[3], -p[2], p[1], p[0]};
      for (int k = 0; k < 16; k++) C.Gpq[k] = Gpq[k];
      const double *q = B.qpre;
      const double Gpw[12] = {-q[1], -q[2], -q[3], q[0], q[3], -q[2], -q[3], q[0], q[1], q[2], -q[1], q[0]};
      for (int k = 0; k < 12; k++) C.Gpw[k] = Gpw[k];
    }
  }
}

// Block x: the state's columns first, then (with tape_step) the step maps' columns.
static __global__ void __launch_bounds__(32) k_manager_columns(MgrConsts mc, const MgrCoef *__restrict__ coefs,
                                                               const double *__restrict__ M,
                                                               const double *__restrict__ Mc, double *__restrict__ S,
                                                               double *__restrict__ tape_step) {
  if (threadIdx.x != 0) return;
  const int nb = mc.nb;
  if (nb > DFSPH_MAX_BODIES_DEV) return;
  const int n = NSTATE * nb, ncol = 6 * nb;
  int c = blockIdx.x;
  double s[NSTATE * DFSPH_MAX_BODIES_DEV];
  if (c < ncol) {
    for (int r = 0; r < n; r++) s[r] = S[(size_t)r * ncol + c];
    mgr_apply(coefs, mc, M, Mc, s, (c % 6) >= 3);
    for (int r = 0; r < n; r++) S[(size_t)r * ncol + c] = s[r];
    return;
  }
  c -= ncol;
  if (!tape_step || c >= 2 * n) return;
  const int cc = c % n;
  const bool wcol = c >= n;
  for (int r = 0; r < n; r++) s[r] = (r == cc) ? 1.0 : 0.0;
  mgr_apply(coefs, mc, M, Mc, s, wcol);
  double *A = tape_step + (wcol ? (size_t)n * n : 0);
  for (int r = 0; r < n; r++) A[(size_t)r * n + cc] = s[r];
}

static __global__ void k_manager_blocks(const BodyState *__restrict__ bs, int nb, double *__restrict__ M,
                                        const double *__restrict__ Mc) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nb * nb * NJAC; k += gridDim.x * blockDim.x) {
    const int pr = k / NJAC, a = pr / nb, c = pr % nb;
    if (bs[a].dyn && bs[c].dyn) M[k] = Mc[k];
  }
}

// Reverse sweep over the manager's step maps: lam_v <- A_v^T lam_v, lam_w <- A_w^T lam_w
// for n = last..first; lam holds 2 n doubles (v0 sweep, then omega0 sweep).
static __global__ void __launch_bounds__(256) k_backward_mgr(const double *__restrict__ tape, int nsteps, int n,
                                                             const double *__restrict__ lam_in,
                                                             double *__restrict__ lam_out) {
  __shared__ double lam[2 * NSTATE * DFSPH_MAX_BODIES_DEV], nl[2 * NSTATE * DFSPH_MAX_BODIES_DEV];
  const int t = threadIdx.x;
  if (n > NSTATE * DFSPH_MAX_BODIES_DEV) return;
  for (int k = t; k < 2 * n; k += blockDim.x) lam[k] = lam_in[k];
  __syncthreads();
  for (int st = nsteps - 1; st >= 0; st--) {
    const double *A0 = tape + (size_t)st * 2 * n * n;
    for (int k = t; k < 2 * n; k += blockDim.x) {
      const int w = k >= n, i = k % n;
      const double *A = A0 + (w ? (size_t)n * n : 0);
      const double *l = lam + (w ? n : 0);
      double acc = 0.0;
      for (int r = 0; r < n; r++) acc += A[(size_t)r * n + i] * l[r];
      nl[k] = acc;
    }
    __syncthreads();
    for (int k = t; k < 2 * n; k += blockDim.x) lam[k] = nl[k];
    __syncthreads();
  }
  for (int k = t; k < 2 * n; k += blockDim.x) lam_out[k] = lam[k];
}

}  // namespace dfsph
