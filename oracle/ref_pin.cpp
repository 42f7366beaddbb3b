// ref_pin.cpp — driver that evaluates the reference's own CubicKernel (SPHKernels.h) and
// quaternion Jacobians (GradientUtils.cpp), compiled from the reference sources by
// oracle/build_ref.sh, to produce golden vectors for the oracle (test infrastructure).
//
// stdin (binary): double h, int32 n, n x 3 doubles (kernel offsets), int32 m,
//                 m x (4 + 3) doubles (quaternion w,x,y,z and a point p)
// stdout (binary, Real = float or double per build): for each offset W, gradW[3],
//                 gradGradW[9]; for each (q, p): Rqp[12] RqTp[12] pq[16] wq[12]; then
//                 for each offset the cohesion and adhesion kernels (support h)
#include <cstdio>
#include <cstdint>
#include <vector>
#include "SPlisHSPlasH/SPHKernels.h"
#include "SPlisHSPlasH/GradientUtils.h"

static void put(const Real &v) { fwrite(&v, sizeof(Real), 1, stdout); }

int main() {
  double h; int32_t n;
  if (fread(&h, sizeof(double), 1, stdin) != 1 || fread(&n, sizeof(int32_t), 1, stdin) != 1) return 1;
  std::vector<double> r(3 * (size_t)n);
  if (fread(r.data(), sizeof(double), r.size(), stdin) != r.size()) return 1;
  int32_t m;
  if (fread(&m, sizeof(int32_t), 1, stdin) != 1) return 1;
  std::vector<double> qp(7 * (size_t)m);
  if (fread(qp.data(), sizeof(double), qp.size(), stdin) != qp.size()) return 1;
  SPH::CubicKernel::setRadius((Real)h);
  for (int i = 0; i < n; i++) {
    Vector3r v((Real)r[3 * i], (Real)r[3 * i + 1], (Real)r[3 * i + 2]);
    put(SPH::CubicKernel::W(v));
    Vector3r g = SPH::CubicKernel::gradW(v);
    for (int c = 0; c < 3; c++) put(g[c]);
    Matrix3r H = SPH::CubicKernel::gradGradW(v);
    for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) put(H(a, b));
  }
  for (int i = 0; i < m; i++) {
    const double *e = &qp[7 * (size_t)i];
    Quaternionr q((Real)e[0], (Real)e[1], (Real)e[2], (Real)e[3]);
    Vector3r p((Real)e[4], (Real)e[5], (Real)e[6]);
    Matrix34r A = get_grad_Rqp_to_q(q, p), B = get_grad_RqTp_to_q(q, p);
    Quaternionr pq(0.0, p[0], p[1], p[2]);
    Matrix4r C = get_grad_p_q_product_to_q(pq);
    Matrix43r D = get_grad_omega_q_product_to_omega(q);
    for (int a = 0; a < 3; a++) for (int b = 0; b < 4; b++) put(A(a, b));
    for (int a = 0; a < 3; a++) for (int b = 0; b < 4; b++) put(B(a, b));
    for (int a = 0; a < 4; a++) for (int b = 0; b < 4; b++) put(C(a, b));
    for (int a = 0; a < 4; a++) for (int b = 0; b < 3; b++) put(D(a, b));
  }
  SPH::CohesionKernel::setRadius((Real)h);
  SPH::AdhesionKernel::setRadius((Real)h);
  for (int i = 0; i < n; i++) {
    Vector3r v((Real)r[3 * i], (Real)r[3 * i + 1], (Real)r[3 * i + 2]);
    put(SPH::CohesionKernel::W(v));
    put(SPH::AdhesionKernel::W(v));
  }
  return 0;
}
