// engine_impl.cuh — Engine<T> member definitions (included by engine_fp32.cu / engine_fp64.cu).
#pragma once
#include <type_traits>

#include "engine.cuh"

namespace dfsph {

namespace {
inline void rotate_unit_q(const double q[4], const double p[3], double out[3]) {
  // v + w (2 u x v) + u x (2 u x v), the rotation of a unit quaternion
  const double u[3] = {q[1], q[2], q[3]};
  double uv[3] = {u[1] * p[2] - u[2] * p[1], u[2] * p[0] - u[0] * p[2], u[0] * p[1] - u[1] * p[0]};
  for (int k = 0; k < 3; k++) uv[k] += uv[k];
  const double uuv[3] = {u[1] * uv[2] - u[2] * uv[1], u[2] * uv[0] - u[0] * uv[2], u[0] * uv[1] - u[1] * uv[0]};
  for (int k = 0; k < 3; k++) out[k] = p[k] + q[0] * uv[k] + uuv[k];
}
inline void q_to_R_h(const double *q, double *R) {
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = 1 - (tyy + tzz); R[1] = txy - twz; R[2] = txz + twy;
  R[3] = txy + twz; R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
  R[6] = txz - twy; R[7] = tyz + twx; R[8] = 1 - (txx + tyy);
}
inline void inv3_h(const double *m, double *r) {
  const double c00 = m[4] * m[8] - m[5] * m[7];
  const double c01 = m[5] * m[6] - m[3] * m[8];
  const double c02 = m[3] * m[7] - m[4] * m[6];
  const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
  const double id = 1.0 / det;
  r[0] = c00 * id; r[1] = (m[2] * m[7] - m[1] * m[8]) * id; r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  r[3] = c01 * id; r[4] = (m[0] * m[8] - m[2] * m[6]) * id; r[5] = (m[3] * m[2] - m[0] * m[5]) * id;
  r[6] = c02 * id; r[7] = (m[6] * m[1] - m[0] * m[7]) * id; r[8] = (m[0] * m[4] - m[3] * m[1]) * id;
}
inline void world_inertia(BodyState &B) {
  double R[9], RI[9];
  q_to_R_h(B.q, R);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) RI[3 * i + j] = R[3 * i] * B.I0[j] + R[3 * i + 1] * B.I0[3 + j] + R[3 * i + 2] * B.I0[6 + j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) B.I[3 * i + j] = RI[3 * i] * R[3 * j] + RI[3 * i + 1] * R[3 * j + 1] + RI[3 * i + 2] * R[3 * j + 2];
  inv3_h(B.I, B.Iinv);
}
inline void chain_state_reset(BodyState &B) {
  for (int k = 0; k < NSTATE * 6; k++) B.G[k] = 0.0;
  for (int k = 0; k < 3; k++) { B.G[(7 + k) * 6 + k] = 1.0; B.G[(10 + k) * 6 + 3 + k] = 1.0; }
  for (int k = 0; k < NJAC; k++) B.nets[k] = 0.0;
}
}  // namespace

template <class T>
Engine<T>::Engine(const dfsph_scene *sc) {
  if (!sc) throw DfsphException(DFSPH_ERR_INVALID_ARG, "scene is NULL");
  if (sc->struct_size != (int)sizeof(dfsph_scene)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "dfsph_scene.struct_size mismatch");
  P_ = sc->params;
  if (P_.struct_size != (int)sizeof(dfsph_params)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "dfsph_params.struct_size mismatch");
  if (!(P_.particle_radius > 0) || !(P_.time_step > 0) || !(P_.density0 > 0))
    throw DfsphException(DFSPH_ERR_INVALID_ARG, "particle_radius, time_step and density0 must be positive");
  // neighbour passes index up to LPP_MAX threads per particle in int: keep n * LPP_MAX below 2^31
  if (sc->n_fluid < 0 || sc->n_fluid > (int64_t)INT32_MAX / 8) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n_fluid out of range");
  if (sc->n_fluid > 0 && !sc->fluid_x) throw DfsphException(DFSPH_ERR_INVALID_ARG, "fluid_x is NULL");
  if (sc->n_bodies < 0 || sc->n_bodies > DFSPH_MAX_BODIES) throw DfsphException(DFSPH_ERR_INVALID_ARG, "n_bodies out of range");
  if (sc->n_bodies > 0 && !sc->bodies) throw DfsphException(DFSPH_ERR_INVALID_ARG, "bodies is NULL");
  if (P_.gradient_mode < 0 || P_.gradient_mode > 2) throw DfsphException(DFSPH_ERR_INVALID_ARG, "gradient_mode");
  if (P_.max_iterations < 1 || P_.max_iterations_v < 1 || P_.min_iterations < 0)
    throw DfsphException(DFSPH_ERR_INVALID_ARG, "iteration limits");
  n_ = (int)sc->n_fluid;
  nb_ = sc->n_bodies;

  // ---- constants (in the fluid scalar type, as the reference's Real)
  const T r = (T)P_.particle_radius;
  const T h = T(4) * r;
  const T pi = (T)M_PI;
  const T h3 = h * h * h;
  fc_.n = n_;
  fc_.kc.h = h;
  fc_.kc.k = T(8) / (pi * h3);
  fc_.kc.l = T(48) / (pi * h3);
  fc_.kc.w0 = fc_.kc.k;  // W(0) = k (6*0 - 6*0 + 1)
  fc_.kc.invh = T(1) / h;
  fc_.h2 = h * h;
  fc_.rho0 = (T)P_.density0;
  const T diam = T(2) * r;
  fc_.V = T(0.8) * diam * diam * diam;
  fc_.m = fc_.V * fc_.rho0;
  fc_.eps = T(1.0e-5);
  if (!(P_.time_step > 0)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "time_step must be positive");
  if (P_.cfl_method != 0 && P_.cfl_method != 1)
    throw DfsphException(DFSPH_ERR_UNSUPPORTED, "cfl_method: 0 (fixed) or 1 (CFL)");
  if (P_.cfl_method == 1 && !(P_.cfl_min_time_step > 0 && P_.cfl_max_time_step >= P_.cfl_min_time_step))
    throw DfsphException(DFSPH_ERR_INVALID_ARG, "CFL time step bounds");
  fc_.visc = (T)P_.viscosity;
  fc_.visc_b = (T)P_.viscosity_boundary;
  {  // Akinci2013 surface tension constants (SPHKernels.h:446-452, 516-520)
    const double hs = 4.0 * P_.particle_radius;
    fc_.st_k = (T)P_.surface_tension;
    fc_.st_kb = (T)P_.surface_tension_boundary;
    fc_.coh_k = (T)(32.0 / (M_PI * std::pow(hs, 9.0)));
    fc_.coh_c = (T)(std::pow(hs, 6.0) / 64.0);
    fc_.adh_k = (T)(0.007 / std::pow(hs, 3.25));
  }
  if (P_.surface_tension_method != 0 && P_.surface_tension_method != 2)
    throw DfsphException(DFSPH_ERR_UNSUPPORTED, "surface_tension_method: 0 (none) or 2 (Akinci2013)");
  fc_.gx = (T)P_.gravity[0]; fc_.gy = (T)P_.gravity[1]; fc_.gz = (T)P_.gravity[2];
  // list capacities, rounded up to whole 16-byte groups for the vector loads
  fc_.kf = ((P_.max_fluid_neighbors > 0 ? P_.max_fluid_neighbors : 96) + 3) / 4 * 4;
  fc_.kb = ((P_.max_boundary_neighbors > 0 ? P_.max_boundary_neighbors : 96) + 3) / 4 * 4;
  pcP_.optimize_rotation = pcD_.optimize_rotation = P_.optimize_rotation;
  set_dt(P_.time_step);
  rc_.gx = (double)fc_.gx; rc_.gy = (double)fc_.gy; rc_.gz = (double)fc_.gz;
  rc_.gradient_mode = P_.gradient_mode;
  rc_.gyroscopic = P_.rigid_body_mode == DFSPH_RB_GYROSCOPIC;
  rc_.optimize_rotation = P_.optimize_rotation;
  rc_.enable_gradient = P_.enable_gradient;
  contact_ = P_.use_rigid_contact_solver != 0;
  manager_ = P_.use_rigid_gradient_manager != 0;
  rc_.manager = manager_ ? 1 : 0;
  rc_.nbodies = nb_;
  if (contact_) {
    if (!(P_.rigid_contact_support_radius_factor > 0) || !(P_.rigid_contact_gamma > 0))
      throw DfsphException(DFSPH_ERR_INVALID_ARG, "rigid contact support radius factor and gamma must be positive");
    const double sr = P_.rigid_contact_support_radius_factor * P_.particle_radius;
    const double s3 = sr * sr * sr;
    cc_.kc.h = sr; cc_.kc.k = 8.0 / (M_PI * s3); cc_.kc.l = 48.0 / (M_PI * s3); cc_.kc.w0 = cc_.kc.k; cc_.kc.invh = 1.0 / sr;
    const double hh = (double)h, h3d = hh * hh * hh;
    cc_.kh.h = hh; cc_.kh.k = 8.0 / (M_PI * h3d); cc_.kh.l = 48.0 / (M_PI * h3d); cc_.kh.w0 = cc_.kh.k; cc_.kh.invh = 1.0 / hh;
    cc_.beta = P_.rigid_contact_beta;
    cc_.mu = P_.rigid_contact_friction_coeff;
    cc_.gx = rc_.gx; cc_.gy = rc_.gy; cc_.gz = rc_.gz;
    cc_.dt = rc_.dt;
    // the contact blocks are carried forward even with gradients off: the next step's
    // fluid stage reads them, and a checkpoint must hold them for an exact replay
    cc_.grad = manager_ ? 1 : 0;
  }

  // ---- bodies (mass model of Dynamic3dRigidBody::determineMassProperties, :184-213)
  std::vector<double> static_world;  // xyz
  std::vector<int> static_orig_unsorted;
  std::vector<double> dyn_local;
  std::vector<int> dyn_body;
  std::vector<int> bnd_body;       // boundary index -> body
  std::vector<double> bnd_local;   // boundary index -> local coordinates (as T)
  int boundary_index = 0;
  const double rr = (double)r;
  for (int b = 0; b < nb_; b++) {
    const dfsph_body_desc &d = sc->bodies[b];
    if (d.n_samples < 0 || (d.n_samples > 0 && !d.samples)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body samples");
    BodyState B;
    std::memset(&B, 0, sizeof(B));
    const double qn = std::sqrt(d.rotation[0] * d.rotation[0] + d.rotation[1] * d.rotation[1] +
                                d.rotation[2] * d.rotation[2] + d.rotation[3] * d.rotation[3]);
    if (!(qn > 0)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body rotation quaternion is zero");
    for (int k = 0; k < 4; k++) B.q[k] = d.rotation[k] / qn;
    for (int k = 0; k < 3; k++) B.x[k] = d.translation[k];
    const double vol = static_cast<double>(4.0 / 3.0 * M_PI) * rr * rr * rr;
    const double dm = vol * d.density;
    for (int s = 0; s < d.n_samples; s++) {
      const double p[3] = {d.samples[3 * s], d.samples[3 * s + 1], d.samples[3 * s + 2]};
      const double pp = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
      B.mass += dm;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) B.I0[3 * i + j] += dm * ((i == j ? pp : 0.0) - p[i] * p[j]);
    }
    B.invMass = B.mass > 0 ? 1.0 / B.mass : 0.0;
    B.dyn = d.is_dynamic ? 1 : 0;
    B.anim = d.is_animated ? 1 : 0;
    world_inertia(B);
    chain_state_reset(B);
    body_dyn_.push_back(B.dyn);
    body_anim0_.push_back(B.anim);
    init_v_.insert(init_v_.end(), d.init_velocity, d.init_velocity + 3);
    init_w_.insert(init_w_.end(), d.init_angular_velocity, d.init_angular_velocity + 3);
    for (int s = 0; s < d.n_samples; s++) {
      bnd_body.push_back(b);
      for (int k = 0; k < 3; k++) bnd_local.push_back((double)(T)d.samples[3 * s + k]);
    }
    if (B.dyn) {
      B.dstart = nd_;
      B.dcount = (int)d.n_samples;
      for (int s = 0; s < d.n_samples; s++) {
        for (int k = 0; k < 3; k++) dyn_local.push_back((double)(T)d.samples[3 * s + k]);
        dyn_body.push_back(b);
        dyn_orig_.push_back(boundary_index + s);
      }
      nd_ += (int)d.n_samples;
    } else {
      for (int s = 0; s < d.n_samples; s++) {
        const double p[3] = {(double)(T)d.samples[3 * s], (double)(T)d.samples[3 * s + 1], (double)(T)d.samples[3 * s + 2]};
        double w[3];
        rotate_unit_q(B.q, p, w);
        for (int k = 0; k < 3; k++) static_world.push_back((double)(T)(w[k] + B.x[k]));
        static_orig_unsorted.push_back(boundary_index + s);
      }
      ns_ += (int)d.n_samples;
    }
    boundary_index += (int)d.n_samples;
    body_init_.push_back(B);
  }
  anim_ = body_anim0_;
  fc_.nbr = ns_ + nd_;
  boundary_is_dyn_.assign(boundary_index, 0);
  boundary_slot_.assign(boundary_index, 0);

  // ---- grid over fluid + boundary (+ dynamic bodies' reach), padded
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  auto grow = [&](const double *p) { for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); } };
  for (int i = 0; i < n_; i++) grow(sc->fluid_x + 3 * i);
  for (size_t s = 0; s < static_world.size() / 3; s++) grow(&static_world[3 * s]);
  for (int b = 0; b < nb_; b++)
    if (body_init_[b].dyn) {
      const dfsph_body_desc &d = sc->bodies[b];
      for (int s = 0; s < d.n_samples; s++) {
        double w[3], p[3] = {d.samples[3 * s], d.samples[3 * s + 1], d.samples[3 * s + 2]};
        rotate_unit_q(body_init_[b].q, p, w);
        for (int k = 0; k < 3; k++) w[k] += body_init_[b].x[k];
        grow(w);
      }
    }
  if (lo[0] > hi[0]) { for (int k = 0; k < 3; k++) { lo[k] = 0; hi[k] = 1; } }
  double cell = (double)h * (1.0 + 1e-4);
  const double pad = 3.0 * cell;
  double ext[3];
  for (int k = 0; k < 3; k++) { lo[k] -= pad; hi[k] += pad; ext[k] = hi[k] - lo[k]; }
  const double max_cells = 64.0 * 1024 * 1024;
  while ((ext[0] / cell + 1) * (ext[1] / cell + 1) * (ext[2] / cell + 1) > max_cells) cell *= 1.25;
  fc_.grid.ox = (T)lo[0]; fc_.grid.oy = (T)lo[1]; fc_.grid.oz = (T)lo[2];
  fc_.grid.inv_cell = (T)(1.0 / cell);
  fc_.grid.nx = (int)std::ceil(ext[0] / cell) + 1;
  fc_.grid.ny = (int)std::ceil(ext[1] / cell) + 1;
  fc_.grid.nz = (int)std::ceil(ext[2] / cell) + 1;
  ncell_ = fc_.grid.nx * fc_.grid.ny * fc_.grid.nz;

  DF_CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  DF_CK(cudaStreamCreateWithFlags(&stream2_, cudaStreamNonBlocking));
  DF_CK(cudaStreamCreateWithFlags(&stream3_, cudaStreamNonBlocking));
  DF_CK(cudaEventCreateWithFlags(&ev_fluid_done_, cudaEventDisableTiming));
  DF_CK(cudaEventCreateWithFlags(&ev_rigid_done_, cudaEventDisableTiming));
  DF_CK(cudaEventCreateWithFlags(&ev_rigid_state_, cudaEventDisableTiming));
  DF_CK(cudaEventCreateWithFlags(&ev_contact_in_, cudaEventDisableTiming));
  DF_CK(cudaEventCreateWithFlags(&ev_chain_done_, cudaEventDisableTiming));
  {
    int dev = 0;
    DF_CK(cudaGetDevice(&dev));
    DF_CK(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
  }
  // lanes per particle of the neighbour passes: LPP_MAX where one lane per particle would
  // leave the passes below 256 threads per SM (small scenes), else 1
  fc_.lpp = (int64_t)n_ <= (int64_t)num_sms_ * 256 ? LPP_MAX : 1;
  scan_.prepare((size_t)ncell_ + 1);

  // ---- fluid buffers
  x_init_.assign(sc->fluid_x, sc->fluid_x + 3 * (size_t)n_);
  v_init_.assign(3 * (size_t)n_, 0.0);
  if (sc->fluid_v) v_init_.assign(sc->fluid_v, sc->fluid_v + 3 * (size_t)n_);
  const size_t N = std::max(n_, 1);
  for (int k = 0; k < 2; k++) { R_[k].alloc(N); kappa_[k].alloc(N); kappaV_[k].alloc(N); perm_[k].alloc(N); }
  Q_.alloc(N);
  rho_.alloc(N); alpha_.alloc(N); rhoAdv_.alloc(N); sumgrad_.alloc(N);
  speed2_.alloc(1);
  if (P_.surface_tension_method == 2) N_.alloc(N);
  fcount_.alloc(N); bcount_.alloc(N);
  // +8 entries: a batched 16-byte load may read up to 7 entries past a short last row
  flist_.alloc(N * (size_t)fc_.kf + 8);
  blist_.alloc(N * (size_t)fc_.kb + 8);
  key_.alloc(N); rank_.alloc(N); order_.alloc(N);
  cstartF_.alloc((size_t)ncell_ + 1);
  cstartS_.alloc((size_t)ncell_ + 1);
  cstartD_.alloc((size_t)ncell_ + 1);
  partials_.alloc((size_t)blocks(std::max(n_, 1) * LPP_MAX, PASS_THREADS));
  resid_.alloc(4);
  err_.alloc(1);
  DF_CK(cudaHostAlloc((void **)&resid_host_, 4 * sizeof(double), cudaHostAllocMapped));
  DF_CK(cudaHostAlloc((void **)&err_host_, sizeof(int), cudaHostAllocDefault));
  DF_CK(cudaHostAlloc((void **)&hbs_pin_, std::max(nb_, 1) * sizeof(BodyState), cudaHostAllocDefault));
  DF_CK(cudaHostGetDevicePointer((void **)&resid_host_dev_, resid_host_, 0));
  DF_CK(cudaMemsetAsync(err_.p, 0, sizeof(int), stream_));

  // ---- boundary buffers
  const size_t NB = std::max(ns_ + nd_, 1);
  BR_.alloc(NB); psi_.alloc(NB);
  const size_t ND = std::max(nd_, 1);
  xd_.alloc(ND); vd_.alloc(ND); x0d_.alloc(ND); bodyd_.alloc(ND); keyD_.alloc(ND); rankD_.alloc(ND);
  orderD_.alloc(ND); dynSortedToBody_.alloc(ND); bfcount_.alloc(ND); bflist_.alloc(ND * (size_t)kbf_);
  acc_.alloc(ND * ACC_STRIDE);
  bs_.alloc(std::max(nb_, 1));
  {  // reduction chunks: RED_CHUNK consecutive samples of one dynamic body each
    std::vector<RedChunk> ch;
    std::vector<int2> bc(std::max(nb_, 1), make_int2(0, 0));
    for (int b = 0; b < nb_; b++) {
      const BodyState &B = body_init_[b];
      bc[b].x = (int)ch.size();
      if (B.dyn)
        for (int d = 0; d < B.dcount; d += RED_CHUNK) ch.push_back(RedChunk{b, B.dstart + d, std::min(RED_CHUNK, B.dcount - d)});
      bc[b].y = (int)ch.size();
    }
    nchunks_ = (int)ch.size();
    chunks_.alloc(std::max<size_t>(ch.size(), 1));
    body_chunks_.alloc(bc.size());
    red_part_.alloc(std::max<size_t>(ch.size(), 1) * RED_VALUES);
    if (!ch.empty()) DF_CK(cudaMemcpy(chunks_.p, ch.data(), ch.size() * sizeof(RedChunk), cudaMemcpyHostToDevice));
    DF_CK(cudaMemcpy(body_chunks_.p, bc.data(), bc.size() * sizeof(int2), cudaMemcpyHostToDevice));
  }
  DF_CK(cudaMemsetAsync(BR_.p, 0, NB * sizeof(Rec<T>), stream_));
  DF_CK(cudaMemsetAsync(acc_.p, 0, ND * ACC_STRIDE * sizeof(double), stream_));
  if (nd_ > 0) {
    std::vector<V4<T>> x0h(nd_);
    for (int d = 0; d < nd_; d++) x0h[d] = V4<T>{(T)dyn_local[3 * d], (T)dyn_local[3 * d + 1], (T)dyn_local[3 * d + 2], T(0)};
    DF_CK(cudaMemcpyAsync(x0d_.p, x0h.data(), nd_ * sizeof(V4<T>), cudaMemcpyHostToDevice, stream_));
    DF_CK(cudaMemcpyAsync(bodyd_.p, dyn_body.data(), nd_ * sizeof(int), cudaMemcpyHostToDevice, stream_));
    DF_CK(cudaMemsetAsync(xd_.p, 0, nd_ * sizeof(V4<T>), stream_));
    for (int d = 0; d < nd_; d++) { boundary_is_dyn_[dyn_orig_[d]] = 1; boundary_slot_[dyn_orig_[d]] = d; }
  }
  // static samples: sorted by cell once
  DF_CK(cudaMemsetAsync(cstartS_.p, 0, ((size_t)ncell_ + 1) * sizeof(int), stream_));
  if (ns_ > 0) {
    std::vector<V4<T>> sh(ns_);
    for (int s = 0; s < ns_; s++) sh[s] = V4<T>{(T)static_world[3 * s], (T)static_world[3 * s + 1], (T)static_world[3 * s + 2], T(0)};
    DBuf<V4<T>> tmp; tmp.alloc(ns_);
    DBuf<int> k1, k2, k3;
    k1.alloc(ns_); k2.alloc(ns_); k3.alloc(ns_);
    DF_CK(cudaMemcpyAsync(tmp.p, sh.data(), ns_ * sizeof(V4<T>), cudaMemcpyHostToDevice, stream_));
    sort_points(tmp.p, 1, ns_, k1.p, k2.p, cstartS_.p, k3.p);
    std::vector<int> order(ns_);
    DF_CK(cudaMemcpyAsync(order.data(), k3.p, ns_ * sizeof(int), cudaMemcpyDeviceToHost, stream_));
    sync_all();
    std::vector<V4<T>> sorted(ns_);
    static_orig_.resize(ns_);
    for (int s = 0; s < ns_; s++) {
      sorted[s] = sh[order[s]];
      static_orig_[s] = static_orig_unsorted[order[s]];
      boundary_is_dyn_[static_orig_[s]] = 0;
      boundary_slot_[static_orig_[s]] = s;
    }
    std::vector<Rec<T>> srec(ns_);
    for (int q = 0; q < ns_; q++) srec[q] = Rec<T>{sorted[q], V4<T>{T(0), T(0), T(0), T(0)}};
    DF_CK(cudaMemcpyAsync(BR_.p, srec.data(), ns_ * sizeof(Rec<T>), cudaMemcpyHostToDevice, stream_));
    if (contact_) {
      std::vector<int> bs_h(ns_);
      std::vector<V4<T>> x0s_h(ns_);
      for (int q = 0; q < ns_; q++) {
        const int o = static_orig_[q];
        bs_h[q] = bnd_body[o];
        x0s_h[q] = V4<T>{(T)bnd_local[3 * o], (T)bnd_local[3 * o + 1], (T)bnd_local[3 * o + 2], T(0)};
      }
      bodyS_.alloc(ns_); x0S_.alloc(ns_);
      DF_CK(cudaMemcpyAsync(bodyS_.p, bs_h.data(), ns_ * sizeof(int), cudaMemcpyHostToDevice, stream_));
      DF_CK(cudaMemcpyAsync(x0S_.p, x0s_h.data(), ns_ * sizeof(V4<T>), cudaMemcpyHostToDevice, stream_));
    }
    sync_all();
  } else {
    // keep the empty table's scan consistent (all zero)
  }
  if (contact_) {
    if (!bodyS_.p) { bodyS_.alloc(1); x0S_.alloc(1); }
    cvol0S_.alloc(std::max(ns_, 1)); cdens0S_.alloc(std::max(ns_, 1));
    cvol0D_.alloc(ND); cdens0D_.alloc(ND);
    crec_.alloc(ND); clist_.alloc(ND);
    if (manager_) cblk_.alloc(ND * (size_t)CONTACT_BLK);
  }
  ccount_.alloc(2 * (size_t)std::max(nb_, 1));
  DF_CK(cudaMemsetAsync(ccount_.p, 0, 2 * (size_t)std::max(nb_, 1) * sizeof(int), stream_));
  if (manager_) {
    const size_t nbb = (size_t)std::max(nb_, 1);
    Mc_.alloc(nbb * nbb * NJAC);
    mgrM_.alloc(nbb * nbb * NJAC);
    mgrS_.alloc((size_t)NSTATE * nbb * 6 * nbb);
    mgrC_.alloc(nbb);
  }
  if (nd_ > 0 && P_.enable_gradient) {
    tape_cap_ = 256;
    tape_.alloc((size_t)tape_cap_ * tape_stride());
  }
  reset();
  if (contact_) contact_init();
}

// RigidContactSolver::RigidContactSolver (RigidContactSolver.cpp:23-262): rest volume and
// rest density of every boundary sample, once, from the positions after the first reset.
template <class T>
void Engine<T>::contact_init() {
  if (ns_ + nd_ == 0) return;
  for (int phase = 0; phase < 2; phase++) {
    k_contact_rest<T><<<blocks(ns_ + nd_), 256, 0, stream_>>>(
        cc_, fc_.grid, fc_.h2, ns_, nd_, BR_.p, cstartS_.p, nd_ ? cstartD_.p : nullptr, bodyS_.p,
        nd_ ? bodyd_.p : nullptr, nd_ ? dynSortedToBody_.p : nullptr, P_.rigid_contact_gamma, phase, cvol0S_.p,
        cvol0D_.p, cdens0S_.p, cdens0D_.p);
    launched();
  }
  check_launch();
  sync_all();
}

// RigidBodyGradientManager::reset (RigidBodyGradientManager.cpp:477-524): identity in the
// v / omega slots of each body's own columns; with blocks == true also zero blocks (a full
// reset). The blocks are kept by dfsph_reset_gradient because the next step's fluid stage
// reads the last contact blocks, so that a segment replayed from a checkpoint maps exactly
// as it did in the first run.
template <class T>
void Engine<T>::manager_reset(bool blocks) {
  if (!manager_ || nb_ == 0) return;
  const size_t ncol = 6 * (size_t)nb_, nrow = (size_t)NSTATE * nb_;
  std::vector<double> S(nrow * ncol, 0.0);
  for (int a = 0; a < nb_; a++)
    for (int j = 0; j < 3; j++) {
      S[((size_t)NSTATE * a + 7 + j) * ncol + 6 * a + j] = 1.0;
      S[((size_t)NSTATE * a + 10 + j) * ncol + 6 * a + 3 + j] = 1.0;
    }
  DF_CK(cudaMemcpyAsync(mgrS_.p, S.data(), S.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
  if (blocks) {
    DF_CK(cudaMemsetAsync(mgrM_.p, 0, (size_t)nb_ * nb_ * NJAC * sizeof(double), stream_));
    DF_CK(cudaMemsetAsync(Mc_.p, 0, (size_t)nb_ * nb_ * NJAC * sizeof(double), stream_));
  }
  sync_all();
}

template <class T>
Engine<T>::~Engine() {
  if (stream3_) cudaStreamSynchronize(stream3_);
  if (stream2_) cudaStreamSynchronize(stream2_);
  if (stream_) cudaStreamSynchronize(stream_);
  if (ev_fluid_done_) cudaEventDestroy(ev_fluid_done_);
  if (ev_rigid_done_) cudaEventDestroy(ev_rigid_done_);
  if (ev_rigid_state_) cudaEventDestroy(ev_rigid_state_);
  if (ev_contact_in_) cudaEventDestroy(ev_contact_in_);
  if (ev_chain_done_) cudaEventDestroy(ev_chain_done_);
  if (stream2_) cudaStreamDestroy(stream2_);
  if (stream3_) cudaStreamDestroy(stream3_);
  for (auto &e : ev_) if (e) cudaEventDestroy(e);
  for (auto &r : pending_) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto &e : pool_) cudaEventDestroy(e);
  if (resid_host_) cudaFreeHost(resid_host_);
  if (err_host_) cudaFreeHost(err_host_);
  if (hbs_pin_) cudaFreeHost(hbs_pin_);
  if (stream_) cudaStreamDestroy(stream_);
}

template <class T>
void Engine<T>::sort_points(const V4<T> *pts, int stride, int count, int *key, int *rank, int *cstart, int *order) {
  DF_CK(cudaMemsetAsync(cstart, 0, ((size_t)ncell_ + 1) * sizeof(int), stream_));
  if (count == 0) return;
  k_cell_keys<T><<<blocks(count), 256, 0, stream_>>>(count, pts, stride, fc_.grid, key, rank, cstart, err_.p);
  launched();
  scan_.run(cstart, ncell_ + 1, stream_, launches_);
  k_scatter_order<<<blocks(count), 256, 0, stream_>>>(count, key, rank, cstart, order);
  k_cell_insertion_sort<<<blocks(ncell_), 256, 0, stream_>>>(ncell_, cstart, order);
  launched(2);
  check_launch();
}

template <class T>
void Engine<T>::sort_fluid() {
  if (n_ == 0) {
    DF_CK(cudaMemsetAsync(cstartF_.p, 0, ((size_t)ncell_ + 1) * sizeof(int), stream_));
    return;
  }
  pbegin();
  sort_points(reinterpret_cast<const V4<T> *>(R_[cur_].p), 2, n_, key_.p, rank_.p, cstartF_.p, order_.p);
  const int nx = 1 - cur_;
  k_gather_fluid<T><<<blocks(n_), 256, 0, stream_>>>(n_, order_.p, R_[cur_].p, kappa_[cur_].p, kappaV_[cur_].p,
                                                     perm_[cur_].p, R_[nx].p, kappa_[nx].p, kappaV_[nx].p,
                                                     perm_[nx].p);
  launched();
  pend(DFSPH_K_SORT, n_);
  cur_ = nx;
}

template <class T>
void Engine<T>::sort_dynamic() {
  if (nd_ == 0) return;
  pbegin();
  if (nd_ <= SMALL_SORT_MAX) {
    k_sort_dynamic_small<T><<<1, 1024, 0, stream_>>>(nd_, ns_, fc_.grid, xd_.p, vd_.p, BR_.p, dynSortedToBody_.p,
                                                     keyD_.p, err_.p);
    k_cstart_from_keys<<<blocks(ncell_ + 1), 256, 0, stream_>>>(ncell_, nd_, keyD_.p, cstartD_.p);
    launched(2);
    pend(DFSPH_K_SORT, nd_);
    return;
  }
  sort_points(xd_.p, 1, nd_, keyD_.p, rankD_.p, cstartD_.p, orderD_.p);
  k_gather_dynamic<T><<<blocks(nd_), 256, 0, stream_>>>(nd_, ns_, orderD_.p, xd_.p, vd_.p, BR_.p,
                                                        dynSortedToBody_.p);
  launched();
  pend(DFSPH_K_SORT, nd_);
}

// The static samples' psi is computed once: they never move, and every reset puts the
// dynamic samples back at the same initial poses, so their neighbourhoods repeat exactly;
// later resets recompute the dynamic samples only.
template <class T>
void Engine<T>::compute_psi() {
  if (ns_ + nd_ == 0) return;
  const int p0 = psi_static_done_ ? ns_ : 0;
  const int cnt = ns_ + nd_ - p0;
  if (cnt > 0) {
    k_boundary_psi<T><<<blocks(cnt), 256, 0, stream_>>>(fc_, ns_, nd_, BR_.p, cstartS_.p, nd_ ? cstartD_.p : nullptr,
                                                      psi_.p, p0);
    k_set_psi<T><<<blocks(cnt), 256, 0, stream_>>>(ns_, nd_, psi_.p, BR_.p, xd_.p, dynSortedToBody_.p, p0);
    launched(2);
  }
  psi_static_done_ = true;
  check_launch();
}

template <class T>
void Engine<T>::upload_fluid_initial() {
  cur_ = 0;
  if (n_ == 0) return;
  // the initial records are converted and uploaded once; later resets copy them on the device
  if (R_init_.n < (size_t)n_) {
    std::vector<Rec<T>> rh(n_);
    for (int i = 0; i < n_; i++) {
      rh[i].x = V4<T>{(T)x_init_[3 * i], (T)x_init_[3 * i + 1], (T)x_init_[3 * i + 2], T(0)};
      rh[i].v = V4<T>{(T)v_init_[3 * i], (T)v_init_[3 * i + 1], (T)v_init_[3 * i + 2], T(0)};
    }
    R_init_.alloc(n_);
    DF_CK(cudaMemcpyAsync(R_init_.p, rh.data(), n_ * sizeof(Rec<T>), cudaMemcpyHostToDevice, stream_));
    sync_all();
  }
  DF_CK(cudaMemcpyAsync(R_[0].p, R_init_.p, n_ * sizeof(Rec<T>), cudaMemcpyDeviceToDevice, stream_));
  // perm[1] must also be a valid permutation before the first gather
  k_iota2<<<blocks(n_), 256, 0, stream_>>>(n_, perm_[0].p, perm_[1].p);
  launched();
  DF_CK(cudaMemsetAsync(kappa_[0].p, 0, n_ * sizeof(T), stream_));
  DF_CK(cudaMemsetAsync(kappaV_[0].p, 0, n_ * sizeof(T), stream_));
  DF_CK(cudaMemsetAsync(rho_.p, 0, n_ * sizeof(T), stream_));
  DF_CK(cudaMemsetAsync(alpha_.p, 0, n_ * sizeof(T), stream_));
  DF_CK(cudaMemsetAsync(rhoAdv_.p, 0, n_ * sizeof(T), stream_));
  DF_CK(cudaMemsetAsync(sumgrad_.p, 0, n_ * sizeof(V4<T>), stream_));
  DF_CK(cudaMemsetAsync(fcount_.p, 0, n_ * sizeof(int), stream_));
  DF_CK(cudaMemsetAsync(bcount_.p, 0, n_ * sizeof(int), stream_));
  check_launch();
  sync_all();
}
template <class T>
void Engine<T>::body_state_download(std::vector<BodyState> &out) {
  out.resize(nb_);
  if (nb_ == 0) return;
  sync_all();
  DF_CK(cudaMemcpy(out.data(), bs_.p, nb_ * sizeof(BodyState), cudaMemcpyDeviceToHost));
}
template <class T>
void Engine<T>::body_state_upload(const std::vector<BodyState> &in) {
  if (nb_ == 0) return;
  dev_epoch_++;
  wait_rigid();  // no rigid kernel may still write the records
  DF_CK(cudaMemcpyAsync(bs_.p, in.data(), nb_ * sizeof(BodyState), cudaMemcpyHostToDevice, stream_));
  sync_all();
}

template <class T>
void Engine<T>::reset() {
  sync_all();
  upload_fluid_initial();
  std::vector<BodyState> bsv = body_init_;  // pose x0/q0, v = omega = 0 (Dynamic3dRigidBody::reset)
  anim_ = body_anim0_;
  body_state_upload(bsv);
  if (nd_ > 0) {
    k_boundary_update<T><<<blocks(nd_), 256, 0, stream_>>>(bs_.p, nd_, x0d_.p, bodyd_.p, xd_.p, vd_.p, 0);
    launched();
    DF_CK(cudaMemsetAsync(acc_.p, 0, (size_t)nd_ * ACC_STRIDE * sizeof(double), stream_));
  }
  sort_dynamic();
  compute_psi();
  DF_CK(cudaMemsetAsync(err_.p, 0, sizeof(int), stream_));
  t_ = 0.0;
  step_count_ = 0;
  finished_ = false;
  tape_len_ = 0;
  set_dt(P_.time_step);
  manager_reset(true);
  sync_all();
}

template <class T>
void Engine<T>::reset_gradient() {
  std::vector<BodyState> bsv;
  body_state_download(bsv);
  for (auto &B : bsv) chain_state_reset(B);
  body_state_upload(bsv);
  if (nd_ > 0) DF_CK(cudaMemsetAsync(acc_.p, 0, (size_t)nd_ * ACC_STRIDE * sizeof(double), stream_));
  tape_len_ = 0;
  manager_reset(false);
  sync_all();
}

// TimeStepDiffDFSPH::beginStep (:353-430)
template <class T>
void Engine<T>::begin_step() {
  step_count_++;
  if (nb_ == 0) return;
  BeginCmd cmd;
  std::memset(&cmd, 0, sizeof(cmd));
  cmd.n = nb_;
  const double uat = P_.uniform_accelerate_rb_time, dt = dt_cur_;
  for (int b = 0; b < nb_; b++) {
    if (!body_dyn_[b]) { cmd.anim[b] = anim_[b]; continue; }
    if (P_.release_rigid_body_mode) {
      if (b == 1) {
        if (t_ <= uat + dt) {
          if (uat > 1e-3) anim_[b] = 1;
          cmd.set[b] = 1;
        } else {
          cmd.set[b] = 1;
          for (int k = 0; k < 3; k++) { cmd.v[b][k] = init_v_[3 * b + k]; cmd.w[b][k] = init_w_[3 * b + k]; }
          anim_[b] = 0;
        }
      }
    } else {
      if (t_ <= uat + dt) {
        double fac = 1.0;
        if (uat > 1e-3) { fac = (t_ / uat) > 1.0 ? 1.0 : (t_ / uat); anim_[b] = 1; }
        cmd.set[b] = 1;
        for (int k = 0; k < 3; k++) { cmd.v[b][k] = fac * init_v_[3 * b + k]; cmd.w[b][k] = fac * init_w_[3 * b + k]; }
      } else {
        anim_[b] = 0;
      }
    }
    cmd.anim[b] = anim_[b];
  }
  k_rigid_begin<<<1, 32, 0, stream_>>>(bs_.p, cmd);
  launched();
}

template <class T>
double Engine<T>::read_residual() {
  sync_all();
  const int e = (int)resid_host_[1];
  if (e) check_error_word();
  return resid_host_[0];
}

template <class T>
void Engine<T>::check_error_word() {
  int e = 0;
  DF_CK(cudaMemcpy(&e, err_.p, sizeof(int), cudaMemcpyDeviceToHost));
  raise_error_word(e);
}

template <class T>
void Engine<T>::raise_error_word(int e) {
  if (e) {
    std::string m = "device error word:";
    if (e & ERR_FLUID_LIST_OVERFLOW) m += " fluid neighbour list overflow (raise max_fluid_neighbors);";
    if (e & ERR_BOUNDARY_LIST_OVERFLOW) m += " boundary neighbour list overflow (raise max_boundary_neighbors);";
    if (e & ERR_BF_LIST_OVERFLOW) m += " dynamic-boundary fluid list overflow;";
    if (e & ERR_NONFINITE_POSITION) m += " non-finite particle position;";
    if (e & ERR_MLP_TIMEOUT) m += " tensor-core wait timed out in the warm-start model;";
    throw DfsphException(DFSPH_ERR_DEVICE, m);
  }
}

template <class T>
void Engine<T>::launch_density(int mode, T *kappa_io, bool partials, float4 *feat) {
  const int nbk = blocks(n_ * fc_.lpp, PASS_THREADS);
  double *pp = partials ? partials_.p : nullptr;
  pbegin();
#define DF_DENS_L(M, XS, L)                                                                                        \
  k_density_pass<T, M, XS, L><<<nbk, PASS_THREADS, 0, stream_>>>(fc_, R_[cur_].p, Q_.p, BR_.p, flist_.p, fcount_.p,  \
                                                                 blist_.p, bcount_.p, rho_.p, alpha_.p, rhoAdv_.p,  \
                                                                 kappa_io, pp, feat, R_[1 - cur_].p)
#define DF_DENS(M, XS)                   \
  if (fc_.lpp == 1) DF_DENS_L(M, XS, 1); \
  else DF_DENS_L(M, XS, LPP_MAX)
  // the divergence solve's checked passes also advance the XSPH phase (see k_density_pass)
  const bool xs = mode == PASS_DIVERGENCE && partials && xs_fuse_;
  switch (mode) {
    case PASS_PRESSURE: DF_DENS(PASS_PRESSURE, false); break;
    case PASS_DIVERGENCE:
      if (xs) { DF_DENS(PASS_DIVERGENCE, true); xs_done_ = true; }
      else DF_DENS(PASS_DIVERGENCE, false);
      break;
    case PASS_PRESSURE_WARM: DF_DENS(PASS_PRESSURE_WARM, false); break;
    default: DF_DENS(PASS_DIVERGENCE_WARM, false); break;
  }
#undef DF_DENS
#undef DF_DENS_L
  launched();
  pend(DFSPH_K_DENSITY_PASS, n_);
}

template <class T>
void Engine<T>::launch_velocity(T *kappa_acc) {
  const int nbk = blocks(n_ * fc_.lpp, PASS_THREADS);
  pbegin();
  auto go = [&](auto acc, auto lanes) {
    k_velocity_pass<T, decltype(acc)::value, decltype(lanes)::value><<<nbk, PASS_THREADS, 0, stream_>>>(
        fc_, Q_.p, R_[cur_].p, BR_.p, flist_.p, fcount_.p, blist_.p, bcount_.p, kappa_acc);
  };
  using One = std::integral_constant<int, 1>;
  using Wide = std::integral_constant<int, LPP_MAX>;
  using Acc = std::integral_constant<int, 1>;
  using NoAcc = std::integral_constant<int, 0>;
  if (kappa_acc) { if (fc_.lpp == 1) go(Acc{}, One{}); else go(Acc{}, Wide{}); }
  else { if (fc_.lpp == 1) go(NoAcc{}, One{}); else go(NoAcc{}, Wide{}); }
  launched();
  pend(DFSPH_K_VELOCITY_PASS, n_);
}

template <class T>
void Engine<T>::launch_pairs(bool pressure, bool warm, bool grad) {
  if (nd_ == 0) return;
  const int ndw = blocks(nd_ * 32, PAIR_THREADS);
  PairConsts<T> pc = pressure ? pcP_ : pcD_;
  pc.grad = (grad && !warm) ? 1 : 0;
  pbegin();
#define DF_PAIRS(M)                                                                                                \
  k_pairs<T, M><<<ndw, PAIR_THREADS, 0, stream_>>>(fc_, pc, nd_, xd_.p, vd_.p, x0d_.p, bodyd_.p, bs_.p, bflist_.p, bfcount_.p, \
                                          Q_.p, R_[cur_].p, alpha_.p, rhoAdv_.p, sumgrad_.p, acc_.p)
  if (pressure) DF_PAIRS(0);
  else DF_PAIRS(1);
#undef DF_PAIRS
  launched();
  pend(DFSPH_K_PAIRS, nd_);
}

// pressureSolve (TimeStepDiffDFSPH.cpp:654-768) and divergenceSolve (:770-881):
// warm start, then Jacobi sweeps of [pair Jacobians + boundary reaction forces,
// velocity correction, density advection / change + residual] until the average
// error is below eta (after at least min iterations) or max iterations are reached.
template <class T>
void Engine<T>::solve(bool pressure) {
  cudaEvent_t ph = phase_begin();
  solve_impl(pressure);
  phase_end(pressure ? DFSPH_PHASE_PRESSURE_SOLVE : DFSPH_PHASE_DIVERGENCE_SOLVE, ph, n_);
}

template <class T>
void Engine<T>::solve_impl(bool pressure) {
  const bool warm = pressure ? P_.use_pressure_warmstart : P_.use_divergence_warmstart;
  T *kap = pressure ? kappa_[cur_].p : kappaV_[cur_].p;
  const int wm = pressure ? PASS_PRESSURE_WARM : PASS_DIVERGENCE_WARM;
  const int im = pressure ? PASS_PRESSURE : PASS_DIVERGENCE;
  if (warm) {
    const bool ml = pressure && (ml_record_ || ml_on_);
    // the divergence warm start's density pass ran inside the list build
    if (pressure) launch_density(wm, kap, false, ml ? F_.p : nullptr);
    if (pressure && ml_on_) launch_mlp_warmstart(kap);
    launch_pairs(pressure, true, false);
    launch_velocity(nullptr);
  }
  launch_density(im, nullptr, false);
  int it = 0;
  bool chk = false;
  double avg = 0.0;
  const T eta = pressure ? (T)P_.max_error * T(0.01) * fc_.rho0
                         : (T(1) / fc_.dt) * (T)P_.max_error_v * T(0.01) * fc_.rho0;
  const int minIt = pressure ? P_.min_iterations : 1;
  const int maxIt = pressure ? P_.max_iterations : P_.max_iterations_v;
  const int nbk = blocks(n_ * fc_.lpp, PASS_THREADS);
  while ((!chk || it < minIt) && it < maxIt) {
    launch_pairs(pressure, false, P_.enable_gradient != 0);
    launch_velocity(warm ? kap : nullptr);
    const bool need = (it + 1 >= minIt) || (it + 1 >= maxIt);
    launch_density(im, nullptr, need);
    if (need) {
      k_final_sum<<<1, FINAL_SUM_THREADS, 0, stream_>>>(nbk, partials_.p, 1.0 / (double)std::max(n_, 1), resid_.p,
                                                        resid_host_dev_, err_.p);
      launched();
      check_launch();
      avg = read_residual();
      chk = (T)avg <= eta;
    }
    it++;
  }
  if (pressure) { last_iters_ = it; last_err_ = avg; }
  else { last_iters_v_ = it; last_err_v_ = avg; }
}

template <class T>
void Engine<T>::grow_tape() {
  wait_rigid();  // earlier steps' tape rows are written on the rigid stream
  const int64_t ncap = std::max<int64_t>(tape_cap_ * 2, 256);
  DBuf<double> nt;
  nt.alloc((size_t)ncap * tape_stride());
  if (tape_len_ > 0)
    DF_CK(cudaMemcpyAsync(nt.p, tape_.p, (size_t)tape_len_ * tape_stride() * sizeof(double),
                          cudaMemcpyDeviceToDevice, stream_));
  sync_all();
  std::swap(tape_.p, nt.p);
  std::swap(tape_.n, nt.n);
  tape_cap_ = ncap;
}

// backwardPerStep's chain rule (:493-524) + velocityTimeStep + positionTimeStep +
// updateBoundaryParticles, all on the device.
template <class T>
// The rigid kernels run on a second stream after the fluid's integration, so that they
// overlap the next step's fluid sort (which touches no rigid data); every later use of
// rigid data on the main stream, and every host synchronisation, waits for them.
void Engine<T>::rigid_end() {
  if (nd_ == 0) return;
  double *tape_step = nullptr;
  if (P_.enable_gradient) {
    if (tape_len_ >= tape_cap_) grow_tape();
    tape_step = tape_.p + (size_t)tape_len_ * tape_stride();
    tape_len_++;
  }
  const bool mgr_chain = manager_ && P_.enable_gradient;
  const bool mgr_blocks = manager_ && contact_;
  if (contact_ && !contact_launched_) launch_contact();
  contact_launched_ = false;
  if (!fluid_done_recorded_) DF_CK(cudaEventRecord(ev_fluid_done_, stream_));
  fluid_done_recorded_ = false;
  DF_CK(cudaStreamWaitEvent(stream2_, ev_fluid_done_, 0));
  // k_rigid_step writes whole body records: the previous step's chain (which writes G) first
  DF_CK(cudaStreamWaitEvent(stream2_, ev_chain_done_, 0));
  pbegin(stream2_);
  int nl = 0;
  if (nchunks_ > 0) {
    k_body_partials<T><<<nchunks_, RED_THREADS, 0, stream2_>>>(bs_.p, chunks_.p, xd_.p, acc_.p, red_part_.p);
    nl++;
  }
  ContactStep cs{nullptr, nullptr, nullptr, ccount_.p, nullptr, mgr_chain ? mgrM_.p : nullptr};
  if (contact_) {
    cs.rec = crec_.p;
    cs.list = clist_.p;
    if (mgr_blocks) { cs.blk = cblk_.p; cs.Mc = Mc_.p; }
  }
  k_rigid_step<T><<<nb_, RIGID_THREADS, 0, stream2_>>>(bs_.p, nb_, rc_, cs, body_chunks_.p, red_part_.p, x0d_.p,
                                                        xd_.p, vd_.p);
  nl++;
  DF_CK(cudaEventRecord(ev_rigid_state_, stream2_));
  if (!manager_ && P_.enable_gradient) {
    // the per-body chain rule and its tape rows, beside the next step
    DF_CK(cudaStreamWaitEvent(stream3_, ev_rigid_state_, 0));
    pend(DFSPH_K_RIGID, nd_, stream2_);
    pbegin(stream3_);
    k_rigid_chain<<<nb_, CHAIN_THREADS, 0, stream3_>>>(bs_.p, nb_, rc_, tape_step);
    launched();
    pend(DFSPH_K_RIGID, nd_, stream3_);
    DF_CK(cudaEventRecord(ev_chain_done_, stream3_));
    chain_pending_ = true;
    pbegin(stream2_);
  }
  if (mgr_chain || mgr_blocks) {
    MgrConsts mc{rc_.dt, nb_, rc_.gyroscopic, n_ > 0 ? 1 : 0, contact_ ? 1 : 0, mgr_chain ? 1 : 0};
    if (mgr_chain) {
      const int ncol = 6 * nb_ + (tape_step ? 2 * NSTATE * nb_ : 0);
      k_manager_coef<<<1, 64, 0, stream2_>>>(bs_.p, mc, mgrC_.p);
      k_manager_columns<<<ncol, 32, 0, stream2_>>>(mc, mgrC_.p, mgrM_.p, Mc_.p, mgrS_.p, tape_step);
      nl += 2;
    }
    if (mgr_blocks) {
      k_manager_blocks<<<blocks(nb_ * nb_ * NJAC), 256, 0, stream2_>>>(bs_.p, nb_, mgrM_.p, Mc_.p);
      nl++;
    }
  }
  launched(nl);
  pend(DFSPH_K_RIGID, nd_, stream2_);
  DF_CK(cudaEventRecord(ev_rigid_done_, stream2_));
  rigid_pending_ = true;
  rigid_state_pending_ = true;
  check_launch();
}

// The contact pass reads only the bodies and their samples as the step found them (after
// the velocity overrides and this step's sort of the samples), which the fluid solve does
// not change: it runs on the rigid stream from the point the fluid stream has reached.
template <class T>
void Engine<T>::launch_contact() {
  if (nd_ == 0) return;
  DF_CK(cudaEventRecord(ev_contact_in_, stream_));
  DF_CK(cudaStreamWaitEvent(stream2_, ev_contact_in_, 0));
  pbegin(stream2_);
  cc_.dt = rc_.dt;
  cc_.grad = manager_ ? 1 : 0;
  // samples of the dynamic bodies against every boundary sample; the dynamic cell table
  // is this step's
  k_contact_samples<T><<<blocks(nd_ * CONTACT_LANES, 128), 128, 0, stream2_>>>(
      cc_, fc_.grid, fc_.h2, ns_, nd_, bs_.p, BR_.p, cstartS_.p, cstartD_.p, bodyS_.p, x0S_.p, bodyd_.p,
      dynSortedToBody_.p, xd_.p, x0d_.p, cvol0S_.p, cvol0D_.p, cdens0D_.p, crec_.p, cc_.grad ? cblk_.p : nullptr);
  launched();
  pend(DFSPH_K_RIGID, nd_, stream2_);
  contact_launched_ = true;
  check_launch();
}

template <class T>
int Engine<T>::step(int nsteps, dfsph_step_stats *st) {
  if (nsteps < 0) throw DfsphException(DFSPH_ERR_INVALID_ARG, "nsteps < 0");
  dev_epoch_++;
  int rc = DFSPH_OK;
  int64_t ti = 0, tv = 0;
  for (int s = 0; s < nsteps; s++) {
    const double h_step = dt_cur_;  // the step's initial size (positions, time)
    sort_fluid();  // overlaps the previous step's rigid kernels
    wait_rigid_state();
    begin_step();
    sort_dynamic();
    if (n_ > 0) {
      {
        // the divergence solve's warm-start density change is computed by the list build
        const bool divwarm = P_.enable_divergence_solver && P_.use_divergence_warmstart;
        pbegin();
#define DF_LISTS(W)                                                                                                \
  k_lists_density_factor<T, W><<<blocks(n_, LIST_THREADS), LIST_THREADS, 0, stream_>>>(                            \
      fc_, R_[cur_].p, cstartF_.p, BR_.p, cstartS_.p, nd_ ? cstartD_.p : nullptr, ns_, flist_.p, fcount_.p, blist_.p, \
      bcount_.p, rho_.p, alpha_.p, sumgrad_.p, err_.p, Q_.p, rhoAdv_.p, kappaV_[cur_].p)
#define DF_FROM_LISTS(W)                                                                                           \
  k_density_factor_from_lists<T, W><<<blocks(n_, LIST_THREADS), LIST_THREADS, 0, stream_>>>(                       \
      fc_, R_[cur_].p, BR_.p, flist_.p, fcount_.p, blist_.p, bcount_.p, rho_.p, alpha_.p, sumgrad_.p, Q_.p,         \
      rhoAdv_.p, kappaV_[cur_].p)
        if (fc_.lpp == 1) {
          if (divwarm) DF_LISTS(true);
          else DF_LISTS(false);
        } else {
          // small scenes: the candidate scan one warp per particle, then the same arithmetic
          k_lists_scan_warp<T><<<blocks(n_ * 32, LIST_THREADS), LIST_THREADS, 0, stream_>>>(
              fc_, R_[cur_].p, cstartF_.p, BR_.p, cstartS_.p, nd_ ? cstartD_.p : nullptr, ns_, flist_.p, fcount_.p,
              blist_.p, bcount_.p, err_.p);
          launched();
          if (divwarm) DF_FROM_LISTS(true);
          else DF_FROM_LISTS(false);
        }
#undef DF_FROM_LISTS
#undef DF_LISTS
        launched();
        pend(DFSPH_K_LISTS_DENSITY, n_);
      }
      if (nd_) {
        pbegin();
        k_bf_lists<T><<<blocks(nd_ * 32, 128), 128, 0, stream_>>>(fc_, nd_, xd_.p, R_[cur_].p, cstartF_.p, kbf_, bflist_.p,
                                                        bfcount_.p, err_.p);
        launched();
        pend(DFSPH_K_BF_LISTS, nd_);
      }
      check_launch();
      xs_fuse_ = P_.surface_tension_method != 2 && P_.viscosity_boundary == 0.0;
      xs_done_ = false;
      if (P_.enable_divergence_solver) solve(false);
      else { last_iters_v_ = 0; last_err_v_ = 0.0; }
      const int nv = 1 - cur_;
      const int scale_kv = (P_.enable_divergence_solver && P_.use_divergence_warmstart) ? 1 : 0;
      pbegin();
      if (!xs_done_) {
        if (P_.surface_tension_method == 2) {
          k_normals<T><<<blocks(n_), 256, 0, stream_>>>(fc_, R_[cur_].p, flist_.p, fcount_.p, rho_.p, N_.p);
          if (fc_.lpp == 1)
            k_xsph_advect<T, true, 1><<<blocks(n_), 256, 0, stream_>>>(fc_, R_[cur_].p, R_[nv].p, flist_.p, fcount_.p,
                                                                       kappaV_[cur_].p, scale_kv, N_.p, BR_.p, blist_.p,
                                                                       bcount_.p, rho_.p);
          else
            k_xsph_advect<T, true, LPP_MAX><<<blocks(n_ * LPP_MAX), 256, 0, stream_>>>(
                fc_, R_[cur_].p, R_[nv].p, flist_.p, fcount_.p, kappaV_[cur_].p, scale_kv, N_.p, BR_.p, blist_.p,
                bcount_.p, rho_.p);
          launched();
        } else {
          if (fc_.lpp == 1)
            k_xsph_advect<T, false, 1><<<blocks(n_), 256, 0, stream_>>>(fc_, R_[cur_].p, R_[nv].p, flist_.p, fcount_.p,
                                                                        kappaV_[cur_].p, scale_kv, nullptr, BR_.p,
                                                                        blist_.p, bcount_.p, rho_.p);
          else
            k_xsph_advect<T, false, LPP_MAX><<<blocks(n_ * LPP_MAX), 256, 0, stream_>>>(
                fc_, R_[cur_].p, R_[nv].p, flist_.p, fcount_.p, kappaV_[cur_].p, scale_kv, nullptr, BR_.p, blist_.p,
                bcount_.p, rho_.p);
        }
        launched();
        if (P_.viscosity_boundary != 0.0 && nd_ > 0) {
          // the bodies' reaction, from the velocities before the XSPH update (still in R_[cur_])
          k_visc_boundary_force<T><<<blocks(nd_), 256, 0, stream_>>>(fc_, nd_, xd_.p, vd_.p, R_[cur_].p, rho_.p,
                                                                     bflist_.p, bfcount_.p, acc_.p);
          launched();
        }
      }
      pend(DFSPH_K_XSPH, n_);
      // the advected state lives in the other record buffer: swap the record pair only
      std::swap(R_[cur_].p, R_[nv].p);
      // CFL: the new step size takes effect from the pressure solve on, as in the reference
      // (updateTimeStepSize runs after the non-pressure forces, TimeStepDiffDFSPH.cpp:583;
      // the advection, position update and time advance keep the step's initial size)
      if (P_.cfl_method == 1) set_dt(cfl_time_step());
      // the contact pass overlaps the pressure solve (it needs the step size of the rigid step)
      if (contact_) launch_contact();
      solve(true);
      if (ml_record_ && P_.use_pressure_warmstart) {
        k_ml_target<T><<<blocks(n_), 256, 0, stream_>>>(n_, kappa_[cur_].p, kfin_.p);
        launched();
      }
      // the rigid kernels need the bodies' forces of the last sweep, not the positions
      // update: they start beside it
      DF_CK(cudaEventRecord(ev_fluid_done_, stream_));
      fluid_done_recorded_ = true;
      pbegin();
      k_integrate<T><<<blocks(n_), 256, 0, stream_>>>(fc_, R_[cur_].p, kappa_[cur_].p,
                                                      P_.use_pressure_warmstart ? 1 : 0, (T)h_step,
                                                      (xs_done_ && scale_kv) ? kappaV_[cur_].p : nullptr, (T)h_step);
      launched();
      pend(DFSPH_K_INTEGRATE, n_);
    } else {
      last_iters_ = last_iters_v_ = 0;
    }
    t_ += h_step;
    rigid_end();
    finished_ = t_ >= P_.target_time + P_.uniform_accelerate_rb_time;
    ti += last_iters_;
    tv += last_iters_v_;
    if (last_iters_ >= P_.max_iterations || (P_.enable_divergence_solver && last_iters_v_ >= P_.max_iterations_v))
      rc = DFSPH_ERR_NOT_CONVERGED;
  }
  // the error word and the body states come back with the step's final synchronisation
  // (the host mirror of the bodies is then current without another round trip). The bodies
  // are final after k_rigid_step: the per-body chain rule (the mirror's G is refreshed by
  // get_rigid_grad) and the gradient manager's kernels may still run; what reads their
  // results (gradient getters, checkpoints, the adjoint, body uploads, reset) waits for them.
  wait_rigid_state();
  if (nb_ > 0)
    DF_CK(cudaMemcpyAsync(hbs_pin_, bs_.p, nb_ * sizeof(BodyState), cudaMemcpyDeviceToHost, stream_));
  DF_CK(cudaMemcpyAsync(err_host_, err_.p, sizeof(int), cudaMemcpyDeviceToHost, stream_));
  DF_CK(cudaStreamSynchronize(stream_));
  hbs_.assign(hbs_pin_, hbs_pin_ + nb_);
  hbs_epoch_ = dev_epoch_;
  hbs_chain_stale_ = chain_pending_;
#ifdef DFSPH_BOUNDS_CHECK
  {
    int be = 0;
    DF_CK(cudaMemcpyFromSymbol(&be, g_dfsph_bounds_err, sizeof(int)));
    if (be) {
      const int zero = 0;
      DF_CK(cudaMemcpyToSymbol(g_dfsph_bounds_err, &zero, sizeof(int)));
      std::string m = "bounds-checked build: index out of range:";
      if (be & BOUNDS_FLUID_LIST) m += " fluid neighbour list;";
      if (be & BOUNDS_BOUNDARY_LIST) m += " boundary neighbour list;";
      if (be & BOUNDS_SAMPLE_LIST) m += " dynamic sample's fluid list;";
      if (be & BOUNDS_CELL_RANGE) m += " cell range;";
      throw DfsphException(DFSPH_ERR_DEVICE, m);
    }
  }
#endif
  raise_error_word(*err_host_);
  if (st) {
    st->steps_done = nsteps;
    st->pressure_iterations = last_iters_;
    st->divergence_iterations = last_iters_v_;
    st->trajectory_finished = finished_ ? 1 : 0;
    st->pressure_avg_error = last_err_;
    st->divergence_avg_error = last_err_v_;
    st->total_pressure_iterations = ti;
    st->total_divergence_iterations = tv;
    st->time = t_;
    st->time_step = dt_cur_;
  }
  return rc;
}

// ----------------------------------------------------------------- accessors
template <class T>
void Engine<T>::set_rigid_init(int b, const double *v, const double *w) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  for (int k = 0; k < 3; k++) { init_v_[3 * b + k] = v[k]; init_w_[3 * b + k] = w[k]; }
}
template <class T>
void Engine<T>::get_rigid_init(int b, double *v, double *w) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  for (int k = 0; k < 3; k++) { v[k] = init_v_[3 * b + k]; w[k] = init_w_[3 * b + k]; }
}
template <class T>
void Engine<T>::get_rigid_state(int b, double *x, double *q, double *v, double *w) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  const BodyState &B = host_body(b);
  for (int k = 0; k < 3; k++) { if (x) x[k] = B.x[k]; if (v) v[k] = B.v[k]; if (w) w[k] = B.w[k]; }
  if (q) for (int k = 0; k < 4; k++) q[k] = B.q[k];
}
template <class T>
void Engine<T>::set_rigid_velocity(int b, const double *v, const double *w) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  std::vector<BodyState> bsv;
  body_state_download(bsv);
  for (int k = 0; k < 3; k++) { bsv[b].v[k] = v[k]; bsv[b].w[k] = w[k]; }
  body_state_upload(bsv);
  if (nd_ > 0) {
    k_boundary_update<T><<<blocks(nd_), 256, 0, stream_>>>(bs_.p, nd_, x0d_.p, bodyd_.p, xd_.p, vd_.p, 1);
    launched();
    sync_all();
  }
}
template <class T>
void Engine<T>::get_rigid_force(int b, double *F, double *Tq) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  const BodyState &B = host_body(b);
  for (int k = 0; k < 3; k++) { F[k] = B.F[k]; Tq[k] = B.T[k]; }
}
template <class T>
void Engine<T>::get_rigid_mass(int b, double *m, double *I) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  const BodyState &B = host_body(b);
  *m = B.mass;
  for (int k = 0; k < 9; k++) I[k] = B.I[k];
}
template <class T>
void Engine<T>::get_rigid_grad(int b, double *out) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  if (hbs_chain_stale_) {  // the mirror was copied while the last step's chain rule could run
    body_state_download(hbs_);  // (waits for it)
    hbs_epoch_ = dev_epoch_;
    hbs_chain_stale_ = false;
  }
  const double *G = host_body(b).G;
  double *o = out;
  // x_v0 x_w0 q_v0 q_w0 v_v0 v_w0 w_v0 w_w0
  const int r0[4] = {0, 3, 7, 10}, nr[4] = {3, 4, 3, 3};
  for (int blk = 0; blk < 4; blk++)
    for (int c0 = 0; c0 < 6; c0 += 3)
      for (int r = 0; r < nr[blk]; r++)
        for (int c = 0; c < 3; c++) *o++ = G[(r0[blk] + r) * 6 + c0 + c];
}
template <class T>
void Engine<T>::get_net_jacobians(int b, double *out) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  const BodyState &B = host_body(b);
  for (int k = 0; k < NJAC; k++) out[k] = B.nets[k];
}
template <class T>
void Engine<T>::backward(const double *dL, double *out) {
  if (!dL || !out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL buffer");
  if (manager_) {
    // two sweeps (v0 and omega0 columns) from the same dL_dstate
    const size_t n = (size_t)NSTATE * nb_;
    std::vector<double> lam(2 * n), res(2 * n);
    for (size_t k = 0; k < n; k++) lam[k] = lam[n + k] = dL[k];
    adjoint_sweep(lam.data(), res.data());
    for (int b = 0; b < nb_; b++)
      for (int k = 0; k < 3; k++) {
        out[6 * b + k] = res[(size_t)NSTATE * b + 7 + k];
        out[6 * b + 3 + k] = res[n + (size_t)NSTATE * b + 10 + k];
      }
    return;
  }
  std::vector<double> lam(dL, dL + (size_t)NSTATE * nb_), res((size_t)NSTATE * nb_);
  if (tape_len_ > 0 && nb_ > 0) {
    DBuf<double> li, lo;
    li.alloc(lam.size());
    lo.alloc(lam.size());
    DF_CK(cudaMemcpyAsync(li.p, lam.data(), lam.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
    wait_rigid();
    k_backward<<<nb_, 32, 0, stream_>>>(tape_.p, (int)tape_len_, nb_, li.p, lo.p);
    launched();
    check_launch();
    DF_CK(cudaMemcpyAsync(res.data(), lo.p, res.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    sync_all();
  } else {
    res = lam;
  }
  for (int b = 0; b < nb_; b++)
    for (int k = 0; k < 6; k++) out[6 * b + k] = res[(size_t)NSTATE * b + 7 + k];
}

template <class T>
void Engine<T>::copy_field(int f, double *dst, int64_t n) {
  sync_all();
  const bool bfield = f == DFSPH_FIELD_BOUNDARY_X || f == DFSPH_FIELD_BOUNDARY_V || f == DFSPH_FIELD_BOUNDARY_PSI;
  const int comps = (f == DFSPH_FIELD_X || f == DFSPH_FIELD_V || f == DFSPH_FIELD_SUM_GRAD_P ||
                     f == DFSPH_FIELD_BOUNDARY_X || f == DFSPH_FIELD_BOUNDARY_V) ? 3 : 1;
  const int64_t rows = bfield ? (ns_ + nd_) : n_;
  if (f < 0 || f > DFSPH_FIELD_BOUNDARY_PSI) throw DfsphException(DFSPH_ERR_INVALID_ARG, "field id");
  if (n != rows * comps) throw DfsphException(DFSPH_ERR_INVALID_ARG, "field buffer size mismatch");
  if (!bfield) {
    if (n_ == 0) return;
    std::vector<int> perm(n_);
    DF_CK(cudaMemcpy(perm.data(), perm_[cur_].p, n_ * sizeof(int), cudaMemcpyDeviceToHost));
    if (comps == 3) {
      std::vector<V4<T>> h(n_);
      if (f == DFSPH_FIELD_SUM_GRAD_P) {
        DF_CK(cudaMemcpy(h.data(), sumgrad_.p, n_ * sizeof(V4<T>), cudaMemcpyDeviceToHost));
      } else {
        std::vector<Rec<T>> rr(n_);
        DF_CK(cudaMemcpy(rr.data(), R_[cur_].p, n_ * sizeof(Rec<T>), cudaMemcpyDeviceToHost));
        for (int i = 0; i < n_; i++) h[i] = f == DFSPH_FIELD_X ? rr[i].x : rr[i].v;
      }
      for (int i = 0; i < n_; i++) {
        double *o = dst + 3 * (size_t)perm[i];
        o[0] = h[i].x; o[1] = h[i].y; o[2] = h[i].z;
      }
    } else {
      std::vector<T> h(n_);
      const T *src = f == DFSPH_FIELD_DENSITY ? rho_.p
                     : f == DFSPH_FIELD_FACTOR ? alpha_.p
                     : f == DFSPH_FIELD_KAPPA ? kappa_[cur_].p
                     : f == DFSPH_FIELD_KAPPA_V ? kappaV_[cur_].p
                                                : rhoAdv_.p;
      DF_CK(cudaMemcpy(h.data(), src, n_ * sizeof(T), cudaMemcpyDeviceToHost));
      for (int i = 0; i < n_; i++) dst[perm[i]] = h[i];
    }
    return;
  }
  std::vector<V4<T>> sx(ns_), sd(nd_);
  const bool wantv = f == DFSPH_FIELD_BOUNDARY_V;
  if (ns_) {
    std::vector<Rec<T>> sr(ns_);
    DF_CK(cudaMemcpy(sr.data(), BR_.p, ns_ * sizeof(Rec<T>), cudaMemcpyDeviceToHost));
    for (int q = 0; q < ns_; q++) sx[q] = wantv ? sr[q].v : sr[q].x;
  }
  if (nd_) DF_CK(cudaMemcpy(sd.data(), wantv ? vd_.p : xd_.p, nd_ * sizeof(V4<T>), cudaMemcpyDeviceToHost));
  auto put = [&](int orig, const V4<T> &p) {
    if (f == DFSPH_FIELD_BOUNDARY_PSI) dst[orig] = p.w;
    else { dst[3 * (size_t)orig] = p.x; dst[3 * (size_t)orig + 1] = p.y; dst[3 * (size_t)orig + 2] = p.z; }
  };
  for (int s = 0; s < ns_; s++) put(static_orig_[s], sx[s]);
  for (int d = 0; d < nd_; d++) put(dyn_orig_[d], sd[d]);
}

template <class T>
void Engine<T>::set_field(int f, const double *src, int64_t n) {
  sync_all();
  const int comps = (f == DFSPH_FIELD_X || f == DFSPH_FIELD_V) ? 3 : 1;
  if (!(f == DFSPH_FIELD_X || f == DFSPH_FIELD_V || f == DFSPH_FIELD_KAPPA || f == DFSPH_FIELD_KAPPA_V))
    throw DfsphException(DFSPH_ERR_INVALID_ARG, "field is not settable");
  if (n != (int64_t)n_ * comps) throw DfsphException(DFSPH_ERR_INVALID_ARG, "field buffer size mismatch");
  if (n_ == 0) return;
  std::vector<int> perm(n_);
  DF_CK(cudaMemcpy(perm.data(), perm_[cur_].p, n_ * sizeof(int), cudaMemcpyDeviceToHost));
  if (comps == 3) {
    std::vector<Rec<T>> rr(n_);
    DF_CK(cudaMemcpy(rr.data(), R_[cur_].p, n_ * sizeof(Rec<T>), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n_; i++) {
      const double *s = src + 3 * (size_t)perm[i];
      V4<T> &dst = f == DFSPH_FIELD_X ? rr[i].x : rr[i].v;
      dst.x = (T)s[0]; dst.y = (T)s[1]; dst.z = (T)s[2];
    }
    DF_CK(cudaMemcpy(R_[cur_].p, rr.data(), n_ * sizeof(Rec<T>), cudaMemcpyHostToDevice));
  } else {
    std::vector<T> h(n_);
    for (int i = 0; i < n_; i++) h[i] = (T)src[perm[i]];
    DF_CK(cudaMemcpy(f == DFSPH_FIELD_KAPPA ? kappa_[cur_].p : kappaV_[cur_].p, h.data(), n_ * sizeof(T),
                     cudaMemcpyHostToDevice));
  }
}

template <class T>
void Engine<T>::neighbors(int which, int64_t *start, int32_t *idx, int64_t *total) {
  sync_all();
  if (step_count_ == 0) throw DfsphException(DFSPH_ERR_STATE, "no neighbour search has run yet");
  std::vector<std::vector<int32_t>> rows;
  std::vector<int> perm(std::max(n_, 1));
  if (n_) DF_CK(cudaMemcpy(perm.data(), perm_[cur_].p, n_ * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> d2b(std::max(nd_, 1));
  if (nd_) DF_CK(cudaMemcpy(d2b.data(), dynSortedToBody_.p, nd_ * sizeof(int), cudaMemcpyDeviceToHost));
  auto bmap = [&](int k) { return k < ns_ ? static_orig_[k] : dyn_orig_[d2b[k - ns_]]; };
  if ((which == DFSPH_NB_FLUID_FLUID || which == DFSPH_NB_FLUID_BOUNDARY) && !start && !idx) {
    // total only: the list lengths suffice
    std::vector<int> cnt(std::max(n_, 1));
    if (n_)
      DF_CK(cudaMemcpy(cnt.data(), which == DFSPH_NB_FLUID_FLUID ? fcount_.p : bcount_.p, n_ * sizeof(int),
                       cudaMemcpyDeviceToHost));
    int64_t t = 0;
    for (int i = 0; i < n_; i++) t += cnt[i];
    if (total) *total = t;
    return;
  }
  if (which == DFSPH_NB_FLUID_FLUID || which == DFSPH_NB_FLUID_BOUNDARY) {
    const bool ff = which == DFSPH_NB_FLUID_FLUID;
    const int K = ff ? fc_.kf : fc_.kb;
    std::vector<int> cnt(std::max(n_, 1)), lst((size_t)std::max(n_, 1) * K);
    if (n_) {
      DF_CK(cudaMemcpy(cnt.data(), ff ? fcount_.p : bcount_.p, n_ * sizeof(int), cudaMemcpyDeviceToHost));
      DF_CK(cudaMemcpy(lst.data(), ff ? flist_.p : blist_.p, (size_t)n_ * K * sizeof(int), cudaMemcpyDeviceToHost));
    }
    rows.assign(n_, {});
    for (int i = 0; i < n_; i++) {
      auto &r = rows[perm[i]];
      for (int k = 0; k < cnt[i]; k++) {
        const int j = lst[(size_t)k * n_ + i];
        r.push_back(ff ? perm[j] : bmap(j));
      }
    }
  } else if (which == DFSPH_NB_BOUNDARY_FLUID) {
    rows.assign(ns_ + nd_, {});
    std::vector<int> cnt(std::max(nd_, 1)), lst((size_t)std::max(nd_, 1) * kbf_);
    if (nd_) {
      DF_CK(cudaMemcpy(cnt.data(), bfcount_.p, nd_ * sizeof(int), cudaMemcpyDeviceToHost));
      DF_CK(cudaMemcpy(lst.data(), bflist_.p, (size_t)nd_ * kbf_ * sizeof(int), cudaMemcpyDeviceToHost));
    }
    for (int d = 0; d < nd_; d++) {
      auto &r = rows[dyn_orig_[d]];
      for (int k = 0; k < cnt[d]; k++) r.push_back(perm[lst[(size_t)k * nd_ + d]]);
    }
  } else {
    throw DfsphException(DFSPH_ERR_INVALID_ARG, "neighbour set id");
  }
  int64_t tot = 0;
  for (auto &r : rows) { std::sort(r.begin(), r.end()); tot += (int64_t)r.size(); }
  *total = tot;
  if (start) {
    start[0] = 0;
    for (size_t i = 0; i < rows.size(); i++) start[i + 1] = start[i] + (int64_t)rows[i].size();
  }
  if (idx) {
    int64_t o = 0;
    for (auto &r : rows) for (int v : r) idx[o++] = v;
  }
}

}  // namespace dfsph

namespace dfsph {
template <class T>
void Engine<T>::record_event(int slot) {
  if (slot < 0 || slot >= 8) throw DfsphException(DFSPH_ERR_INVALID_ARG, "event slot");
  if (!ev_[slot]) DF_CK(cudaEventCreate(&ev_[slot]));
  DF_CK(cudaEventRecord(ev_[slot], stream_));
}
template <class T>
double Engine<T>::event_elapsed(int a, int b) {
  if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ev_[a] || !ev_[b]) throw DfsphException(DFSPH_ERR_INVALID_ARG, "event slot");
  DF_CK(cudaEventSynchronize(ev_[b]));
  float ms = 0.f;
  DF_CK(cudaEventElapsedTime(&ms, ev_[a], ev_[b]));
  return (double)ms;
}
template <class T>
void Engine<T>::resolve_profile() {
  if (pending_.empty()) return;
  sync_all();
  for (auto &r : pending_) {
    float ms = 0.f;
    DF_CK(cudaEventElapsedTime(&ms, r.a, r.b));
    prof_launches_[r.k] += 1;
    prof_ms_[r.k] += ms;
    prof_units_[r.k] += r.units;
    pool_.push_back(r.a);
    pool_.push_back(r.b);
  }
  pending_.clear();
}
template <class T>
void Engine<T>::profile_enable(bool on) {
  resolve_profile();
  for (int k = 0; k < DFSPH_PROFILE_COUNT; k++) { prof_launches_[k] = 0; prof_ms_[k] = 0; prof_units_[k] = 0; }
  prof_on_ = on;
}
template <class T>
void Engine<T>::profile_read(int k, int64_t *launches, double *ms, int64_t *units) {
  if (k < 0 || k >= DFSPH_PROFILE_COUNT) throw DfsphException(DFSPH_ERR_INVALID_ARG, "kernel class or phase");
  resolve_profile();
  if (launches) *launches = prof_launches_[k];
  if (ms) *ms = prof_ms_[k];
  if (units) *units = prof_units_[k];
}
}  // namespace dfsph

namespace dfsph {
template <class T>
void Engine<T>::set_rigid_state(int b, const double *x, const double *q, const double *v, const double *w) {
  if (b < 0 || b >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  if (!x || !q || !v || !w) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL vector");
  const double qn = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  if (!(qn > 0)) throw DfsphException(DFSPH_ERR_INVALID_ARG, "zero quaternion");
  std::vector<BodyState> bsv;
  body_state_download(bsv);
  BodyState &B = bsv[b];
  for (int k = 0; k < 3; k++) { B.x[k] = x[k]; B.v[k] = v[k]; B.w[k] = w[k]; }
  for (int k = 0; k < 4; k++) B.q[k] = q[k] / qn;
  world_inertia(B);
  body_state_upload(bsv);
  if (nd_ > 0) {
    k_boundary_update<T><<<blocks(nd_), 256, 0, stream_>>>(bs_.p, nd_, x0d_.p, bodyd_.p, xd_.p, vd_.p, 1);
    launched();
    sync_all();
  }
}

template <class T>
void Engine<T>::set_gradient_enabled(bool on) {
  P_.enable_gradient = on ? 1 : 0;
  rc_.enable_gradient = P_.enable_gradient;
  if (on && nd_ > 0 && tape_cap_ == 0) {
    tape_cap_ = 256;
    tape_.alloc((size_t)tape_cap_ * tape_stride());
  }
}

template <class T>
int Engine<T>::checkpoint_save() {
  sync_all();
  std::unique_ptr<Snap> s(new Snap());
  const size_t N = std::max(n_, 1), ND = std::max(nd_, 1), NBd = std::max(nb_, 1);
  s->R.alloc(N); s->kap.alloc(N); s->kapV.alloc(N); s->perm.alloc(N);
  s->bs.alloc(NBd); s->xd.alloc(ND); s->vd.alloc(ND);
  DF_CK(cudaMemcpyAsync(s->R.p, R_[cur_].p, N * sizeof(Rec<T>), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(s->kap.p, kappa_[cur_].p, N * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(s->kapV.p, kappaV_[cur_].p, N * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(s->perm.p, perm_[cur_].p, N * sizeof(int), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(s->bs.p, bs_.p, NBd * sizeof(BodyState), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(s->xd.p, xd_.p, ND * sizeof(V4<T>), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(s->vd.p, vd_.p, ND * sizeof(V4<T>), cudaMemcpyDeviceToDevice, stream_));
  if (manager_) {
    s->mgrM.alloc(mgrM_.n); s->mgrS.alloc(mgrS_.n);
    DF_CK(cudaMemcpyAsync(s->mgrM.p, mgrM_.p, mgrM_.n * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
    DF_CK(cudaMemcpyAsync(s->mgrS.p, mgrS_.p, mgrS_.n * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
  }
  sync_all();
  s->t = t_; s->sc = step_count_; s->finished = finished_; s->anim = anim_; s->dt = dt_cur_;
  for (size_t k = 0; k < snaps_.size(); k++)
    if (!snaps_[k]) { snaps_[k] = std::move(s); return (int)k; }
  snaps_.push_back(std::move(s));
  return (int)snaps_.size() - 1;
}

template <class T>
void Engine<T>::checkpoint_restore(int slot) {
  if (slot < 0 || slot >= (int)snaps_.size() || !snaps_[slot]) throw DfsphException(DFSPH_ERR_INVALID_ARG, "checkpoint slot");
  Snap &s = *snaps_[slot];
  const size_t N = std::max(n_, 1), ND = std::max(nd_, 1), NBd = std::max(nb_, 1);
  sync_all();
  DF_CK(cudaMemcpyAsync(R_[cur_].p, s.R.p, N * sizeof(Rec<T>), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(kappa_[cur_].p, s.kap.p, N * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(kappaV_[cur_].p, s.kapV.p, N * sizeof(T), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(perm_[cur_].p, s.perm.p, N * sizeof(int), cudaMemcpyDeviceToDevice, stream_));
  dev_epoch_++;
  DF_CK(cudaMemcpyAsync(bs_.p, s.bs.p, NBd * sizeof(BodyState), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(xd_.p, s.xd.p, ND * sizeof(V4<T>), cudaMemcpyDeviceToDevice, stream_));
  DF_CK(cudaMemcpyAsync(vd_.p, s.vd.p, ND * sizeof(V4<T>), cudaMemcpyDeviceToDevice, stream_));
  if (manager_) {
    DF_CK(cudaMemcpyAsync(mgrM_.p, s.mgrM.p, mgrM_.n * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
    DF_CK(cudaMemcpyAsync(mgrS_.p, s.mgrS.p, mgrS_.n * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
  }
  if (nd_ > 0) DF_CK(cudaMemsetAsync(acc_.p, 0, (size_t)nd_ * ACC_STRIDE * sizeof(double), stream_));
  sync_all();
  t_ = s.t; step_count_ = s.sc; finished_ = s.finished; anim_ = s.anim;
  set_dt(s.dt);
}

template <class T>
void Engine<T>::checkpoint_free(int slot) {
  if (slot < 0 || slot >= (int)snaps_.size() || !snaps_[slot]) throw DfsphException(DFSPH_ERR_INVALID_ARG, "checkpoint slot");
  sync_all();
  snaps_[slot].reset();
}

template <class T>
void Engine<T>::adjoint_sweep(const double *lam_in, double *lam_out) {
  if (!lam_in || !lam_out) throw DfsphException(DFSPH_ERR_INVALID_ARG, "NULL buffer");
  if (manager_) {
    const size_t n2 = 2 * (size_t)NSTATE * nb_;
    if (tape_len_ == 0 || nb_ == 0) {
      for (size_t k = 0; k < n2; k++) lam_out[k] = lam_in[k];
      return;
    }
    DBuf<double> li, lo;
    li.alloc(n2);
    lo.alloc(n2);
    DF_CK(cudaMemcpyAsync(li.p, lam_in, n2 * sizeof(double), cudaMemcpyHostToDevice, stream_));
    wait_rigid();
    k_backward_mgr<<<1, 256, 0, stream_>>>(tape_.p, (int)tape_len_, NSTATE * nb_, li.p, lo.p);
    launched();
    check_launch();
    DF_CK(cudaMemcpyAsync(lam_out, lo.p, n2 * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    sync_all();
    return;
  }
  const size_t m = (size_t)NSTATE * std::max(nb_, 1);
  if (tape_len_ == 0 || nb_ == 0) {
    for (size_t k = 0; k < (size_t)NSTATE * nb_; k++) lam_out[k] = lam_in[k];
    return;
  }
  DBuf<double> li, lo;
  li.alloc(m);
  lo.alloc(m);
  DF_CK(cudaMemcpyAsync(li.p, lam_in, (size_t)NSTATE * nb_ * sizeof(double), cudaMemcpyHostToDevice, stream_));
  wait_rigid();
  k_backward<<<nb_, 32, 0, stream_>>>(tape_.p, (int)tape_len_, nb_, li.p, lo.p);
  launched();
  check_launch();
  DF_CK(cudaMemcpyAsync(lam_out, lo.p, (size_t)NSTATE * nb_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  sync_all();
}
template <class T>
void Engine<T>::get_manager_grad(int b, int b2, double *out) {
  if (!manager_) throw DfsphException(DFSPH_ERR_UNSUPPORTED, "the gradient manager is off (use_rigid_gradient_manager)");
  if (b < 0 || b >= nb_ || b2 < 0 || b2 >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  sync_all();
  const size_t ncol = 6 * (size_t)nb_;
  std::vector<double> rows((size_t)NSTATE * ncol);
  DF_CK(cudaMemcpy(rows.data(), mgrS_.p + (size_t)NSTATE * b * ncol, rows.size() * sizeof(double), cudaMemcpyDeviceToHost));
  // x_v0 x_w0 (3x3), q_v0 q_w0 (4x3), v_v0 v_w0, w_v0 w_w0 (3x3): rows of one component
  // group, columns v0 (0..2) or omega0 (3..5) of body b2
  double *o = out;
  const int groups[4][2] = {{0, 3}, {3, 4}, {7, 3}, {10, 3}};
  for (auto &g : groups)
    for (int half = 0; half < 2; half++)
      for (int r = 0; r < g[1]; r++)
        for (int j = 0; j < 3; j++) *o++ = rows[(size_t)(g[0] + r) * ncol + 6 * b2 + 3 * half + j];
}

template <class T>
void Engine<T>::get_manager_jacobians(int b, int b2, double *out) {
  if (!manager_) throw DfsphException(DFSPH_ERR_UNSUPPORTED, "the gradient manager is off (use_rigid_gradient_manager)");
  if (b < 0 || b >= nb_ || b2 < 0 || b2 >= nb_) throw DfsphException(DFSPH_ERR_INVALID_ARG, "body index");
  sync_all();
  DF_CK(cudaMemcpy(out, mgrM_.p + ((size_t)b * nb_ + b2) * NJAC, NJAC * sizeof(double), cudaMemcpyDeviceToHost));
}

template <class T>
void Engine<T>::contact_count(int64_t *nc, int64_t *na) {
  sync_all();
  *nc = 0; *na = 0;
  if (!contact_ || nb_ == 0) return;
  std::vector<int> c(2 * (size_t)nb_);
  DF_CK(cudaMemcpy(c.data(), ccount_.p, c.size() * sizeof(int), cudaMemcpyDeviceToHost));
  for (int b = 0; b < nb_; b++) { *nc += c[2 * b]; *na += c[2 * b + 1]; }
}

// ----------------------------------------------------------------- learned warm start
template <class T>
void Engine<T>::ml_buffers() {
  if (F_.n >= (size_t)std::max(n_, 1)) return;
  const size_t N = std::max(n_, 1);
  F_.alloc(N);
  kfin_.alloc(N);
  mlflag_.alloc(N);
  mlscan_.prepare(N);
  DF_CK(cudaMemsetAsync(F_.p, 0, N * sizeof(float4), stream_));
  DF_CK(cudaMemsetAsync(kfin_.p, 0, N * sizeof(float), stream_));
}

template <class T>
void Engine<T>::set_warmstart_model(const MlpView *v) {
  if (!v) { ml_on_ = false; return; }
  int dev = 0;
  DF_CK(cudaGetDevice(&dev));
  if (v->device != dev) throw DfsphException(DFSPH_ERR_INVALID_ARG, "model and context live on different devices");
  if (!P_.use_pressure_warmstart)
    throw DfsphException(DFSPH_ERR_STATE, "the learned warm start needs use_pressure_warmstart");
  ml_buffers();
  mlv_ = *v;
  ml_on_ = true;
}

template <class T>
void Engine<T>::ml_record(bool on) {
  if (on && !P_.use_pressure_warmstart)
    throw DfsphException(DFSPH_ERR_STATE, "recording warm-start samples needs use_pressure_warmstart");
  if (on) ml_buffers();
  ml_record_ = on;
}

// inference inside the pressure warm start: kappa_warm = MLP(features) where rho_adv > 1
template <class T>
void Engine<T>::launch_mlp_warmstart(T *kap) {
  if (n_ == 0) return;
  pbegin();
  const int ntiles = (n_ + MLP_TILE - 1) / MLP_TILE;
  const int grid = std::min(ntiles, num_sms_ * 8);
  k_mlp_infer<MlpWarmIO<T>><<<grid, MLP_THREADS, MLP_INFER_SMEM, stream_>>>(mlv_, MlpWarmIO<T>{F_.p, Q_.p, kap}, n_,
                                                                           err_.p, ERR_MLP_TIMEOUT);
  launched();
  pend(DFSPH_K_MLP, n_);
}

template <class T>
int64_t Engine<T>::ml_capture(float *x, float *y, int64_t cap) {
  if (!ml_record_ || F_.n == 0) throw DfsphException(DFSPH_ERR_STATE, "recording is off");
  if (n_ == 0) return 0;
  k_ml_flags<<<blocks(n_), 256, 0, stream_>>>(n_, F_.p, mlflag_.p);
  launched();
  int last_flag = 0, last_scan = 0;
  DF_CK(cudaMemcpyAsync(&last_flag, mlflag_.p + n_ - 1, sizeof(int), cudaMemcpyDeviceToHost, stream_));
  int64_t ls = 0;
  mlscan_.run(mlflag_.p, n_, stream_, ls);
  launches_ += ls;
  DF_CK(cudaMemcpyAsync(&last_scan, mlflag_.p + n_ - 1, sizeof(int), cudaMemcpyDeviceToHost, stream_));
  k_ml_scatter<<<blocks(n_), 256, 0, stream_>>>(n_, F_.p, kfin_.p, mlflag_.p, cap, x, y);
  launched();
  check_launch();
  sync_all();
  return std::min<int64_t>((int64_t)last_scan + last_flag, cap);
}
// ----------------------------------------------------------------- time step size
// The constants that follow from the time step (the TimeManager's size in the reference):
// dt, 1/dt, 1/dt^2 of the passes, computeGradient's Real 1/dt/dt and 1/dt with the
// unsigned copy of TimeStepDiffDFSPH.cpp:1266, and the rigid integration's dt.
template <class T>
void Engine<T>::set_dt(double h) {
  dt_cur_ = h;
  fc_.dt = (T)h;
  fc_.invH = T(1) / fc_.dt;
  fc_.invH2 = T(1) / (fc_.dt * fc_.dt);
  const T cg2 = T(1) / fc_.dt / fc_.dt, cg1 = T(1) / fc_.dt;
  pcP_.cReal = cg2;
  pcD_.cReal = cg1;
  pcP_.cTrunc = P_.truncate_gradient_coeff ? (T)(unsigned int)cg2 : cg2;
  pcD_.cTrunc = P_.truncate_gradient_coeff ? (T)(unsigned int)cg1 : cg1;
  rc_.dt = (double)fc_.dt;
  cc_.dt = rc_.dt;
}

// Simulation::updateTimeStepSizeCFL (Simulation.cpp:541-616): max(0.1, |v + h a|^2 over the
// fluid, |v_j|^2 over samples of dynamic or animated bodies); h' = factor 0.4 2r / sqrt(max)
// clamped to [min, max]. The fluid records hold v + h a once the XSPH pass has run.
template <class T>
double Engine<T>::cfl_time_step() {
  DF_CK(cudaMemsetAsync(speed2_.p, 0, sizeof(unsigned long long), stream_));
  if (n_ > 0) {
    k_max_speed2<T><<<std::min(blocks(n_), num_sms_ * 8), 256, 0, stream_>>>(n_, R_[cur_].p, nd_, vd_.p, bodyd_.p,
                                                                           bs_.p, speed2_.p);
    launched();
  }
  unsigned long long bits = 0;
  DF_CK(cudaMemcpyAsync(&bits, speed2_.p, sizeof(bits), cudaMemcpyDeviceToHost, stream_));
  sync_all();
  double m;
  std::memcpy(&m, &bits, sizeof(m));
  const T maxVel = std::max((T)0.1, (T)m);
  const T diameter = T(2) * (T)P_.particle_radius;
  T h = (T)P_.cfl_factor * T(0.4) * (diameter / std::sqrt(maxVel));
  h = std::min(h, (T)P_.cfl_max_time_step);
  h = std::max(h, (T)P_.cfl_min_time_step);
  return (double)h;
}
}  // namespace dfsph
