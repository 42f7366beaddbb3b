// engine.cuh — host orchestration of the DiffDFSPH step on one GPU (three CUDA streams per
// context: fluid, rigid bodies, per-body chain rule). Engine<T> is instantiated for float
// and double fluid arithmetic in engine_fp32.cu / engine_fp64.cu; the C ABI (abi.cu) only
// sees EngineBase.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dfsph.h"
#include "engine_api.h"
#include "common.cuh"
#include "kernels_fluid.cuh"
#include "kernels_rigid.cuh"
#include "kernels_contact.cuh"
#include "kernels_mlp.cuh"

namespace dfsph {

// ----------------------------------------------------------------- device buffer
// Owning device allocation; move-only (a copy would free the same pointer twice).
template <class E>
struct DBuf {
  E *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) { free(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  void alloc(size_t count) {
    free();
    n = count;
    if (count) DF_CK(cudaMalloc(&p, count * sizeof(E)));
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { free(); }
};

// int exclusive scan in place over n entries: out[k] = sum_{j<k} in[j]
static __global__ void k_scan_block(int n, int *__restrict__ data, int *__restrict__ block_sums) {
  constexpr int ITEMS = 4;
  __shared__ int warp_tot[32];
  const int base = (blockIdx.x * blockDim.x + threadIdx.x) * ITEMS;
  int v[ITEMS];
  int s = 0;
#pragma unroll
  for (int k = 0; k < ITEMS; k++) { v[k] = (base + k < n) ? data[base + k] : 0; s += v[k]; }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = s;
  for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, inc, o); if (lane >= o) inc += t; }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    int t = lane < nw ? warp_tot[lane] : 0;
    int ti = t;
    for (int o = 1; o < 32; o <<= 1) { int u = __shfl_up_sync(0xffffffffu, ti, o); if (lane >= o) ti += u; }
    if (lane < nw) warp_tot[lane] = ti - t;
    if (lane == nw - 1 && block_sums) block_sums[blockIdx.x] = ti;
  }
  __syncthreads();
  int run = warp_tot[w] + inc - s;
#pragma unroll
  for (int k = 0; k < ITEMS; k++) { if (base + k < n) data[base + k] = run; run += v[k]; }
}
static __global__ void k_scan_add(int n, int *__restrict__ data, const int *__restrict__ block_sums) {
  constexpr int ITEMS = 4;
  const int base = (blockIdx.x * blockDim.x + threadIdx.x) * ITEMS;
  const int add = block_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < ITEMS; k++) if (base + k < n) data[base + k] += add;
}

struct Scanner {
  static constexpr int THREADS = 1024, PER_BLOCK = THREADS * 4;
  std::vector<DBuf<int>> levels;
  void prepare(size_t n) {
    levels.clear();
    levels.reserve(8);
    size_t m = n;
    while (true) {
      size_t blocks = (m + PER_BLOCK - 1) / PER_BLOCK;
      levels.emplace_back();
      levels.back().alloc(std::max<size_t>(blocks, 1));
      if (blocks <= 1) break;
      m = blocks;
    }
  }
  // exclusive scan of data[0..n)
  void run(int *data, int n, cudaStream_t s, int64_t &launches, int level = 0) {
    const int blocks = (n + PER_BLOCK - 1) / PER_BLOCK;
    int *bs = levels[level].p;
    k_scan_block<<<blocks, THREADS, 0, s>>>(n, data, blocks > 1 ? bs : nullptr);
    launches++;
    if (blocks > 1) {
      run(bs, blocks, s, launches, level + 1);
      k_scan_add<<<blocks, THREADS, 0, s>>>(n, data, bs);
      launches++;
    }
  }
};

// ----------------------------------------------------------------- learned warm start glue
// Inference IO inside the pressure warm start: features from F, prediction only where
// rho_adv > 1 (feature x > 0, the same gate as the reference warm start); the result is
// the stiffness of the warm-start velocity correction (Q.w) and the start of the
// solver's stiffness accumulator.
template <class T>
struct MlpWarmIO {
  const float4 *F;
  V4<T> *Q;
  T *kappa;
  __device__ bool load(int i, float f[4]) const {
    const float4 v = F[i];
    f[0] = v.x; f[1] = v.y; f[2] = v.z; f[3] = v.w;
    return v.x > 0.f;
  }
  __device__ void store(int i, float y) const {
    Q[i].w = (T)y;
    kappa[i] = (T)y;
  }
};

// the step's accumulated pressure stiffness (pass units) before the end-of-step scaling
template <class T>
static __global__ void k_ml_target(int n, const T *__restrict__ kappa, float *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)kappa[i];
}
static __global__ void k_ml_flags(int n, const float4 *__restrict__ F, int *__restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = F[i].x > 0.f ? 1 : 0;
}
static __global__ void k_ml_scatter(int n, const float4 *__restrict__ F, const float *__restrict__ kfin,
                                    const int *__restrict__ pos, int64_t cap, float *__restrict__ x,
                                    float *__restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 f = F[i];
  if (!(f.x > 0.f)) return;
  const int64_t k = pos[i];
  if (k >= cap) return;
  reinterpret_cast<float4 *>(x)[k] = f;
  y[k] = kfin[i];
}

static __global__ void k_iota2(int n, int *__restrict__ a, int *__restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { a[i] = i; b[i] = i; }
}

// ----------------------------------------------------------------- engine
template <class T>
class Engine : public EngineBase {
 public:
  explicit Engine(const dfsph_scene *sc);
  ~Engine() override;

  int step(int nsteps, dfsph_step_stats *st) override;
  void reset() override;
  void reset_gradient() override;
  void set_rigid_init(int b, const double *v, const double *w) override;
  void get_rigid_init(int b, double *v, double *w) override;
  void get_rigid_state(int b, double *x, double *q, double *v, double *w) override;
  void set_rigid_velocity(int b, const double *v, const double *w) override;
  void get_rigid_force(int b, double *F, double *Tq) override;
  void get_rigid_mass(int b, double *m, double *I) override;
  void get_rigid_grad(int b, double *out) override;
  void get_net_jacobians(int b, double *out) override;
  void backward(const double *dL, double *out) override;
  int64_t tape_length() override { return tape_len_; }
  void copy_field(int f, double *dst, int64_t n) override;
  void set_field(int f, const double *src, int64_t n) override;
  void counts(int64_t *nf, int64_t *nb) override { *nf = n_; *nb = ns_ + nd_; }
  void neighbors(int which, int64_t *start, int32_t *idx, int64_t *total) override;
  void get_time(double *t, int64_t *sc) override { *t = t_; *sc = step_count_; }
  void synchronize() override { sync_all(); }
  int64_t launches() override { return launches_; }
  void record_event(int slot) override;
  double event_elapsed(int a, int b) override;
  void profile_enable(bool on) override;
  void profile_read(int k, int64_t *launches, double *ms, int64_t *units) override;
  void set_time(double t, int64_t sc) override { t_ = t; step_count_ = sc; finished_ = t_ >= P_.target_time + P_.uniform_accelerate_rb_time; }
  void set_rigid_state(int b, const double *x, const double *q, const double *v, const double *w) override;
  void set_gradient_enabled(bool on) override;
  int checkpoint_save() override;
  void checkpoint_restore(int slot) override;
  void checkpoint_free(int slot) override;
  void adjoint_sweep(const double *lam_in, double *lam_out) override;
  void set_warmstart_model(const MlpView *v) override;
  void ml_record(bool on) override;
  int64_t ml_capture(float *x, float *y, int64_t cap) override;
  void get_manager_grad(int b, int b2, double *out) override;
  void get_manager_jacobians(int b, int b2, double *out) override;
  void contact_count(int64_t *nc, int64_t *na) override;

 private:
  // configuration
  dfsph_params P_;
  FluidConsts<T> fc_;
  RigidConsts rc_;
  PairConsts<T> pcP_{}, pcD_{};
  int n_ = 0, ns_ = 0, nd_ = 0, nb_ = 0, kbf_ = 128;
  int ncell_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaStream_t stream2_ = nullptr;  // rigid kernels (overlap the next step's fluid sort)
  cudaStream_t stream3_ = nullptr;  // the per-body chain rule (overlaps the next step)
  cudaEvent_t ev_fluid_done_ = nullptr, ev_rigid_done_ = nullptr;
  cudaEvent_t ev_rigid_state_ = nullptr;  // after k_rigid_step (bodies and samples of the step)
  cudaEvent_t ev_contact_in_ = nullptr;   // the fluid stream's point where the contact pass may start
  cudaEvent_t ev_chain_done_ = nullptr;   // after k_rigid_chain
  bool chain_pending_ = false;            // k_rigid_chain may still run (G and the tape not final)
  bool hbs_chain_stale_ = false;          // the host mirror was copied while k_rigid_chain could run
  bool rigid_pending_ = false, rigid_state_pending_ = false;
  bool contact_launched_ = false;  // this step's contact pass is already on the rigid stream
  bool fluid_done_recorded_ = false;  // ev_fluid_done_ marks this step's last solver sweep
  int64_t launches_ = 0;

  // host copies
  std::vector<double> x_init_, v_init_;
  std::vector<BodyState> body_init_;
  std::vector<double> init_v_, init_w_;  // per body
  std::vector<int> body_dyn_, body_anim0_;
  std::vector<int> static_orig_;   // sorted static index -> boundary index (body-concatenated)
  std::vector<int> dyn_orig_;      // body-order dynamic index -> boundary index
  std::vector<int> boundary_is_dyn_, boundary_slot_;  // boundary index -> (dynamic?, slot)

  // fluid (sorted order), double-buffered where the sort gathers
  DBuf<Rec<T>> R_[2];
  DBuf<Rec<T>> R_init_;  // initial records (caller order), restored by reset()
  DBuf<V4<T>> Q_;
  DBuf<V4<T>> N_;  // surface-tension normals and densities (when enabled)
  DBuf<T> kappa_[2], kappaV_[2];
  DBuf<int> perm_[2];
  int cur_ = 0;
  DBuf<T> rho_, alpha_, rhoAdv_;
  DBuf<V4<T>> sumgrad_;
  DBuf<int> fcount_, flist_, bcount_, blist_;
  DBuf<int> key_, rank_, order_, cstartF_;
  // boundary
  DBuf<Rec<T>> BR_;           // [ns + nd] static (fixed) then dynamic (cell-sorted copy)
  DBuf<int> cstartS_, cstartD_;
  DBuf<V4<T>> xd_, vd_, x0d_;  // dynamic, body order
  DBuf<int> bodyd_, keyD_, rankD_, orderD_, dynSortedToBody_, bfcount_, bflist_;
  DBuf<double> acc_;
  DBuf<RedChunk> chunks_;      // per-body reduction chunks
  DBuf<int2> body_chunks_;     // chunk range of each body
  DBuf<double> red_part_;      // chunk partial sums
  int nchunks_ = 0;
  DBuf<T> psi_;
  DBuf<BodyState> bs_;
  // reductions and flags
  DBuf<double> partials_, resid_;
  double *resid_host_ = nullptr;  // pinned, mapped
  int *err_host_ = nullptr;        // pinned: the error word, copied at the end of each step call
  BodyState *hbs_pin_ = nullptr;   // pinned: the body states, copied at the end of each step call
  double *resid_host_dev_ = nullptr;
  DBuf<int> err_;
  Scanner scan_;
  // device-resident snapshots
  struct Snap {
    DBuf<Rec<T>> R;
    DBuf<T> kap, kapV;
    DBuf<int> perm;
    DBuf<BodyState> bs;
    DBuf<V4<T>> xd, vd;
    DBuf<double> mgrM, mgrS;
    double t = 0, dt = 0;
    int64_t sc = 0;
    bool finished = false;
    std::vector<int> anim;
  };
  std::vector<std::unique_ptr<Snap>> snaps_;
  // learned warm start: features at the pressure warm start, the step's final stiffness,
  // capture flags, and the model view
  bool ml_record_ = false, ml_on_ = false;
  MlpView mlv_;
  DBuf<float4> F_;
  DBuf<float> kfin_;
  DBuf<int> mlflag_;
  Scanner mlscan_;
  int num_sms_ = 152;
  // adjoint tape: per step nb 13x13 maps (per-body chain) or two 13nb x 13nb maps (manager)
  DBuf<double> tape_;
  int64_t tape_len_ = 0, tape_cap_ = 0;
  size_t tape_stride() const {
    return manager_ ? (size_t)2 * NSTATE * nb_ * NSTATE * nb_ : (size_t)nb_ * NSTATE * NSTATE;
  }
  // rigid-rigid contact (penalty form) and the gradient manager's multi-body chain
  bool contact_ = false, manager_ = false;
  bool psi_static_done_ = false;  // static samples' psi computed (once)
  ContactConsts cc_;
  DBuf<int> bodyS_;            // body of each static sample (sorted order)
  DBuf<V4<T>> x0S_;            // local coordinates of each static sample (sorted order)
  DBuf<double> cvol0S_, cdens0S_, cvol0D_, cdens0D_;  // rest volume / density (static sorted, dynamic body order)
  DBuf<ContactRec> crec_;
  DBuf<double> cblk_;
  DBuf<int> clist_, ccount_;
  DBuf<double> Mc_, mgrM_, mgrS_;  // contact blocks of the step, manager blocks, manager chain state
  DBuf<MgrCoef> mgrC_;              // the manager's per-body coefficients of the step
  void contact_init();
  void manager_reset(bool blocks);

  // trajectory state (host)
  double dt_cur_ = 0.0;  // the time step size (changes under CFL)
  bool xs_fuse_ = false, xs_done_ = false;  // XSPH advanced by the divergence solve's last pass
  DBuf<unsigned long long> speed2_;  // CFL: max squared speed (bits of a non-negative double)
  double t_ = 0.0;
  int64_t step_count_ = 0;
  bool finished_ = false;
  std::vector<int> anim_;  // current animated flags (host mirror of the begin-step logic)
  int last_iters_ = 0, last_iters_v_ = 0;
  double last_err_ = 0.0, last_err_v_ = 0.0;

  // timing: user event slots and per-kernel-class event pairs
  cudaEvent_t ev_[8] = {};
  struct ProfRec { int k; cudaEvent_t a, b; int64_t units; };
  bool prof_on_ = false;
  std::vector<ProfRec> pending_;
  std::vector<cudaEvent_t> pool_;
  cudaEvent_t open_ev_ = nullptr;
  int64_t prof_launches_[DFSPH_PROFILE_COUNT] = {};
  double prof_ms_[DFSPH_PROFILE_COUNT] = {};
  int64_t prof_units_[DFSPH_PROFILE_COUNT] = {};
  cudaEvent_t take_event() {
    if (pool_.empty()) { cudaEvent_t e; DF_CK(cudaEventCreate(&e)); return e; }
    cudaEvent_t e = pool_.back(); pool_.pop_back(); return e;
  }
  void pbegin(cudaStream_t s = nullptr) {
    if (!prof_on_) return;
    open_ev_ = take_event();
    DF_CK(cudaEventRecord(open_ev_, s ? s : stream_));
  }
  void pend(int k, int64_t units, cudaStream_t s = nullptr) {
    if (!prof_on_ || !open_ev_) return;
    cudaEvent_t b = take_event();
    DF_CK(cudaEventRecord(b, s ? s : stream_));
    pending_.push_back({k, open_ev_, b, units});
    open_ev_ = nullptr;
  }
  // the rigid kernels' stream: the main stream waits for them before it touches rigid
  // data; host synchronisation waits for both
  // everything queued on the rigid streams (the bodies, the gradient manager and the
  // per-body chain rule)
  void wait_rigid() {
    wait_rigid_except_chain();
    if (chain_pending_) {
      DF_CK(cudaStreamWaitEvent(stream_, ev_chain_done_, 0));
      chain_pending_ = false;
    }
  }
  // the end of a step call: the bodies and the manager, while the per-body chain rule (which
  // only gradient reads and the adjoint need) may still run on its own stream
  void wait_rigid_except_chain() {
    if (!rigid_pending_) return;
    DF_CK(cudaStreamWaitEvent(stream_, ev_rigid_done_, 0));
    rigid_pending_ = false;
    rigid_state_pending_ = false;
  }
  // the next step's fluid work needs the bodies and their samples after k_rigid_step, not
  // the gradient manager's kernels, which only the rigid stream and host calls read
  void wait_rigid_state() {
    if (!rigid_state_pending_) return;
    DF_CK(cudaStreamWaitEvent(stream_, ev_rigid_state_, 0));
    rigid_state_pending_ = false;
  }
  void sync_all() {
    wait_rigid();
    DF_CK(cudaStreamSynchronize(stream_));
  }
  void resolve_profile();
  // phase timers (a whole solve); independent of the per-launch pair above
  cudaEvent_t phase_begin() {
    if (!prof_on_) return nullptr;
    cudaEvent_t e = take_event();
    DF_CK(cudaEventRecord(e, stream_));
    return e;
  }
  void phase_end(int k, cudaEvent_t a, int64_t units) {
    if (!prof_on_ || !a) return;
    cudaEvent_t b = take_event();
    DF_CK(cudaEventRecord(b, stream_));
    pending_.push_back({k, a, b, units});
  }

  int blocks(int n, int t = 256) const { return (n + t - 1) / t; }
  void launched(int k = 1) { launches_ += k; dev_epoch_++; }
  // host copy of the body states, refreshed when anything was launched or uploaded since
  int64_t dev_epoch_ = 0, hbs_epoch_ = -1;
  std::vector<BodyState> hbs_;
  const BodyState &host_body(int b) {
    if (hbs_epoch_ != dev_epoch_) { body_state_download(hbs_); hbs_epoch_ = dev_epoch_; hbs_chain_stale_ = false; }
    return hbs_[b];
  }
  void check_launch() { DF_CK(cudaGetLastError()); }

  void sort_fluid();
  void sort_dynamic();
  void sort_points(const V4<T> *pts, int stride, int count, int *key, int *rank, int *cstart, int *order);
  void compute_psi();
  void begin_step();
  void solve(bool pressure);
  void set_dt(double h);
  double cfl_time_step();
  void solve_impl(bool pressure);
  void launch_density(int mode, T *kappa_io, bool partials, float4 *feat = nullptr);
  void launch_mlp_warmstart(T *kap);
  void ml_buffers();
  void launch_velocity(T *kappa_acc);
  void launch_pairs(bool pressure, bool warm, bool grad);
  void rigid_end();
  void launch_contact();
  double read_residual();
  void grow_tape();
  void upload_fluid_initial();
  void body_state_download(std::vector<BodyState> &out);
  void body_state_upload(const std::vector<BodyState> &in);
  void check_error_word();
  void raise_error_word(int e);
};

}  // namespace dfsph
