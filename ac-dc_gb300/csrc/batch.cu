// Batched lambda paths (many instances per launch) and the serving loop.
//
// The lambda path with warm starts follows
// cpp/src/experiments/lasso_console_solver.cpp:149-172 (a geometric sequence of
// lambdas, x carried from one lambda to the next), run here for many instances
// at once.  One round is: the update kernel over every live slot, the FP64
// refresh and gap kernels over every live slot, and a control kernel with one
// block per slot that records converged lambdas and advances the path.  The
// path solver captures one round in a CUDA graph and replays it until every
// slot is done; the server runs rounds between admissions and retirements.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "acdc_internal.cuh"

namespace {

// Closed-form choice of tau (batch option autotune = 2): the largest power of
// two whose beta = 1 + (omega-1)(tau-1)/(n-1) stays at most beta_max, with at
// least 32 columns per concurrent update and no more than 1024 warps.
int autotune_tau(int64_t n, int64_t omega, double beta_max) {
  int best = 1;
  for (int tau = 1; tau <= 1024; tau *= 2) {
    const double beta =
        n > 1 ? 1.0 + ((double)omega - 1.0) * ((double)tau - 1.0) / ((double)n - 1.0) : 1.0;
    if (beta > beta_max || (int64_t)tau * 32 > std::max<int64_t>(32, n)) break;
    best = tau;
  }
  return best;
}

// Measured choice of tau for one instance.  Candidates: powers of two with
// beta = 1 + (omega-1)(tau-1)/(n-1) at most kTuneBetaMax, at least 32 columns per
// update in flight, at most 1024.  Each candidate runs a probe launch of a
// quarter epoch (at least 64 tau updates) timed with CUDA events; the probes
// use the step constants of the largest candidate's beta, which is safe for
// every smaller tau, and their updates are real progress of the solve.  A
// coordinate step is scaled by 1/beta, so the time to a given gap goes as
// beta(tau) / (updates per second at tau): the candidate with the smallest
// ratio wins.  The choice is cached per size class (log2 of n and m, mean
// column length) on the context, so a batch or a server pays the probes once
// per class.
uint64_t size_class(const acdc_problem* p) {
  auto lg = [](int64_t v) {
    uint64_t b = 0;
    while (v > 1) {
      v >>= 1;
      ++b;
    }
    return b;
  };
  const uint64_t mean_len = (uint64_t)(p->d.nnz / std::max<int64_t>(1, p->d.n));
  return (lg(p->d.n) << 40) | (lg(p->d.m) << 20) | std::min<uint64_t>(mean_len, 0xfffff) |
         ((uint64_t)p->loss << 60);
}

// Largest ESO beta among the tuner's candidates: a step scaled by 1/beta is
// always safe, and an instance whose rows are dense (beta grows fast with tau,
// underdetermined Lasso) can gain more from updates in flight than it loses to
// the smaller steps; the measurement decides.
constexpr double kTuneBetaMax = 4.0;

int measured_tau(acdc_problem* p, int wpb_cap, int* tau_out) {
  acdc_ctx* ctx = p->ctx;
  const uint64_t key = size_class(p);
  auto it = ctx->tau_cache.find(key);
  if (it != ctx->tau_cache.end()) {
    *tau_out = it->second;
    return ACDC_OK;
  }
  const int64_t n = p->d.n;
  std::vector<int> cand;
  for (int tau = 1; tau <= 1024; tau *= 2) {
    const double beta =
        n > 1 ? 1.0 + ((double)p->omega - 1.0) * ((double)tau - 1.0) / ((double)n - 1.0) : 1.0;
    if (beta > kTuneBetaMax || (int64_t)tau * 32 > std::max<int64_t>(32, n)) break;
    cand.push_back(tau);
  }
  // step constants of the largest candidate's beta for every probe
  acdc_settings s = p->s;
  s.tau = cand.back();
  s.sigma = 0;
  int rc = acdc_problem_set_settings(p, &s);
  if (rc) return rc;
  double best_cost = 0;
  int best = cand.front();
  for (int tau : cand) {
    const uint64_t count = std::max<uint64_t>((uint64_t)n / 4, 64u * (uint64_t)tau);
    UpdateParams u{};
    u.meta = p->d.meta;
    u.vals = p->d.vals;
    u.idx = p->d.idx;
    u.r = p->d.r32;
    u.active = p->d.active;
    u.counters = p->d.counters;
    u.x64 = p->d.x64;
    u.r64 = p->d.r64;
    u.x32 = p->d.x32;
    u.n = n;
    u.count = count;
    u.seed = p->s.seed;
    if (p->loss == ACDC_LOSS_SVM_DUAL) {
      u.lambda_d = p->lambda * (double)n;
      u.inv_lambda_n_d = 1.0 / (p->lambda * (double)n);
    } else {
      u.lambda_d = p->lambda;
    }
    u.li_scale = 1.0;
    u.n_warps = tau;
    u.loss = p->loss;
    u.fp64 = p->fp64_mode ? 1 : 0;
    u.sm_count = ctx->sm_count;
    ACDC_CK(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    ACDC_CK(ctx, launch_update(u, p->k_next, std::min(wpb_cap, tau), ctx->stream));
    ACDC_CK(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    ACDC_CK(ctx, cudaEventSynchronize(ctx->ev[1]));
    float ms = 0;
    ACDC_CK(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    p->k_next += count;
    p->updates_done += count;
    const double beta =
        n > 1 ? 1.0 + ((double)p->omega - 1.0) * ((double)tau - 1.0) / ((double)n - 1.0) : 1.0;
    const double cost = beta * (double)std::max(ms, 1e-3f) / (double)count;
    if (tau == cand.front() || cost < best_cost) {
      best_cost = cost;
      best = tau;
    }
  }
  ctx->tau_cache[key] = best;
  ctx->tune_probes += (int64_t)cand.size();
  *tau_out = best;
  return ACDC_OK;
}

// Evaluation blocks for one instance: enough to stream its entries and rows.
int eval_blocks_for(const acdc_problem* p) {
  const int64_t work = std::max<int64_t>(p->d.nnz_pad / 16384, std::max(p->d.n, p->d.m) / 4096);
  return (int)std::min<int64_t>(ACDC_RED_BLOCKS, std::max<int64_t>(1, work));
}

double now_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename T>
cudaError_t upload(acdc_ctx* ctx, T** dst, const std::vector<T>& src) {
  cudaError_t e = acdc_dev_alloc(ctx, (void**)dst, sizeof(T) * std::max<size_t>(1, src.size()));
  if (e == cudaSuccess && !src.empty())
    e = cudaMemcpyAsync(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice,
                        ctx->stream);
  return e;
}

struct SolveOpts {
  double gap_target;
  int32_t max_epochs;
  int32_t refresh_every;
  int32_t autotune;
  int32_t tau_override;
  int32_t use_shrinking = 0;
  int32_t active_passes = 20;
};

SolveOpts solve_opts(const acdc_batch_options* opt) {
  SolveOpts o{opt->gap_target, opt->max_epochs, opt->refresh_every, opt->autotune,
              opt->tau_override};
  o.use_shrinking = opt->use_shrinking;
  o.active_passes = opt->active_passes > 0 ? opt->active_passes : 20;
  return o;
}

// Settings of one problem for batched or plain solving: tau from the
// autotuner (or the override), relative gap, q-shrinking for the Lasso when
// asked (from the first epoch on; the batched rounds start each lambda with
// one uniform round).
int prepare(acdc_problem* p, const SolveOpts& o, int wpb_cap) {
  acdc_settings s = p->s;
  s.gap_target = o.gap_target;
  s.gap_relative = 1;
  s.max_epochs = o.max_epochs;
  s.refresh_every = o.refresh_every;
  s.use_shrinking = o.use_shrinking && p->loss == ACDC_LOSS_L1_SQUARE ? 1 : 0;
  s.shrinking_starting_iter = 1;
  s.active_passes = o.active_passes;
  s.tau_active = 0;
  if (o.tau_override > 0) {
    s.tau = o.tau_override;
  } else if (o.autotune == 2) {
    s.tau = autotune_tau(p->d.n, p->omega, 1.3);
  } else if (o.autotune) {
    int tau = 1;
    const int rc = measured_tau(p, wpb_cap, &tau);
    if (rc) return rc;
    s.tau = tau;
  }
  s.warps_per_block = std::min(wpb_cap, s.tau);
  return acdc_problem_set_settings(p, &s);
}

// Rounds of a captured batch launched between two host synchronisations.
constexpr int kRoundsPerSync = 4;

// Device tables and per-slot state of one set of problems solved together.
class BatchEngine {
 public:
  explicit BatchEngine(acdc_ctx* ctx) : ctx_(ctx) {}
  ~BatchEngine() {
    release();
    if (h_live_) {
      cudaStreamSynchronize(ctx_->stream);  // the last copy into h_live_ has landed
      cudaFreeHost(h_live_);
    }
  }

  // Slot i solves problems[i] along lambdas[i*path .. i*path+path-1].
  int build(const std::vector<acdc_problem*>& probs, const std::vector<double>& lambdas, int path,
            const SolveOpts& o, const std::vector<double>* gap_targets = nullptr) {
    release();
    cudaStream_t st = ctx_->stream;
    const int count = (int)probs.size();
    path_ = path;
    count_ = count;
    up_.assign((size_t)count, UpdateParams());
    std::vector<EvalParams> ep((size_t)count);
    std::vector<SlotCtl> ctl((size_t)count);
    std::vector<int32_t> ublk_slot, ublk_first((size_t)count), eblk_slot, eblk_first((size_t)count),
        eblk_count((size_t)count);
    ACDC_CK(ctx_, upload(ctx_, &lambdas_, lambdas));
    const size_t rows = (size_t)count * path * ACDC_BATCH_RESULT_LEN;
    ACDC_CK(ctx_, acdc_dev_alloc(ctx_, (void**)&results_, sizeof(double) * std::max<size_t>(1, rows)));
    ACDC_CK(ctx_, cudaMemsetAsync(results_, 0, sizeof(double) * std::max<size_t>(1, rows), st));
    for (int i = 0; i < count; ++i) {
      acdc_problem* p = probs[(size_t)i];
      int rc = prepare(p, o, 8);
      if (rc) return rc;
      p->lambda = lambdas[(size_t)i * path];
      p->active_valid = false;
      UpdateParams& u = up_[(size_t)i];
      std::memset(&u, 0, sizeof(u));
      u.meta = p->d.meta;
      u.vals = p->d.vals;
      u.idx = p->d.idx;
      u.r = p->d.r32;
      u.active = p->d.active;
      u.counters = p->d.counters;
      u.x64 = p->d.x64;
      u.r64 = p->d.r64;
      u.x32 = p->d.x32;
      u.n = p->d.n;
      u.count = (uint64_t)o.refresh_every * (uint64_t)p->d.n;
      u.seed = p->s.seed;
      if (p->loss == ACDC_LOSS_SVM_DUAL) {
        u.lambda_d = p->lambda * (double)p->d.n;
        u.inv_lambda_n_d = 1.0 / (p->lambda * (double)p->d.n);
      } else {
        u.lambda_d = p->lambda;
      }
      u.li_scale = 1.0;
      u.n_warps = p->s.tau;
      u.loss = p->loss;
      u.fp64 = p->fp64_mode ? 1 : 0;
      u.k_base = p->k_next;
      EvalParams& e = ep[(size_t)i];
      std::memset(&e, 0, sizeof(e));
      e.meta = p->d.meta;
      e.vals = p->d.vals;
      e.idx = p->d.idx;
      e.r32 = p->d.r32;
      e.r64 = p->d.r64;
      e.rhs64 = p->d.rhs64;
      e.active = nullptr;
      e.counters = p->d.counters;
      e.part = p->d.part;
      e.eval_out = p->d.eval_out;
      e.x64 = p->fp64_mode ? p->d.x64 : nullptr;
      e.x32 = p->d.x32;
      e.long_cols = p->d.long_cols;
      e.n_long = p->d.n_long;
      e.m = p->d.m;
      e.n = p->d.n;
      e.lambda = p->lambda;
      e.shrink_thresh = (1.0 - p->s.shrink_eps) * p->lambda;
      e.loss = p->loss;
      const bool shrink = p->s.use_shrinking != 0;
      if (shrink) {
        e.active = p->d.active;
        e.rowcnt = p->d.rowcnt;
      }
      SlotCtl& c = ctl[(size_t)i];
      std::memset(&c, 0, sizeof(c));
      c.live = 1;
      c.shrink = shrink ? 1 : 0;
      c.active_passes = o.active_passes;
      c.q = p->s.shrinking_probability;
      c.q32 = c.q >= 1 ? 0xffffffffu : (uint32_t)(c.q * 4294967296.0);
      c.omega = (double)p->omega;
      c.beta = p->beta;
      c.path_len = path;
      c.max_updates = (uint64_t)o.max_epochs * (uint64_t)p->d.n;
      c.round_updates = u.count;
      c.gap_target = gap_targets ? (*gap_targets)[(size_t)i] : o.gap_target;
      c.polish_rel_gap = p->s.polish_rel_gap;
      c.best_gap = 1e300;
      c.gain_at = 0;
      c.stall_updates = (uint64_t)(p->s.polish_stall_epochs > 0 ? p->s.polish_stall_epochs : 10) *
                        (uint64_t)p->d.n;
      c.lambdas = lambdas_ + (size_t)i * path;
      c.results = results_ + (size_t)i * path * ACDC_BATCH_RESULT_LEN;
      ublk_first[(size_t)i] = (int32_t)ublk_slot.size();
      for (int b = 0; b < (p->s.tau + 7) / 8; ++b) ublk_slot.push_back(i);
      eblk_first[(size_t)i] = (int32_t)eblk_slot.size();
      eblk_count[(size_t)i] = eval_blocks_for(p);
      for (int b = 0; b < eblk_count[(size_t)i]; ++b) eblk_slot.push_back(i);
      ACDC_CK(ctx_, cudaMemsetAsync(p->d.counters + CNT_WORK, 0, sizeof(unsigned long long), st));
    }
    ACDC_CK(ctx_, upload(ctx_, &up_dev_, up_));
    ACDC_CK(ctx_, upload(ctx_, &ep_dev_, ep));
    ACDC_CK(ctx_, upload(ctx_, &ctl_dev_, ctl));
    ACDC_CK(ctx_, upload(ctx_, &ublk_slot_, ublk_slot));
    ACDC_CK(ctx_, upload(ctx_, &ublk_first_, ublk_first));
    ACDC_CK(ctx_, upload(ctx_, &eblk_slot_, eblk_slot));
    ACDC_CK(ctx_, upload(ctx_, &eblk_first_, eblk_first));
    ACDC_CK(ctx_, upload(ctx_, &eblk_count_, eblk_count));
    ACDC_CK(ctx_, upload(ctx_, &live_, std::vector<int32_t>{count}));
    if (!h_live_) ACDC_CK(ctx_, cudaMallocHost((void**)&h_live_, sizeof(int32_t)));
    *h_live_ = count;
    bd_.up = up_dev_;
    bd_.ep = ep_dev_;
    bd_.ctl = ctl_dev_;
    bd_.ublk_slot = ublk_slot_;
    bd_.ublk_first = ublk_first_;
    bd_.eblk_slot = eblk_slot_;
    bd_.eblk_first = eblk_first_;
    bd_.eblk_count = eblk_count_;
    bd_.live_count = live_;
    bd_.n_slots = count;
    ublocks_ = (int)ublk_slot.size();
    eblocks_ = (int)eblk_slot.size();
    ACDC_CK(ctx_, cudaStreamSynchronize(st));
    return ACDC_OK;
  }

  // One round on the stream, ending with the live count copied to the host.
  cudaError_t enqueue_round() {
    cudaStream_t st = ctx_->stream;
    cudaError_t e = launch_batch_update(bd_, ublocks_, st);
    if (e == cudaSuccess) e = launch_batch_eval(bd_, eblocks_, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_live_, live_, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    return e;
  }

  // Replays one captured round until no slot is live or max_rounds is reached.
  int run_graph(int64_t max_rounds) {
    cudaStream_t st = ctx_->stream;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ACDC_CK(ctx_, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = enqueue_round();
    cudaError_t ce2 = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess || ce2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return acdc_cuda_error(ctx_, ce != cudaSuccess ? ce : ce2, "batch graph capture");
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return acdc_cuda_error(ctx_, ce, "cudaGraphInstantiate");
    // A few rounds per host synchronisation: a round whose slots have all
    // finished does no work, and the host reads the live count only to stop.
    for (int64_t r = 0; r < max_rounds && *h_live_ > 0;) {
      for (int k = 0; k < kRoundsPerSync && r < max_rounds && ce == cudaSuccess; ++k, ++r)
        ce = cudaGraphLaunch(exec, st);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
      if (ce != cudaSuccess) break;
    }
    cudaGraphExecDestroy(exec);
    if (ce != cudaSuccess) return acdc_cuda_error(ctx_, ce, "batch round");
    return ACDC_OK;
  }

  // Runs rounds without a graph (the slot set changes between calls).
  int run_rounds(int rounds, int64_t* count = nullptr) {
    int rc = enqueue_rounds(rounds, count);
    if (rc) return rc;
    ACDC_CK(ctx_, cudaStreamSynchronize(ctx_->stream));
    return ACDC_OK;
  }

  // Enqueues the rounds back to back without waiting for them.
  int enqueue_rounds(int rounds, int64_t* count = nullptr) {
    if (*h_live_ <= 0) return ACDC_OK;
    for (int r = 0; r < rounds; ++r) {
      ACDC_CK(ctx_, enqueue_round());
      if (count) ++*count;
    }
    return ACDC_OK;
  }

  int32_t live() const { return h_live_ ? *h_live_ : 0; }

  // Result rows and per-slot control state; also writes the device-side
  // sampler counter and precision back into the problems.
  int collect(const std::vector<acdc_problem*>& probs, std::vector<double>& rows,
              std::vector<SlotCtl>& ctl) {
    cudaStream_t st = ctx_->stream;
    rows.assign((size_t)count_ * path_ * ACDC_BATCH_RESULT_LEN, 0.0);
    ctl.assign((size_t)count_, SlotCtl());
    ACDC_CK(ctx_, cudaMemcpyAsync(rows.data(), results_, sizeof(double) * rows.size(),
                                  cudaMemcpyDeviceToHost, st));
    ACDC_CK(ctx_, cudaMemcpyAsync(ctl.data(), ctl_dev_, sizeof(SlotCtl) * ctl.size(),
                                  cudaMemcpyDeviceToHost, st));
    ACDC_CK(ctx_, cudaMemcpyAsync(up_.data(), up_dev_, sizeof(UpdateParams) * up_.size(),
                                  cudaMemcpyDeviceToHost, st));
    ACDC_CK(ctx_, cudaStreamSynchronize(st));
    for (int i = 0; i < count_; ++i) {
      acdc_problem* p = probs[(size_t)i];
      p->k_next = up_[(size_t)i].k_base;
      p->fp64_mode = up_[(size_t)i].fp64 != 0;
    }
    return ACDC_OK;
  }

  void release() {
    acdc_dev_free(ctx_, up_dev_);
    acdc_dev_free(ctx_, ep_dev_);
    acdc_dev_free(ctx_, ctl_dev_);
    acdc_dev_free(ctx_, ublk_slot_);
    acdc_dev_free(ctx_, ublk_first_);
    acdc_dev_free(ctx_, eblk_slot_);
    acdc_dev_free(ctx_, eblk_first_);
    acdc_dev_free(ctx_, eblk_count_);
    acdc_dev_free(ctx_, live_);
    acdc_dev_free(ctx_, lambdas_);
    acdc_dev_free(ctx_, results_);
    up_dev_ = nullptr;
    ep_dev_ = nullptr;
    ctl_dev_ = nullptr;
    ublk_slot_ = ublk_first_ = eblk_slot_ = eblk_first_ = eblk_count_ = live_ = nullptr;
    lambdas_ = results_ = nullptr;
    count_ = 0;
  }

 private:
  acdc_ctx* ctx_;
  std::vector<UpdateParams> up_;
  UpdateParams* up_dev_ = nullptr;
  EvalParams* ep_dev_ = nullptr;
  SlotCtl* ctl_dev_ = nullptr;
  int32_t *ublk_slot_ = nullptr, *ublk_first_ = nullptr, *eblk_slot_ = nullptr,
          *eblk_first_ = nullptr, *eblk_count_ = nullptr, *live_ = nullptr;
  double *lambdas_ = nullptr, *results_ = nullptr;
  int32_t* h_live_ = nullptr;
  BatchDev bd_{};
  int ublocks_ = 0, eblocks_ = 0, count_ = 0, path_ = 1;
};

void row_to_result(const double* row, acdc_batch_result* out) {
  std::memset(out, 0, sizeof(*out));
  out->eval.primal = row[0];
  out->eval.dual = row[1];
  out->eval.gap = row[2];
  out->eval.rel_gap = row[3];
  out->eval.zero_one_accuracy = row[4];
  out->eval.reg_norm = row[5];
  out->eval.sq_norm = row[6];
  out->eval.max_abs_grad = row[7];
  out->eval.support = (int64_t)row[8];
  out->eval.active = (int64_t)row[9];
  out->lambda = row[10];
  out->converged = row[11] != 0.0;
  out->epochs = (int32_t)row[12];
  out->tau = (int32_t)row[13];
}

int plain_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems, const double* lambdas,
               const acdc_batch_options* opt, acdc_batch_result* results, double* const* x_out) {
  (void)ctx;
  const SolveOpts o = solve_opts(opt);
  for (int32_t i = 0; i < count; ++i) {
    acdc_problem* p = problems[i];
    int rc = prepare(p, o, 8);
    if (rc) return rc;
    for (int32_t k = 0; k < opt->path_len; ++k) {
      const double lam = lambdas[(size_t)i * opt->path_len + k];
      rc = acdc_problem_set_lambda(p, lam);
      if (rc) return rc;
      acdc_solve_result r;
      rc = acdc_solve(p, &r);
      if (rc) return rc;
      acdc_batch_result& out = results[(size_t)i * opt->path_len + k];
      std::memset(&out, 0, sizeof(out));
      out.eval = r.eval;
      out.lambda = lam;
      out.converged = r.converged;
      out.epochs = r.epochs;
      out.tau = p->s.tau;
    }
    if (x_out && x_out[i]) {
      rc = acdc_get_x(p, x_out[i]);
      if (rc) return rc;
    }
  }
  return ACDC_OK;
}

int batched_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems,
                 const double* lambdas, const acdc_batch_options* opt,
                 acdc_batch_result* results, double* const* x_out) {
  const int path = opt->path_len;
  const SolveOpts o = solve_opts(opt);
  std::vector<acdc_problem*> probs(problems, problems + count);
  BatchEngine eng(ctx);
  int rc = eng.build(probs, std::vector<double>(lambdas, lambdas + (size_t)count * path), path, o);
  if (rc) return rc;
  // Each slot advances refresh_every epochs per round and spends at most
  // max_epochs per lambda.
  // (a shrinking round is at least a quarter epoch).
  const int64_t rounds_per_lambda =
      o.use_shrinking ? 4 * (int64_t)opt->max_epochs
                      : (opt->max_epochs + opt->refresh_every - 1) / opt->refresh_every;
  const int64_t max_rounds = (int64_t)path * rounds_per_lambda + path + 1;
  rc = eng.run_graph(max_rounds);
  if (rc) return rc;
  std::vector<double> rows;
  std::vector<SlotCtl> ctl;
  rc = eng.collect(probs, rows, ctl);
  if (rc) return rc;
  for (int32_t i = 0; i < count; ++i) {
    problems[i]->lambda = lambdas[(size_t)i * path + path - 1];
    for (int k = 0; k < path; ++k)
      row_to_result(rows.data() + ((size_t)i * path + k) * ACDC_BATCH_RESULT_LEN,
                    &results[(size_t)i * path + k]);
    if (x_out && x_out[i]) {
      rc = acdc_get_x(problems[i], x_out[i]);
      if (rc) return rc;
    }
  }
  return ACDC_OK;
}
}  // namespace

extern "C" int acdc_batch_solve_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems,
                                     const double* lambdas, const acdc_batch_options* opt,
                                     acdc_batch_result* results, double* const* x_out) {
  if (!ctx || count < 0 || (count > 0 && (!problems || !lambdas || !results)) || !opt ||
      opt->path_len < 1 || opt->refresh_every < 1 || opt->max_epochs < 1 ||
      !(opt->gap_target >= 0))
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid batch arguments");
  for (int32_t i = 0; i < count; ++i) {
    if (!problems[i] || problems[i]->ctx != ctx)
      return acdc_set_error(ctx, ACDC_EINVAL, "problem missing or from another context");
    if (problems[i]->loss != ACDC_LOSS_L1_SQUARE && problems[i]->loss != ACDC_LOSS_SVM_DUAL)
      return acdc_set_error(ctx, ACDC_EUNSUPPORTED, "batched paths cover losses 0 and 2");
  }
  for (int64_t i = 0; i < (int64_t)count * opt->path_len; ++i)
    if (!positive_finite(lambdas[i]))
      return acdc_set_error(ctx, ACDC_EINVAL, "lambdas must be positive and finite");
  if (count == 0) return ACDC_OK;
  ACDC_CK(ctx, cudaSetDevice(ctx->device));
  NvtxRange range(opt->plain ? "acdc_batch_plain" : "acdc_batch_solve_path");
  if (opt->plain) return plain_path(ctx, count, problems, lambdas, opt, results, x_out);
  return batched_path(ctx, count, problems, lambdas, opt, results, x_out);
}

// ---- serving ----

namespace {
struct Request {
  int64_t ticket = 0;
  int32_t loss = 0;
  int64_t m = 0, n = 0;
  std::vector<int64_t> col_ptr;
  std::vector<int32_t> row_idx;
  std::vector<double> vals, rhs;
  double lambda = 0, gap_target = 1e-6;
  uint64_t seed = 0;
  int64_t footprint = 0;
  acdc_problem* prob = nullptr;
  acdc_request_result res{};
  std::vector<double> x;
};

// Device bytes a request holds while resident, including its upload staging.
int64_t footprint_of(int64_t m, int64_t n, int64_t nnz) {
  const int64_t nnz_pad = nnz + 3 * n;
  return 8 * nnz_pad + 12 * nnz + 112 * n + 32 * m + (1 << 20);
}
}  // namespace

struct acdc_server;
namespace {
void admit_one(acdc_server* s, Request* r, const int64_t* col_ptr, const int32_t* row_idx,
               const double* vals, const double* rhs);
}  // namespace

struct acdc_server {
  acdc_ctx* ctx = nullptr;
  acdc_server_options opt{};
  int64_t next_ticket = 1;
  int64_t used_bytes = 0;
  std::deque<Request*> queue;               // submitted, not yet admitted
  std::vector<Request*> resident;           // on the device
  std::map<int64_t, std::unique_ptr<Request>> all;
  BatchEngine* engine = nullptr;
  bool dirty = true;                        // resident set changed since the last build
  bool in_flight = false;                   // rounds enqueued by the last step, not yet waited for
  std::vector<Request*> built;              // the requests of the engine's slots, in slot order
  acdc_server_stats stats{};
};

namespace {
// Makes the context's admission stream the one its calls use for the scope:
// problems created inside are uploaded, laid out and checked on it, so their
// work and their synchronisations do not wait for the rounds on the main
// stream.
struct AdmitStream {
  acdc_ctx* ctx;
  cudaStream_t main;
  explicit AdmitStream(acdc_ctx* c) : ctx(c), main(c->stream) { ctx->stream = ctx->admit_stream; }
  ~AdmitStream() { ctx->stream = main; }
  AdmitStream(const AdmitStream&) = delete;
  AdmitStream& operator=(const AdmitStream&) = delete;
};

// Waits for the rounds the last step enqueued.
int finish_rounds(acdc_server* s) {
  if (!s->in_flight) return ACDC_OK;
  const double t0 = now_seconds();
  ACDC_CK(s->ctx, cudaStreamSynchronize(s->ctx->stream));
  s->in_flight = false;
  s->stats.rounds_s += now_seconds() - t0;
  return ACDC_OK;
}
}  // namespace

extern "C" int acdc_server_create(acdc_ctx* ctx, const acdc_server_options* opt, acdc_server** out) {
  if (!ctx || !opt || !out) return ACDC_EINVAL;
  if (opt->memory_budget_bytes <= 0 || opt->max_slots < 1 || opt->quantum_epochs < 1 ||
      opt->max_epochs < 1)
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid server options");
  if (!ctx->admit_stream) {
    ACDC_CK(ctx, cudaSetDevice(ctx->device));
    ACDC_CK(ctx, cudaStreamCreateWithFlags(&ctx->admit_stream, cudaStreamNonBlocking));
  }
  acdc_server* s = new acdc_server();
  s->ctx = ctx;
  s->opt = *opt;
  s->engine = new BatchEngine(ctx);
  ctx->live_problems++;
  *out = s;
  return ACDC_OK;
}

extern "C" int acdc_server_submit(acdc_server* s, const acdc_request* req, int64_t* ticket) {
  if (!s || !req || !ticket) return ACDC_EINVAL;
  acdc_ctx* ctx = s->ctx;
  if ((req->loss != ACDC_LOSS_L1_SQUARE && req->loss != ACDC_LOSS_SVM_DUAL) || req->m <= 0 ||
      req->n <= 0 || !req->col_ptr || !req->rhs || !positive_finite(req->lambda) ||
      !(req->gap_target >= 0))
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid request");
  const int64_t nnz = req->col_ptr[req->n];
  if (req->col_ptr[0] != 0 || nnz < 0 || (nnz > 0 && (!req->row_idx || !req->vals)))
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid request matrix");
  const int64_t fp = footprint_of(req->m, req->n, nnz);
  if (fp > s->opt.memory_budget_bytes)
    return acdc_set_error(ctx, ACDC_EBUSY, "request larger than the memory budget");
  auto r = std::make_unique<Request>();
  r->ticket = s->next_ticket++;
  r->loss = req->loss;
  r->m = req->m;
  r->n = req->n;
  r->lambda = req->lambda;
  r->gap_target = req->gap_target;
  r->seed = req->seed;
  r->footprint = fp;
  r->res.state = 0;
  r->res.submit_time = now_seconds();
  *ticket = r->ticket;
  Request* rp = r.get();
  s->all[r->ticket] = std::move(r);
  // Admitted at once when nothing waits ahead of it and a slot and the memory
  // are free: the device copy is made from the caller's arrays.  Otherwise the
  // request is copied (the caller's arrays are only read during this call) and
  // waits in arrival order.
  if (s->queue.empty() && (int32_t)s->resident.size() < s->opt.max_slots &&
      s->used_bytes + fp <= s->opt.memory_budget_bytes) {
    admit_one(s, rp, req->col_ptr, req->row_idx, req->vals, req->rhs);
    return ACDC_OK;
  }
  rp->col_ptr.assign(req->col_ptr, req->col_ptr + req->n + 1);
  rp->row_idx.assign(req->row_idx, req->row_idx + nnz);
  rp->vals.assign(req->vals, req->vals + nnz);
  const int64_t rhs_len = req->loss == ACDC_LOSS_L1_SQUARE ? req->m : req->n;
  rp->rhs.assign(req->rhs, req->rhs + rhs_len);
  s->queue.push_back(rp);
  return ACDC_OK;
}

namespace {
// Retires the requests of the engine's slots whose lambda is done: records the
// result, reads x back and frees the device buffers.  Only the slots of the
// last build are looked at (requests admitted since then have no slot yet);
// every slot's sampler counter and precision go back into its problem.
int retire_finished(acdc_server* s) {
  if (s->built.empty()) return ACDC_OK;
  std::vector<acdc_problem*> probs;
  for (Request* r : s->built) probs.push_back(r->prob);
  std::vector<double> rows;
  std::vector<SlotCtl> ctl;
  int rc = s->engine->collect(probs, rows, ctl);
  if (rc) return rc;
  std::vector<Request*> gone;
  for (size_t i = 0; i < s->built.size(); ++i) {
    Request* r = s->built[i];
    if (ctl[i].live) continue;
    acdc_batch_result br;
    row_to_result(rows.data() + i * ACDC_BATCH_RESULT_LEN, &br);
    r->res.eval = br.eval;
    r->res.converged = br.converged;
    r->res.epochs = br.epochs;
    r->res.status = ACDC_OK;
    r->x.assign((size_t)r->n, 0.0);
    rc = acdc_get_x(r->prob, r->x.data());
    if (rc) r->res.status = rc;
    acdc_problem_destroy(r->prob);
    r->prob = nullptr;
    s->used_bytes -= r->footprint;
    r->res.finish_time = now_seconds();
    r->res.state = r->res.status == ACDC_OK ? 2 : 3;
    gone.push_back(r);
    s->stats.retired++;
  }
  if (!gone.empty()) {
    std::vector<Request*> keep;
    for (Request* r : s->resident)
      if (std::find(gone.begin(), gone.end(), r) == gone.end()) keep.push_back(r);
    s->resident.swap(keep);
    s->built.clear();  // the tables list retired slots: rebuilt before the next round
    s->dirty = true;
  }
  return ACDC_OK;
}

// Creates the device problem of request r from the given arrays and makes it
// resident (or records the failure).
void admit_one(acdc_server* s, Request* r, const int64_t* col_ptr, const int32_t* row_idx,
               const double* vals, const double* rhs) {
  const double t0 = now_seconds();
  acdc_problem* p = nullptr;
  int rc;
  {
    AdmitStream on(s->ctx);
    rc = acdc_problem_create(s->ctx, r->loss, r->m, r->n, col_ptr, row_idx, vals, rhs, r->lambda,
                             &p);
  }
  r->res.start_time = now_seconds();
  s->stats.admit_s += r->res.start_time - t0;
  if (rc != ACDC_OK) {
    r->res.state = 3;
    r->res.status = rc;
    r->res.finish_time = r->res.start_time;
    return;
  }
  p->s.seed = r->seed;
  r->prob = p;
  r->res.state = 1;
  s->used_bytes += r->footprint;
  s->resident.push_back(r);
  s->dirty = true;
  s->stats.admitted++;
}

// Admits queued requests in arrival order while slots and memory allow.
void admit(acdc_server* s) {
  while (!s->queue.empty() && (int32_t)s->resident.size() < s->opt.max_slots) {
    Request* r = s->queue.front();
    if (s->used_bytes + r->footprint > s->opt.memory_budget_bytes) break;
    s->queue.pop_front();
    admit_one(s, r, r->col_ptr.data(), r->row_idx.empty() ? nullptr : r->row_idx.data(),
              r->vals.empty() ? nullptr : r->vals.data(), r->rhs.data());
    // the host copy is no longer needed
    std::vector<int64_t>().swap(r->col_ptr);
    std::vector<int32_t>().swap(r->row_idx);
    std::vector<double>().swap(r->vals);
    std::vector<double>().swap(r->rhs);
  }
}
}  // namespace

// A step is pipelined: it waits for the rounds the previous step enqueued,
// retires the requests that finished, rebuilds the slot tables if the resident
// set changed, enqueues this step's rounds and returns without waiting for
// them, after admitting queued requests on the admission stream while those
// rounds run (they join the next step's tables).
extern "C" int acdc_server_step(acdc_server* s, int32_t* pending) {
  if (!s) return ACDC_EINVAL;
  acdc_ctx* ctx = s->ctx;
  ACDC_CK(ctx, cudaSetDevice(ctx->device));
  NvtxRange range("acdc_server_step");
  int rc = finish_rounds(s);
  if (rc) return rc;
  {
    const double t1 = now_seconds();
    rc = retire_finished(s);
    if (rc) return rc;
    s->stats.retire_s += now_seconds() - t1;
  }
  if (s->resident.empty()) admit(s);  // nothing to overlap with: admit first
  if (!s->resident.empty()) {
    if (s->dirty) {
      // Rebuild the slot tables over the resident set: running slots keep their
      // x, residual and sampler state; new ones start from x = 0.
      std::vector<acdc_problem*> probs;
      std::vector<double> lams, targets;
      SolveOpts o{1e-6, s->opt.max_epochs, 1, 1, 0};
      o.use_shrinking = s->opt.use_shrinking;
      for (Request* r : s->resident) {
        probs.push_back(r->prob);
        lams.push_back(r->lambda);
        targets.push_back(r->gap_target);
      }
      const double t0 = now_seconds();
      rc = s->engine->build(probs, lams, 1, o, &targets);
      if (rc) return rc;
      s->built = s->resident;
      s->dirty = false;
      s->stats.builds++;
      s->stats.build_s += now_seconds() - t0;
    }
    rc = s->engine->enqueue_rounds(s->opt.quantum_epochs, &s->stats.rounds);
    if (rc) return rc;
    s->in_flight = true;
  }
  admit(s);
  s->stats.steps++;
  if (pending) *pending = (int32_t)(s->queue.size() + s->resident.size());
  return ACDC_OK;
}

extern "C" int acdc_server_get_stats(acdc_server* s, acdc_server_stats* out) {
  if (!s || !out) return ACDC_EINVAL;
  *out = s->stats;
  return ACDC_OK;
}

extern "C" int acdc_server_poll(acdc_server* s, int64_t ticket, acdc_request_result* res, double* x) {
  if (!s || !res) return ACDC_EINVAL;
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return ACDC_ENOTFOUND;
  Request* r = it->second.get();
  *res = r->res;
  if (x && r->res.state == 2) std::memcpy(x, r->x.data(), sizeof(double) * r->x.size());
  return ACDC_OK;
}

extern "C" int acdc_server_release(acdc_server* s, int64_t ticket) {
  if (!s) return ACDC_EINVAL;
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return ACDC_ENOTFOUND;
  if (it->second->res.state < 2) return acdc_set_error(s->ctx, ACDC_EBUSY, "request still pending");
  s->all.erase(it);
  return ACDC_OK;
}

extern "C" int acdc_server_cancel(acdc_server* s, int64_t ticket) {
  if (!s) return ACDC_EINVAL;
  auto it = s->all.find(ticket);
  if (it == s->all.end()) return ACDC_ENOTFOUND;
  Request* r = it->second.get();
  if (r->res.state >= 2) return ACDC_OK;
  // no round may be in flight while a resident problem goes away, and the
  // finished slots are retired before the tables are dropped
  int rc = finish_rounds(s);
  if (rc == ACDC_OK) rc = retire_finished(s);
  if (rc) return rc;
  if (r->res.state >= 2) return ACDC_OK;
  if (r->res.state == 0) {
    for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
      if (*q == r) {
        s->queue.erase(q);
        break;
      }
  } else {
    // Running: no round is in flight between steps.  The engine's tables still
    // point at the problem, so they are rebuilt before the next round.
    for (auto q = s->resident.begin(); q != s->resident.end(); ++q)
      if (*q == r) {
        s->resident.erase(q);
        break;
      }
    if (r->prob) acdc_problem_destroy(r->prob);
    r->prob = nullptr;
    s->used_bytes -= r->footprint;
    s->built.clear();
    s->dirty = true;
  }
  r->res.state = 3;
  r->res.status = ACDC_ECANCELED;
  r->res.finish_time = now_seconds();
  return ACDC_OK;
}

extern "C" int acdc_server_destroy(acdc_server* s) {
  if (!s) return ACDC_EINVAL;
  finish_rounds(s);
  if (s->ctx->admit_stream) cudaStreamSynchronize(s->ctx->admit_stream);
  for (Request* r : s->resident)
    if (r->prob) acdc_problem_destroy(r->prob);
  delete s->engine;
  s->ctx->live_problems--;
  delete s;
  return ACDC_OK;
}
