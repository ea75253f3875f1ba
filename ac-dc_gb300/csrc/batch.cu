// Batched lambda paths (many instances per launch) and the serving loop.
//
// The lambda path with warm starts follows
// cpp/src/experiments/lasso_console_solver.cpp:149-172 (a geometric sequence of
// lambdas, x carried from one lambda to the next), run here for many instances
// at once.  One round is: the update kernel over every live slot, the FP64
// refresh and gap kernels over every live slot, and a control kernel with one
// block per slot that records converged lambdas and advances the path.  The
// round is captured once in a CUDA graph and replayed until every slot is done.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "acdc_internal.cuh"

namespace {

// ESO-aware choice of tau for one instance: the largest power of two whose
// beta = 1 + (omega-1)(tau-1)/(n-1) stays at most beta_max, with at least 32
// columns per concurrent update and no more than 1024 warps.
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

// Evaluation blocks for one instance: enough to stream its entries and rows.
int eval_blocks_for(const acdc_problem* p) {
  const int64_t work = std::max<int64_t>(p->d.nnz_pad / 16384, std::max(p->d.n, p->d.m) / 4096);
  return (int)std::min<int64_t>(ACDC_RED_BLOCKS, std::max<int64_t>(1, work));
}

int plain_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems, const double* lambdas,
               const acdc_batch_options* opt, acdc_batch_result* results, double* const* x_out) {
  for (int32_t i = 0; i < count; ++i) {
    acdc_problem* p = problems[i];
    acdc_settings s = p->s;
    s.gap_target = opt->gap_target;
    s.gap_relative = 1;
    s.max_epochs = opt->max_epochs;
    s.refresh_every = opt->refresh_every;
    s.use_shrinking = 0;
    if (opt->tau_override > 0)
      s.tau = opt->tau_override;
    else if (opt->autotune)
      s.tau = autotune_tau(p->d.n, p->omega, 1.3);
    s.warps_per_block = std::min(8, s.tau);
    int rc = acdc_problem_set_settings(p, &s);
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
      out.tau = s.tau;
    }
    if (x_out && x_out[i]) {
      rc = acdc_get_x(p, x_out[i]);
      if (rc) return rc;
    }
  }
  return ACDC_OK;
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src, cudaStream_t st) {
  cudaError_t e = cudaMalloc((void**)dst, sizeof(T) * std::max<size_t>(1, src.size()));
  if (e == cudaSuccess && !src.empty())
    e = cudaMemcpyAsync(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, st);
  return e;
}

struct BatchBuffers {
  UpdateParams* up = nullptr;
  EvalParams* ep = nullptr;
  SlotCtl* ctl = nullptr;
  int32_t* ublk_slot = nullptr;
  int32_t* ublk_first = nullptr;
  int32_t* eblk_slot = nullptr;
  int32_t* eblk_first = nullptr;
  int32_t* eblk_count = nullptr;
  int32_t* live = nullptr;
  double* lambdas = nullptr;
  double* results = nullptr;
  int32_t* h_live = nullptr;
  ~BatchBuffers() {
    cudaFree(up);
    cudaFree(ep);
    cudaFree(ctl);
    cudaFree(ublk_slot);
    cudaFree(ublk_first);
    cudaFree(eblk_slot);
    cudaFree(eblk_first);
    cudaFree(eblk_count);
    cudaFree(live);
    cudaFree(lambdas);
    cudaFree(results);
    if (h_live) cudaFreeHost(h_live);
  }
};

int batched_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems,
                 const double* lambdas, const acdc_batch_options* opt,
                 acdc_batch_result* results, double* const* x_out) {
  cudaStream_t st = ctx->stream;
  const int path = opt->path_len;
  std::vector<UpdateParams> up((size_t)count);
  std::vector<EvalParams> ep((size_t)count);
  std::vector<SlotCtl> ctl((size_t)count);
  std::vector<int32_t> ublk_slot, ublk_first((size_t)count), eblk_slot, eblk_first((size_t)count),
      eblk_count((size_t)count);
  BatchBuffers bb;
  ACDC_CK(ctx, upload(&bb.lambdas, std::vector<double>(lambdas, lambdas + (size_t)count * path), st));
  ACDC_CK(ctx, cudaMalloc((void**)&bb.results,
                          sizeof(double) * (size_t)count * path * ACDC_BATCH_RESULT_LEN));
  ACDC_CK(ctx, cudaMemsetAsync(bb.results, 0,
                               sizeof(double) * (size_t)count * path * ACDC_BATCH_RESULT_LEN, st));
  for (int32_t i = 0; i < count; ++i) {
    acdc_problem* p = problems[i];
    // Settings: tau per instance from the autotuner (or the override), no shrinking.
    acdc_settings s = p->s;
    s.gap_target = opt->gap_target;
    s.gap_relative = 1;
    s.max_epochs = opt->max_epochs;
    s.refresh_every = opt->refresh_every;
    s.use_shrinking = 0;
    s.tau = opt->tau_override > 0 ? opt->tau_override
                                  : (opt->autotune ? autotune_tau(p->d.n, p->omega, 1.3) : s.tau);
    s.warps_per_block = 8;
    int rc = acdc_problem_set_settings(p, &s);
    if (rc) return rc;
    p->lambda = lambdas[(size_t)i * path];
    p->active_valid = false;
    // The slot's parameters (the control kernel keeps them current on the device).
    UpdateParams u;
    std::memset(&u, 0, sizeof(u));
    u.meta = p->d.meta;
    u.vals = p->d.vals;
    u.idx = p->d.idx;
    u.r = p->d.r32;
    u.active = p->d.active;
    u.counters = p->d.counters;
    u.x64 = p->d.x64;
    u.r64 = p->d.r64;
    u.n = p->d.n;
    u.count = (uint64_t)opt->refresh_every * (uint64_t)p->d.n;
    u.seed = p->s.seed;
    if (p->loss == ACDC_LOSS_SVM_DUAL) {
      u.lambda_d = p->lambda * (double)p->d.n;
      u.inv_lambda_n_d = 1.0 / (p->lambda * (double)p->d.n);
    } else {
      u.lambda_d = p->lambda;
    }
    u.li_scale = 1.0;
    u.n_warps = s.tau;
    u.loss = p->loss;
    u.fp64 = p->fp64_mode ? 1 : 0;
    u.k_base = p->k_next;
    up[(size_t)i] = u;
    EvalParams e;
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
    e.long_cols = p->d.long_cols;
    e.n_long = p->d.n_long;
    e.m = p->d.m;
    e.n = p->d.n;
    e.lambda = p->lambda;
    e.shrink_thresh = 0.9 * p->lambda;
    e.loss = p->loss;
    ep[(size_t)i] = e;
    SlotCtl c;
    std::memset(&c, 0, sizeof(c));
    c.live = 1;
    c.k = 0;
    c.path_len = path;
    c.max_updates = (uint64_t)opt->max_epochs * (uint64_t)p->d.n;
    c.round_updates = u.count;
    c.gap_target = opt->gap_target;
    c.polish_rel_gap = p->s.polish_rel_gap;
    c.lambdas = bb.lambdas + (size_t)i * path;
    c.results = bb.results + (size_t)i * path * ACDC_BATCH_RESULT_LEN;
    ctl[(size_t)i] = c;
    // Blocks: tau/8 update blocks and a size-proportional share of evaluation blocks.
    ublk_first[(size_t)i] = (int32_t)ublk_slot.size();
    for (int b = 0; b < (s.tau + 7) / 8; ++b) ublk_slot.push_back(i);
    eblk_first[(size_t)i] = (int32_t)eblk_slot.size();
    eblk_count[(size_t)i] = eval_blocks_for(p);
    for (int b = 0; b < eblk_count[(size_t)i]; ++b) eblk_slot.push_back(i);
    ACDC_CK(ctx, cudaMemsetAsync(p->d.counters + CNT_WORK, 0, sizeof(unsigned long long), st));
  }
  ACDC_CK(ctx, upload(&bb.up, up, st));
  ACDC_CK(ctx, upload(&bb.ep, ep, st));
  ACDC_CK(ctx, upload(&bb.ctl, ctl, st));
  ACDC_CK(ctx, upload(&bb.ublk_slot, ublk_slot, st));
  ACDC_CK(ctx, upload(&bb.ublk_first, ublk_first, st));
  ACDC_CK(ctx, upload(&bb.eblk_slot, eblk_slot, st));
  ACDC_CK(ctx, upload(&bb.eblk_first, eblk_first, st));
  ACDC_CK(ctx, upload(&bb.eblk_count, eblk_count, st));
  ACDC_CK(ctx, upload(&bb.live, std::vector<int32_t>{count}, st));
  ACDC_CK(ctx, cudaMallocHost((void**)&bb.h_live, sizeof(int32_t)));
  BatchDev bd;
  bd.up = bb.up;
  bd.ep = bb.ep;
  bd.ctl = bb.ctl;
  bd.ublk_slot = bb.ublk_slot;
  bd.ublk_first = bb.ublk_first;
  bd.eblk_slot = bb.eblk_slot;
  bd.eblk_first = bb.eblk_first;
  bd.eblk_count = bb.eblk_count;
  bd.live_count = bb.live;
  bd.n_slots = count;
  const int ublocks = (int)ublk_slot.size();
  const int eblocks = (int)eblk_slot.size();

  // Refresh every slot's residual for its first lambda, then capture one round.
  ACDC_CK(ctx, cudaStreamSynchronize(st));
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ACDC_CK(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  cudaError_t ce = launch_batch_update(bd, ublocks, st);
  if (ce == cudaSuccess) ce = launch_batch_eval(bd, eblocks, st);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(bb.h_live, bb.live, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  cudaError_t ce2 = cudaStreamEndCapture(st, &graph);
  if (ce != cudaSuccess || ce2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return acdc_cuda_error(ctx, ce != cudaSuccess ? ce : ce2, "batch graph capture");
  }
  ce = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return acdc_cuda_error(ctx, ce, "cudaGraphInstantiate");
  // Rounds: each slot advances refresh_every epochs per round; a slot can take
  // at most path_len * ceil(max_epochs / refresh_every) rounds.
  const int64_t max_rounds =
      (int64_t)path * ((opt->max_epochs + opt->refresh_every - 1) / opt->refresh_every) + path + 1;
  int rc = ACDC_OK;
  *bb.h_live = count;
  for (int64_t round = 0; round < max_rounds && *bb.h_live > 0; ++round) {
    ce = cudaGraphLaunch(exec, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) {
      rc = acdc_cuda_error(ctx, ce, "batch round");
      break;
    }
  }
  cudaGraphExecDestroy(exec);
  if (rc != ACDC_OK) return rc;
  // Results and the per-problem host state.
  std::vector<double> rows((size_t)count * path * ACDC_BATCH_RESULT_LEN);
  ACDC_CK(ctx, cudaMemcpyAsync(rows.data(), bb.results, sizeof(double) * rows.size(),
                               cudaMemcpyDeviceToHost, st));
  ACDC_CK(ctx, cudaMemcpyAsync(up.data(), bb.up, sizeof(UpdateParams) * up.size(),
                               cudaMemcpyDeviceToHost, st));
  ACDC_CK(ctx, cudaStreamSynchronize(st));
  for (int32_t i = 0; i < count; ++i) {
    acdc_problem* p = problems[i];
    p->k_next = up[(size_t)i].k_base;
    p->fp64_mode = up[(size_t)i].fp64 != 0;
    p->lambda = lambdas[(size_t)i * path + path - 1];
    for (int k = 0; k < path; ++k) {
      const double* row = rows.data() + ((size_t)i * path + k) * ACDC_BATCH_RESULT_LEN;
      acdc_batch_result& out = results[(size_t)i * path + k];
      std::memset(&out, 0, sizeof(out));
      out.eval.primal = row[0];
      out.eval.dual = row[1];
      out.eval.gap = row[2];
      out.eval.rel_gap = row[3];
      out.eval.zero_one_accuracy = row[4];
      out.eval.reg_norm = row[5];
      out.eval.sq_norm = row[6];
      out.eval.max_abs_grad = row[7];
      out.eval.support = (int64_t)row[8];
      out.eval.active = (int64_t)row[9];
      out.lambda = row[10];
      out.converged = row[11] != 0.0;
      out.epochs = (int32_t)row[12];
      out.tau = (int32_t)row[13];
    }
    if (x_out && x_out[i]) {
      rc = acdc_get_x(p, x_out[i]);
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
  for (int32_t i = 0; i < count; ++i)
    if (!problems[i] || problems[i]->ctx != ctx)
      return acdc_set_error(ctx, ACDC_EINVAL, "problem missing or from another context");
  for (int64_t i = 0; i < (int64_t)count * opt->path_len; ++i)
    if (!(lambdas[i] > 0)) return acdc_set_error(ctx, ACDC_EINVAL, "lambdas must be positive");
  if (count == 0) return ACDC_OK;
  ACDC_CK(ctx, cudaSetDevice(ctx->device));
  if (opt->plain) return plain_path(ctx, count, problems, lambdas, opt, results, x_out);
  return batched_path(ctx, count, problems, lambdas, opt, results, x_out);
}

struct acdc_server {
  acdc_ctx* ctx;
};

extern "C" int acdc_server_create(acdc_ctx* ctx, const acdc_server_options* opt, acdc_server** out) {
  (void)opt;
  if (!ctx || !out) return ACDC_EINVAL;
  return acdc_set_error(ctx, ACDC_EUNSUPPORTED, "server not built yet");
}
extern "C" int acdc_server_submit(acdc_server* s, const acdc_request* req, int64_t* ticket) {
  (void)s; (void)req; (void)ticket;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_step(acdc_server* s, int32_t* pending) {
  (void)s; (void)pending;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_poll(acdc_server* s, int64_t ticket, acdc_request_result* res, double* x) {
  (void)s; (void)ticket; (void)res; (void)x;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_release(acdc_server* s, int64_t ticket) {
  (void)s; (void)ticket;
  return ACDC_EUNSUPPORTED;
}
extern "C" int acdc_server_destroy(acdc_server* s) {
  (void)s;
  return ACDC_EUNSUPPORTED;
}
