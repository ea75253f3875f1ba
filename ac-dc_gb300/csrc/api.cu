// C-ABI of libacdc_gpu.so: contexts, problem upload, the engine calls and the
// solve loop.  See include/acdc_gpu.h for the contract of every entry point.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "acdc_internal.cuh"

// ---- errors ----

int acdc_set_error(acdc_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int acdc_cuda_error(acdc_ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return acdc_set_error(ctx, ACDC_ENOMEM, m);
  return acdc_set_error(ctx, ACDC_ECUDA, m);
}

extern "C" const char* acdc_last_error(const acdc_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" const char* acdc_status_string(int status) {
  switch (status) {
    case ACDC_OK: return "ok";
    case ACDC_EINVAL: return "invalid argument";
    case ACDC_ENOMEM: return "out of memory";
    case ACDC_EUNSUPPORTED: return "unsupported loss";
    case ACDC_ECUDA: return "CUDA error";
    case ACDC_ETIMEOUT: return "device wait timed out";
    case ACDC_EDEVICE: return "device reported a bad index or state";
    case ACDC_EBUSY: return "admission refused";
    case ACDC_ENOTFOUND: return "unknown ticket";
    case ACDC_ENODEV: return "no CUDA device";
    case ACDC_ECANCELED: return "request cancelled";
    default: return "unknown status";
  }
}

extern "C" void acdc_settings_default(acdc_settings* s) {
  if (!s) return;
  std::memset(s, 0, sizeof(*s));
  s->loss = ACDC_LOSS_L1_SQUARE;
  s->tau = 4096;
  s->warps_per_block = 8;
  s->refresh_every = 5;
  s->seed = 0;
  s->sigma = 0;
  s->gap_target = 1e-6;
  s->gap_relative = 1;
  s->max_epochs = 1000;
  s->use_shrinking = 0;
  s->shrinking_starting_iter = 2;
  s->shrinking_probability = 0.9;
  s->shrink_eps = 0.1;
  s->precision = ACDC_PREC_AUTO;
  s->polish_rel_gap = 1e-5;
  s->screened_eval = 1;
  s->hot_threshold = 0.1;
  s->hot_polish_sweeps = 16;
  s->polish_active_passes = 2;
}

const char* settings_fault(const acdc_settings* s) {
  if (s->loss < ACDC_LOSS_L1_SQUARE || s->loss > ACDC_LOSS_LOGISTIC) return "loss";
  if (s->tau < 1) return "tau";
  if (s->tau_active < 0) return "tau_active";
  if (s->warps_per_block < 1 || s->warps_per_block > 8) return "warps_per_block";
  if (s->refresh_every < 1) return "refresh_every";
  if (s->max_epochs < 0) return "max_epochs";
  // sigma <= 0 asks for the computed beta; NaN and infinities are no beta.
  if (!(std::fabs(s->sigma) <= 1.7976931348623157e308)) return "sigma";
  // finite and non-negative: +inf would end every solve at its first evaluation
  if (!(std::isfinite(s->gap_target) && s->gap_target >= 0)) return "gap_target";
  if (!(s->shrinking_probability >= 0 && s->shrinking_probability <= 1))
    return "shrinking_probability";
  if (!(s->shrink_eps >= 0 && s->shrink_eps < 1)) return "shrink_eps";
  if (s->precision < ACDC_PREC_AUTO || s->precision > ACDC_PREC_FP64) return "precision";
  if (!(std::isfinite(s->polish_rel_gap) && s->polish_rel_gap >= 0)) return "polish_rel_gap";
  if (!(std::isfinite(s->hot_threshold) && s->hot_threshold >= 0)) return "hot_threshold";
  if (s->polish_stall_epochs < 0) return "polish_stall_epochs";
  if (s->hot_polish_sweeps < 0) return "hot_polish_sweeps";
  if (s->polish_active_passes < 0) return "polish_active_passes";
  if (s->lanes_per_update != 0 && s->lanes_per_update != -1 && s->lanes_per_update != 1 &&
      s->lanes_per_update != 8 && s->lanes_per_update != 16 && s->lanes_per_update != 32)
    return "lanes_per_update";
  if (s->minibatch != 0 && (s->minibatch != 1 || s->loss != ACDC_LOSS_SVM_DUAL)) return "minibatch";
  return nullptr;
}

extern "C" int acdc_settings_check(const acdc_settings* s) {
  if (!s) return ACDC_EINVAL;
  return settings_fault(s) ? ACDC_EINVAL : ACDC_OK;
}

// ---- context ----

extern "C" int acdc_ctx_create(int device, acdc_ctx** out) {
  if (!out) return ACDC_EINVAL;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return ACDC_ENODEV;
  if (device < 0 || device >= count) return ACDC_EINVAL;
  acdc_ctx* ctx = new acdc_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    e = cudaMemPoolCreate(&ctx->pool, &props);
  }
  if (e == cudaSuccess) {
    // keep freed blocks in the pool until the context goes away
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->ev[i]);
  if (e == cudaSuccess) e = update_kernels_init();
  if (e != cudaSuccess) {
    for (int i = 0; i < 6; ++i)
      if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    delete ctx;
    return e == cudaErrorMemoryAllocation ? ACDC_ENOMEM : ACDC_ECUDA;
  }
  *out = ctx;
  return ACDC_OK;
}

extern "C" int acdc_ctx_destroy(acdc_ctx* ctx) {
  if (!ctx) return ACDC_EINVAL;
  if (ctx->live_problems > 0)
    return acdc_set_error(ctx, ACDC_EBUSY, "destroy every problem of the context first");
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);  // frees in flight complete
  if (ctx->admit_stream) {
    cudaStreamSynchronize(ctx->admit_stream);
    cudaStreamDestroy(ctx->admit_stream);
  }
  for (int i = 0; i < 6; ++i)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  for (void* b : ctx->host_blocks) cudaFreeHost(b);
  delete ctx;
  return ACDC_OK;
}

extern "C" int acdc_ctx_memory(acdc_ctx* ctx, int64_t* reserved, int64_t* used) {
  if (!ctx || !reserved || !used) return ACDC_EINVAL;
  uint64_t r = 0, u = 0;
  ACDC_CK(ctx, cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &r));
  ACDC_CK(ctx, cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemCurrent, &u));
  *reserved = (int64_t)r;
  *used = (int64_t)u;
  return ACDC_OK;
}

cudaError_t acdc_dev_alloc(acdc_ctx* ctx, void** p, size_t bytes) {
  return cudaMallocFromPoolAsync(p, bytes > 0 ? bytes : 1, ctx->pool, ctx->stream);
}

void acdc_dev_free(acdc_ctx* ctx, void* p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

cudaError_t acdc_host_slot_take(acdc_ctx* ctx, double** slot) {
  if (ctx->host_free.empty()) {
    constexpr int kPerBlock = 64;
    void* block = nullptr;
    cudaError_t e = cudaMallocHost(&block, sizeof(double) * kHostSlotDoubles * kPerBlock);
    if (e != cudaSuccess) return e;
    ctx->host_blocks.push_back(block);
    for (int i = kPerBlock - 1; i >= 0; --i)
      ctx->host_free.push_back(static_cast<double*>(block) + (size_t)i * kHostSlotDoubles);
  }
  *slot = ctx->host_free.back();
  ctx->host_free.pop_back();
  return cudaSuccess;
}

void acdc_host_slot_give(acdc_ctx* ctx, double* slot) {
  if (slot) ctx->host_free.push_back(slot);
}

// ---- problem ----

namespace {

template <typename T>
cudaError_t dalloc(acdc_ctx* ctx, T** p, int64_t count, int64_t* bytes) {
  size_t b = sizeof(T) * (size_t)(count > 0 ? count : 1);
  *bytes += (int64_t)b;
  return acdc_dev_alloc(ctx, (void**)p, b);
}

void free_problem_buffers(acdc_ctx* ctx, DevProblem& d) {
  acdc_dev_free(ctx, d.meta);
  acdc_dev_free(ctx, d.x32);
  acdc_dev_free(ctx, d.vals);
  acdc_dev_free(ctx, d.idx);
  acdc_dev_free(ctx, d.r32);
  acdc_dev_free(ctx, d.r64);
  acdc_dev_free(ctx, d.rhs64);
  acdc_dev_free(ctx, d.col_sq);
  acdc_dev_free(ctx, d.active);
  acdc_dev_free(ctx, d.xbuf);
  acdc_dev_free(ctx, d.x64);
  acdc_dev_free(ctx, d.rowcnt);
  acdc_dev_free(ctx, d.long_cols);
  acdc_dev_free(ctx, d.r_ref);
  acdc_dev_free(ctx, d.viol);
  acdc_dev_free(ctx, d.hot);
  acdc_dev_free(ctx, d.row_flag);
  acdc_dev_free(ctx, d.mb_draws);
  acdc_dev_free(ctx, d.mb_delta);
  acdc_dev_free(ctx, d.mb_mark);
  acdc_dev_free(ctx, d.part);
  acdc_dev_free(ctx, d.eval_out);
  acdc_dev_free(ctx, d.counters);
  d = DevProblem();
}

int check_status_word(acdc_problem* p) {
  acdc_ctx* ctx = p->ctx;
  ACDC_CK(ctx, cudaMemcpyAsync(p->h_counters, p->d.counters, sizeof(unsigned long long) * CNT_SLOTS,
                               cudaMemcpyDeviceToHost, ctx->stream));
  ACDC_CK(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned long long st = p->h_counters[CNT_STATUS];
  if (st) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "device status 0x%llx (%s%s%s)", st,
                  (st & DEV_ERR_BAD_INDEX) ? "row index out of range " : "",
                  (st & DEV_ERR_BAD_LAYOUT) ? "decreasing column pointers " : "",
                  (st & DEV_ERR_BAD_STATE) ? "bad state" : "");
    return acdc_set_error(ctx, ACDC_EDEVICE, buf);
  }
  return ACDC_OK;
}

// The hot-set tier: Lasso with q-shrinking and screened evaluations.
bool hot_enabled(const acdc_problem* p) {
  return p->loss == ACDC_LOSS_L1_SQUARE && p->s.use_shrinking && p->s.screened_eval &&
         p->s.hot_threshold > 0;
}

EvalParams eval_params(acdc_problem* p, bool build_active) {
  EvalParams e;
  e.meta = p->d.meta;
  e.vals = p->d.vals;
  e.idx = p->d.idx;
  e.r32 = p->d.r32;
  e.r64 = p->d.r64;
  e.rhs64 = p->d.rhs64;
  e.active = build_active ? p->d.active : nullptr;
  e.counters = p->d.counters;
  e.part = p->d.part;
  e.eval_out = p->d.eval_out;
  e.m = p->d.m;
  e.n = p->d.n;
  e.lambda = p->lambda;
  e.shrink_thresh = (1.0 - p->s.shrink_eps) * p->lambda;
  e.loss = p->loss;
  e.x64 = p->fp64_mode ? p->d.x64 : nullptr;
  e.x32 = p->d.x32;
  e.long_cols = p->d.long_cols;
  e.n_long = p->d.n_long;
  if (build_active && p->loss == ACDC_LOSS_L1_SQUARE) e.r_ref = p->d.r_ref;
  if (p->loss == ACDC_LOSS_LOGISTIC) e.roww = p->d.r_ref;
  e.col_norm_max = p->col_norm_max;
  if (build_active && hot_enabled(p)) {
    e.viol = p->d.viol;
    e.hot = p->d.hot;
    e.row_flag = p->d.row_flag;
    e.rowcnt = p->d.rowcnt;
    e.hot_frac = p->s.hot_threshold;
  }
  return e;
}

// Update kernel of the problem's launches (settings.lanes_per_update): 0 = the
// lean one-warp kernel for the q-shrinking launches and the ring kernel for the
// others, 1 = the lean kernel for all, -1 = the ring kernel for all, 8/16/32 =
// the grouped kernel.
int32_t lanes_for(const acdc_problem* p) {
  const int32_t l = p->s.lanes_per_update;
  if (l == 1 || l == -1 || l == 8 || l == 16 || l == 32) return l;
  return 0;
}

UpdateParams update_params(acdc_problem* p, uint64_t count, bool shrink) {
  UpdateParams u;
  u.meta = p->d.meta;
  u.vals = p->d.vals;
  u.idx = p->d.idx;
  u.r = p->d.r32;
  u.active = p->d.active;
  u.counters = p->d.counters;
  u.n = p->d.n;
  u.count = count;
  u.seed = p->s.seed;
  if (p->loss == ACDC_LOSS_SVM_DUAL) {
    u.lambda_d = p->lambda * (double)p->d.n;
    u.inv_lambda_n_d = 1.0 / (p->lambda * (double)p->d.n);
  } else {
    u.lambda_d = p->lambda;
    u.inv_lambda_n_d = 0.0;
  }
  u.li_scale = shrink ? p->li_scale_shrink : 1.0;
  u.x64 = p->d.x64;
  u.r64 = p->d.r64;
  u.x32 = p->d.x32;
  u.fp64 = p->fp64_mode ? 1 : 0;
  double q = p->s.shrinking_probability;
  if (!shrink || q <= 0)
    u.shrink_q32 = 0;
  else if (q >= 1)
    u.shrink_q32 = 0xffffffffu;
  else
    u.shrink_q32 = (uint32_t)(q * 4294967296.0);
  u.n_warps = (shrink && p->s.tau_active > 0) ? p->s.tau_active : p->s.tau;
  u.loss = p->loss;
  u.lanes = lanes_for(p);
  u.sm_count = p->ctx->sm_count;
  if (shrink && u.shrink_q32 && p->hot_count > 0 && p->hot_q > 0) {
    u.hot = p->d.hot;
    u.hot_q32 = (uint32_t)std::min(4294967295.0, p->hot_q * 4294967296.0);
    if (u.hot_q32 > u.shrink_q32) u.hot_q32 = u.shrink_q32;
    u.li_scale_hot = p->li_scale_hot;
  }
  return u;
}

void fill_eval(const double* h, acdc_eval* out) {
  out->primal = h[0];
  out->dual = h[1];
  out->gap = h[2];
  out->rel_gap = h[3];
  out->zero_one_accuracy = h[4];
  out->reg_norm = h[5];
  out->sq_norm = h[6];
  out->max_abs_grad = h[7];
  out->support = (int64_t)h[8];
  out->active = (int64_t)h[9];
}

bool shrink_now(const acdc_problem* p) {
  return p->s.use_shrinking && p->active_valid && p->epochs_done >= p->s.shrinking_starting_iter;
}

int apply_settings(acdc_problem* p, const acdc_settings* s) {
  acdc_ctx* ctx = p->ctx;
  if (s->loss != p->loss) return acdc_set_error(ctx, ACDC_EINVAL, "settings.loss differs from the problem's loss");
  if (const char* bad = settings_fault(s))
    return acdc_set_error(ctx, ACDC_EINVAL, std::string("invalid settings value: ") + bad);
  p->s = *s;
  // q-shrinking and its screened evaluations cover losses 0 and 2 only, and
  // the asynchronous draws only.
  if (p->loss == ACDC_LOSS_L2_SQUARE || p->loss == ACDC_LOSS_LOGISTIC || p->s.minibatch)
    p->s.use_shrinking = 0;
  p->screen_valid = false;
  const double n = (double)p->d.n;
  if (s->sigma > 0)
    p->beta = s->sigma;
  else
    p->beta = n > 1 ? 1.0 + ((double)p->omega - 1.0) * ((double)s->tau - 1.0) / (n - 1.0) : 1.0;
  ACDC_CK(ctx, launch_set_li(p->d, p->loss, p->beta, p->lambda, ctx->stream));
  return ACDC_OK;
}

// Matrix given by rows (acdc_problem_create_rows): row_ptr[0..m], the column
// index and value of every entry.
struct RowsInput {
  const int64_t* row_ptr;
  const int32_t* col_idx;
  const double* vals;
};

int create_impl(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n, const int64_t* col_ptr64,
                const int32_t* col_ptr32, const int32_t* row_idx, const double* vals,
                const double* rhs, double lambda, acdc_problem** out,
                const RowsInput* by_rows = nullptr) {
  if (!ctx || !out) return ACDC_EINVAL;
  *out = nullptr;
  NvtxRange range("acdc_problem_create");
  if (loss < ACDC_LOSS_L1_SQUARE || loss > ACDC_LOSS_LOGISTIC)
    return acdc_set_error(ctx, ACDC_EINVAL, "unknown loss code");
  if (m <= 0 || n <= 0 || m > INT32_MAX || n > INT32_MAX || !positive_finite(lambda) || !rhs ||
      (!by_rows && !col_ptr64 && !col_ptr32) || (by_rows && !by_rows->row_ptr))
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid sizes, lambda or null pointer");
  int64_t nnz = 0;
  if (by_rows) {
    const int64_t* rp = by_rows->row_ptr;
    if (rp[0] != 0) return acdc_set_error(ctx, ACDC_EINVAL, "row_ptr must start at 0");
    for (int64_t i = 0; i < m; ++i)
      if (rp[i + 1] < rp[i]) return acdc_set_error(ctx, ACDC_EINVAL, "decreasing row_ptr");
    nnz = rp[m];
    if (nnz > 0 && (!by_rows->col_idx || !by_rows->vals))
      return acdc_set_error(ctx, ACDC_EINVAL, "null col_idx or vals");
  } else {
    const int64_t c0 = col_ptr64 ? col_ptr64[0] : col_ptr32[0];
    nnz = col_ptr64 ? col_ptr64[n] : col_ptr32[n];
    if (c0 != 0 || nnz < 0) return acdc_set_error(ctx, ACDC_EINVAL, "col_ptr must start at 0 and end at nnz >= 0");
    if (nnz > 0 && (!row_idx || !vals)) return acdc_set_error(ctx, ACDC_EINVAL, "null row_idx or vals");
  }
  ACDC_CK(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;

  acdc_problem* p = new acdc_problem();
  p->ctx = ctx;
  p->loss = loss;
  p->lambda = lambda;
  std::memset(&p->stats, 0, sizeof(p->stats));
  DevProblem& d = p->d;
  d.m = m;
  d.n = n;
  d.nnz = nnz;
  int rc = ACDC_OK;
  // Staging: col_ptr (int64), row_idx, FP64 values, scan scratch / row counts.
  const int64_t tiles = layout_scan_tiles(n);
  const int64_t scratch_len = std::max<int64_t>(n + tiles + 1, (m + 1) / 2 + 1);
  int64_t* s_colptr = nullptr;
  int32_t* s_rows = nullptr;
  double* s_vals = nullptr;
  int64_t* s_scratch = nullptr;
  int64_t stage_bytes = 0;
  auto fail = [&](int code) {
    acdc_dev_free(ctx, s_colptr);
    acdc_dev_free(ctx, s_rows);
    acdc_dev_free(ctx, s_vals);
    acdc_dev_free(ctx, s_scratch);
    free_problem_buffers(ctx, d);
    acdc_host_slot_give(ctx, p->h_eval);
    delete p;
    return code;
  };
#define STEP(call)                                          \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return fail(acdc_cuda_error(ctx, _e, #call)); \
  } while (0)
  STEP(acdc_host_slot_take(ctx, &p->h_eval));
  p->h_counters = reinterpret_cast<unsigned long long*>(p->h_eval + 16);
  STEP(dalloc(ctx, &d.counters, CNT_SLOTS, &d.bytes));
  STEP(cudaMemsetAsync(d.counters, 0, sizeof(unsigned long long) * CNT_SLOTS, st));
  STEP(dalloc(ctx, &s_colptr, n + 1, &stage_bytes));
  STEP(dalloc(ctx, &s_scratch, scratch_len, &stage_bytes));
  if (by_rows) {
    // Upload the rows and transpose them on the device into the staging arrays.
    int64_t* r_ptr = nullptr;
    int32_t* r_col = nullptr;
    double* r_val = nullptr;
    char* t_scratch = nullptr;
    cudaError_t e = dalloc(ctx, &r_ptr, m + 1, &stage_bytes);
    if (e == cudaSuccess) e = dalloc(ctx, &r_col, nnz, &stage_bytes);
    if (e == cudaSuccess) e = dalloc(ctx, &r_val, nnz, &stage_bytes);
    if (e == cudaSuccess) e = dalloc(ctx, &t_scratch, rows_to_columns_scratch_bytes(m, n, nnz), &stage_bytes);
    if (e == cudaSuccess) e = dalloc(ctx, &s_rows, nnz, &stage_bytes);
    if (e == cudaSuccess) e = dalloc(ctx, &s_vals, nnz, &stage_bytes);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(r_ptr, by_rows->row_ptr, sizeof(int64_t) * (m + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nnz > 0)
      e = cudaMemcpyAsync(r_col, by_rows->col_idx, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nnz > 0)
      e = cudaMemcpyAsync(r_val, by_rows->vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = launch_rows_to_columns(r_ptr, r_col, r_val, m, n, nnz, t_scratch, s_colptr, s_rows,
                                 s_vals, d.counters + CNT_STATUS, st);
    acdc_dev_free(ctx, r_ptr);
    acdc_dev_free(ctx, r_col);
    acdc_dev_free(ctx, r_val);
    acdc_dev_free(ctx, t_scratch);
    if (e != cudaSuccess) return fail(acdc_cuda_error(ctx, e, "rows to columns"));
    rc = check_status_word(p);  // column indices out of range
    if (rc != ACDC_OK) return fail(rc);
  } else if (col_ptr64) {
    STEP(cudaMemcpyAsync(s_colptr, col_ptr64, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st));
  } else {
    // Stage the int32 pointers in the scratch area and widen them on the device.
    int32_t* tmp = reinterpret_cast<int32_t*>(s_scratch);
    STEP(cudaMemcpyAsync(tmp, col_ptr32, sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, st));
    STEP(launch_widen_i32(tmp, s_colptr, n + 1, st));
  }
  if (nnz > 0 && !by_rows) {
    STEP(dalloc(ctx, &s_rows, nnz, &stage_bytes));
    STEP(dalloc(ctx, &s_vals, nnz, &stage_bytes));
    STEP(cudaMemcpyAsync(s_rows, row_idx, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
    STEP(cudaMemcpyAsync(s_vals, vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
  }
  // Layout pass 1 and the padded size.
  STEP(launch_layout_scan(s_colptr, n, s_scratch, d.counters, st));
  // Decreasing column pointers would send the fill pass outside the staged
  // arrays: stop here if the scan flagged any.
  rc = check_status_word(p);
  if (rc != ACDC_OK) return fail(rc);
  int64_t units = 0;
  STEP(cudaMemcpyAsync(&units, s_scratch + n + tiles, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  STEP(cudaStreamSynchronize(st));
  if (units < 0 || units >= ((int64_t)1 << 32))
    return fail(acdc_set_error(ctx, ACDC_EINVAL, "matrix too large for 32-bit column starts"));
  d.nnz_pad = units * 4;
  const int64_t rhs_len = loss == ACDC_LOSS_SVM_DUAL ? n : m;
  STEP(dalloc(ctx, &d.meta, n, &d.bytes));
  STEP(dalloc(ctx, &d.x32, n, &d.bytes));
  STEP(cudaMemsetAsync(d.x32, 0, sizeof(float) * n, st));
  STEP(dalloc(ctx, &d.vals, d.nnz_pad, &d.bytes));
  STEP(dalloc(ctx, &d.idx, d.nnz_pad, &d.bytes));
  STEP(dalloc(ctx, &d.r32, m, &d.bytes));
  STEP(dalloc(ctx, &d.r64, m, &d.bytes));
  STEP(dalloc(ctx, &d.rhs64, rhs_len, &d.bytes));
  STEP(dalloc(ctx, &d.col_sq, n, &d.bytes));
  STEP(dalloc(ctx, &d.active, n, &d.bytes));
  STEP(dalloc(ctx, &d.xbuf, n, &d.bytes));
  STEP(dalloc(ctx, &d.x64, n, &d.bytes));
  STEP(dalloc(ctx, &d.rowcnt, m, &d.bytes));
  if (loss == ACDC_LOSS_LOGISTIC) STEP(dalloc(ctx, &d.r_ref, m, &d.bytes));  // row weights
  if (loss == ACDC_LOSS_L1_SQUARE) {
    STEP(dalloc(ctx, &d.r_ref, m, &d.bytes));
    STEP(dalloc(ctx, &d.viol, n, &d.bytes));
    STEP(dalloc(ctx, &d.hot, n, &d.bytes));
    STEP(dalloc(ctx, &d.row_flag, m, &d.bytes));
    STEP(cudaMemsetAsync(d.row_flag, 0, m, st));
  }
  STEP(dalloc(ctx, &d.part, (int64_t)ACDC_RED_BLOCKS * ACDC_NPART, &d.bytes));
  STEP(dalloc(ctx, &d.eval_out, 16, &d.bytes));
  STEP(cudaMemsetAsync(d.part, 0, sizeof(double) * ACDC_RED_BLOCKS * ACDC_NPART, st));
  STEP(cudaMemcpyAsync(d.rhs64, rhs, sizeof(double) * rhs_len, cudaMemcpyHostToDevice, st));
  STEP(launch_layout_fill(s_colptr, s_rows, s_vals, m, n, s_scratch, d, loss, st));
  // omega: the largest number of entries in one residual row, counted on the
  // unpadded input (pad entries all point at row 0).
  int32_t* counts = reinterpret_cast<int32_t*>(s_scratch);
  STEP(cudaMemsetAsync(counts, 0, sizeof(int32_t) * m, st));
  STEP(launch_row_counts(s_rows, nnz, counts, m, d.counters, st));
  unsigned long long* omega_slot = d.counters + CNT_GMAX_BITS;
  STEP(cudaMemsetAsync(omega_slot, 0, sizeof(unsigned long long), st));
  STEP(launch_max_i32(counts, m, omega_slot, st));
  // Columns too long for the thread-per-column gap pass.
  STEP(dalloc(ctx, &d.long_cols, n, &d.bytes));
  STEP(launch_list_long(d, d.long_cols, d.counters + CNT_NLONG, st));
  rc = check_status_word(p);
  if (rc != ACDC_OK) return fail(rc);
  // The reference starts its running maximum at 1 (MultiCoreSolver.cpp:24).
  p->omega = std::max<int64_t>(1, (int64_t)p->h_counters[CNT_GMAX_BITS]);
  d.n_long = (int64_t)p->h_counters[CNT_NLONG];
  acdc_dev_free(ctx, s_colptr);
  s_colptr = nullptr;
  acdc_dev_free(ctx, s_rows);
  s_rows = nullptr;
  acdc_dev_free(ctx, s_vals);
  s_vals = nullptr;
  acdc_dev_free(ctx, s_scratch);
  s_scratch = nullptr;
#undef STEP
  acdc_settings s;
  acdc_settings_default(&s);
  s.loss = loss;
  if (loss == ACDC_LOSS_SVM_DUAL) s.gap_relative = 0;
  rc = apply_settings(p, &s);
  if (rc != ACDC_OK) return fail(rc);
  // The engine constructor refreshes the residual from x = 0
  // (MulticoreEngineExecutor.h:59): r = -b (Lasso) or w = 0 (SVM).
  {
    EvalParams e = eval_params(p, false);
    cudaError_t ce = launch_refresh(e, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return fail(acdc_cuda_error(ctx, ce, "initial refresh"));
  }
  rc = check_status_word(p);
  if (rc != ACDC_OK) return fail(rc);
  {
    const unsigned long long bits = p->h_counters[CNT_COLSQ_BITS];
    double sq;
    std::memcpy(&sq, &bits, sizeof(sq));
    p->col_norm_max = std::sqrt(sq);
  }
  ctx->live_problems++;
  *out = p;
  return ACDC_OK;
}

}  // namespace

extern "C" int acdc_problem_create(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n,
                                   const int64_t* col_ptr, const int32_t* row_idx,
                                   const double* vals, const double* rhs, double lambda,
                                   acdc_problem** out) {
  return create_impl(ctx, loss, m, n, col_ptr, nullptr, row_idx, vals, rhs, lambda, out);
}

extern "C" int acdc_problem_create_i32(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n,
                                       const int32_t* col_ptr, const int32_t* row_idx,
                                       const double* vals, const double* rhs, double lambda,
                                       acdc_problem** out) {
  return create_impl(ctx, loss, m, n, nullptr, col_ptr, row_idx, vals, rhs, lambda, out);
}

extern "C" int acdc_problem_create_rows(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n,
                                        const int64_t* row_ptr, const int32_t* col_idx,
                                        const double* vals, const double* rhs, double lambda,
                                        acdc_problem** out) {
  RowsInput r{row_ptr, col_idx, vals};
  return create_impl(ctx, loss, m, n, nullptr, nullptr, nullptr, nullptr, rhs, lambda, out, &r);
}

extern "C" int acdc_problem_destroy(acdc_problem* p) {
  if (!p) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  cudaSetDevice(ctx->device);
  // copies into the problem's pinned slot must land before the slot is reused
  cudaStreamSynchronize(ctx->stream);
  if (p->mb_graph) cudaGraphExecDestroy(p->mb_graph);
  free_problem_buffers(ctx, p->d);
  acdc_host_slot_give(ctx, p->h_eval);
  ctx->live_problems--;
  delete p;
  return ACDC_OK;
}

extern "C" int acdc_problem_info_get(acdc_problem* p, acdc_problem_info* info) {
  if (!p || !info) return ACDC_EINVAL;
  info->m = p->d.m;
  info->n = p->d.n;
  info->nnz = p->d.nnz;
  info->nnz_padded = p->d.nnz_pad;
  info->omega = p->omega;
  info->sigma = p->beta;
  info->lambda = p->lambda;
  info->device_bytes = p->d.bytes;
  info->loss = p->loss;
  info->tau = p->s.tau;
  info->omega_active = p->omega_active;
  info->active_step_scale = p->li_scale_shrink;
  info->long_columns = p->d.n_long;
  return ACDC_OK;
}

extern "C" int acdc_problem_reset(acdc_problem* p) {
  if (!p) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  ACDC_CK(ctx, cudaMemsetAsync(p->d.xbuf, 0, sizeof(double) * p->d.n, ctx->stream));
  p->fp64_mode = false;
  ACDC_CK(ctx, launch_set_x(p->d, false, ctx->stream));
  p->k_next = 0;
  p->epochs_done = 0;
  p->updates_done = 0;
  p->mb_updates = 0;
  ACDC_CK(ctx, cudaMemsetAsync(p->d.counters + CNT_MB_COUNTER, 0, sizeof(unsigned long long),
                               ctx->stream));
  p->active_valid = false;
  p->screen_valid = false;
  p->li_scale_shrink = 1.0;
  p->omega_active = 1;
  p->hot_count = 0;
  p->hot_q = 0;
  p->li_scale_hot = 1.0;
  EvalParams e = eval_params(p, false);
  ACDC_CK(ctx, launch_refresh(e, ctx->stream));
  return ACDC_OK;
}

extern "C" int acdc_problem_set_settings(acdc_problem* p, const acdc_settings* s) {
  if (!p || !s) return ACDC_EINVAL;
  return apply_settings(p, s);
}

namespace {
// Polish-mode transitions.  Entering copies x exactly (FP32 -> FP64); the FP64
// residual of the last refresh already equals A x - b for that x.  Leaving
// rounds x to FP32 and refreshes both residuals from it.
int enter_fp64(acdc_problem* p) {
  if (p->fp64_mode) return ACDC_OK;
  ACDC_CK(p->ctx, launch_x32_to_x64(p->d, p->ctx->stream));
  p->fp64_mode = true;
  return ACDC_OK;
}

int leave_fp64(acdc_problem* p) {
  if (!p->fp64_mode) return ACDC_OK;
  ACDC_CK(p->ctx, launch_x64_to_x32(p->d, p->ctx->stream));
  p->fp64_mode = false;
  EvalParams e = eval_params(p, false);
  ACDC_CK(p->ctx, launch_refresh(e, p->ctx->stream));
  return ACDC_OK;
}
}  // namespace

extern "C" int acdc_problem_set_lambda(acdc_problem* p, double lambda) {
  if (!p) return ACDC_EINVAL;
  if (!positive_finite(lambda))
    return acdc_set_error(p->ctx, ACDC_EINVAL, "lambda must be positive and finite");
  p->lambda = lambda;
  p->active_valid = false;
  p->screen_valid = false;
  // Losses 1 and 3 carry lambda in their Lipschitz constants.
  if (p->loss == ACDC_LOSS_L2_SQUARE || p->loss == ACDC_LOSS_LOGISTIC)
    ACDC_CK(p->ctx, launch_set_li(p->d, p->loss, p->beta, p->lambda, p->ctx->stream));
  // A new lambda starts with the FP32 bulk again (AUTO precision).
  if (p->s.precision == ACDC_PREC_AUTO) return leave_fp64(p);
  return ACDC_OK;
}

namespace {
bool minibatch_mode(const acdc_problem* p) {
  return p->s.minibatch != 0 && p->loss == ACDC_LOSS_SVM_DUAL;
}

// Updates of one mini-batch epoch: ceil(n / tau) steps of tau (tau <= n).
uint64_t minibatch_epoch(const acdc_problem* p) {
  const uint64_t n = (uint64_t)p->d.n;
  const uint64_t tau = (uint64_t)std::min<int64_t>(std::max(1, p->s.tau), p->d.n);
  return (n + tau - 1) / tau * tau;
}

// Synchronous mini-batch steps (settings.minibatch, SVM dual): enough steps of
// tau distinct draws for n_updates updates (at least one), drawn an epoch's
// worth at a time.  *done gets the updates made.
int run_minibatch(acdc_problem* p, uint64_t n_updates, uint64_t* done) {
  acdc_ctx* ctx = p->ctx;
  DevProblem& d = p->d;
  const int32_t tau = (int32_t)std::min<int64_t>(std::max(1, p->s.tau), d.n);
  const int64_t per_epoch = (d.n + tau - 1) / tau;
  if (!d.mb_draws) {
    const size_t words = (size_t)((d.n + 31) / 32);
    ACDC_CK(ctx, acdc_dev_alloc(ctx, (void**)&d.mb_draws, sizeof(int32_t) * (size_t)(per_epoch * tau)));
    ACDC_CK(ctx, acdc_dev_alloc(ctx, (void**)&d.mb_delta, sizeof(double) * (size_t)tau));
    ACDC_CK(ctx, acdc_dev_alloc(ctx, (void**)&d.mb_mark, sizeof(uint32_t) * words));
    ACDC_CK(ctx, cudaMemsetAsync(d.mb_mark, 0, sizeof(uint32_t) * words, ctx->stream));
    d.bytes += (int64_t)(sizeof(int32_t) * per_epoch * tau + sizeof(double) * tau +
                         sizeof(uint32_t) * words);
    p->mb_tau = tau;
  }
  if (tau != p->mb_tau)
    return acdc_set_error(ctx, ACDC_EINVAL, "minibatch: tau changed after the first mini-batch step");
  int64_t steps = (int64_t)((n_updates + (uint64_t)tau - 1) / (uint64_t)tau);
  if (steps < 1) steps = 1;
  UpdateParams u = update_params(p, (uint64_t)tau, false);
  auto enqueue = [&](int32_t batch) -> cudaError_t {
    cudaError_t e = launch_tau_nice(p->s.seed, d.n, tau, batch, d.counters + CNT_MB_COUNTER,
                                    d.mb_draws, d.mb_mark, ctx->stream);
    for (int32_t t = 0; t < batch && e == cudaSuccess; ++t)
      e = launch_minibatch_step(u, d.mb_draws + (int64_t)t * tau, tau, d.mb_delta, ctx->stream);
    return e;
  };
  // A whole epoch (the sampler and 2 ceil(n / tau) kernels) replays from a
  // CUDA graph captured once for the current precision, lambda and seed; the
  // draw counter lives on the device, so every replay continues the stream.
  const bool key_ok = p->mb_graph && p->mb_graph_fp64 == p->fp64_mode &&
                      p->mb_graph_lambda == p->lambda && p->mb_graph_seed == p->s.seed;
  if (!key_ok && p->mb_graph) {
    cudaGraphExecDestroy(p->mb_graph);
    p->mb_graph = nullptr;
  }
  if (!p->mb_graph && steps >= per_epoch) {
    cudaGraph_t g = nullptr;
    ACDC_CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue((int32_t)per_epoch);
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->mb_graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      p->mb_graph = nullptr;
      return acdc_cuda_error(ctx, e, "mini-batch epoch graph");
    }
    p->mb_graph_fp64 = p->fp64_mode;
    p->mb_graph_lambda = p->lambda;
    p->mb_graph_seed = p->s.seed;
  }
  int64_t s0 = 0;
  for (; p->mb_graph && s0 + per_epoch <= steps; s0 += per_epoch)
    ACDC_CK(ctx, cudaGraphLaunch(p->mb_graph, ctx->stream));
  for (; s0 < steps; s0 += per_epoch)
    ACDC_CK(ctx, enqueue((int32_t)std::min<int64_t>(per_epoch, steps - s0)));
  const uint64_t made = (uint64_t)steps * (uint64_t)tau;
  p->mb_updates += made;
  p->updates_done += made;
  p->epochs_done = (int64_t)(p->updates_done / (uint64_t)d.n);
  p->stats.update_launches += 2 * steps;
  *done = made;
  return ACDC_OK;
}
}  // namespace

extern "C" int acdc_run_updates(acdc_problem* p, uint64_t n_updates) {
  if (!p) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  if (minibatch_mode(p)) {
    uint64_t done = 0;
    return run_minibatch(p, n_updates, &done);
  }
  UpdateParams u = update_params(p, n_updates, shrink_now(p));
  ACDC_CK(ctx, launch_update(u, p->k_next, p->s.warps_per_block, ctx->stream));
  p->k_next += n_updates;
  p->updates_done += n_updates;
  p->epochs_done = (int64_t)(p->updates_done / (uint64_t)p->d.n);
  p->stats.update_launches++;
  return ACDC_OK;
}

extern "C" int acdc_recompute_residuals(acdc_problem* p) {
  if (!p) return ACDC_EINVAL;
  EvalParams e = eval_params(p, false);
  ACDC_CK(p->ctx, launch_refresh(e, p->ctx->stream));
  return ACDC_OK;
}

namespace {
// Refresh + gap; copies the result to the pinned host buffer and waits.  A
// screened evaluation (Lasso, after a full one that built the active set)
// gathers only the active columns and bounds the others.
int evaluate_impl(acdc_problem* p, acdc_eval* out, float* ms, bool screened = false) {
  acdc_ctx* ctx = p->ctx;
  screened = screened && p->screen_valid;
  NvtxRange range(screened ? "acdc_evaluate_screened" : "acdc_evaluate");
  const bool build_active = p->s.use_shrinking != 0 && !screened;
  EvalParams e = eval_params(p, p->s.use_shrinking != 0);
  e.screened = screened ? 1 : 0;
  ACDC_CK(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
  ACDC_CK(ctx, launch_refresh(e, ctx->stream));
  ACDC_CK(ctx, launch_gap(e, ctx->stream));
  if (build_active) ACDC_CK(ctx, launch_active_omega(e, p->d.rowcnt, ctx->stream));
  const bool hot = e.viol != nullptr;
  if (hot) ACDC_CK(ctx, launch_hot_set(e, ctx->stream));
  ACDC_CK(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
  ACDC_CK(ctx, cudaMemcpyAsync(p->h_eval, p->d.eval_out, sizeof(double) * 16,
                               cudaMemcpyDeviceToHost, ctx->stream));
  int rc = check_status_word(p);  // synchronises the stream
  if (rc != ACDC_OK) return rc;
  float t = 0;
  ACDC_CK(ctx, cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]));
  p->stats.eval_ms += t;
  p->stats.eval_launches++;
  if (screened) p->stats.screened_evals++;
  if (ms) *ms = t;
  if (!screened) p->screen_valid = build_active && e.r_ref != nullptr;
  if (build_active) {
    p->active_valid = true;
    // ESO parameter of the active-set draws: q*tau of them land on the
    // |A| active columns, whose rows hold at most omega_A of them.
    const double a = p->h_eval[9];
    p->omega_active = std::max<int64_t>(1, (int64_t)p->h_counters[CNT_OMEGA_ACTIVE]);
    const double tau_shrink = p->s.tau_active > 0 ? p->s.tau_active : p->s.tau;
    const double tau_a = std::max(1.0, p->s.shrinking_probability * tau_shrink);
    const double beta_a =
        a > 1 ? 1.0 + ((double)p->omega_active - 1.0) * (tau_a - 1.0) / (a - 1.0) : 1.0;
    p->li_scale_shrink = p->beta / std::max(p->beta, beta_a);
  }
  p->hot_count = 0;
  p->hot_q = 0;
  p->li_scale_hot = 1.0;
  if (hot) {
    // About one draw per hot column per tau_active updates, at most half of the
    // active-set draws; ESO over the hot columns, whose rows hold at most
    // omega_H of them.
    const int64_t h = std::min<int64_t>((int64_t)p->h_counters[CNT_HOT], p->d.n);
    const double tau_shrink = p->s.tau_active > 0 ? p->s.tau_active : p->s.tau;
    if (h > 0) {
      p->hot_count = h;
      p->hot_q = std::min(0.5 * p->s.shrinking_probability, (double)h / tau_shrink);
      const double w_h = std::max<double>(1.0, (double)p->h_counters[CNT_OMEGA_HOT]);
      const double draws = p->hot_q * tau_shrink;
      const double beta_h = h > 1 && draws > 1 ? 1.0 + (w_h - 1.0) * (draws - 1.0) / ((double)h - 1.0)
                                               : 1.0;
      p->li_scale_hot = p->beta / std::max(p->beta, beta_h);
    }
  }
  if (out) fill_eval(p->h_eval, out);
  if (!std::isfinite(p->h_eval[0]))
    return acdc_set_error(ctx, ACDC_EDEVICE, "objective is not finite (diverged or bad input)");
  return ACDC_OK;
}

bool converged(const acdc_settings& s, const acdc_eval& ev) {
  return (s.gap_relative ? ev.rel_gap : ev.gap) <= s.gap_target;
}

// Launches one update bulk of u.count updates and counts them.
int run_counted(acdc_problem* p, const UpdateParams& u, int warps_per_block, uint64_t* done,
                uint64_t* done_fp64) {
  ACDC_CK(p->ctx, launch_update(u, p->k_next, warps_per_block, p->ctx->stream));
  p->k_next += u.count;
  p->updates_done += u.count;
  *done += u.count;
  if (p->fp64_mode) *done_fp64 += u.count;
  return ACDC_OK;
}

// FP64 polish for the certificate.  The FP32 iterate moves x_j only in steps
// of its FP32 spacing, which can leave KKT violations just above what the
// target needs.  So: x64 = x32 exactly (r64 of the evaluation just made is
// exact for it), polish_active_passes passes of the usual q-shrinking draws in
// FP64, one warp of exact steps over the hot list in FP64 with nothing else in
// flight, then a new evaluation.  Kept (*ev replaced, x left in FP64) if it
// meets the target; otherwise x goes back to FP32 (rounded) and the bulks
// continue.  The new evaluation's time is added to *ms.
int polish_for_certificate(acdc_problem* p, acdc_eval* ev, bool screen, uint64_t* done,
                           uint64_t* done_fp64, float* ms) {
  NvtxRange range("acdc_polish");
  int rc = enter_fp64(p);
  if (rc != ACDC_OK) return rc;
  if (p->s.polish_active_passes > 0 && ev->active > 0) {
    const double q = std::max(1e-3, p->s.shrinking_probability);
    const uint64_t cnt = (uint64_t)((double)p->s.polish_active_passes * (double)ev->active / q);
    rc = run_counted(p, update_params(p, cnt, true), p->s.warps_per_block, done, done_fp64);
    if (rc != ACDC_OK) return rc;
  }
  // Hot draws only, one warp, Li = 1/(beta ||a||^2) scaled back by beta.
  UpdateParams h = update_params(p, (uint64_t)p->s.hot_polish_sweeps * (uint64_t)p->hot_count, true);
  h.shrink_q32 = 0xffffffffu;
  h.hot_q32 = 0xffffffffu;
  h.li_scale_hot = p->beta;
  h.n_warps = 1;
  rc = run_counted(p, h, 1, done, done_fp64);
  if (rc != ACDC_OK) return rc;
  acdc_eval ev2;
  float ms2 = 0;
  rc = evaluate_impl(p, &ev2, &ms2, screen);
  if (rc != ACDC_OK) return rc;
  *ms += ms2;
  if (converged(p->s, ev2)) {
    *ev = ev2;
    return ACDC_OK;
  }
  return leave_fp64(p);
}
}  // namespace

extern "C" int acdc_evaluate(acdc_problem* p, acdc_eval* out) {
  if (!p) return ACDC_EINVAL;
  return evaluate_impl(p, out, nullptr);
}

extern "C" int acdc_solve(acdc_problem* p, acdc_solve_result* out) {
  return acdc_solve_traced(p, out, nullptr, 0, nullptr);
}

extern "C" int acdc_solve_traced(acdc_problem* p, acdc_solve_result* out, acdc_trace_row* rows,
                                 int64_t cap, int64_t* n_rows) {
  if (!p || !out || cap < 0 || (cap > 0 && !rows)) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  std::memset(out, 0, sizeof(*out));
  int64_t n_trace = 0;
  auto trace = [&](uint64_t updates, const acdc_eval& e, float upd_ms, float ev_ms, bool shrink,
                   bool fp64, bool screened) {
    if (n_trace < cap) {
      acdc_trace_row& t = rows[n_trace];
      std::memset(&t, 0, sizeof(t));
      t.updates = updates;
      t.primal = e.primal;
      t.gap = e.gap;
      t.rel_gap = e.rel_gap;
      t.active = e.active;
      t.hot = p->hot_count;
      t.omega_active = p->omega_active;
      t.omega_hot = p->hot_count > 0 ? (int64_t)p->h_counters[CNT_OMEGA_HOT] : 0;
      t.update_ms = upd_ms;
      t.eval_ms = ev_ms;
      t.shrink = shrink ? 1 : 0;
      t.fp64 = fp64 ? 1 : 0;
      t.screened = screened ? 1 : 0;
    }
    ++n_trace;
    if (n_rows) *n_rows = n_trace;
  };
  if (n_rows) *n_rows = 0;
  NvtxRange range("acdc_solve");
  auto t0 = std::chrono::steady_clock::now();
  ACDC_CK(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
  int rc = ACDC_OK;
  if (p->s.precision == ACDC_PREC_FP64) rc = enter_fp64(p);
  if (p->s.precision == ACDC_PREC_FP32) rc = leave_fp64(p);
  if (rc != ACDC_OK) return rc;
  acdc_eval ev;
  float ev_ms = 0;
  rc = evaluate_impl(p, &ev, &ev_ms);
  if (rc != ACDC_OK) return rc;
  trace(0, ev, 0.f, ev_ms, false, p->fp64_mode, false);
  // Work is counted in updates; an epoch is n of them (in mini-batch mode,
  // ceil(n / tau) steps of tau, so that bulks and the epoch budget are whole
  // steps).
  const uint64_t n = minibatch_mode(p) ? minibatch_epoch(p) : (uint64_t)p->d.n;
  const uint64_t budget = (uint64_t)p->s.max_epochs * n;
  uint64_t done = 0, done_fp64 = 0;
  double best = ev.rel_gap;
  uint64_t last_gain = 0;  // updates done when the gap last halved
  while (!converged(p->s, ev) && done < budget) {
    // AUTO: the FP32 iterate bounds the certificate near 1e-7 relative (higher
    // for badly scaled columns, or where x_j's FP32 spacing is coarse against
    // the KKT tolerance); finish in FP64 once the gap is small or has not
    // halved over polish_stall_epochs (default 10) epochs of updates.
    const uint64_t stall = p->s.polish_stall_epochs > 0 ? (uint64_t)p->s.polish_stall_epochs : 10u;
    const bool stalled = done - last_gain >= stall * n && ev.rel_gap < 1e-2;
    if (p->s.precision == ACDC_PREC_AUTO && !p->fp64_mode &&
        (ev.rel_gap <= p->s.polish_rel_gap || stalled)) {
      rc = enter_fp64(p);
      if (rc != ACDC_OK) return rc;
    }
    const bool shrink = shrink_now(p);
    uint64_t count = (uint64_t)p->s.refresh_every * n;
    if (shrink && p->s.active_passes > 0 && ev.active > 0) {
      // Passes over the active set: |A| / q updates each.
      const double q = std::max(1e-3, p->s.shrinking_probability);
      count = (uint64_t)((double)p->s.active_passes * (double)ev.active / q);
      count = std::max<uint64_t>(count, 32u * (uint64_t)p->s.tau);
      count = std::min<uint64_t>(count, (uint64_t)p->s.refresh_every * n);
    }
    count = std::min(count, budget - done);
    const bool screen = shrink && p->s.screened_eval != 0 && p->screen_valid;
    UpdateParams u = update_params(p, count, shrink);
    if (minibatch_mode(p)) {
      NvtxRange bulk("acdc_bulk_minibatch");
      uint64_t made = 0;
      ACDC_CK(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
      rc = run_minibatch(p, count, &made);
      if (rc != ACDC_OK) return rc;
      ACDC_CK(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
      count = made;
      done += count;
      if (p->fp64_mode) done_fp64 += count;
    } else {
      {
        NvtxRange bulk(shrink ? "acdc_bulk_active" : "acdc_bulk");
        ACDC_CK(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
        ACDC_CK(ctx, launch_update(u, p->k_next, p->s.warps_per_block, ctx->stream));
        ACDC_CK(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
      }
      p->k_next += count;
      p->stats.update_launches++;
      done += count;
      if (p->fp64_mode) done_fp64 += count;
      p->updates_done += count;
      p->epochs_done = (int64_t)(p->updates_done / n);
    }
    const bool screened_now = screen && p->screen_valid;
    rc = evaluate_impl(p, &ev, &ev_ms, screen);
    if (rc != ACDC_OK) return rc;
    float bulk_ms = 0;
    ACDC_CK(ctx, cudaEventElapsedTime(&bulk_ms, ctx->ev[0], ctx->ev[1]));
    float extra_ms = 0;
    if (screen) {
      // The bound of the inactive columns: past (1 - eps/2) lambda the next
      // evaluation is a full one (new reference residual and active set); past
      // lambda it may inflate this certificate, so run the full one now.
      const double bound = p->h_eval[11];
      if (bound >= (1.0 - 0.5 * p->s.shrink_eps) * p->lambda) p->screen_valid = false;
      if (bound >= p->lambda && !converged(p->s, ev)) {
        rc = evaluate_impl(p, &ev, &extra_ms);
        if (rc != ACDC_OK) return rc;
      }
    }
    if (p->s.hot_polish_sweeps > 0 && shrink && !p->fp64_mode && p->hot_count > 0 &&
        !converged(p->s, ev) && ev.rel_gap < p->s.polish_rel_gap) {
      rc = polish_for_certificate(p, &ev, screen, &done, &done_fp64, &extra_ms);
      if (rc != ACDC_OK) return rc;
    }
    trace(done, ev, bulk_ms, ev_ms + extra_ms, shrink, u.fp64 != 0, screened_now && extra_ms == 0);
    p->stats.update_ms += bulk_ms;
    if (ev.rel_gap < 0.5 * best) {
      best = ev.rel_gap;
      last_gain = done;
    }
  }
  const int epochs = (int)((done + n - 1) / n);
  out->fp64_epochs = (int32_t)((done_fp64 + n - 1) / n);
  ACDC_CK(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
  ACDC_CK(ctx, cudaEventSynchronize(ctx->ev[5]));
  float dev_ms = 0;
  ACDC_CK(ctx, cudaEventElapsedTime(&dev_ms, ctx->ev[4], ctx->ev[5]));
  out->device_ms = dev_ms;
  out->eval = ev;
  out->converged = converged(p->s, ev) ? 1 : 0;
  out->epochs = epochs;
  out->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return acdc_get_stats(p, &out->stats);
}

extern "C" int acdc_get_x(acdc_problem* p, double* x) {
  if (!p || !x) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  ACDC_CK(ctx, launch_get_x(p->d, p->fp64_mode, ctx->stream));
  ACDC_CK(ctx, cudaMemcpyAsync(x, p->d.xbuf, sizeof(double) * p->d.n, cudaMemcpyDeviceToHost,
                               ctx->stream));
  ACDC_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return ACDC_OK;
}

extern "C" int acdc_set_x(acdc_problem* p, const double* x) {
  if (!p || !x) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  ACDC_CK(ctx, cudaMemcpyAsync(p->d.xbuf, x, sizeof(double) * p->d.n, cudaMemcpyHostToDevice,
                               ctx->stream));
  ACDC_CK(ctx, launch_set_x(p->d, p->fp64_mode, ctx->stream));
  ACDC_CK(ctx, cudaStreamSynchronize(ctx->stream));
  p->active_valid = false;
  p->screen_valid = false;
  return acdc_recompute_residuals(p);
}

namespace {
// Checkpoint layout: this header, then x as n doubles.
struct CheckpointHeader {
  char magic[8];            // "ACDCCKP2"
  int32_t loss, fp64;
  int64_t m, n;
  uint64_t k_next, updates_done;
  int64_t epochs_done;
  double lambda;
  uint64_t mb_counter;      // sampler counter of the synchronous mini-batch draws
  uint64_t mb_updates;
};
constexpr char kCheckpointMagic[8] = {'A', 'C', 'D', 'C', 'C', 'K', 'P', '2'};
}  // namespace

extern "C" int64_t acdc_checkpoint_size(const acdc_problem* p) {
  if (!p) return 0;
  return (int64_t)sizeof(CheckpointHeader) + (int64_t)sizeof(double) * p->d.n;
}

extern "C" int acdc_checkpoint_save(acdc_problem* p, void* buf, int64_t size) {
  if (!p || !buf || size != acdc_checkpoint_size(p)) return ACDC_EINVAL;
  CheckpointHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kCheckpointMagic, sizeof(h.magic));
  h.loss = p->loss;
  h.fp64 = p->fp64_mode ? 1 : 0;
  h.m = p->d.m;
  h.n = p->d.n;
  h.k_next = p->k_next;
  h.updates_done = p->updates_done;
  h.epochs_done = p->epochs_done;
  h.lambda = p->lambda;
  h.mb_updates = p->mb_updates;
  ACDC_CK(p->ctx, cudaMemcpyAsync(&h.mb_counter, p->d.counters + CNT_MB_COUNTER, sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, p->ctx->stream));
  ACDC_CK(p->ctx, cudaStreamSynchronize(p->ctx->stream));
  std::memcpy(buf, &h, sizeof(h));
  return acdc_get_x(p, reinterpret_cast<double*>(static_cast<char*>(buf) + sizeof(h)));
}

extern "C" int acdc_checkpoint_load(acdc_problem* p, const void* buf, int64_t size) {
  if (!p || !buf || size != acdc_checkpoint_size(p)) return ACDC_EINVAL;
  CheckpointHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, kCheckpointMagic, sizeof(h.magic)) != 0 || h.loss != p->loss ||
      h.m != p->d.m || h.n != p->d.n || !positive_finite(h.lambda))
    return acdc_set_error(p->ctx, ACDC_EINVAL, "checkpoint of another problem");
  int rc = ACDC_OK;
  if (h.lambda != p->lambda) rc = acdc_problem_set_lambda(p, h.lambda);
  if (rc != ACDC_OK) return rc;
  p->fp64_mode = h.fp64 != 0;
  rc = acdc_set_x(p, reinterpret_cast<const double*>(static_cast<const char*>(buf) + sizeof(h)));
  if (rc != ACDC_OK) return rc;
  p->k_next = h.k_next;
  p->updates_done = h.updates_done;
  p->epochs_done = h.epochs_done;
  p->mb_updates = h.mb_updates;
  ACDC_CK(p->ctx, cudaMemcpyAsync(p->d.counters + CNT_MB_COUNTER, &h.mb_counter, sizeof(uint64_t),
                                  cudaMemcpyHostToDevice, p->ctx->stream));
  ACDC_CK(p->ctx, cudaStreamSynchronize(p->ctx->stream));
  p->hot_count = 0;
  return ACDC_OK;
}

extern "C" int acdc_get_residuals(acdc_problem* p, double* r) {
  if (!p || !r) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  std::vector<float> h((size_t)p->d.m);
  ACDC_CK(ctx, cudaMemcpyAsync(h.data(), p->d.r32, sizeof(float) * p->d.m, cudaMemcpyDeviceToHost, ctx->stream));
  ACDC_CK(ctx, cudaStreamSynchronize(ctx->stream));
  for (int64_t i = 0; i < p->d.m; ++i) r[i] = (double)h[(size_t)i];
  return ACDC_OK;
}

extern "C" int acdc_get_stats(acdc_problem* p, acdc_stats* s) {
  if (!p || !s) return ACDC_EINVAL;
  int rc = check_status_word(p);
  if (rc != ACDC_OK) return rc;
  p->stats.updates = p->h_counters[CNT_UPDATES];
  p->stats.nonzero_updates = p->h_counters[CNT_NONZERO];
  p->stats.nnz_read = p->h_counters[CNT_NNZ_READ];
  p->stats.nnz_scattered = p->h_counters[CNT_NNZ_SCATTERED];
  *s = p->stats;
  return ACDC_OK;
}

extern "C" int acdc_reset_stats(acdc_problem* p) {
  if (!p) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  ACDC_CK(ctx, cudaMemsetAsync(p->d.counters + CNT_UPDATES, 0, sizeof(unsigned long long) * 4, ctx->stream));
  ACDC_CK(ctx, cudaStreamSynchronize(ctx->stream));
  std::memset(&p->stats, 0, sizeof(p->stats));
  return ACDC_OK;
}

extern "C" int acdc_synchronize(acdc_problem* p) {
  if (!p) return ACDC_EINVAL;
  ACDC_CK(p->ctx, cudaStreamSynchronize(p->ctx->stream));
  return check_status_word(p);
}

extern "C" int acdc_debug_sample(acdc_ctx* ctx, uint64_t seed, uint64_t k0, uint64_t count,
                                 int64_t n, int64_t* out) {
  if (!ctx || (count > 0 && !out) || n <= 0) return ACDC_EINVAL;
  int64_t* d = nullptr;
  ACDC_CK(ctx, acdc_dev_alloc(ctx, (void**)&d, sizeof(int64_t) * (count > 0 ? count : 1)));
  cudaError_t e = launch_debug_sample(seed, k0, count, n, d, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  acdc_dev_free(ctx, d);
  if (e != cudaSuccess) return acdc_cuda_error(ctx, e, "acdc_debug_sample");
  return ACDC_OK;
}

extern "C" int acdc_debug_tau_nice(acdc_ctx* ctx, uint64_t seed, uint64_t k0, int64_t n,
                                   int32_t tau, int32_t steps, int32_t* out, uint64_t* k_out) {
  if (!ctx || n <= 0 || n > INT32_MAX || tau < 1 || tau > n || steps < 0 ||
      (steps > 0 && !out) || !k_out)
    return ACDC_EINVAL;
  ACDC_CK(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t words = (size_t)((n + 31) / 32);
  const size_t draws = (size_t)steps * (size_t)tau;
  unsigned long long* d_k = nullptr;
  int32_t* d_s = nullptr;
  uint32_t* d_mark = nullptr;
  cudaError_t e = acdc_dev_alloc(ctx, (void**)&d_k, sizeof(unsigned long long));
  if (e == cudaSuccess) e = acdc_dev_alloc(ctx, (void**)&d_s, sizeof(int32_t) * (draws > 0 ? draws : 1));
  if (e == cudaSuccess) e = acdc_dev_alloc(ctx, (void**)&d_mark, sizeof(uint32_t) * words);
  unsigned long long k = k0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_k, &k, sizeof(k), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_mark, 0, sizeof(uint32_t) * words, st);
  if (e == cudaSuccess) e = launch_tau_nice(seed, n, tau, steps, d_k, d_s, d_mark, st);
  if (e == cudaSuccess && draws > 0)
    e = cudaMemcpyAsync(out, d_s, sizeof(int32_t) * draws, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&k, d_k, sizeof(k), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  acdc_dev_free(ctx, d_k);
  acdc_dev_free(ctx, d_s);
  acdc_dev_free(ctx, d_mark);
  if (e != cudaSuccess) return acdc_cuda_error(ctx, e, "acdc_debug_tau_nice");
  *k_out = k;
  return ACDC_OK;
}

// Test-set accuracy: the test loop of MulticoreSVMDualLoss::computeObjectiveValue
// (cpp/src/solver/lossFunctions/SVMDualLoss/MulticoreSVMDualLoss.h:95-112) for the
// SVM dual, with w refreshed from the current alpha in FP64, and of
// MulticoreL2SquareRegLogisticLoss::computeObjectiveValue (MulticoreL2SquareRegLogisticLoss.h:65-81)
// for the logistic loss, with the coordinates x as weights (that loop reads the
// training matrix's feature indices; the test matrix's own are read here).
extern "C" int acdc_test_accuracy(acdc_problem* p, int64_t n_test, const int64_t* row_ptr,
                                  const int32_t* col_idx, const double* vals,
                                  const double* labels, double* accuracy) {
  if (!p || !accuracy || n_test < 0 || (n_test > 0 && (!row_ptr || !labels))) return ACDC_EINVAL;
  acdc_ctx* ctx = p->ctx;
  if (p->loss != ACDC_LOSS_SVM_DUAL && p->loss != ACDC_LOSS_LOGISTIC)
    return acdc_set_error(ctx, ACDC_EUNSUPPORTED, "test accuracy is for losses 2 and 3");
  *accuracy = 0;
  if (n_test == 0) return ACDC_OK;
  const int64_t nnz = row_ptr[n_test];
  if (row_ptr[0] != 0 || nnz < 0 || (nnz > 0 && (!col_idx || !vals)))
    return acdc_set_error(ctx, ACDC_EINVAL, "invalid test matrix");
  for (int64_t i = 0; i < n_test; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return acdc_set_error(ctx, ACDC_EINVAL, "invalid test matrix");
  cudaStream_t st = ctx->stream;
  const double* w64 = nullptr;
  const float* w32 = nullptr;
  int64_t w_len = 0;
  if (p->loss == ACDC_LOSS_SVM_DUAL) {
    int rc = acdc_recompute_residuals(p);
    if (rc != ACDC_OK) return rc;
    w64 = p->d.r64;
    w_len = p->d.m;
  } else {
    if (p->fp64_mode)
      w64 = p->d.x64;
    else
      w32 = p->d.x32;
    w_len = p->d.n;
  }
  int64_t* d_ptr = nullptr;
  int32_t* d_idx = nullptr;
  double *d_vals = nullptr, *d_lab = nullptr;
  unsigned long long* d_good = nullptr;
  unsigned long long good = 0;
  cudaError_t e = acdc_dev_alloc(ctx, (void**)&d_ptr, sizeof(int64_t) * (n_test + 1));
  if (e == cudaSuccess) e = acdc_dev_alloc(ctx, (void**)&d_idx, sizeof(int32_t) * (nnz > 0 ? nnz : 1));
  if (e == cudaSuccess) e = acdc_dev_alloc(ctx, (void**)&d_vals, sizeof(double) * (nnz > 0 ? nnz : 1));
  if (e == cudaSuccess) e = acdc_dev_alloc(ctx, (void**)&d_lab, sizeof(double) * n_test);
  if (e == cudaSuccess) e = acdc_dev_alloc(ctx, (void**)&d_good, sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_ptr, row_ptr, sizeof(int64_t) * (n_test + 1), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && nnz > 0)
    e = cudaMemcpyAsync(d_idx, col_idx, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && nnz > 0)
    e = cudaMemcpyAsync(d_vals, vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_lab, labels, sizeof(double) * n_test, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = launch_test_accuracy(n_test, d_ptr, d_idx, d_vals, d_lab, w64, w32, w_len, d_good, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&good, d_good, sizeof(good), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  acdc_dev_free(ctx, d_ptr);
  acdc_dev_free(ctx, d_idx);
  acdc_dev_free(ctx, d_vals);
  acdc_dev_free(ctx, d_lab);
  acdc_dev_free(ctx, d_good);
  if (e != cudaSuccess) return acdc_cuda_error(ctx, e, "acdc_test_accuracy");
  *accuracy = (double)good / (double)n_test;
  return ACDC_OK;
}
