// Internal declarations of libacdc_gpu.so (sm_103a).
//
// Device layout of one problem (the column operand: A for the Lasso, X^T for
// the SVM dual; "column" = coordinate, "row" = residual entry):
//   meta[n]   int4 {start4, len, Li, 0}: start4 = column start / 4 in the
//             padded arrays, len = nonzeros, Li = 1/(beta ||a_j||^2) (FP32
//             bits; for the SVM the sign carries y_j).
//   x32[n]    FP32 coordinates, updated in place with red.global.add.f32
//             (contiguous, so passes over every coordinate read 4 bytes each).
//   vals[]    FP32 values, each column starting on a 16-byte boundary and
//             zero-padded to a multiple of 4 entries (so one 128-bit load
//             covers 4 entries and never crosses into the next column).
//   idx[]     int32 row indices, same padding (pad index 0, pad value 0).
//   r32[m]    FP32 working residual: Ax - b (Lasso) or w (SVM).
//   r64[m]    FP64 residual of the last refresh.
//   rhs64[]   FP64 b (m entries, Lasso) or y (n entries, SVM).
//   col_sq[n] FP64 ||a_j||^2.
//   active[n] q-shrinking active set (int32 coordinate list).
//   r_ref[m]  FP64 residual of the last full evaluation (screened evaluations
//             bound the inactive columns by their distance from it).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/acdc_gpu.h"
#include "acdc_philox.h"

#define ACDC_FULL_MASK 0xffffffffu

// Slots of the per-problem counter block (unsigned long long).
enum {
  CNT_WORK = 0,        // per-launch work counter of the update kernel
  CNT_UPDATES = 1,
  CNT_NONZERO = 2,
  CNT_NNZ_READ = 3,
  CNT_NNZ_SCATTERED = 4,
  CNT_ACTIVE = 5,      // active-set length written by the gap kernel
  CNT_STATUS = 6,      // device-side error flags (DEV_ERR_*)
  CNT_K_BASE = 7,      // sampler counter of the next update (graph-friendly)
  CNT_GMAX_BITS = 8,   // max |a_j^T r| as FP64 bits (non-negative, so integer max works)
  CNT_OMEGA_ACTIVE = 9,// max entries per residual row over the active columns
  CNT_NLONG = 10,      // number of columns with more than 32 entries
  CNT_COLSQ_BITS = 11, // max ||a_j||^2 as FP64 bits
  CNT_HOT = 12,        // hot-set length
  CNT_OMEGA_HOT = 13,  // max entries per residual row over the hot columns
  CNT_MB_COUNTER = 14, // sampler counter of the synchronous mini-batch draws
  CNT_SLOTS = 16
};

enum { DEV_ERR_BAD_INDEX = 1, DEV_ERR_BAD_LAYOUT = 2, DEV_ERR_BAD_STATE = 4 };

// Fixed grid for the reductions, so partial sums are combined in a fixed order.
#define ACDC_RED_BLOCKS 1216
#define ACDC_RED_THREADS 256
#define ACDC_NPART 10  // partial slots per block
// Partial slots: 0 sum r^2, 1 sum b r, 2 sum |x|, 3 max |a_j^T r| (short columns;
// screened: active columns), 4 support, 5 max |a_j^T r| (long columns), 6 sum
// (r - r_ref)^2 (screened), 7 and 8 max |a_j^T r| over the columns left out of
// the active set (short, long), 9 max KKT violation over the active set.  SVM:
// 2 sum alpha, 3 sum hinge, 4 support, 5 correct signs.

// Parameters of one launch of the update kernel.
struct UpdateParams {
  int4* meta;
  const float* vals;
  const int32_t* idx;
  float* r;
  const int32_t* active;
  unsigned long long* counters;
  double* x64;          // FP64 coordinates (polish mode)
  double* r64;          // FP64 residual (polish mode)
  float* x32;           // FP32 coordinates
  int64_t n;
  uint64_t count;       // updates in this launch
  uint64_t seed;
  double lambda_d;      // Lasso: lambda; SVM: lambda * n
  double inv_lambda_n_d;// SVM scatter factor 1/(lambda n)
  double li_scale;      // multiplies the stored Li (1 unless beta changes)
  uint32_t shrink_q32;  // probability of an active-set draw, scaled by 2^32 (0 = off)
  uint32_t hot_q32 = 0;         // probability of a hot-set draw (part of shrink_q32)
  const int32_t* hot = nullptr;  // hot list (length in counters[CNT_HOT])
  double li_scale_hot = 1.0;     // step scale of hot-set draws
  int32_t n_warps;      // tau
  int32_t loss;
  int32_t fp64;         // 1: x and r in FP64 (x64, r64)
  uint64_t k_base;      // sampler counter of the launch's first update (batched launches)
  // Lanes per update: 8 or 32 select the grouped kernel (32 / lanes updates
  // per warp, register prefetch); anything else the one-warp ring kernel.
  int32_t lanes = 0;
  int32_t sm_count = 0;  // SMs of the device (the grouped kernel spreads its warps over them)
};

// Parameters of the evaluation kernels.
struct EvalParams {
  int4* meta;
  const float* vals;
  const int32_t* idx;
  float* r32;
  double* r64;
  const double* rhs64;
  int32_t* active;
  unsigned long long* counters;
  double* part;         // ACDC_RED_BLOCKS * ACDC_NPART
  double* eval_out;     // 16 doubles
  double* x64;          // FP64 coordinates when in polish mode, else nullptr (x in x32)
  float* x32;           // FP32 coordinates
  const int32_t* long_cols;  // columns with more than 32 entries
  int64_t n_long;
  int64_t m, n;
  double lambda;
  double shrink_thresh; // Lasso: (1-eps) lambda
  int32_t loss;
  // Lasso with an active set: a full evaluation copies r64 into r_ref and
  // reports the largest |a_j^T r| outside the active set (eval_out[10]); a
  // screened one (screened = 1) gathers only the active columns and bounds
  // the rest by eval_out[10] + col_norm_max ||r64 - r_ref|| (eval_out[11]).
  double* r_ref = nullptr;
  double col_norm_max = 0;
  int32_t screened = 0;
  // Active-set KKT violations (Lasso with an active set): the active pass writes
  // viol[t] for active[t] and the block maxima (slot 9); the hot-set kernels
  // list the columns above hot_frac times the maximum and their row neighbours.
  float* viol = nullptr;
  int32_t* hot = nullptr;
  uint8_t* row_flag = nullptr;  // m bytes, zero between evaluations
  int32_t* rowcnt = nullptr;
  double hot_frac = 0;
  // Logistic loss: sigma(r_i) per row, written by the refresh pass for the
  // column pass of the duality gap.
  double* roww = nullptr;
};

// ---- batched solves: many problems ("slots") served by one launch per kernel ----

// Control state of one slot, owned by the device between rounds.
struct SlotCtl {
  int32_t live;          // 1 while the slot still has lambdas to solve
  int32_t k;             // index of the current lambda on the path
  int32_t path_len;
  int32_t to_fp64;       // set by the control kernel for its own block
  uint64_t updates_here; // updates spent on the current lambda
  uint64_t max_updates;  // per-lambda budget
  uint64_t round_updates;// updates per round
  double gap_target;     // relative gap per lambda
  double polish_rel_gap;
  const double* lambdas; // path_len values
  double* results;       // path_len rows of kBatchResultLen doubles
  // q-shrinking (Lasso): from the second round of each lambda, q of the draws
  // come from the active set the round's gap pass built, with the step scale of
  // beta_A = 1 + (omega_A-1)(q tau-1)/(|A|-1) (omega_A counted over the active
  // columns each round), and a round is active_passes |A|/q updates.
  int32_t shrink;
  int32_t active_passes;
  int32_t shrink_next;   // 1 when the next round may draw from the active set
  uint32_t q32;
  double q;
  double omega;
  double beta;
  // A stall rule like the single-problem solve's AUTO precision: the best
  // relative gap of the current lambda and the updates spent when it last
  // halved; a slot whose gap (below 1e-4) has not halved over stall_updates
  // switches to FP64.
  double best_gap;
  uint64_t gain_at;
  uint64_t stall_updates;
};

// Row of a per-lambda result: eval_out[0..9], lambda, converged, epochs, tau.
#define ACDC_BATCH_RESULT_LEN 14

// Device view of a batch: per-slot parameters and block -> slot maps.
struct BatchDev {
  UpdateParams* up;
  EvalParams* ep;
  SlotCtl* ctl;
  const int32_t* ublk_slot;   // update grid: slot of each block
  const int32_t* ublk_first;  // first update block of each slot
  const int32_t* eblk_slot;   // evaluation grid: slot of each block
  const int32_t* eblk_first;  // first evaluation block of each slot
  const int32_t* eblk_count;  // evaluation blocks of each slot
  int32_t* live_count;        // slots still running
  int32_t n_slots;
};

struct DevProblem {
  int64_t m = 0, n = 0, nnz = 0, nnz_pad = 0;
  int4* meta = nullptr;
  float* x32 = nullptr;     // n FP32 coordinates
  float* vals = nullptr;
  int32_t* idx = nullptr;
  float* r32 = nullptr;
  double* r64 = nullptr;
  double* rhs64 = nullptr;
  double* col_sq = nullptr;
  int32_t* active = nullptr;
  double* x64 = nullptr;    // n doubles: coordinates in polish mode
  int32_t* rowcnt = nullptr;// m ints: per-row counts of active columns
  int32_t* long_cols = nullptr;  // columns with more than 32 entries (n_long of them)
  int64_t n_long = 0;
  double* xbuf = nullptr;   // n doubles: staging for x up/downloads
  double* r_ref = nullptr;  // m doubles: residual of the last full evaluation (Lasso)
  float* viol = nullptr;    // n floats: KKT violation of active[t] (Lasso)
  int32_t* hot = nullptr;   // n ints: hot list (Lasso)
  uint8_t* row_flag = nullptr;  // m bytes: rows of the hot columns (Lasso)
  // synchronous mini-batch (SVM dual): one epoch of draws, the step's deltas,
  // the n-bit draw marks (allocated on first use)
  int32_t* mb_draws = nullptr;
  double* mb_delta = nullptr;
  uint32_t* mb_mark = nullptr;
  double* part = nullptr;
  double* eval_out = nullptr;
  unsigned long long* counters = nullptr;
  int64_t bytes = 0;
};

struct acdc_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  // Second stream for the server's admissions (created by the first server):
  // problems are created on it while rounds run on `stream`.
  cudaStream_t admit_stream = nullptr;
  cudaMemPool_t pool = nullptr;  // device memory of the context's problems and tables
  // Pinned host slots (16 doubles of evaluation results + CNT_SLOTS counters
  // each) handed to problems: cut from blocks allocated once, so creating and
  // destroying a problem makes no pinned allocation (cudaFreeHost would wait
  // for the device).
  std::vector<double*> host_free;
  std::vector<void*> host_blocks;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::string last_error;
  int64_t live_problems = 0;  // problems (and servers) created on this context
  // tau chosen by the measured autotuner per size class, and its probe count
  std::map<uint64_t, int> tau_cache;
  int64_t tune_probes = 0;
};

struct acdc_problem {
  acdc_ctx* ctx = nullptr;
  int32_t loss = 0;
  DevProblem d;
  acdc_settings s;
  double lambda = 0;
  double beta = 1;
  int64_t omega = 1;
  uint64_t k_next = 0;      // sampler counter of the next update
  // synchronous mini-batch: updates made in that mode and the tau its buffers
  // were sized for (the sampler counter itself lives in counters[CNT_MB_COUNTER])
  uint64_t mb_updates = 0;
  int32_t mb_tau = 0;
  // one mini-batch epoch as a CUDA graph, with the precision, lambda and seed
  // it was captured for
  cudaGraphExec_t mb_graph = nullptr;
  bool mb_graph_fp64 = false;
  double mb_graph_lambda = 0;
  uint64_t mb_graph_seed = 0;
  int64_t epochs_done = 0;  // epochs since the start (shrinking starts after a few)
  uint64_t updates_done = 0;
  bool active_valid = false;
  bool fp64_mode = false;   // x and r kept in FP64 (polish stage or precision FP64)
  // Step scale while sampling from the active set: beta / max(beta, beta_A) with
  // beta_A the ESO parameter of q*tau draws over the active columns.
  double li_scale_shrink = 1.0;
  int64_t omega_active = 1;
  // Screened evaluations: valid after a full evaluation that built the active
  // set; stale once the bound of the inactive columns reaches (1 - eps/2) lambda.
  bool screen_valid = false;
  double col_norm_max = 0;  // max ||a_j|| (from col_sq)
  // Hot set (built after each evaluation while shrinking, Lasso).
  int64_t hot_count = 0;
  double hot_q = 0;
  double li_scale_hot = 1.0;
  acdc_stats stats;
  double* h_eval = nullptr;               // pinned, 16 doubles
  unsigned long long* h_counters = nullptr;  // pinned, CNT_SLOTS
};

// ---- helpers shared by the translation units ----
// Device memory of a context: stream-ordered allocations on its stream from its
// own pool, which keeps freed blocks for reuse.  Once the pool has grown, an
// allocation or a free is neither a driver call nor a device-wide
// synchronisation (a cudaFree synchronises the device), which matters for the
// server, whose requests come and go while other solves run.
cudaError_t acdc_dev_alloc(acdc_ctx* ctx, void** p, size_t bytes);
void acdc_dev_free(acdc_ctx* ctx, void* p);
// A pinned host slot of kHostSlotDoubles doubles, and its return.
constexpr int kHostSlotDoubles = 16 + CNT_SLOTS;
cudaError_t acdc_host_slot_take(acdc_ctx* ctx, double** slot);
void acdc_host_slot_give(acdc_ctx* ctx, double* slot);
int acdc_set_error(acdc_ctx* ctx, int code, const std::string& msg);
// lambda and the like: false for zero, negatives, infinities and NaN.
inline bool positive_finite(double v) { return v > 0 && v <= 1.7976931348623157e308; }
// Name of the first field of s outside its range, or nullptr when every one is valid.
const char* settings_fault(const acdc_settings* s);
int acdc_cuda_error(acdc_ctx* ctx, cudaError_t e, const char* what);

// A named range on a profiler's timeline for the scope it lives in (NVTX 3,
// header-only: a no-op unless a tool is attached).  ncu can select the kernels
// of one range, e.g. --nvtx --nvtx-include "acdc_evaluate/".
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

#define ACDC_CK(ctx, call)                                             \
  do {                                                                 \
    cudaError_t _e = (call);                                           \
    if (_e != cudaSuccess) return acdc_cuda_error((ctx), _e, #call);   \
  } while (0)

// ---- kernel launchers (kernels_*.cu) ----
int64_t layout_scan_tiles(int64_t n);
cudaError_t launch_layout_scan(const int64_t* col_ptr, int64_t n, int64_t* scratch,
                               unsigned long long* counters, cudaStream_t st);
cudaError_t launch_layout_fill(const int64_t* col_ptr, const int32_t* row_idx,
                               const double* vals64, int64_t m, int64_t n, int64_t* scratch,
                               DevProblem& d, int32_t loss, cudaStream_t st);
cudaError_t launch_row_counts(const int32_t* idx, int64_t nnz, int32_t* counts, int64_t m,
                              unsigned long long* counters, cudaStream_t st);
cudaError_t launch_max_i32(const int32_t* v, int64_t len, unsigned long long* out_slot,
                           cudaStream_t st);
cudaError_t launch_widen_i32(const int32_t* src, int64_t* dst, int64_t len, cudaStream_t st);
cudaError_t launch_set_li(const DevProblem& d, int32_t loss, double beta, double lambda,
                          cudaStream_t st);
// x: host-order doubles in d.xbuf <-> x32 (and FP64 x64 when fp64).
cudaError_t launch_set_x(const DevProblem& d, bool fp64, cudaStream_t st);
cudaError_t launch_get_x(const DevProblem& d, bool fp64, cudaStream_t st);
// Polish-mode transitions: x64 = (double) meta.w, or meta.w = (float) x64.
cudaError_t launch_x32_to_x64(const DevProblem& d, cudaStream_t st);
cudaError_t launch_x64_to_x32(const DevProblem& d, cudaStream_t st);
cudaError_t launch_update(const UpdateParams& p, uint64_t k_base, int warps_per_block,
                          cudaStream_t st);
cudaError_t launch_refresh(const EvalParams& p, cudaStream_t st);
// Lists the columns with more than 32 entries into list; count (device) gets their number.
cudaError_t launch_list_long(const DevProblem& d, int32_t* list, unsigned long long* count,
                             cudaStream_t st);
// omega over the active list (counters[CNT_OMEGA_ACTIVE]); rowcnt holds m ints.
cudaError_t launch_active_omega(const EvalParams& p, int32_t* rowcnt, cudaStream_t st);
cudaError_t launch_gap(const EvalParams& p, cudaStream_t st);
// Test-set 0-1 accuracy (count of positive margins into *good).
cudaError_t launch_test_accuracy(int64_t n_test, const int64_t* row_ptr, const int32_t* col_idx,
                                 const double* vals, const double* labels, const double* w64,
                                 const float* w32, int64_t w_len, unsigned long long* good,
                                 cudaStream_t st);
// Hot list from the violations of the last evaluation; zeroes CNT_HOT first.
cudaError_t launch_hot_set(const EvalParams& p, cudaStream_t st);
// Compressed rows (m x n, row_ptr on the device) -> compressed columns with
// the entries of each column in row order (transpose.cu).  col is checked
// (an index outside [0, n) sets DEV_ERR_BAD_INDEX in *status) and, like val,
// overwritten; scratch holds rows_to_columns_scratch_bytes bytes.
int64_t rows_to_columns_scratch_bytes(int64_t m, int64_t n, int64_t nnz);
cudaError_t launch_rows_to_columns(const int64_t* row_ptr, int32_t* col, double* val, int64_t m,
                                   int64_t n, int64_t nnz, char* scratch, int64_t* col_ptr,
                                   int32_t* rows_out, double* vals_out,
                                   unsigned long long* status, cudaStream_t st);
// Synchronous mini-batch SDCA (hinge dual): `steps` steps of tau distinct
// draws from the sampler stream at *counter into S (steps x tau), with the n-bit
// scratch `mark` clear on entry and exit; and one step: deltas from the same w
// into delta (tau values of the update precision), then applied.
cudaError_t launch_tau_nice(uint64_t seed, int64_t n, int32_t tau, int32_t steps,
                            unsigned long long* counter, int32_t* S, uint32_t* mark,
                            cudaStream_t st);
cudaError_t launch_minibatch_step(const UpdateParams& p, const int32_t* S, int32_t tau, void* delta,
                                  cudaStream_t st);
cudaError_t launch_debug_sample(uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                                int64_t* out, cudaStream_t st);
// Batched round: update, refresh, gap and control kernels over every live slot.
cudaError_t launch_batch_update(const BatchDev& b, int update_blocks, cudaStream_t st);
cudaError_t launch_batch_eval(const BatchDev& b, int eval_blocks, cudaStream_t st);
// One-time kernel attributes (shared-memory carveout), set at context creation.
cudaError_t update_kernels_init();
