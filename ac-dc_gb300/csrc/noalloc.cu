// acdc_debug_sample_noalloc: the sampler diagnostic of acdc_debug_sample
// without any allocation.  acdc_debug_sample takes its device output buffer
// from the context's memory pool on every call; this variant writes the draws
// into a fixed device array of this file and copies them out of it.
//
// Who needs it: a caller that must not allocate device memory while it runs.
// One example is a process whose device memory the server's admission budget
// has already handed to resident problems: any new allocation may fail there,
// or grow the pool past the budget.  Another is a caller checking the sampler
// while solves run, which wants no allocation call on their stream (growing
// the pool is a driver call).
//
// Scratch: ACDC_NOALLOC_MAX_SAMPLES int64 draws (512 KiB) and one status word,
// both file-scope __device__ arrays of this module.  Every call makes the
// context's device current and restores the caller's device before it
// returns.  The device addresses of the arrays are looked up once per device
// with cudaGetSymbolAddress, with that device current, by the first call on
// the device; the lookup may load the module, so
// the first call on a device should come before any stream capture.  The status
// word must start at zero and is cleared by every call.  There is one scratch
// array per device, so calls that overlap on one device (two host threads, or
// two contexts on the same device) race on it and must be serialised by the
// caller.
#include <cstring>
#include <mutex>

#include "acdc_internal.cuh"

namespace {

constexpr int kMaxDevices = 64;

static __device__ __align__(256) int64_t g_sample_scratch[ACDC_NOALLOC_MAX_SAMPLES];
static __device__ __align__(256) unsigned long long g_sample_status;

struct ScratchAddr {
  int64_t* draws = nullptr;
  unsigned long long* status = nullptr;
};

std::mutex g_setup_mu;
ScratchAddr g_addr[kMaxDevices];

// Makes dev current for the scope and gives the caller's thread its previous
// device back on every return path.
struct CurrentDevice {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit CurrentDevice(int dev) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess) err = cudaSetDevice(dev);
  }
  ~CurrentDevice() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  CurrentDevice(const CurrentDevice&) = delete;
  CurrentDevice& operator=(const CurrentDevice&) = delete;
};

// The same draw as k_debug_sample; a draw outside [0, n) (impossible for the
// 64x64 high product, checked all the same) sets bit 0 of the status word.
__global__ void k_debug_sample_fixed(uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                                     int64_t* out, unsigned long long* status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t k = k0 + i;
    acdc_u32x4 o = acdc_philox4x32_10((uint32_t)k, (uint32_t)(k >> 32), ACDC_STREAM_SAMPLER, 0u,
                                      (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t u = ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
    const int64_t j = (int64_t)__umul64hi(u, (uint64_t)n);
    if (j < 0 || j >= n) atomicOr(status, 1ull);
    out[i] = j;
  }
}

// Device addresses of the scratch for ctx's device (looked up on first use);
// the caller has made ctx's device current.
int scratch_for(acdc_ctx* ctx, ScratchAddr* out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  ScratchAddr& a = g_addr[ctx->device];
  if (!a.draws) {
    void* draws = nullptr;
    void* status = nullptr;
    ACDC_CK(ctx, cudaGetSymbolAddress(&draws, g_sample_scratch));
    ACDC_CK(ctx, cudaGetSymbolAddress(&status, g_sample_status));
    a.draws = static_cast<int64_t*>(draws);
    a.status = static_cast<unsigned long long*>(status);
  }
  *out = a;
  return ACDC_OK;
}

}  // namespace

extern "C" int acdc_debug_sample_noalloc(acdc_ctx* ctx, uint64_t seed, uint64_t k0,
                                         uint64_t count, int64_t n, int64_t* out) {
  if (!ctx || (count > 0 && !out) || n <= 0) return ACDC_EINVAL;
  if (count > (uint64_t)ACDC_NOALLOC_MAX_SAMPLES)
    return acdc_set_error(ctx, ACDC_EINVAL, "count exceeds ACDC_NOALLOC_MAX_SAMPLES");
  if (ctx->device < 0 || ctx->device >= kMaxDevices)
    return acdc_set_error(ctx, ACDC_EINVAL, "device index out of range for the fixed scratch");
  // Every call runs on the context's device, whatever the calling thread has
  // current, and leaves the thread's current device as it found it.
  CurrentDevice on(ctx->device);
  if (on.err != cudaSuccess) return acdc_cuda_error(ctx, on.err, "cudaSetDevice");
  ScratchAddr a;
  int rc = scratch_for(ctx, &a);
  if (rc != ACDC_OK) return rc;
  if (count == 0) return ACDC_OK;
  cudaStream_t st = ctx->stream;
  ACDC_CK(ctx, cudaMemsetAsync(a.status, 0, sizeof(unsigned long long), st));
  const uint64_t blocks = (count + 255) / 256 < 256 ? (count + 255) / 256 : 256;
  k_debug_sample_fixed<<<(unsigned)blocks, 256, 0, st>>>(seed, k0, count, n, a.draws, a.status);
  ACDC_CK(ctx, cudaGetLastError());
  unsigned long long status = 0;
  ACDC_CK(ctx, cudaMemcpyAsync(out, a.draws, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, st));
  ACDC_CK(ctx, cudaMemcpyAsync(&status, a.status, sizeof(status), cudaMemcpyDeviceToHost, st));
  ACDC_CK(ctx, cudaStreamSynchronize(st));
  if (status != 0) return acdc_set_error(ctx, ACDC_EDEVICE, "sampler draw outside [0, n)");
  return ACDC_OK;
}
