// Fused pricing for callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc at all: a host application that owns
// and budgets every byte of device memory itself (a risk engine embedding this
// library as a plugin), a latency-critical pricing service whose request path
// must never hit the allocator (cudaMalloc can synchronise the device and
// takes milliseconds), or a process whose memory pool is capped by its
// operator.  stocha_price_noalloc serves them: it runs the same fused pricing
// kernels as stocha_price_device, but its scratch memory (the per-block
// partial sums), the ziggurat tables and the device status word live in
// file-scope static __device__ arrays that are part of the loaded module, and
// the caller passes the output buffer and the stream.
//
// Limits.  The scratch array holds kNoAllocMaxBlocks partial records of up to
// kNoAllocMaxAssets assets (1 MiB).  Calls for more assets, or whose launch
// would write more records than that, are rejected with an error before
// anything is launched.
// Every GPU that loads the library keeps these arrays until the process exits.
//
// Set-up.  The first call on a device (with that device current) takes the
// arrays' device addresses with cudaGetSymbolAddress and copies the ziggurat
// tables in with cudaMemcpyToSymbol; make that first call before any stream
// capture on the device.
//
// Sharing.  All calls share the arrays, which keep the last call's contents.
// The status word is cleared at the start of every call and each launch
// overwrites exactly the partial records it reads, so no other clearing is
// needed; calls that overlap on the GPU (concurrent streams, threads) race on
// the arrays and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "host_common.h"

namespace stocha {
namespace {

constexpr int kNoAllocMaxAssets = 4;
constexpr int kNoAllocMaxBlocks = 16384;
constexpr size_t kNoAllocScratch = (size_t)kNoAllocMaxBlocks * 2 * kNoAllocMaxAssets;  // doubles (1 MiB)

static __device__ __align__(256) double g_scratch[kNoAllocScratch];
static __device__ __align__(256) ZigTables g_tables[1];
static __device__ __align__(256) unsigned g_status[64];
static __device__ __align__(256) unsigned long long g_work[32];  // work-queue counter of the FP32 forms

constexpr int kMaxDevices = 64;
struct DeviceArrays {
  bool ready = false;
  double* scratch = nullptr;
  ZigTables* tables = nullptr;
  unsigned* status = nullptr;
  unsigned long long* work = nullptr;
};
std::mutex g_setup_mu;
DeviceArrays g_dev[kMaxDevices];

// Once per device, with the device current.
int setup(int dev, DeviceArrays** out) {
  if (dev < 0 || dev >= kMaxDevices) return set_error(STOCHA_ERR_VALUE, "device index out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceArrays& d = g_dev[dev];
  if (!d.ready) {
    STOCHA_CUDA(cudaGetSymbolAddress((void**)&d.scratch, g_scratch));
    STOCHA_CUDA(cudaGetSymbolAddress((void**)&d.tables, g_tables));
    STOCHA_CUDA(cudaGetSymbolAddress((void**)&d.status, g_status));
    STOCHA_CUDA(cudaGetSymbolAddress((void**)&d.work, g_work));
    ZigTables host;
    fill_zig_tables(&host);
    STOCHA_CUDA(cudaMemcpyToSymbol(g_tables, &host, sizeof host));
    d.ready = true;
  }
  *out = &d;
  return STOCHA_OK;
}

}  // namespace
}  // namespace stocha

using namespace stocha;

extern "C" int stocha_price_noalloc(const stocha_model* m, uint64_t seed, int32_t precision, int32_t payoff,
                                    double strike, double* sums_dev, void* stream) {
  if (payoff != STOCHA_PAYOFF_CALL && payoff != STOCHA_PAYOFF_PUT)
    return set_error(STOCHA_ERR_VALUE, "payoff must be call or put");
  if (precision != STOCHA_FP64 && precision != STOCHA_FP32)
    return set_error(STOCHA_ERR_VALUE, "precision must be STOCHA_FP64 or STOCHA_FP32");
  if (!sums_dev) return set_error(STOCHA_ERR_VALUE, "sums_dev must be a device buffer");
  PathLaunch L;
  uint64_t row_len = 0;
  u128 block = 0;
  int rc = prepare_model(m, &L, &row_len, &block);
  if (rc) return rc;
  const int na = m->kind == STOCHA_MODEL_MULTI_GBM ? m->n_assets : 1;
  if (na > kNoAllocMaxAssets)
    return set_error(STOCHA_ERR_VALUE, "stocha_price_noalloc prices at most " + std::to_string(kNoAllocMaxAssets) +
                                           " assets (its static scratch holds " + std::to_string(kNoAllocMaxBlocks) +
                                           " partial records of " + std::to_string(kNoAllocMaxAssets) + " assets)");
  int dev = 0;
  STOCHA_CUDA(cudaGetDevice(&dev));
  DeviceArrays* d = nullptr;
  if ((rc = setup(dev, &d))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  make_stream_spec((u128)seed, block, &L.ss);
  L.tabs = d->tables;
  L.err = d->status;
  L.partials = d->scratch;
  if (precision == STOCHA_FP32) {
    // the FP32 forms' work queue: one record per batch, at most the scratch's
    // kNoAllocMaxBlocks records (batches of 32 rows, more for large counts)
    const uint64_t per_lane = (L.rows + 32ull * kNoAllocMaxBlocks - 1) / (32ull * kNoAllocMaxBlocks);
    L.batch_rows = (uint32_t)(32 * (per_lane ? per_lane : 1));
    L.work = d->work;
  }
  L.strike = strike;
  L.payoff = payoff;
  // the launchers compute their record count first and launch nothing when it
  // exceeds the static scratch, so no launch can write past the array
  L.max_records = kNoAllocMaxBlocks;
  fill_f32_constants(&L);
  STOCHA_CUDA(cudaMemsetAsync(d->status, 0, sizeof(unsigned), st));
  if (L.rows == 0) {
    STOCHA_CUDA(cudaMemsetAsync(sums_dev, 0, 2 * na * sizeof(double), st));
  } else {
    const int nb = precision == STOCHA_FP32 ? launch_paths_f32(L, st) : launch_paths_f64(L, st);
    if (nb == kRecordsExceeded)
      return set_error(STOCHA_ERR_VALUE, "stocha_price_noalloc: the launch would need more than " +
                                             std::to_string(kNoAllocMaxBlocks) +
                                             " partial records (the static scratch's size)");
    if (nb < 0) return cuda_error(cudaGetLastError(), "pricing kernel launch");
    launch_reduce_partials(d->scratch, nb, 2 * na, sums_dev, st);
  }
  STOCHA_CUDA(cudaGetLastError());
  // the status word comes back on the caller's stream: no wait on the legacy
  // default stream (and so on the application's other blocking streams)
  unsigned status = 0;
  STOCHA_CUDA(cudaMemcpyAsync(&status, d->status, sizeof status, cudaMemcpyDeviceToHost, st));
  STOCHA_CUDA(cudaStreamSynchronize(st));
  if (status) return set_error(STOCHA_ERR_DEVICE, "device check failed (sampler iteration cap)");
  return STOCHA_OK;
}
