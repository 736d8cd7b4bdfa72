// Host side of var_cvar (src/lib.rs:505-520, src/risk/var_cvar.rs:7-43):
// argument checks with the reference's messages, the device radix select of
// risk.cu, and the VaR / CVaR values from its counts.
#include <cmath>
#include <cstring>

#include "host_common.h"
#include "risk_kernels.h"

using namespace stocha;

namespace {

double key_to_loss(uint64_t key) {  // inverse of risk.cu's loss_key
  const uint64_t b = (key >> 63) ? (key & ~0x8000000000000000ull) : ~key;
  double v;
  std::memcpy(&v, &b, 8);
  return v;
}

int check_args(uint64_t n, double confidence) {
  if (!(confidence > 0.0 && confidence < 1.0)) return set_error(STOCHA_ERR_VALUE, "confidence must be in (0, 1)");
  if (n == 0) return set_error(STOCHA_ERR_VALUE, "returns must not be empty");
  return STOCHA_OK;
}

// returns: device pointer to n returns (already checked: n > 0, confidence).
int var_cvar_dev(stocha_ctx* c, const double* returns, uint64_t n, double confidence, double* out2) {
  // var_cvar.rs:24-26: rank of the VaR loss in ascending order
  uint64_t idx = (uint64_t)std::ceil(confidence * (double)n);
  if (idx > n - 1) idx = n - 1;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const uint64_t want = (n + 255) / 256;
  const int grid = (int)(want < (uint64_t)sms * 8 ? (want ? want : 1) : (uint64_t)sms * 8);
  int rc;
  // scratch: [state 64 B | hist 2 KB | flag] in `starts`, partials in `partials`, total in `small`
  if ((rc = ensure_buf(c, c->starts, 64 + 256 * 8 + 64))) return rc;
  if ((rc = ensure_buf(c, c->partials, (size_t)grid * 2 * sizeof(double)))) return rc;
  if ((rc = ensure_buf(c, c->small, 64 * sizeof(double)))) return rc;
  char* base = (char*)c->starts.ptr;
  SelectState* state = (SelectState*)base;
  unsigned long long* hist = (unsigned long long*)(base + 64);
  unsigned* bad = (unsigned*)(base + 64 + 256 * 8);
  double* part = (double*)c->partials.ptr;
  double* total = (double*)c->small.ptr;
  SelectState init;
  std::memset(&init, 0, sizeof init);
  init.rank = idx;
  std::memcpy(c->h_small, &init, sizeof init);  // pinned staging
  if ((rc = begin_call(c))) return rc;
  STOCHA_CUDA(cudaMemcpyAsync(state, c->h_small, sizeof init, cudaMemcpyHostToDevice, c->stream));
  STOCHA_CUDA(cudaMemsetAsync(hist, 0, 256 * 8 + 64, c->stream));
  launch_select(returns, n, state, hist, bad, grid, c->stream);
  launch_tail_sum(returns, n, state, part, grid, c->stream);
  launch_reduce_partials(part, grid, 2, total, c->stream);
  STOCHA_CUDA(cudaGetLastError());
  double* h = c->h_small + 16;  // after the staged init state
  STOCHA_CUDA(cudaMemcpyAsync(h, state, sizeof(SelectState), cudaMemcpyDeviceToHost, c->stream));
  STOCHA_CUDA(cudaMemcpyAsync(h + 8, total, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  STOCHA_CUDA(cudaMemcpyAsync(h + 9, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  if ((rc = finish_call(c))) return rc;
  unsigned flag;
  std::memcpy(&flag, h + 9, sizeof flag);
  if (flag) return set_error(STOCHA_ERR_VALUE, "returns must not contain NaN or Inf");  // var_cvar.rs:14-16
  SelectState fin;
  std::memcpy(&fin, h, sizeof fin);
  const double var = key_to_loss(fin.prefix);
  // the sorted tail losses[idx..]: every larger loss, and the copies of the
  // VaR loss at positions >= idx (var_cvar.rs:36-42)
  const double copies = (double)(fin.less + fin.equal - idx);
  out2[0] = var;
  out2[1] = (h[8] + copies * var) / (double)(n - idx);
  return STOCHA_OK;
}

}  // namespace

extern "C" {

int stocha_var_cvar(stocha_ctx* ctx, const double* returns, uint64_t n, double confidence, double* out2) {
  STOCHA_RANGE("stocha_var_cvar");
  int rc = check_args(n, confidence);
  if (rc) return rc;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if ((rc = ensure_buf(ctx, ctx->aux, n * sizeof(double)))) return rc;
  STOCHA_CUDA(cudaMemcpyAsync(ctx->aux.ptr, returns, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  return var_cvar_dev(ctx, (const double*)ctx->aux.ptr, n, confidence, out2);
}

int stocha_var_cvar_device(stocha_ctx* ctx, const double* returns_dev, uint64_t n, double confidence, double* out2) {
  STOCHA_RANGE("stocha_var_cvar_device");
  int rc = check_args(n, confidence);
  if (rc) return rc;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  return var_cvar_dev(ctx, returns_dev, n, confidence, out2);
}

}  // extern "C"
