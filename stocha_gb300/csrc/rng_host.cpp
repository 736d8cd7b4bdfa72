// Host side of the RNG surface (src/lib.rs:74-184, src/prng/pcg64.rs): state
// bookkeeping, JSON state files, and the launches of rng.cu.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "host_common.h"
#include "copula_t_kernels.h"
#include "rng_kernels.h"

using namespace stocha;

namespace {

u128 rng_state(const stocha_rng* r) { return ((u128)r->state_hi << 64) | r->state_lo; }
u128 rng_inc(const stocha_rng* r) { return ((u128)r->inc_hi << 64) | r->inc_lo; }
void set_state(stocha_rng* r, u128 s) {
  r->state_lo = (uint64_t)s;
  r->state_hi = (uint64_t)(s >> 64);
}

PcgJump affine_jump(u128 inc, u128 delta) {
  u128 st = 0;
  // A*0 + C = C; A from advancing the state 1 by delta minus C.
  u128 one = 1;
  u128 c = st;
  pcg_advance(&c, inc, delta);  // c = C
  u128 a = one;
  pcg_advance(&a, inc, delta);  // a = A + C
  a -= c;
  PcgJump J;
  J.mul_lo = (uint64_t)a;
  J.mul_hi = (uint64_t)(a >> 64);
  J.add_lo = (uint64_t)c;
  J.add_hi = (uint64_t)(c >> 64);
  return J;
}

int device_count_threads(int device) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return sms * 1024;
}

// raw (kind 0) or uniform (kind 1) draws into host memory
int fill_raw(stocha_ctx* ctx, stocha_rng* r, uint64_t n, int kind, void* out) {
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  if (n == 0) return STOCHA_OK;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const uint64_t bytes = n * 8;
  if ((rc = ensure_buf(ctx, ctx->out, bytes))) return rc;
  uint64_t threads = (uint64_t)device_count_threads(ctx->device);
  if (threads > n) threads = n;
  StreamSpec ss;
  make_stream_spec_state(rng_state(r), rng_inc(r), 1, &ss);
  PcgJump stride = affine_jump(rng_inc(r), threads);
  if ((rc = begin_call(ctx))) return rc;
  launch_rng_raw(ss, stride, threads, n, kind, ctx->out.ptr, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  if ((rc = copy_to_host_populated(ctx->stream, out, ctx->out.ptr, bytes))) return rc;
  if ((rc = finish_call(ctx))) return rc;
  u128 s = rng_state(r);
  pcg_advance(&s, rng_inc(r), n);
  set_state(r, s);
  return STOCHA_OK;
}

// The next n values (kind 1: standard normal, 2: loc + scale z) of the stream
// at (state, inc) into ctx->out on the device, by the parallel parse of
// rng.cu; *final_pos receives the draws consumed.  ctx locked by the caller.
int normals_to_device(stocha_ctx* ctx, u128 state, u128 inc, uint64_t n, int kind, double loc, double scale,
                      uint64_t* final_pos_out) {
  const uint32_t C = kRngChunk;
  // expected 1.0296 draws per normal; generous margin, doubled on shortfall
  double need = (double)n * 1.04 + 16.0 * std::sqrt((double)n) + 2.0 * C;
  uint64_t nchunks = (uint64_t)(need / C) + 2;
  StreamSpec ss;
  make_stream_spec_state(state, inc, 1, &ss);
  int rc;
  for (int attempt = 0; attempt < 8; ++attempt) {
    const size_t off_counts = 0;
    const size_t off_exits = off_counts + nchunks * kRngEntries * 4;
    const size_t off_entry = off_exits + nchunks * kRngEntries * 4;
    const size_t off_cnt = off_entry + nchunks * 4;
    const size_t off_offset = ((off_cnt + nchunks * 4) + 7) & ~(size_t)7;
    const size_t off_total = off_offset + nchunks * 8;
    const size_t aux_bytes = off_total + 16;
    if ((rc = ensure_buf(ctx, ctx->aux, aux_bytes))) return rc;
    if ((rc = ensure_buf(ctx, ctx->out, n * 8))) return rc;
    char* aux = (char*)ctx->aux.ptr;
    uint32_t* counts = (uint32_t*)(aux + off_counts);
    uint32_t* exits = (uint32_t*)(aux + off_exits);
    uint32_t* entry = (uint32_t*)(aux + off_entry);
    uint32_t* cnt = (uint32_t*)(aux + off_cnt);
    uint64_t* offset = (uint64_t*)(aux + off_offset);
    uint64_t* total = (uint64_t*)(aux + off_total);
    uint64_t* final_pos = total + 1;
    if ((rc = begin_call(ctx))) return rc;
    launch_rng_parse(ss, ctx->d_tabs, nchunks, C, counts, exits, entry, cnt, offset, total, ctx->d_err, ctx->stream);
    STOCHA_CUDA(cudaGetLastError());
    STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, total, 8, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = finish_call(ctx))) return rc;
    uint64_t got;
    std::memcpy(&got, ctx->h_small, 8);
    if (got < n) {
      nchunks = nchunks * 3 / 2 + 2;
      continue;
    }
    if ((rc = begin_call(ctx))) return rc;
    launch_rng_emit(ss, ctx->d_tabs, nchunks, C, entry, cnt, offset, n, kind, loc, scale, (double*)ctx->out.ptr,
                    final_pos, ctx->d_err, ctx->stream);
    STOCHA_CUDA(cudaGetLastError());
    STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, final_pos, 8, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = finish_call(ctx))) return rc;
    std::memcpy(final_pos_out, ctx->h_small, 8);
    return STOCHA_OK;
  }
  return set_error(STOCHA_ERR_DEVICE, "normal stream parse did not cover the request");
}

int fill_normal(stocha_ctx* ctx, stocha_rng* r, uint64_t n, int kind, double loc, double scale, double* out) {
  int rc = resolve_ctx(&ctx);
  if (rc) return rc;
  if (n == 0) return STOCHA_OK;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  uint64_t fp = 0;
  if ((rc = normals_to_device(ctx, rng_state(r), rng_inc(r), n, kind, loc, scale, &fp))) return rc;
  if ((rc = copy_to_host_populated(ctx->stream, out, ctx->out.ptr, n * 8))) return rc;
  STOCHA_CUDA(cudaStreamSynchronize(ctx->stream));
  u128 s = rng_state(r);
  pcg_advance(&s, rng_inc(r), fp);
  set_state(r, s);
  return STOCHA_OK;
}

// gaussian.rs:21-47 checks and gaussian.rs:76-99 Cholesky, with the
// reference's messages; l receives the factor (dim x dim, row-major).
int copula_factor(const double* corr, size_t rows, size_t cols, std::vector<double>* l) {
  const size_t dim = rows;
  if (cols != dim) return set_error(STOCHA_ERR_VALUE, "correlation matrix must be square");
  for (size_t i = 0; i < dim; ++i) {
    if (std::fabs(corr[i * dim + i] - 1.0) > 1e-10)
      return set_error(STOCHA_ERR_VALUE, "correlation matrix diagonal element [" + std::to_string(i) + "][" +
                                             std::to_string(i) + "] must be 1.0, got " + rust_f64(corr[i * dim + i]));
    for (size_t j = i + 1; j < dim; ++j)
      if (std::fabs(corr[i * dim + j] - corr[j * dim + i]) > 1e-10)
        return set_error(STOCHA_ERR_VALUE, "correlation matrix is not symmetric: [" + std::to_string(i) + "," +
                                               std::to_string(j) + "]=" + rust_f64(corr[i * dim + j]) + " vs [" +
                                               std::to_string(j) + "," + std::to_string(i) +
                                               "]=" + rust_f64(corr[j * dim + i]));
  }
  l->assign(dim * dim, 0.0);
  for (size_t i = 0; i < dim; ++i)
    for (size_t j = 0; j <= i; ++j) {
      double sum = corr[i * dim + j];
      for (size_t k = 0; k < j; ++k) sum -= (*l)[i * dim + k] * (*l)[j * dim + k];
      if (i == j) {
        if (sum <= 0.0)
          return set_error(STOCHA_ERR_VALUE, "matrix is not positive-definite (diagonal element " +
                                                 std::to_string(i) + " = " + rust_f64(sum) + ")");
        (*l)[i * dim + j] = std::sqrt(sum);
      } else {
        (*l)[i * dim + j] = sum / (*l)[j * dim + j];
      }
    }
  return STOCHA_OK;
}

// ---- minimal JSON reader for the state files of pcg64.rs:10-20 ----------
struct Json {
  const char* p;
  const char* end;
  bool ok = true;

  void ws() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r')) ++p;
  }
  bool eat(char c) {
    ws();
    if (p < end && *p == c) {
      ++p;
      return true;
    }
    return false;
  }
  // value kinds: 0 other, 1 unsigned integer (fits u128), 2 object
  struct Val {
    int kind = 0;
    u128 u = 0;
    std::vector<std::pair<std::string, Val>> obj;
  };
  bool str(std::string* s) {
    ws();
    if (p >= end || *p != '"') return false;
    ++p;
    while (p < end && *p != '"') {
      if (*p == '\\') {
        ++p;
        if (p >= end) return false;
      }
      s->push_back(*p++);
    }
    if (p >= end) return false;
    ++p;
    return true;
  }
  bool value(Val* v, int depth) {
    ws();
    if (p >= end || depth > 32) return false;
    if (*p == '{') {
      ++p;
      v->kind = 2;
      if (eat('}')) return true;
      for (;;) {
        std::string k;
        if (!str(&k) || !eat(':')) return false;
        Val c;
        if (!value(&c, depth + 1)) return false;
        v->obj.emplace_back(k, c);
        if (eat(',')) continue;
        return eat('}');
      }
    }
    if (*p == '[') {
      ++p;
      if (eat(']')) return true;
      for (;;) {
        Val c;
        if (!value(&c, depth + 1)) return false;
        if (eat(',')) continue;
        return eat(']');
      }
    }
    if (*p == '"') {
      std::string s;
      return str(&s);
    }
    if (*p >= '0' && *p <= '9') {
      const char* q = p;
      u128 acc = 0;
      bool overflow = false;
      while (p < end && *p >= '0' && *p <= '9') {
        u128 nxt = acc * 10 + (u128)(*p - '0');
        if (nxt / 10 != acc) overflow = true;
        acc = nxt;
        ++p;
      }
      bool integral = !(p < end && (*p == '.' || *p == 'e' || *p == 'E'));
      while (p < end && (*p == '.' || *p == 'e' || *p == 'E' || *p == '+' || *p == '-' || (*p >= '0' && *p <= '9')))
        ++p;
      if (integral && !overflow && !(p - q > 1 && *q == '0')) {
        v->kind = 1;
        v->u = acc;
      }
      return true;
    }
    if (*p == '-') {
      ++p;
      while (p < end && (*p == '.' || *p == 'e' || *p == 'E' || *p == '+' || *p == '-' || (*p >= '0' && *p <= '9')))
        ++p;
      return true;
    }
    for (const char* lit : {"true", "false", "null"}) {
      size_t L = std::strlen(lit);
      if ((size_t)(end - p) >= L && std::strncmp(p, lit, L) == 0) {
        p += L;
        return true;
      }
    }
    return false;
  }
};

const Json::Val* field(const Json::Val& o, const char* k) {
  const Json::Val* hit = nullptr;
  for (auto& kv : o.obj)
    if (kv.first == k) hit = &kv.second;
  return hit;
}

}  // namespace

extern "C" {

int stocha_rng_uniform(stocha_ctx* ctx, stocha_rng* r, uint64_t size, double* out) {
  STOCHA_RANGE("stocha_rng_uniform");
  return fill_raw(ctx, r, size, 1, out);
}

int stocha_rng_raw_u64(stocha_ctx* ctx, stocha_rng* r, uint64_t size, uint64_t* out) {
  STOCHA_RANGE("stocha_rng_raw_u64");
  return fill_raw(ctx, r, size, 0, out);
}

int stocha_rng_standard_normal(stocha_ctx* ctx, stocha_rng* r, uint64_t size, double* out) {
  STOCHA_RANGE("stocha_rng_standard_normal");
  return fill_normal(ctx, r, size, 1, 0.0, 1.0, out);
}

int stocha_rng_normal(stocha_ctx* ctx, stocha_rng* r, uint64_t size, double loc, double scale, double* out) {
  STOCHA_RANGE("stocha_rng_normal");
  if (scale <= 0.0) return set_error(STOCHA_ERR_VALUE, "scale must be positive");  // lib.rs:137-141
  return fill_normal(ctx, r, size, 2, loc, scale, out);
}

// pcg64.rs:68-77: the full state {"version", "rng": {"state", "increment"},
// "seed"} restores the exact position; {"seed": N} restarts the stream.
int stocha_rng_from_state(const char* json, stocha_rng* out) {
  if (!json) return set_error(STOCHA_ERR_VALUE, "invalid state JSON");
  Json J{json, json + std::strlen(json)};
  Json::Val root;
  bool parsed = J.value(&root, 0);
  J.ws();
  if (!parsed || J.p != J.end) {
    size_t col = (size_t)(J.p - json) + 1;
    return set_error(STOCHA_ERR_VALUE, "invalid state JSON at line 1 column " + std::to_string(col));
  }
  if (root.kind == 2) {
    const Json::Val* ver = field(root, "version");
    const Json::Val* rng = field(root, "rng");
    const Json::Val* seed = field(root, "seed");
    if (ver && ver->kind == 1 && ver->u <= 255 && rng && rng->kind == 2 && seed && seed->kind == 1) {
      const Json::Val* st = field(*rng, "state");
      const Json::Val* inc = field(*rng, "increment");
      if (st && st->kind == 1 && inc && inc->kind == 1) {
        set_state(out, st->u);
        out->inc_lo = (uint64_t)inc->u;
        out->inc_hi = (uint64_t)(inc->u >> 64);
        out->seed_lo = (uint64_t)seed->u;
        out->seed_hi = (uint64_t)(seed->u >> 64);
        return STOCHA_OK;
      }
    }
    if (seed && seed->kind == 1) return stocha_rng_new((uint64_t)seed->u, (uint64_t)(seed->u >> 64), nullptr, out);
    return set_error(STOCHA_ERR_VALUE, "missing field `seed`");
  }
  return set_error(STOCHA_ERR_VALUE, "invalid type: expected struct SeedOnly");
}

int stocha_gaussian_copula(stocha_ctx* ctx, const double* corr, size_t rows, size_t cols, uint64_t n_samples,
                           uint64_t seed, double* out) {
  STOCHA_RANGE("stocha_gaussian_copula");
  std::vector<double> l;
  int rc = copula_factor(corr, rows, cols, &l);  // gaussian.rs:21-51
  if (rc) return rc;
  const size_t dim = rows;
  if (n_samples == 0 || dim == 0) return STOCHA_OK;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (n_samples > (SIZE_MAX / 8) / dim) return set_error(STOCHA_ERR_NOMEM, "output size overflows the address space");
  // one sequential stream Pcg64Dxsm::new(seed): sample i takes normals
  // i*dim .. i*dim+dim-1 (NormalSampler::sample_into, gaussian.rs:55-60)
  u128 st, inc;
  pcg_seed((u128)seed, &st, &inc);
  uint64_t fp = 0;
  const uint64_t nz = n_samples * dim;
  if ((rc = normals_to_device(ctx, st, inc, nz, 1, 0.0, 1.0, &fp))) return rc;
  if ((rc = ensure_buf(ctx, ctx->aux, nz * 8 + dim * dim * 8 + 256))) return rc;
  double* u = (double*)ctx->aux.ptr;
  double* dl = (double*)((char*)ctx->aux.ptr + ((nz * 8 + 255) & ~(size_t)255));
  if ((rc = begin_call(ctx))) return rc;
  STOCHA_CUDA(cudaMemcpyAsync(dl, l.data(), dim * dim * 8, cudaMemcpyHostToDevice, ctx->stream));
  launch_copula_gaussian((const double*)ctx->out.ptr, dl, n_samples, (int)dim, ctx->d_tabs,
                         1.0 / std::sqrt(2.0 * M_PI), u, ctx->stream);
  STOCHA_CUDA(cudaGetLastError());
  if ((rc = copy_to_host_populated(ctx->stream, out, u, nz * 8))) return rc;
  return finish_call(ctx);  // l outlives the copy (synchronous)
}

// Log-gamma by the Lanczos approximation, g = 7, nine coefficients
// (copula/student_t.rs:74-91), for the incomplete beta's log B(a, b).
static double lgamma_lanczos(double x) {
  static const double C[9] = {0.99999999999980993,  676.5203681218851,     -1259.1392167224028,
                              771.32342877765313,   -176.61502916214059,   12.507343278686905,
                              -0.13857109526572012, 9.9843695780195716e-6, 1.5056327351493116e-7};
  const double pi = 3.14159265358979323846;
  if (x < 0.5) return std::log(pi) - std::log(std::sin(pi * x)) - lgamma_lanczos(1.0 - x);
  x -= 1.0;
  double acc = C[0];
  for (int i = 1; i < 9; ++i) acc += C[i] / (x + (double)i);
  const double t = x + 7.0 + 0.5;
  return 0.5 * std::log(2.0 * pi) + (x + 0.5) * std::log(t) - t + std::log(acc);
}

int stocha_student_t_copula(stocha_ctx* ctx, const double* corr, size_t rows, size_t cols, double nu,
                            uint64_t n_samples, uint64_t seed, double* out) {
  STOCHA_RANGE("stocha_student_t_copula");
  if (nu <= 2.0) return set_error(STOCHA_ERR_VALUE, "nu must be > 2");  // lib.rs:570-572 (NaN passes, as there)
  std::vector<double> l;
  if (cols != rows) return set_error(STOCHA_ERR_VALUE, "correlation matrix must be square");  // student_t.rs:146-148
  // student_t.rs:149 factors the matrix without the diagonal / symmetry checks
  {
    const size_t dim = rows;
    l.assign(dim * dim, 0.0);
    for (size_t i = 0; i < dim; ++i)
      for (size_t j = 0; j <= i; ++j) {
        double sum = corr[i * dim + j];
        for (size_t k = 0; k < j; ++k) sum -= l[i * dim + k] * l[j * dim + k];
        if (i == j) {
          if (sum <= 0.0)
            return set_error(STOCHA_ERR_VALUE, "matrix is not positive-definite (diagonal element " +
                                                   std::to_string(i) + " = " + rust_f64(sum) + ")");
          l[i * dim + j] = std::sqrt(sum);
        } else {
          l[i * dim + j] = sum / l[j * dim + j];
        }
      }
  }
  const size_t dim = rows;
  if (n_samples == 0 || dim == 0) return STOCHA_OK;
  int rc;
  if ((rc = resolve_ctx(&ctx))) return rc;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (n_samples > (SIZE_MAX / 8) / (dim + 1)) return set_error(STOCHA_ERR_NOMEM, "output size overflows the address space");
  u128 st, inc;
  pcg_seed((u128)seed, &st, &inc);
  TParse a;
  std::memset(&a, 0, sizeof a);
  make_stream_spec_state(st, inc, 1, &a.ss);
  a.tabs = ctx->d_tabs;
  a.err = ctx->d_err;
  a.n = n_samples;
  a.C = 1024;
  a.dim = (int)dim;
  // A sample takes dim + 2 draws plus a few on rejections, so the true entry
  // of a chunk (the overshoot of the sample that straddles its start) lies
  // below dim + 8 except after 7 or more extra draws in that one sample; such
  // an entry is parsed where the stitch meets it.
  a.E = (int)std::min<size_t>(dim + 8, a.C);
  const double shape = nu / 2.0;  // student_t.rs:121-124, 102-103
  std::vector<double> cf_host(800);
  a.d = shape - 1.0 / 3.0;
  a.c = 1.0 / std::sqrt(9.0 * a.d);
  // ~2.1 draws for the chi-square and 1.03 per normal
  double need = (double)n_samples * (2.3 + 1.06 * (double)dim) + 8.0 * a.C;
  a.nchunks = (uint64_t)(need / a.C) + 2;
  for (int attempt = 0; attempt < 8; ++attempt) {
    const uint64_t nc = a.nchunks;
    const size_t o_exits = 0;
    const size_t o_counts = o_exits + nc * a.E * 8;
    const size_t o_entry = (o_counts + nc * a.E * 4 + 7) & ~(size_t)7;
    const size_t o_first = o_entry + nc * 8;
    const size_t o_status = o_first + nc * 8;
    a.G = 8;
    while (a.G * a.G < nc) a.G *= 2;
    a.ngroups = (nc + a.G - 1) / a.G;
    const size_t o_gexit = o_status + 64;
    const size_t o_gcount = o_gexit + a.ngroups * a.E * 8;
    const size_t o_gentry = o_gcount + a.ngroups * a.E * 8;
    const size_t o_gfirst = o_gentry + a.ngroups * 8;
    const size_t o_raw = (o_gfirst + a.ngroups * 8 + 255) & ~(size_t)255;
    const size_t o_l = (o_raw + n_samples * (dim + 1) * 8 + 255) & ~(size_t)255;
    const size_t o_cf = (o_l + dim * dim * 8 + 255) & ~(size_t)255;
    const size_t o_u = (o_cf + 800 * 8 + 255) & ~(size_t)255;
    const size_t bytes = o_u + n_samples * dim * 8;
    if ((rc = ensure_buf(ctx, ctx->aux, bytes))) return rc;
    char* base = (char*)ctx->aux.ptr;
    a.exits = (uint64_t*)(base + o_exits);
    a.counts = (uint32_t*)(base + o_counts);
    a.entry = (uint64_t*)(base + o_entry);
    a.first = (uint64_t*)(base + o_first);
    a.status = (uint64_t*)(base + o_status);
    a.gexit = (uint64_t*)(base + o_gexit);
    a.gcount = (uint64_t*)(base + o_gcount);
    a.gentry = (uint64_t*)(base + o_gentry);
    a.gfirst = (uint64_t*)(base + o_gfirst);
    a.raw = (double*)(base + o_raw);
    double* dl = (double*)(base + o_l);
    double* u = (double*)(base + o_u);
    if ((rc = begin_call(ctx))) return rc;
    launch_tparse(a, ctx->stream);
    launch_tstitch(a, ctx->stream);
    STOCHA_CUDA(cudaGetLastError());
    STOCHA_CUDA(cudaMemcpyAsync(ctx->h_small, a.status, 16, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = finish_call(ctx))) return rc;
    uint64_t covered;
    std::memcpy(&covered, ctx->h_small + 1, 8);
    if (covered < n_samples) {
      a.nchunks = a.nchunks * 3 / 2 + 2;
      continue;
    }
    if ((rc = begin_call(ctx))) return rc;
    launch_temit(a, a.status, ctx->stream);
    STOCHA_CUDA(cudaMemcpyAsync(dl, l.data(), dim * dim * 8, cudaMemcpyHostToDevice, ctx->stream));
    const double a2 = nu / 2.0;
    const double log_beta = lgamma_lanczos(a2) + lgamma_lanczos(0.5) - lgamma_lanczos(a2 + 0.5);
    // continued-fraction coefficients (student_t.rs:48,54) for (a2, 1/2) and (1/2, a2)
    for (int flip = 0; flip < 2; ++flip) {
      const double A = flip ? 0.5 : a2, B = flip ? a2 : 0.5;
      for (int m = 1; m <= 200; ++m) {
        const double mf = m, m2 = 2.0 * mf;
        cf_host[flip * 400 + 2 * (m - 1)] = mf * (B - mf) / ((A - 1.0 + m2) * (A + m2));
        cf_host[flip * 400 + 2 * (m - 1) + 1] = -(A + mf) * (A + B + mf) / ((A + m2) * (A + 1.0 + m2));
      }
    }
    double* dcf = (double*)(base + o_cf);
    STOCHA_CUDA(cudaMemcpyAsync(dcf, cf_host.data(), 800 * 8, cudaMemcpyHostToDevice, ctx->stream));
    launch_tcdf(a.raw, dl, n_samples, (int)dim, nu, log_beta, dcf, u, ctx->stream);
    STOCHA_CUDA(cudaGetLastError());
    if ((rc = copy_to_host_populated(ctx->stream, out, u, n_samples * dim * 8))) return rc;
    return finish_call(ctx);
  }
  return set_error(STOCHA_ERR_DEVICE, "sample stream parse did not cover the request");
}

}  // extern "C"
