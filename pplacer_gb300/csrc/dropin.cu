// Plain drop-in for pplacer_src/linear_c.c: one FP64 sm_103a kernel per
// external of pplacer_src/linear.ml:13-89.  Host buffers in and out; the
// device staging buffer and stream are created lazily on the first call (so a
// process may fork before its first call) and reused.
#include <math.h>
#include <stdarg.h>

#include <mutex>
#include <vector>

#include "pgb_common.cuh"

namespace pgb {

std::atomic<uint64_t> g_launches{0};
static thread_local std::string t_error;

void set_error(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_error = buf;
}

void code_lv(int K, int c, double *lv) {
  if (K == 4) {
    static const int bits[kNucCodes] = {1, 2, 4, 8, 5, 10, 3, 12, 6, 9, 11, 14, 7, 13, 15, 15, 15, 15};
    for (int k = 0; k < 4; k++) lv[k] = (bits[c] >> k) & 1 ? 1.0 : 0.0;
    return;
  }
  for (int k = 0; k < K; k++) lv[k] = 0.0;
  if (c < 20) { lv[c] = 1.0; return; }
  // B = D|N, J = I|L, Z = E|Q, X - ? = any (prot_models.ml:20-43)
  switch (c) {
    case 20: lv[3] = lv[2] = 1.0; break;
    case 21: lv[9] = lv[10] = 1.0; break;
    case 22: lv[6] = lv[5] = 1.0; break;
    default: for (int k = 0; k < K; k++) lv[k] = 1.0;
  }
}

namespace {

struct DropinCtx {
  std::mutex mu;
  cudaStream_t st = nullptr;
  char *buf = nullptr;
  size_t cap = 0;
};
DropinCtx g_ctx;

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 1024;

// Staging: carve 256-byte aligned regions out of one grow-only device buffer.
struct Stage {
  size_t off = 0;
  template <class T>
  size_t take(size_t n) {
    size_t o = off;
    off += (n * sizeof(T) + 255) & ~(size_t)255;
    return o;
  }
};

pgb_status ensure(size_t bytes) {
  if (!g_ctx.st) PGB_CUDA(cudaStreamCreateWithFlags(&g_ctx.st, cudaStreamNonBlocking));
  if (bytes > g_ctx.cap) {
    if (g_ctx.buf) PGB_CUDA(cudaFree(g_ctx.buf));
    g_ctx.buf = nullptr;
    size_t cap = bytes + (bytes >> 2) + 4096;
    PGB_CUDA(cudaMalloc(&g_ctx.buf, cap));
    g_ctx.cap = cap;
  }
  return PGB_OK;
}

template <class T>
T *at(size_t off) { return reinterpret_cast<T *>(g_ctx.buf + off); }

pgb_status h2d(size_t off, const void *src, size_t bytes) {
  if (bytes) PGB_CUDA(cudaMemcpyAsync(g_ctx.buf + off, src, bytes, cudaMemcpyHostToDevice, g_ctx.st));
  return PGB_OK;
}
pgb_status d2h(void *dst, size_t off, size_t bytes) {
  if (bytes) PGB_CUDA(cudaMemcpyAsync(dst, g_ctx.buf + off, bytes, cudaMemcpyDeviceToHost, g_ctx.st));
  return PGB_OK;
}
pgb_status finish() {
  PGB_CUDA(cudaStreamSynchronize(g_ctx.st));
  return PGB_OK;
}

int blocks_for(long n) {
  long b = (n + kThreads - 1) / kThreads;
  return (int)(b < 1 ? 1 : (b > kMaxBlocks ? kMaxBlocks : b));
}

// ---- kernels --------------------------------------------------------------

// dst[s,i] = sum_j a[i,j] b[s,j]  (gemmish_c, linear_c.c:29-90)
__global__ void k_gemmish(double *dst, const double *__restrict__ a, const double *__restrict__ b, long n_sites,
                          int K) {
  long n = n_sites * K;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    long s = t / K;
    int i = (int)(t - s * K);
    const double *ai = a + (long)i * K, *bs = b + s * K;
    double acc = 0;
    for (int j = 0; j < K; j++) acc += ai[j] * bs[j];
    dst[t] = acc;
  }
}

// dst[i,j] = sum_k lambda[k] u[i,k] uit[j,k]  (dediagonalize, linear_c.c:92-146)
__global__ void k_dediag(double *dst, const double *__restrict__ u, const double *__restrict__ lambda,
                         const double *__restrict__ uit, int n) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  int i = t / n, j = t - i * n;
  double acc = 0;
  for (int k = 0; k < n; k++) acc += lambda[k] * u[i * n + k] * uit[j * n + k];
  dst[t] = acc;
}

// Per-site log reductions of linear_c.c.  mode:
//   0 mat_log_like3 (statd x y z)        1 ten_log_like3 (writes util)
//   2 mat masked / bounded logdot (x y)  3 ten masked / bounded logdot (writes util)
// Sites [first, first + n_used); mask (may be null) selects sites.  Each block
// writes its partial sum of logs and its count of used sites.
__global__ void k_site_logs(int mode, const double *__restrict__ statd, const double *__restrict__ x,
                            const double *__restrict__ y, const double *__restrict__ z, const uint16_t *mask,
                            double *util, int n_rates, long n_sites, int K, long first, long n_used,
                            double *part_sum, long long *part_cnt) {
  double acc = 0;
  long long cnt = 0;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n_used; t += (long)gridDim.x * blockDim.x) {
    long s = first + t;
    bool use = mask ? mask[s] != 0 : true;
    double u = 0;
    if (mode == 0) {
      const double *xs = x + s * K, *ys = y + s * K, *zs = z + s * K;
      for (int k = 0; k < K; k++) u += statd[k] * xs[k] * ys[k] * zs[k];
    } else if (mode == 1) {
      for (int r = 0; r < n_rates; r++) {
        long o = ((long)r * n_sites + s) * K;
        for (int k = 0; k < K; k++) u += statd[k] * x[o + k] * y[o + k] * z[o + k];
      }
      util[s] = u;
    } else if (mode == 2) {
      if (use) {
        const double *xs = x + s * K, *ys = y + s * K;
        for (int k = 0; k < K; k++) u += xs[k] * ys[k];
      }
    } else {
      if (use)
        for (int r = 0; r < n_rates; r++) {
          long o = ((long)r * n_sites + s) * K;
          for (int k = 0; k < K; k++) u += x[o + k] * y[o + k];
        }
      util[mask ? s : t] = u;
    }
    if (use) {
      acc += log(u);
      cnt++;
    }
  }
  __shared__ double sh[kThreads / 32];
  __shared__ long long shc[kThreads / 32];
  acc = warp_sum_d(acc);
  cnt = warp_sum_ll(cnt);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sh[w] = acc; shc[w] = cnt; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    long long c = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) { s += sh[i]; c += shc[i]; }
    part_sum[blockIdx.x] = s;
    part_cnt[blockIdx.x] = c;
  }
}

// Sum the block partials in order; for the tensor forms subtract
// n_used * log(n_rates) as linear_c.c:421,536,602 do.
__global__ void k_finish_logs(const double *part_sum, const long long *part_cnt, int n_parts, int sub_log_rates,
                              int n_rates, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0;
  long long c = 0;
  for (int i = 0; i < n_parts; i++) { s += part_sum[i]; c += part_cnt[i]; }
  if (sub_log_rates) s -= ((double)(float)c) * log((double)(float)n_rates);
  *out = s;
}

// dst = x * y (mode 0) or dst[.., k] = statd[k] x y (mode 1)
__global__ void k_pairwise(int mode, double *dst, const double *__restrict__ x, const double *__restrict__ y,
                           const double *__restrict__ statd, long n, int K) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    dst[t] = mode == 0 ? x[t] * y[t] : statd[t % K] * x[t] * y[t];
}

__global__ void k_int_vec_tot(const uint16_t *x, long n, long long *part) {
  long long acc = 0;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) acc += x[t];
  __shared__ long long sh[kThreads / 32];
  acc = warp_sum_ll(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long s = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
    part[blockIdx.x] = s;
  }
}

__global__ void k_int_vec_prod(uint16_t *dst, const uint16_t *x, const uint16_t *y, long n) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
    dst[t] = (uint16_t)((int)x[t] * (int)y[t]);
}

// dst[j] += sum_{i: vec[i] != 0} mat[i,j] vec[i], rows in order (linear_c.c:644-670)
__global__ void k_fmat_ivec(double *dst, const double *__restrict__ mat, const uint16_t *__restrict__ vec, int n,
                            int k) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  double acc = dst[j];
  for (int i = 0; i < n; i++) {
    uint16_t v = vec[i];
    if (v) acc += mat[(long)i * k + j] * v;
  }
  dst[j] = acc;
}

// One per-site log reduction end to end.
double site_logs(int mode, const double *statd, const double *x, const double *y, const double *z,
                 const uint16_t *mask, double *util, int n_rates, int n_sites, int K, int first, int last,
                 bool sub_log_rates) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  t_error.clear();
  long n_used = (long)last - first + 1;
  if (n_sites < 0 || K <= 0 || n_rates <= 0 || first < 0 || n_used < 0 || first + n_used > n_sites) {
    set_error("site_logs: bad dimensions");
    return NAN;
  }
  bool ten = mode == 1 || mode == 3;
  long planes = ten ? n_rates : 1;
  long elems = planes * n_sites * K;
  int nb = blocks_for(n_used);
  Stage sg;
  size_t o_st = sg.take<double>(K), o_x = sg.take<double>(elems), o_y = sg.take<double>(elems);
  size_t o_z = (mode <= 1) ? sg.take<double>(elems) : 0;
  size_t o_m = mask ? sg.take<uint16_t>(n_sites) : 0;
  size_t o_u = sg.take<double>(n_sites + 1);
  size_t o_ps = sg.take<double>(nb), o_pc = sg.take<long long>(nb), o_out = sg.take<double>(1);
  if (ensure(sg.off) != PGB_OK) return NAN;
  if ((mode <= 1 && statd && h2d(o_st, statd, K * sizeof(double))) || h2d(o_x, x, elems * sizeof(double)) ||
      h2d(o_y, y, elems * sizeof(double)) || (mode <= 1 && h2d(o_z, z, elems * sizeof(double))) ||
      (mask && h2d(o_m, mask, n_sites * sizeof(uint16_t))))
    return NAN;
  k_site_logs<<<nb, kThreads, 0, g_ctx.st>>>(mode, at<double>(o_st), at<double>(o_x), at<double>(o_y),
                                             mode <= 1 ? at<double>(o_z) : nullptr,
                                             mask ? at<uint16_t>(o_m) : nullptr, at<double>(o_u), n_rates,
                                             n_sites, K, first, n_used, at<double>(o_ps), at<long long>(o_pc));
  count_launch();
  k_finish_logs<<<1, 32, 0, g_ctx.st>>>(at<double>(o_ps), at<long long>(o_pc), nb, sub_log_rates ? 1 : 0,
                                        n_rates, at<double>(o_out));
  count_launch();
  if (cudaGetLastError() != cudaSuccess) { set_error("site_logs: launch failed"); return NAN; }
  double res = NAN;
  if (d2h(&res, o_out, sizeof(double))) return NAN;
  if (util && ten) {
    long n_util = mask ? n_sites : n_used;
    if (d2h(util, o_u, n_util * sizeof(double))) return NAN;
  }
  if (finish() != PGB_OK) return NAN;
  return res;
}

pgb_status pairwise(int mode, double *dst, const double *x, const double *y, const double *statd, long n, int K) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (n < 0 || K <= 0) { set_error("pairwise: bad dimensions"); return PGB_ERR_ARG; }
  Stage sg;
  size_t o_d = sg.take<double>(n), o_x = sg.take<double>(n), o_y = sg.take<double>(n), o_s = sg.take<double>(K);
  pgb_status st;
  if ((st = ensure(sg.off))) return st;
  if ((st = h2d(o_x, x, n * sizeof(double))) || (st = h2d(o_y, y, n * sizeof(double)))) return st;
  if (mode == 1 && (st = h2d(o_s, statd, K * sizeof(double)))) return st;
  if (n > 0) {
    k_pairwise<<<blocks_for(n), kThreads, 0, g_ctx.st>>>(mode, at<double>(o_d), at<double>(o_x), at<double>(o_y),
                                                        at<double>(o_s), n, K);
    PGB_LAUNCH_CHECK();
  }
  if ((st = d2h(dst, o_d, n * sizeof(double)))) return st;
  return finish();
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

const char *pgb_last_error(void) { return t_error.c_str(); }
uint64_t pgb_kernel_launch_count(void) { return g_launches.load(); }

pgb_status pgb_gemmish(double *dst, const double *a, const double *b, int n_sites, int n_states) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (n_sites < 0 || n_states <= 0) { set_error("gemmish: bad dimensions"); return PGB_ERR_ARG; }
  long n = (long)n_sites * n_states;
  Stage sg;
  size_t o_d = sg.take<double>(n), o_a = sg.take<double>((long)n_states * n_states), o_b = sg.take<double>(n);
  pgb_status st;
  if ((st = ensure(sg.off))) return st;
  if ((st = h2d(o_a, a, (size_t)n_states * n_states * sizeof(double))) || (st = h2d(o_b, b, n * sizeof(double))))
    return st;
  if (n > 0) {
    k_gemmish<<<blocks_for(n), kThreads, 0, g_ctx.st>>>(at<double>(o_d), at<double>(o_a), at<double>(o_b),
                                                       n_sites, n_states);
    PGB_LAUNCH_CHECK();
  }
  if ((st = d2h(dst, o_d, n * sizeof(double)))) return st;
  return finish();
}

pgb_status pgb_dediagonalize(double *dst, const double *u, const double *lambda, const double *uit, int n) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (n <= 0) { set_error("dediagonalize: bad dimensions"); return PGB_ERR_ARG; }
  long nn = (long)n * n;
  Stage sg;
  size_t o_d = sg.take<double>(nn), o_u = sg.take<double>(nn), o_l = sg.take<double>(n), o_w = sg.take<double>(nn);
  pgb_status st;
  if ((st = ensure(sg.off))) return st;
  if ((st = h2d(o_u, u, nn * sizeof(double))) || (st = h2d(o_l, lambda, n * sizeof(double))) ||
      (st = h2d(o_w, uit, nn * sizeof(double))))
    return st;
  k_dediag<<<(int)((nn + kThreads - 1) / kThreads), kThreads, 0, g_ctx.st>>>(at<double>(o_d), at<double>(o_u),
                                                                            at<double>(o_l), at<double>(o_w), n);
  PGB_LAUNCH_CHECK();
  if ((st = d2h(dst, o_d, nn * sizeof(double)))) return st;
  return finish();
}

double pgb_mat_log_like3(const double *statd, const double *x, const double *y, const double *z, int n_sites,
                         int n_states) {
  return site_logs(0, statd, x, y, z, nullptr, nullptr, 1, n_sites, n_states, 0, n_sites - 1, false);
}

pgb_status pgb_mat_pairwise_prod(double *dst, const double *x, const double *y, int n_sites, int n_states) {
  return pairwise(0, dst, x, y, nullptr, (long)n_sites * n_states, n_states);
}

pgb_status pgb_mat_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                       int n_sites, int n_states) {
  return pairwise(1, dst, a, b, statd, (long)n_sites * n_states, n_states);
}

double pgb_mat_masked_logdot(const double *x, const double *y, const uint16_t *mask, int n_sites, int n_states) {
  return site_logs(2, nullptr, x, y, nullptr, mask, nullptr, 1, n_sites, n_states, 0, n_sites - 1, false);
}

double pgb_mat_bounded_logdot(const double *x, const double *y, int first, int last, int n_sites, int n_states) {
  return site_logs(2, nullptr, x, y, nullptr, nullptr, nullptr, 1, n_sites, n_states, first, last, false);
}

double pgb_ten_log_like3(const double *statd, const double *x, const double *y, const double *z, double *util,
                         int n_rates, int n_sites, int n_states) {
  return site_logs(1, statd, x, y, z, nullptr, util, n_rates, n_sites, n_states, 0, n_sites - 1, true);
}

pgb_status pgb_ten_pairwise_prod(double *dst, const double *x, const double *y, int n_rates, int n_sites,
                                 int n_states) {
  return pairwise(0, dst, x, y, nullptr, (long)n_rates * n_sites * n_states, n_states);
}

pgb_status pgb_ten_statd_pairwise_prod(const double *statd, double *dst, const double *a, const double *b,
                                       int n_rates, int n_sites, int n_states) {
  return pairwise(1, dst, a, b, statd, (long)n_rates * n_sites * n_states, n_states);
}

double pgb_ten_masked_logdot(const double *x, const double *y, const uint16_t *mask, double *util, int n_rates,
                             int n_sites, int n_states) {
  return site_logs(3, nullptr, x, y, nullptr, mask, util, n_rates, n_sites, n_states, 0, n_sites - 1, true);
}

double pgb_ten_bounded_logdot(const double *x, const double *y, int first, int last, double *util, int n_rates,
                              int n_sites, int n_states) {
  return site_logs(3, nullptr, x, y, nullptr, nullptr, util, n_rates, n_sites, n_states, first, last, true);
}

pgb_status pgb_vec_pairwise_prod(double *dst, const double *x, const double *y, int n) {
  return pairwise(0, dst, x, y, nullptr, n, 1);
}

int pgb_int_vec_tot(const uint16_t *x, int n) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  t_error.clear();
  if (n < 0) { set_error("int_vec_tot: bad dimensions"); return 0; }
  int nb = blocks_for(n);
  Stage sg;
  size_t o_x = sg.take<uint16_t>(n), o_p = sg.take<long long>(nb);
  if (ensure(sg.off) || h2d(o_x, x, (size_t)n * sizeof(uint16_t))) return 0;
  k_int_vec_tot<<<nb, kThreads, 0, g_ctx.st>>>(at<uint16_t>(o_x), n, at<long long>(o_p));
  count_launch();
  std::vector<long long> part(nb);
  if (d2h(part.data(), o_p, nb * sizeof(long long)) || finish()) return 0;
  long long s = 0;
  for (long long v : part) s += v;
  return (int)s;
}

pgb_status pgb_int_vec_pairwise_prod(uint16_t *dst, const uint16_t *x, const uint16_t *y, int n) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (n < 0) { set_error("int_vec_pairwise_prod: bad dimensions"); return PGB_ERR_ARG; }
  Stage sg;
  size_t o_d = sg.take<uint16_t>(n), o_x = sg.take<uint16_t>(n), o_y = sg.take<uint16_t>(n);
  pgb_status st;
  if ((st = ensure(sg.off))) return st;
  if ((st = h2d(o_x, x, (size_t)n * 2)) || (st = h2d(o_y, y, (size_t)n * 2))) return st;
  if (n > 0) {
    k_int_vec_prod<<<blocks_for(n), kThreads, 0, g_ctx.st>>>(at<uint16_t>(o_d), at<uint16_t>(o_x),
                                                            at<uint16_t>(o_y), n);
    PGB_LAUNCH_CHECK();
  }
  if ((st = d2h(dst, o_d, (size_t)n * 2))) return st;
  return finish();
}

pgb_status pgb_float_mat_int_vec_mul(double *dst, const double *mat, const uint16_t *vec, int n, int k) {
  std::lock_guard<std::mutex> lk(g_ctx.mu);
  if (n < 0 || k < 0) { set_error("float_mat_int_vec_mul: bad dimensions"); return PGB_ERR_ARG; }
  Stage sg;
  size_t o_d = sg.take<double>(k), o_m = sg.take<double>((long)n * k), o_v = sg.take<uint16_t>(n);
  pgb_status st;
  if ((st = ensure(sg.off))) return st;
  if ((st = h2d(o_d, dst, (size_t)k * 8)) || (st = h2d(o_m, mat, (size_t)n * k * 8)) ||
      (st = h2d(o_v, vec, (size_t)n * 2)))
    return st;
  if (k > 0) {
    k_fmat_ivec<<<(k + kThreads - 1) / kThreads, kThreads, 0, g_ctx.st>>>(at<double>(o_d), at<double>(o_m),
                                                                         at<uint16_t>(o_v), n, k);
    PGB_LAUNCH_CHECK();
  }
  if ((st = d2h(dst, o_d, (size_t)k * 8))) return st;
  return finish();
}

}  // extern "C"
