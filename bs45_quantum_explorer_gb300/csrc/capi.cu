// capi.cu - context management and the host side of the Hall tables.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "bsfh_internal.cuh"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int bs_cuda_fail(cudaError_t e) {
  if (e == cudaErrorMemoryAllocation) return BS_ERR_NOMEM;
  return BS_ERR_CUDA;
}

#define CK(x)                                   \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return bs_cuda_fail(e_); \
  } while (0)

int bs_ensure_dev(void **ptr, long long *cap, long long need, size_t elem) {
  if (need <= *cap && *ptr) return BS_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  long long n = need < 1024 ? 1024 : need;
  cudaError_t e = cudaMalloc(ptr, (size_t)n * elem);
  if (e != cudaSuccess) { *ptr = nullptr; return bs_cuda_fail(e); }
  *cap = n;
  return BS_OK;
}

int bs_ensure_pinned(bs_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->pinned_bytes && ctx->h_pinned) return BS_OK;
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  ctx->h_pinned = nullptr;
  ctx->pinned_bytes = 0;
  cudaError_t e = cudaMallocHost(&ctx->h_pinned, bytes);
  if (e != cudaSuccess) { ctx->h_pinned = nullptr; return bs_cuda_fail(e); }
  ctx->pinned_bytes = bytes;
  return BS_OK;
}

extern "C" int bs_version(void) { return 100; }

extern "C" const char *bs_strerror(int code) {
  switch (code) {
    case BS_OK: return "ok";
    case BS_STOPPED: return "stopped by the context's stop flag (partial result)";
    case BS_WALLED: return "stream stopped by its wall limit (partial result)";
    case BS_ERR_ARG: return "bad argument";
    case BS_ERR_CUDA: return "CUDA runtime error";
    case BS_ERR_NOMEM: return "out of memory";
    case BS_ERR_TIMEOUT: return "device wait limit reached";
    case BS_ERR_INTERNAL: return "internal consistency check failed";
    case BS_ERR_CAP: return "output capacity exceeded";
    case BS_ERR_NODEV: return "no sm_103 CUDA device";
    default: return "unknown error";
  }
}

// ---- fp16 / bf16 encodings of exactly representable table values -------------------
static uint16_t to_bf16_exact(double v) {
  float f = (float)v;
  uint32_t u;
  memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);  // v carries <= 8 significant bits, so the low half is zero
}

static uint16_t to_f16_exact(double v) {
  if (v == 0.0) return 0;
  uint16_t sign = v < 0 ? 0x8000 : 0;
  double a = fabs(v);
  int e;
  double m = frexp(a, &e);  // a = m * 2^e, m in [0.5, 1)
  int exp16 = e - 1 + 15;   // biased exponent of 1.xxx * 2^(e-1)
  if (exp16 <= 0) {         // subnormal: value = k * 2^-24
    int k = (int)llrint(a * 16777216.0);
    return (uint16_t)(sign | (uint16_t)k);
  }
  int frac = (int)llrint((m * 2.0 - 1.0) * 1024.0);
  return (uint16_t)(sign | (uint16_t)(exp16 << 10) | (uint16_t)frac);
}

// Place element k of table row `row` (a DFT column) in the 128B-swizzled K-major image.
static inline void put_sw128(uint8_t *img, int row, int k, uint16_t bits) {
  size_t off = (size_t)row * 128 + ((size_t)(((k >> 3) ^ (row & 7))) << 4) + (size_t)(k & 7) * 2;
  img[off] = (uint8_t)(bits & 0xFF);
  img[off + 1] = (uint8_t)(bits >> 8);
}

// Unique angle index u -> reference angle j (the twin 200-j has the same PSD).
static inline int angle_of(int u) { return u < 100 ? u + 1 : 200; }

// Build the tensor-core table image for one form and its certified thresholds.
//   fp16 form: q(t) = round(t * 2^11) / 2^11, one part.
//   bf16 form: hi = round(t * 2^8) / 2^8, lo = round((t - hi) * 2^17) / 2^17, two parts.
// Every quantised value is exact in its format, so Re_q = sum_i x_i q(t_i) is a multiple of
// the quantum with fewer than 24 significant bits and the FP32 accumulator holds it exactly.
// e = max over angles of sum_i |t_i - q(t_i)| bounds |Re - Re_q| and |Im - Im_q|.
static int build_tc_form(bs_ctx *ctx, const double *ct, const double *st, int mode, int L,
                         bs_hall_tc_form &F) {
  F.nparts = (mode == BS_HALL_TC_BF16X2) ? 2 : 1;
  F.fmt = (mode == BS_HALL_TC_BF16X2) ? 1 : 0;
  size_t bytes = (size_t)F.nparts * BS_TC_PART_BYTES;
  uint8_t *img = (uint8_t *)calloc(bytes, 1);
  if (!img) return BS_ERR_NOMEM;
  double e = 0.0;
  for (int u = 0; u < BS_TC_NANG; u++) {
    int j = angle_of(u);
    for (int part_kind = 0; part_kind < 2; part_kind++) {  // 0 = cos (Re), 1 = sin (Im)
      const double *tab = part_kind ? st : ct;
      int col = bs_tc_row(u, part_kind);
      double esum = 0.0;
      for (int i = 0; i < L; i++) {
        double t = tab[(size_t)j * (ctx->n1) + i];
        if (F.nparts == 1) {
          double q = nearbyint(t * 2048.0) / 2048.0;
          put_sw128(img, col, i, to_f16_exact(q));
          esum += fabs(t - q);
        } else {
          double hi = nearbyint(t * 256.0) / 256.0;
          double lo = nearbyint((t - hi) * 131072.0) / 131072.0;
          put_sw128(img, col, i, to_bf16_exact(hi));
          put_sw128(img + BS_TC_PART_BYTES, col, i, to_bf16_exact(lo));
          esum += fabs((t - hi) - lo);
        }
      }
      if (esum > e) e = esum;
    }
  }
  e = e * (1.0 + 1e-9) + 1e-12;
  // Certified thresholds on the fp32 pair PSD pf_c:
  //   |pf_exact - pf_q| <= 4 e sqrt(pf_q) + 4 e^2, |pf_c - pf_q| <= rho pf_q (kappa = 1+4 rho),
  //   |pf_ref - pf_exact| <= eps64 (FP64 rounding of the reference and twin-angle spread).
  const double eps64 = 1e-9, rho = ldexp(1.0, -20), kappa = 1.0 + 4.0 * rho;
  double lim = ctx->lim;
  double pb = (sqrt(lim - eps64) - 2.0 * e);
  pb = pb * pb / kappa;
  double ra = 2.0 * e + sqrt(lim + 8.0 * e * e + eps64);
  ra = ra * ra * kappa;
  float pbf = (float)pb;
  if ((double)pbf > pb) pbf = nextafterf(pbf, 0.0f);
  float raf = (float)ra;
  if ((double)raf < ra) raf = nextafterf(raf, 1e30f);
  raf = nextafterf(raf, 1e30f);
  F.quant_err = e;
  F.pass_below = pbf;
  F.reject_above = raf;
  cudaError_t ce = cudaSuccess;
  if (!F.d_image) ce = cudaMalloc(&F.d_image, bytes);  // one size per form: kept on retarget
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(F.d_image, img, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  free(img);
  if (ce != cudaSuccess) return bs_cuda_fail(ce);
  return BS_OK;
}

// The fixed-point Hall form for sequences of length L: every table entry of the 101 unique
// angles as T = round(t * 2^30) (|T| <= 2^30), so a sequence's Re and Im are exact int64 sums
// and their error against the FP64 table is at most e1 = max over angles of sum |t - T/2^30|.
// The pair PSD F' is formed from them in FP64 with relative error below 2^-48 (kappa2); the
// same argument as the tensor-core form then certifies its thresholds.
static int build_fix_form(bs_ctx *ctx, const double *ct, const double *st, int L, bs_hall_fix_form &F) {
  std::vector<int64_t> tab(BS_FIX_WORDS, 0);
  int64_t *tc = tab.data(), *ts = tc + BS_TC_NANG * L, *sc = tc + 2 * BS_TC_NANG * L, *ss = sc + BS_TC_NANG;
  double e = 0.0;
  for (int u = 0; u < BS_TC_NANG; u++) {
    const int j = angle_of(u);
    double ec = 0.0, es = 0.0;
    for (int i = 0; i < L; i++) {
      const double c = ct[(size_t)j * ctx->n1 + i], s = st[(size_t)j * ctx->n1 + i];
      const int64_t qc = llrint(ldexp(c, 30)), qs = llrint(ldexp(s, 30));
      tc[u * L + i] = qc;
      ts[u * L + i] = qs;
      sc[u] += qc;
      ss[u] += qs;
      ec += fabs(c - ldexp((double)qc, -30));
      es += fabs(s - ldexp((double)qs, -30));
    }
    e = std::max(e, std::max(ec, es));
  }
  e = e * (1.0 + 1e-9) + 1e-15;
  const double eps64 = 1e-9, kappa2 = 1.0 + ldexp(1.0, -48);
  double pb = sqrt(ctx->lim - eps64) - 2.0 * e;
  pb = pb * pb / kappa2;
  double ra = 2.0 * e + sqrt(ctx->lim + 8.0 * e * e + eps64);
  ra = ra * ra * kappa2;
  F.err = e;
  F.pass_below = nextafter(pb, 0.0);
  F.reject_above = nextafter(ra, 1e300);
  cudaError_t ce = cudaSuccess;
  if (!F.d_tab) ce = cudaMalloc(&F.d_tab, sizeof(int64_t) * BS_FIX_WORDS);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(F.d_tab, tab.data(), sizeof(int64_t) * BS_FIX_WORDS, cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  if (ce != cudaSuccess) return bs_cuda_fail(ce);
  return BS_OK;
}

// Loads the tables of BS(n+1,n) into a context whose stream and buffers exist: host tables
// exactly as init_hall_tables builds them (wz_match.cpp:106-114), their FP64 copies and the
// tensor-core images for both sequence lengths (C,D: n; A,B: n+1).
static int load_tables(bs_ctx *ctx, int n, int a, int b, int c, int d) {
  ctx->n = n; ctx->n1 = n + 1;
  ctx->sig[0] = a; ctx->sig[1] = b; ctx->sig[2] = c; ctx->sig[3] = d;
  ctx->lim = (4.0 * n + 2.0) + 0.5;
  int rc = BS_OK;
  const int w = n + 1;
  double *ct = (double *)calloc((size_t)201 * w, sizeof(double));
  double *st = (double *)calloc((size_t)201 * w, sizeof(double));
  double *gc = (double *)calloc((size_t)200 * BS_MAXL, sizeof(double));
  double *gs = (double *)calloc((size_t)200 * BS_MAXL, sizeof(double));
  if (!ct || !st || !gc || !gs) rc = BS_ERR_NOMEM;
  if (rc == BS_OK) {
    for (int j = 1; j <= 200; j++) {
      double th = j * M_PI / 100.0;
      for (int i = 0; i < w; i++) {
        ct[(size_t)j * w + i] = cos(i * th);
        st[(size_t)j * w + i] = sin(i * th);
        gc[(size_t)(j - 1) * BS_MAXL + i] = ct[(size_t)j * w + i];
        gs[(size_t)(j - 1) * BS_MAXL + i] = st[(size_t)j * w + i];
      }
    }
    cudaError_t e1 = cudaMemcpyAsync(ctx->d_cos, gc, sizeof(double) * 200 * BS_MAXL, cudaMemcpyHostToDevice, ctx->stream);
    if (e1 == cudaSuccess) e1 = cudaMemcpyAsync(ctx->d_sin, gs, sizeof(double) * 200 * BS_MAXL, cudaMemcpyHostToDevice, ctx->stream);
    if (e1 == cudaSuccess) e1 = cudaStreamSynchronize(ctx->stream);
    if (e1 != cudaSuccess) rc = bs_cuda_fail(e1);
  }
  if (rc == BS_OK) rc = build_tc_form(ctx, ct, st, BS_HALL_TC_FP16, n, ctx->tc[BS_HALL_TC_FP16]);
  if (rc == BS_OK) rc = build_tc_form(ctx, ct, st, BS_HALL_TC_BF16X2, n, ctx->tc[BS_HALL_TC_BF16X2]);
  if (rc == BS_OK) rc = build_tc_form(ctx, ct, st, BS_HALL_TC_FP16, n + 1, ctx->tc_ab[BS_HALL_TC_FP16]);
  if (rc == BS_OK)
    rc = build_tc_form(ctx, ct, st, BS_HALL_TC_BF16X2, n + 1, ctx->tc_ab[BS_HALL_TC_BF16X2]);
  if (rc == BS_OK) rc = build_fix_form(ctx, ct, st, n, ctx->fix[0]);
  if (rc == BS_OK) rc = build_fix_form(ctx, ct, st, n + 1, ctx->fix[1]);
  free(ct); free(st); free(gc); free(gs);
  return rc;
}

extern "C" int bs_ctx_create(int n, int a, int b, int c, int d, int device, bs_ctx **out) {
  if (!out) return BS_ERR_ARG;
  *out = nullptr;
  if (n < 4 || n + 1 > BS_MAXL) return BS_ERR_ARG;
  if (a * a + b * b + c * c + d * d != 4 * n + 2) return BS_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return BS_ERR_NODEV;
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3) return BS_ERR_NODEV;
  CK(cudaSetDevice(device));
  bs_ctx *ctx = (bs_ctx *)calloc(1, sizeof(bs_ctx));
  if (!ctx) return BS_ERR_NOMEM;
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  int rc = BS_OK;
  cudaError_t e1 = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  ctx->stream = ctx->own_stream;
  if (e1 == cudaSuccess) e1 = cudaMalloc(&ctx->d_cos, sizeof(double) * 200 * BS_MAXL);
  if (e1 == cudaSuccess) e1 = cudaMalloc(&ctx->d_sin, sizeof(double) * 200 * BS_MAXL);
  if (e1 == cudaSuccess) e1 = cudaMalloc(&ctx->d_status, sizeof(int));
  if (e1 == cudaSuccess) e1 = cudaMemset(ctx->d_status, 0, sizeof(int));
  if (e1 == cudaSuccess) e1 = cudaMalloc(&ctx->d_count, sizeof(unsigned long long) * 8);
  if (e1 == cudaSuccess) {
    void *h = nullptr;
    e1 = cudaHostAlloc(&h, sizeof(int32_t), cudaHostAllocMapped);
    if (e1 == cudaSuccess) {
      ctx->h_stop = (volatile int32_t *)h;
      *ctx->h_stop = 0;
      void *dp = nullptr;
      e1 = cudaHostGetDevicePointer(&dp, h, 0);
      ctx->d_stop = (int32_t *)dp;
    }
  }
  if (e1 != cudaSuccess) rc = bs_cuda_fail(e1);
  if (rc == BS_OK) rc = load_tables(ctx, n, a, b, c, d);
  if (rc != BS_OK) { bs_ctx_destroy(ctx); return rc; }
  *out = ctx;
  return BS_OK;
}

extern "C" int bs_ctx_retarget(bs_ctx *ctx, int n, int a, int b, int c, int d) {
  if (!ctx) return BS_ERR_ARG;
  if (n < 4 || n + 1 > BS_MAXL) return BS_ERR_ARG;
  if (a * a + b * b + c * c + d * d != 4 * n + 2) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));  // earlier work may still read the old tables
  if (n == ctx->n) {
    ctx->sig[0] = a; ctx->sig[1] = b; ctx->sig[2] = c; ctx->sig[3] = d;
    return BS_OK;
  }
  const int rc = load_tables(ctx, n, a, b, c, d);
  if (rc != BS_OK) ctx->n = 0;  // tables half loaded: the next retarget reloads them all
  return rc;
}

extern "C" void bs_ctx_destroy(bs_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  cudaFree(ctx->d_cos); cudaFree(ctx->d_sin);
  for (int m = 1; m < 3; m++) {
    cudaFree(ctx->tc[m].d_image);
    cudaFree(ctx->tc_ab[m].d_image);
  }
  cudaFree(ctx->fix[0].d_tab); cudaFree(ctx->fix[1].d_tab);
  cudaFree(ctx->d_status); cudaFree(ctx->d_count);
  cudaFree(ctx->d_bits); cudaFree(ctx->d_pass); cudaFree(ctx->d_rows); cudaFree(ctx->d_unc);
  cudaFree(ctx->d_unc2); cudaFree(ctx->d_scr);
  bs_stream_free(ctx);
  bs_ab_free(ctx);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->h_stop) cudaFreeHost((void *)ctx->h_stop);
  if (ctx->ev[0])
    for (int i = 0; i < 2 * 512; i++) cudaEventDestroy(ctx->ev[i]);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  free(ctx);
}

extern "C" int bs_ctx_set_stream(bs_ctx *ctx, void *s) {
  if (!ctx) return BS_ERR_ARG;
  ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
  return BS_OK;
}

extern "C" volatile int32_t *bs_ctx_stop_flag(bs_ctx *ctx) { return ctx ? ctx->h_stop : nullptr; }

extern "C" int bs_ctx_device_status(bs_ctx *ctx) {
  if (!ctx) return BS_ERR_ARG;
  int st = 0;
  CK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (st) CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  return st;
}

static void flush_events(bs_ctx *ctx) {
  for (int i = 0; i < ctx->nev; i++) {
    float ms = 0.f;
    cudaEventSynchronize(ctx->ev[2 * i + 1]);
    if (cudaEventElapsedTime(&ms, ctx->ev[2 * i], ctx->ev[2 * i + 1]) == cudaSuccess)
      ctx->timed_ms += ms;
  }
  ctx->nev = 0;
}

void bs_timed_begin(bs_ctx *ctx) {
  ctx->launches++;
  if (!ctx->timing) return;
  if (ctx->nev == 512) flush_events(ctx);
  cudaEventRecord(ctx->ev[2 * ctx->nev], ctx->stream);
}

void bs_timed_end(bs_ctx *ctx) {
  if (!ctx->timing) return;
  cudaEventRecord(ctx->ev[2 * ctx->nev + 1], ctx->stream);
  ctx->nev++;
  ctx->timed_launches++;
}

extern "C" int bs_ctx_timing(bs_ctx *ctx, int enable) {
  if (!ctx) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  if (enable && !ctx->ev[0]) {
    for (int i = 0; i < 2 * 512; i++) CK(cudaEventCreate(&ctx->ev[i]));
  }
  ctx->timing = enable && ctx->ev[0];
  ctx->nev = 0;
  ctx->timed_ms = 0.0;
  ctx->timed_launches = 0;
  return BS_OK;
}

extern "C" int bs_ctx_timing_read(bs_ctx *ctx, double *ms, long long *timed, long long *all) {
  if (!ctx) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  flush_events(ctx);
  if (ms) *ms = ctx->timed_ms;
  if (timed) *timed = ctx->timed_launches;
  if (all) *all = ctx->launches;
  ctx->timed_ms = 0.0;
  ctx->timed_launches = 0;
  return BS_OK;
}

extern "C" int bs_pack_rows(const int8_t *seq, long long rows, int L, uint64_t *words) {
  if (!seq || !words || L < 1 || L > BS_MAXL || rows < 0) return BS_ERR_ARG;
  for (long long r = 0; r < rows; r++) {
    uint64_t w = 0;
    const int8_t *s = seq + r * L;
    for (int i = 0; i < L; i++) {
      if (s[i] == 1) w |= 1ULL << i;
      else if (s[i] != -1) return BS_ERR_ARG;
    }
    words[r] = w;
  }
  return BS_OK;
}
