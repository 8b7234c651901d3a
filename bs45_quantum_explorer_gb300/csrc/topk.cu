// topk.cu - per-cell flattest-k keep: flat_score (src/solver/wz_match.cpp:2569-2583) and the
// stable sort + front-only cut of drain() (wz_match.cpp:2656-2714), on the GPU.
//
// A cell's survivors, in stream order, are split into batches of buf_cap. Inside a batch the
// reference stable-sorts by flat score, so ties keep stream order. A stable sort by a small
// integer key is a counting sort: one warp per batch builds the score histogram in shared
// memory, scans it, and scatters positions in stream order, ranking equal scores inside each
// 32-wide step with __match_any_sync. Only the first `keep` positions are written.
#include <stdint.h>

#include <vector>

#include "bsfh_internal.cuh"

namespace {

#define FULL_MASK 0xffffffffu
constexpr int MAX_SCORE = 4096;  // n(n-1) < 4096 for n <= 64

// flat score of one packed pair: sum over s = 1..n-1 of |N_C(s) + N_D(s)|; with +-1 entries
// N_X(s) = (n - s) - 2 * popcount((X ^ (X >> s)) restricted to the n - s overlapping bits).
__global__ void flat_score_kernel(const uint64_t *__restrict__ words, long long count, int n,
                                  int32_t *__restrict__ scores) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t c = words[2 * i], d = words[2 * i + 1];
    int sc = 0;
    for (int s = 1; s < n; s++) {
      const uint64_t mask = (s >= 64) ? 0 : ((n - s >= 64) ? ~0ULL : ((1ULL << (n - s)) - 1));
      int dc = __popcll((c ^ (c >> s)) & mask), dd = __popcll((d ^ (d >> s)) & mask);
      int v = 2 * (n - s) - 2 * (dc + dd);
      sc += v < 0 ? -v : v;
    }
    scores[i] = sc;
  }
}

// One warp per batch [b*buf_cap, min(nsurv, (b+1)*buf_cap)).
__global__ void __launch_bounds__(32) batch_counting_sort_kernel(
    const int32_t *__restrict__ scores, long long nsurv, long long buf_cap, long long keep,
    int64_t *__restrict__ order, int32_t *__restrict__ out_scores) {
  __shared__ unsigned hist[MAX_SCORE];
  const int lane = threadIdx.x;
  const long long b = blockIdx.x;
  const long long lo = b * buf_cap;
  const long long hi = (lo + buf_cap < nsurv) ? lo + buf_cap : nsurv;
  const long long len = hi - lo;
  const long long kept = (keep > 0 && keep < len) ? keep : len;
  const long long out0 = b * ((keep > 0 && keep < buf_cap) ? keep : buf_cap);
  for (int i = lane; i < MAX_SCORE; i += 32) hist[i] = 0;
  __syncwarp();
  for (long long i = lo + lane; i < hi; i += 32) atomicAdd(&hist[scores[i]], 1u);
  __syncwarp();
  // exclusive scan over the histogram: 128 bins per lane, then a warp scan of lane totals
  unsigned local = 0;
  for (int k = 0; k < MAX_SCORE / 32; k++) local += hist[lane * (MAX_SCORE / 32) + k];
  unsigned incl = local;
  for (int off = 1; off < 32; off <<= 1) {
    unsigned v = __shfl_up_sync(FULL_MASK, incl, off);
    if (lane >= off) incl += v;
  }
  unsigned run = incl - local;
  __syncwarp();
  for (int k = 0; k < MAX_SCORE / 32; k++) {
    unsigned &h = hist[lane * (MAX_SCORE / 32) + k];
    unsigned c = h;
    h = run;
    run += c;
  }
  __syncwarp();
  // stable scatter in stream order
  for (long long base = lo; base < hi; base += 32) {
    const long long i = base + lane;
    const bool valid = i < hi;
    const int s = valid ? scores[i] : -1 - lane;  // invalid lanes get unique dummy keys
    const unsigned peers = __match_any_sync(FULL_MASK, s);
    const unsigned rank = __popc(peers & ((1u << lane) - 1u));
    unsigned pos = 0;
    if (valid) pos = hist[s] + rank;
    __syncwarp();
    if (valid && (peers >> lane) == 1u) hist[s] += __popc(peers);  // highest lane of the group
    __syncwarp();
    if (valid && pos < (unsigned long long)kept) {
      order[out0 + pos] = i;
      if (out_scores) out_scores[out0 + pos] = s;
    }
  }
}

}  // namespace

#define CK(x)                                       \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return bs_cuda_fail(e_); \
  } while (0)

extern "C" int bs_flat_topk_dev(bs_ctx *ctx, const uint64_t *d_words, long long nsurv,
                                long long buf_cap, long long keep, int64_t *d_order,
                                int32_t *d_scores_sorted, int32_t *d_scores) {
  if (!ctx || nsurv < 0 || buf_cap <= 0) return BS_ERR_ARG;
  if (nsurv == 0) return BS_OK;
  if (!d_words || !d_order || !d_scores) return BS_ERR_ARG;
  if (ctx->n * (ctx->n - 1) >= MAX_SCORE || buf_cap >= (1LL << 32)) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  ctx->launches += 2;
  flat_score_kernel<<<bs_grid_for(nsurv, 256, 16 * ctx->num_sms), 256, 0, ctx->stream>>>(
      d_words, nsurv, ctx->n, d_scores);
  CK(cudaGetLastError());
  long long nb = (nsurv + buf_cap - 1) / buf_cap;
  if (nb > (1LL << 31) - 1) return BS_ERR_ARG;
  batch_counting_sort_kernel<<<(unsigned)nb, 32, 0, ctx->stream>>>(d_scores, nsurv, buf_cap, keep,
                                                                   d_order, d_scores_sorted);
  CK(cudaGetLastError());
  return BS_OK;
}

extern "C" int bs_flat_topk(bs_ctx *ctx, const uint64_t *words, long long nsurv, long long buf_cap,
                            long long keep, int64_t *order, int32_t *scores, long long *nkept) {
  if (!ctx || nsurv < 0 || buf_cap <= 0 || !nkept) return BS_ERR_ARG;
  long long nb = (nsurv + buf_cap - 1) / buf_cap, total = 0;
  for (long long b = 0; b < nb; b++) {
    long long len = (b + 1) * buf_cap < nsurv ? buf_cap : nsurv - b * buf_cap;
    total += (keep > 0 && keep < len) ? keep : len;
  }
  *nkept = total;
  if (nsurv == 0) return BS_OK;
  if (!words || !order) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  const long long per = (keep > 0 && keep < buf_cap) ? keep : buf_cap;
  uint64_t *dw = nullptr;
  int32_t *ds = nullptr, *dss = nullptr;
  int64_t *dord = nullptr;
  cudaError_t e = cudaMallocAsync(&dw, sizeof(uint64_t) * 2 * nsurv, ctx->stream);
  if (e == cudaSuccess) e = cudaMallocAsync(&ds, sizeof(int32_t) * nsurv, ctx->stream);
  if (e == cudaSuccess) e = cudaMallocAsync(&dss, sizeof(int32_t) * nb * per, ctx->stream);
  if (e == cudaSuccess) e = cudaMallocAsync(&dord, sizeof(int64_t) * nb * per, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dw, words, sizeof(uint64_t) * 2 * nsurv, cudaMemcpyHostToDevice, ctx->stream);
  int rc = e == cudaSuccess ? BS_OK : bs_cuda_fail(e);
  if (!rc) rc = bs_flat_topk_dev(ctx, dw, nsurv, buf_cap, keep, dord, dss, ds);
  if (!rc) {
    // compact the per-batch slots (the last batch may hold fewer than `per`)
    std::vector<int64_t> h_ord(nb * per);
    std::vector<int32_t> h_sc(nb * per);
    e = cudaMemcpyAsync(h_ord.data(), dord, sizeof(int64_t) * nb * per, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_sc.data(), dss, sizeof(int32_t) * nb * per, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = bs_cuda_fail(e);
    long long o = 0;
    for (long long b = 0; !rc && b < nb; b++) {
      long long len = (b + 1) * buf_cap < nsurv ? buf_cap : nsurv - b * buf_cap;
      long long kb = (keep > 0 && keep < len) ? keep : len;
      for (long long t = 0; t < kb; t++, o++) {
        order[o] = h_ord[b * per + t];
        if (scores) scores[o] = h_sc[b * per + t];
      }
    }
  }
  cudaFreeAsync(dw, ctx->stream);
  cudaFreeAsync(ds, ctx->stream);
  cudaFreeAsync(dss, ctx->stream);
  cudaFreeAsync(dord, ctx->stream);
  return rc;
}
