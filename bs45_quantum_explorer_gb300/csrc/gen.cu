// gen.cu - seeded synthetic input for the Hall filter microbench (C,D pairs at length n).
// The generator is defined per pair index (see bs45_quantum_explorer_gb300/workloads.py), so
// device, oracle and Python forms produce identical words.
#include "bsfh_internal.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t sm64(uint64_t seed, uint64_t k) {
  return mix64(seed + (k + 1) * 0x9E3779B97F4A7C15ULL);
}

// Quad index -> 4 sign bits (C[d], D[d], C[n-1-d], D[n-1-d]) as set bits for +1.
// All 16 quads: index i has bits i&8, i&4, i&2, i&1. Positive-product quads: the indices
// with an even number of zero bits, in increasing order.
__constant__ uint8_t kPosQuad[8] = {0, 3, 5, 6, 9, 10, 12, 15};

__global__ void gen_pairs_kernel(int n, long long npairs, uint64_t seed, uint64_t *words,
                                 int *status) {
  const long long half = npairs / 2;
  const uint64_t mask = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npairs;
       p += (long long)gridDim.x * blockDim.x) {
    uint64_t cw, dw;
    if (p < half || (n & 1) || n > 42) {
      cw = sm64(seed, 2 * (uint64_t)p) & mask;
      dw = sm64(seed, 2 * (uint64_t)p + 1) & mask;
    } else {
      const int hd = n / 2;
      uint64_t t = 0;
      for (;;) {
        uint64_t r = sm64(seed ^ 0xA5A5A5A5A5A5A5A5ULL, ((uint64_t)p << 20) + t);
        t++;
        cw = 0;
        dw = 0;
        for (int d = 0; d < hd; d++) {
          uint32_t q;
          if (d == 0) { q = (uint32_t)(r & 15); r >>= 4; }
          else { q = kPosQuad[r & 7]; r >>= 3; }
          cw |= (uint64_t)((q >> 3) & 1) << d;
          dw |= (uint64_t)((q >> 2) & 1) << d;
          cw |= (uint64_t)((q >> 1) & 1) << (n - 1 - d);
          dw |= (uint64_t)(q & 1) << (n - 1 - d);
        }
        if (__popcll(cw) * 2 == n && __popcll(dw) * 2 == n) break;
        if (t > (1ULL << 20)) { atomicCAS(status, 0, BS_ERR_INTERNAL); break; }
      }
    }
    words[2 * p] = cw;
    words[2 * p + 1] = dw;
  }
}

}  // namespace

extern "C" int bs_gen_hall_pairs_dev(bs_ctx *ctx, long long npairs, uint64_t seed,
                                     uint64_t *d_words) {
  if (!ctx || npairs < 0 || (npairs && !d_words)) return BS_ERR_ARG;
  if (npairs == 0) return BS_OK;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return bs_cuda_fail(e);
  ctx->launches++;
  gen_pairs_kernel<<<bs_grid_for(npairs, 256, 64 * ctx->num_sms), 256, 0, ctx->stream>>>(
      ctx->n, npairs, seed, d_words, ctx->d_status);
  e = cudaGetLastError();
  return e == cudaSuccess ? BS_OK : bs_cuda_fail(e);
}
