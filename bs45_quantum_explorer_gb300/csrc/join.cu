// join.cu - exact NPAF verification of quads and the autocorrelation-key hash join.
//
// NPAF (npaf_at, src/solver/wz_match.cpp:184-192; tools/verify_npaf.py:42-53): for packed
// +-1 words, N_X(s) = (L - s) - 2 * popcount((X ^ (X >> s)) on the L - s overlapping bits).
//
// Join (the reference's WZ_JOIN22 mode, wz_match.cpp:2894-3104): a solution needs
// AB[s] = -CD[s] for s = 1..n (AB[n] = 0 since CD[n] is empty). Each C,D is inserted into an
// open-addressed device table under a 64-bit key of its vector (-CD[1..n-1], 0); each A,B
// probes with the key of (AB[1..n]). Every equal-key pairing is then checked with the exact
// integer NPAF on the device, so key collisions can only cost time, never a wrong quad, and
// equal vectors always meet (no false negatives). Unlike the reference, every C,D is kept
// (a multi-map), so the join returns every quad, not one representative per key.
#include <stdint.h>

#include <vector>

#include "bsfh_internal.cuh"

namespace {

__device__ __forceinline__ int nacf(uint64_t x, int L, int s) {
  if (s >= L) return 0;
  const uint64_t mask = (L - s >= 64) ? ~0ULL : ((1ULL << (L - s)) - 1ULL);
  return (L - s) - 2 * __popcll((x ^ (x >> s)) & mask);
}

// max_s |NPAF(s)| for s = 1..n1 of a quad (A,B length n1, C,D length n)
__global__ void npaf_kernel(const uint64_t *__restrict__ q, long long count, int n,
                            int32_t *__restrict__ maxabs) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t A = q[4 * i], B = q[4 * i + 1], C = q[4 * i + 2], D = q[4 * i + 3];
    int mx = 0;
    for (int s = 1; s <= n + 1; s++) {
      int v = nacf(A, n + 1, s) + nacf(B, n + 1, s) + nacf(C, n, s) + nacf(D, n, s);
      v = v < 0 ? -v : v;
      mx = v > mx ? v : mx;
    }
    maxabs[i] = mx;
  }
}

// Odd 64-bit multipliers of the key, one per shift (splitmix64 outputs, fixed).
__constant__ uint64_t kKeyMul[64] = {
    0x39E7EF6C1B54F617ULL, 0x29BB7C882170A7D7ULL, 0x45446DEFE0440477ULL, 0x9A0FC648C9C19C21ULL,
    0xDB939B7D1D9E4ACFULL, 0x958796FCC2A073FDULL, 0x4F001AA287E5A101ULL, 0x19AD5ABED7952F1DULL,
    0xB18BACE16B914A33ULL, 0x22CFCFEB9E985FBFULL, 0xDCC16F773BD10E33ULL, 0xE858FD9950CC3281ULL,
    0xE082EAAA6D1427E9ULL, 0x9214C05752910273ULL, 0x12EB34A8184E5841ULL, 0x5E132981F11873DBULL,
    0x1053A9814BC69167ULL, 0xA66BC82B20C5DCC5ULL, 0x1E5BCDFBD5B409E1ULL, 0xA80DF6AFAF6A81F5ULL,
    0xB95F8C15A4FDD58BULL, 0x120146AB0808746DULL, 0xB004AF8618026361ULL, 0x254C98A925B77EE9ULL,
    0x5BE0CC7CF6E85DA9ULL, 0xEADE1A126AC6190BULL, 0x34172784B4E05D37ULL, 0x1A4729CF3086F7F1ULL,
    0x1A7FE47FE14700B3ULL, 0x57F470CD5207D86BULL, 0x3F7060EEF64F6BF7ULL, 0x47ED631F621F1B21ULL,
    0x42946B3F061D3D05ULL, 0xB869F62456532C89ULL, 0x313D74B541ECD14FULL, 0xCC31EEA712C6DA7BULL,
    0x9651FEC138130CF1ULL, 0x413DA377C06A6005ULL, 0x4D0ABC1748D12427ULL, 0xB571932ACCC61087ULL,
    0x7B568766CB7755E3ULL, 0x574EFCA124FAEF0DULL, 0xA60EB03F3FBA60C7ULL, 0x9F27AA4A403F1B39ULL,
    0xF829834DF712FB7BULL, 0xD823EA850CF4441BULL, 0x3C62A8E8AA8F6691ULL, 0x6EF181920695A531ULL,
    0xC86C597ED57E94B9ULL, 0x09DB76C570325CE7ULL, 0x97D770D7BFC70C4FULL, 0xC4B9C52219209D7FULL,
    0x245F3965340006EDULL, 0xA3351A49368E6ACFULL, 0x7755814858AE75F9ULL, 0x5FD53C5EDDF91E3BULL,
    0x0BDAD738F57B5F1DULL, 0x9346372A11FB282FULL, 0xBFB1C8C156E4B5BBULL, 0xA57C8B14B20AB549ULL,
    0x8F7753582ECC36E3ULL, 0x81C1BF1F8C532779ULL, 0xD3FD3EE04FB9C48DULL, 0x89444C017283BBFBULL,
};

// 64-bit key of an autocorrelation vector v[1..n]: the linear form sum_s v[s] * kKeyMul[s]
// (mod 2^64), then a splitmix64-style finaliser to spread it over the table. One multiply-add
// per shift. Equal vectors give equal keys; different vectors can share a key, and the exact
// NPAF check after a key match rules those out.
template <typename F>
__device__ __forceinline__ uint64_t vec_key(F value, int n) {
  uint64_t h = 0;
  for (int s = 1; s <= n; s++) h += (uint64_t)(int64_t)value(s) * kKeyMul[s];
  h ^= h >> 31;
  h *= 0xBF58476D1CE4E5B9ULL;
  h ^= h >> 29;
  h *= 0x94D049BB133111EBULL;
  h ^= h >> 32;
  return h ? h : 1;  // 0 marks an empty slot
}

// the same autocorrelation on 32-bit words, for sequences of length <= 32 (every length the
// full-space join runs at): half the integer instructions of the 64-bit form
__device__ __forceinline__ int nacf32(uint32_t x, int L, int s) {
  if (s >= L) return 0;
  const uint32_t mask = (L - s >= 32) ? ~0u : ((1u << (L - s)) - 1u);
  return (L - s) - 2 * __popc((x ^ (x >> s)) & mask);
}

__device__ __forceinline__ uint64_t cd_key(uint64_t C, uint64_t D, int n) {
  if (n <= 32) {
    const uint32_t c = (uint32_t)C, d = (uint32_t)D;
    return vec_key([&](int s) { return -(nacf32(c, n, s) + nacf32(d, n, s)); }, n);
  }
  return vec_key([&](int s) { return -(nacf(C, n, s) + nacf(D, n, s)); }, n);
}

__device__ __forceinline__ uint64_t ab_key(uint64_t A, uint64_t B, int n) {
  if (n + 1 <= 32) {
    const uint32_t a = (uint32_t)A, b = (uint32_t)B;
    return vec_key([&](int s) { return nacf32(a, n + 1, s) + nacf32(b, n + 1, s); }, n);
  }
  return vec_key([&](int s) { return nacf(A, n + 1, s) + nacf(B, n + 1, s); }, n);
}

// table: keys[slot] (0 = empty) and idx[slot] (the C,D entry index)
__global__ void join_build_kernel(const uint64_t *__restrict__ cd, long long count, int n,
                                  unsigned long long *keys, long long *idx, unsigned long long mask,
                                  int *status) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = cd_key(cd[2 * i], cd[2 * i + 1], n);
    unsigned long long slot = k & mask;
    unsigned long long probes = 0;
    while (true) {
      unsigned long long prev = atomicCAS(keys + slot, 0ULL, k);
      if (prev == 0ULL) {
        idx[slot] = i;
        break;
      }
      slot = (slot + 1) & mask;
      if (++probes > mask) { atomicCAS(status, 0, BS_ERR_CAP); break; }  // table full
    }
  }
}

// Probe every A,B; for each table entry with the same key, verify the quad exactly and
// append it. The table's idx entries are written before their keys become visible to this
// later launch, so every key seen has its index.
__global__ void join_probe_kernel(const uint64_t *__restrict__ ab, long long count,
                                  const uint64_t *__restrict__ cd, int n,
                                  const unsigned long long *__restrict__ keys,
                                  const long long *__restrict__ idx, unsigned long long mask,
                                  uint64_t *out, unsigned long long cap, unsigned long long *nout,
                                  unsigned long long *key_hits) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t A = ab[2 * i], B = ab[2 * i + 1];
    const unsigned long long k = ab_key(A, B, n);
    unsigned long long slot = k & mask;
    while (true) {
      const unsigned long long cur = keys[slot];
      if (cur == 0ULL) break;
      if (cur == k) {
        atomicAdd(key_hits, 1ULL);
        const long long j = idx[slot];
        const uint64_t C = cd[2 * j], D = cd[2 * j + 1];
        bool ok = true;
        if (n + 1 <= 32) {
          const uint32_t a = (uint32_t)A, b = (uint32_t)B, c = (uint32_t)C, dd = (uint32_t)D;
          for (int s = 1; s <= n && ok; s++)
            ok = (nacf32(a, n + 1, s) + nacf32(b, n + 1, s) + nacf32(c, n, s) + nacf32(dd, n, s)) == 0;
        } else {
          for (int s = 1; s <= n && ok; s++)
            ok = (nacf(A, n + 1, s) + nacf(B, n + 1, s) + nacf(C, n, s) + nacf(D, n, s)) == 0;
        }
        if (ok) {
          unsigned long long o = atomicAdd(nout, 1ULL);
          if (o < cap) {
            out[4 * o] = A;
            out[4 * o + 1] = B;
            out[4 * o + 2] = C;
            out[4 * o + 3] = D;
          }
        }
      }
      slot = (slot + 1) & mask;
    }
  }
}

}  // namespace

#define CK(x)                                       \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return bs_cuda_fail(e_); \
  } while (0)

extern "C" int bs_npaf_verify_batch(bs_ctx *ctx, const uint64_t *quads, long long count,
                                    int32_t *maxabs) {
  if (!ctx || count < 0 || (count && (!quads || !maxabs))) return BS_ERR_ARG;
  if (count == 0) return BS_OK;
  CK(cudaSetDevice(ctx->device));
  uint64_t *dq = nullptr;
  int32_t *dm = nullptr;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMallocAsync(&dq, sizeof(uint64_t) * 4 * count, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dm, sizeof(int32_t) * count, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dq, quads, sizeof(uint64_t) * 4 * count, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    ctx->launches++;
    npaf_kernel<<<bs_grid_for(count, 256, 16 * ctx->num_sms), 256, 0, s>>>(dq, count, ctx->n, dm);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(maxabs, dm, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(dq, s);
  cudaFreeAsync(dm, s);
  return e == cudaSuccess ? BS_OK : bs_cuda_fail(e);
}

extern "C" int bs_join_quads(bs_ctx *ctx, const uint64_t *cd_words, long long ncd,
                             const uint64_t *ab_words, long long nab, uint64_t *out_quads,
                             long long out_cap, long long *nout, long long *key_hits) {
  if (!ctx || ncd < 0 || nab < 0 || !nout) return BS_ERR_ARG;
  if ((ncd && !cd_words) || (nab && !ab_words) || (out_cap > 0 && !out_quads)) return BS_ERR_ARG;
  *nout = 0;
  if (key_hits) *key_hits = 0;
  if (ncd == 0 || nab == 0) return BS_OK;
  CK(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  // table at <= 50% load: the next power of two >= 2 * ncd
  unsigned long long slots = 1024;
  while (slots < 2ULL * (unsigned long long)ncd) slots <<= 1;
  uint64_t *dcd = nullptr, *dab = nullptr, *dout = nullptr;
  unsigned long long *keys = nullptr, *cnt = nullptr;
  long long *idx = nullptr;
  const long long cap = out_cap > 0 ? out_cap : 1;
  cudaError_t e = cudaMallocAsync(&dcd, sizeof(uint64_t) * 2 * ncd, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dab, sizeof(uint64_t) * 2 * nab, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dout, sizeof(uint64_t) * 4 * cap, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&keys, sizeof(unsigned long long) * slots, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&idx, sizeof(long long) * slots, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&cnt, sizeof(unsigned long long) * 2, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(keys, 0, sizeof(unsigned long long) * slots, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * 2, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dcd, cd_words, sizeof(uint64_t) * 2 * ncd, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dab, ab_words, sizeof(uint64_t) * 2 * nab, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    ctx->launches++;
    join_build_kernel<<<bs_grid_for(ncd, 256, 16 * ctx->num_sms), 256, 0, s>>>(dcd, ncd, ctx->n, keys, idx,
                                                                                slots - 1, ctx->d_status);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    bs_timed_begin(ctx);
    join_probe_kernel<<<bs_grid_for(nab, 256, 16 * ctx->num_sms), 256, 0, s>>>(
        dab, nab, dcd, ctx->n, keys, idx, slots - 1, dout, (unsigned long long)cap, cnt, cnt + 1);
    bs_timed_end(ctx);
    e = cudaGetLastError();
  }
  unsigned long long h_cnt[2] = {0, 0};
  int status = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_cnt, cnt, sizeof h_cnt, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && out_cap > 0 && h_cnt[0] > 0) {
    unsigned long long k = h_cnt[0] < (unsigned long long)out_cap ? h_cnt[0] : (unsigned long long)out_cap;
    e = cudaMemcpyAsync(out_quads, dout, sizeof(uint64_t) * 4 * k, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  cudaFreeAsync(dcd, s); cudaFreeAsync(dab, s); cudaFreeAsync(dout, s);
  cudaFreeAsync(keys, s); cudaFreeAsync(idx, s); cudaFreeAsync(cnt, s);
  if (e != cudaSuccess) return bs_cuda_fail(e);
  if (status) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s);
    return status;
  }
  *nout = (long long)h_cnt[0];
  if (key_hits) *key_hits = (long long)h_cnt[1];
  return (long long)h_cnt[0] > out_cap ? BS_ERR_CAP : BS_OK;
}
