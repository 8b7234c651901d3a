// hall.cu - Theorem 2.4 spectral filter (the reference's hall_ok_pair_fast,
// src/solver/wz_match.cpp:143-168) over batches of packed (C,D) pairs.
//
// Two device forms:
//   * FP64, CUDA cores: the reference's summation order and expressions, one rounding per
//     operation (no FMA contraction), early exit at the first failing angle. Exact.
//   * tcgen05 tensor cores: every sequence's DFT at the 101 unique angles is one row of a
//     [128 x K] x [K x 208] UMMA with +-1 operands and a quantised table, accumulated exactly
//     in FP32 in TMEM. A certified margin decides almost every pair; the few pairs inside the
//     margin band are rechecked by the FP64 form. Decisions equal the FP64 form's.
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>

#include "bsfh_internal.cuh"
#include "tmem_ld.cuh"

namespace {

#define FULL_MASK 0xffffffffu

// ------------------------------------------------------------------------------------
// Shared helpers
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void set_status(int *status, int code) { atomicCAS(status, 0, code); }

// One sequence's Thm 2.4 terms at angle row jr (j-1) in the reference's order.
__device__ __forceinline__ void dft64(uint64_t x, int L, const double *c, const double *s,
                                      double &re, double &im) {
  double r = 0.0, q = 0.0;
  for (int i = 0; i < L; i++) {
    double cv = c[i], sv = s[i];
    bool plus = (x >> i) & 1ULL;
    r = __dadd_rn(r, plus ? cv : -cv);
    q = __dadd_rn(q, plus ? sv : -sv);
  }
  re = r;
  im = q;
}

// The reference's decision for one pair: at every angle X alone, Y alone, then the pair.
__device__ __forceinline__ bool hall_pair64(uint64_t x, uint64_t y, int L, double lim,
                                            const double *tc, const double *ts) {
  for (int jr = 0; jr < 200; jr++) {
    const double *c = tc + jr * L, *s = ts + jr * L;
    double rx, ix;
    dft64(x, L, c, s, rx, ix);
    double fx = __dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ix, ix));
    if (fx > lim) return false;
    double ry, iy;
    dft64(y, L, c, s, ry, iy);
    double ry2 = __dmul_rn(ry, ry), iy2 = __dmul_rn(iy, iy);
    double fy = __dadd_rn(ry2, iy2);
    double fp = __dadd_rn(__dadd_rn(fx, ry2), iy2);
    if (fy > lim || fp > lim) return false;
  }
  return true;
}

// Load the FP64 tables for rows j = 1..200, columns i < L, into shared memory.
__device__ __forceinline__ void load_tables64(double *sc, double *ss, const double *gc,
                                              const double *gs, int L) {
  for (int t = threadIdx.x; t < 200 * L; t += blockDim.x) {
    int jr = t / L, i = t - jr * L;
    sc[t] = gc[jr * BS_MAXL + i];
    ss[t] = gs[jr * BS_MAXL + i];
  }
  __syncthreads();
}

// FP64 form over all pairs, or over an index list (the margin-band recheck; the list length
// is read from device memory so it can follow the tensor-core kernel without a host sync).
__global__ void __launch_bounds__(512) hall_fp64_kernel(
    const uint64_t *__restrict__ bits, long long npairs, const unsigned *__restrict__ list,
    const unsigned long long *list_len, unsigned long long list_cap, int L, double lim,
    const double *__restrict__ gc, const double *__restrict__ gs, uint8_t *__restrict__ pass,
    unsigned long long *pass_count) {
  extern __shared__ double tabs[];
  double *sc = tabs, *ss = tabs + 200 * L;
  load_tables64(sc, ss, gc, gs, L);
  long long count = npairs;
  if (list) {
    unsigned long long n = *list_len;
    count = (long long)(n < list_cap ? n : list_cap);
  }
  unsigned local = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    long long p = list ? (long long)list[t] : t;
    bool ok = hall_pair64(bits[2 * p], bits[2 * p + 1], L, lim, sc, ss);
    pass[p] = ok ? 1 : 0;
    local += ok;
  }
  unsigned warp_sum = __reduce_add_sync(FULL_MASK, local);
  if ((threadIdx.x & 31) == 0 && warp_sum) atomicAdd(pass_count, (unsigned long long)warp_sum);
}

// The reference's test of one pair at one angle row jr (true = this angle rejects the pair).
__device__ __forceinline__ bool angle_rejects(uint64_t x, uint64_t y, int L, double lim,
                                              const double *c, const double *s) {
  double rx, ix, ry, iy;
  dft64(x, L, c, s, rx, ix);
  double fx = __dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ix, ix));
  if (fx > lim) return true;
  dft64(y, L, c, s, ry, iy);
  double ry2 = __dmul_rn(ry, ry), iy2 = __dmul_rn(iy, iy);
  double fy = __dadd_rn(ry2, iy2);
  double fp = __dadd_rn(__dadd_rn(fx, ry2), iy2);
  return fy > lim || fp > lim;
}

// Margin-band recheck: one warp per listed pair, the 200 angles split over the lanes. The
// pair passes when no angle rejects it, the same conjunction the reference evaluates.
__global__ void __launch_bounds__(256) hall_fp64_recheck_kernel(
    const uint64_t *__restrict__ bits, const unsigned *__restrict__ list,
    const unsigned long long *list_len, unsigned long long list_cap, int L, double lim,
    const double *__restrict__ gc, const double *__restrict__ gs, uint8_t *__restrict__ pass,
    unsigned long long *pass_count) {
  const unsigned long long n = *list_len;
  const long long count = (long long)(n < list_cap ? n : list_cap);
  if (count == 0) return;  // an empty band (the common case): no table to load
  extern __shared__ double tabs[];
  double *sc = tabs, *ss = tabs + 200 * L;
  load_tables64(sc, ss, gc, gs, L);
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned local = 0;
  for (long long t = w0; t < count; t += nw) {
    const long long p = (long long)list[t];
    const uint64_t x = bits[2 * p], y = bits[2 * p + 1];
    bool rej = false;
    for (int jr = lane; jr < 200 && !rej; jr += 32) rej = angle_rejects(x, y, L, lim, sc + jr * L, ss + jr * L);
    const bool ok = !__any_sync(FULL_MASK, rej);
    if (lane == 0) {
      pass[p] = ok ? 1 : 0;
      local += ok;
    }
  }
  if (lane == 0 && local) atomicAdd(pass_count, (unsigned long long)local);
}

// Second test of the margin band, exact up to a tiny certified error: a warp per listed pair,
// the 101 unique angles over the lanes. Re and Im of each sequence are int64 sums of the
// fixed-point table T = round(t * 2^30): Re = 2 * (sum of T over the +1 positions) - (row sum).
// The pair PSD is formed in FP64 from those exact integers and its maximum over the angles is
// compared with the form's certified thresholds; a pair between them goes on to the FP64 test.
__global__ void __launch_bounds__(256) hall_fix_band_kernel(
    const uint64_t *__restrict__ bits, const unsigned *__restrict__ list,
    const unsigned long long *list_len, unsigned long long list_cap, int L,
    const int64_t *__restrict__ tab, double pass_below, double reject_above,
    uint8_t *__restrict__ pass, unsigned long long *pass_count, unsigned *__restrict__ list2,
    unsigned long long *list2_len, unsigned long long list2_cap) {
  const unsigned long long n = *list_len;
  const long long count = (long long)(n < list_cap ? n : list_cap);
  if (count == 0) return;
  // The table in shared memory transposed to [position][angle] (cos rows, then sin rows), so
  // that the lanes' reads at one position are consecutive words; then the row sums.
  extern __shared__ int64_t ftab[];
  int64_t *tc = ftab, *ts = ftab + BS_TC_NANG * L;
  int64_t *sc = ftab + 2 * BS_TC_NANG * L, *ss = sc + BS_TC_NANG;
  for (int k = threadIdx.x; k < BS_TC_NANG * L; k += blockDim.x) {
    const int u = k / L, i = k - u * L;  // the device table is [angle][position]
    tc[i * BS_TC_NANG + u] = tab[k];
    ts[i * BS_TC_NANG + u] = tab[BS_TC_NANG * L + k];
  }
  for (int k = threadIdx.x; k < 2 * BS_TC_NANG; k += blockDim.x) sc[k] = tab[2 * BS_TC_NANG * L + k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  constexpr int R = (BS_TC_NANG + 31) / 32;  // angles per lane: u = lane + 32 r
  unsigned local = 0;
  for (long long t = w0; t < count; t += nw) {
    const long long p = (long long)list[t];
    const uint64_t x = bits[2 * p], y = bits[2 * p + 1];
    // one walk over each sequence's +1 positions feeds the lane's R angles at once
    int64_t rx[R], ix[R], ry[R], iy[R];
#pragma unroll
    for (int r = 0; r < R; r++) rx[r] = ix[r] = ry[r] = iy[r] = 0;
    for (uint64_t b = x; b; b &= b - 1) {
      const int i = __ffsll((long long)b) - 1;
      const int64_t *cr = tc + i * BS_TC_NANG + lane, *sr = ts + i * BS_TC_NANG + lane;
#pragma unroll
      for (int r = 0; r < R; r++)
        if (lane + 32 * r < BS_TC_NANG) {
          rx[r] += cr[32 * r];
          ix[r] += sr[32 * r];
        }
    }
    for (uint64_t b = y; b; b &= b - 1) {
      const int i = __ffsll((long long)b) - 1;
      const int64_t *cr = tc + i * BS_TC_NANG + lane, *sr = ts + i * BS_TC_NANG + lane;
#pragma unroll
      for (int r = 0; r < R; r++)
        if (lane + 32 * r < BS_TC_NANG) {
          ry[r] += cr[32 * r];
          iy[r] += sr[32 * r];
        }
    }
    double mx = 0.0;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int u = lane + 32 * r;
      if (u < BS_TC_NANG) {
        const int64_t a0 = 2 * rx[r] - sc[u], b0 = 2 * ix[r] - ss[u];
        const int64_t c0 = 2 * ry[r] - sc[u], d0 = 2 * iy[r] - ss[u];
        const double a = (double)a0, b2 = (double)b0, c = (double)c0, d = (double)d0;
        const double f = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b2, b2)),
                                   __dadd_rn(__dmul_rn(c, c), __dmul_rn(d, d))) * 0x1p-60;
        mx = fmax(mx, f);
      }
    }
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL_MASK, mx, o));
    if (lane == 0) {
      if (mx <= pass_below) {
        pass[p] = 1;
        local++;
      } else if (mx < reject_above) {
        const unsigned long long k = atomicAdd(list2_len, 1ULL);
        if (k < list2_cap) list2[k] = (unsigned)p;
      }  // else rejected: the tensor-core kernel already wrote 0
    }
  }
  if (lane == 0 && local) atomicAdd(pass_count, (unsigned long long)local);
}

__global__ void pack_kernel(const int8_t *__restrict__ rows, long long nrows, int L,
                            uint64_t *__restrict__ words, int *status) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < nrows;
       r += (long long)gridDim.x * blockDim.x) {
    const int8_t *s = rows + r * L;
    uint64_t w = 0;
    bool bad = false;
    for (int i = 0; i < L; i++) {
      int8_t v = s[i];
      w |= (uint64_t)(v == 1) << i;
      bad |= (v != 1 && v != -1);
    }
    words[r] = w;
    if (bad) set_status(status, BS_ERR_ARG);
  }
}

// ------------------------------------------------------------------------------------
// tcgen05 form
// ------------------------------------------------------------------------------------
// A tile is 128 pairs. Its C sequences are the rows of one [128 x K] operand and its D
// sequences the rows of a second, so after the MMAs TMEM lane r holds the DFT of C_r in one
// accumulator and that of D_r in another: a thread owns a whole pair and forms the pair PSD
// without exchanging values. The 208 table columns are split into the two angle blocks of
// bs_tc_row (N = 128 and N = 80); block b of a tile has its own accumulators (C and D), so
// the epilogue's reads of block 0 overlap the MMAs of block 1 and the other way round:
//   TMEM columns [0, 256): block 0 (C at 0, D at 128); [256, 416): block 1 (C at 256, D at 336).
constexpr int TC_STAGES = 4;
// warps [0, TC_PRODUCERS) producers, TC_MMA_WARP the MMA issuer (and TMEM owner), then two
// epilogue groups of four warps, each reading half of the angles of both blocks
constexpr int TC_PRODUCERS = 2;
constexpr int TC_MMA_WARP = TC_PRODUCERS;
constexpr int TC_THREADS = 32 * (TC_PRODUCERS + 1 + 8);
constexpr int TC_TILE = 128;                    // pairs per tile
constexpr int A_SEQ_BYTES = 128 * 128;          // one operand: 128 rows x 64 halves
constexpr int A_STAGE_BYTES = 2 * A_SEQ_BYTES;  // the C operand, then the D operand
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t TM_BLK1 = 256;               // first TMEM column of block 1
constexpr int N_BLK0 = 2 * BS_TC_BLK0, N_BLK1 = 2 * BS_TC_BLK1;
constexpr int TC_SLOTS = 4;  // decision slots: tiles whose two blocks may be in flight at once

struct TcParams {
  const uint64_t *bits;
  long long npairs, ntiles;
  const uint8_t *image;
  int nparts, ksteps;
  uint32_t idesc[2];  // instruction descriptors of the two angle blocks (N = 128, N = 80)
  uint32_t idesc_screen;  // the screening MMA (N = 64)
  int bits_a16;       // bits is 16-byte aligned: a pair's two words are read as one vector
  // the full test over a list of pairs (the screen's survivors): pair = list[t] for
  // t < min(*list_len, list_cap); NULL: pairs 0..npairs-1
  const unsigned *list;
  const unsigned long long *list_len;
  unsigned long long list_cap;
  // the screen's output: pairs it could not reject, appended to scr (count in count[4])
  unsigned *scr;
  unsigned long long scr_cap;
  uint32_t one2;  // two packed +1.0 halves in the operand format
  float pass_below, reject_above;
  uint8_t *pass;
  unsigned *unc;
  unsigned long long unc_cap;
  unsigned long long *count;  // [0] uncertain, [1] passes, [2] overflow
  int *status;
  float *dump;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the abort flag is raised or the cycle limit passes.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile int *abort_flag,
                                          bool honour_abort = true) {
  long long t0 = clock64();
  while (!mbar_try(a, parity)) {
    if (honour_abort && *abort_flag) return false;
    if ((unsigned long long)(clock64() - t0) > BS_WAIT_CYCLES) return false;
  }
  return true;
}
// arrive once on the mbarrier and add `bytes` to the transaction count of its current phase
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// One contiguous global -> shared copy on the async proxy, completing `bytes` on the mbarrier:
// both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}

// Shared-memory matrix descriptor, K-major operand in the 128-byte swizzle layout:
// start address >> 4, leading offset 1 (unused for this layout), stride offset 1024 B
// between 8-row groups, descriptor version 1, layout type 2 (128B swizzle).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// The pair PSD at two adjacent angles with the packed f32x2 multiply and FMAs:
// f = ((imC^2 + reC^2) + imD^2) + reD^2 per element, each step rounded to nearest.
__device__ __forceinline__ void pair_psd2(const float *rc, const float *ic, const float *rd,
                                          const float *id, float &f0, float &f1) {
  uint64_t a, b, c, d, r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(rc[0]), "f"(rc[1]));
  asm("mov.b64 %0, {%1, %2};" : "=l"(b) : "f"(ic[0]), "f"(ic[1]));
  asm("mov.b64 %0, {%1, %2};" : "=l"(c) : "f"(rd[0]), "f"(rd[1]));
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(id[0]), "f"(id[1]));
  asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(r) : "l"(b));
  asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(r) : "l"(a));
  asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(r) : "l"(d));
  asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(r) : "l"(c));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(f0), "=f"(f1) : "l"(r));
}

__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Four operand halves per 32-bit word pair: the 8 bits of `byte` (bit set = +1) as 8 halves
// +-1.0 in the operand format. neg2 holds two -1.0 halves; z = byte * 0x8001 places bit i at
// positions i and i + 15, so a shift brings bits 2k and 2k + 1 to the sign positions 15 and 31
// of word k, and the XOR turns the -1.0 of every set bit into +1.0.
__device__ __forceinline__ uint4 expand_byte(uint32_t byte, uint32_t neg2) {
  const uint32_t z = byte * 0x8001u;
  uint4 v;
  v.x = neg2 ^ ((z << 15) & 0x80008000u);
  v.y = neg2 ^ ((z << 13) & 0x80008000u);
  v.z = neg2 ^ ((z << 11) & 0x80008000u);
  v.w = neg2 ^ ((z << 9) & 0x80008000u);
  return v;
}

// The C and D words of one pair (one 16-byte load when the array is 16-byte aligned).
__device__ __forceinline__ uint4 load_pair(const uint64_t *bits, long long pair, int a16) {
  if (a16) return __ldg((const uint4 *)(bits + 2 * pair));
  const unsigned long long c = __ldg((const unsigned long long *)(bits + 2 * pair));
  const unsigned long long d = __ldg((const unsigned long long *)(bits + 2 * pair + 1));
  return make_uint4((uint32_t)c, (uint32_t)(c >> 32), (uint32_t)d, (uint32_t)(d >> 32));
}

// One sequence word as one operand row (row r of a 128-row K-major operand, 128B swizzle):
// chunk c (16 bytes, elements 8c..8c+7) goes to chunk c ^ (r & 7) of the row.
__device__ __forceinline__ void put_row(uint8_t *A, int r, uint64_t w, int nchunks, uint32_t neg2) {
#pragma unroll
  for (int c = 0; c < 8; c++) {
    if (c < nchunks)
      *(uint4 *)(A + r * 128 + ((c ^ (r & 7)) << 4)) =
          expand_byte((uint32_t)(w >> (8 * c)) & 0xFFu, neg2);
  }
}

// the angle u of a table slot (-1: a padding slot); for the diagnostic dump only
__device__ __forceinline__ int u_of_slot(int slot) {
  for (int u = 0; u < BS_TC_NANG; u++)
    if (bs_tc_slot_of(u) == slot) return u;
  return -1;
}

__global__ void __launch_bounds__(TC_THREADS, 1) hall_tc_kernel(TcParams P) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *sA = base;
  uint8_t *sB = sA + TC_STAGES * A_STAGE_BYTES;
  float *pmax = (float *)(sB + P.nparts * BS_TC_PART_BYTES);  // [TC_SLOTS][2][128]
  int *pcnt = (int *)(pmax + TC_SLOTS * 2 * TC_TILE);         // [TC_SLOTS][4]
  uint64_t *bars = (uint64_t *)(pcnt + TC_SLOTS * 4);
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * TC_STAGES + 4);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + TC_STAGES);
  const uint32_t tfull0 = smem_u32(bars + 2 * TC_STAGES), tempty0 = tfull0 + 16;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long G = gridDim.x;

  {  // table image -> shared memory
    const uint4 *src = (const uint4 *)P.image;
    uint4 *dst = (uint4 *)sB;
    int nvec = P.nparts * BS_TC_PART_BYTES / 16;
    for (int i = threadIdx.x; i < nvec; i += TC_THREADS) dst[i] = src[i];
  }
  for (int i = threadIdx.x; i < TC_SLOTS * 4; i += TC_THREADS) pcnt[i] = 0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, 8);  // every epilogue warp releases every block
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == TC_MMA_WARP) tc_alloc(smem_u32(tmem_slot), TMEM_COLS);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // the pairs of this launch: P.npairs, or the length of the list (written by the screen)
  long long count = P.npairs, ntiles = P.ntiles;
  if (P.list) {
    const unsigned long long len = *P.list_len;
    count = (long long)(len < P.list_cap ? len : P.list_cap);
    ntiles = (count + TC_TILE - 1) / TC_TILE;
  }

  if (warp < TC_PRODUCERS) {
    // ---- producers: packed words -> +-1 operand rows. Producer p fills the CTA's tiles
    // it = p, p + TC_PRODUCERS, ...; lane l handles pairs l + 32 rr of the tile (one 16-byte
    // load: the pair's C and D words), and the next tile's words are loaded before the current
    // tile is expanded so the global-load latency overlaps the work. ----
    const uint32_t neg2 = P.one2 | 0x80008000u;
    const int nchunks = 2 * P.ksteps;
    auto fetch = [&](long long t) -> uint4 {
      if (t >= count) return make_uint4(0, 0, 0, 0);
      const long long pair = P.list ? (long long)__ldg(P.list + t) : t;
      return load_pair(P.bits, pair, P.bits_a16);
    };
    int it = warp;
    long long tile = blockIdx.x + (long long)it * G;
    uint4 wv[4];
#pragma unroll
    for (int rr = 0; rr < 4; rr++) wv[rr] = tile < ntiles ? fetch(tile * TC_TILE + lane + 32 * rr) : make_uint4(0, 0, 0, 0);
    while (tile < ntiles) {
      const long long next = tile + TC_PRODUCERS * G;
      uint4 nw[4];
#pragma unroll
      for (int rr = 0; rr < 4; rr++) nw[rr] = next < ntiles ? fetch(next * TC_TILE + lane + 32 * rr) : make_uint4(0, 0, 0, 0);
      const int s = it % TC_STAGES;
      const uint32_t par = ((it / TC_STAGES) & 1) ^ 1;
      if (!mbar_wait(empty0 + 8 * s, par, abort_flag)) {
        if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
        break;
      }
      uint8_t *AC = sA + s * A_STAGE_BYTES, *AD = AC + A_SEQ_BYTES;
#pragma unroll
      for (int rr = 0; rr < 4; rr++) {
        const int r = lane + 32 * rr;
        put_row(AC, r, ((uint64_t)wv[rr].y << 32) | wv[rr].x, nchunks, neg2);
        put_row(AD, r, ((uint64_t)wv[rr].w << 32) | wv[rr].z, nchunks, neg2);
      }
      fence_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(full0 + 8 * s);
#pragma unroll
      for (int rr = 0; rr < 4; rr++) wv[rr] = nw[rr];
      tile = next;
      it += TC_PRODUCERS;
    }
  } else if (warp == TC_MMA_WARP) {
    // ---- MMA issuer (one thread): per tile, block 0 then block 1, each the C operand into
    // the block's C accumulator and the D operand into its D accumulator ----
    if (lane == 0) {
      const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
      int it = 0, last = -1;
      for (long long tile = blockIdx.x; tile < ntiles; tile += G, it++) {
        const int s = it % TC_STAGES;
        if (!mbar_wait(full0 + 8 * s, (it / TC_STAGES) & 1, abort_flag)) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        bool ok = true;
        for (int blk = 0; blk < 2 && ok; blk++) {
          if (!mbar_wait(tempty0 + 8 * blk, (it & 1) ^ 1, abort_flag)) {
            if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d0 = tmem + (blk ? TM_BLK1 : 0u);
          const uint32_t nblk = blk ? (uint32_t)N_BLK1 : (uint32_t)N_BLK0;
          const uint32_t b_off = blk ? (uint32_t)(N_BLK0 * 128) : 0u;
          for (int seq = 0; seq < 2; seq++) {
            uint32_t acc = 0;
            for (int p = 0; p < P.nparts; p++)
              for (int k = 0; k < P.ksteps; k++) {
                const uint64_t ad = sw128_desc(a_base + s * A_STAGE_BYTES + seq * A_SEQ_BYTES + k * 32);
                const uint64_t bd = sw128_desc(b_base + p * BS_TC_PART_BYTES + b_off + k * 32);
                tc_mma(d0 + seq * nblk, ad, bd, P.idesc[blk], acc);
                acc = 1;
              }
          }
          tc_commit(tfull0 + 8 * blk);
        }
        if (!ok) break;
        tc_commit(empty0 + 8 * s);
        last = it;
      }
      // Before TMEM is released, the last issued MMAs must have finished.
      if (last >= 0) mbar_wait(tfull0 + 8, last & 1, abort_flag, false);
    }
    __syncwarp();
  } else {
    // ---- epilogue: both groups read both blocks of every tile, group g the angles
    // [32g, 32g + 32) of block 0 and [20g, 20g + 20) of block 1; warp quarter q owns pairs
    // 32q..32q+31 of the tile, one per lane. A group copies its columns of a block to
    // registers in one round of loads and releases the block at once (the MMA issuer waits
    // for both groups), then forms the pair PSDs. Of the two groups, the one that finishes
    // a tile second takes the max of both (shared memory slot, a counter per quarter) and
    // decides the 32 pairs. ----
    const int g = (warp - TC_MMA_WARP - 1) >> 2;
    const int q = warp & 3;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    const int row = q * 32 + lane;
    // block 0 columns: [Re slots 0..31][Im 0..31][Re 32..63][Im 32..63]; block 1: [Re][Im]
    const uint32_t tC0 = tmem + lane_off + 64u * g;                 // block 0, C accumulator
    const uint32_t tC1 = tmem + lane_off + TM_BLK1 + 20u * g;       // block 1, C accumulator
    const uint32_t nb0 = 32, nb1 = BS_TC_BLK1;                     // Im at column + nb
    for (int it = 0;; it++) {
      const long long tile = blockIdx.x + (long long)it * G;
      if (tile >= ntiles) break;
      const long long t = tile * TC_TILE + row;
      const long long pair = t < count ? (P.list ? (long long)__ldg(P.list + t) : t) : -1;
      float *dump = (P.dump && pair >= 0) ? P.dump + (size_t)pair * 2 * BS_TC_COLS : nullptr;
      float mx = 0.0f;
      bool ok = true;
      {  // block 0: 32 angles
        // warp-uniform outcome: the TMEM loads below are .sync.aligned
        ok = __all_sync(FULL_MASK, mbar_wait(tfull0, it & 1, abort_flag));
        if (!ok) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        tc_fence_after();
        float v[128];  // Re C, Im C, Re D, Im D at the group's 32 angles
        tmem_ld_32x4(tC0, tC0 + nb0, tC0 + N_BLK0, tC0 + N_BLK0 + nb0, v);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tempty0);
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
          float f0, f1;
          pair_psd2(v + k, v + 32 + k, v + 64 + k, v + 96 + k, f0, f1);
          mx = fmax3(mx, f0, f1);
        }
        if (dump)
#pragma unroll
          for (int k = 0; k < 32; k++) {
            const int u = u_of_slot(32 * g + k);
            dump[u] = v[k];
            dump[BS_TC_IM0 + u] = v[32 + k];
            dump[BS_TC_COLS + u] = v[64 + k];
            dump[BS_TC_COLS + BS_TC_IM0 + u] = v[96 + k];
          }
      }
      {  // block 1: 20 angles
        ok = __all_sync(FULL_MASK, mbar_wait(tfull0 + 8, it & 1, abort_flag));
        if (!ok) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        tc_fence_after();
        float v[80];  // Re C, Im C, Re D, Im D at the group's 20 angles
        tmem_ld_20x4(tC1, tC1 + nb1, tC1 + N_BLK1, tC1 + N_BLK1 + nb1, v);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tempty0 + 8);
#pragma unroll
        for (int k = 0; k < 20; k += 2) {
          float f0, f1;
          pair_psd2(v + k, v + 20 + k, v + 40 + k, v + 60 + k, f0, f1);
          mx = fmax3(mx, f0, f1);
        }
        if (dump)
#pragma unroll
          for (int k = 0; k < 20; k++) {
            const int u = u_of_slot(BS_TC_BLK0 + 20 * g + k);
            if (u < 0) continue;  // a padding slot
            dump[u] = v[k];
            dump[BS_TC_IM0 + u] = v[20 + k];
            dump[BS_TC_COLS + u] = v[40 + k];
            dump[BS_TC_COLS + BS_TC_IM0 + u] = v[60 + k];
          }
      }
      // hand-over between the two groups: the second to finish this tile decides
      const int slot = it & (TC_SLOTS - 1);
      pmax[(slot * 2 + g) * TC_TILE + row] = mx;
      __threadfence_block();
      __syncwarp();
      int order = 0;
      if (lane == 0) order = atomicAdd(&pcnt[slot * 4 + q], 1);
      order = __shfl_sync(FULL_MASK, order, 0);
      if (order == 1) {
        __threadfence_block();
        const float m = fmaxf(mx, pmax[(slot * 2 + (g ^ 1)) * TC_TILE + row]);
        const bool mine = pair >= 0;
        const bool sure_pass = mine && m <= P.pass_below;
        const bool unsure = mine && m > P.pass_below && m < P.reject_above;
        if (mine) P.pass[pair] = sure_pass ? 1 : 0;
        if (unsure) {
          unsigned long long k = atomicAdd(P.count, 1ULL);
          if (k < P.unc_cap) P.unc[k] = (unsigned)pair;
          else atomicExch(P.count + 2, 1ULL);
        }
        const unsigned np = __popc(__ballot_sync(FULL_MASK, sure_pass));
        if (lane == 0) {
          if (np) atomicAdd(P.count + 1, (unsigned long long)np);
          atomicExch(&pcnt[slot * 4 + q], 0);
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == TC_MMA_WARP) tc_dealloc(tmem, TMEM_COLS);
}

// ---- the screening pass: the 32 screening angles (table slots 0..31) of every pair ----
// The same producers and operands as the full test, but one MMA of N = 64 per sequence and
// part, into one of four TMEM buffers of 128 columns (C: Re 0..31, Im 32..63; D: 64..127),
// so the MMA runs up to three tiles ahead of the epilogue. A thread reads its pair's 128
// accumulator values, releases the buffer and takes the max pair PSD over the 32 angles: at
// or above the certified reject_above the pair is rejected for good (the max over all angles
// can only be larger); otherwise its index goes to the survivor list, which the full test
// then decides. The full test reads four accumulator values per angle and pair out of TMEM,
// and that read, not the MMA, bounds it; on the microbench mix and on stream leaves about
// 2-3 % of pairs survive the screen, so the full reads are paid for those alone.
constexpr int SC_BUFS = 4;
constexpr int SC_RUN = 256;  // survivors a screen epilogue warp holds before it writes them out
constexpr int SC_RING = 4;   // tiles of packed words each screen producer has in flight
// Warp roles of the screen: SC_PRODUCERS producer warps (the expansion of packed words to
// operand rows is most of the kernel's instructions, so it is spread over the SM
// sub-partitions), one MMA warp, and SC_GROUPS epilogue groups of four warps. With more than
// two groups a warp reads its pair's 128 values in two halves of 64 to fit the register budget.
constexpr int SC_PRODUCERS = 2;
constexpr int SC_MMA_WARP = SC_PRODUCERS;
constexpr int SC_GROUPS = 2;
constexpr bool SC_HALVES = SC_GROUPS > 2;
constexpr int SC_EPI = 4 * SC_GROUPS;  // epilogue warps
constexpr int SC_THREADS = 32 * (SC_PRODUCERS + 1 + SC_EPI);
constexpr int SC_RAW_BYTES = TC_TILE * 16;  // one tile of pairs: two 8-byte words each
constexpr uint32_t SC_COLS = 128;  // TMEM columns per buffer (C then D, 64 each)

__global__ void __launch_bounds__(SC_THREADS, 1) hall_screen_kernel(TcParams P) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *sA = base;
  uint8_t *sB = sA + TC_STAGES * A_STAGE_BYTES;  // rows 0..63 of each part, 8 KB per part
  uint8_t *sraw = sB + P.nparts * 64 * 128;      // [SC_PRODUCERS][SC_RING] tiles of packed words
  uint32_t *srun = (uint32_t *)(sraw + SC_PRODUCERS * SC_RING * SC_RAW_BYTES);  // [SC_EPI][SC_RUN]
  uint64_t *bars = (uint64_t *)(srun + SC_EPI * SC_RUN);
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * TC_STAGES + 2 * SC_BUFS + SC_PRODUCERS * SC_RING);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + TC_STAGES);
  const uint32_t tfull0 = smem_u32(bars + 2 * TC_STAGES), tempty0 = tfull0 + 8 * SC_BUFS;
  const uint32_t raw0 = tempty0 + 8 * SC_BUFS;  // [SC_PRODUCERS][SC_RING]: a ring tile landed
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long G = gridDim.x;

  {  // rows 0..63 (the screening angles' cos and sin rows) of each part -> shared memory
    for (int p = 0; p < P.nparts; p++) {
      const uint4 *src = (const uint4 *)(P.image + (size_t)p * BS_TC_PART_BYTES);
      uint4 *dst = (uint4 *)(sB + p * 64 * 128);
      for (int i = threadIdx.x; i < 64 * 128 / 16; i += SC_THREADS) dst[i] = src[i];
    }
  }
  if (threadIdx.x == 0) {
    for (int st = 0; st < TC_STAGES; st++) {
      mbar_init(full0 + 8 * st, 1);
      mbar_init(empty0 + 8 * st, 1);
    }
    for (int b = 0; b < SC_BUFS; b++) {
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, 4);  // the four warps of the group that reads the buffer
    }
    for (int r = 0; r < SC_PRODUCERS * SC_RING; r++) mbar_init(raw0 + 8 * r, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == SC_MMA_WARP) tc_alloc(smem_u32(tmem_slot), TMEM_COLS);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < SC_PRODUCERS) {
    const uint32_t neg2 = P.one2 | 0x80008000u;
    const int nchunks = 2 * P.ksteps;
    const long long stride = (long long)SC_PRODUCERS * G;  // between this warp's tiles
    int it = warp;
    long long tile = blockIdx.x + (long long)it * G;
    auto expand = [&](const uint4 *wv, int st) {
      uint8_t *AC = sA + st * A_STAGE_BYTES, *AD = AC + A_SEQ_BYTES;
#pragma unroll
      for (int rr = 0; rr < 4; rr++) {
        const int r = lane + 32 * rr;
        put_row(AC, r, ((uint64_t)wv[rr].y << 32) | wv[rr].x, nchunks, neg2);
        put_row(AD, r, ((uint64_t)wv[rr].w << 32) | wv[rr].z, nchunks, neg2);
      }
      fence_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(full0 + 8 * st);
    };
    if (P.bits_a16) {
      // The warp's tiles arrive by bulk copies into its ring, SC_RING tiles ahead of the one
      // it expands; the j-th tile of the warp lands in slot j % SC_RING, phase (j / SC_RING) & 1.
      // A tile is 128 pairs of two words, 2 KB, contiguous (the last one shorter).
      uint8_t *ring = sraw + warp * SC_RING * SC_RAW_BYTES;
      const uint32_t rbar = raw0 + 8 * warp * SC_RING;
      auto issue = [&](long long t, int slot) {
        const long long p0 = t * TC_TILE;
        const long long np = P.npairs - p0 < TC_TILE ? P.npairs - p0 : TC_TILE;
        const uint32_t bytes = (uint32_t)np * 16u;
        mbar_expect_tx(rbar + 8 * slot, bytes);
        bulk_g2s(smem_u32(ring + slot * SC_RAW_BYTES), P.bits + 2 * p0, bytes, rbar + 8 * slot);
      };
      long long issued = 0, j = 0;  // copies issued and tiles consumed by this warp (uniform)
      for (int r = 0; r < SC_RING; r++)
        if (tile + r * stride < P.ntiles) {
          if (lane == 0) issue(tile + r * stride, r);
          issued++;
        }
      while (tile < P.ntiles) {
        const int slot = (int)(j % SC_RING);
        if (!__all_sync(FULL_MASK, mbar_wait(rbar + 8 * slot, (uint32_t)(j / SC_RING) & 1, abort_flag))) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        uint4 wv[4];
        const uint4 *src = (const uint4 *)(ring + slot * SC_RAW_BYTES);
#pragma unroll
        for (int rr = 0; rr < 4; rr++) wv[rr] = src[lane + 32 * rr];
        __syncwarp();
        j++;
        const long long ahead = tile + SC_RING * stride;
        if (ahead < P.ntiles) {  // refill the slot just read
          if (lane == 0) {
            fence_async_smem();
            issue(ahead, slot);
          }
          issued++;
        }
        const int st = it % TC_STAGES;
        if (!__all_sync(FULL_MASK, mbar_wait(empty0 + 8 * st, ((it / TC_STAGES) & 1) ^ 1, abort_flag))) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        expand(wv, st);
        tile += stride;
        it += SC_PRODUCERS;
      }
      // after an abort: wait (bounded) for the copies still landing in the ring before the
      // block exits
      for (long long k = j; k < issued; k++)
        mbar_wait(rbar + 8 * (int)(k % SC_RING), (uint32_t)(k / SC_RING) & 1, abort_flag, false);
    } else {
      auto fetch = [&](long long pair) -> uint4 {
        return pair < P.npairs ? load_pair(P.bits, pair, 0) : make_uint4(0, 0, 0, 0);
      };
      uint4 wv[4];
#pragma unroll
      for (int rr = 0; rr < 4; rr++) wv[rr] = tile < P.ntiles ? fetch(tile * TC_TILE + lane + 32 * rr) : make_uint4(0, 0, 0, 0);
      while (tile < P.ntiles) {
        const long long next = tile + stride;
        uint4 nw[4];
#pragma unroll
        for (int rr = 0; rr < 4; rr++) nw[rr] = next < P.ntiles ? fetch(next * TC_TILE + lane + 32 * rr) : make_uint4(0, 0, 0, 0);
        const int st = it % TC_STAGES;
        if (!mbar_wait(empty0 + 8 * st, ((it / TC_STAGES) & 1) ^ 1, abort_flag)) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        expand(wv, st);
#pragma unroll
        for (int rr = 0; rr < 4; rr++) wv[rr] = nw[rr];
        tile = next;
        it += SC_PRODUCERS;
      }
    }
  } else if (warp == SC_MMA_WARP) {
    if (lane == 0) {
      const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
      int it = 0, last = -1;
      for (long long tile = blockIdx.x; tile < P.ntiles; tile += G, it++) {
        const int st = it % TC_STAGES, b = it % SC_BUFS;
        if (!mbar_wait(full0 + 8 * st, (it / TC_STAGES) & 1, abort_flag) ||
            !mbar_wait(tempty0 + 8 * b, ((it / SC_BUFS) & 1) ^ 1, abort_flag)) {
          if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
          break;
        }
        tc_fence_after();
        for (int seq = 0; seq < 2; seq++) {
          uint32_t acc = 0;
          for (int p = 0; p < P.nparts; p++)
            for (int k = 0; k < P.ksteps; k++) {
              const uint64_t ad = sw128_desc(a_base + st * A_STAGE_BYTES + seq * A_SEQ_BYTES + k * 32);
              const uint64_t bd = sw128_desc(b_base + p * 64 * 128 + k * 32);
              tc_mma(tmem + b * SC_COLS + seq * 64, ad, bd, P.idesc_screen, acc);
              acc = 1;
            }
        }
        tc_commit(empty0 + 8 * st);
        tc_commit(tfull0 + 8 * b);
        last = it;
      }
      if (last >= 0) mbar_wait(tfull0 + 8 * (last % SC_BUFS), (last / SC_BUFS) & 1, abort_flag, false);
    }
    __syncwarp();
  } else {
    // ---- epilogue: group g reads the tiles it = g, g + SC_GROUPS, ... (buffer it % 4) ----
    const int g = (warp - SC_MMA_WARP - 1) >> 2;
    const int q = warp & 3;
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    const int row = q * 32 + lane;
    // Survivors collect in the warp's own shared-memory run and go to the list in batches,
    // one global atomic per batch, so no tile waits for an atomic's round trip.
    uint32_t *run = srun + (warp - SC_MMA_WARP - 1) * SC_RUN;
    int nrun = 0;
    auto flush = [&]() {
      __syncwarp();
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(P.count + 4, (unsigned long long)nrun);
      base = __shfl_sync(FULL_MASK, base, 0);
      bool over = false;
      for (int i = lane; i < nrun; i += 32) {
        if (base + i < P.scr_cap) P.scr[base + i] = run[i];
        else over = true;
      }
      if (__any_sync(FULL_MASK, over) && lane == 0) atomicExch(P.count + 2, 1ULL);
      __syncwarp();
      nrun = 0;
    };
    for (int it = g;; it += SC_GROUPS) {
      const long long tile = blockIdx.x + (long long)it * G;
      if (tile >= P.ntiles) break;
      const int b = it % SC_BUFS;
      const bool ready = __all_sync(FULL_MASK, mbar_wait(tfull0 + 8 * b, (it / SC_BUFS) & 1, abort_flag));
      if (!ready) {
        if (!*abort_flag) { set_status(P.status, BS_ERR_TIMEOUT); *abort_flag = 1; }
        break;
      }
      tc_fence_after();
      const uint32_t t0 = tmem + lane_off + b * SC_COLS;
      float mx = 0.0f;
      if (SC_HALVES) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          float v[64];  // Re C, Im C, Re D, Im D at screening angles 16h .. 16h + 15
          tmem_ld_16x4(t0 + 16 * h, t0 + 32 + 16 * h, t0 + 64 + 16 * h, t0 + 96 + 16 * h, v);
          if (h == 1) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty0 + 8 * b);
          }
#pragma unroll
          for (int k = 0; k < 16; k += 2) {
            float f0, f1;
            pair_psd2(v + k, v + 16 + k, v + 32 + k, v + 48 + k, f0, f1);
            mx = fmax3(mx, f0, f1);
          }
        }
      } else {
        float v[128];  // Re C, Im C, Re D, Im D at the 32 screening angles
        tmem_ld_32x4(t0, t0 + 32, t0 + 64, t0 + 96, v);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tempty0 + 8 * b);
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
          float f0, f1;
          pair_psd2(v + k, v + 32 + k, v + 64 + k, v + 96 + k, f0, f1);
          mx = fmax3(mx, f0, f1);
        }
      }
      const long long pair = tile * TC_TILE + row;
      const bool mine = pair < P.npairs;
      const bool keep = mine && mx < P.reject_above;
      if (mine && !keep) P.pass[pair] = 0;
      const unsigned ball = __ballot_sync(FULL_MASK, keep);
      if (keep) run[nrun + __popc(ball & ((1u << lane) - 1u))] = (uint32_t)pair;
      nrun += __popc(ball);
      if (nrun > SC_RUN - 32) flush();
    }
    if (nrun) flush();
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == SC_MMA_WARP) tc_dealloc(tmem, TMEM_COLS);
}

size_t screen_smem_bytes(int nparts) {
  return 1024 + (size_t)TC_STAGES * A_STAGE_BYTES + (size_t)nparts * 64 * 128 +
         (size_t)SC_PRODUCERS * SC_RING * SC_RAW_BYTES + sizeof(uint32_t) * SC_EPI * SC_RUN +
         (2 * TC_STAGES + 2 * SC_BUFS + SC_PRODUCERS * SC_RING) * 8 + 16;
}

size_t tc_smem_bytes(int nparts) {
  return 1024 + (size_t)TC_STAGES * A_STAGE_BYTES + (size_t)nparts * BS_TC_PART_BYTES +
         sizeof(float) * TC_SLOTS * 2 * TC_TILE + sizeof(int) * TC_SLOTS * 4 +
         (2 * TC_STAGES + 4) * 8 + 16;
}

// Instruction descriptors (kind::f16): D fp32, A and B of format fmt (0 f16, 1 bf16), both
// K-major, M = 128, N = 128 for angle block 0 and N = 80 for block 1.
void tc_idesc(int fmt, uint32_t idesc[2]) {
  const uint32_t base = (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) |
                        ((uint32_t)(128 >> 4) << 24);
  idesc[0] = base | ((uint32_t)(N_BLK0 >> 3) << 17);
  idesc[1] = base | ((uint32_t)(N_BLK1 >> 3) << 17);
}
uint32_t tc_idesc_screen(int fmt) {
  return (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)(128 >> 4) << 24) |
         ((uint32_t)(64 >> 3) << 17);
}

}  // namespace

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------
#define CK(x)                                       \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return bs_cuda_fail(e_); \
  } while (0)

// Shared-memory opt-ins of the Hall kernels (the tensor-core kernel takes ~100 KB, the FP64
// kernels up to 200 KB). The attribute belongs to the device that is current when it is set,
// so it is set once per device, with that device current; serving slots call from several
// host threads, and one process may hold contexts on several GPUs. A failed attempt is
// retried by the next call.
static int hall_kernel_attrs(int dev) {
  static std::atomic<bool> done[64];
  static std::mutex mu;
  if (dev < 0 || dev >= 64) return BS_ERR_ARG;
  if (done[dev].load(std::memory_order_acquire)) return BS_OK;
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev].load(std::memory_order_relaxed)) return BS_OK;
  const int fp64_smem = (int)(sizeof(double) * 2 * 200 * BS_MAXL);
  CK(cudaFuncSetAttribute(hall_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, fp64_smem));
  CK(cudaFuncSetAttribute(hall_fp64_recheck_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          fp64_smem));
  CK(cudaFuncSetAttribute(hall_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)tc_smem_bytes(2)));
  CK(cudaFuncSetAttribute(hall_screen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)screen_smem_bytes(2)));
  CK(cudaFuncSetAttribute(hall_fix_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)(sizeof(int64_t) * BS_FIX_WORDS)));
  done[dev].store(true, std::memory_order_release);
  return BS_OK;
}

static int launch_fp64(bs_ctx *ctx, const uint64_t *d_bits, long long npairs,
                       const unsigned *list, const unsigned long long *list_len,
                       unsigned long long list_cap, uint8_t *d_pass, int L) {
  size_t smem = sizeof(double) * 2 * 200 * L;
  if (list) {  // the margin band after the tensor-core kernel: a warp per pair on every SM
    ctx->launches++;
    hall_fp64_recheck_kernel<<<ctx->num_sms, 256, smem, ctx->stream>>>(
        d_bits, list, list_len, list_cap, L, ctx->lim, ctx->d_cos, ctx->d_sin, d_pass,
        ctx->d_count + 1);
    CK(cudaGetLastError());
    return BS_OK;
  }
  int grid = bs_grid_for(npairs, 512, ctx->num_sms);
  bs_timed_begin(ctx);  // the FP64 form alone: it is the dominant kernel of the call
  hall_fp64_kernel<<<grid, 512, smem, ctx->stream>>>(d_bits, npairs, nullptr, nullptr, 0, L,
                                                     ctx->lim, ctx->d_cos, ctx->d_sin, d_pass,
                                                     ctx->d_count + 1);
  bs_timed_end(ctx);
  CK(cudaGetLastError());
  return BS_OK;
}

// The tensor-core test of a batch: the screen over every pair (rejects most of them and lists
// the rest in d_scr), then the full test over that list. With a dump (diagnostics) the full
// test runs over every pair and the screen is skipped. Both kernels are one timed section.
static int launch_tc(bs_ctx *ctx, int mode, const uint64_t *d_bits, long long npairs,
                     uint8_t *d_pass, float *d_dump, int L) {
  const bs_hall_tc_form &F = (L == ctx->n) ? ctx->tc[mode] : ctx->tc_ab[mode];
  TcParams P;
  memset(&P, 0, sizeof P);
  P.bits = d_bits;
  P.npairs = npairs;
  P.ntiles = (npairs + TC_TILE - 1) / TC_TILE;
  P.bits_a16 = ((uintptr_t)d_bits & 15) == 0;
  P.image = F.d_image;
  P.nparts = F.nparts;
  P.ksteps = (L + 15) / 16;
  tc_idesc(F.fmt, P.idesc);
  P.idesc_screen = tc_idesc_screen(F.fmt);
  P.one2 = F.fmt ? 0x3F803F80u : 0x3C003C00u;
  P.pass_below = F.pass_below;
  P.reject_above = F.reject_above;
  P.pass = d_pass;
  P.unc = ctx->d_unc;
  P.unc_cap = (unsigned long long)ctx->unc_cap;
  P.count = ctx->d_count;
  P.status = ctx->d_status;
  P.dump = d_dump;
  const long long grid = P.ntiles < ctx->num_sms ? (P.ntiles < 1 ? 1 : P.ntiles) : ctx->num_sms;
  bs_timed_begin(ctx);
  if (!d_dump) {
    P.scr = ctx->d_scr;
    P.scr_cap = (unsigned long long)ctx->scr_cap;
    hall_screen_kernel<<<(int)grid, SC_THREADS, screen_smem_bytes(F.nparts), ctx->stream>>>(P);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { bs_timed_end(ctx); return bs_cuda_fail(e); }
    ctx->launches++;
    // the full test over the survivors (their count is read on the device)
    P.list = ctx->d_scr;
    P.list_len = ctx->d_count + 4;
    P.list_cap = (unsigned long long)ctx->scr_cap;
    P.scr = nullptr;
  }
  hall_tc_kernel<<<(int)grid, TC_THREADS, tc_smem_bytes(F.nparts), ctx->stream>>>(P);
  bs_timed_end(ctx);
  CK(cudaGetLastError());
  return BS_OK;
}

// The band's fixed-point test: from the tensor-core list (d_unc, d_count[0]) to the FP64
// list (d_unc2, d_count[3]).
static int launch_fix(bs_ctx *ctx, const uint64_t *d_bits, uint8_t *d_pass, int L) {
  const bs_hall_fix_form &F = ctx->fix[L == ctx->n ? 0 : 1];
  const size_t smem = sizeof(int64_t) * (2 * BS_TC_NANG * L + 2 * BS_TC_NANG);
  ctx->launches++;
  hall_fix_band_kernel<<<ctx->num_sms, 256, smem, ctx->stream>>>(
      d_bits, ctx->d_unc, ctx->d_count, (unsigned long long)ctx->unc_cap, L, F.d_tab,
      F.pass_below, F.reject_above, d_pass, ctx->d_count + 1, ctx->d_unc2, ctx->d_count + 3,
      (unsigned long long)ctx->unc2_cap);
  CK(cudaGetLastError());
  return BS_OK;
}

static int hall_dev(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                    uint8_t *d_pass, bs_hall_stats *stats, float *d_dump, int L) {
  if (!ctx || (L != ctx->n && L != ctx->n1)) return BS_ERR_ARG;
  if (!ctx || npairs < 0 || (npairs && (!d_bits || !d_pass))) return BS_ERR_ARG;
  if (mode < BS_HALL_FP64 || mode > BS_HALL_TC_BF16X2) return BS_ERR_ARG;
  if (npairs >= (1LL << 32)) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  if (int rc = hall_kernel_attrs(ctx->device)) return rc;
  CK(cudaMemsetAsync(ctx->d_count, 0, sizeof(unsigned long long) * 8, ctx->stream));
  if (npairs > 0) {
    if (mode == BS_HALL_FP64) {
      int rc = launch_fp64(ctx, d_bits, npairs, nullptr, nullptr, 0, d_pass, L);
      if (rc) return rc;
    } else {
      int rc = bs_ensure_dev((void **)&ctx->d_unc, &ctx->unc_cap, npairs, sizeof(unsigned));
      if (!rc) rc = bs_ensure_dev((void **)&ctx->d_unc2, &ctx->unc2_cap, npairs, sizeof(unsigned));
      if (!rc) rc = bs_ensure_dev((void **)&ctx->d_scr, &ctx->scr_cap, npairs, sizeof(unsigned));
      if (rc) return rc;
      rc = launch_tc(ctx, mode, d_bits, npairs, d_pass, d_dump, L);
      if (rc) return rc;
      // the margin band: the exact fixed-point test, then FP64 for what it leaves
      rc = launch_fix(ctx, d_bits, d_pass, L);
      if (rc) return rc;
      rc = launch_fp64(ctx, d_bits, npairs, ctx->d_unc2, ctx->d_count + 3,
                       (unsigned long long)ctx->unc2_cap, d_pass, L);
      if (rc) return rc;
    }
  }
  if (stats) {
    unsigned long long cnt[8];
    int status = 0;
    CK(cudaMemcpyAsync(cnt, ctx->d_count, sizeof cnt, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (status) {
      cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
      return status;
    }
    if (cnt[2]) return BS_ERR_INTERNAL;  // cannot happen: the list holds every pair
    stats->pairs = npairs;
    stats->passed = (long long)cnt[1];
    stats->rechecked = mode == BS_HALL_FP64 ? 0 : (long long)cnt[0];
    stats->fp64_rechecked = mode == BS_HALL_FP64 ? 0 : (long long)cnt[3];
    stats->mode = mode;
    if (mode == BS_HALL_FP64) {
      stats->pass_below = ctx->lim;
      stats->reject_above = ctx->lim;
      stats->quant_err = 0.0;
    } else {
      const bs_hall_tc_form &F = (L == ctx->n) ? ctx->tc[mode] : ctx->tc_ab[mode];
      stats->pass_below = F.pass_below;
      stats->reject_above = F.reject_above;
      stats->quant_err = F.quant_err;
    }
  }
  return BS_OK;
}

extern "C" int bs_hall_filter_dev(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                                  uint8_t *d_pass, bs_hall_stats *stats) {
  return hall_dev(ctx, d_bits, npairs, mode, d_pass, stats, nullptr, ctx ? ctx->n : 0);
}

int bs_hall_dev_len(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                    uint8_t *d_pass, int L) {
  return hall_dev(ctx, d_bits, npairs, mode, d_pass, nullptr, nullptr, L);
}

extern "C" int bs_hall_tc_dump_dev(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                                   float *d_acc) {
  if (!ctx || !d_acc || npairs <= 0 || npairs % 64 || npairs > 65536) return BS_ERR_ARG;
  if (mode != BS_HALL_TC_FP16 && mode != BS_HALL_TC_BF16X2) return BS_ERR_ARG;
  int rc = bs_ensure_dev((void **)&ctx->d_pass, &ctx->pass_cap, npairs, 1);
  if (rc) return rc;
  bs_hall_stats st;
  return hall_dev(ctx, d_bits, npairs, mode, ctx->d_pass, &st, d_acc, ctx->n);
}

static int hall_host(bs_ctx *ctx, const void *src, bool packed, long long npairs, int mode,
                     uint8_t *pass, bs_hall_stats *stats) {
  if (!ctx || !src || !pass || npairs < 0) return BS_ERR_ARG;
  if (npairs == 0) {
    if (stats) { bs_hall_stats z = {}; z.mode = mode; *stats = z; }
    return BS_OK;
  }
  CK(cudaSetDevice(ctx->device));
  const int L = ctx->n;
  int rc = bs_ensure_dev((void **)&ctx->d_bits, &ctx->bits_cap, 2 * npairs, sizeof(uint64_t));
  if (!rc) rc = bs_ensure_dev((void **)&ctx->d_pass, &ctx->pass_cap, npairs, 1);
  if (rc) return rc;
  if (packed) {
    CK(cudaMemcpyAsync(ctx->d_bits, src, sizeof(uint64_t) * 2 * npairs, cudaMemcpyHostToDevice,
                       ctx->stream));
  } else {
    rc = bs_ensure_dev((void **)&ctx->d_rows, &ctx->rows_cap, 2 * npairs * L, 1);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->d_rows, src, (size_t)2 * npairs * L, cudaMemcpyHostToDevice,
                       ctx->stream));
    ctx->launches++;
    pack_kernel<<<bs_grid_for(2 * npairs, 256, 8 * ctx->num_sms), 256, 0, ctx->stream>>>(
        ctx->d_rows, 2 * npairs, L, ctx->d_bits, ctx->d_status);
    CK(cudaGetLastError());
  }
  bs_hall_stats st;
  rc = hall_dev(ctx, ctx->d_bits, npairs, mode, ctx->d_pass, &st, nullptr, ctx->n);
  if (rc) return rc;
  CK(cudaMemcpyAsync(pass, ctx->d_pass, (size_t)npairs, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (stats) *stats = st;
  return BS_OK;
}

extern "C" int bs_hall_filter_batch(bs_ctx *ctx, const int8_t *XY, long long npairs, int mode,
                                    uint8_t *pass, bs_hall_stats *stats) {
  return hall_host(ctx, XY, false, npairs, mode, pass, stats);
}

extern "C" int bs_hall_filter_packed(bs_ctx *ctx, const uint64_t *bits, long long npairs,
                                     int mode, uint8_t *pass, bs_hall_stats *stats) {
  return hall_host(ctx, bits, true, npairs, mode, pass, stats);
}

// ------------------------------------------------------------------------------------
// Allocation-free Hall filter (bs_hall_filter_noalloc)
//
// For callers that may not allocate device memory: code that runs under a device-memory
// budget owned by someone else (a scheduler or host framework that pre-reserves the GPU's
// memory and forbids allocations during a job), and latency-sensitive callers in the middle
// of overlapped multi-stream work, where cudaMalloc/cudaFree would synchronise the device.
// The tensor-core form needs scratch memory (the margin-band list, its counters, the status
// word) and its tables; here all of it lives in one file-scope __device__ array of fixed
// size, which every GPU that loads this library holds until the process exits.
// ------------------------------------------------------------------------------------
namespace {
constexpr long long NOALLOC_MAX_PAIRS = 1LL << 20;  // pairs per call
constexpr size_t NA_COUNT_OFF = 0;                   // 8 x uint64 counters
constexpr size_t NA_STATUS_OFF = 64;                 // int status word
constexpr size_t NA_COS_OFF = 256;                   // FP64 cos [200][BS_MAXL]
constexpr size_t NA_SIN_OFF = NA_COS_OFF + sizeof(double) * 200 * BS_MAXL;
constexpr size_t NA_IMG_OFF = NA_SIN_OFF + sizeof(double) * 200 * BS_MAXL;  // fp16 table image
constexpr size_t NA_UNC_OFF = NA_IMG_OFF + BS_TC_PART_BYTES;                // uint32 band list
constexpr size_t NA_SCR_OFF = NA_UNC_OFF + sizeof(unsigned) * NOALLOC_MAX_PAIRS;  // screen list
constexpr size_t NA_BYTES = NA_SCR_OFF + sizeof(unsigned) * NOALLOC_MAX_PAIRS;

struct NoallocDevice {
  unsigned char *scratch;  // device address of g_hall_noalloc_scratch on this device
  int n;                   // sequence length whose tables the scratch holds (0: none)
  double lim;
  float pass_below, reject_above;
};
NoallocDevice g_na[64];
std::mutex g_na_mutex;
// host staging of the tables (static storage, no heap)
double g_na_cos[200 * BS_MAXL], g_na_sin[200 * BS_MAXL];
uint8_t g_na_img[BS_TC_PART_BYTES];
}  // namespace

static __device__ __align__(256) unsigned char g_hall_noalloc_scratch[NA_BYTES];

// Tables of length n (as bs_ctx_create builds them: host libm, then the fp16 quantisation
// q(t) = round(t * 2^11) / 2^11 in the 128B-swizzled image) and the certified thresholds.
static void noalloc_tables(int n, NoallocDevice &S) {
  memset(g_na_cos, 0, sizeof g_na_cos);
  memset(g_na_sin, 0, sizeof g_na_sin);
  memset(g_na_img, 0, sizeof g_na_img);
  for (int j = 1; j <= 200; j++) {
    double th = j * 3.14159265358979323846 / 100.0;
    for (int i = 0; i <= n; i++) {
      g_na_cos[(j - 1) * BS_MAXL + i] = cos(i * th);
      g_na_sin[(j - 1) * BS_MAXL + i] = sin(i * th);
    }
  }
  double e = 0.0;
  for (int u = 0; u < BS_TC_NANG; u++) {
    const int j = u < 100 ? u + 1 : 200;
    for (int kind = 0; kind < 2; kind++) {
      const double *tab = kind ? g_na_sin : g_na_cos;
      const int row = bs_tc_row(u, kind);
      double esum = 0.0;
      for (int i = 0; i < n; i++) {
        const double t = tab[(j - 1) * BS_MAXL + i];
        const double q = nearbyint(t * 2048.0) / 2048.0;
        esum += fabs(t - q);
        // exact fp16 bits of q (a multiple of 2^-11 in [-1, 1])
        uint16_t bits = 0;
        if (q != 0.0) {
          int ex;
          const double m = frexp(fabs(q), &ex);
          const int e16 = ex - 1 + 15;
          bits = (uint16_t)((q < 0 ? 0x8000 : 0) | (e16 << 10) | (int)llrint((m * 2.0 - 1.0) * 1024.0));
        }
        const size_t off = (size_t)row * 128 + ((size_t)((i >> 3) ^ (row & 7)) << 4) + (size_t)(i & 7) * 2;
        g_na_img[off] = (uint8_t)(bits & 0xFF);
        g_na_img[off + 1] = (uint8_t)(bits >> 8);
      }
      if (esum > e) e = esum;
    }
  }
  e = e * (1.0 + 1e-9) + 1e-12;
  const double eps64 = 1e-9, rho = ldexp(1.0, -20), kappa = 1.0 + 4.0 * rho;
  const double lim = (4.0 * n + 2.0) + 0.5;
  double pb = sqrt(lim - eps64) - 2.0 * e;
  pb = pb * pb / kappa;
  double ra = 2.0 * e + sqrt(lim + 8.0 * e * e + eps64);
  ra = ra * ra * kappa;
  float pbf = (float)pb;
  if ((double)pbf > pb) pbf = nextafterf(pbf, 0.0f);
  float raf = (float)ra;
  if ((double)raf < ra) raf = nextafterf(raf, 1e30f);
  S.lim = lim;
  S.pass_below = pbf;
  S.reject_above = nextafterf(raf, 1e30f);
}

extern "C" int bs_hall_filter_noalloc(int n, const uint64_t *d_bits, long long npairs,
                                      uint8_t *d_pass, void *stream) {
  if (n < 4 || n + 1 > BS_MAXL || npairs < 0 || (npairs && (!d_bits || !d_pass))) return BS_ERR_ARG;
  if (npairs > NOALLOC_MAX_PAIRS) return BS_ERR_CAP;  // beyond the fixed scratch size
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return BS_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  NoallocDevice &S = g_na[dev];
  if (!S.scratch) {  // set-up, once per device, with that device current
    void *p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_hall_noalloc_scratch));
    if (int rc = hall_kernel_attrs(dev)) return rc;
    S.n = 0;
    S.scratch = (unsigned char *)p;  // only once every set-up step has succeeded
  }
  if (S.n != n) {  // tables of another length: rebuild and upload (no device allocation)
    S.n = 0;  // a failure below leaves no length marked as loaded: the next call rebuilds
    noalloc_tables(n, S);
    CK(cudaMemcpyAsync(S.scratch + NA_COS_OFF, g_na_cos, sizeof g_na_cos, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(S.scratch + NA_SIN_OFF, g_na_sin, sizeof g_na_sin, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(S.scratch + NA_IMG_OFF, g_na_img, sizeof g_na_img, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the host staging arrays are reused by the next call
    S.n = n;
  }
  unsigned long long *count = (unsigned long long *)(S.scratch + NA_COUNT_OFF);
  int *status = (int *)(S.scratch + NA_STATUS_OFF);
  CK(cudaMemsetAsync(S.scratch, 0, 128, s));  // counters and status start at zero
  if (npairs > 0) {
    TcParams P;
    memset(&P, 0, sizeof P);
    P.bits = d_bits;
    P.npairs = npairs;
    P.ntiles = (npairs + TC_TILE - 1) / TC_TILE;
    P.bits_a16 = ((uintptr_t)d_bits & 15) == 0;
    P.image = S.scratch + NA_IMG_OFF;
    P.nparts = 1;
    P.ksteps = (n + 15) / 16;
    tc_idesc(0, P.idesc);
    P.idesc_screen = tc_idesc_screen(0);
    P.one2 = 0x3C003C00u;
    P.pass_below = S.pass_below;
    P.reject_above = S.reject_above;
    P.pass = d_pass;
    P.unc = (unsigned *)(S.scratch + NA_UNC_OFF);
    P.unc_cap = (unsigned long long)NOALLOC_MAX_PAIRS;
    P.count = count;
    P.status = status;
    P.dump = nullptr;
    int dev_sms = 0;
    CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev));
    const long long grid = P.ntiles < dev_sms ? P.ntiles : dev_sms;
    // the screen, then the full test over its survivors (as bs_hall_filter_dev does)
    P.scr = (unsigned *)(S.scratch + NA_SCR_OFF);
    P.scr_cap = (unsigned long long)NOALLOC_MAX_PAIRS;
    hall_screen_kernel<<<(int)grid, SC_THREADS, screen_smem_bytes(1), s>>>(P);
    CK(cudaGetLastError());
    P.list = P.scr;
    P.list_len = count + 4;
    P.list_cap = (unsigned long long)NOALLOC_MAX_PAIRS;
    P.scr = nullptr;
    hall_tc_kernel<<<(int)grid, TC_THREADS, tc_smem_bytes(1), s>>>(P);
    CK(cudaGetLastError());
    hall_fp64_recheck_kernel<<<dev_sms, 256, sizeof(double) * 2 * 200 * n, s>>>(
        d_bits, P.unc, count, (unsigned long long)NOALLOC_MAX_PAIRS, n, S.lim,
        (const double *)(S.scratch + NA_COS_OFF), (const double *)(S.scratch + NA_SIN_OFF), d_pass,
        count + 1);
    CK(cudaGetLastError());
  }
  int st = 0;
  CK(cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return st ? st : BS_OK;
}
