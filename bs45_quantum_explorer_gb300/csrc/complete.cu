// complete.cu - budgeted A,B completion (the reference's fh_complete_ab / fh_ab_search,
// src/solver/wz_match.cpp:1115-1341) for a batch of C,D candidates on the GPU.
//
// One warp per candidate. Lane l owns the shifts s = l+1 and s = l+33: their target
// -N_CD(s), partial A,B autocorrelation Dab[s] and remaining capacity Kab[s] live in its
// registers, so placing a position costs O(1) per lane. The depth-first search, its control
// state (per level: next quad, outer-lag mask, reversal-canon ties, early-check residual) and
// the per-level allowed-row lists are uniform across the warp. Every decision, node charge
// and budget abort follows the reference's order, so verdicts, charged node counts and the
// first completion (A,B) are identical. Warps take candidates from a queue in index order; a
// hit lowers hit_min and candidates after it are skipped (verdict -1).
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "bsfh_internal.cuh"

namespace {

#define FULL_MASK 0xffffffffu
constexpr int AB_WARPS = 8;  // warps per block
constexpr int AB_MAXLV = 34; // levels 0..half (n1 <= 64)

struct AbCandDev {
  uint64_t c, d;
  long long mask_off;  // first word of the candidate's row-set masks (see AbParams::masks)
  long long row_off;   // its first row in AbParams::rows8 (the A2 test reads the rows)
  int nrows, W;        // allowed rows of its cell, 64-bit words per row bitset
};

struct AbParams {
  int n, n1, L, half, m, absA, absB;
  int outer_k, early, canon, first_hit;
  long long budget;
  long long max_cycles;
  const AbCandDev *cands;
  long long ncand;
  // Allowed rows as bitsets. For each row set (a cell's rows) and class c, four families of
  // W-word row masks indexed by a value v in [-T-1, T+1] (vi = v + T + 1, V = 2T + 3 values):
  // kind 0 rows with k_c >= v, 1 rows with k_c <= v, 2 rows with r_c >= v, 3 rows with
  // r_c <= v, at masks[mask_off + ((c * 4 + kind) * V + vi) * W].
  const uint64_t *masks;
  int T, V;
  uint64_t *bits;   // per warp slot: levels 0..half, Wcap words each (the surviving rows)
  int Wcap;
  // WZ_FH_A2 = 2 (wz_match.cpp:977-1047): each row that passes the box is kept only if its
  // residuals are reachable block by block with the quads left (a2_row_ok)
  int a2, a2_nblk;
  const int8_t *rows8;     // the rows (k[8], r[8]) of every row set, for the A2 test
  int8_t a2_r[8], a2_s[8], a2_mid[8];
  uint8_t a2_cnt[AB_MAXLV + 2][8];  // quads left in block b from depth p on
  const uint8_t *outer2, *outer3;
  unsigned long long *next;
  long long *hit_min;
  int32_t *verdict;
  long long *nodes_out;
  uint64_t *ab_out;
  const volatile int *stop_flag;
  int *status;
  int tic[8];
};

// quad index -> sign bits (bit 3 = A[i1], bit 2 = B[i1], bit 1 = A[i2], bit 0 = B[i2])
__constant__ uint8_t kQPos[8] = {0, 3, 5, 6, 9, 10, 12, 15};
__constant__ uint8_t kQNeg[8] = {1, 2, 4, 7, 8, 11, 13, 14};
__constant__ int8_t kPosOf[16] = {0, -1, -1, 1, -1, 2, 3, -1, -1, 4, 5, -1, 6, -1, -1, 7};

__device__ __forceinline__ int absi(int x) { return x < 0 ? -x : x; }

struct Lanes {
  int t0, t1;    // target at s0 = lane+1, s1 = lane+33
  int D0, D1;    // Dab of the placed set, as of the last corr()
  int K0, K1;    // Kab: twice the pairs at the shift with a position still free
  int s0, s1;    // shifts (0 when out of range)
  int kb0, kb1;  // 2 (L - s): Kab with nothing placed
};

// The placed positions as bits: bit p of Pm is set when position p is placed, of A (B) when
// A[p] (B[p]) is +1. Positions go in mirror pairs (d, L-1-d), so Pm holds the first and last
// d positions (and the middle one at an odd length's leaf). Everything the search reads
// (Dab, Kab, the class sums, sum A, sum B) is a popcount of these words, so removing a
// position only clears its bits. The reference keeps Dab, Kab and the class sums
// incrementally (fh_place / fh_unplace, wz_match.cpp:1127-1161); the values are the same.
struct Uni {
  uint64_t A, B, Pm;
};

// sum of the +-1 values placed at the positions of sel (A or B as X): 2 #(+1) - #placed
__device__ __forceinline__ int ssum(uint64_t X, uint64_t Pm, uint64_t sel) {
  return 2 * __popcll(X & sel) - __popcll(Pm & sel);
}

// Dab and Kab at the lane's shifts. The pairs (q, q+s) with both positions placed are the set
// bits of Pm & Pm >> s; each adds a_q a_{q+s} + b_q b_{q+s} = 2 - 2 [a_q != a_{q+s}] -
// 2 [b_q != b_{q+s}] to Dab[s] and takes 2 from Kab[s]. The search reads them only right
// after a placement. two: whether the shifts 33.. need recomputing (uniform): they exist
// (n >= 33) and the placement can add a pair at one of them.
__device__ __forceinline__ void corr(Lanes &v, const Uni &u, bool two) {
  {
    const uint64_t vv = u.Pm & (u.Pm >> v.s0);
    const int np = __popcll(vv);
    const int dis = __popcll((u.A ^ (u.A >> v.s0)) & vv) + __popcll((u.B ^ (u.B >> v.s0)) & vv);
    v.D0 = 2 * (np - dis);
    v.K0 = v.kb0 - 2 * np;
  }
  if (two) {
    const uint64_t vv = u.Pm & (u.Pm >> v.s1);
    const int np = __popcll(vv);
    const int dis = __popcll((u.A ^ (u.A >> v.s1)) & vv) + __popcll((u.B ^ (u.B >> v.s1)) & vv);
    v.D1 = 2 * (np - dis);
    v.K1 = v.kb1 - 2 * np;
  }
}

// residual target[s] - Dab[s] at shift s (1 <= s <= n), uniform
__device__ __forceinline__ int resid_at(const Lanes &v, int s) {
  int mine = ((s - 1) >> 5) ? (v.t1 - v.D1) : (v.t0 - v.D0);
  return __shfl_sync(FULL_MASK, mine, (s - 1) & 31);
}

// place the quad q (sign bits: 3 = A at b1m's position, 2 = B there, 1 = A at b2m's, 0 = B
// there; a set bit is +1)
__device__ __forceinline__ void place2(Uni &u, uint64_t b1m, uint64_t b2m, uint32_t q) {
  u.Pm |= b1m | b2m;
  u.A |= ((q & 8) ? b1m : 0ULL) | ((q & 2) ? b2m : 0ULL);
  u.B |= ((q & 4) ? b1m : 0ULL) | ((q & 1) ? b2m : 0ULL);
}
__device__ __forceinline__ void clear_bits(Uni &u, uint64_t bits) {
  u.Pm &= ~bits;
  u.A &= ~bits;
  u.B &= ~bits;
}
__device__ __forceinline__ uint64_t pair_bits(int d, int L) { return (1ULL << d) | (1ULL << (L - 1 - d)); }

// Reversal-canon filter of wz_match.cpp:1222-1239 for quad (a1,b1,a2,b2) at level d with the
// level's incoming ties. Returns false to skip; writes the outgoing ties.
__device__ __forceinline__ bool canon_ok(const AbParams &P, int d, uint32_t ties, int a1, int b1,
                                         int a2, int b2, uint32_t &out) {
  if (!P.canon) { out = ties; return true; }
  int a_tied = ties & 1, a_cmp = (ties & 2) ? 1 : -1, b_tied = (ties >> 2) & 1, b_cmp = (ties & 8) ? 1 : -1;
  if (d == 0) {
    if (a1 != 1 || b1 != 1) return false;
    out = 1u | (a2 > 0 ? 2u : 0u) | 4u | (b2 > 0 ? 8u : 0u);
    return true;
  }
  int na_tied = a_tied, nb_tied = b_tied;
  if (a_tied) {
    int cv = a_cmp * a2;
    if (a1 != cv) { if (a1 != 1) return false; na_tied = 0; }
  }
  if (b_tied) {
    int cv = b_cmp * b2;
    if (b1 != cv) { if (b1 != 1) return false; nb_tied = 0; }
  }
  out = (uint32_t)na_tied | (ties & 2) | ((uint32_t)nb_tied << 2) | (ties & 8);
  return true;
}

__device__ __forceinline__ uint32_t quad_bits(int d, int k) { return d == 0 ? kQNeg[k] : kQPos[k]; }

// outer_mask, wz_match.cpp:601-618, in two parts. outer_pat: the pattern of the k outermost
// quads (levels 0..k-1), or -1 when the table does not apply; it is fixed while the search is
// below level k, so it is taken once on the way down through level k.
__device__ __forceinline__ int outer_pat(const AbParams &P, const Uni &u) {
  const int k = P.outer_k, L = P.L;
  if (!(u.A & 1ULL) || !(u.B & 1ULL)) return -1;
  int pat = (int)((u.A >> (L - 1)) & 1ULL), mul = 2;
  for (int t = 1; t < k; t++) {
    int sb = (int)(((u.A >> t) & 1) << 3 | ((u.B >> t) & 1) << 2 | ((u.A >> (L - 1 - t)) & 1) << 1 |
                   ((u.B >> (L - 1 - t)) & 1));
    int q = kPosOf[sb];
    if (q < 0) return -1;
    pat += mul * q;
    mul *= 8;
  }
  return pat;
}

// the mask at level d >= 1 from the pattern and the residuals at L-1-d-j (r0 at j = 0). A
// residual must be even with |R_j| <= 4 (j + 1); then R_j / 2 is R_j >> 1.
__device__ __forceinline__ unsigned outer_mask(const AbParams &P, int pat, const Lanes &v, int d, int r0) {
  const int k = P.outer_k, L = P.L;
  if (k < 2 || d < k || d + k > L / 2 || pat < 0) return 0xFFu;
  const int s1 = L - 2 - d;  // the shift of R_1
  int r1, r2 = 0;
  if (s1 <= 32) {  // every shift below 33: one slot (the common case)
    const int mine = v.t0 - v.D0;
    r1 = __shfl_sync(FULL_MASK, mine, s1 - 1);
    if (k == 3) r2 = __shfl_sync(FULL_MASK, mine, s1 - 2);
  } else {
    r1 = resid_at(v, s1);
    if (k == 3) r2 = resid_at(v, s1 - 1);
  }
  if ((r0 | r1 | r2) & 1) return 0u;
  if ((unsigned)(r0 + 4) > 8u || (unsigned)(r1 + 8) > 16u || (unsigned)(r2 + 12) > 24u) return 0u;
  if (k == 2) return P.outer2[pat * 45 + (r0 >> 1) * 9 + (r1 >> 1) + 22];
  return P.outer3[pat * 585 + (r0 >> 1) * 117 + (r1 >> 1) * 13 + (r2 >> 1) + 292];
}

// The level filter of the allowed rows (fh_abp_filter, wz_match.cpp:1055-1075): a row
// survives while |k_c - pa_c| <= rem_c and |r_c - pb_c| <= rem_c for every class c. Placing
// the mirror positions d and L-1-d changes pa, pb and rem of their two classes only, and the
// parent's list already meets the box of every other class, so the child's list is the
// parent's AND the four range masks of each of the two classes.
__device__ __forceinline__ const uint64_t *mask_of(const AbParams &P, const AbCandDev &cd, int c,
                                                   int kind, int v) {
  v = v < -P.T - 1 ? -P.T - 1 : (v > P.T + 1 ? P.T + 1 : v);
  return P.masks + cd.mask_off + ((size_t)(c * 4 + kind) * P.V + (size_t)(v + P.T + 1)) * cd.W;
}
// a2_self_ok / a2_row_ok (wz_match.cpp:1017-1038): residuals (u, v) of a self-reflected block
// reachable with q quads of (+-2, +-2) or (0, 0); of a block {r, s}, H (ur, vr, us, vs) / 4
// integral with an L1 norm of the same parity as q and at most q.
__device__ __forceinline__ bool a2_self(int u, int v, int q) {
  if ((u | v) & 1) return false;
  if (u > 2 * q || -u > 2 * q || v > 2 * q || -v > 2 * q) return false;
  return ((u - v) & 3) == 0;
}
__device__ __forceinline__ bool a2_row(const AbParams &P, const int8_t *row, const int *pa,
                                       const int *pb, int p) {
  for (int b = 0; b < P.a2_nblk; b++) {
    const int r = P.a2_r[b], s = P.a2_s[b], q = P.a2_cnt[p][b];
    const int ur = row[r] - pa[r], vr = row[8 + r] - pb[r];
    if (r != s) {
      const int us = row[s] - pa[s], vs = row[8 + s] - pb[s];
      const int t0 = ur + vr + us + vs, t1 = ur - vr + us - vs, t2 = ur + vr - us - vs,
                t3 = ur - vr - us + vs;
      if ((t0 | t1 | t2 | t3) & 3) return false;
      const int l1 = (absi(t0) + absi(t1) + absi(t2) + absi(t3)) >> 2;
      if (l1 > q || ((q - l1) & 1)) return false;
    } else if (P.a2_mid[b]) {
      if (!a2_self(ur - 1, vr - 1, q) && !a2_self(ur - 1, vr + 1, q) &&
          !a2_self(ur + 1, vr - 1, q) && !a2_self(ur + 1, vr + 1, q))
        return false;
    } else if (!a2_self(ur, vr, q)) {
      return false;
    }
  }
  return true;
}

// all rows of the cell, as bitset word w
__device__ __forceinline__ uint64_t all_rows(int w, int nrows) {
  const int lo = w * 64;
  return nrows - lo >= 64 ? ~0ULL : ((1ULL << (nrows - lo)) - 1ULL);
}

// MINB: resident blocks per SM the register budget is cut for (2: up to 128 registers a
// thread; 3: up to 85, with a few spills)
template <int MINB>
__global__ void __launch_bounds__(32 * AB_WARPS, MINB) ab_kernel(AbParams P) {
  // the quad loop's canon filter as tables (entry 16 is the root level d = 0): bit k of
  // s_elig[t] says quad k passes canon_ok with incoming ties t, s_ntie[t][k] its outgoing ties
  __shared__ uint8_t s_elig[17];
  __shared__ uint8_t s_ntie[17][8];
  if (threadIdx.x < 17) {
    const int t = threadIdx.x, dd = t == 16 ? 0 : 1;
    uint32_t elig = 0;
    for (int k = 0; k < 8; k++) {
      const uint32_t q = quad_bits(dd, k);
      uint32_t o = 0;
      if (canon_ok(P, dd, t == 16 ? 5u : (uint32_t)t, (q & 8) ? 1 : -1, (q & 4) ? 1 : -1,
                   (q & 2) ? 1 : -1, (q & 1) ? 1 : -1, o))
        elig |= 1u << k;
      s_ntie[t][k] = (uint8_t)o;
    }
    s_elig[t] = (uint8_t)elig;
  }
  __shared__ uint8_t s_cls[64];   // residue class of each position
  __shared__ uint64_t s_cm[8];    // positions of each class, as bits
  __shared__ int s_tic[8];        // positions in each class
  if (threadIdx.x < 64) s_cls[threadIdx.x] = (uint8_t)(threadIdx.x % P.m);
  if (threadIdx.x < 8) {
    uint64_t cm = 0;
    for (int p = threadIdx.x; p < P.L; p += P.m) cm |= 1ULL << p;
    s_cm[threadIdx.x] = threadIdx.x < P.m ? cm : 0ULL;
    s_tic[threadIdx.x] = P.tic[threadIdx.x];
  }
  __syncthreads();
  // first eligible quad >= k at level d (next_quad): the outer mask applies from d = 1
  auto next_q = [&](int dd, int k, unsigned om, uint32_t ties) -> int {
    const uint32_t e = (dd == 0 ? s_elig[16] : (s_elig[ties] & om)) & (0xFFu << k) & 0xFFu;
    return e ? __ffs(e) - 1 : 8;
  };
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long slot = (long long)blockIdx.x * AB_WARPS + wib;
  // Per-level control state: k | omask << 4 | ties << 12 and the early-check residual. The
  // current level's is held in registers (cur, cres, warp-uniform); the levels above it are
  // saved one level per lane (levels 0..half-1 <= 31: lane j holds level j's), written by that
  // lane when the search descends and read back with one shuffle when it returns, so no
  // shared memory or warp barrier is involved.
  uint32_t my_ctrl = 0;
  int my_res = 0;
  // and the level's row bitset range: its nonzero words lie in [lo, hi), saved as lo | hi << 16
  // (W < 65536 words, checked on the host); the current level's in clo, chi
  uint32_t my_rng = 0;
  uint64_t *lv = P.bits + (size_t)slot * (P.half + 1) * P.Wcap;
  const int L = P.L, n = P.n, half = P.half, m = P.m;
  // A second shift slot per lane when n >= 33. Its shifts s >= 33 pair position d only with
  // d + s <= L - 1, so placing level d changes them only while d <= L - 34; after that their
  // Dab is final (and was checked against the target with Kab = 0), so it is not recomputed.
  const bool two = n >= 33;

  while (true) {
    unsigned long long idx = 0;
    if (lane == 0) idx = atomicAdd(P.next, 1ULL);
    idx = __shfl_sync(FULL_MASK, idx, 0);
    if (idx >= (unsigned long long)P.ncand) break;
    if ((long long)idx > *(volatile long long *)P.hit_min || *P.stop_flag) {
      if (lane == 0) { P.verdict[idx] = -1; P.nodes_out[idx] = 0; }
      continue;
    }
    const AbCandDev cd = P.cands[idx];
    const bool rows = cd.nrows > 0;
    // targets -N_CD(s) and the prefilter of wz_match.cpp:1300-1308
    Lanes v;
    v.s0 = (lane + 1 <= n) ? lane + 1 : 0;
    v.s1 = (lane + 33 <= n) ? lane + 33 : 0;
    auto ncd = [&](int s) {
      if (s <= 0 || s >= n) return 0;
      uint64_t mask = (1ULL << (n - s)) - 1ULL;
      int dc = __popcll((cd.c ^ (cd.c >> s)) & mask), dd = __popcll((cd.d ^ (cd.d >> s)) & mask);
      return 2 * (n - s) - 2 * (dc + dd);
    };
    v.t0 = -ncd(v.s0);
    v.t1 = -ncd(v.s1);
    bool pre = (v.s0 && absi(v.t0) > 2 * (P.n1 - v.s0)) || (v.s1 && absi(v.t1) > 2 * (P.n1 - v.s1));
    if (__any_sync(FULL_MASK, pre)) {
      if (lane == 0) { P.verdict[idx] = 1; P.nodes_out[idx] = 0; }
      continue;
    }
    v.D0 = v.D1 = 0;
    v.kb0 = v.s0 ? 2 * (P.n1 - v.s0) : 0;
    v.kb1 = v.s1 ? 2 * (P.n1 - v.s1) : 0;
    v.K0 = v.kb0;
    v.K1 = v.kb1;
    Uni u;
    u.A = u.B = u.Pm = 0;
    int opat = -1;   // outer_pat, taken when the search passes level outer_k
    uint32_t e4 = 0;  // early check: A[L-1], B[L-1], A[0], B[0] as bits 3..0 (set at level 1)
    long long nodes = 0, spent = 0;  // nodes charged; the budget's count (fh_cur)
    bool aborted = false, found = false, abandoned = false;
    const long long t_start = clock64();
    int d = 0;
    uint32_t cur = 0u | (0xFFu << 4) | (5u << 12);  // level 0; ties: a_tied = b_tied = 1
    int cres = 0;
    int clo = 0, chi = cd.W;
    unsigned steps = 0;
    while (true) {
      if ((++steps & 1023) == 0) {
        bool stop = (long long)idx > *(volatile long long *)P.hit_min || *P.stop_flag ||
                    (P.max_cycles > 0 && clock64() - t_start > P.max_cycles);
        if (__shfl_sync(FULL_MASK, (int)stop, 0)) { abandoned = true; break; }
      }
      if (d == half) {
        // ---- leaf: final_ok (and the free middle for odd length), wz_match.cpp:1178-1205 ----
        auto final_ok = [&]() -> bool {
          const int sA = 2 * __popcll(u.A) - __popcll(u.Pm), sB = 2 * __popcll(u.B) - __popcll(u.Pm);
          if (absi(sA) != P.absA || absi(sB) != P.absB) return false;
          bool eq = (!v.s0 || v.D0 == v.t0) && (!v.s1 || v.D1 == v.t1);
          if (!__all_sync(FULL_MASK, eq)) return false;
          if (rows) {
            // fh_abp_leaf_ok: a row of the last list equals the placed class sums exactly
            const uint64_t *lst = lv + (size_t)half * P.Wcap;
            bool any = false;
            for (int w = clo + lane; w < chi; w += 32) {
              uint64_t x = lst[w];
              for (int c = 0; c < m; c++) {
                const int pa = ssum(u.A, u.Pm, s_cm[c]), pb = ssum(u.B, u.Pm, s_cm[c]);
                x &= mask_of(P, cd, c, 0, pa)[w] & mask_of(P, cd, c, 1, pa)[w] &
                     mask_of(P, cd, c, 2, pb)[w] & mask_of(P, cd, c, 3, pb)[w];
              }
              any |= x != 0;
            }
            if (!__any_sync(FULL_MASK, any)) return false;
          }
          return true;
        };
        if (L & 1) {
          const uint64_t mb = 1ULL << half;
          for (int km = 0; km < 4 && !found; km++) {
            // (A, B) of the middle: (+,+), (+,-), (-,+), (-,-)
            place2(u, mb, 0ULL, (km < 2 ? 8u : 0u) | ((km & 1) ? 0u : 4u));
            corr(v, u, false);  // the middle pairs at shifts up to L - 1 - half < 33 only
            nodes++;
            if (final_ok()) found = true;
            else clear_bits(u, mb);
          }
        } else if (final_ok()) {
          found = true;
        }
        if (found) break;
        // back to the parent level: its saved state, with the next quad
        d--;
        cur = __shfl_sync(FULL_MASK, my_ctrl, d);
        cres = __shfl_sync(FULL_MASK, my_res, d);
        {
          const uint32_t rg = __shfl_sync(FULL_MASK, my_rng, d);
          clo = (int)(rg & 0xFFFFu);
          chi = (int)(rg >> 16);
        }
        clear_bits(u, pair_bits(d, L));
        cur = (cur & ~15u) | ((cur & 15) + 1);
        continue;
      }
      const uint32_t c0 = cur;
      const unsigned omask = (c0 >> 4) & 0xFF;
      const uint32_t ties = (c0 >> 12) & 15;
      int k = next_q(d, c0 & 15, omask, ties);
      if (k == 8) {
        if (d == 0) break;  // clean exhaustion
        d--;
        cur = __shfl_sync(FULL_MASK, my_ctrl, d);
        cres = __shfl_sync(FULL_MASK, my_res, d);
        {
          const uint32_t rg = __shfl_sync(FULL_MASK, my_rng, d);
          clo = (int)(rg & 0xFFFFu);
          chi = (int)(rg >> 16);
        }
        clear_bits(u, pair_bits(d, L));
        cur = (cur & ~15u) | ((cur & 15) + 1);
        continue;
      }
      const uint32_t q = quad_bits(d, k);  // a1, b1, a2, b2 as bits 3..0 (set: +1)
      // charge the node before placing (wz_match.cpp:1243-1248)
      nodes++;
      if (P.budget > 0 && ++spent > P.budget) {
        aborted = true;
        break;
      }
      // early outer-correlation check (wz_match.cpp:1256-1259): A[0] a2 + B[0] b2 +
      // A[L-1] a1 + B[L-1] b1, whose four products are +1 where the quad's bit (a1, b1, a2,
      // b2 as bits 3..0) matches e4's and -1 where not
      if (P.early && d > 0) {
        const int lhs = 4 - 2 * __popc((e4 ^ q) & 15u);
        if (lhs != cres) {
          cur = (c0 & ~15u) | (uint32_t)(k + 1);
          continue;
        }
      }
      const uint64_t pbits = pair_bits(d, L);
      place2(u, 1ULL << d, 1ULL << (L - 1 - d), q);
      const int rem = L - 2 * (d + 1);
      // 2 (d + 1) positions are placed: sum = 2 #(+1) - 2 (d + 1)
      const int sumA = 2 * (__popcll(u.A) - d - 1), sumB = 2 * (__popcll(u.B) - d - 1);
      bool prune = !(((absi(P.absA - sumA) <= rem) || (absi(-P.absA - sumA) <= rem)) &&
                     ((absi(P.absB - sumB) <= rem) || (absi(-P.absB - sumB) <= rem)));
      if (!prune) {
        corr(v, u, two && d <= L - 34);
        bool bad = (v.s0 && absi(v.t0 - v.D0) > v.K0) || (v.s1 && absi(v.t1 - v.D1) > v.K1);
        prune = __any_sync(FULL_MASK, bad);
      }
      int child_lo = 0, child_hi = 0;  // the child level's row range (from the filter)
      if (!prune && rows) {
        // fh_abp_filter(d): the level-(d+1) list from the level-d list (all rows at d = 0)
        const int c1 = s_cls[d], c2 = s_cls[L - 1 - d];
        const uint64_t *src = lv + (size_t)d * P.Wcap;
        uint64_t *dst = lv + (size_t)(d + 1) * P.Wcap;
        const int lo = clo, hi = chi;
        int nlo, nhi;
        if (!P.a2 && hi - lo <= 24) {
          // Narrow lists (the deep levels, where the nodes are): lane 8i + j loads mask j
          // (class c1 for j < 4, c2 for j >= 4; kind j & 3: bounds on k_c = sum A or r_c =
          // sum B over the class) of word base + i, four words per pass, and three butterfly
          // steps AND the eight together. Each lane forms the one bound it needs: the class's
          // placed sum pv and what its free positions can add, r.
          const int j = lane & 7, kind = j & 3;
          const int c = j < 4 ? c1 : c2;
          const uint64_t mc = s_cm[c];
          const int placed = __popcll(u.Pm & mc);
          const int pv = 2 * __popcll((kind < 2 ? u.A : u.B) & mc) - placed;
          const int r = s_tic[c] - placed;
          const uint64_t *mk = mask_of(P, cd, c, kind, (kind & 1) ? pv + r : pv - r);
          nlo = 1 << 30;
          nhi = -1;
          for (int base = lo; base < hi; base += 4) {
            const int w = base + (lane >> 3);
            const bool live = w < hi;
            uint64_t x = live ? mk[w] : ~0ULL;
            x &= __shfl_xor_sync(FULL_MASK, x, 1);
            x &= __shfl_xor_sync(FULL_MASK, x, 2);
            x &= __shfl_xor_sync(FULL_MASK, x, 4);
            if (j == 0 && live) {
              x &= d == 0 ? all_rows(w, cd.nrows) : src[w];
              dst[w] = x;
            }
            const unsigned ball = __ballot_sync(FULL_MASK, j == 0 && live && x != 0);
            if (ball) {
              if (nhi < 0) nlo = base + ((__ffs(ball) - 1) >> 3);
              nhi = base + ((31 - __clz(ball)) >> 3);
            }
          }
        } else {
          const uint64_t m1 = s_cm[c1], m2 = s_cm[c2];
          const int r1 = s_tic[c1] - __popcll(u.Pm & m1), pa1 = ssum(u.A, u.Pm, m1), pb1 = ssum(u.B, u.Pm, m1);
          const int r2 = s_tic[c2] - __popcll(u.Pm & m2), pa2 = ssum(u.A, u.Pm, m2), pb2 = ssum(u.B, u.Pm, m2);
          const uint64_t *k1a = mask_of(P, cd, c1, 0, pa1 - r1), *k1b = mask_of(P, cd, c1, 1, pa1 + r1);
          const uint64_t *q1a = mask_of(P, cd, c1, 2, pb1 - r1), *q1b = mask_of(P, cd, c1, 3, pb1 + r1);
          const uint64_t *k2a = mask_of(P, cd, c2, 0, pa2 - r2), *k2b = mask_of(P, cd, c2, 1, pa2 + r2);
          const uint64_t *q2a = mask_of(P, cd, c2, 2, pb2 - r2), *q2b = mask_of(P, cd, c2, 3, pb2 + r2);
          int pa[8], pb[8];
          if (P.a2)
            for (int c = 0; c < 8; c++) {
              pa[c] = c < m ? ssum(u.A, u.Pm, s_cm[c]) : 0;
              pb[c] = c < m ? ssum(u.B, u.Pm, s_cm[c]) : 0;
            }
          int mylo = 1 << 30, myhi = -1;
          for (int w = lo + lane; w < hi; w += 32) {
            uint64_t x = d == 0 ? all_rows(w, cd.nrows) : src[w];
            x &= k1a[w] & k1b[w] & q1a[w] & q1b[w];
            if (c2 != c1) x &= k2a[w] & k2b[w] & q2a[w] & q2b[w];
            if (P.a2)  // A2 on the rows that passed the box, at depth d + 1
              for (uint64_t y = x; y; y &= y - 1) {
                const int bit = __ffsll((long long)y) - 1;
                if (!a2_row(P, P.rows8 + 16 * (cd.row_off + (long long)w * 64 + bit), pa, pb, d + 1))
                  x &= ~(1ULL << bit);
              }
            dst[w] = x;
            if (x) {
              mylo = min(mylo, w);
              myhi = w;
            }
          }
          nlo = __reduce_min_sync(FULL_MASK, mylo);
          nhi = __reduce_max_sync(FULL_MASK, myhi);
        }
        child_lo = nlo;
        child_hi = nhi + 1;
        prune = nhi < 0;
      }
      if (prune) {
        clear_bits(u, pbits);
        cur = (c0 & ~15u) | (uint32_t)(k + 1);
        continue;
      }
      // descend: the child level's entry work (its outer mask may end it immediately)
      const int nd = d + 1;
      unsigned om = 0xFFu;
      int r_e = 0;
      if (nd == 1)
        e4 = (uint32_t)(((u.A >> (L - 1)) & 1) << 3 | ((u.B >> (L - 1)) & 1) << 2 | (u.A & 1) << 1 | (u.B & 1));
      if (nd < half) {
        r_e = resid_at(v, L - 1 - nd);
        if (P.outer_k) {
          if (nd == P.outer_k) opat = outer_pat(P, u);
          om = outer_mask(P, opat, v, nd, r_e);
        }
      }
      if (om == 0u) {  // fh_ab_search(d+1) returns false at once: undo and try the next quad
        clear_bits(u, pbits);
        cur = (c0 & ~15u) | (uint32_t)(k + 1);
        continue;
      }
      if (lane == d) {  // save this level (at the quad taken) for the way back
        my_ctrl = (c0 & ~15u) | (uint32_t)k;
        my_res = cres;
        my_rng = (uint32_t)clo | ((uint32_t)chi << 16);
      }
      if (rows) {
        clo = child_lo;
        chi = child_hi;
      }
      cur = 0u | (om << 4) | ((uint32_t)s_ntie[d == 0 ? 16 : ties][k] << 12);
      cres = r_e;
      d = nd;
    }
    if (aborted) {
      // Every ancestor level whose loop has another eligible quad charges one more node before
      // it returns (wz_match.cpp:1243-1247 reached again with fh_cur already over budget).
      for (int j = d - 1; j >= 0; j--) {
        uint32_t cj = __shfl_sync(FULL_MASK, my_ctrl, j);
        if (next_q(j, (cj & 15) + 1, (cj >> 4) & 0xFF, (cj >> 12) & 15) < 8) nodes++;
      }
    }
    if (lane == 0) {
      int verdict = abandoned ? -1 : found ? 0 : aborted ? 3 : 2;
      if (abandoned && P.max_cycles > 0 && !(*P.stop_flag) &&
          !((long long)idx > *(volatile long long *)P.hit_min))
        verdict = -2;  // wall limit reached
      P.verdict[idx] = verdict;
      P.nodes_out[idx] = nodes;
      if (found) {
        P.ab_out[2 * idx] = u.A;
        P.ab_out[2 * idx + 1] = u.B;
        if (P.first_hit) atomicMin((unsigned long long *)P.hit_min, idx);
      }
    }
    __syncwarp();
  }
}

// ---- host tables (the A1 outer-lag tables, built from their definition) ----
struct OuterTables {
  uint8_t o2[16 * 5 * 9];
  uint8_t o3[128 * 5 * 9 * 13];
  OuterTables() {
    int pos[8][4], neg[8][4], np = 0, nn = 0;
    for (int i = 0; i < 16; i++) {
      int v[4] = {(i & 8) ? 1 : -1, (i & 4) ? 1 : -1, (i & 2) ? 1 : -1, (i & 1) ? 1 : -1};
      if (v[0] * v[1] * v[2] * v[3] == 1) memcpy(pos[np++], v, sizeof v);
      else memcpy(neg[nn++], v, sizeof v);
    }
    int root[2] = {0, 0};
    for (int q = 0; q < 8; q++)
      if (neg[q][0] == 1 && neg[q][1] == 1) root[neg[q][2] > 0] = q;
    memset(o2, 0, sizeof o2);
    memset(o3, 0, sizeof o3);
    for (int k = 2; k <= 3; k++) {
      int npat = k == 2 ? 16 : 128;
      for (int pat = 0; pat < npat; pat++) {
        int lA[3], lB[3], rA[3], rB[3];
        const int *rq = neg[root[pat & 1]];
        lA[0] = rq[0]; lB[0] = rq[1]; rA[0] = rq[2]; rB[0] = rq[3];
        int rest = pat >> 1;
        for (int t = 1; t < k; t++) {
          const int *qv = pos[rest % 8];
          rest /= 8;
          lA[t] = qv[0]; lB[t] = qv[1]; rA[t] = qv[2]; rB[t] = qv[3];
        }
        for (int asg = 0; asg < (k == 2 ? 64 : 512); asg++) {
          int idx[3], a = asg;
          for (int r = 0; r < k; r++) { idx[r] = a % 8; a /= 8; }
          int F[3] = {0, 0, 0};
          for (int j = 0; j < k; j++)
            for (int r = 0; r <= j; r++) {
              const int *qv = pos[idx[r]];
              F[j] += lA[j - r] * qv[2] + lB[j - r] * qv[3] + rA[j - r] * qv[0] + rB[j - r] * qv[1];
            }
          if (k == 2) o2[(pat * 5 + F[0] / 2 + 2) * 9 + F[1] / 2 + 4] |= (uint8_t)(1u << idx[0]);
          else o3[((pat * 5 + F[0] / 2 + 2) * 9 + F[1] / 2 + 4) * 13 + F[2] / 2 + 6] |= (uint8_t)(1u << idx[0]);
        }
      }
    }
  }
};

}  // namespace

#define CK(x)                                       \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return bs_cuda_fail(e_); \
  } while (0)

struct AbBufs {
  uint8_t *outer = nullptr;  // o2 then o3
  AbCandDev *cands = nullptr; long long cand_cap = 0;
  uint64_t *masks = nullptr; long long masks_cap = 0;  // row-set masks (AbParams::masks)
  uint64_t *bits = nullptr; long long bits_cap = 0;    // per-warp level bitsets
  int8_t *rows8 = nullptr; long long rows8_cap = 0;     // the rows themselves (A2 test)
  // the row sets whose masks are on the device: the rows they were built from, their
  // (row_off, nrows) and mask offsets, and the modulus and length
  std::vector<int8_t> mask_rows;
  std::vector<std::pair<long long, int>> mask_sets;
  std::vector<long long> mask_offs;
  int mask_m = 0, mask_n1 = 0;
  int32_t *verdict = nullptr; long long v_cap = 0;
  long long *nodes = nullptr; long long n_cap = 0;
  uint64_t *ab = nullptr; long long ab_cap = 0;
  unsigned long long *next = nullptr;
  long long *hit_min = nullptr;
};

static AbBufs *ab_bufs(bs_ctx *ctx) {
  if (!ctx->ab_bufs) ctx->ab_bufs = new AbBufs();
  return (AbBufs *)ctx->ab_bufs;
}

void bs_ab_free(bs_ctx *ctx) {
  AbBufs *b = (AbBufs *)ctx->ab_bufs;
  if (!b) return;
  cudaFree(b->outer); cudaFree(b->cands); cudaFree(b->masks); cudaFree(b->bits); cudaFree(b->rows8);
  cudaFree(b->verdict); cudaFree(b->nodes); cudaFree(b->ab); cudaFree(b->next);
  cudaFree(b->hit_min);
  delete b;
  ctx->ab_bufs = nullptr;
}

static void words_to_seq(uint64_t w, int L, int8_t *out) {
  for (int i = 0; i < L; i++) out[i] = ((w >> i) & 1ULL) ? 1 : -1;
}

extern "C" int bs_complete_ab_batch(bs_ctx *ctx, const bs_ab_cand *cands, long long ncand,
                                    const int8_t *rows, long long nrows_total,
                                    const bs_ab_opts *opt, int32_t *verdict, long long *nodes,
                                    int8_t *A, int8_t *B) {
  if (!ctx || ncand < 0 || !opt || (ncand && (!cands || !verdict || !nodes))) return BS_ERR_ARG;
  if (opt->m != 3 && opt->m != 6) return BS_ERR_ARG;
  if (opt->outer_k != 0 && opt->outer_k != 2 && opt->outer_k != 3) return BS_ERR_ARG;
  if (opt->a2 != 0 && opt->a2 != 2) return BS_ERR_ARG;
  if (ncand == 0) return BS_OK;
  const int n = ctx->n, n1 = n + 1, half = n1 / 2;
  if (n1 > 64 || half + 1 > AB_MAXLV) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  AbBufs *Bf = ab_bufs(ctx);
  cudaStream_t s = ctx->stream;
  static const OuterTables T;
  int rc = BS_OK;
  if (!Bf->outer) {
    CK(cudaMalloc(&Bf->outer, sizeof T.o2 + sizeof T.o3));
    CK(cudaMemcpy(Bf->outer, T.o2, sizeof T.o2, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(Bf->outer + sizeof T.o2, T.o3, sizeof T.o3, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&Bf->next, sizeof(unsigned long long)));
    CK(cudaMalloc(&Bf->hit_min, sizeof(long long)));
  }
  std::vector<AbCandDev> hc(ncand);
  for (long long i = 0; i < ncand; i++) {
    if (cands[i].nrows < 0 || cands[i].nrows > 65535) return BS_ERR_ARG;
    if (cands[i].nrows > 0 &&
        (!rows || cands[i].row_off < 0 || cands[i].row_off + cands[i].nrows > nrows_total))
      return BS_ERR_ARG;
  }
  // ---- the allowed-row masks of every distinct row set (kept on the device for the next
  // batch when it has the same rows: the lane completes one cell in several batches) ----
  const int m = opt->m;
  int tic[8] = {0};
  for (int c = 0; c < m; c++)
    for (int p = c; p < n1; p += m) tic[c]++;
  int TV = 0;
  for (int c = 0; c < m; c++) TV = tic[c] > TV ? tic[c] : TV;
  const int V = 2 * TV + 3;
  std::vector<std::pair<long long, int>> sets;
  std::vector<int> set_of(ncand, -1);
  for (long long i = 0; i < ncand; i++) {
    if (cands[i].nrows == 0) continue;
    const std::pair<long long, int> key(cands[i].row_off, cands[i].nrows);
    int k = (int)sets.size() - 1;
    while (k >= 0 && sets[k] != key) k--;
    if (k < 0) {
      sets.push_back(key);
      k = (int)sets.size() - 1;
    }
    set_of[i] = k;
  }
  bool same = Bf->mask_m == m && Bf->mask_n1 == n1 && sets.size() <= Bf->mask_sets.size();
  std::vector<long long> offs(sets.size(), 0);
  for (size_t k = 0; same && k < sets.size(); k++) {
    size_t j = 0;
    while (j < Bf->mask_sets.size() && Bf->mask_sets[j] != sets[k]) j++;
    if (j == Bf->mask_sets.size()) { same = false; break; }
    const long long lo = sets[k].first * 16, len = (long long)sets[k].second * 16;
    if ((long long)Bf->mask_rows.size() < lo + len ||
        memcmp(Bf->mask_rows.data() + lo, rows + lo, (size_t)len) != 0) { same = false; break; }
    offs[k] = Bf->mask_offs[j];
  }
  int Wcap = 1;
  for (auto &k : sets) Wcap = std::max(Wcap, (k.second + 63) / 64);
  if (Wcap > 65535) return BS_ERR_CAP;  // a row range is kept in 16-bit halves
  if (!same && !sets.empty()) {
    long long total = 0;
    for (size_t k = 0; k < sets.size(); k++) {
      offs[k] = total;
      total += (long long)m * 4 * V * ((sets[k].second + 63) / 64);
    }
    std::vector<uint64_t> hm((size_t)total, 0);
    for (size_t k = 0; k < sets.size(); k++) {
      const int W = (sets[k].second + 63) / 64;
      for (int r = 0; r < sets[k].second; r++) {
        const int8_t *row = rows + 16 * (sets[k].first + r);
        const uint64_t bit = 1ULL << (r & 63);
        for (int c = 0; c < m; c++)
          for (int kind = 0; kind < 4; kind++) {
            const int x = kind < 2 ? row[c] : row[8 + c];
            // kinds 0, 2: value >= v for v <= x; kinds 1, 3: value <= v for v >= x
            const int lo = (kind & 1) ? x : -TV - 1, hi = (kind & 1) ? TV + 1 : x;
            uint64_t *base = hm.data() + offs[k] + (size_t)(c * 4 + kind) * V * W + (r >> 6);
            for (int v = std::max(lo, -TV - 1); v <= std::min(hi, TV + 1); v++)
              base[(size_t)(v + TV + 1) * W] |= bit;
          }
      }
    }
    rc = bs_ensure_dev((void **)&Bf->masks, &Bf->masks_cap, total, sizeof(uint64_t));
    if (rc) return rc;
    CK(cudaMemcpyAsync(Bf->masks, hm.data(), sizeof(uint64_t) * total, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // hm is freed on return
    Bf->mask_rows.assign(rows, rows + 16 * nrows_total);
    Bf->mask_sets = sets;
    Bf->mask_offs = offs;
    Bf->mask_m = m;
    Bf->mask_n1 = n1;
  }
  for (long long i = 0; i < ncand; i++) {
    hc[i].c = cands[i].c;
    hc[i].d = cands[i].d;
    hc[i].nrows = cands[i].nrows;
    hc[i].W = cands[i].nrows > 0 ? (cands[i].nrows + 63) / 64 : 0;
    hc[i].mask_off = set_of[i] >= 0 ? offs[set_of[i]] : 0;
    hc[i].row_off = cands[i].nrows > 0 ? cands[i].row_off : 0;
  }
  if (opt->blocks_per_sm < 0 || opt->blocks_per_sm > 3) return BS_ERR_ARG;
  const int grid = ctx->num_sms * (opt->blocks_per_sm ? opt->blocks_per_sm : 2);
  const long long slots = (long long)grid * AB_WARPS;
  rc = bs_ensure_dev((void **)&Bf->cands, &Bf->cand_cap, ncand, sizeof(AbCandDev));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->verdict, &Bf->v_cap, ncand, sizeof(int32_t));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->nodes, &Bf->n_cap, ncand, sizeof(long long));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->ab, &Bf->ab_cap, 2 * ncand, sizeof(uint64_t));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->bits, &Bf->bits_cap, slots * (half + 1) * (long long)Wcap,
                              sizeof(uint64_t));
  if (!rc && opt->a2 && nrows_total > 0)
    rc = bs_ensure_dev((void **)&Bf->rows8, &Bf->rows8_cap, 16 * nrows_total, 1);
  if (rc) return rc;
  CK(cudaMemcpyAsync(Bf->cands, hc.data(), sizeof(AbCandDev) * ncand, cudaMemcpyHostToDevice, s));
  if (opt->a2 && nrows_total > 0)
    CK(cudaMemcpyAsync(Bf->rows8, rows, (size_t)16 * nrows_total, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(Bf->next, 0, sizeof(unsigned long long), s));
  const long long big = 1LL << 62;
  CK(cudaMemcpyAsync(Bf->hit_min, &big, sizeof big, cudaMemcpyHostToDevice, s));
  AbParams P;
  P.n = n; P.n1 = n1; P.L = n1; P.half = half; P.m = opt->m;
  P.absA = ctx->sig[0] < 0 ? -ctx->sig[0] : ctx->sig[0];
  P.absB = ctx->sig[1] < 0 ? -ctx->sig[1] : ctx->sig[1];
  P.outer_k = opt->outer_k; P.early = opt->early; P.canon = opt->canon;
  P.first_hit = opt->first_hit;
  P.budget = opt->budget;
  P.max_cycles = opt->max_seconds > 0 ? (long long)(opt->max_seconds * 2.0e9) : 0;
  P.cands = Bf->cands; P.ncand = ncand;
  P.masks = Bf->masks; P.T = TV; P.V = V;
  P.bits = Bf->bits; P.Wcap = Wcap;
  // A2 blocks (init_a2_tables, wz_match.cpp:1000-1016): residues paired by the reflection
  // r -> (L-1-r) mod m, the free middle's block at odd L, and per depth p the quads left in
  // each block (mirror positions i = p..half-1 of residue i mod m)
  P.a2 = opt->a2;
  P.rows8 = Bf->rows8;
  P.a2_nblk = 0;
  memset(P.a2_r, 0, sizeof P.a2_r); memset(P.a2_s, 0, sizeof P.a2_s);
  memset(P.a2_mid, 0, sizeof P.a2_mid); memset(P.a2_cnt, 0, sizeof P.a2_cnt);
  {
    int blk_of[8];
    for (int c = 0; c < 8; c++) blk_of[c] = -1;
    for (int c = 0; c < m; c++) {
      if (blk_of[c] >= 0) continue;
      const int sref = ((n1 - 1 - c) % m + m) % m;
      P.a2_r[P.a2_nblk] = (int8_t)c;
      P.a2_s[P.a2_nblk] = (int8_t)sref;
      blk_of[c] = blk_of[sref] = P.a2_nblk++;
    }
    if (n1 % 2 == 1) P.a2_mid[blk_of[half % m]] = 1;
    for (int p = 0; p <= half + 1 && p < AB_MAXLV + 2; p++)
      for (int i = p; i < half; i++) P.a2_cnt[p][blk_of[i % m]]++;
  }
  P.outer2 = Bf->outer; P.outer3 = Bf->outer + sizeof T.o2;
  P.next = Bf->next; P.hit_min = Bf->hit_min;
  P.verdict = Bf->verdict; P.nodes_out = Bf->nodes; P.ab_out = Bf->ab;
  P.stop_flag = ctx->d_stop; P.status = ctx->d_status;
  for (int c = 0; c < 8; c++) {
    P.tic[c] = 0;
    if (c < opt->m)
      for (int p = c; p < n1; p += opt->m) P.tic[c]++;
  }
  bs_timed_begin(ctx);
  if (opt->blocks_per_sm == 3)
    ab_kernel<3><<<grid, 32 * AB_WARPS, 0, s>>>(P);
  else
    ab_kernel<2><<<grid, 32 * AB_WARPS, 0, s>>>(P);
  bs_timed_end(ctx);
  CK(cudaGetLastError());
  std::vector<uint64_t> ab(2 * ncand);
  CK(cudaMemcpyAsync(verdict, Bf->verdict, sizeof(int32_t) * ncand, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(nodes, Bf->nodes, sizeof(long long) * ncand, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(ab.data(), Bf->ab, sizeof(uint64_t) * 2 * ncand, cudaMemcpyDeviceToHost, s));
  int status = 0;
  CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (status) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s);
    return status;
  }
  // independent exact NPAF recheck of every completion (wz_match.cpp:1328-1335): verdict 4
  for (long long i = 0; i < ncand; i++) {
    if (verdict[i] != 0) continue;
    int8_t a[64], b[64], c[64], d[64];
    words_to_seq(ab[2 * i], n1, a);
    words_to_seq(ab[2 * i + 1], n1, b);
    words_to_seq(cands[i].c, n, c);
    words_to_seq(cands[i].d, n, d);
    for (int sh = 1; sh <= n; sh++) {
      int v = 0;
      for (int t = 0; t + sh < n1; t++) v += a[t] * a[t + sh] + b[t] * b[t + sh];
      for (int t = 0; t + sh < n; t++) v += c[t] * c[t + sh] + d[t] * d[t + sh];
      if (v != 0) { verdict[i] = 4; break; }
    }
    if (A) memcpy(A + i * n1, a, n1);
    if (B) memcpy(B + i * n1, b, n1);
  }
  // the stop flag was raised: candidates not run are marked -1, the others are final
  return *ctx->h_stop ? BS_STOPPED : BS_OK;
}
