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

#include <vector>

#include "bsfh_internal.cuh"

namespace {

#define FULL_MASK 0xffffffffu
constexpr int AB_WARPS = 8;  // warps per block
constexpr int AB_MAXLV = 34; // levels 0..half (n1 <= 64)

struct AbCandDev {
  uint64_t c, d;
  long long row_off;
  int nrows, pad;
};

struct AbParams {
  int n, n1, L, half, m, absA, absB;
  int outer_k, early, canon, first_hit;
  long long budget;
  long long max_cycles;
  const AbCandDev *cands;
  long long ncand;
  const uint64_t *roww;  // allowed rows as 4 words each (see RowBox)
  uint64_t m7, mb;       // bit 7 / all bits of each used class byte
  uint16_t *stacks;  // per warp slot: levels 1..half, maxrows entries each
  int maxrows;
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

__device__ __forceinline__ int sgnbit(uint64_t w, int p) { return ((w >> p) & 1ULL) ? 1 : -1; }
__device__ __forceinline__ int fld(uint64_t w, int c) { return (int)((w >> (8 * c)) & 255) - 64; }
__device__ __forceinline__ int absi(int x) { return x < 0 ? -x : x; }

struct Lanes {
  int t0, t1;    // target at s0 = lane+1, s1 = lane+33
  int D0, D1;    // Dab
  int K0, K1;    // Kab
  int s0, s1;    // shifts (0 when out of range)
};

// Place (sign +1) or remove (sign -1) position p with values (av, bv) against the placed set
// Pm (which excludes p); A,B hold the placed signs as bits.
__device__ __forceinline__ void lane_update(Lanes &v, int p, int av, int bv, uint64_t A, uint64_t B,
                                            uint64_t Pm, int L, int sign) {
  if (v.s0) {
    int q = p - v.s0;
    if (q >= 0 && ((Pm >> q) & 1ULL)) { v.D0 += sign * (sgnbit(A, q) * av + sgnbit(B, q) * bv); v.K0 -= 2 * sign; }
    q = p + v.s0;
    if (q < L && ((Pm >> q) & 1ULL)) { v.D0 += sign * (sgnbit(A, q) * av + sgnbit(B, q) * bv); v.K0 -= 2 * sign; }
  }
  if (v.s1) {
    int q = p - v.s1;
    if (q >= 0 && ((Pm >> q) & 1ULL)) { v.D1 += sign * (sgnbit(A, q) * av + sgnbit(B, q) * bv); v.K1 -= 2 * sign; }
    q = p + v.s1;
    if (q < L && ((Pm >> q) & 1ULL)) { v.D1 += sign * (sgnbit(A, q) * av + sgnbit(B, q) * bv); v.K1 -= 2 * sign; }
  }
}

// residual target[s] - Dab[s] at shift s (1 <= s <= n), uniform
__device__ __forceinline__ int resid_at(const Lanes &v, int s) {
  int mine = ((s - 1) >> 5) ? (v.t1 - v.D1) : (v.t0 - v.D0);
  return __shfl_sync(FULL_MASK, mine, (s - 1) & 31);
}

struct Uni {
  uint64_t A, B, Pm;
  uint64_t pa, pb, plc;  // class partial sums / placed counts, 8-bit fields (bias 64)
  int sumA, sumB;
};

__device__ __forceinline__ void place(Uni &u, Lanes &v, int p, int av, int bv, int L, int m) {
  lane_update(v, p, av, bv, u.A, u.B, u.Pm, L, +1);
  u.Pm |= 1ULL << p;
  if (av > 0) u.A |= 1ULL << p;
  if (bv > 0) u.B |= 1ULL << p;
  const int c = p % m;
  u.pa += (uint64_t)(int64_t)av << (8 * c);
  u.pb += (uint64_t)(int64_t)bv << (8 * c);
  u.plc += 1ULL << (8 * c);
  u.sumA += av;
  u.sumB += bv;
}

__device__ __forceinline__ void unplace(Uni &u, Lanes &v, int p, int L, int m) {
  const int av = sgnbit(u.A, p), bv = sgnbit(u.B, p);
  u.Pm &= ~(1ULL << p);
  u.A &= ~(1ULL << p);
  u.B &= ~(1ULL << p);
  const int c = p % m;
  u.pa -= (uint64_t)(int64_t)av << (8 * c);
  u.pb -= (uint64_t)(int64_t)bv << (8 * c);
  u.plc -= 1ULL << (8 * c);
  u.sumA -= av;
  u.sumB -= bv;
  lane_update(v, p, av, bv, u.A, u.B, u.Pm, L, -1);
}

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

// outer_mask, wz_match.cpp:601-618
__device__ __forceinline__ unsigned outer_mask(const AbParams &P, const Uni &u, const Lanes &v, int d) {
  const int k = P.outer_k, L = P.L;
  if (k < 2 || d < k || d + k > L / 2 || !(u.A & 1ULL) || !(u.B & 1ULL)) return 0xFFu;
  int pat = (int)((u.A >> (L - 1)) & 1ULL), mul = 2;
  for (int t = 1; t < k; t++) {
    int sb = (int)(((u.A >> t) & 1) << 3 | ((u.B >> t) & 1) << 2 | ((u.A >> (L - 1 - t)) & 1) << 1 |
                   ((u.B >> (L - 1 - t)) & 1));
    int q = kPosOf[sb];
    if (q < 0) return 0xFFu;
    pat += mul * q;
    mul *= 8;
  }
  int R[3];
  for (int j = 0; j < k; j++) {
    R[j] = resid_at(v, L - 1 - d - j);
    if ((R[j] & 1) || R[j] < -4 * (j + 1) || R[j] > 4 * (j + 1)) return 0u;
  }
  if (k == 2) return P.outer2[(pat * 5 + (R[0] / 2 + 2)) * 9 + (R[1] / 2 + 4)];
  return P.outer3[((pat * 5 + (R[0] / 2 + 2)) * 9 + (R[1] / 2 + 4)) * 13 + (R[2] / 2 + 6)];
}

// first quad index >= k at level d that passes the outer mask and the canon filter
__device__ __forceinline__ int next_quad(const AbParams &P, int d, int k, unsigned omask, uint32_t ties) {
  for (; k < 8; k++) {
    if (d > 0 && !((omask >> k) & 1u)) continue;
    uint32_t q = quad_bits(d, k), o;
    int a1 = (q & 8) ? 1 : -1, b1 = (q & 4) ? 1 : -1, a2 = (q & 2) ? 1 : -1, b2 = (q & 1) ? 1 : -1;
    if (canon_ok(P, d, ties, a1, b1, a2, b2, o)) return k;
  }
  return 8;
}

// An allowed row (k, r) as four words of biased class bytes: k+64, 64-k, r+64, 64-r. A level's
// box test |k_c - pa_c| <= rem_c, |r_c - pb_c| <= rem_c (wz_match.cpp:1055-1075) then reads
// k_c - pa_c + rem_c + 128 >= 128 and pa_c - k_c + rem_c + 128 >= 128 (and the same for r) off
// bit 7 of four byte-wise sums: every byte stays in [84, 194], so no carry crosses a class.
struct RowBox { uint64_t k1, k2, r1, r2; };

__device__ __forceinline__ RowBox row_box_of(const Uni &u, const AbParams &P) {
  RowBox b = {0, 0, 0, 0};
  for (int c = 0; c < 6; c++) {
    if (c >= P.m) break;
    const int rem = P.tic[c] - fld(u.plc, c), pa = fld(u.pa, c), pb = fld(u.pb, c);
    b.k1 |= (uint64_t)(rem - pa + 64) << (8 * c);
    b.k2 |= (uint64_t)(rem + pa + 64) << (8 * c);
    b.r1 |= (uint64_t)(rem - pb + 64) << (8 * c);
    b.r2 |= (uint64_t)(rem + pb + 64) << (8 * c);
  }
  return b;
}
__device__ __forceinline__ bool row_box(const uint64_t *row, const RowBox &b, const AbParams &P) {
  const uint64_t t = (row[0] + b.k1) & (row[1] + b.k2) & (row[2] + b.r1) & (row[3] + b.r2);
  return (t & P.m7) == P.m7;
}
// the leaf test of a row: its class sums equal the placed ones (pa, pb hold sum + 64)
__device__ __forceinline__ bool row_exact(const uint64_t *row, const Uni &u, const AbParams &P) {
  return ((row[0] ^ u.pa) & P.mb) == 0 && ((row[2] ^ u.pb) & P.mb) == 0;
}

__global__ void __launch_bounds__(32 * AB_WARPS) ab_kernel(AbParams P) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long slot = (long long)blockIdx.x * AB_WARPS + wib;
  __shared__ uint32_t s_ctrl[AB_WARPS][AB_MAXLV];  // k | omask << 4 | ties << 12
  __shared__ int s_res[AB_WARPS][AB_MAXLV];        // early-check residual of the level
  __shared__ int s_len[AB_WARPS][AB_MAXLV];        // allowed-row list length of the level
  uint32_t *ctrl = s_ctrl[wib];
  int *res = s_res[wib], *len = s_len[wib];
  uint16_t *stk = P.stacks + (size_t)slot * P.half * P.maxrows;
  const int L = P.L, n = P.n, half = P.half, m = P.m;

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
    const uint64_t *rows = cd.nrows > 0 ? P.roww + 4 * (size_t)cd.row_off : nullptr;
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
    v.K0 = v.s0 ? 2 * (P.n1 - v.s0) : 0;
    v.K1 = v.s1 ? 2 * (P.n1 - v.s1) : 0;
    Uni u;
    u.A = u.B = u.Pm = 0;
    u.pa = u.pb = u.plc = 0;
    for (int c = 0; c < 8; c++) {
      u.pa |= 64ULL << (8 * c);
      u.pb |= 64ULL << (8 * c);
      u.plc |= 64ULL << (8 * c);
    }
    u.sumA = u.sumB = 0;
    long long nodes = 0, cur = 0;
    bool aborted = false, found = false, abandoned = false;
    const long long t_start = clock64();
    int d = 0;
    if (lane == 0) {
      ctrl[0] = 0u | (0xFFu << 4) | (5u << 12);  // ties: a_tied = b_tied = 1
      res[0] = 0;
      len[0] = cd.nrows;
    }
    __syncwarp();
    unsigned long long steps = 0;
    while (true) {
      if ((++steps & 1023) == 0) {
        bool stop = (long long)idx > *(volatile long long *)P.hit_min || *P.stop_flag ||
                    (P.max_cycles > 0 && clock64() - t_start > P.max_cycles);
        if (__shfl_sync(FULL_MASK, (int)stop, 0)) { abandoned = true; break; }
      }
      if (d == half) {
        // ---- leaf: final_ok (and the free middle for odd length), wz_match.cpp:1178-1205 ----
        auto final_ok = [&](int sA, int sB) -> bool {
          if (absi(sA) != P.absA || absi(sB) != P.absB) return false;
          bool eq = (!v.s0 || v.D0 == v.t0) && (!v.s1 || v.D1 == v.t1);
          if (!__all_sync(FULL_MASK, eq)) return false;
          if (rows) {
            const int cnt = len[half];
            const uint16_t *lst = stk + (size_t)(half - 1) * P.maxrows;
            bool any = false;
            for (int base = 0; base < cnt && !any; base += 32) {
              int t = base + lane;
              bool hit = t < cnt && row_exact(rows + 4 * (size_t)lst[t], u, P);
              any = __any_sync(FULL_MASK, hit);
            }
            if (!any) return false;
          }
          return true;
        };
        if (L & 1) {
          const int mid = half;
          for (int km = 0; km < 4 && !found; km++) {
            int av = (km < 2) ? 1 : -1, bv = (km & 1) ? -1 : 1;
            place(u, v, mid, av, bv, L, m);
            nodes++;
            if (final_ok(u.sumA, u.sumB)) found = true;
            else unplace(u, v, mid, L, m);
          }
        } else if (final_ok(u.sumA, u.sumB)) {
          found = true;
        }
        if (found) break;
        // back to the parent level
        d--;
        {
          uint32_t c0 = ctrl[d];
          int k = c0 & 15;
          unplace(u, v, L - 1 - d, L, m);
          unplace(u, v, d, L, m);
          __syncwarp();
          if (lane == 0) ctrl[d] = (c0 & ~15u) | (uint32_t)(k + 1);
          __syncwarp();
        }
        continue;
      }
      const uint32_t c0 = ctrl[d];
      const unsigned omask = (c0 >> 4) & 0xFF;
      const uint32_t ties = (c0 >> 12) & 15;
      int k = next_quad(P, d, c0 & 15, omask, ties);
      if (k == 8) {
        if (d == 0) break;  // clean exhaustion
        d--;
        uint32_t cp = ctrl[d];
        unplace(u, v, L - 1 - d, L, m);
        unplace(u, v, d, L, m);
        __syncwarp();
        if (lane == 0) ctrl[d] = (cp & ~15u) | (uint32_t)((cp & 15) + 1);
        __syncwarp();
        continue;
      }
      const uint32_t q = quad_bits(d, k);
      const int a1 = (q & 8) ? 1 : -1, b1 = (q & 4) ? 1 : -1, a2 = (q & 2) ? 1 : -1, b2 = (q & 1) ? 1 : -1;
      uint32_t nties;
      canon_ok(P, d, ties, a1, b1, a2, b2, nties);
      // charge the node before placing (wz_match.cpp:1243-1248)
      nodes++;
      if (P.budget > 0 && ++cur > P.budget) {
        __syncwarp();
        if (lane == 0) ctrl[d] = (c0 & ~15u) | (uint32_t)k;
        __syncwarp();
        aborted = true;
        break;
      }
      // early outer-correlation check (wz_match.cpp:1256-1259)
      if (P.early && d > 0) {
        int lhs = sgnbit(u.A, 0) * a2 + sgnbit(u.B, 0) * b2 + sgnbit(u.A, L - 1) * a1 + sgnbit(u.B, L - 1) * b1;
        if (lhs != res[d]) {
          __syncwarp();
          if (lane == 0) ctrl[d] = (c0 & ~15u) | (uint32_t)(k + 1);
          __syncwarp();
          continue;
        }
      }
      place(u, v, d, a1, b1, L, m);
      place(u, v, L - 1 - d, a2, b2, L, m);
      const int rem = L - 2 * (d + 1);
      bool prune = !(((absi(P.absA - u.sumA) <= rem) || (absi(-P.absA - u.sumA) <= rem)) &&
                     ((absi(P.absB - u.sumB) <= rem) || (absi(-P.absB - u.sumB) <= rem)));
      if (!prune) {
        bool bad = (v.s0 && absi(v.t0 - v.D0) > v.K0) || (v.s1 && absi(v.t1 - v.D1) > v.K1);
        prune = __any_sync(FULL_MASK, bad);
      }
      if (!prune && rows) {
        // fh_abp_filter(d): the level-(d+1) list from the level-d list (all rows at d = 0)
        const int srclen = (d == 0) ? cd.nrows : len[d];
        const uint16_t *src = stk + (size_t)(d - 1) * P.maxrows;
        uint16_t *dst = stk + (size_t)d * P.maxrows;
        const RowBox box = row_box_of(u, P);
        int cnt = 0;
        for (int base = 0; base < srclen; base += 32) {
          int t = base + lane;
          int ri = 0;
          bool ok = false;
          if (t < srclen) {
            ri = (d == 0) ? t : src[t];
            ok = row_box(rows + 4 * (size_t)ri, box, P);
          }
          unsigned ball = __ballot_sync(FULL_MASK, ok);
          if (ok) dst[cnt + __popc(ball & ((1u << lane) - 1u))] = (uint16_t)ri;
          cnt += __popc(ball);
        }
        __syncwarp();
        if (lane == 0) len[d + 1] = cnt;
        __syncwarp();
        prune = (cnt == 0);
      }
      if (prune) {
        unplace(u, v, L - 1 - d, L, m);
        unplace(u, v, d, L, m);
        __syncwarp();
        if (lane == 0) ctrl[d] = (c0 & ~15u) | (uint32_t)(k + 1);
        __syncwarp();
        continue;
      }
      // descend: the child level's entry work (its outer mask may end it immediately)
      __syncwarp();
      if (lane == 0) ctrl[d] = (c0 & ~15u) | (uint32_t)k;
      __syncwarp();
      const int nd = d + 1;
      unsigned om = 0xFFu;
      int r_e = 0;
      if (nd < half) {
        if (P.outer_k) om = outer_mask(P, u, v, nd);
        r_e = resid_at(v, L - 1 - nd);
      }
      if (om == 0u) {  // fh_ab_search(d+1) returns false at once: undo and try the next quad
        unplace(u, v, L - 1 - d, L, m);
        unplace(u, v, d, L, m);
        __syncwarp();
        if (lane == 0) ctrl[d] = (c0 & ~15u) | (uint32_t)(k + 1);
        __syncwarp();
        continue;
      }
      __syncwarp();
      if (lane == 0) {
        ctrl[nd] = 0u | (om << 4) | (nties << 12);
        res[nd] = r_e;
      }
      __syncwarp();
      d = nd;
    }
    if (aborted) {
      // Every ancestor level whose loop has another eligible quad charges one more node before
      // it returns (wz_match.cpp:1243-1247 reached again with fh_cur already over budget).
      for (int j = d - 1; j >= 0; j--) {
        uint32_t cj = ctrl[j];
        if (next_quad(P, j, (cj & 15) + 1, (cj >> 4) & 0xFF, (cj >> 12) & 15) < 8) nodes++;
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
  uint64_t *rows = nullptr; long long rows_cap = 0;  // 4 words per row
  uint16_t *stacks = nullptr; long long stack_cap = 0;
  int32_t *verdict = nullptr; long long v_cap = 0;
  long long *nodes = nullptr; long long n_cap = 0;
  uint64_t *ab = nullptr; long long ab_cap = 0;
  unsigned long long *next = nullptr;
  long long *hit_min = nullptr;
  int *stop = nullptr;
};

static AbBufs *ab_bufs(bs_ctx *ctx) {
  if (!ctx->ab_bufs) ctx->ab_bufs = new AbBufs();
  return (AbBufs *)ctx->ab_bufs;
}

void bs_ab_free(bs_ctx *ctx) {
  AbBufs *b = (AbBufs *)ctx->ab_bufs;
  if (!b) return;
  cudaFree(b->outer); cudaFree(b->cands); cudaFree(b->rows); cudaFree(b->stacks);
  cudaFree(b->verdict); cudaFree(b->nodes); cudaFree(b->ab); cudaFree(b->next);
  cudaFree(b->hit_min); cudaFree(b->stop);
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
    CK(cudaMalloc(&Bf->stop, sizeof(int)));
    CK(cudaMemset(Bf->stop, 0, sizeof(int)));
  }
  int maxrows = 1;
  std::vector<AbCandDev> hc(ncand);
  for (long long i = 0; i < ncand; i++) {
    hc[i].c = cands[i].c;
    hc[i].d = cands[i].d;
    hc[i].row_off = cands[i].row_off;
    hc[i].nrows = cands[i].nrows;
    hc[i].pad = 0;
    if (cands[i].nrows < 0 || cands[i].nrows > 65535) return BS_ERR_ARG;
    if (cands[i].nrows > 0 &&
        (!rows || cands[i].row_off < 0 || cands[i].row_off + cands[i].nrows > nrows_total))
      return BS_ERR_ARG;
    if (cands[i].nrows > maxrows) maxrows = cands[i].nrows;
  }
  const int grid = ctx->num_sms * 2;
  const long long slots = (long long)grid * AB_WARPS;
  rc = bs_ensure_dev((void **)&Bf->cands, &Bf->cand_cap, ncand, sizeof(AbCandDev));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->verdict, &Bf->v_cap, ncand, sizeof(int32_t));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->nodes, &Bf->n_cap, ncand, sizeof(long long));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->ab, &Bf->ab_cap, 2 * ncand, sizeof(uint64_t));
  if (!rc && nrows_total > 0)
    rc = bs_ensure_dev((void **)&Bf->rows, &Bf->rows_cap, nrows_total * 4, sizeof(uint64_t));
  if (!rc) rc = bs_ensure_dev((void **)&Bf->stacks, &Bf->stack_cap, slots * half * (long long)maxrows,
                              sizeof(uint16_t));
  if (rc) return rc;
  CK(cudaMemcpyAsync(Bf->cands, hc.data(), sizeof(AbCandDev) * ncand, cudaMemcpyHostToDevice, s));
  std::vector<uint64_t> roww;
  if (nrows_total > 0) {
    // each row (k[8], r[8], int8) as four words of biased class bytes: k+64, 64-k, r+64, 64-r
    roww.assign(4 * (size_t)nrows_total, 0);
    for (long long r = 0; r < nrows_total; r++)
      for (int c = 0; c < opt->m; c++) {
        const int k = rows[16 * r + c], q = rows[16 * r + 8 + c];
        roww[4 * r + 0] |= (uint64_t)(k + 64) << (8 * c);
        roww[4 * r + 1] |= (uint64_t)(64 - k) << (8 * c);
        roww[4 * r + 2] |= (uint64_t)(q + 64) << (8 * c);
        roww[4 * r + 3] |= (uint64_t)(64 - q) << (8 * c);
      }
    CK(cudaMemcpyAsync(Bf->rows, roww.data(), sizeof(uint64_t) * 4 * nrows_total, cudaMemcpyHostToDevice, s));
  }
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
  P.roww = Bf->rows; P.stacks = Bf->stacks; P.maxrows = maxrows;
  P.m7 = 0; P.mb = 0;
  for (int c = 0; c < opt->m; c++) { P.m7 |= 0x80ULL << (8 * c); P.mb |= 0xFFULL << (8 * c); }
  P.outer2 = Bf->outer; P.outer3 = Bf->outer + sizeof T.o2;
  P.next = Bf->next; P.hit_min = Bf->hit_min;
  P.verdict = Bf->verdict; P.nodes_out = Bf->nodes; P.ab_out = Bf->ab;
  P.stop_flag = Bf->stop; P.status = ctx->d_status;
  for (int c = 0; c < 8; c++) {
    P.tic[c] = 0;
    if (c < opt->m)
      for (int p = c; p < n1; p += opt->m) P.tic[c]++;
  }
  bs_timed_begin(ctx);
  ab_kernel<<<grid, 32 * AB_WARPS, 0, s>>>(P);
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
  return BS_OK;
}
