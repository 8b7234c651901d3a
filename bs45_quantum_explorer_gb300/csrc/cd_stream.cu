// cd_stream.cu - the C,D mirror-quad stream (the reference's count_pairs22,
// src/solver/wz_match.cpp:678-784) for a batch of cells, on the GPU.
//
// Structure:
//   1. Host: each cell's DFS tree is expanded to a split depth D in the reference's branch
//      order (quad index order, reversed under STREAM_REV), giving coarse prefixes in DFS
//      order. Nodes above D are counted here exactly as the reference counts rec() calls.
//   2. Waves: runs of coarse prefixes, in order, refined on the host to enough subtree roots
//      to fill the GPU. Device, cd_dfs_kernel: groups of eight lanes take roots from a queue
//      and walk each subtree iteratively; the eight lanes test a node's eight children in
//      one step. A class-exact leaf is appended with its branch path as key. A launch stops
//      when the leaf buffer is full or its time is up; suspended walks resume in the next
//      launch, and when few remain the host splits them into their remaining subtrees.
//   3. Device: the Hall filter (tensor-core form by default) decides every leaf; survivors are
//      compacted with their keys; sorting by (cell, path) restores the reference's order.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <chrono>
#include <cmath>
#include <vector>

#include "bsfh_internal.cuh"

namespace {

#define FULL_MASK 0xffffffffu

struct CellDev {
  int8_t tx[8], ty[8];
};

// A subtree root handed to the device: the node reached by the branch indices of depths
// 0..depth-1 (4 bits per depth; depths 0-15 in dig0, 16-31 in dig1).
struct Prefix {
  uint32_t cell;
  uint32_t depth;
  uint64_t dig0, dig1;
};

// A suspended walk: the subtree of root depth D, now at the node of depth d with next child
// kk, and the leaf children of that node (bit k = child k) not yet written.
struct Saved {
  uint32_t cell;
  uint16_t D, d, kk, owed;
  uint32_t pad;
  uint64_t dig0, dig1;  // branch indices of depths 0..d-1
};

struct CdParams {
  int L, m, half;
  uint64_t feas_mask;   // bit 6 of every used class byte
  const void *fx;       // QuadFx[32][16]: effect of branch kk at depth d (reversal applied)
  const uint64_t *posmask;  // [32]: bits of positions d and L-1-d
  const CellDev *cells;
  const Prefix *prefixes;
  long long nprefix;
  unsigned long long *next_prefix;
  const Saved *saved_in;
  int nsaved_in;
  Saved *saved_out;
  unsigned *nsaved_out;
  int saved_cap;
  uint64_t *leaf_words;  // [cap][2]: C, D
  uint64_t *leaf_keys;   // [cap][2]: the leaf's path key (see path_key)
  uint32_t *leaf_cell;   // [cap]
  unsigned long long *leaf_count;
  unsigned long long leaf_cap;
  unsigned long long *cell_nodes, *cell_leaves;
  int *stop_flag;         // set when the leaf buffer is full or the round's time is up
  unsigned long long round_ns;  // > 0: suspend every walk after about this long
  int *status;
  // CD_PRUNE bit 2 (the REACH kernels only): the mirror blocks {r, s} as 4-bit class pairs
  // per byte, and per depth the quads left in each block (one byte per block)
  uint32_t reach_blk;
  const uint32_t *reach_q;  // [32]
};


// The digits of a walk live in two registers (depths 0-15 and 16-31); selecting between
// them, rather than indexing an array, keeps them out of local memory.
__device__ __forceinline__ int getdig(uint64_t d0, uint64_t d1, int d) {
  const uint64_t w = (d < 16) ? d0 : d1;
  return (int)((w >> (4 * (d & 15))) & 15);
}
__device__ __forceinline__ void setdig(uint64_t &d0, uint64_t &d1, int d, int v) {
  const int s = 4 * (d & 15);
  if (d < 16) d0 = (d0 & ~(15ULL << s)) | ((uint64_t)v << s);
  else d1 = (d1 & ~(15ULL << s)) | ((uint64_t)v << s);
}

// Per-class feasibility as four "slack" words: for each class c (byte c, bias 64)
//   rem - dx, rem + dx, rem - dy, rem + dy,  dx = tx - px, dy = ty - py, rem = free slots.
// The reference's capacity test |dx| <= rem and |dy| <= rem holds exactly when all four are
// >= 0, i.e. when bit 6 of every used byte is set (bytes stay in [0, 127]: a valid node has
// slack in [0, 22] and one quad lowers a byte by at most 4). Its parity test is invariant
// once the root passes, so the walk needs neither. A quad at depth d, branch kk, changes the
// words by a constant: dsl[d][kk][0..3] (host-built), and the sequences by bits bx/by.
struct Walk {
  uint64_t s0, s1, s2, s3;
  uint64_t X, Y;
};

struct QuadFx {  // the effect of branch kk at depth d
  int64_t ds[4];
  uint64_t bx, by;
};

__host__ __device__ __forceinline__ int fld(uint64_t w, int c) { return (int)((w >> (8 * c)) & 255) - 64; }

__host__ __device__ __forceinline__ void place(Walk &w, const QuadFx &f) {
  w.s0 += (uint64_t)f.ds[0];
  w.s1 += (uint64_t)f.ds[1];
  w.s2 += (uint64_t)f.ds[2];
  w.s3 += (uint64_t)f.ds[3];
  w.X |= f.bx;
  w.Y |= f.by;
}
__device__ __forceinline__ void unplace(Walk &w, const QuadFx &f, uint64_t posmask) {
  w.s0 -= (uint64_t)f.ds[0];
  w.s1 -= (uint64_t)f.ds[1];
  w.s2 -= (uint64_t)f.ds[2];
  w.s3 -= (uint64_t)f.ds[3];
  w.X &= ~posmask;
  w.Y &= ~posmask;
}

__host__ __device__ __forceinline__ void init_walk(Walk &w, const CellDev &cell, int L, int m) {
  w.s0 = w.s1 = w.s2 = w.s3 = 0x4040404040404040ULL;
  for (int c = 0; c < m; c++) {
    const int cnt = (L - c + m - 1) / m;  // positions p < L with p % m == c
    const uint64_t clear = ~(0xFFULL << (8 * c));
    w.s0 = (w.s0 & clear) | ((uint64_t)(cnt - cell.tx[c] + 64) << (8 * c));
    w.s1 = (w.s1 & clear) | ((uint64_t)(cnt + cell.tx[c] + 64) << (8 * c));
    w.s2 = (w.s2 & clear) | ((uint64_t)(cnt - cell.ty[c] + 64) << (8 * c));
    w.s3 = (w.s3 & clear) | ((uint64_t)(cnt + cell.ty[c] + 64) << (8 * c));
  }
  w.X = w.Y = 0;
}

// leaf bits for an odd length: the free middle takes the only values that make the cell exact,
// dx and dy of the middle class (each +-1)
__device__ __forceinline__ void middle_bits(const Walk &w, int half, int cm, uint64_t &lx, uint64_t &ly) {
  const int dx = (fld(w.s1, cm) - fld(w.s0, cm)) / 2, dy = (fld(w.s3, cm) - fld(w.s2, cm)) / 2;
  if (dx > 0) lx |= 1ULL << half;
  if (dy > 0) ly |= 1ULL << half;
}

// The order key of a leaf: its branch index at every depth, depth 0 most significant (the
// reference's DFS visits leaves in exactly this lexicographic order). The digit words hold
// depth t at bits 4t..4t+3, so the key is each word with its 16 nibbles reversed.
__device__ __forceinline__ uint64_t nibble_reverse(uint64_t x) {
  x = ((x & 0x0F0F0F0F0F0F0F0FULL) << 4) | ((x >> 4) & 0x0F0F0F0F0F0F0F0FULL);
  const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
  return ((uint64_t)__byte_perm(lo, 0, 0x0123) << 32) | (uint64_t)__byte_perm(hi, 0, 0x0123);
}

// CD_PRUNE bit 2 for a child whose slack words are a0..a3 (it passed the capacity test, so
// every used byte is in [64, 86]): dx = ((rem + dx) - (rem - dx)) / 2, likewise dy; each of
// the three mirror blocks must be reachable with the q3 quads it has left.
__host__ __device__ __forceinline__ bool reach_ok(uint64_t a0, uint64_t a1, uint64_t a2, uint64_t a3,
                                         uint32_t blk, uint32_t q3) {
#pragma unroll
  for (int b = 0; b < 3; b++) {
    const int r = (blk >> (8 * b)) & 15, s = (blk >> (8 * b + 4)) & 15;
    const int q = (q3 >> (8 * b)) & 255;
    const int D0 = (fld(a1, r) - fld(a0, r)) >> 1, D1 = (fld(a3, r) - fld(a2, r)) >> 1;
    const int D2 = (fld(a1, s) - fld(a0, s)) >> 1, D3 = (fld(a3, s) - fld(a2, s)) >> 1;
    const int t0 = D0 + D1 + D2 + D3, t1 = D0 - D1 + D2 - D3, t2 = D0 + D1 - D2 - D3,
              t3 = D0 - D1 - D2 + D3;
    if ((t0 | t1 | t2 | t3) & 3) return false;
    const int l1 = (abs(t0) + abs(t1) + abs(t2) + abs(t3)) >> 2;
    if (l1 > q || ((q - l1) & 1)) return false;
  }
  return true;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// MINB: the blocks of 256 threads the register budget is set for (4: 64 registers, no spill;
// 5: 48 registers, 6: 40 registers, both with a few spills). The launch sizes the grid to the
// blocks that are resident at once, so saved walks never wait for a block to be scheduled.
//
// Eight lanes walk one subtree together: lane j of a group tests child j of the group's
// current node, so a node's eight children take one step instead of eight, and the lanes of
// a group never diverge. A step then descends into the first feasible untried child (the
// children before it count as nodes, as the reference counts them when it tries them), or,
// when none is left, returns to the parent; at the leaf level all feasible children are
// written at once. A warp holds four walks; warp-wide collectives run every step in every
// lane, walks that have ended idle until the whole warp has. REACH adds CD_PRUNE bit 2 to
// every child's test (a child that fails it is still a node, as in the reference).
template <int MINB, bool REACH>
__global__ void __launch_bounds__(256, MINB) cd_dfs_kernel(CdParams P) {
  __shared__ QuadFx fx[32][16];
  __shared__ uint64_t posm[32];
  __shared__ uint32_t rq[32];
  for (int t = threadIdx.x; t < 32 * 16; t += blockDim.x)
    fx[t >> 4][t & 15] = ((const QuadFx *)P.fx)[t];
  if (threadIdx.x < 32) posm[threadIdx.x] = P.posmask[threadIdx.x];
  if (REACH && threadIdx.x < 32) rq[threadIdx.x] = P.reach_q[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int j = lane & 7;               // the child this lane tests
  const int g = lane >> 3;              // the walk of this lane within the warp
  const unsigned gmask = 0xFFu << (8 * g);
  const int leader = 8 * g;             // lane 0 of the group
  const int L = P.L, m = P.m, half = P.half;
  const uint64_t M = P.feas_mask;
  const int cm = half % m;
  const unsigned long long t_start = globaltimer();
  bool have = false, done = false;
  uint32_t cell = 0;
  int D = 0, d = 0, kk = 0;
  uint64_t dig0 = 0, dig1 = 0;
  Walk w;
  unsigned long long nodes = 0, leaves = 0;  // kept by the group's lane 0
  uint32_t owed = 0;  // leaf children (bit k = child k) of the node at depth d not yet written
  const int gid = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 3);
  int saved_slot = gid;
  unsigned iter = 0;

  while (true) {
    // ---- acquire work (group-uniform): this group's saved walk first, then prefixes ----
    if (!have && !done) {
      if (saved_slot < P.nsaved_in) {
        const Saved sv = P.saved_in[saved_slot];
        saved_slot = P.nsaved_in;  // at most one saved walk per group
        cell = sv.cell;
        D = sv.D;
        d = sv.d;
        kk = sv.kk;
        owed = sv.owed;
        dig0 = sv.dig0;
        dig1 = sv.dig1;
        have = true;
      } else {
        unsigned long long p = ~0ULL;
        if (j == 0 && !*(volatile int *)P.stop_flag) p = atomicAdd(P.next_prefix, 1ULL);
        p = __shfl_sync(gmask, p, leader);
        if (p >= (unsigned long long)P.nprefix) {
          done = true;
        } else {
          const Prefix pf = P.prefixes[p];
          cell = pf.cell;
          D = (int)pf.depth;
          d = D;
          kk = 0;
          owed = 0;
          dig0 = pf.dig0;
          dig1 = pf.dig1;
          have = true;
        }
      }
      if (have) {
        init_walk(w, P.cells[cell], L, m);
        for (int t = 0; t < d; t++) place(w, fx[t][getdig(dig0, dig1, t)]);
      }
    }
    if (__all_sync(FULL_MASK, done)) break;

    // ---- test the children (one per lane) ----
    const bool leaf_level = have && d + 1 == half;
    bool ok = false;
    if (have && owed == 0 && j >= kk) {
      const QuadFx &f = fx[d][j];
      const uint64_t a0 = w.s0 + (uint64_t)f.ds[0], a1 = w.s1 + (uint64_t)f.ds[1];
      const uint64_t a2 = w.s2 + (uint64_t)f.ds[2], a3 = w.s3 + (uint64_t)f.ds[3];
      ok = ((a0 & a1 & a2 & a3) & M) == M;
      if (REACH && ok) ok = reach_ok(a0, a1, a2, a3, P.reach_blk, rq[d + 1]);
    }
    const unsigned gm = (__ballot_sync(FULL_MASK, ok) >> (8 * g)) & 0xFFu;

    // ---- leaves: a leaf-level node's feasible children, or leaves owed from before ----
    bool emit = false;
    if (have) {
      if (owed) emit = (owed >> j) & 1u;
      else if (leaf_level) emit = ok;
    }
    const unsigned eb = __ballot_sync(FULL_MASK, emit);
    bool written = false;
    if (eb) {
      unsigned long long base = 0;
      const int first = __ffs(eb) - 1;
      if (lane == first) base = atomicAdd(P.leaf_count, (unsigned long long)__popc(eb));
      base = __shfl_sync(FULL_MASK, base, first);
      if (emit) {
        const unsigned long long slot = base + __popc(eb & ((1u << lane) - 1u));
        if (slot < P.leaf_cap) {
          const QuadFx &f = fx[d][j];
          uint64_t lx = w.X | f.bx, ly = w.Y | f.by;
          if (L & 1) {
            Walk t;
            t.s0 = w.s0 + (uint64_t)f.ds[0];
            t.s1 = w.s1 + (uint64_t)f.ds[1];
            t.s2 = w.s2 + (uint64_t)f.ds[2];
            t.s3 = w.s3 + (uint64_t)f.ds[3];
            middle_bits(t, half, cm, lx, ly);
          }
          uint64_t p0 = dig0, p1 = dig1;
          setdig(p0, p1, d, j);
          P.leaf_words[2 * slot] = lx;
          P.leaf_words[2 * slot + 1] = ly;
          P.leaf_keys[2 * slot] = nibble_reverse(p0);
          P.leaf_keys[2 * slot + 1] = nibble_reverse(p1);
          P.leaf_cell[slot] = cell;
          written = true;
        } else {
          atomicExch(P.stop_flag, 1);  // buffer full: the rest stays owed, the walk suspends
        }
      }
    }
    // which of the group's leaves were written and which are still owed (no leaf in the
    // warp: nothing to ask, the common case above the leaf level)
    unsigned gw = 0, gunw = 0;
    if (eb) {
      gw = (__ballot_sync(FULL_MASK, written) >> (8 * g)) & 0xFFu;
      gunw = (__ballot_sync(FULL_MASK, emit && !written) >> (8 * g)) & 0xFFu;
    }

    // ---- move the walk (group-uniform) ----
    bool finished = false;
    if (have) {
      if (j == 0) leaves += __popc(gw);
      if (owed || leaf_level) {
        if (!owed && j == 0) nodes += 8 - kk;  // every child of a leaf-level node is a node
        owed = gunw;
        kk = 8;
      } else if (gm) {
        const int c = __ffs(gm) - 1;  // the first feasible untried child
        if (j == 0) nodes += c - kk + 1;
        setdig(dig0, dig1, d, c);
        place(w, fx[d][c]);
        d++;
        kk = 0;
      } else {
        if (j == 0) nodes += 8 - kk;
        kk = 8;
      }
      if (kk == 8 && owed == 0) {  // the node is done: back to its parent
        if (d == D) {
          finished = true;
        } else {
          d--;
          const int c = getdig(dig0, dig1, d);
          unplace(w, fx[d][c], posm[d]);
          kk = c + 1;
        }
      }
    }

    // ---- suspend with leaves still owed, or at a clean point once asked to stop ----
    iter++;
    bool suspend = have && !finished && owed != 0;
    if (have && !finished && !suspend && (iter & 255) == 0) {
      int st = 0;
      if (j == 0) {
        if (*(volatile int *)P.stop_flag) st = 1;
        else if (P.round_ns && globaltimer() - t_start > P.round_ns) { atomicExch(P.stop_flag, 1); st = 1; }
      }
      suspend = __shfl_sync(gmask, st, leader) != 0;
    }
    if (suspend && j == 0) {
      const unsigned k = atomicAdd(P.nsaved_out, 1u);
      if ((int)k < P.saved_cap) {
        Saved sv;
        sv.cell = cell;
        sv.D = (uint16_t)D;
        sv.d = (uint16_t)d;
        sv.kk = (uint16_t)kk;
        sv.owed = (uint16_t)owed;
        sv.pad = 0;
        sv.dig0 = dig0;
        sv.dig1 = dig1;
        P.saved_out[k] = sv;
      } else {
        atomicCAS(P.status, 0, BS_ERR_INTERNAL);
      }
    }
    if (finished || suspend) {
      if (j == 0) {
        if (nodes) atomicAdd(P.cell_nodes + cell, nodes);
        if (leaves) atomicAdd(P.cell_leaves + cell, leaves);
      }
      nodes = 0;
      leaves = 0;
      have = false;
      owed = 0;
      if (suspend) done = true;
    }
  }
}

// Compact the leaves that passed the Hall filter (with their keys and cells), count passes
// per cell.
__global__ void compact_kernel(const uint64_t *__restrict__ words, const uint64_t *__restrict__ keys,
                               const uint32_t *__restrict__ lcell, const uint8_t *__restrict__ pass,
                               long long count, uint64_t *out_words, uint64_t *out_keys,
                               uint32_t *out_cell, unsigned long long *out_count,
                               unsigned long long out_cap, unsigned long long *cell_ok) {
  const int lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < count;
       base += (long long)gridDim.x * blockDim.x) {
    long long i = base + threadIdx.x;
    bool p = i < count && pass[i];
    unsigned ball = __ballot_sync(FULL_MASK, p);
    if (!ball) continue;
    int leader = __ffs(ball) - 1;
    unsigned long long o = 0;
    if (lane == leader) o = atomicAdd(out_count, (unsigned long long)__popc(ball));
    o = __shfl_sync(FULL_MASK, o, leader);
    if (p) {
      unsigned long long slot = o + __popc(ball & ((1u << lane) - 1u));
      const uint32_t c = lcell[i];
      if (slot < out_cap) {
        out_words[2 * slot] = words[2 * i];
        out_words[2 * slot + 1] = words[2 * i + 1];
        out_keys[2 * slot] = keys[2 * i];
        out_keys[2 * slot + 1] = keys[2 * i + 1];
        out_cell[slot] = c;
      }
      atomicAdd(cell_ok + c, 1ULL);
    }
  }
}

// ------------------------------------------------------------------------------------
// Host: frontier of each cell in the reference's order
// ------------------------------------------------------------------------------------
struct HostQuads {
  int all[16][4], pos[8][4], neg[8][4];
  HostQuads() {
    int np = 0, nn = 0;
    for (int i = 0; i < 16; i++) {
      int v[4] = {(i & 8) ? 1 : -1, (i & 4) ? 1 : -1, (i & 2) ? 1 : -1, (i & 1) ? 1 : -1};
      memcpy(all[i], v, sizeof v);
      if (v[0] * v[1] * v[2] * v[3] == 1) memcpy(pos[np++], v, sizeof v);
      else memcpy(neg[nn++], v, sizeof v);
    }
  }
};

// The optional C,D prunes (WZ_FH_CD_PRUNE, wz_match.cpp:655-711, 719-731; C,D side, m = 6,
// even L only). Both cut only subtrees without a class-exact leaf, so the stream is the same
// and only the node count falls.
//   bit 1: the root quad's entry sum must equal sum(tx) + sum(ty) mod 4 (every later quad is
//          positive-product, entry sum 0 mod 4).
//   bit 2: from depth 1, for each mirror block {r, s = (L-1-r) mod 6} with q quads left, the
//          residual Delta = (dx_r, dy_r, dx_s, dy_s) is reachable by q positive-product quads
//          (the +-columns of a 4x4 Hadamard H) iff t = H^T Delta / 4 is integral, |t|_1 <= q
//          and q - |t|_1 is even.
struct CdPrune {
  bool root = false, reach = false;
  int root_mod = 0;
  int blk_r[3] = {0, 0, 0}, blk_s[3] = {0, 0, 0};
  int qrem[33][3] = {};  // quads left per block at depths d..half-1

  void setup(int mode, bool ab_side, int L, int m, const int8_t *tx, const int8_t *ty) {
    const bool okk = !ab_side && m == 6 && L % 2 == 0;
    root = okk && (mode & 1);
    reach = okk && (mode & 2);
    if (!okk || !mode) return;
    int nb = 0, blk_of[6] = {0, 0, 0, 0, 0, 0};
    for (int r = 0; r < 6; r++) {
      const int s = (L - 1 - r) % 6;
      if (r < s) { blk_r[nb] = r; blk_s[nb] = s; blk_of[r] = blk_of[s] = nb; nb++; }
    }
    const int half = L / 2;
    for (int b = 0; b < 3; b++) qrem[half][b] = 0;
    for (int d = half - 1; d >= 0; d--) {
      for (int b = 0; b < 3; b++) qrem[d][b] = qrem[d + 1][b];
      qrem[d][blk_of[d % 6]]++;
    }
    int tot = 0;
    for (int c = 0; c < 6; c++) tot += tx[c] + ty[c];
    root_mod = (tot % 4 + 4) % 4;
  }
  // bit 2's test at a node of depth d >= 1 with residuals dx[c] = tx - px, dy[c] = ty - py
  bool reachable(int d, const int *dx, const int *dy) const {
    for (int b = 0; b < 3; b++) {
      const int r = blk_r[b], s = blk_s[b], q = qrem[d][b];
      const int D0 = dx[r], D1 = dy[r], D2 = dx[s], D3 = dy[s];
      const int t0 = D0 + D1 + D2 + D3, t1 = D0 - D1 + D2 - D3, t2 = D0 + D1 - D2 - D3,
                t3 = D0 - D1 - D2 + D3;
      if ((t0 | t1 | t2 | t3) & 3) return false;
      const int l1 = (abs(t0) + abs(t1) + abs(t2) + abs(t3)) / 4;
      if (l1 > q || ((q - l1) & 1)) return false;
    }
    return true;
  }
  // the per-launch form for the device: blocks as 4-bit class pairs, qrem as bytes
  uint32_t blk_packed() const {
    uint32_t v = 0;
    for (int b = 0; b < 3; b++) v |= (uint32_t)blk_r[b] << (8 * b) | (uint32_t)blk_s[b] << (8 * b + 4);
    return v;
  }
  uint32_t qrem_packed(int d) const {
    return (uint32_t)qrem[d][0] | (uint32_t)qrem[d][1] << 8 | (uint32_t)qrem[d][2] << 16;
  }
};

struct Frontier {
  int L, m, half, D, rev, root, pinX, pinY, ns0;
  int tot[8], px[8], py[8], placed[8];
  const int8_t *tx, *ty;
  const HostQuads *Q;
  const CdPrune *prune;
  uint32_t cell;
  long long nodes;
  std::vector<Prefix> *out;

  bool check() const {
    for (int c = 0; c < m; c++) {
      int rem = tot[c] - placed[c];
      int dx = tx[c] - px[c], dy = ty[c] - py[c];
      if (dx < -rem || dx > rem || dy < -rem || dy > rem) return false;
      if (((dx + rem) & 1) != 0 || ((dy + rem) & 1) != 0) return false;
    }
    return true;
  }
  // the whole test a node of depth d passes before its children are tried
  bool node_ok(int d) const {
    if (!check()) return false;
    if (prune->reach && d >= 1) {
      int dx[8], dy[8];
      for (int c = 0; c < m; c++) { dx[c] = tx[c] - px[c]; dy[c] = ty[c] - py[c]; }
      if (!prune->reachable(d, dx, dy)) return false;
    }
    return true;
  }

  void rec(int d, uint64_t digits) {
    nodes++;
    if (!node_ok(d)) return;
    if (d == D) {
      out->push_back(Prefix{cell, (uint32_t)D, digits, 0});
      return;
    }
    const int i1 = d, i2 = L - 1 - d, c1 = i1 % m, c2 = i2 % m;
    const int(*S)[4] = (d == 0) ? (root == 2 ? Q->neg : (root == 1 ? Q->pos : Q->all)) : Q->pos;
    const int ns = (d == 0) ? ns0 : 8;
    for (int kk = 0; kk < ns; kk++) {
      int k = rev ? ns - 1 - kk : kk;
      if (d == 0 && pinX && S[k][0] != 1) continue;
      if (d == 0 && pinY && S[k][1] != 1) continue;
      if (d == 0 && prune->root &&
          (((S[k][0] + S[k][1] + S[k][2] + S[k][3]) % 4 + 4) % 4) != prune->root_mod)
        continue;
      px[c1] += S[k][0]; py[c1] += S[k][1]; px[c2] += S[k][2]; py[c2] += S[k][3];
      placed[c1]++; placed[c2]++;
      rec(d + 1, digits | ((uint64_t)kk << (4 * d)));
      px[c1] -= S[k][0]; py[c1] -= S[k][1]; px[c2] -= S[k][2]; py[c2] -= S[k][3];
      placed[c1]--; placed[c2]--;
    }
  }
};

}  // namespace

// ------------------------------------------------------------------------------------
// Entry point
// ------------------------------------------------------------------------------------
#define CK(x)                                       \
  do {                                              \
    cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return bs_cuda_fail(e_); \
  } while (0)

struct StreamBufs {
  CellDev *cells = nullptr; long long cells_cap = 0;
  Prefix *prefixes = nullptr; long long prefix_cap = 0;
  Saved *saved[2] = {nullptr, nullptr}; long long saved_cap = 0;
  uint64_t *leaf_words = nullptr, *leaf_keys = nullptr; long long leaf_cap = 0;
  uint32_t *leaf_cell = nullptr;
  uint8_t *leaf_pass = nullptr; long long pass_cap = 0;
  uint64_t *surv_words = nullptr, *surv_keys = nullptr; long long surv_cap = 0;
  uint32_t *surv_cell = nullptr;
  unsigned long long *counters = nullptr;  // see below
  unsigned long long *cell_stats = nullptr; long long cell_stats_cap = 0;
  unsigned *nsaved = nullptr;
  int *stop = nullptr;
  QuadFx *fx = nullptr;      // [32][16] branch effects
  uint64_t *posm = nullptr;  // [32] position masks
  uint32_t *reach_q = nullptr;  // [32] CD_PRUNE bit 2: quads left per mirror block and depth
};

static StreamBufs *bufs_of(bs_ctx *ctx) {
  if (!ctx->stream_bufs) ctx->stream_bufs = new StreamBufs();
  return (StreamBufs *)ctx->stream_bufs;
}

void bs_stream_free(bs_ctx *ctx) {
  StreamBufs *b = (StreamBufs *)ctx->stream_bufs;
  if (!b) return;
  cudaFree(b->cells); cudaFree(b->prefixes); cudaFree(b->saved[0]); cudaFree(b->saved[1]);
  cudaFree(b->leaf_words); cudaFree(b->leaf_keys); cudaFree(b->leaf_cell); cudaFree(b->leaf_pass);
  cudaFree(b->surv_words); cudaFree(b->surv_keys); cudaFree(b->surv_cell); cudaFree(b->counters);
  cudaFree(b->cell_stats); cudaFree(b->nsaved); cudaFree(b->stop); cudaFree(b->fx);
  cudaFree(b->posm); cudaFree(b->reach_q);
  delete b;
  ctx->stream_bufs = nullptr;
}

// Grows a leaf or survivor store (words and keys: 2 words each; cells) to at least `want`.
static int ensure_store(uint64_t **words, uint64_t **keys, uint32_t **cellv, long long *cap,
                        long long want) {
  if (*cap >= want && *words) return BS_OK;
  cudaFree(*words); cudaFree(*keys); cudaFree(*cellv);
  *words = nullptr; *keys = nullptr; *cellv = nullptr; *cap = 0;
  cudaError_t e = cudaMalloc(words, sizeof(uint64_t) * 2 * want);
  if (e == cudaSuccess) e = cudaMalloc(keys, sizeof(uint64_t) * 2 * want);
  if (e == cudaSuccess) e = cudaMalloc(cellv, sizeof(uint32_t) * want);
  if (e != cudaSuccess) return bs_cuda_fail(e);
  *cap = want;
  return BS_OK;
}

// Stream order of a wave's survivors: by (cell, path key hi, path key lo), as a stable LSD
// radix sort over the bytes that vary (a leaf's path occupies only the top 4 x half bits, so
// most bytes of the low key word, and of the cell index, are skipped).
static void stream_order(const std::vector<uint64_t> &keys, const std::vector<uint32_t> &cellv, size_t n,
                         std::vector<uint32_t> &order) {
  order.resize(n);
  for (size_t i = 0; i < n; i++) order[i] = (uint32_t)i;
  std::vector<uint32_t> tmp(n);
  size_t cnt[256];
  auto pass = [&](auto byte_of) {
    memset(cnt, 0, sizeof cnt);
    for (size_t i = 0; i < n; i++) cnt[byte_of(order[i])]++;
    for (int b = 0; b < 256; b++)
      if (cnt[b] == n) return;  // one value: this byte orders nothing
    size_t run = 0;
    for (int b = 0; b < 256; b++) {
      const size_t c = cnt[b];
      cnt[b] = run;
      run += c;
    }
    for (size_t i = 0; i < n; i++) tmp[cnt[byte_of(order[i])]++] = order[i];
    order.swap(tmp);
  };
  for (int b = 0; b < 8; b++) pass([&](uint32_t i) { return (unsigned)((keys[2 * i + 1] >> (8 * b)) & 255); });
  for (int b = 0; b < 8; b++) pass([&](uint32_t i) { return (unsigned)((keys[2 * i] >> (8 * b)) & 255); });
  for (int b = 0; b < 4; b++) pass([&](uint32_t i) { return (unsigned)((cellv[i] >> (8 * b)) & 255); });
}

extern "C" int bs_cd_stream(bs_ctx *ctx, const bs_cell *cells, int ncells, const bs_stream_opts *opt,
                            uint64_t *out_words, uint32_t *out_cell, long long out_cap,
                            long long *nout, bs_cell_stats *stats) {
  if (!ctx || !cells || ncells <= 0 || !opt || !nout) return BS_ERR_ARG;
  if (out_cap > 0 && !out_words) return BS_ERR_ARG;
  // the C,D side has length n; the A,B side (ab_side, the reference's abSide) length n+1 with
  // negative-product root quads (wz_match.cpp:766-768)
  const int L = opt->ab_side ? ctx->n1 : ctx->n, m = opt->m;
  const int root_kind = opt->ab_side ? 2 : (opt->endpos ? 1 : 0);
  if (m != 3 && m != 6) return BS_ERR_ARG;
  if (L > 64 || L / 2 > 31) return BS_ERR_ARG;
  int hall_mode = opt->hall_mode;
  if (hall_mode < BS_HALL_FP64 || hall_mode > BS_HALL_TC_BF16X2) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  StreamBufs *B = bufs_of(ctx);
  const int half = L / 2;

  // ---- coarse frontier of each cell on the host, in the reference's order ----
  // The first split stops at depth 16 (one digit word); later splits go deeper.
  static const HostQuads Q;
  const int max_depth = std::min(half - 1, 16);
  std::vector<Frontier> F(ncells);
  std::vector<CdPrune> prune(ncells);  // CD_PRUNE: the root rule depends on the cell
  std::vector<Prefix> coarse;
  std::vector<long long> host_nodes(ncells, 0);
  long long target = opt->target_prefixes > 0 ? opt->target_prefixes : 262144;
  long long per_cell_target = std::max<long long>(64, target / ncells);
  int deepest = 1;
  for (int ci = 0; ci < ncells; ci++) {
    const bs_cell &c = cells[ci];
    Frontier &f = F[ci];
    f.L = L; f.m = m; f.half = half; f.rev = opt->rev; f.root = root_kind;
    f.pinX = c.pinX; f.pinY = c.pinY;
    f.ns0 = root_kind == 0 ? 16 : 8;
    for (int k = 0; k < m; k++) {
      f.tot[k] = 0;
      for (int p = k; p < L; p += m) f.tot[k]++;
    }
    f.tx = c.tx; f.ty = c.ty; f.Q = &Q; f.cell = (uint32_t)ci;
    prune[ci].setup(opt->cd_prune, opt->ab_side != 0, L, m, c.tx, c.ty);
    f.prune = &prune[ci];
    // deepen until the cell has enough prefixes or the split reaches the deepest prefix depth
    std::vector<Prefix> mine;
    int D = 1;
    for (;;) {
      mine.clear();
      memset(f.px, 0, sizeof f.px); memset(f.py, 0, sizeof f.py); memset(f.placed, 0, sizeof f.placed);
      f.D = D; f.nodes = 0; f.out = &mine;
      f.rec(0, 0);
      if ((long long)mine.size() >= per_cell_target || D >= max_depth || mine.empty()) break;
      D++;
    }
    deepest = std::max(deepest, D);
    host_nodes[ci] = f.nodes;
    coarse.insert(coarse.end(), mine.begin(), mine.end());
  }
  const long long ncoarse = (long long)coarse.size();

  // Places (sign +1) or removes (-1) branch k of depth t on a cell's host walker.
  auto apply = [&](Frontier &f, int t, int k, int sign) {
    const int(*S)[4] = (t == 0) ? (f.root == 2 ? Q.neg : (f.root == 1 ? Q.pos : Q.all)) : Q.pos;
    const int ns = (t == 0) ? f.ns0 : 8;
    const int q = f.rev ? ns - 1 - k : k;
    const int c1 = t % m, c2 = (L - 1 - t) % m;
    f.px[c1] += sign * S[q][0]; f.py[c1] += sign * S[q][1];
    f.px[c2] += sign * S[q][2]; f.py[c2] += sign * S[q][3];
    f.placed[c1] += sign; f.placed[c2] += sign;
  };
  auto digit = [](uint64_t d0, uint64_t d1, int t) {
    return (int)((((t < 16) ? d0 : d1) >> (4 * (t & 15))) & 15);
  };
  auto reset = [](Frontier &f) {
    memset(f.px, 0, sizeof f.px); memset(f.py, 0, sizeof f.py); memset(f.placed, 0, sizeof f.placed);
  };

  // The subtrees of coarse prefix p, refined by k more levels: the fine prefixes of its
  // subtree at depth p.depth + k, in stream order. Returns the host nodes it adds (the coarse
  // node itself was counted when the frontier was built).
  auto refine = [&](const Prefix &p, int k, std::vector<Prefix> &out) -> long long {
    if (k <= 0) {
      out.push_back(p);
      return 0;
    }
    Frontier &f = F[p.cell];
    reset(f);
    for (int t = 0; t < (int)p.depth; t++) apply(f, t, digit(p.dig0, p.dig1, t), +1);
    f.D = (int)p.depth + k;
    f.out = &out;
    const long long before = f.nodes;
    f.rec((int)p.depth, p.dig0);
    return f.nodes - before - 1;
  };

  // A suspended walk's remaining work as subtree roots: its node at depth d itself if none
  // of its children was tried yet, else the children kk.. of that node; then the later
  // siblings of each node on its path up to its root depth D. Each sibling is a node the
  // device would have counted on placing it; infeasible ones end there.
  auto split_walk = [&](const Saved &w, std::vector<Prefix> &out) -> long long {
    Frontier &f = F[w.cell];
    reset(f);
    for (int t = 0; t < (int)w.d; t++) apply(f, t, digit(w.dig0, w.dig1, t), +1);
    long long added = 0;
    for (int t = (int)w.d; t >= (int)w.D; t--) {
      if (t < (int)w.d) apply(f, t, digit(w.dig0, w.dig1, t), -1);
      // the path's digits above depth t
      uint64_t p0 = w.dig0, p1 = w.dig1;
      for (int u = t; u < 32; u++) {
        const int s = 4 * (u & 15);
        if (u < 16) p0 &= ~(15ULL << s);
        else p1 &= ~(15ULL << s);
      }
      int first;
      if (t == (int)w.d) {
        if (w.kk == 0) {  // untouched below (already counted): it is a subtree root as it is
          out.push_back(Prefix{w.cell, (uint32_t)t, p0, p1});
          continue;
        }
        if (t + 1 >= half) continue;  // a leaf-level node: its children were tested together
        first = (int)w.kk;
      } else {
        first = digit(w.dig0, w.dig1, t) + 1;
      }
      for (int k = first; k < 8; k++) {
        apply(f, t, k, +1);
        added++;
        if (f.node_ok(t + 1)) {
          uint64_t q0 = p0, q1 = p1;
          if (t < 16) q0 |= (uint64_t)k << (4 * t);
          else q1 |= (uint64_t)k << (4 * (t - 16));
          out.push_back(Prefix{w.cell, (uint32_t)(t + 1), q0, q1});
        }
        apply(f, t, k, -1);
      }
    }
    return added;
  };

  // ---- device buffers ----
  int rc = bs_ensure_dev((void **)&B->cells, &B->cells_cap, ncells, sizeof(CellDev));
  if (!rc) rc = bs_ensure_dev((void **)&B->cell_stats, &B->cell_stats_cap, 3LL * ncells, sizeof(unsigned long long));
  long long leaf_cap = opt->leaf_chunk > 0 ? opt->leaf_chunk : (1LL << 24);
  if (!rc) rc = ensure_store(&B->leaf_words, &B->leaf_keys, &B->leaf_cell, &B->leaf_cap, leaf_cap);
  if (!rc) rc = bs_ensure_dev((void **)&B->leaf_pass, &B->pass_cap, leaf_cap, 1);
  const int block = 256;
  // register budget variant (BS_DFS_BLOCKS=5 or 6 select the 48- and 40-register builds) and
  // the grid of exactly the blocks that fit at once
  static const int env_blocks = [] {
    const char *e = getenv("BS_DFS_BLOCKS");
    const int b = e ? atoi(e) : 4;
    return (b == 5 || b == 6) ? b : 4;
  }();
  if (opt->dfs_blocks != 0 && (opt->dfs_blocks < 4 || opt->dfs_blocks > 6)) return BS_ERR_ARG;
  const int dfs_blocks = opt->dfs_blocks ? opt->dfs_blocks : env_blocks;
  const bool reach = prune[0].reach;  // the same for every cell of the batch
  auto dfs_kernel = reach ? cd_dfs_kernel<4, true>
                          : dfs_blocks == 6 ? cd_dfs_kernel<6, false>
                                            : (dfs_blocks == 5 ? cd_dfs_kernel<5, false> : cd_dfs_kernel<4, false>);
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dfs_kernel, block, 0));
  if (per_sm < 1) per_sm = 1;
  const int grid = ctx->num_sms * per_sm;
  const int saved_cap = grid * block;
  if (!rc && B->saved_cap < saved_cap) {
    cudaFree(B->saved[0]); cudaFree(B->saved[1]);
    CK(cudaMalloc(&B->saved[0], sizeof(Saved) * saved_cap));
    CK(cudaMalloc(&B->saved[1], sizeof(Saved) * saved_cap));
    B->saved_cap = saved_cap;
  }
  if (!rc && !B->counters) {
    CK(cudaMalloc(&B->counters, sizeof(unsigned long long) * 8));
    CK(cudaMalloc(&B->nsaved, sizeof(unsigned) * 2));
    CK(cudaMalloc(&B->stop, sizeof(int)));
    CK(cudaMalloc(&B->fx, sizeof(QuadFx) * 32 * 16));
    CK(cudaMalloc(&B->posm, sizeof(uint64_t) * 32));
    CK(cudaMalloc(&B->reach_q, sizeof(uint32_t) * 32));
  }
  long long surv_cap = opt->survivor_cap > 0 ? opt->survivor_cap : (1LL << 22);
  if (!rc) rc = ensure_store(&B->surv_words, &B->surv_keys, &B->surv_cell, &B->surv_cap, surv_cap);
  if (rc) return rc;
  surv_cap = B->surv_cap;
  leaf_cap = B->leaf_cap;

  std::vector<CellDev> hc(ncells);
  for (int ci = 0; ci < ncells; ci++) {
    memset(&hc[ci], 0, sizeof(CellDev));
    for (int k = 0; k < m; k++) { hc[ci].tx[k] = cells[ci].tx[k]; hc[ci].ty[k] = cells[ci].ty[k]; }
  }
  // effect of branch kk at depth d: slack deltas of the two classes it touches and the sign
  // bits it sets; the branch -> quad map includes the reversal and the root table.
  std::vector<QuadFx> fxh(32 * 16);
  std::vector<uint64_t> posm(32, 0);
  memset(fxh.data(), 0, sizeof(QuadFx) * fxh.size());
  for (int dd = 0; dd < half && dd < 32; dd++) {
    const int i1 = dd, i2 = L - 1 - dd, c1 = i1 % m, c2 = i2 % m;
    posm[dd] = (1ULL << i1) | (1ULL << i2);
    const int(*S)[4] = (dd == 0) ? (root_kind == 2 ? Q.neg : (root_kind == 1 ? Q.pos : Q.all)) : Q.pos;
    const int ns = (dd == 0 && root_kind == 0) ? 16 : 8;
    for (int kk = 0; kk < ns; kk++) {
      const int k = opt->rev ? ns - 1 - kk : kk;
      const int a = S[k][0], b = S[k][1], c = S[k][2], e = S[k][3];
      QuadFx &f = fxh[dd * 16 + kk];
      // placing value v of C in class c: rem -= 1, dx -= v -> (rem - dx) += v - 1, (rem + dx) -= v + 1
      f.ds[0] = (int64_t)(a - 1) * (1LL << (8 * c1)) + (int64_t)(c - 1) * (1LL << (8 * c2));
      f.ds[1] = (int64_t)(-a - 1) * (1LL << (8 * c1)) + (int64_t)(-c - 1) * (1LL << (8 * c2));
      f.ds[2] = (int64_t)(b - 1) * (1LL << (8 * c1)) + (int64_t)(e - 1) * (1LL << (8 * c2));
      f.ds[3] = (int64_t)(-b - 1) * (1LL << (8 * c1)) + (int64_t)(-e - 1) * (1LL << (8 * c2));
      f.bx = (a > 0 ? 1ULL << i1 : 0) | (c > 0 ? 1ULL << i2 : 0);
      f.by = (b > 0 ? 1ULL << i1 : 0) | (e > 0 ? 1ULL << i2 : 0);
    }
  }
  uint64_t feas = 0;
  for (int c = 0; c < m; c++) feas |= 0x40ULL << (8 * c);
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(B->fx, fxh.data(), sizeof(QuadFx) * fxh.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(B->posm, posm.data(), sizeof(uint64_t) * 32, cudaMemcpyHostToDevice, s));
  std::vector<uint32_t> rqh(32, 0);
  if (reach)
    for (int dd = 1; dd <= half && dd < 32; dd++) rqh[dd] = prune[0].qrem_packed(dd);
  CK(cudaMemcpyAsync(B->reach_q, rqh.data(), sizeof(uint32_t) * 32, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(B->cells, hc.data(), sizeof(CellDev) * ncells, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(B->cell_stats, 0, sizeof(unsigned long long) * 3 * ncells, s));
  // counters: [0] next prefix of the queue, [1] leaf count of the round, [2] survivors of the wave
  unsigned long long *cell_nodes = B->cell_stats, *cell_leaves = B->cell_stats + ncells,
                     *cell_ok = B->cell_stats + 2 * ncells;

  // ---- waves: runs of coarse prefixes, in stream order, refined to fill the GPU ----
  // A leaf's key is its branch path, so survivors sort into stream order however the work
  // was divided; a wave's survivors all precede the next wave's, so each wave is ordered on
  // its own and appended. The width (coarse prefixes per wave) and the refinement depth adapt
  // to the nodes per coarse prefix seen so far: fine subtrees of ~FINE_NODES nodes, waves of
  // ~WAVE_NODES nodes, and under `limit` no wider than the survivors still owed suggest.
  // Inside a wave, a launch lasts at most ROUND_NS; when the queue is empty and fewer walks
  // than walkers remain, the suspended walks are split into their remaining subtrees, so one
  // large subtree never holds the GPU with a few walkers.
  const long long limit = opt->limit > 0 ? opt->limit : 0;
  const double FINE_NODES = opt->fine_nodes > 0 ? opt->fine_nodes : 2e4;
  const double WAVE_NODES = opt->wave_nodes > 0 ? opt->wave_nodes : 8e9, NOMINAL_RATE = 2e10;
  const unsigned long long ROUND_NS = opt->round_us > 0 ? (unsigned long long)opt->round_us * 1000ULL
                                                        : 25000000ULL;
  const long long walkers = (long long)grid * block / 8;  // eight lanes walk one subtree
  std::vector<uint64_t> res_words;
  std::vector<uint32_t> res_cell;
  std::vector<Prefix> fine, pieces;
  std::vector<Saved> walks, keep_walks;
  std::vector<uint64_t> wkeys, wwords;
  std::vector<uint32_t> wcell;
  std::vector<unsigned long long> cs_prev(3 * (size_t)ncells, 0), cs(3 * (size_t)ncells, 0);
  // the first wave is a probe: small under `limit` (a few coarse prefixes can hold far more
  // survivors than asked for; later waves then grow at most 4x at a time), wider otherwise
  long long pos = 0, wave_width = std::min<long long>(ncoarse, limit ? 8 : 256);
  int k_refine = (half - deepest >= 6) ? 2 : 0;
  long long have = 0;
  static const bool trace = getenv("BS_STREAM_TRACE") != nullptr;  // per-wave figures on stderr
  // the stop flag and the wall limit are checked between launches (each at most ROUND_NS)
  int stop_rc = 0;
  auto t_last_surv = std::chrono::steady_clock::now();
  unsigned long long wave_surv_seen = 0;
  while (pos < ncoarse && !(limit && have >= limit) && !stop_rc) {
    const long long take = std::min<long long>(std::max<long long>(1, wave_width), ncoarse - pos);
    fine.clear();
    for (long long i = pos; i < pos + take; i++) {
      const int k = std::min(k_refine, max_depth - (int)coarse[i].depth);
      host_nodes[coarse[i].cell] += refine(coarse[i], k, fine);
    }
    pos += take;
    long long nprefix = (long long)fine.size();
    if (nprefix == 0) continue;  // the refinement pruned the whole run
    rc = bs_ensure_dev((void **)&B->prefixes, &B->prefix_cap, nprefix, sizeof(Prefix));
    if (rc) return rc;
    CK(cudaMemcpyAsync(B->prefixes, fine.data(), sizeof(Prefix) * nprefix, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(B->counters, 0, sizeof(unsigned long long) * 8, s));
    const auto t_wave = std::chrono::steady_clock::now();
    int nsaved = 0, cur = 0, rounds = 0, splits = 0;
    wave_surv_seen = 0;
    for (;;) {
      CK(cudaMemsetAsync(B->nsaved, 0, sizeof(unsigned), s));
      CK(cudaMemsetAsync(B->stop, 0, sizeof(int), s));
      CK(cudaMemsetAsync(B->counters + 1, 0, sizeof(unsigned long long), s));
      CdParams P;
      P.L = L; P.m = m; P.half = half;
      P.feas_mask = feas;
      P.fx = B->fx;
      P.posmask = B->posm;
      P.cells = B->cells; P.prefixes = B->prefixes; P.nprefix = nprefix;
      P.next_prefix = B->counters;
      P.saved_in = B->saved[cur]; P.nsaved_in = nsaved;
      P.saved_out = B->saved[cur ^ 1]; P.nsaved_out = B->nsaved; P.saved_cap = saved_cap;
      P.leaf_words = B->leaf_words; P.leaf_keys = B->leaf_keys; P.leaf_cell = B->leaf_cell;
      P.leaf_count = B->counters + 1; P.leaf_cap = (unsigned long long)leaf_cap;
      P.cell_nodes = cell_nodes; P.cell_leaves = cell_leaves;
      P.stop_flag = B->stop; P.round_ns = ROUND_NS; P.status = ctx->d_status;
      P.reach_blk = prune[0].blk_packed(); P.reach_q = B->reach_q;
      bs_timed_begin(ctx);
      dfs_kernel<<<grid, block, 0, s>>>(P);
      bs_timed_end(ctx);
      CK(cudaGetLastError());
      unsigned long long leaf_count = 0, nextp = 0, wave_surv = 0;
      unsigned nsv = 0;
      CK(cudaMemcpyAsync(&leaf_count, B->counters + 1, sizeof leaf_count, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&nextp, B->counters, sizeof nextp, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&wave_surv, B->counters + 2, sizeof wave_surv, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&nsv, B->nsaved, sizeof nsv, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      rounds++;
      if ((long long)nsv > walkers) {
        // A group suspends at most once per launch, so a launch saves at most `walkers` walks
        // (saved_cap = 8 x walkers); anything more is a broken invariant, reported loudly.
        fprintf(stderr, "[bs_cd_stream] saved-walk invariant broken: nsaved=%u walkers=%lld "
                        "saved_cap=%d nsaved_in=%d round=%d splits=%d nprefix=%lld\n",
                nsv, walkers, saved_cap, nsaved, rounds, splits, nprefix);
        return BS_ERR_INTERNAL;
      }
      if (wave_surv > wave_surv_seen) {  // survivors found since the last look (wall clock)
        wave_surv_seen = wave_surv;
        t_last_surv = std::chrono::steady_clock::now();
      }
      if (*ctx->h_stop) stop_rc = BS_STOPPED;
      else if (opt->wall_sec > 0 &&
               std::chrono::duration<double>(std::chrono::steady_clock::now() - t_last_surv).count() >
                   opt->wall_sec)
        stop_rc = BS_WALLED;
      if (stop_rc) break;  // this wave is abandoned: its survivors are not a prefix
      long long nleaf = (long long)std::min<unsigned long long>(leaf_count, (unsigned long long)leaf_cap);
      if (nleaf > 0) {
        int r2 = bs_hall_dev_len(ctx, B->leaf_words, nleaf, hall_mode, B->leaf_pass, L);
        if (r2) return r2;
        ctx->launches++;
        compact_kernel<<<bs_grid_for(nleaf, 256, 8 * ctx->num_sms), 256, 0, s>>>(
            B->leaf_words, B->leaf_keys, B->leaf_cell, B->leaf_pass, nleaf, B->surv_words,
            B->surv_keys, B->surv_cell, B->counters + 2, (unsigned long long)surv_cap, cell_ok);
        CK(cudaGetLastError());
      }
      nsaved = (int)nsv;
      cur ^= 1;
      const bool queue_empty = nextp >= (unsigned long long)nprefix;
      if (nsaved == 0 && queue_empty) break;
      // few walks left and nothing queued: split the walks into their remaining subtrees
      if (queue_empty && nsaved > 0 && (long long)nsaved * 4 < walkers * 3 && leaf_count < (unsigned long long)leaf_cap) {
        walks.resize(nsaved);
        CK(cudaMemcpyAsync(walks.data(), B->saved[cur], sizeof(Saved) * nsaved, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        pieces.clear();
        keep_walks.clear();
        for (const Saved &w : walks) {
          if (w.owed) keep_walks.push_back(w);  // leaves still to write: resume as is
          else host_nodes[w.cell] += split_walk(w, pieces);
        }
        nprefix = (long long)pieces.size();
        if (nprefix >= (1LL << 40)) return BS_ERR_CAP;
        if (nprefix > 0) {
          rc = bs_ensure_dev((void **)&B->prefixes, &B->prefix_cap, nprefix, sizeof(Prefix));
          if (rc) return rc;
          CK(cudaMemcpyAsync(B->prefixes, pieces.data(), sizeof(Prefix) * nprefix, cudaMemcpyHostToDevice, s));
        }
        nsaved = (int)keep_walks.size();
        if (nsaved > 0)
          CK(cudaMemcpyAsync(B->saved[cur], keep_walks.data(), sizeof(Saved) * nsaved, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(B->counters, 0, sizeof(unsigned long long), s));
        splits++;
        if (nsaved == 0 && nprefix == 0) break;
      }
    }

    if (stop_rc) break;
    // ---- the wave's survivors, in stream order ----
    unsigned long long nsurv = 0;
    int status = 0;
    CK(cudaMemcpyAsync(&nsurv, B->counters + 2, sizeof nsurv, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof status, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cs.data(), B->cell_stats, sizeof(unsigned long long) * 3 * ncells, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (status) {
      cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s);
      return status;
    }
    if ((long long)nsurv > surv_cap) {
      // one wave found more survivors than the device buffer holds: report the size to retry
      // with (as survivor_cap; the output needs at least as much)
      *nout = have + (long long)nsurv;
      return BS_ERR_CAP;
    }
    if (nsurv > 0) {
      wkeys.resize(2 * nsurv);
      wwords.resize(2 * nsurv);
      wcell.resize(nsurv);
      CK(cudaMemcpyAsync(wkeys.data(), B->surv_keys, sizeof(uint64_t) * 2 * nsurv, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(wwords.data(), B->surv_words, sizeof(uint64_t) * 2 * nsurv, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(wcell.data(), B->surv_cell, sizeof(uint32_t) * nsurv, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      std::vector<uint32_t> order;
      stream_order(wkeys, wcell, (size_t)nsurv, order);
      long long keep = (long long)nsurv;
      if (limit) keep = std::min(keep, limit - have);
      for (long long i = 0; i < keep; i++) {
        res_words.push_back(wwords[2 * order[i]]);
        res_words.push_back(wwords[2 * order[i] + 1]);
        res_cell.push_back(wcell[order[i]]);
      }
      have += keep;
      t_last_surv = std::chrono::steady_clock::now();
    }

    // ---- size the next wave from what this one cost ----
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_wave).count();
    unsigned long long wave_nodes = 0;
    for (int ci = 0; ci < ncells; ci++) wave_nodes += cs[ci] - cs_prev[ci];
    cs_prev = cs;
    const double per_coarse = std::max(1.0, (double)wave_nodes / (double)take);
    const double rate = std::max(NOMINAL_RATE, secs > 0 ? (double)wave_nodes / secs : 0.0);
    k_refine = 0;
    while (k_refine < 16 && per_coarse / std::pow(8.0, k_refine) > FINE_NODES) k_refine++;
    double width = std::max(WAVE_NODES, rate * 0.25) / per_coarse;
    // enough fine prefixes for every walker, twice over
    width = std::max(width, 2.0 * (double)walkers / std::pow(8.0, k_refine));
    if (limit) width = std::min(width, 4.0 * (double)take);  // approach the limit gradually
    if (limit && nsurv > 0) {
      const double per_coarse_surv = (double)nsurv / (double)take;
      width = std::min(width, std::max(8.0, 1.5 * (double)(limit - have) / per_coarse_surv));
    }
    wave_width = (long long)std::min<double>(width, (double)(1LL << 40));
    if (trace)
      fprintf(stderr, "[bs_cd_stream] wave coarse=%lld fine=%lld rounds=%d splits=%d nodes=%llu "
                      "surv=%llu have=%lld secs=%.4f next_width=%lld next_k=%d pos=%lld/%lld\n",
              take, (long long)fine.size(), rounds, splits, wave_nodes, nsurv, have, secs, wave_width,
              k_refine, pos, ncoarse);
  }

  // ---- results ----
  if (stop_rc) {  // the counts of the part explored, the abandoned wave included
    int status = 0;
    CK(cudaMemcpyAsync(cs_prev.data(), B->cell_stats, sizeof(unsigned long long) * 3 * ncells,
                       cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&status, ctx->d_status, sizeof status, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (status) {
      cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s);
      return status;
    }
  }
  if (stats)
    for (int ci = 0; ci < ncells; ci++) {
      stats[ci].nodes = host_nodes[ci] + (long long)cs_prev[ci];
      stats[ci].leaves = (long long)cs_prev[ncells + ci];
      stats[ci].ok = (long long)cs_prev[2 * ncells + ci];
    }
  *nout = have;
  if (have > out_cap) return BS_ERR_CAP;
  if (have > 0) {
    memcpy(out_words, res_words.data(), sizeof(uint64_t) * 2 * have);
    if (out_cell) memcpy(out_cell, res_cell.data(), sizeof(uint32_t) * have);
  }
  return stop_rc ? stop_rc : BS_OK;
}
