// cd_stream.cu - the C,D mirror-quad stream (the reference's count_pairs22,
// src/solver/wz_match.cpp:678-784) for a batch of cells, on the GPU.
//
// Structure:
//   1. Host: each cell's DFS tree is expanded to a split depth D in the reference's branch
//      order (quad index order, reversed under STREAM_REV), giving prefixes in DFS order.
//      Nodes above D are counted here exactly as the reference counts rec() calls.
//   2. Device, cd_dfs_kernel: persistent threads take prefixes from a queue and walk the
//      subtree below each one iteratively, one tree step per loop iteration (so a warp's lanes
//      stay busy on different subtrees). A class-exact leaf is appended to the leaf buffer with
//      key (prefix index << 32 | leaf sequence inside the prefix). When the buffer is full a
//      thread saves its position and stops; the next launch resumes it.
//   3. Device: the Hall filter (tensor-core form by default) decides every leaf; survivors are
//      compacted with their keys; sorting by key restores the reference's stream order.
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

struct Prefix {
  uint32_t cell;
  uint32_t depth;   // D: quads placed at depths 0..D-1
  uint64_t digits;  // 4 bits per depth: the loop index kk chosen at that depth
};

// A suspended subtree walk: the node at depth d with its next child index kk.
struct Saved {
  uint32_t prefix;
  uint32_t seq;        // leaves emitted so far inside this prefix
  uint16_t d, kk;
  uint16_t owed;       // leaf children of node d (bit k = child k) not yet written
  uint16_t pad;
  uint64_t dig[2];     // digits of depths 0..d-1 (4 bits each, depths 0-15 and 16-31)
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
  uint64_t *leaf_words;  // [cap][2]
  uint64_t *leaf_keys;   // [cap]
  unsigned long long *leaf_count;
  unsigned long long leaf_cap;
  unsigned long long *cell_nodes, *cell_leaves;
  int *full_flag;
  int *status;
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

__device__ __forceinline__ int fld(uint64_t w, int c) { return (int)((w >> (8 * c)) & 255) - 64; }

__device__ __forceinline__ void place(Walk &w, const QuadFx &f) {
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
__device__ __forceinline__ bool feasible(const Walk &w, uint64_t M) {
  return ((w.s0 & w.s1 & w.s2 & w.s3) & M) == M;
}

__device__ __forceinline__ void init_walk(Walk &w, const CellDev &cell, int L, int m) {
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

// MINB: the blocks of 256 threads the register budget is set for (4: 64 registers, no spill;
// 6: 40 registers with a few spills on the rare paths). The launch sizes the grid to the
// blocks that are resident at once, so saved walks never wait for a block to be scheduled.
template <int MINB>
__global__ void __launch_bounds__(256, MINB) cd_dfs_kernel(CdParams P) {
  __shared__ QuadFx fx[32][16];
  __shared__ uint64_t posm[32];
  for (int t = threadIdx.x; t < 32 * 16; t += blockDim.x)
    fx[t >> 4][t & 15] = ((const QuadFx *)P.fx)[t];
  if (threadIdx.x < 32) posm[threadIdx.x] = P.posmask[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int L = P.L, m = P.m, half = P.half;
  const uint64_t M = P.feas_mask;
  const int cm = half % m;
  bool have = false;
  uint32_t prefix = 0, cell = 0, seq = 0;
  int D = 0, d = 0, kk = 0;
  uint64_t dig0 = 0, dig1 = 0;
  Walk w;
  unsigned long long nodes = 0, leaves = 0;
  uint32_t owed = 0;  // leaf children (bit k = child k) of the node at depth d not yet written
  int saved_slot = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  unsigned iter = 0;

  while (true) {
    // ---- acquire work: this thread's saved walk first, then fresh prefixes ----
    if (!have) {
      if (saved_slot < P.nsaved_in) {
        const Saved sv = P.saved_in[saved_slot];
        saved_slot = P.nsaved_in;  // at most one saved walk per thread
        prefix = sv.prefix;
        const Prefix pf = P.prefixes[prefix];
        cell = pf.cell;
        D = (int)pf.depth;
        d = sv.d;
        kk = sv.kk;
        seq = sv.seq;
        dig0 = sv.dig[0];
        dig1 = sv.dig[1];
        owed = sv.owed;
      } else {
        if (*(volatile int *)P.full_flag) break;
        unsigned long long p = atomicAdd(P.next_prefix, 1ULL);
        if (p >= (unsigned long long)P.nprefix) break;
        prefix = (uint32_t)p;
        const Prefix pf = P.prefixes[p];
        cell = pf.cell;
        D = (int)pf.depth;
        d = D;
        kk = 0;
        seq = 0;
        dig0 = pf.digits;
        dig1 = 0;
        owed = 0;
      }
      init_walk(w, P.cells[cell], L, m);
      for (int t = 0; t < d; t++) place(w, fx[t][getdig(dig0, dig1, t)]);
      have = true;
    }

    // ---- one tree step ----
    bool finished = false;
    if (owed == 0) {
      if (kk == 8) {
        if (d == D) {
          finished = true;
        } else {
          d--;
          kk = getdig(dig0, dig1, d);
          unplace(w, fx[d][kk], posm[d]);
          kk++;
        }
      } else if (d + 1 == half) {
        // the children are leaves: test the remaining ones together (each is one node, as
        // the reference counts them), then write the class-exact ones below
        uint32_t lm = 0;
        for (int k = kk; k < 8; k++) {
          const QuadFx &f = fx[d][k];
          const uint64_t a0 = w.s0 + (uint64_t)f.ds[0], a1 = w.s1 + (uint64_t)f.ds[1];
          const uint64_t a2 = w.s2 + (uint64_t)f.ds[2], a3 = w.s3 + (uint64_t)f.ds[3];
          if (((a0 & a1 & a2 & a3) & M) == M) lm |= 1u << k;
        }
        nodes += 8 - kk;
        owed = lm;
        kk = 8;
      } else {
        const QuadFx &f = fx[d][kk];
        place(w, f);
        nodes++;
        if (!feasible(w, M)) {
          unplace(w, f, posm[d]);
          kk++;
        } else {
          setdig(dig0, dig1, d, kk);
          d++;
          kk = 0;
        }
      }
    }

    // ---- warp-aggregated append of the owed leaves, in child order ----
    // Each lane owes at most 8 leaves; four ballots of the count's bits give every lane its
    // exclusive prefix and the warp total, so one atomic reserves the warp's slots.
    const unsigned act = __activemask();
    const unsigned cnt = (unsigned)__popc(owed);
    const unsigned b0 = __ballot_sync(act, cnt & 1u), b1 = __ballot_sync(act, cnt & 2u);
    const unsigned b2 = __ballot_sync(act, cnt & 4u), b3 = __ballot_sync(act, cnt & 8u);
    const unsigned total = __popc(b0) + 2u * __popc(b1) + 4u * __popc(b2) + 8u * __popc(b3);
    if (total) {
      const unsigned lt = (1u << lane) - 1u;
      const unsigned before = __popc(b0 & lt) + 2u * __popc(b1 & lt) + 4u * __popc(b2 & lt) +
                              8u * __popc(b3 & lt);
      const int leader = __ffs(act) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(P.leaf_count, (unsigned long long)total);
      base = __shfl_sync(act, base, leader);
      unsigned long long slot = base + before;
      while (owed) {
        if (slot >= P.leaf_cap) {
          atomicExch(P.full_flag, 1);  // the rest stays owed: suspend below
          break;
        }
        const int k = __ffs(owed) - 1;
        const QuadFx &f = fx[d][k];
        uint64_t lx = w.X | f.bx, ly = w.Y | f.by;
        if (L & 1) {
          Walk t;
          t.s0 = w.s0 + (uint64_t)f.ds[0];
          t.s1 = w.s1 + (uint64_t)f.ds[1];
          t.s2 = w.s2 + (uint64_t)f.ds[2];
          t.s3 = w.s3 + (uint64_t)f.ds[3];
          middle_bits(t, half, cm, lx, ly);
        }
        P.leaf_words[2 * slot] = lx;
        P.leaf_words[2 * slot + 1] = ly;
        P.leaf_keys[slot] = ((unsigned long long)prefix << 32) | seq;
        seq++;
        leaves++;
        slot++;
        owed &= owed - 1;
      }
    }

    // ---- suspend with leaves still owed, or at a clean point once the buffer is full ----
    iter++;
    const bool suspend = !finished &&
                         (owed != 0 || ((iter & 255) == 0 && *(volatile int *)P.full_flag));
    if (suspend) {
      const unsigned k = atomicAdd(P.nsaved_out, 1u);
      if ((int)k < P.saved_cap) {
        Saved sv;
        sv.prefix = prefix;
        sv.seq = seq;
        sv.d = (uint16_t)d;
        sv.kk = (uint16_t)kk;
        sv.owed = (uint16_t)owed;
        sv.pad = 0;
        sv.dig[0] = dig0;
        sv.dig[1] = dig1;
        P.saved_out[k] = sv;
      } else {
        atomicCAS(P.status, 0, BS_ERR_INTERNAL);
      }
    }
    if (finished || suspend) {
      if (nodes) atomicAdd(P.cell_nodes + cell, nodes);
      if (leaves) atomicAdd(P.cell_leaves + cell, leaves);
      nodes = 0;
      leaves = 0;
      have = false;
      owed = 0;
      if (suspend) break;
    }
  }
}

// Compact the leaves that passed the Hall filter (with their keys), count passes per cell.
__global__ void compact_kernel(const uint64_t *__restrict__ words, const uint64_t *__restrict__ keys,
                               const uint8_t *__restrict__ pass, long long count,
                               const Prefix *__restrict__ prefixes, uint64_t *out_words,
                               uint64_t *out_keys, unsigned long long *out_count,
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
      uint64_t k = keys[i];
      if (slot < out_cap) {
        out_words[2 * slot] = words[2 * i];
        out_words[2 * slot + 1] = words[2 * i + 1];
        out_keys[slot] = k;
      }
      atomicAdd(cell_ok + prefixes[k >> 32].cell, 1ULL);
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

struct Frontier {
  int L, m, half, D, rev, root, pinX, pinY, ns0;
  int tot[8], px[8], py[8], placed[8];
  const int8_t *tx, *ty;
  const HostQuads *Q;
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

  void rec(int d, uint64_t digits) {
    nodes++;
    if (!check()) return;
    if (d == D) {
      out->push_back(Prefix{cell, (uint32_t)D, digits});
      return;
    }
    const int i1 = d, i2 = L - 1 - d, c1 = i1 % m, c2 = i2 % m;
    const int(*S)[4] = (d == 0) ? (root == 2 ? Q->neg : (root == 1 ? Q->pos : Q->all)) : Q->pos;
    const int ns = (d == 0) ? ns0 : 8;
    for (int kk = 0; kk < ns; kk++) {
      int k = rev ? ns - 1 - kk : kk;
      if (d == 0 && pinX && S[k][0] != 1) continue;
      if (d == 0 && pinY && S[k][1] != 1) continue;
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
  uint8_t *leaf_pass = nullptr; long long pass_cap = 0;
  uint64_t *surv_words = nullptr, *surv_keys = nullptr; long long surv_cap = 0;
  unsigned long long *counters = nullptr;  // see below
  unsigned long long *cell_stats = nullptr; long long cell_stats_cap = 0;
  unsigned *nsaved = nullptr;
  int *full = nullptr;
  QuadFx *fx = nullptr;      // [32][16] branch effects
  uint64_t *posm = nullptr;  // [32] position masks
};

static StreamBufs *bufs_of(bs_ctx *ctx) {
  if (!ctx->stream_bufs) ctx->stream_bufs = new StreamBufs();
  return (StreamBufs *)ctx->stream_bufs;
}

void bs_stream_free(bs_ctx *ctx) {
  StreamBufs *b = (StreamBufs *)ctx->stream_bufs;
  if (!b) return;
  cudaFree(b->cells); cudaFree(b->prefixes); cudaFree(b->saved[0]); cudaFree(b->saved[1]);
  cudaFree(b->leaf_words); cudaFree(b->leaf_keys); cudaFree(b->leaf_pass);
  cudaFree(b->surv_words); cudaFree(b->surv_keys); cudaFree(b->counters);
  cudaFree(b->cell_stats); cudaFree(b->nsaved); cudaFree(b->full); cudaFree(b->fx);
  cudaFree(b->posm);
  delete b;
  ctx->stream_bufs = nullptr;
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
  if (opt->cd_prune != 0) return BS_ERR_ARG;  // optional CD_PRUNE is not built on the device
  int hall_mode = opt->hall_mode;
  if (hall_mode < BS_HALL_FP64 || hall_mode > BS_HALL_TC_BF16X2) return BS_ERR_ARG;
  CK(cudaSetDevice(ctx->device));
  StreamBufs *B = bufs_of(ctx);
  const int half = L / 2;

  // ---- coarse frontier of each cell on the host, in the reference's order ----
  // A Prefix holds the digits of 16 depths, so no prefix is deeper than that.
  static const HostQuads Q;
  const int max_depth = std::min(half - 1, 16);
  std::vector<Frontier> F(ncells);
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

  // The subtrees of coarse prefix p, refined by k more levels: the fine prefixes of its
  // subtree at depth p.depth + k, in stream order. Returns the host nodes it adds (the coarse
  // node itself was counted when the frontier was built).
  auto refine = [&](const Prefix &p, int k, std::vector<Prefix> &out) -> long long {
    if (k <= 0) {
      out.push_back(p);
      return 0;
    }
    Frontier &f = F[p.cell];
    memset(f.px, 0, sizeof f.px); memset(f.py, 0, sizeof f.py); memset(f.placed, 0, sizeof f.placed);
    for (int t = 0; t < (int)p.depth; t++) {
      const int(*S)[4] = (t == 0) ? (f.root == 2 ? Q.neg : (f.root == 1 ? Q.pos : Q.all)) : Q.pos;
      const int ns = (t == 0) ? f.ns0 : 8;
      const int kk = (int)((p.digits >> (4 * t)) & 15);
      const int q = f.rev ? ns - 1 - kk : kk;
      const int c1 = t % m, c2 = (L - 1 - t) % m;
      f.px[c1] += S[q][0]; f.py[c1] += S[q][1]; f.px[c2] += S[q][2]; f.py[c2] += S[q][3];
      f.placed[c1]++; f.placed[c2]++;
    }
    f.D = (int)p.depth + k;
    f.out = &out;
    const long long before = f.nodes;
    f.rec((int)p.depth, p.digits);
    return f.nodes - before - 1;
  };

  // ---- device buffers ----
  int rc = bs_ensure_dev((void **)&B->cells, &B->cells_cap, ncells, sizeof(CellDev));
  if (!rc) rc = bs_ensure_dev((void **)&B->cell_stats, &B->cell_stats_cap, 3LL * ncells, sizeof(unsigned long long));
  long long leaf_cap = opt->leaf_chunk > 0 ? opt->leaf_chunk : (1LL << 24);
  if (!rc) {
    long long c0 = B->leaf_cap;
    rc = bs_ensure_dev((void **)&B->leaf_keys, &B->leaf_cap, leaf_cap, sizeof(uint64_t));
    if (!rc && (B->leaf_cap != c0 || !B->leaf_words)) {
      cudaFree(B->leaf_words);
      B->leaf_words = nullptr;
      CK(cudaMalloc(&B->leaf_words, sizeof(uint64_t) * 2 * B->leaf_cap));
    }
  }
  if (!rc) rc = bs_ensure_dev((void **)&B->leaf_pass, &B->pass_cap, leaf_cap, 1);
  const int block = 256;
  // register budget variant (BS_DFS_BLOCKS=6 selects the 40-register one) and the grid of
  // exactly the blocks that fit at once
  static const int dfs_blocks = [] {
    const char *e = getenv("BS_DFS_BLOCKS");
    return (e && atoi(e) == 6) ? 6 : 4;
  }();
  auto dfs_kernel = dfs_blocks == 6 ? cd_dfs_kernel<6> : cd_dfs_kernel<4>;
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
    CK(cudaMalloc(&B->full, sizeof(int)));
    CK(cudaMalloc(&B->fx, sizeof(QuadFx) * 32 * 16));
    CK(cudaMalloc(&B->posm, sizeof(uint64_t) * 32));
  }
  long long surv_cap = opt->survivor_cap > 0 ? opt->survivor_cap : (1LL << 22);
  if (!rc) {
    long long c0 = B->surv_cap;
    rc = bs_ensure_dev((void **)&B->surv_keys, &B->surv_cap, surv_cap, sizeof(uint64_t));
    if (!rc && (B->surv_cap != c0 || !B->surv_words)) {
      cudaFree(B->surv_words);
      B->surv_words = nullptr;
      CK(cudaMalloc(&B->surv_words, sizeof(uint64_t) * 2 * B->surv_cap));
    }
  }
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
  CK(cudaMemcpyAsync(B->cells, hc.data(), sizeof(CellDev) * ncells, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(B->cell_stats, 0, sizeof(unsigned long long) * 3 * ncells, s));
  // counters: [0] next prefix of the wave, [1] leaf count of the round, [2] survivors of the wave
  unsigned long long *cell_nodes = B->cell_stats, *cell_leaves = B->cell_stats + ncells,
                     *cell_ok = B->cell_stats + 2 * ncells;

  // ---- waves: runs of coarse prefixes, in stream order, refined to fill the GPU ----
  // A wave's survivors all precede the next wave's, so each wave is ordered on its own and
  // appended. The width (coarse prefixes per wave) and the refinement depth adapt to the
  // nodes per coarse prefix seen so far: fine subtrees of ~FINE_NODES nodes, waves of
  // ~WAVE_NODES nodes, and under `limit` no wider than the survivors still owed suggest.
  const long long limit = opt->limit > 0 ? opt->limit : 0;
  const double FINE_NODES = 2e4, WAVE_NODES = 8e9, NOMINAL_RATE = 2e10;
  const long long threads = (long long)grid * block;
  std::vector<uint64_t> res_words;
  std::vector<uint32_t> res_cell;
  std::vector<Prefix> fine;
  std::vector<uint64_t> wkeys, wwords;
  std::vector<unsigned long long> cs_prev(3 * (size_t)ncells, 0), cs(3 * (size_t)ncells, 0);
  long long pos = 0, wave_width = std::min<long long>(ncoarse, 1024);
  int k_refine = (half - deepest >= 6) ? 2 : 0;
  long long have = 0;
  static const bool trace = getenv("BS_STREAM_TRACE") != nullptr;  // per-wave figures on stderr
  while (pos < ncoarse && !(limit && have >= limit)) {
    const long long take = std::min<long long>(std::max<long long>(1, wave_width), ncoarse - pos);
    fine.clear();
    for (long long i = pos; i < pos + take; i++) {
      const int k = std::min(k_refine, max_depth - (int)coarse[i].depth);
      host_nodes[coarse[i].cell] += refine(coarse[i], k, fine);
    }
    pos += take;
    const long long nprefix = (long long)fine.size();
    if (nprefix == 0) continue;  // the refinement pruned the whole run
    if (nprefix >= (1LL << 32)) return BS_ERR_CAP;
    rc = bs_ensure_dev((void **)&B->prefixes, &B->prefix_cap, nprefix, sizeof(Prefix));
    if (rc) return rc;
    CK(cudaMemcpyAsync(B->prefixes, fine.data(), sizeof(Prefix) * nprefix, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(B->counters, 0, sizeof(unsigned long long) * 8, s));
    const auto t_wave = std::chrono::steady_clock::now();

    int nsaved = 0, cur = 0;
    for (;;) {
      CK(cudaMemsetAsync(B->nsaved, 0, sizeof(unsigned), s));
      CK(cudaMemsetAsync(B->full, 0, sizeof(int), s));
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
      P.leaf_words = B->leaf_words; P.leaf_keys = B->leaf_keys;
      P.leaf_count = B->counters + 1; P.leaf_cap = (unsigned long long)leaf_cap;
      P.cell_nodes = cell_nodes; P.cell_leaves = cell_leaves;
      P.full_flag = B->full; P.status = ctx->d_status;
      bs_timed_begin(ctx);
      dfs_kernel<<<grid, block, 0, s>>>(P);
      bs_timed_end(ctx);
      CK(cudaGetLastError());
      unsigned long long leaf_count = 0;
      unsigned nsv = 0;
      CK(cudaMemcpyAsync(&leaf_count, B->counters + 1, sizeof leaf_count, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&nsv, B->nsaved, sizeof nsv, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if ((int)nsv > saved_cap) return BS_ERR_INTERNAL;
      long long nleaf = (long long)std::min<unsigned long long>(leaf_count, (unsigned long long)leaf_cap);
      if (nleaf > 0) {
        int r2 = bs_hall_dev_len(ctx, B->leaf_words, nleaf, hall_mode, B->leaf_pass, L);
        if (r2) return r2;
        ctx->launches++;
        compact_kernel<<<bs_grid_for(nleaf, 256, 8 * ctx->num_sms), 256, 0, s>>>(
            B->leaf_words, B->leaf_keys, B->leaf_pass, nleaf, B->prefixes, B->surv_words, B->surv_keys,
            B->counters + 2, (unsigned long long)surv_cap, cell_ok);
        CK(cudaGetLastError());
      }
      nsaved = (int)nsv;
      cur ^= 1;
      if (nsaved == 0) {
        unsigned long long nextp = 0;
        CK(cudaMemcpyAsync(&nextp, B->counters, sizeof nextp, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (nextp >= (unsigned long long)nprefix) break;
      }
    }

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
      wkeys.resize(nsurv);
      wwords.resize(2 * nsurv);
      CK(cudaMemcpyAsync(wkeys.data(), B->surv_keys, sizeof(uint64_t) * nsurv, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(wwords.data(), B->surv_words, sizeof(uint64_t) * 2 * nsurv, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      std::vector<uint32_t> order(nsurv);
      for (uint32_t i = 0; i < (uint32_t)nsurv; i++) order[i] = i;
      std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return wkeys[a] < wkeys[b]; });
      long long keep = (long long)nsurv;
      if (limit) keep = std::min(keep, limit - have);
      for (long long i = 0; i < keep; i++) {
        res_words.push_back(wwords[2 * order[i]]);
        res_words.push_back(wwords[2 * order[i] + 1]);
        res_cell.push_back(fine[wkeys[order[i]] >> 32].cell);
      }
      have += keep;
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
    // enough fine prefixes for every thread, twice over
    width = std::max(width, 2.0 * (double)threads / std::pow(8.0, k_refine));
    if (limit && nsurv > 0) {
      const double per_coarse_surv = (double)nsurv / (double)take;
      width = std::min(width, std::max(64.0, 1.5 * (double)(limit - have) / per_coarse_surv));
    }
    wave_width = (long long)std::min<double>(width, (double)(1LL << 40));
    if (trace)
      fprintf(stderr, "[bs_cd_stream] wave coarse=%lld fine=%lld nodes=%llu surv=%llu have=%lld "
                      "secs=%.4f next_width=%lld next_k=%d pos=%lld/%lld\n",
              take, nprefix, wave_nodes, nsurv, have, secs, wave_width, k_refine, pos, ncoarse);
  }

  // ---- results ----
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
  return BS_OK;
}
