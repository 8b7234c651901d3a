// oracle_device.cpp - TEST INFRASTRUCTURE ONLY, never part of the product.
//
// Answers the device calls the lane binary makes (bs_ctx_*, bs_cd_stream, bs_flat_topk,
// bs_complete_ab_batch; include/bsfh.h) with the CPU oracle (oracle/bs_oracle.h), so that a
// test build of bin/bs_firsthit's host logic -- the cell list, the probe replay, the drain
// order, the checkpoint file, the stdout protocol -- can be replayed against the reference's
// own lane runs on a machine without a GPU (tests/test_lane_host_cpu.py). The product binary
// links libbsfh.so and runs these calls on the GPU; this file is linked only into the test
// build under tests/_build/.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/bsfh.h"
#include "../../oracle/bs_oracle.h"

struct bs_ctx {
  int n, a, b, c, d;
  int32_t stop;
};

namespace {
void unpack(uint64_t w, int L, int8_t *x) {
  for (int i = 0; i < L; i++) x[i] = ((w >> i) & 1ULL) ? 1 : -1;
}
uint64_t pack(const int8_t *x, int L) {
  uint64_t w = 0;
  for (int i = 0; i < L; i++)
    if (x[i] > 0) w |= 1ULL << i;
  return w;
}
}  // namespace

extern "C" const char *bs_strerror(int code) {
  return code == BS_OK ? "ok" : code == BS_STOPPED ? "stopped" : "error (oracle-backed test build)";
}

extern "C" int bs_ctx_create(int n, int a, int b, int c, int d, int, bs_ctx **out) {
  if (!out || n < 4 || n + 1 > 64) return BS_ERR_ARG;
  *out = new bs_ctx{n, a, b, c, d, 0};
  return BS_OK;
}

extern "C" void bs_ctx_destroy(bs_ctx *ctx) { delete ctx; }

extern "C" volatile int32_t *bs_ctx_stop_flag(bs_ctx *ctx) { return &ctx->stop; }

// Every cell streamed whole by the oracle (its survivors in the reference's order, its
// counts those of the whole cell); `limit` keeps the batch's first `limit` survivors.
extern "C" int bs_cd_stream(bs_ctx *ctx, const bs_cell *cells, int ncells, const bs_stream_opts *opt,
                            uint64_t *out_words, uint32_t *out_cell, long long out_cap,
                            long long *nout, bs_cell_stats *stats) {
  if (!ctx || !opt || !nout || ncells < 0) return BS_ERR_ARG;
  if (ctx->stop) { *nout = 0; return BS_STOPPED; }
  const int n = ctx->n, L = n, m = opt->m;
  std::vector<uint64_t> words;
  std::vector<uint32_t> owner;
  for (int ci = 0; ci < ncells; ci++) {
    int tx[8], ty[8];
    for (int c = 0; c < m; c++) { tx[c] = cells[ci].tx[c]; ty[c] = cells[ci].ty[c]; }
    or_stream_stats st{};
    const long long total = or_cd_stream(n, L, m, tx, ty, cells[ci].pinX, cells[ci].pinY, opt->rev,
                                         opt->endpos, opt->cd_prune, 0, nullptr, nullptr, 0, &st);
    std::vector<int8_t> xy((size_t)std::max(1LL, total) * 2 * L);
    or_stream_stats st2{};
    or_cd_stream(n, L, m, tx, ty, cells[ci].pinX, cells[ci].pinY, opt->rev, opt->endpos,
                 opt->cd_prune, 0, xy.data(), nullptr, total, &st2);
    if (stats) stats[ci] = bs_cell_stats{st2.nodes, st2.leaves, st2.ok};
    for (long long k = 0; k < total; k++) {
      words.push_back(pack(&xy[(size_t)k * 2 * L], L));
      words.push_back(pack(&xy[(size_t)k * 2 * L + L], L));
      owner.push_back((uint32_t)ci);
    }
  }
  long long count = (long long)owner.size();
  if (opt->limit > 0) count = std::min(count, opt->limit);
  *nout = count;
  if (count > out_cap) return BS_ERR_CAP;
  if (count > 0 && out_words) memcpy(out_words, words.data(), sizeof(uint64_t) * 2 * (size_t)count);
  if (count > 0 && out_cell) memcpy(out_cell, owner.data(), sizeof(uint32_t) * (size_t)count);
  return BS_OK;
}

// Batches of buf_cap survivors, each ordered by the reference's flat score (ties in stream
// order), its first `keep` (keep <= 0: all) returned as stream indices.
extern "C" int bs_flat_topk(bs_ctx *ctx, const uint64_t *words, long long nsurv, long long buf_cap,
                            long long keep, int64_t *order, int32_t *scores, long long *nkept) {
  if (!ctx || !nkept || nsurv < 0 || buf_cap <= 0) return BS_ERR_ARG;
  const int n = ctx->n;
  std::vector<int8_t> C(n), D(n);
  long long out = 0;
  for (long long b0 = 0; b0 < nsurv; b0 += buf_cap) {
    const long long b1 = std::min(nsurv, b0 + buf_cap);
    std::vector<long long> sc((size_t)(b1 - b0)), idx((size_t)(b1 - b0));
    for (long long i = b0; i < b1; i++) {
      unpack(words[2 * i], n, C.data());
      unpack(words[2 * i + 1], n, D.data());
      sc[(size_t)(i - b0)] = or_flat_score(C.data(), D.data(), n);
    }
    std::iota(idx.begin(), idx.end(), 0LL);
    std::stable_sort(idx.begin(), idx.end(), [&](long long x, long long y) { return sc[x] < sc[y]; });
    const long long k = keep > 0 ? std::min(keep, b1 - b0) : b1 - b0;
    for (long long t = 0; t < k; t++, out++) {
      order[out] = b0 + idx[(size_t)t];
      if (scores) scores[out] = (int32_t)sc[(size_t)idx[(size_t)t]];
    }
  }
  *nkept = out;
  return BS_OK;
}

// fh_complete_ab per candidate by the oracle, on all host threads in runs of candidates; in
// first-hit mode the candidates after the first hit are reported as not run (verdict -1), as
// the device reports them.
extern "C" int bs_complete_ab_batch(bs_ctx *ctx, const bs_ab_cand *cands, long long ncand,
                                    const int8_t *rows, long long nrows_total, const bs_ab_opts *opt,
                                    int32_t *verdict, long long *nodes, int8_t *A, int8_t *B) {
  if (!ctx || !opt || ncand < 0 || (ncand > 0 && (!cands || !verdict || !nodes))) return BS_ERR_ARG;
  if (opt->a2 != 0 && opt->a2 != 2) return BS_ERR_ARG;
  const int n = ctx->n, n1 = n + 1;
  std::vector<int32_t> v((size_t)ncand, -1);
  std::vector<long long> nd((size_t)ncand, 0);
  std::vector<int8_t> ab((size_t)ncand * 2 * n1, 0);
  auto one = [&](long long i) {
    std::vector<int8_t> C(n), D(n);
    unpack(cands[i].c, n, C.data());
    unpack(cands[i].d, n, D.data());
    const bool ranged = cands[i].nrows > 0 && rows && cands[i].row_off + cands[i].nrows <= nrows_total;
    v[(size_t)i] = or_complete_ab_a2(n, ctx->a, ctx->b, C.data(), D.data(), opt->budget,
                                     opt->outer_k, opt->early, opt->canon, opt->m,
                                     ranged ? rows + 16 * cands[i].row_off : nullptr,
                                     ranged ? cands[i].nrows : 0, opt->a2, &ab[(size_t)i * 2 * n1],
                                     &ab[(size_t)i * 2 * n1 + n1], &nd[(size_t)i]);
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  long long done = 0;
  bool hit = false;
  while (done < ncand && !(hit && opt->first_hit) && !ctx->stop) {
    const long long end = std::min(ncand, done + 64LL * hw);
    std::atomic<long long> next(done);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < hw; t++)
      th.emplace_back([&] {
        for (long long i; (i = next.fetch_add(1)) < end;) one(i);
      });
    for (auto &x : th) x.join();
    for (long long i = done; i < end && !hit; i++) hit = v[(size_t)i] == 0;
    done = end;
  }
  bool seen_hit = false;
  for (long long i = 0; i < ncand; i++) {
    const bool run = i < done && !(seen_hit && opt->first_hit);
    verdict[i] = run ? v[(size_t)i] : -1;
    nodes[i] = run ? nd[(size_t)i] : 0;
    if (A) memcpy(A + i * n1, &ab[(size_t)i * 2 * n1], (size_t)n1);
    if (B) memcpy(B + i * n1, &ab[(size_t)i * 2 * n1 + n1], (size_t)n1);
    if (run && v[(size_t)i] == 0) seen_hit = true;
  }
  return ctx->stop ? BS_STOPPED : BS_OK;
}
