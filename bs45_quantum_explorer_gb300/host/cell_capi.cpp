// cell_capi.cpp - C ABI of the host-side cell algebra (bs_cell_list, bs_ab_rows in
// include/bsfh.h). Host only: these calls touch no device and need no context, so a
// scheduler can plan a lane's cells (and its HBM needs) before it opens a GPU.
#include <cstring>
#include <exception>
#include <mutex>
#include <unordered_map>

#include "../../include/bsfh.h"
#include "celllist.h"

using namespace bsfh;

namespace {
// The last list a bs_cell_list call built but could not return (its buffer was short). The
// usual caller asks again with the size it was told, so that call copies this list instead
// of building it a second time. One list is held at most; any call with other arguments
// drops it.
struct PendingList {
  bool valid = false;
  int n = 0, a = 0, b = 0, c = 0, d = 0;
  bs_list_opts opt{};
  CellList list;
};
std::mutex g_pending_mu;
PendingList g_pending;

bool same_request(const PendingList &p, int n, int a, int b, int c, int d, const bs_list_opts &o) {
  const bs_list_opts &q = p.opt;
  return p.valid && p.n == n && p.a == a && p.b == b && p.c == c && p.d == d && q.m6 == o.m6 &&
         q.thm211b == o.thm211b && q.thm212 == o.thm212 && q.endpos == o.endpos &&
         q.orbit_canon == o.orbit_canon && q.orbit_q == o.orbit_q && q.qprune == o.qprune &&
         q.prof_order == o.prof_order && q.nshard == o.nshard;
}
}  // namespace

extern "C" int bs_cell_list(int n, int a, int b, int c, int d, const bs_list_opts *opt,
                            bs_cell *cells, uint8_t *kept, long long cap, long long *ncells,
                            char *digest) {
  if (!opt || !ncells || n < 4 || n + 1 > 64 || cap < 0) return BS_ERR_ARG;
  if (a * a + b * b + c * c + d * d != 4 * n + 2) return BS_ERR_ARG;
  if (opt->prof_order < 0 || opt->prof_order > 3 || opt->orbit_q < 0 || opt->orbit_q > 2)
    return BS_ERR_ARG;
  if (opt->prof_order == 3 && !opt->orbit_canon) return BS_ERR_ARG;
  ListOptions lo;
  lo.m6 = opt->m6 != 0;
  lo.thm211b = opt->thm211b != 0;
  lo.thm212 = opt->thm212 != 0;
  lo.endpos = opt->endpos != 0;
  lo.orbit_canon = opt->orbit_canon != 0;
  lo.orbit_q = opt->orbit_q;
  lo.qprune = opt->qprune != 0;
  lo.prof_order = opt->prof_order;
  lo.nshard = opt->nshard > 0 ? opt->nshard : 1;
  CellList list;
  bool reused = false;
  {
    std::lock_guard<std::mutex> lock(g_pending_mu);
    if (same_request(g_pending, n, a, b, c, d, *opt) &&
        (long long)g_pending.list.cells.size() <= cap) {
      list = std::move(g_pending.list);
      reused = true;
    }
    if (reused || g_pending.valid) {
      g_pending.valid = false;
      g_pending.list = CellList();
    }
  }
  if (!reused) {
    try {
      if (build_cell_list(n, a, b, c, d, lo, list, nullptr) != 0) return 2;
    } catch (const std::exception &) {
      return BS_ERR_NOMEM;
    }
  }
  *ncells = (long long)list.cells.size();
  if (digest) {
    memset(digest, 0, 40);
    strncpy(digest, list.digest.c_str(), 39);
  }
  if ((long long)list.cells.size() > cap) {
    std::lock_guard<std::mutex> lock(g_pending_mu);
    g_pending.valid = true;
    g_pending.n = n; g_pending.a = a; g_pending.b = b; g_pending.c = c; g_pending.d = d;
    g_pending.opt = *opt;
    g_pending.list = std::move(list);
    return BS_ERR_CAP;
  }
  const bool pin = !lo.orbit_canon;
  for (size_t i = 0; i < list.cells.size(); i++) {
    if (cells) {
      bs_cell &o = cells[i];
      memset(&o, 0, sizeof o);
      for (int k = 0; k < list.m; k++) {
        o.tx[k] = (int8_t)list.cells[i].px[k];
        o.ty[k] = (int8_t)list.cells[i].py[k];
      }
      o.pinX = pin && c == 0;
      o.pinY = pin && d == 0;
    }
    if (kept) kept[i] = list.kept[i];
  }
  return BS_OK;
}

extern "C" int bs_ab_rows(int n, int a, int b, int m, const bs_cell *cells, long long ncells,
                          int8_t *rows, long long rows_cap, long long *row_off, int32_t *nrows,
                          long long *nrows_total) {
  if (!nrows_total || n < 4 || n + 1 > 64 || (m != 3 && m != 6) || ncells < 0 ||
      (ncells > 0 && (!cells || !row_off || !nrows)) || rows_cap < 0)
    return BS_ERR_ARG;
  std::vector<uint64_t> keys(ncells);
  for (long long i = 0; i < ncells; i++) {
    Profile p;
    p.px.assign(cells[i].tx, cells[i].tx + m);
    p.py.assign(cells[i].ty, cells[i].ty + m);
    keys[i] = AbpRows::cell_key_of(p, n, m);
  }
  AbpRows abp;
  try {
    abp.build(keys, n, a, b, m);
  } catch (const std::exception &) {
    return BS_ERR_NOMEM;
  }
  // one copy of each invariant's rows, in the order its first cell appears
  std::unordered_map<uint64_t, long long> placed;
  long long total = 0;
  for (long long i = 0; i < ncells; i++) {
    const auto &v = abp.by_key[keys[i]];
    const long long k = (long long)v.size() / 16;
    if (k > 0x7fffffff) return BS_ERR_CAP;
    nrows[i] = (int32_t)k;
    auto it = placed.find(keys[i]);
    if (it != placed.end()) {
      row_off[i] = it->second;
      continue;
    }
    row_off[i] = total;
    placed.emplace(keys[i], total);
    if (rows && total + k <= rows_cap) memcpy(rows + 16 * total, v.data(), v.size());
    total += k;
  }
  *nrows_total = total;
  return total > rows_cap ? BS_ERR_CAP : BS_OK;
}
