// celllist.cpp - residue-class cell algebra of the first-hit lane (host side).
// Each function states the reference lines (src/solver/wz_match.cpp) whose result it
// reproduces; the enumeration orders are part of the lane's contract (raw cell indices,
// digests and checkpoints depend on them).
#include "celllist.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <thread>

namespace bsfh {

// Runs f(lo, hi, part) over [0, n) split into contiguous parts, one host thread each. Callers
// keep one output per part and join them in part order, so every result is the same as the
// serial loop's, whatever the thread count.
template <class F>
static int parallel_parts(size_t n, F f, size_t min_per_part = 256) {
  unsigned hw = std::thread::hardware_concurrency();
  size_t parts = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, 64));
  parts = std::min(parts, std::max<size_t>(1, n / min_per_part));
  if (parts <= 1) {
    f((size_t)0, n, (size_t)0);
    return 1;
  }
  const size_t chunk = (n + parts - 1) / parts;
  std::vector<std::thread> th;
  for (size_t t = 0; t < parts; t++) {
    const size_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back(f, lo, hi, t);
  }
  for (auto &x : th) x.join();
  return (int)parts;
}

// std::sort on all host threads: contiguous parts sorted at once, then merged pairwise. The
// result is sorted by `cmp`; elements that compare equal may come out in another order than a
// serial std::sort would leave them (callers sort by keys that are distinct, or do not
// depend on the order of ties).
template <class T, class Cmp>
static void parallel_sort(std::vector<T> &v, Cmp cmp) {
  const size_t n = v.size();
  const unsigned hw = std::thread::hardware_concurrency();
  size_t parts = 1;
  while (parts * 2 <= std::min<size_t>(hw ? hw : 1, 64)) parts *= 2;
  if (parts <= 1 || n < ((size_t)1 << 16)) {
    std::sort(v.begin(), v.end(), cmp);
    return;
  }
  std::vector<size_t> b(parts + 1);
  for (size_t i = 0; i <= parts; i++) b[i] = n * i / parts;
  std::vector<std::thread> th;
  for (size_t i = 0; i < parts; i++)
    th.emplace_back([&, i] { std::sort(v.begin() + b[i], v.begin() + b[i + 1], cmp); });
  for (auto &x : th) x.join();
  for (size_t w = 1; w < parts; w *= 2) {
    th.clear();
    for (size_t i = 0; i + w < parts; i += 2 * w)
      th.emplace_back([&, i, w] {
        std::inplace_merge(v.begin() + b[i], v.begin() + b[i + w],
                           v.begin() + b[std::min(i + 2 * w, parts)], cmp);
      });
    for (auto &x : th) x.join();
  }
}

int class_count(int L, int c, int m) {
  int k = 0;
  for (int p = c; p < L; p += m) k++;
  return k;
}

// Odometer over classes 0..m-2 (each from -count to +count in steps of 2, the first class
// varying slowest); the last class takes what is left when it fits its count and parity.
std::vector<Vec> enum_class_sums(int L, int target, int m) {
  std::vector<int> cnt(m);
  for (int c = 0; c < m; c++) cnt[c] = class_count(L, c, m);
  std::vector<Vec> out;
  Vec cur(m);
  for (int c = 0; c < m - 1; c++) cur[c] = -cnt[c];
  for (;;) {
    int acc = 0;
    for (int c = 0; c < m - 1; c++) acc += cur[c];
    int last = target - acc;
    if (last >= -cnt[m - 1] && last <= cnt[m - 1] && ((last + cnt[m - 1]) & 1) == 0) {
      cur[m - 1] = last;
      out.push_back(cur);
    }
    int c = m - 2;
    while (c >= 0) {
      cur[c] += 2;
      if (cur[c] <= cnt[c]) break;
      cur[c] = -cnt[c];
      c--;
    }
    if (c < 0) break;
  }
  return out;
}

int norm_vec(const Vec &v) {
  int s = 0;
  for (int x : v) s += x * x;
  return s;
}

int autocorr_vec(const Vec &v, int s) {
  int m = (int)v.size(), t = 0;
  for (int i = 0; i + s < m; i++) t += v[i] * v[i + s];
  return t;
}

int pair_auto(const Vec &x, const Vec &y, int s) {
  int m = (int)x.size();
  return autocorr_vec(x, s) + autocorr_vec(y, s) + autocorr_vec(x, m - s) + autocorr_vec(y, m - s);
}

uint64_t auto_key(const Vec &T, int norm) {
  uint64_t k = (uint64_t)(uint16_t)norm;
  for (size_t i = 0; i < T.size() && i < 3; i++)
    k |= (uint64_t)(uint16_t)(T[i] + 8192) << (16 * (i + 1));
  return k;
}

static inline int mod4(int v) { return ((v % 4) + 4) % 4; }

bool thm212_ok(const Vec &x, const Vec &y, int m, int n, bool abSide) {
  if (abSide) {
    const int c1 = n % m, want = (n % m) ? 2 : 0;
    if (mod4(x[0] + y[0] + x[c1] + y[c1]) != want) return false;
    for (int j = 2; j <= m; j++) {
      if (j == c1 + 1) continue;
      const int c = ((n + 1 - j) % m + m) % m;
      if (mod4(x[j - 1] + y[j - 1] + x[c] + y[c]) != 0) return false;
    }
  } else {
    for (int j = 1; j <= m; j++) {
      const int c = ((n - j) % m + m) % m;
      if (mod4(x[j - 1] + y[j - 1] + x[c] + y[c]) != 0) return false;
    }
  }
  return true;
}

// The set of norm(k) + norm(r) <= 4n+2 over every (k, r) pair depends only on the distinct
// norms on each side, so the pairs are taken over those.
void NormSet::build(int L, int a, int b, int m, int n) {
  const auto K = enum_class_sums(L, a, m), R = enum_class_sums(L, b, m);
  const int tgt = 4 * n + 2;
  std::vector<char> kn(tgt + 1, 0), rn(tgt + 1, 0);
  for (const auto &kv : K) {
    const int v = norm_vec(kv);
    if (v <= tgt) kn[v] = 1;
  }
  for (const auto &rv : R) {
    const int v = norm_vec(rv);
    if (v <= tgt) rn[v] = 1;
  }
  vals.assign(tgt + 1, 0);
  for (int x = 0; x <= tgt; x++)
    if (kn[x])
      for (int y = 0; x + y <= tgt; y++)
        if (rn[y]) vals[x + y] = 1;
}

// One side's share of pair_auto at shift s: pair_auto(x, y, s) = side_auto(x, s) + side_auto(y, s).
static inline int side_auto(const Vec &v, int s) {
  return autocorr_vec(v, s) + autocorr_vec(v, (int)v.size() - s);
}

namespace {
// What a class-sum vector contributes to a (k, r) pair's 2.11b key and 2.12 test: its norm,
// its shares of the residue autocorrelations, and its entries mod 4 (thm212_ok reads sums of
// entries mod 4 only). Vectors with equal features give equal keys and verdicts in every pair.
struct SideFeat {
  int norm;
  int ca[3];
  uint32_t mod4;  // two bits per entry
  bool operator==(const SideFeat &o) const {
    return norm == o.norm && ca[0] == o.ca[0] && ca[1] == o.ca[1] && ca[2] == o.ca[2] && mod4 == o.mod4;
  }
};
struct SideFeatHash {
  size_t operator()(const SideFeat &f) const {
    uint64_t h = (uint64_t)(uint32_t)f.norm * 0x9E3779B97F4A7C15ULL;
    for (int v : f.ca) h = (h ^ (uint32_t)v) * 0xBF58476D1CE4E5B9ULL;
    return (size_t)((h ^ f.mod4) * 0x94D049BB133111EBULL);
  }
};
// The distinct features of `vs` (norm <= tgt), each with the first vector that has them.
std::vector<std::pair<SideFeat, const Vec *>> distinct_features(const std::vector<Vec> &vs, int half,
                                                                int tgt) {
  std::unordered_set<SideFeat, SideFeatHash> seen;
  std::vector<std::pair<SideFeat, const Vec *>> out;
  for (const Vec &v : vs) {
    SideFeat f{norm_vec(v), {0, 0, 0}, 0};
    if (f.norm > tgt) continue;
    for (int s = 1; s <= half && s <= 3; s++) f.ca[s - 1] = side_auto(v, s);
    for (size_t c = 0; c < v.size(); c++) f.mod4 |= (uint32_t)(((v[c] % 4) + 4) % 4) << (2 * c);
    if (seen.insert(f).second) out.push_back({f, &v});
  }
  return out;
}
}  // namespace

// Every key auto_key(T(k, r), norm(k) + norm(r)) over the (k, r) pairs that pass, taken over
// the distinct features of each side (the key set is the same as over all pairs).
void AutoSet::build(int L, int a, int b, int m, int n, bool thm212) {
  const auto K = enum_class_sums(L, a, m), R = enum_class_sums(L, b, m);
  const int tgt = 4 * n + 2, half = m / 2;
  const bool abSide = (L == n + 1);
  const auto FK = distinct_features(K, half, tgt), FR = distinct_features(R, half, tgt);
  std::vector<std::unordered_set<uint64_t>> part(64);
  parallel_parts(FK.size(), [&](size_t lo, size_t hi, size_t t) {
    Vec T(half);
    for (size_t i = lo; i < hi; i++) {
      const SideFeat &fk = FK[i].first;
      for (const auto &r : FR) {
        const SideFeat &fr = r.first;
        if (fk.norm + fr.norm > tgt) continue;
        if (thm212 && !thm212_ok(*FK[i].second, *r.second, m, n, abSide)) continue;
        for (int s = 1; s <= half && s <= 3; s++) T[s - 1] = fk.ca[s - 1] + fr.ca[s - 1];
        part[t].insert(auto_key(T, fk.norm + fr.norm));
      }
    }
  }, 16);
  for (auto &p : part) keys.insert(p.begin(), p.end());
}

static Vec reduce63(const Vec &v6) { return Vec{v6[0] + v6[3], v6[1] + v6[4], v6[2] + v6[5]}; }

std::vector<Profile> survive_profiles3(int L, int sigX, int sigY, int n, const NormSet &comp3,
                                       const NormSet &comp6, const AutoSet *comp6auto, bool thm212,
                                       bool thm211b) {
  const int tgt = 4 * n + 2;
  const bool abSide = (L == n + 1);
  const auto PX3 = enum_class_sums(L, sigX, 3), PY3 = enum_class_sums(L, sigY, 3);
  const auto PX6 = enum_class_sums(L, sigX, 6), PY6 = enum_class_sums(L, sigY, 6);
  // the mod-6 refinements of each mod-3 vector, in enumeration order, with their norms and
  // residue-autocorrelation shares (the existential search below visits only these)
  std::unordered_map<std::string, std::vector<size_t>> x_of, y_of;
  for (size_t i = 0; i < PX6.size(); i++) x_of[cell_key(reduce63(PX6[i]), Vec())].push_back(i);
  for (size_t j = 0; j < PY6.size(); j++) y_of[cell_key(reduce63(PY6[j]), Vec())].push_back(j);
  auto shares = [](const std::vector<Vec> &V, std::vector<int> &nv, std::vector<int> &ca) {
    nv.resize(V.size());
    ca.resize(3 * V.size());
    for (size_t i = 0; i < V.size(); i++) {
      nv[i] = norm_vec(V[i]);
      for (int s = 1; s <= 3; s++) ca[3 * i + s - 1] = side_auto(V[i], s);
    }
  };
  std::vector<int> nx6, cax6, ny6, cay6;
  shares(PX6, nx6, cax6);
  shares(PY6, ny6, cay6);
  static const std::vector<size_t> none;
  std::vector<std::vector<Profile>> part(64);
  parallel_parts(PX3.size(), [&](size_t lo, size_t hi, size_t t) {
  std::vector<Profile> &out = part[t];
  Vec needT(3);
  for (size_t ix = lo; ix < hi; ix++) {
    const Vec &px = PX3[ix];
    const int npx = norm_vec(px);
    if (npx > tgt) continue;
    auto xi = x_of.find(cell_key(px, Vec()));
    const std::vector<size_t> &xs = xi == x_of.end() ? none : xi->second;
    for (const auto &py : PY3) {
      const int need = tgt - npx - norm_vec(py);
      if (need < 0 || !comp3.has(need)) continue;
      if (thm212 && !thm212_ok(px, py, 3, n, abSide)) continue;
      auto yi = y_of.find(cell_key(py, Vec()));
      const std::vector<size_t> &ys = yi == y_of.end() ? none : yi->second;
      bool ok6 = false;
      for (size_t ii = 0; ii < xs.size() && !ok6; ii++) {
        const size_t i = xs[ii];
        const int npx6 = nx6[i];
        if (npx6 > tgt) continue;
        for (size_t j : ys) {
          const int need6 = tgt - npx6 - ny6[j];
          if (need6 < 0) continue;
          if (thm212 && !thm212_ok(PX6[i], PY6[j], 6, n, abSide)) continue;
          if (thm211b && comp6auto) {
            for (int s = 0; s < 3; s++) needT[s] = -(cax6[3 * i + s] + cay6[3 * j + s]);
            if (comp6auto->has(needT, need6)) { ok6 = true; break; }
          } else if (comp6.has(need6)) {
            ok6 = true;
            break;
          }
        }
      }
      if (ok6) out.push_back({px, py});
    }
  }
  }, 4);
  std::vector<Profile> out;
  for (auto &p : part) out.insert(out.end(), p.begin(), p.end());
  return out;
}

std::vector<Profile> survive_profiles6(int L, int sigX, int sigY, int n, const NormSet &comp3,
                                       const NormSet &comp6, const AutoSet *comp6auto, bool thm212,
                                       bool thm211b, size_t cap, bool *capped, FILE *log) {
  const int tgt = 4 * n + 2;
  const bool abSide = (L == n + 1);
  const auto PX = enum_class_sums(L, sigX, 6), PY = enum_class_sums(L, sigY, 6);
  std::vector<int> npy(PY.size()), npy3(PY.size()), cay(3 * PY.size());
  for (size_t j = 0; j < PY.size(); j++) {
    npy[j] = norm_vec(PY[j]);
    npy3[j] = norm_vec(reduce63(PY[j]));
    for (int s = 1; s <= 3; s++) cay[3 * j + s - 1] = side_auto(PY[j], s);
  }
  std::vector<std::vector<Profile>> part(64);
  parallel_parts(PX.size(), [&](size_t lo, size_t hi, size_t t) {
    std::vector<Profile> &out = part[t];
    Vec needT(3);
    for (size_t ix = lo; ix < hi && out.size() < cap; ix++) {
      const Vec &px = PX[ix];
      const int npx = norm_vec(px);
      if (npx > tgt) continue;
      const int npx3 = norm_vec(reduce63(px));
      if (npx3 > tgt) continue;
      int cax[3];
      for (int s = 1; s <= 3; s++) cax[s - 1] = side_auto(px, s);
      for (size_t j = 0; j < PY.size(); j++) {
        const auto &py = PY[j];
        const int need = tgt - npx - npy[j];
        if (need < 0 || !comp6.has(need)) continue;
        if (thm212 && !thm212_ok(px, py, 6, n, abSide)) continue;
        const int need3 = tgt - npx3 - npy3[j];
        if (need3 < 0 || !comp3.has(need3)) continue;
        if (thm211b && comp6auto) {
          for (int s = 0; s < 3; s++) needT[s] = -(cax[s] + cay[3 * j + s]);
          if (!comp6auto->has(needT, need)) continue;
        }
        out.push_back({px, py});
      }
    }
  }, 64);
  // the reference stops at the cap-th pair in its loop order: the same first `cap` pairs
  std::vector<Profile> out;
  if (capped) *capped = false;
  for (auto &p : part) {
    for (auto &x : p) {
      out.push_back(std::move(x));
      if (out.size() >= cap) {
        if (log) {
          fprintf(log, "[mod6] WARNING: profile-pair space hit cap %zu — mod-6 PROFILE space itself explodes (Gate-A data)\n", cap);
          fflush(log);
        }
        if (capped) *capped = true;
        return out;
      }
    }
  }
  return out;
}

std::string cell_key(const Vec &px, const Vec &py) {
  std::string k;
  for (int v : px) { k += std::to_string(v); k += ','; }
  k += '|';
  for (int v : py) { k += std::to_string(v); k += ','; }
  return k;
}

uint64_t fnv_str(uint64_t h, const std::string &s) {
  for (unsigned char c : s) { h ^= c; h *= 1099511628211ULL; }
  return h;
}

// ---- the lane's cell list ----------------------------------------------------------------

#define LOGF(...)                    \
  do {                               \
    if (log) {                       \
      fprintf(log, __VA_ARGS__);     \
      fflush(log);                   \
    }                                \
  } while (0)

static long long prof_score(const Profile &p) {
  long long s = 0;
  for (int v : p.px) s += std::abs(v);
  for (int v : p.py) s += std::abs(v);
  return s;
}

typedef unsigned __int128 u128;

// Orders keys as the reference orders its "v,v,...,|v,v,...," strings. All keys of one list
// have the same number of tokens, so string order is token-by-token order, each token being a
// value's decimal text followed by ','. rank[] numbers those tokens in string order, and a key
// packs its 2m ranks, 8 bits each, most significant first.
struct CellKeyOrder {
  uint8_t rank[256];
  int value_of[256];
  CellKeyOrder() {
    std::vector<std::pair<std::string, int>> t;
    for (int v = -128; v < 128; v++) t.push_back({std::to_string(v) + ",", v});
    std::sort(t.begin(), t.end());
    for (int i = 0; i < 256; i++) {
      rank[t[i].second + 128] = (uint8_t)i;
      value_of[i] = t[i].second;
    }
  }
  static const CellKeyOrder &get() {
    static const CellKeyOrder k;
    return k;
  }
  u128 pack(const int *px, const int *py, int m) const {
    u128 k = 0;
    for (int c = 0; c < m; c++) k = (k << 8) | rank[(px[c] + 128) & 255];
    for (int c = 0; c < m; c++) k = (k << 8) | rank[(py[c] + 128) & 255];
    return k;
  }
  std::string str(u128 k, int m) const {
    Vec px(m), py(m);
    for (int c = m - 1; c >= 0; c--) { py[c] = value_of[(int)(k & 255)]; k >>= 8; }
    for (int c = m - 1; c >= 0; c--) { px[c] = value_of[(int)(k & 255)]; k >>= 8; }
    return cell_key(px, py);
  }
};

// class c of a reversed sequence is class (n-1-c) mod m of the original
static inline void rev_classes(const int *p, int *q, int m, int n) {
  for (int c = 0; c < m; c++) q[((n - 1 - c) % m + m) % m] = p[c];
}

// the quad switch Q(C,D) = (U+RV, U-RV), U=(C+D)/2, V=(C-D)/2, on class sums
// (wz_match.cpp:1673-1712; C++ integer division, as there)
static inline void quad_switch(int *px, int *py, int m, int n) {
  int rx[8], ry[8];
  rev_classes(px, rx, m, n);
  rev_classes(py, ry, m, n);
  for (int c = 0; c < m; c++) {
    const int nx = (px[c] + py[c] + rx[c] - ry[c]) / 2;
    const int ny = (px[c] + py[c] - rx[c] + ry[c]) / 2;
    px[c] = nx;
    py[c] = ny;
  }
}

// Smallest key over the orbit of (px, py): negations, reversals, the swap, and with 64
// variants also the quad switch, applied in the order of wz_match.cpp:1721-1730 (variant bit
// 32 the quad switch first, then bits 1 / 2 negate px / py, bits 4 / 8 reverse them, bit 16
// swaps them in the key). A negation or reversal acts on one side only and the two commute,
// so each side's four forms are packed once (one byte per class, as CellKeyOrder::pack packs a
// side) and every variant's key is two packed halves.
static u128 orbit_id(const int *px0, const int *py0, int m, int n, int nvar, const CellKeyOrder &ko) {
  auto halves = [&](const int *v, uint64_t h[4]) {  // [neg | 2 * rev]
    int r[8];
    rev_classes(v, r, m, n);
    for (int f = 0; f < 4; f++) {
      const int *src = (f & 2) ? r : v;
      const int sg = (f & 1) ? -1 : 1;
      uint64_t k = 0;
      for (int c = 0; c < m; c++) k = (k << 8) | ko.rank[(sg * src[c] + 128) & 255];
      h[f] = k;
    }
  };
  u128 best = ~(u128)0;
  int bx[8], by[8];
  for (int c = 0; c < m; c++) { bx[c] = px0[c]; by[c] = py0[c]; }
  for (int base = 0; base < (nvar > 32 ? 2 : 1); base++) {
    if (base) quad_switch(bx, by, m, n);
    uint64_t hx[4], hy[4];
    halves(bx, hx);
    halves(by, hy);
    for (int fx = 0; fx < 4; fx++)
      for (int fy = 0; fy < 4; fy++) {
        const u128 a = ((u128)hx[fx] << (8 * m)) | hy[fy];  // (px, py)
        const u128 b = ((u128)hy[fy] << (8 * m)) | hx[fx];  // swapped
        if (a < best) best = a;
        if (b < best) best = b;
      }
  }
  return best;
}

int build_cell_list(int n, int SA, int SB, int SC, int SD, const ListOptions &opt, CellList &out,
                    FILE *log) {
  const int n1 = n + 1;
  const bool thm211b = opt.thm211b, thm212 = opt.thm212;
  out = CellList();
  NormSet ab3, ab6, cd3, cd6;
  ab3.build(n1, SA, SB, 3, n);
  ab6.build(n1, SA, SB, 6, n);
  cd3.build(n, SC, SD, 3, n);
  cd6.build(n, SC, SD, 6, n);
  AutoSet ab6a, cd6a;
  if (thm211b) {
    ab6a.build(n1, SA, SB, 6, n, thm212);
    cd6a.build(n, SC, SD, 6, n, thm212);
    out.ab_auto = ab6a.keys.size();
    out.cd_auto = cd6a.keys.size();
    LOGF("[thm2.11b] ENABLED — complement (autocorr,norm) tuples: A,B side %zu  C,D side %zu\n",
         ab6a.keys.size(), cd6a.keys.size());
  }
  // wz_match.cpp:1388-1396: both sides' mod-3 survivors are always built and reported
  auto abProfs = survive_profiles3(n1, SA, SB, n, cd3, cd6, thm211b ? &cd6a : nullptr, thm212, thm211b);
  auto cdProfs = survive_profiles3(n, SC, SD, n, ab3, ab6, thm211b ? &ab6a : nullptr, thm212, thm211b);
  out.ab_profiles = abProfs.size();
  out.cd_profiles = cdProfs.size();
  LOGF("[profiles] A,B side surviving: %zu   C,D side surviving: %zu\n", abProfs.size(), cdProfs.size());

  std::vector<Profile> &cells = out.cells;
  if (opt.m6) {
    bool capped = false;
    cells = survive_profiles6(n, SC, SD, n, ab3, ab6, thm211b ? &ab6a : nullptr, thm212, thm211b,
                              20000000, &capped, log);
    LOGF("[firsthit] mod-6 stream source: %zu C,D profile cells (mod-3 atoms exceed walltime at this n)\n",
         cells.size());
    if (cells.size() >= 20000000) {
      LOGF("RESULT: CELL LIST TRUNCATED at the 20M cap — refusing to search an incomplete tile\n");
      return 2;
    }
    if (opt.endpos) {
      // endpoint-parity cell filter, wz_match.cpp:1598-1622
      size_t before = cells.size();
      std::vector<Profile> keep;
      for (size_t i = 0; i < cells.size(); i++) {
        const auto &p = cells[i];
        int s = 0;
        for (int c = 0; c < 6; c++) s += p.px[c] + p.py[c];
        int mid = (n % 2 == 1) ? p.px[(n / 2) % 6] + p.py[(n / 2) % 6] : 0;
        bool ok = (((s - mid) % 4) + 4) % 4 == 0;
        if (opt.endpos_nocell) LOGF("ENDPOS_CELL idx=%zu ok=%d\n", i, ok ? 1 : 0);
        if (ok || opt.endpos_nocell) keep.push_back(p);
      }
      cells.swap(keep);
      LOGF("[endpos] cells %zu -> %zu (endpoint-parity filter%s)\n", before, cells.size(),
           opt.endpos_nocell ? ", NOT applied: test hook" : "");
    }
  } else {
    cells = cdProfs;
  }
  const int m = opt.m6 ? 6 : 3;
  out.m = m;
  // std::sort as the reference calls it: ties keep libstdc++'s introsort order, which the
  // lane's raw cell indices (and so its checkpoints) inherit
  if (opt.prof_order == 1)
    std::sort(cells.begin(), cells.end(),
              [](const Profile &a, const Profile &b) { return prof_score(a) < prof_score(b); });
  else if (opt.prof_order == 2)
    std::sort(cells.begin(), cells.end(),
              [](const Profile &a, const Profile &b) { return prof_score(a) > prof_score(b); });

  // ---- orbit canonicalisation (+ quad switch Q, Q-closure prune), ORDER=3, digests ----
  bool orbit_q = false;
  if (opt.orbit_q) {
    const bool safe = opt.endpos || ((n % 2 == 0) && (((SC + SD) % 4 + 4) % 4 == 0));
    orbit_q = (opt.orbit_q == 2) || (opt.orbit_q == 1 && safe);
    if (opt.orbit_q == 1 && !safe)
      LOGF("[orbitq] DISABLED: needs n even and c+d = 0 mod 4, or WZ_FH_ENDPOS=1 (n=%d c=%d d=%d)\n", n, SC, SD);
    if (opt.orbit_q == 2 && !safe) LOGF("[orbitq] FORCED outside its proven range (test mode only)\n");
  }
  out.orbit_q = orbit_q;
  const int nvar = orbit_q ? 64 : 32;
  out.kept.assign(cells.size(), 1);
  if (!opt.orbit_canon) return 0;

  // Orbit ids are compared as the reference compares its string keys; a key is packed into
  // 128 bits whose integer order is that string order (CellKeyOrder), so the canonicalisation
  // works on integers and builds strings only for the digest and the certificates.
  const CellKeyOrder &ko = CellKeyOrder::get();
  const size_t N = cells.size();
  std::vector<u128> own(N), oid(N);
  parallel_parts(N, [&](size_t lo, size_t hi, size_t) {
    for (size_t i = lo; i < hi; i++) {
      int px[8], py[8];
      for (int c = 0; c < m; c++) { px[c] = cells[i].px[c]; py[c] = cells[i].py[c]; }
      own[i] = ko.pack(px, py, m);
      oid[i] = orbit_id(px, py, m, n, nvar, ko);
    }
  }, 4096);
  // group the cells by orbit; the orbit's representative is its smallest own key
  std::vector<uint32_t> by_orbit(N);
  for (size_t i = 0; i < N; i++) by_orbit[i] = (uint32_t)i;
  parallel_sort(by_orbit, [&](uint32_t x, uint32_t y) {
    if (oid[x] != oid[y]) return oid[x] < oid[y];
    return own[x] < own[y];
  });
  std::vector<uint32_t> gid(N);
  std::vector<u128> rep_own;  // representative own key per orbit
  for (size_t j = 0; j < N; j++) {
    const uint32_t i = by_orbit[j];
    if (j == 0 || oid[i] != oid[by_orbit[j - 1]]) rep_own.push_back(own[i]);
    gid[i] = (uint32_t)(rep_own.size() - 1);
  }
  bool dup_keys = false;
  for (size_t j = 1; j < N; j++)
    if (own[by_orbit[j]] == own[by_orbit[j - 1]]) dup_keys = true;
  std::vector<unsigned char> dead(rep_own.size(), 0);
  size_t ndead = 0;
  if (orbit_q && opt.qprune) {
    if (!opt.m6 || N >= 20000000) {
      LOGF("[qprune] DISABLED (needs mod-6 cells and an untruncated cell list)\n");
    } else {
      // Q-closure orbit elimination, wz_match.cpp:1745-1802
      out.qp_active = true;
      std::vector<u128> S(own);
      parallel_sort(S, [](const u128 &x, const u128 &y) { return x < y; });
      int ccnt[8];
      for (int c = 0; c < m; c++) ccnt[c] = class_count(n, c, m);
      auto realizable = [&](const int *p) {
        for (int c = 0; c < m; c++)
          if (std::abs(p[c]) > ccnt[c] || ((p[c] + ccnt[c]) & 1)) return false;
        return true;
      };
      long long missing = 0, nonreal = 0, eq212 = 0, unknown = 0, nonint = 0;
      std::string cert;
      std::vector<std::string> certs;
      // each cell's verdict on its Q image (0: the image is listed), in parallel; then the
      // counts, dead orbits and certificates in cell order
      enum { Q_LISTED, Q_NONINT, Q_NONREAL, Q_EQ212, Q_UNKNOWN };
      std::vector<unsigned char> qv(N, Q_LISTED);
      parallel_parts(N, [&](size_t lo, size_t hi, size_t) {
        for (size_t i = lo; i < hi; i++) {
          int qx[8], qy[8];
          bool integral = true;
          for (int c = 0; c < m; c++) {
            qx[c] = cells[i].px[c];
            qy[c] = cells[i].py[c];
          }
          for (int c = 0; c < m; c++) {
            int r = ((n - 1 - c) % m + m) % m;
            if ((qx[c] + qy[c] + qx[r] - qy[r]) & 1) integral = false;
          }
          quad_switch(qx, qy, m, n);
          if (integral && std::binary_search(S.begin(), S.end(), ko.pack(qx, qy, m))) continue;
          if (!integral) qv[i] = Q_NONINT;
          else if (!realizable(qx) || !realizable(qy)) qv[i] = Q_NONREAL;
          else if (thm212 && !thm212_ok(Vec(qx, qx + m), Vec(qy, qy + m), m, n, false)) qv[i] = Q_EQ212;
          else qv[i] = Q_UNKNOWN;
        }
      }, 4096);
      for (size_t i = 0; i < N; i++) {
        if (qv[i] == Q_LISTED) continue;
        int qx[8], qy[8];
        for (int c = 0; c < m; c++) {
          qx[c] = cells[i].px[c];
          qy[c] = cells[i].py[c];
        }
        quad_switch(qx, qy, m, n);
        missing++;
        const char *why = nullptr;
        if (qv[i] == Q_NONINT) { nonint++; why = "nonintegral"; }
        else if (qv[i] == Q_NONREAL) { nonreal++; why = "not_realizable"; }
        else if (qv[i] == Q_EQ212) { eq212++; why = "eq2.12"; }
        else { unknown++; continue; }
        if (!dead[gid[i]]) {
          dead[gid[i]] = 1;
          ndead++;
          const std::string okey = ko.str(oid[i], m), mine = cell_key(cells[i].px, cells[i].py);
          const std::string qkey = cell_key(Vec(qx, qx + m), Vec(qy, qy + m));
          certs.push_back(okey + " " + mine + " " + qkey + " " + why);
          if (cert.find(why) == std::string::npos)
            cert += std::string(" ") + why + ":" + mine + "->" + qkey;
        }
      }
      long long removed = 0;
      for (size_t i = 0; i < N; i++) removed += dead[gid[i]];
      if (opt.qprune_dump) {
        if (FILE *df = fopen(opt.qprune_dump, "w")) {
          for (size_t i = 0; i < N; i++)
            if (dead[gid[i]]) fprintf(df, "%zu\n", i);
          fclose(df);
        }
        if (FILE *cf = fopen((std::string(opt.qprune_dump) + ".certs").c_str(), "w")) {
          for (auto &c : certs) fprintf(cf, "%s\n", c.c_str());
          fclose(cf);
        }
      }
      LOGF("[qprune] missing_Q_images=%lld not_realizable=%lld eq212=%lld nonintegral=%lld unknown=%lld dead_orbits=%zu cells_removed=%lld\n[qprune] certificates:%s\n",
           missing, nonreal, eq212, nonint, unknown, ndead, removed, cert.c_str());
    }
  }
  // kept: the orbit's representative, unless the orbit is dead. Raw keys are distinct by
  // construction, so kept cells and kept keys (the reference's keep set) count alike.
  size_t nkept = 0;
  for (size_t i = 0; i < N; i++) {
    out.kept[i] = (own[i] == rep_own[gid[i]] && !dead[gid[i]]) ? 1 : 0;
    nkept += out.kept[i];
  }
  LOGF("[orbitcanon]%s cells=%zu kept_orbits=%zu dedup=%gx\n", orbit_q ? " group=64" : "", N, nkept,
       (double)N / std::max((size_t)1, nkept));
  if (opt.prof_order != 3) return 0;

  // deterministic order: (orbit-min profile score, orbit id, own key), wz_match.cpp:1816-1881
  std::vector<long long> omin(rep_own.size(), -1);
  for (size_t i = 0; i < N; i++) {
    const long long sc = prof_score(cells[i]);
    if (omin[gid[i]] < 0 || sc < omin[gid[i]]) omin[gid[i]] = sc;
  }
  std::vector<uint32_t> perm(by_orbit);  // already in (orbit id, own key) order
  std::stable_sort(perm.begin(), perm.end(),
                   [&](uint32_t x, uint32_t y) { return omin[gid[x]] < omin[gid[y]]; });
  {
    std::vector<Profile> sorted(N);
    std::vector<unsigned char> skept(N);
    for (size_t j = 0; j < N; j++) {
      sorted[j] = std::move(cells[perm[j]]);
      skept[j] = out.kept[perm[j]];
    }
    cells.swap(sorted);
    out.kept.swap(skept);
  }
  // the list digest hashes every cell key in list order: the keys of contiguous parts are
  // formed on all host threads, then hashed one part after the other
  std::vector<std::string> keys_of(64);
  parallel_parts(N, [&](size_t lo, size_t hi, size_t t) {
    std::string &k = keys_of[t];
    for (size_t i = lo; i < hi; i++) k += cell_key(cells[i].px, cells[i].py);
  }, 4096);
  uint64_t dl = 1469598103934665603ULL, dk = 1469598103934665603ULL;
  for (const std::string &k : keys_of) dl = fnv_str(dl, k);
  long long kept_n = 0;
  for (size_t i = 0; i < N; i++) {
    kept_n += out.kept[i];
    dk = fnv_str(dk, out.kept[i] ? "1" : "0");
  }
  if (dup_keys) {
    size_t uniq = 0;
    for (size_t j = 0; j < N; j++)
      if (j == 0 || own[by_orbit[j]] != own[by_orbit[j - 1]]) uniq++;
    LOGF("RESULT: DUPLICATE CELL KEYS in the raw list (%zu) — refusing\n", N - uniq);
    return 2;
  }
  char dbuf[64];
  snprintf(dbuf, sizeof dbuf, "%016llx:%016llx", (unsigned long long)dl, (unsigned long long)dk);
  out.digest = dbuf;
  const int ns = std::max(1, opt.nshard);
  std::vector<long long> per_arm(ns, 0);
  for (size_t i = 0; i < N; i++)
    if (out.kept[i]) per_arm[i % ns]++;
  long long arm_min = *std::min_element(per_arm.begin(), per_arm.end());
  long long arm_max = *std::max_element(per_arm.begin(), per_arm.end());
  LOGF("[order] ord3 cells=%zu kept=%lld windows=%zu digest=%s arms=%d kept_per_arm_min=%lld max=%lld\n",
       N, kept_n, (N + ns - 1) / ns, dbuf, ns, arm_min, arm_max);
  return 0;
}

uint64_t AbpRows::cell_key_of(const Profile &p, int n, int m) {
  const int need = 4 * n + 2 - norm_vec(p.px) - norm_vec(p.py);
  const int hm = m / 2;
  Vec T(hm);
  for (int s = 1; s <= hm; s++) T[s - 1] = -pair_auto(p.px, p.py, s);
  return auto_key(T, need);
}

void AbpRows::build(const std::vector<uint64_t> &keys, int n, int sigA, int sigB, int m) {
  for (uint64_t k : keys) by_key.emplace(k, std::vector<int8_t>());
  const int hm = m / 2, n1 = n + 1, tgt = 4 * n + 2;
  struct Tup { Vec v; int norm; Vec ca; };
  auto tups = [&](int sig) {
    std::vector<Tup> out;
    for (int sgn = 1; sgn >= (sig ? -1 : 1); sgn -= 2)
      for (auto &v : enum_class_sums(n1, sgn * sig, m)) {
        Tup t;
        t.v = v;
        t.norm = norm_vec(v);
        if (t.norm > tgt) continue;
        t.ca.assign(hm, 0);
        for (int s = 1; s <= hm; s++) t.ca[s - 1] = autocorr_vec(v, s) + autocorr_vec(v, m - s);
        out.push_back(std::move(t));
      }
    return out;
  };
  const auto Kt = tups(sigA), Rt = tups(sigB);
  nK = Kt.size();
  nR = Rt.size();
  // The reference pairs every (k, r) tuple and keeps the pair when auto_key(k.ca + r.ca,
  // k.norm + r.norm) is a wanted key. auto_key packs the norm and each residue into its own
  // 16-bit field, so it is one-to-one on these values: for a given k and wanted key (need, T)
  // the pair matches exactly when r has norm need - k.norm and residues T - k.ca. So the r
  // tuples are indexed by auto_key(r.ca, r.norm), and each k looks up, per wanted key, the r
  // that complete it (in r order, so every key's rows come out in the reference's order).
  std::unordered_map<uint64_t, std::vector<int>> r_of;
  for (int j = 0; j < (int)Rt.size(); j++) r_of[auto_key(Rt[j].ca, Rt[j].norm)].push_back(j);
  struct Want { uint64_t key; int need; Vec T; std::vector<int8_t> *out; };
  std::vector<Want> wants;
  for (auto &kv : by_key) {
    Want w;
    w.key = kv.first;
    w.need = (int)(kv.first & 0xFFFF);
    w.T.assign(hm, 0);
    for (int i = 0; i < hm && i < 3; i++) w.T[i] = (int)((kv.first >> (16 * (i + 1))) & 0xFFFF) - 8192;
    w.out = &kv.second;
    wants.push_back(std::move(w));
  }
  Vec need_ca(hm);
  for (const auto &kt : Kt)
    for (const auto &w : wants) {
      if (w.need > tgt) continue;  // every pair's norm sum is above the target
      for (int s = 0; s < hm; s++) need_ca[s] = w.T[s] - kt.ca[s];
      auto it = r_of.find(auto_key(need_ca, w.need - kt.norm));
      if (it == r_of.end()) continue;
      for (int j : it->second) {
        const auto &rt = Rt[j];
        // the key fields are exact, but check the sums themselves all the same
        bool same = rt.norm + kt.norm == w.need;
        for (int s = 0; s < hm && same; s++) same = kt.ca[s] + rt.ca[s] == w.T[s];
        if (!same) continue;
        if (!thm212_ok(kt.v, rt.v, m, n, true)) continue;
        int8_t row[16] = {0};
        for (int c = 0; c < m; c++) {
          row[c] = (int8_t)kt.v[c];
          row[8 + c] = (int8_t)rt.v[c];
        }
        w.out->insert(w.out->end(), row, row + 16);
        rows++;
        max_list = std::max(max_list, w.out->size() / 16);
      }
    }
}

}  // namespace bsfh
