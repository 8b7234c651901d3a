// celllist.cpp - residue-class cell algebra of the first-hit lane (host side).
// Each function states the reference lines (src/solver/wz_match.cpp) whose result it
// reproduces; the enumeration orders are part of the lane's contract (raw cell indices,
// digests and checkpoints depend on them).
#include "celllist.h"

#include <algorithm>
#include <cstdio>

namespace bsfh {

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

void NormSet::build(int L, int a, int b, int m, int n) {
  const auto K = enum_class_sums(L, a, m), R = enum_class_sums(L, b, m);
  const int tgt = 4 * n + 2;
  std::vector<int> rn(R.size());
  for (size_t j = 0; j < R.size(); j++) rn[j] = norm_vec(R[j]);
  for (const auto &kv : K) {
    const int kn = norm_vec(kv);
    if (kn > tgt) continue;
    for (int r : rn)
      if (kn + r <= tgt) vals.insert(kn + r);
  }
}

void AutoSet::build(int L, int a, int b, int m, int n, bool thm212) {
  const auto K = enum_class_sums(L, a, m), R = enum_class_sums(L, b, m);
  const int tgt = 4 * n + 2, half = m / 2;
  const bool abSide = (L == n + 1);
  Vec T(half);
  for (const auto &kv : K) {
    const int kn = norm_vec(kv);
    if (kn > tgt) continue;
    for (const auto &rv : R) {
      const int rn = norm_vec(rv);
      if (kn + rn > tgt) continue;
      if (thm212 && !thm212_ok(kv, rv, m, n, abSide)) continue;
      for (int s = 1; s <= half; s++) T[s - 1] = pair_auto(kv, rv, s);
      keys.insert(auto_key(T, kn + rn));
    }
  }
}

static Vec reduce63(const Vec &v6) { return Vec{v6[0] + v6[3], v6[1] + v6[4], v6[2] + v6[5]}; }

std::vector<Profile> survive_profiles3(int L, int sigX, int sigY, int n, const NormSet &comp3,
                                       const NormSet &comp6, const AutoSet *comp6auto, bool thm212,
                                       bool thm211b) {
  const int tgt = 4 * n + 2;
  const bool abSide = (L == n + 1);
  const auto PX3 = enum_class_sums(L, sigX, 3), PY3 = enum_class_sums(L, sigY, 3);
  const auto PX6 = enum_class_sums(L, sigX, 6), PY6 = enum_class_sums(L, sigY, 6);
  std::vector<Vec> PX6r(PX6.size()), PY6r(PY6.size());
  for (size_t i = 0; i < PX6.size(); i++) PX6r[i] = reduce63(PX6[i]);
  for (size_t i = 0; i < PY6.size(); i++) PY6r[i] = reduce63(PY6[i]);
  std::vector<Profile> out;
  for (const auto &px : PX3) {
    const int npx = norm_vec(px);
    if (npx > tgt) continue;
    for (const auto &py : PY3) {
      const int need = tgt - npx - norm_vec(py);
      if (need < 0 || !comp3.has(need)) continue;
      if (thm212 && !thm212_ok(px, py, 3, n, abSide)) continue;
      bool ok6 = false;
      for (size_t i = 0; i < PX6.size() && !ok6; i++) {
        if (PX6r[i] != px) continue;
        const int npx6 = norm_vec(PX6[i]);
        if (npx6 > tgt) continue;
        for (size_t j = 0; j < PY6.size(); j++) {
          if (PY6r[j] != py) continue;
          const int need6 = tgt - npx6 - norm_vec(PY6[j]);
          if (need6 < 0) continue;
          if (thm212 && !thm212_ok(PX6[i], PY6[j], 6, n, abSide)) continue;
          if (thm211b && comp6auto) {
            Vec needT(3);
            for (int s = 1; s <= 3; s++) needT[s - 1] = -pair_auto(PX6[i], PY6[j], s);
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
  return out;
}

std::vector<Profile> survive_profiles6(int L, int sigX, int sigY, int n, const NormSet &comp3,
                                       const NormSet &comp6, const AutoSet *comp6auto, bool thm212,
                                       bool thm211b, size_t cap, bool *capped) {
  const int tgt = 4 * n + 2;
  const bool abSide = (L == n + 1);
  const auto PX = enum_class_sums(L, sigX, 6), PY = enum_class_sums(L, sigY, 6);
  std::vector<int> npy(PY.size()), npy3(PY.size());
  for (size_t j = 0; j < PY.size(); j++) {
    npy[j] = norm_vec(PY[j]);
    npy3[j] = norm_vec(reduce63(PY[j]));
  }
  std::vector<Profile> out;
  if (capped) *capped = false;
  for (const auto &px : PX) {
    const int npx = norm_vec(px);
    if (npx > tgt) continue;
    const int npx3 = norm_vec(reduce63(px));
    if (npx3 > tgt) continue;
    for (size_t j = 0; j < PY.size(); j++) {
      const auto &py = PY[j];
      const int need = tgt - npx - npy[j];
      if (need < 0 || !comp6.has(need)) continue;
      if (thm212 && !thm212_ok(px, py, 6, n, abSide)) continue;
      const int need3 = tgt - npx3 - npy3[j];
      if (need3 < 0 || !comp3.has(need3)) continue;
      if (thm211b && comp6auto) {
        Vec needT(3);
        for (int s = 1; s <= 3; s++) needT[s - 1] = -pair_auto(px, py, s);
        if (!comp6auto->has(needT, need)) continue;
      }
      out.push_back({px, py});
      if (out.size() >= cap) {
        printf("[mod6] WARNING: profile-pair space hit cap %zu — mod-6 PROFILE space itself explodes (Gate-A data)\n", cap);
        fflush(stdout);
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
  struct Tup { Vec v; int norm; int ca[3]; };
  auto tups = [&](int sig) {
    std::vector<Tup> out;
    for (int sgn = 1; sgn >= (sig ? -1 : 1); sgn -= 2)
      for (auto &v : enum_class_sums(n1, sgn * sig, m)) {
        Tup t;
        t.v = v;
        t.norm = norm_vec(v);
        if (t.norm > tgt) continue;
        for (int s = 1; s <= hm; s++) t.ca[s - 1] = autocorr_vec(v, s) + autocorr_vec(v, m - s);
        out.push_back(std::move(t));
      }
    return out;
  };
  const auto Kt = tups(sigA), Rt = tups(sigB);
  nK = Kt.size();
  nR = Rt.size();
  Vec Tsum(hm);
  for (const auto &kt : Kt)
    for (const auto &rt : Rt) {
      const int nn2 = kt.norm + rt.norm;
      if (nn2 > tgt) continue;
      for (int s = 0; s < hm; s++) Tsum[s] = kt.ca[s] + rt.ca[s];
      auto it = by_key.find(auto_key(Tsum, nn2));
      if (it == by_key.end()) continue;
      if (!thm212_ok(kt.v, rt.v, m, n, true)) continue;
      int8_t row[16] = {0};
      for (int c = 0; c < m; c++) {
        row[c] = (int8_t)kt.v[c];
        row[8 + c] = (int8_t)rt.v[c];
      }
      it->second.insert(it->second.end(), row, row + 16);
      rows++;
      max_list = std::max(max_list, it->second.size() / 16);
    }
}

}  // namespace bsfh
