// celllist.h - residue-class cell algebra of the first-hit lane (host side).
//
// The C,D side of a base sequence is searched one "cell" at a time: a cell fixes the
// class sums of C and D modulo m (m = 3 or 6). These functions build the cell list the way
// the reference's WZ_FIRSTHIT lane does (src/solver/wz_match.cpp): enumeration of class-sum
// vectors, the Thm 2.3 norm (2.11a), residue-autocorrelation (2.11b) and mod-4 (2.12)
// feasibility of the complementary A,B side, and the allowed A,B rows of a cell.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace bsfh {

using Vec = std::vector<int>;

struct Profile {
  Vec px, py;
};

// Number of positions p < L with p % m == c.
int class_count(int L, int c, int m);

// Every m-vector of class sums of a +-1 sequence of length L whose entries total `target`,
// in the reference's enumeration order (classes 0..m-2 ascending from -count, the last
// class determined): wz_match.cpp:203-224.
std::vector<Vec> enum_class_sums(int L, int target, int m);

int norm_vec(const Vec &v);
// Non-circular autocorrelation of a class-sum vector at shift s (eq 2.9).
int autocorr_vec(const Vec &v, int s);
// One side's 2.11b aggregate at shift s (wz_match.cpp:277-281).
int pair_auto(const Vec &x, const Vec &y, int s);
// (T_1..T_3, norm) packed as the reference packs it (wz_match.cpp:284-289).
uint64_t auto_key(const Vec &T, int norm);
// Thm 2.3 eq (18), the mod-4 conditions (wz_match.cpp:302-322).
bool thm212_ok(const Vec &x, const Vec &y, int m, int n, bool abSide);

// Achievable norm(K)+norm(R) of one side (2.11a), wz_match.cpp:233-249.
struct NormSet {
  std::vector<char> vals;  // vals[v] != 0: v is achievable (0 <= v <= 4n+2)
  void build(int L, int a, int b, int m, int n);
  bool has(int need) const { return need >= 0 && (size_t)need < vals.size() && vals[need]; }
};

// Achievable (2.11b tuple, norm) keys of one side, wz_match.cpp:324-350.
struct AutoSet {
  std::unordered_set<uint64_t> keys;
  void build(int L, int a, int b, int m, int n, bool thm212);
  bool has(const Vec &needT, int need) const { return keys.count(auto_key(needT, need)) != 0; }
};

// mod-3 profile pairs with the mod-6 existential tighten (wz_match.cpp:439-487).
std::vector<Profile> survive_profiles3(int L, int sigX, int sigY, int n, const NormSet &comp3,
                                       const NormSet &comp6, const AutoSet *comp6auto, bool thm212,
                                       bool thm211b);
// mod-6 profile pairs (wz_match.cpp:792-837); *capped is set when the cap was reached.
std::vector<Profile> survive_profiles6(int L, int sigX, int sigY, int n, const NormSet &comp3,
                                       const NormSet &comp6, const AutoSet *comp6auto, bool thm212,
                                       bool thm211b, size_t cap, bool *capped, FILE *log = stdout);

// "v,v,...,|v,v,...," cell key (wz_match.cpp:1665-1671).
std::string cell_key(const Vec &px, const Vec &py);

// 64-bit FNV-1a over a string's bytes, continuing from h.
uint64_t fnv_str(uint64_t h, const std::string &s);

// ---- the lane's cell list ----------------------------------------------------------------
// Options of the first-hit lane that shape the C,D cell list (the reference's WZ_FH_M6,
// WZ_THM211B, WZ_THM212, WZ_FH_ENDPOS, WZ_FH_ORBIT_CANON, WZ_FH_ORBIT_Q,
// WZ_FH_ORBIT_QPRUNE, WZ_FH_PROF_ORDER).
struct ListOptions {
  bool m6 = false, thm211b = false, thm212 = false;
  bool endpos = false, endpos_nocell = false;
  bool orbit_canon = false;
  int orbit_q = 0;         // 0 off, 1 on where proven safe, 2 forced (tests)
  bool qprune = false;
  int prof_order = 0;      // 0 natural, 1 flat first, 2 reverse, 3 orbit-deterministic
  int nshard = 1;          // for the [order] per-arm balance line
  const char *qprune_dump = nullptr;
};

struct CellList {
  int m = 6;
  std::vector<Profile> cells;          // in the lane's final order (raw index = position)
  std::vector<unsigned char> kept;     // 1: the cell is its orbit's representative (canon)
  std::string digest;                  // "<list>:<kept>" under ORDER=3, else empty
  bool orbit_q = false, qp_active = false;
  size_t ab_profiles = 0, cd_profiles = 0, ab_auto = 0, cd_auto = 0;
};

// Builds the list exactly as the reference's first-hit block does (wz_match.cpp:1388-1886),
// printing the same bracketed lines to `log` when it is non-null. Returns 0, or 2 where the
// reference refuses (truncated list, duplicate keys, ORDER=3 without canon).
int build_cell_list(int n, int a, int b, int c, int d, const ListOptions &opt, CellList &out,
                    FILE *log);

// Allowed A,B class-sum rows keyed by the cell invariant (need, needT): the reference's
// abpMap (wz_match.cpp:2318-2378). A row is k[8] then r[8] (int8).
struct AbpRows {
  std::unordered_map<uint64_t, std::vector<int8_t>> by_key;  // 16 bytes per row
  long long rows = 0;
  size_t max_list = 0;
  size_t nK = 0, nR = 0;
  static uint64_t cell_key_of(const Profile &p, int n, int m);
  // keys: the invariants of the cells that will be searched; rows are only kept for them
  void build(const std::vector<uint64_t> &keys, int n, int sigA, int sigB, int m);
};

}  // namespace bsfh
