// ref_harness.cpp - exposes the reference solver's own hot-path functions through a C ABI
// so the oracle restatement (bs_oracle.c) can be pinned against them.
//
// TEST INFRASTRUCTURE ONLY. This file contains no reference code: it #includes the
// read-only reference source at build time (path given by -DWZ_MATCH_SRC, main renamed by
// -Dmain=ref_main) and calls its functions. Built by `make -C oracle ref REF=<root>` into
// oracle/_ref/, which is never committed; bench.py's reference arm times the functions below
// the "timed baselines" line.
#include WZ_MATCH_SRC

#include <thread>

extern "C" {

// Global set-up that wz_match.cpp's main performs before the FIRSTHIT block
// (wz_match.cpp:1355-1391, 1553).
void refh_setup(int n, int a, int b, int c, int d, int outer_k) {
  G_N = n; G_N1 = n + 1;
  G_SIG_A = a; G_SIG_B = b; G_SIG_C = c; G_SIG_D = d;
  hall_order_init();
  init_hall_tables();
  G_OUTER_K = outer_k;
  init_p22();
}

int refh_hall_fast(const int *X, const int *Y, int L) { return hall_ok_pair_fast(X, L, Y, L) ? 1 : 0; }

int refh_hall_conj(const int *X, const int *Y, int L) {
  return (hall_ok_single(X, L) && hall_ok_single(Y, L) && hall_ok(X, L, Y, L)) ? 1 : 0;
}

double refh_hall_table(int j, int i, int sin_part) { return sin_part ? G_HALL_SIN[j][i] : G_HALL_COS[j][i]; }

int refh_npaf(const int *A, const int *B, int n1, const int *C, const int *D, int n2, int s) {
  return npaf_at(A, B, n1, C, D, n2, s);
}

unsigned long long refh_autocorr_key(const int *X, const int *Y, int L, int negate) {
  return autocorr_key(X, Y, L, negate != 0);
}

// count_pairs22 with a sink that records every surviving (X,Y) in stream order.
long long refh_stream(int L, const int *tx, const int *ty, int m, int pinX, int pinY, int rev,
                      int endpos, int cd_prune, int hall_fast, int *out, long long cap,
                      long long *nodes, long long *leaves, long long *ok) {
  const bool abSide = (L == G_N1);  // the A,B side is the one of length n+1
  G_STREAM_REV = rev != 0;
  G_ENDPOS = endpos != 0;
  G_CD_PRUNE = cd_prune;
  G_HALL_FAST = hall_fast;
  vector<int> vx(tx, tx + m), vy(ty, ty + m);
  long long written = 0;
  function<void(const vector<int> &, const vector<int> &)> sink =
      [&](const vector<int> &X, const vector<int> &Y) {
        if (written < cap) {
          for (int i = 0; i < L; i++) out[written * 2 * L + i] = X[i];
          for (int i = 0; i < L; i++) out[written * 2 * L + L + i] = Y[i];
        }
        written++;
      };
  long long lv = 0, okc = 0;
  unsigned long long n0 = G_CD_NODES;
  count_pairs22(L, vx, vy, abSide, pinX != 0, pinY != 0, lv, okc, &sink, m, nullptr);
  *nodes = (long long)(G_CD_NODES - n0);
  *leaves = lv;
  *ok = okc;
  return written;
}

// fh_complete_ab on one C,D with an optional allowed-row list (AbpRow k[8], r[8]).
static vector<AbpRow> g_rows;
int refh_complete(const int *C, const int *D, long long budget, int m, const signed char *rows,
                  int nrows, int *Aout, int *Bout, long long *nodes) {
  FH_BUDGET = budget;
  FH_ABP_M = m;
  for (int c = 0; c < m; c++) FH_ABP_TIC[c] = class_count(G_N1, c, m);
  FH_ABP = nullptr;
  if (rows && nrows > 0) {
    g_rows.assign(nrows, AbpRow{});
    for (int r = 0; r < nrows; r++)
      for (int c = 0; c < 8; c++) { g_rows[r].k[c] = rows[16 * r + c]; g_rows[r].r[c] = rows[16 * r + 8 + c]; }
    FH_ABP = &g_rows;
    FH_ABP_STACK.assign(G_N1 / 2 + 2, {});
    FH_ABP_STACK[0].resize(nrows);
    for (int r = 0; r < nrows; r++) FH_ABP_STACK[0][r] = r;
  }
  long long nb = fh_nodes_total;
  int v = fh_complete_ab(C, D);
  *nodes = fh_nodes_total - nb;
  if (v == 0) {
    for (int i = 0; i < G_N1; i++) { Aout[i] = g_solA[i]; Bout[i] = g_solB[i]; }
  }
  FH_ABP = nullptr;
  return v;
}

// ---- timed baselines (bench.py's reference arm) ----
// Each library instance is one arm: the reference keeps its state in globals, so a caller
// that wants several arms in one process loads several copies of this library.

static void unpack_word(unsigned long long w, int L, int *out) {
  for (int i = 0; i < L; i++) out[i] = ((w >> i) & 1ULL) ? 1 : -1;
}

// Hall decisions of the packed pairs [lo, hi) (two words per pair, bit i set <=> +1).
// fast != 0: the reference's default predicate hall_ok_pair_fast (wz_match.cpp:143-168) on
// this instance's adaptive angle order, single-threaded (it re-sorts a global order, so it
// is one arm's predicate). fast == 0: the WZ_FH_HALL_FAST=0 conjunction
// hall_ok_single(X) && hall_ok_single(Y) && hall_ok(X, Y) (wz_match.cpp:773-775) over
// nthreads OpenMP threads. Returns the number of passing pairs; out (may be NULL) gets 0/1.
long long refh_hall_batch(const unsigned long long *words, long long lo, long long hi, int L,
                          int fast, int nthreads, unsigned char *out) {
  long long passed = 0;
  if (fast) {
    int X[256], Y[256];
    for (long long p = lo; p < hi; p++) {
      unpack_word(words[2 * p], L, X);
      unpack_word(words[2 * p + 1], L, Y);
      const bool ok = hall_ok_pair_fast(X, L, Y, L);
      passed += ok;
      if (out) out[p] = ok;
    }
    return passed;
  }
#pragma omp parallel for schedule(static, 4096) num_threads(nthreads) reduction(+ : passed)
  for (long long p = lo; p < hi; p++) {
    int X[256], Y[256];
    unpack_word(words[2 * p], L, X);
    unpack_word(words[2 * p + 1], L, Y);
    const bool ok = hall_ok_single(X, L) && hall_ok_single(Y, L) && hall_ok(X, L, Y, L);
    passed += ok;
    if (out) out[p] = ok;
  }
  return passed;
}

// count_pairs22 on one C,D cell (the arm's stream, hall_ok_pair_fast at the leaves) for at
// most `seconds` of wall time, through the reference's own cooperative stop flag. Returns
// the survivors; nodes/leaves/ok are the cell's counts so far.
long long refh_stream_for(int L, const int *tx, const int *ty, int m, int pinX, int pinY,
                          double seconds, long long *nodes, long long *leaves, long long *ok) {
  G_STREAM_REV = false;
  G_ENDPOS = false;
  G_CD_PRUNE = 0;
  G_HALL_FAST = 1;
  vector<int> vx(tx, tx + m), vy(ty, ty + m);
  atomic<bool> stop(false), done(false);
  std::thread timer([&] {
    const auto t_end = chrono::steady_clock::now() + chrono::duration<double>(seconds);
    while (!done.load() && chrono::steady_clock::now() < t_end)
      std::this_thread::sleep_for(chrono::milliseconds(2));
    stop.store(true);
  });
  long long written = 0;
  function<void(const vector<int> &, const vector<int> &)> sink =
      [&](const vector<int> &, const vector<int> &) { written++; };
  long long lv = 0, okc = 0;
  unsigned long long n0 = G_CD_NODES;
  count_pairs22(L, vx, vy, false, pinX != 0, pinY != 0, lv, okc, &sink, m, &stop);
  done.store(true);
  timer.join();
  *nodes = (long long)(G_CD_NODES - n0);
  *leaves = lv;
  *ok = okc;
  return written;
}

// WZ_FH_A2 mode for later refh_complete calls, with the block tables of modulus m
// (init_a2_tables, as wz_match.cpp's lane does before its first-hit loop).
void refh_set_a2(int mode, int m) {
  G_A2 = mode;
  init_a2_tables(G_N1, m);
}

void refh_outer_tables(unsigned char *o2, unsigned char *o3) {
  memcpy(o2, OUTER2, sizeof OUTER2);
  memcpy(o3, OUTER3, sizeof OUTER3);
}

}  // extern "C"
