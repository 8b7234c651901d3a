// ref_harness.cpp - exposes the reference solver's own hot-path functions through a C ABI
// so the oracle restatement (bs_oracle.c) can be pinned against them.
//
// TEST INFRASTRUCTURE ONLY. This file contains no reference code: it #includes the
// read-only reference source at build time (path given by -DWZ_MATCH_SRC, main renamed by
// -Dmain=ref_main) and calls its functions. Built by `make -C oracle ref` into oracle/_ref/,
// which is never committed. The GPU host never builds it (the reference is not there).
#include WZ_MATCH_SRC

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

void refh_outer_tables(unsigned char *o2, unsigned char *o3) {
  memcpy(o2, OUTER2, sizeof OUTER2);
  memcpy(o3, OUTER3, sizeof OUTER3);
}

}  // extern "C"
