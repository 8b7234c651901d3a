/*
 * bs_oracle.h - CPU oracle for the first-hit search path of base sequences BS(n+1,n).
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference solver's
 * hot-path algorithms (src/solver/wz_match.cpp in DanielGord0n/BS45_Quantum_Explorer).
 * It exists to check the CUDA product path: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it. Nothing in the product links or calls it.
 *
 * Parity pin: every function here is checked against the reference itself, compiled
 * from its own sources into oracle/_ref/ by oracle/Makefile (target `ref`), through the
 * golden fixtures under tests/golden/ (see tests/golden/make_golden.py).
 *
 * Sequences are int8 arrays of +1/-1. All functions are reentrant unless noted.
 */
#ifndef BS_ORACLE_H
#define BS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Hall DFT tables, wz_match.cpp:104-114: cos/sin(i * (j*pi/100)) for j=1..200, i<n+1.
 * Layout: tab[j*(n+1) + i], rows j=0..200 (row 0 unused, zero). */
void or_hall_tables(int n, double *cos_tab, double *sin_tab);

/* Thm 2.4 pair decision, identical to hall_ok_pair_fast / hall_ok_single(X) &&
 * hall_ok_single(Y) && hall_ok(X,Y) (wz_match.cpp:117-181). Returns 1 = pass.
 * If max_pair is non-null it receives max_j (fx+fy) over all 200 angles (no early exit),
 * and min_margin the smallest |value - limit| over all three tests and angles. */
int or_hall_pair(int n, const int8_t *X, const int8_t *Y, int L,
                 const double *cos_tab, const double *sin_tab,
                 double *max_pair, double *min_margin);

/* Batch form over npairs pairs laid out [pair][X(L) | Y(L)]; pass[i] = 0/1.
 * nthreads > 1 uses POSIX threads (the CPU baseline). Returns the smallest margin seen. */
double or_hall_batch(int n, int L, const int8_t *XY, long long npairs, uint8_t *pass,
                     int nthreads);

/* Exact NPAF at shift s, wz_match.cpp:184-192. */
int or_npaf_at(const int8_t *A, const int8_t *B, int n1, const int8_t *C, const int8_t *D,
               int n2, int s);

/* Flatness score sum_{s=1..n} |N_C(s)+N_D(s)|, wz_match.cpp:2569-2583. */
long long or_flat_score(const int8_t *C, const int8_t *D, int n);

/* FNV-1a autocorrelation key, wz_match.cpp:855-871. */
uint64_t or_autocorr_key(const int8_t *X, const int8_t *Y, int L, int n, int negate);

/* ---- C,D mirror-quad stream, count_pairs22 semantics (wz_match.cpp:678-784) ----
 * Emits leaves in DFS order. A leaf is a class-exact (X,Y); its Hall decision is
 * recorded. When keep_all is 0 only passing leaves are written. out_xy receives rows of
 * 2L int8 (X then Y); out_pass (may be null) the decision; at most cap rows are written,
 * the return value is the number of rows the full stream would write. */
typedef struct { long long nodes, leaves, ok; } or_stream_stats;
long long or_cd_stream(int n, int L, int m, const int *tx, const int *ty,
                       int pinX, int pinY, int rev, int endpos, int cd_prune,
                       int keep_all, int8_t *out_xy, uint8_t *out_pass, long long cap,
                       or_stream_stats *st);

/* ---- A,B completion, fh_complete_ab semantics (wz_match.cpp:1298-1341) ----
 * rows: nrows records of 16 int8 (k[8] then r[8]) = the cell's allowed A,B class-sum rows
 * (AbpRow, wz_match.cpp:970); rows == NULL runs unconstrained. m is the class modulus.
 * Returns the verdict 0 hit / 1 prefilter / 2 clean no / 3 budget abort / 4 internal
 * error; *nodes receives the charged node count (fh_nodes_total delta). On a hit A,B
 * (length n+1) are written. */
int or_complete_ab(int n, int sigA, int sigB, const int8_t *C, const int8_t *D,
                   long long budget, int outer_k, int early, int canon, int m,
                   const int8_t *rows, int nrows, int8_t *A, int8_t *B, long long *nodes);
/* The same with WZ_FH_A2 (0 off, 2 the A2 row-reachability prune, wz_match.cpp:977-1047). */
int or_complete_ab_a2(int n, int sigA, int sigB, const int8_t *C, const int8_t *D,
                      long long budget, int outer_k, int early, int canon, int m,
                      const int8_t *rows, int nrows, int a2, int8_t *A, int8_t *B, long long *nodes);

/* Hall microbench input generator (per-pair deterministic; the same definition as the
 * product's device generator): words[2p], words[2p+1] = C, D of pair p. */
void or_gen_hall_pairs(int n, long long npairs, uint64_t seed, uint64_t *words, int nthreads);

/* Outer-lag table dump for cross-checking (OUTER2 16*5*9, OUTER3 128*5*9*13 bytes). */
void or_outer_tables(uint8_t *outer2, uint8_t *outer3);

#ifdef __cplusplus
}
#endif
#endif
