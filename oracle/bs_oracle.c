/*
 * bs_oracle.c - CPU oracle (test infrastructure only) for the first-hit search path.
 *
 * A restatement, in plain C, of the reference's algorithms in
 * src/solver/wz_match.cpp (DanielGord0n/BS45_Quantum_Explorer). Each function cites the
 * lines it follows. Compiled with -ffp-contract=off so that every double expression is
 * evaluated in the reference's written order with one rounding per operation.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this file's
 * library; the product never does.
 */
#include "bs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------------------ */
/* Hall spectral test (Thm 2.4)                                                          */
/* ------------------------------------------------------------------------------------ */

/* wz_match.cpp:106-114: th = j*pi/100, table = cos(i*th), sin(i*th), for i < n+1. */
void or_hall_tables(int n, double *ct, double *st) {
  int w = n + 1;
  memset(ct, 0, sizeof(double) * 201 * (size_t)w);
  memset(st, 0, sizeof(double) * 201 * (size_t)w);
  for (int j = 1; j <= 200; j++) {
    double th = j * M_PI / 100.0;
    for (int i = 0; i < w && i < 256; i++) {
      ct[j * w + i] = cos(i * th);
      st[j * w + i] = sin(i * th);
    }
  }
}

/* Angles 1..200 in a spread order: repeated halving of the range, so that neighbouring
 * (nearly equal) tests come late and a rejected pair is usually found within a few angles. */
static int HALL_ORDER[200];
static pthread_once_t hall_order_once = PTHREAD_ONCE_INIT;
static void build_hall_order(void) {
  int seen[201] = {0}, k = 0;
  for (int step = 128; step >= 1; step /= 2)
    for (int j = step; j <= 200; j += step)
      if (!seen[j]) { seen[j] = 1; HALL_ORDER[k++] = j; }
}

/* The decision of hall_ok_pair_fast (wz_match.cpp:143-168): at every angle, in the
 * reference's expressions, X alone, Y alone, then the pair; reject at the first failure.
 * The angle visiting order of the reference is adaptive but a conjunction does not depend
 * on it, so any order of all 200 angles gives the same decision (HALL_ORDER here). */
int or_hall_pair(int n, const int8_t *X, const int8_t *Y, int L, const double *ct,
                 const double *st, double *max_pair, double *min_margin) {
  pthread_once(&hall_order_once, build_hall_order);
  const int w = n + 1;
  const double limit = 4.0 * n + 2.0;
  const double lim = limit + 0.5;
  int pass = 1;
  double mx = -1.0, mm = 1e300;
  for (int jj = 0; jj < 200; jj++) {
    const int j = HALL_ORDER[jj];
    const double *cj = ct + (size_t)j * w, *sj = st + (size_t)j * w;
    double rx = 0, ix = 0, ry = 0, iy = 0;
    for (int i = 0; i < L; i++) { rx += X[i] * cj[i]; ix += X[i] * sj[i]; }
    for (int i = 0; i < L; i++) { ry += Y[i] * cj[i]; iy += Y[i] * sj[i]; }
    double fx = rx * rx + ix * ix;
    double fy = ry * ry + iy * iy;
    double fp = rx * rx + ix * ix + ry * ry + iy * iy;
    if (fx > lim || fy > lim || fp > lim) {
      pass = 0;
      if (!max_pair && !min_margin) return 0;
    }
    if (fp > mx) mx = fp;
    double a = fabs(fx - lim), b = fabs(fy - lim), c = fabs(fp - lim);
    if (a < mm) mm = a;
    if (b < mm) mm = b;
    if (c < mm) mm = c;
  }
  if (max_pair) *max_pair = mx;
  if (min_margin) *min_margin = mm;
  return pass;
}

typedef struct {
  int n, L;
  const int8_t *XY;
  long long lo, hi;
  uint8_t *pass;
  const double *ct, *st;
} hall_job;

static void *hall_worker(void *arg) {
  hall_job *jb = (hall_job *)arg;
  for (long long p = jb->lo; p < jb->hi; p++) {
    const int8_t *X = jb->XY + (size_t)p * 2 * jb->L;
    jb->pass[p] = (uint8_t)or_hall_pair(jb->n, X, X + jb->L, jb->L, jb->ct, jb->st, 0, 0);
  }
  return 0;
}

double or_hall_batch(int n, int L, const int8_t *XY, long long npairs, uint8_t *pass,
                     int nthreads) {
  int w = n + 1;
  double *ct = (double *)malloc(sizeof(double) * 201 * w);
  double *st = (double *)malloc(sizeof(double) * 201 * w);
  or_hall_tables(n, ct, st);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  hall_job jobs[256];
  long long chunk = (npairs + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].n = n; jobs[t].L = L; jobs[t].XY = XY; jobs[t].pass = pass;
    jobs[t].ct = ct; jobs[t].st = st;
    jobs[t].lo = t * chunk;
    jobs[t].hi = (t + 1) * chunk < npairs ? (t + 1) * chunk : npairs;
    if (jobs[t].lo > jobs[t].hi) jobs[t].lo = jobs[t].hi;
  }
  if (nthreads == 1) {
    hall_worker(&jobs[0]);
  } else {
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], 0, hall_worker, &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], 0);
  }
  free(ct);
  free(st);
  return 0.0;
}

/* ------------------------------------------------------------------------------------ */
/* Exact integer checks                                                                   */
/* ------------------------------------------------------------------------------------ */

/* wz_match.cpp:184-192 */
int or_npaf_at(const int8_t *A, const int8_t *B, int n1, const int8_t *C, const int8_t *D,
               int n2, int s) {
  int c = 0;
  if (s < n1)
    for (int i = 0; i < n1 - s; i++) c += A[i] * A[i + s] + B[i] * B[i + s];
  if (s < n2)
    for (int i = 0; i < n2 - s; i++) c += C[i] * C[i + s] + D[i] * D[i + s];
  return c;
}

/* wz_match.cpp:2569-2583 */
long long or_flat_score(const int8_t *C, const int8_t *D, int n) {
  long long sc = 0;
  for (int s = 1; s <= n; s++) {
    int cd = 0;
    for (int i = 0; i + s < n; i++) cd += C[i] * C[i + s] + D[i] * D[i + s];
    sc += cd < 0 ? -cd : cd;
  }
  return sc;
}

/* wz_match.cpp:855-871: FNV-1a over (uint16 value, uint16 shift) for s = 1..n. */
uint64_t or_autocorr_key(const int8_t *X, const int8_t *Y, int L, int n, int negate) {
  uint64_t h = 1469598103934665603ULL;
  for (int s = 1; s <= n; s++) {
    int v = 0;
    if (s < L)
      for (int i = 0; i < L - s; i++) v += X[i] * X[i + s] + Y[i] * Y[i + s];
    if (negate) v = -v;
    h ^= (uint64_t)(uint16_t)(int16_t)v;
    h *= 1099511628211ULL;
    h ^= (uint64_t)(uint16_t)s;
    h *= 1099511628211ULL;
  }
  return h;
}

/* ------------------------------------------------------------------------------------ */
/* Thm 2.2 quad tables (wz_match.cpp:531-545)                                             */
/* ------------------------------------------------------------------------------------ */
static int QALL[16][4], QPOS[8][4], QNEG[8][4];
static const int QMID[4][2] = {{1, 1}, {1, -1}, {-1, 1}, {-1, -1}};
static uint8_t OUT2[16][5][9];
static uint8_t OUT3[128][5][9][13];
static signed char POS_OF[16];
static int ROOT_OF[2];
static pthread_once_t tables_once = PTHREAD_ONCE_INIT;

static int signbits4(int a, int b, int c, int d) {
  return ((a > 0) << 3) | ((b > 0) << 2) | ((c > 0) << 1) | (d > 0);
}

/* Outer-lag reachable-tuple tables, wz_match.cpp:565-598. For a boundary pattern (root
 * quad with A[0]=B[0]=+1, then k-1 positive quads) and every assignment of the next k
 * positive quads, record which first quads reach the residual tuple (F_0..F_{k-1}). */
static void build_tables(void) {
  int np = 0, nn = 0;
  for (int i = 0; i < 16; i++) {
    int v[4] = {(i & 8) ? 1 : -1, (i & 4) ? 1 : -1, (i & 2) ? 1 : -1, (i & 1) ? 1 : -1};
    memcpy(QALL[i], v, sizeof v);
    if (v[0] * v[1] * v[2] * v[3] == 1) memcpy(QPOS[np++], v, sizeof v);
    else memcpy(QNEG[nn++], v, sizeof v);
  }
  for (int i = 0; i < 16; i++) POS_OF[i] = -1;
  for (int q = 0; q < 8; q++) POS_OF[signbits4(QPOS[q][0], QPOS[q][1], QPOS[q][2], QPOS[q][3])] = (signed char)q;
  for (int q = 0; q < 8; q++)
    if (QNEG[q][0] == 1 && QNEG[q][1] == 1) ROOT_OF[QNEG[q][2] > 0] = q;
  memset(OUT2, 0, sizeof OUT2);
  memset(OUT3, 0, sizeof OUT3);
  for (int k = 2; k <= 3; k++) {
    int npat = (k == 2) ? 16 : 128;
    for (int pat = 0; pat < npat; pat++) {
      int lA[3], lB[3], rA[3], rB[3];
      const int *root = QNEG[ROOT_OF[pat & 1]];
      int rest = pat >> 1;
      lA[0] = root[0]; lB[0] = root[1]; rA[0] = root[2]; rB[0] = root[3];
      for (int t = 1; t < k; t++) {
        const int *q = QPOS[rest % 8];
        rest /= 8;
        lA[t] = q[0]; lB[t] = q[1]; rA[t] = q[2]; rB[t] = q[3];
      }
      int nasg = (k == 2) ? 64 : 512;
      for (int asg = 0; asg < nasg; asg++) {
        int idx[3], a = asg;
        for (int r = 0; r < k; r++) { idx[r] = a % 8; a /= 8; }
        int F[3] = {0, 0, 0};
        for (int j = 0; j < k; j++)
          for (int r = 0; r <= j; r++) {
            const int *v = QPOS[idx[r]];
            F[j] += lA[j - r] * v[2] + lB[j - r] * v[3] + rA[j - r] * v[0] + rB[j - r] * v[1];
          }
        if (k == 2) OUT2[pat][F[0] / 2 + 2][F[1] / 2 + 4] |= (uint8_t)(1u << idx[0]);
        else OUT3[pat][F[0] / 2 + 2][F[1] / 2 + 4][F[2] / 2 + 6] |= (uint8_t)(1u << idx[0]);
      }
    }
  }
}

static void tables_init(void) { pthread_once(&tables_once, build_tables); }

void or_outer_tables(uint8_t *outer2, uint8_t *outer3) {
  tables_init();
  memcpy(outer2, OUT2, sizeof OUT2);
  memcpy(outer3, OUT3, sizeof OUT3);
}

/* ------------------------------------------------------------------------------------ */
/* C,D stream (count_pairs22, wz_match.cpp:678-784)                                       */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  int n, L, m, half;
  const int *tx, *ty;
  int pinX, pinY, rev, endpos, ab_side;
  int cd_root, cd_reach, root_mod;
  int blk_r[3], blk_s[3], blk_of[6];
  int qrem[64][3];
  int tot[8];
  int X[256], Y[256];
  int px[8], py[8], placed[8];
  const double *ct, *st;
  int keep_all;
  int8_t *out;
  uint8_t *out_pass;
  long long cap, written;
  or_stream_stats stats;
} cd_state;

static int class_count(int L, int c, int m) {
  int k = 0;
  for (int p = c; p < L; p += m) k++;
  return k;
}

static void cd_leaf(cd_state *S) {
  S->stats.leaves++;
  int8_t x[256], y[256];
  for (int i = 0; i < S->L; i++) { x[i] = (int8_t)S->X[i]; y[i] = (int8_t)S->Y[i]; }
  int pass = or_hall_pair(S->n, x, y, S->L, S->ct, S->st, 0, 0);
  if (pass) S->stats.ok++;
  if (pass || S->keep_all) {
    if (S->written < S->cap) {
      memcpy(S->out + (size_t)S->written * 2 * S->L, x, S->L);
      memcpy(S->out + (size_t)S->written * 2 * S->L + S->L, y, S->L);
      if (S->out_pass) S->out_pass[S->written] = (uint8_t)pass;
    }
    S->written++;
  }
}

static int cd_exact(cd_state *S) {
  for (int c = 0; c < S->m; c++)
    if (S->px[c] != S->tx[c] || S->py[c] != S->ty[c]) return 0;
  return 1;
}

static void cd_rec(cd_state *S, int d) {
  S->stats.nodes++;
  const int m = S->m;
  for (int c = 0; c < m; c++) {
    int rem = S->tot[c] - S->placed[c];
    int dx = S->tx[c] - S->px[c], dy = S->ty[c] - S->py[c];
    if (dx < -rem || dx > rem || dy < -rem || dy > rem) return;
    if (((dx + rem) & 1) != 0 || ((dy + rem) & 1) != 0) return;
  }
  if (S->cd_reach && d >= 1) {
    for (int b = 0; b < 3; b++) {
      int r = S->blk_r[b], s = S->blk_s[b], q = S->qrem[d][b];
      int D0 = S->tx[r] - S->px[r], D1 = S->ty[r] - S->py[r];
      int D2 = S->tx[s] - S->px[s], D3 = S->ty[s] - S->py[s];
      int t0 = D0 + D1 + D2 + D3, t1 = D0 - D1 + D2 - D3, t2 = D0 + D1 - D2 - D3,
          t3 = D0 - D1 - D2 + D3;
      if ((t0 | t1 | t2 | t3) & 3) return;
      int l1 = (abs(t0) + abs(t1) + abs(t2) + abs(t3)) / 4;
      if (l1 > q || ((q - l1) & 1)) return;
    }
  }
  const int L = S->L;
  if (d == S->half) {
    if (L % 2 == 1) {
      int mid = S->half, c = mid % m;
      for (int k = 0; k < 4; k++) {
        S->X[mid] = QMID[k][0];
        S->Y[mid] = QMID[k][1];
        S->px[c] += S->X[mid]; S->py[c] += S->Y[mid]; S->placed[c]++;
        if (cd_exact(S)) cd_leaf(S);
        S->px[c] -= S->X[mid]; S->py[c] -= S->Y[mid]; S->placed[c]--;
      }
      S->X[mid] = S->Y[mid] = 0;
    } else if (cd_exact(S)) {
      cd_leaf(S);
    }
    return;
  }
  int i1 = d, i2 = L - 1 - d, c1 = i1 % m, c2 = i2 % m;
  /* wz_match.cpp:766-768: the A,B side roots at the negative-product quads */
  const int(*Q)[4] = (d == 0) ? (S->ab_side ? QNEG : (S->endpos ? QPOS : QALL)) : QPOS;
  int ns = (d == 0 && !S->ab_side && !S->endpos) ? 16 : 8;
  for (int kk = 0; kk < ns; kk++) {
    int k = S->rev ? ns - 1 - kk : kk;
    if (d == 0 && S->pinX && Q[k][0] != 1) continue;
    if (d == 0 && S->pinY && Q[k][1] != 1) continue;
    if (d == 0 && S->cd_root &&
        (((Q[k][0] + Q[k][1] + Q[k][2] + Q[k][3]) % 4 + 4) % 4) != S->root_mod)
      continue;
    S->X[i1] = Q[k][0]; S->Y[i1] = Q[k][1]; S->X[i2] = Q[k][2]; S->Y[i2] = Q[k][3];
    S->px[c1] += Q[k][0]; S->py[c1] += Q[k][1]; S->px[c2] += Q[k][2]; S->py[c2] += Q[k][3];
    S->placed[c1]++; S->placed[c2]++;
    cd_rec(S, d + 1);
    S->px[c1] -= Q[k][0]; S->py[c1] -= Q[k][1]; S->px[c2] -= Q[k][2]; S->py[c2] -= Q[k][3];
    S->placed[c1]--; S->placed[c2]--;
  }
  S->X[i1] = S->Y[i1] = S->X[i2] = S->Y[i2] = 0;
}

long long or_cd_stream(int n, int L, int m, const int *tx, const int *ty, int pinX, int pinY,
                       int rev, int endpos, int cd_prune, int keep_all, int8_t *out_xy,
                       uint8_t *out_pass, long long cap, or_stream_stats *st) {
  tables_init();
  cd_state *S = (cd_state *)calloc(1, sizeof(cd_state));
  S->ab_side = (L == n + 1);  /* the A,B side is the one of length n+1 */
  S->n = n; S->L = L; S->m = m; S->half = L / 2;
  S->tx = tx; S->ty = ty;
  S->pinX = pinX; S->pinY = pinY; S->rev = rev; S->endpos = endpos;
  for (int c = 0; c < m; c++) S->tot[c] = class_count(L, c, m);
  /* CD_PRUNE set-up, wz_match.cpp:696-711 */
  int cd_ok = (!S->ab_side && m == 6 && L % 2 == 0);
  S->cd_root = cd_ok && (cd_prune & 1);
  S->cd_reach = cd_ok && (cd_prune & 2);
  if (cd_ok && cd_prune) {
    int nb = 0;
    for (int r = 0; r < 6; r++) {
      int s = (L - 1 - r) % 6;
      if (r < s) { S->blk_r[nb] = r; S->blk_s[nb] = s; S->blk_of[r] = S->blk_of[s] = nb; nb++; }
    }
    int half = L / 2;
    memset(S->qrem, 0, sizeof S->qrem);
    for (int d = half - 1; d >= 0; d--) {
      for (int b = 0; b < 3; b++) S->qrem[d][b] = S->qrem[d + 1][b];
      S->qrem[d][S->blk_of[d % 6]]++;
    }
    int tot = 0;
    for (int c = 0; c < 6; c++) tot += tx[c] + ty[c];
    S->root_mod = (tot % 4 + 4) % 4;
  }
  int w = n + 1;
  double *ct = (double *)malloc(sizeof(double) * 201 * w);
  double *stb = (double *)malloc(sizeof(double) * 201 * w);
  or_hall_tables(n, ct, stb);
  S->ct = ct; S->st = stb;
  S->keep_all = keep_all; S->out = out_xy; S->out_pass = out_pass; S->cap = cap;
  cd_rec(S, 0);
  long long written = S->written;
  if (st) *st = S->stats;
  free(ct);
  free(stb);
  free(S);
  return written;
}

/* ------------------------------------------------------------------------------------ */
/* A,B completion (fh_complete_ab / fh_ab_search, wz_match.cpp:1115-1341)                */
/* ------------------------------------------------------------------------------------ */
typedef struct {
  int n, L, half, m;
  int absA, absB;
  long long budget, cur, nodes;
  int aborted;
  int outer_k, early, canon;
  int target[260];
  int A[256], B[256], Dab[260], Kab[260];
  int pa[8], pb[8], placed[8], tic[8];
  const int8_t *rows;
  int nrows;
  int *stack;  /* (half+2) lists of nrows row indices */
  int *stack_len;
  /* WZ_FH_A2 = 2 (wz_match.cpp:977-1047): blocks of residues {r, s = (L-1-r) mod m}, the
     free middle's block at odd L, quads left per block from depth p on */
  int a2, a2_nblk, a2_r[8], a2_s[8], a2_mid[8], a2_cnt[40][8];
} ab_state;

/* fh_place / fh_unplace, V1 form (wz_match.cpp:1127-1161). */
static void ab_place(ab_state *S, int p, int av, int bv) {
  for (int q = 0; q < S->L; q++) {
    if (S->A[q] == 0 || q == p) continue;
    int s = q > p ? q - p : p - q;
    S->Dab[s] += S->A[q] * av + S->B[q] * bv;
    S->Kab[s] -= 2;
  }
  S->A[p] = av; S->B[p] = bv;
  int pc = p % S->m;
  S->pa[pc] += av; S->pb[pc] += bv; S->placed[pc]++;
}

static void ab_unplace(ab_state *S, int p) {
  int av = S->A[p], bv = S->B[p];
  S->A[p] = 0; S->B[p] = 0;
  int pc = p % S->m;
  S->pa[pc] -= av; S->pb[pc] -= bv; S->placed[pc]--;
  for (int q = 0; q < S->L; q++) {
    if (S->A[q] == 0 || q == p) continue;
    int s = q > p ? q - p : p - q;
    S->Dab[s] -= S->A[q] * av + S->B[q] * bv;
    S->Kab[s] += 2;
  }
}

/* outer_mask, wz_match.cpp:601-618 */
static unsigned ab_outer_mask(ab_state *S, int d) {
  int k = S->outer_k, L = S->L;
  if (k < 2 || d < k || d + k > L / 2 || S->A[0] != 1 || S->B[0] != 1) return 0xFFu;
  int pat = (S->A[L - 1] > 0), mul = 2;
  for (int t = 1; t < k; t++) {
    int q = POS_OF[signbits4(S->A[t], S->B[t], S->A[L - 1 - t], S->B[L - 1 - t])];
    if (q < 0) return 0xFFu;
    pat += mul * q;
    mul *= 8;
  }
  int R[3];
  for (int j = 0; j < k; j++) {
    int sj = L - 1 - d - j;
    R[j] = S->target[sj] - S->Dab[sj];
    if ((R[j] & 1) || R[j] < -4 * (j + 1) || R[j] > 4 * (j + 1)) return 0;
  }
  if (k == 2) return OUT2[pat][R[0] / 2 + 2][R[1] / 2 + 4];
  return OUT3[pat][R[0] / 2 + 2][R[1] / 2 + 4][R[2] / 2 + 6];
}

/* a2_self_ok / a2_row_ok, wz_match.cpp:1017-1038 */
static int a2_self_ok(int u, int v, int q) {
  if ((u | v) & 1) return 0;
  if (abs(u) > 2 * q || abs(v) > 2 * q) return 0;
  return ((u - v) & 3) == 0;
}
static int a2_row_ok(const ab_state *S, const int8_t *row, int p) {
  for (int b = 0; b < S->a2_nblk; b++) {
    int r = S->a2_r[b], s = S->a2_s[b], q = S->a2_cnt[p][b];
    int ur = row[r] - S->pa[r], vr = row[8 + r] - S->pb[r];
    if (r != s) {
      int us = row[s] - S->pa[s], vs = row[8 + s] - S->pb[s];
      int t0 = ur + vr + us + vs, t1 = ur - vr + us - vs, t2 = ur + vr - us - vs, t3 = ur - vr - us + vs;
      if ((t0 | t1 | t2 | t3) & 3) return 0;
      int l1 = (abs(t0) + abs(t1) + abs(t2) + abs(t3)) >> 2;
      if (l1 > q || ((q - l1) & 1)) return 0;
    } else if (S->a2_mid[b]) {
      if (!a2_self_ok(ur - 1, vr - 1, q) && !a2_self_ok(ur - 1, vr + 1, q) &&
          !a2_self_ok(ur + 1, vr - 1, q) && !a2_self_ok(ur + 1, vr + 1, q)) return 0;
    } else if (!a2_self_ok(ur, vr, q)) {
      return 0;
    }
  }
  return 1;
}

/* init_a2_tables, wz_match.cpp:1000-1016 */
static void a2_init(ab_state *S) {
  int L = S->L, m = S->m, half = L / 2, blk_of[8];
  for (int c = 0; c < 8; c++) blk_of[c] = -1;
  S->a2_nblk = 0;
  for (int c = 0; c < m; c++) {
    if (blk_of[c] >= 0) continue;
    int s = ((L - 1 - c) % m + m) % m;
    S->a2_r[S->a2_nblk] = c; S->a2_s[S->a2_nblk] = s; S->a2_mid[S->a2_nblk] = 0;
    blk_of[c] = blk_of[s] = S->a2_nblk++;
  }
  if (L % 2 == 1) S->a2_mid[blk_of[half % m]] = 1;
  for (int p = 0; p <= half + 1 && p < 40; p++) {
    for (int b = 0; b < 8; b++) S->a2_cnt[p][b] = 0;
    for (int i = p; i < half; i++) S->a2_cnt[p][blk_of[i % m]]++;
  }
}

/* fh_abp_filter, wz_match.cpp:1055-1078 (the A2 prune in mode 2). */
static int ab_row_filter(ab_state *S, int d) {
  int *src = S->stack + (size_t)d * S->nrows;
  int *dst = S->stack + (size_t)(d + 1) * S->nrows;
  int ns = S->stack_len[d], nd = 0;
  for (int t = 0; t < ns; t++) {
    const int8_t *row = S->rows + 16 * (size_t)src[t];
    int ok = 1;
    for (int c = 0; c < S->m; c++) {
      int rem = S->tic[c] - S->placed[c];
      int dk = row[c] - S->pa[c], dr = row[8 + c] - S->pb[c];
      if (dk < -rem || dk > rem || dr < -rem || dr > rem) { ok = 0; break; }
    }
    if (ok && S->a2 == 2 && !a2_row_ok(S, row, d + 1)) ok = 0;
    if (ok) dst[nd++] = src[t];
  }
  S->stack_len[d + 1] = nd;
  return nd != 0;
}

/* fh_abp_leaf_ok, wz_match.cpp:1080-1090 */
static int ab_row_leaf(ab_state *S) {
  int lev = (S->n + 1) / 2;
  int *src = S->stack + (size_t)lev * S->nrows;
  for (int t = 0; t < S->stack_len[lev]; t++) {
    const int8_t *row = S->rows + 16 * (size_t)src[t];
    int eq = 1;
    for (int c = 0; c < S->m; c++)
      if (row[c] != S->pa[c] || row[8 + c] != S->pb[c]) { eq = 0; break; }
    if (eq) return 1;
  }
  return 0;
}

static int ab_final(ab_state *S, int sA, int sB) {
  if (abs(sA) != S->absA || abs(sB) != S->absB) return 0;
  for (int s = 1; s <= S->n; s++)
    if (S->Dab[s] != S->target[s]) return 0;
  if (S->rows && !ab_row_leaf(S)) return 0;
  return 1;
}

/* fh_ab_search, wz_match.cpp:1171-1293 (telemetry, A2 and MID_SOLVE off). */
static int ab_search(ab_state *S, int d, int sumA, int sumB, int a_tied, int a_cmp,
                     int b_tied, int b_cmp) {
  if (S->aborted) return 0;
  const int L = S->L, half = S->half, n = S->n;
  if (d == half) {
    if (L % 2 == 1) {
      int mid = half;
      for (int k = 0; k < 4; k++) {
        int av = QMID[k][0], bv = QMID[k][1];
        ab_place(S, mid, av, bv);
        S->nodes++;
        int ok = ab_final(S, sumA + av, sumB + bv);
        if (!ok) ab_unplace(S, mid);
        if (ok) return 1;
      }
      return 0;
    }
    return ab_final(S, sumA, sumB);
  }
  int i1 = d, i2 = L - 1 - d;
  const int(*Q)[4] = (d == 0) ? QNEG : QPOS;
  unsigned omask = (S->outer_k && d > 0) ? ab_outer_mask(S, d) : 0xFFu;
  if (omask == 0) return 0;
  for (int k = 0; k < 8; k++) {
    if (d > 0 && !((omask >> k) & 1u)) continue;
    int a1 = Q[k][0], b1 = Q[k][1], a2 = Q[k][2], b2 = Q[k][3];
    if (d == 0 && S->canon && (a1 != 1 || b1 != 1)) continue;
    int na_tied = a_tied, na_cmp = a_cmp, nb_tied = b_tied, nb_cmp = b_cmp;
    if (S->canon) {
      if (d == 0) {
        na_cmp = a2;
        nb_cmp = b2;
      } else {
        if (a_tied) {
          int cv = a_cmp * a2;
          if (a1 != cv) {
            if (a1 != 1) continue;
            na_tied = 0;
          }
        }
        if (b_tied) {
          int cv = b_cmp * b2;
          if (b1 != cv) {
            if (b1 != 1) continue;
            nb_tied = 0;
          }
        }
      }
    }
    S->nodes++;
    if (S->budget > 0 && ++S->cur > S->budget) {
      S->aborted = 1;
      return 0;
    }
    if (S->early && d > 0) {
      int s = L - 1 - d;
      if (S->A[0] * a2 + S->B[0] * b2 + S->A[L - 1] * a1 + S->B[L - 1] * b1 !=
          S->target[s] - S->Dab[s])
        continue;
    }
    ab_place(S, i1, a1, b1);
    ab_place(S, i2, a2, b2);
    int nsA = sumA + a1 + a2, nsB = sumB + b1 + b2;
    int rem = L - 2 * (d + 1);
    int sum_ok = ((abs(S->absA - nsA) <= rem) || (abs(-S->absA - nsA) <= rem)) &&
                 ((abs(S->absB - nsB) <= rem) || (abs(-S->absB - nsB) <= rem));
    int prune = !sum_ok;
    if (!prune)
      for (int s = 1; s <= n; s++)
        if (abs(S->target[s] - S->Dab[s]) > S->Kab[s]) { prune = 1; break; }
    if (!prune && S->rows && !ab_row_filter(S, d)) prune = 1;
    if (!prune) {
      if (ab_search(S, d + 1, nsA, nsB, na_tied, na_cmp, nb_tied, nb_cmp)) return 1;
    }
    ab_unplace(S, i2);
    ab_unplace(S, i1);
  }
  return 0;
}

int or_complete_ab(int n, int sigA, int sigB, const int8_t *C, const int8_t *D,
                   long long budget, int outer_k, int early, int canon, int m,
                   const int8_t *rows, int nrows, int8_t *Aout, int8_t *Bout,
                   long long *nodes) {
  return or_complete_ab_a2(n, sigA, sigB, C, D, budget, outer_k, early, canon, m, rows, nrows, 0,
                           Aout, Bout, nodes);
}

int or_complete_ab_a2(int n, int sigA, int sigB, const int8_t *C, const int8_t *D,
                      long long budget, int outer_k, int early, int canon, int m,
                      const int8_t *rows, int nrows, int a2, int8_t *Aout, int8_t *Bout,
                      long long *nodes) {
  tables_init();
  ab_state *S = (ab_state *)calloc(1, sizeof(ab_state));
  int n1 = n + 1;
  S->n = n; S->L = n1; S->half = n1 / 2; S->m = m;
  S->a2 = a2;
  if (a2) a2_init(S);
  S->budget = budget; S->outer_k = outer_k; S->early = early; S->canon = canon;
  if (nodes) *nodes = 0;
  /* target = -CD, prefilter: wz_match.cpp:1300-1308 */
  for (int s = 1; s <= n; s++) {
    int cd = 0;
    for (int i = 0; i + s < n; i++) cd += C[i] * C[i + s] + D[i] * D[i + s];
    S->target[s] = -cd;
  }
  for (int s = 1; s < n1; s++)
    if (abs(S->target[s]) > 2 * (n1 - s)) { free(S); return 1; }
  for (int s = 0; s <= n; s++) S->Kab[s] = (s >= 1 && s < n1) ? 2 * (n1 - s) : 0;
  S->absA = abs(sigA);
  S->absB = abs(sigB);
  for (int c = 0; c < m; c++) S->tic[c] = class_count(n1, c, m);
  int *stack = 0, *slen = 0;
  if (rows && nrows > 0) {
    S->rows = rows; S->nrows = nrows;
    stack = (int *)malloc(sizeof(int) * (size_t)(S->half + 2) * nrows);
    slen = (int *)calloc(S->half + 2, sizeof(int));
    for (int r = 0; r < nrows; r++) stack[r] = r;
    slen[0] = nrows;
    S->stack = stack; S->stack_len = slen;
  }
  int found = ab_search(S, 0, 0, 0, 1, 0, 1, 0);
  int verdict;
  if (!found) {
    verdict = S->aborted ? 3 : 2;
  } else {
    int8_t a[256], b[256];
    for (int i = 0; i < n1; i++) { a[i] = (int8_t)S->A[i]; b[i] = (int8_t)S->B[i]; }
    verdict = 0;
    for (int s = 1; s <= n; s++)
      if (or_npaf_at(a, b, n1, C, D, n, s) != 0) { verdict = 4; break; }
    if (Aout) memcpy(Aout, a, n1);
    if (Bout) memcpy(Bout, b, n1);
  }
  if (nodes) *nodes = S->nodes;
  free(stack);
  free(slen);
  free(S);
  return verdict;
}

/* ------------------------------------------------------------------------------------ */
/* Hall microbench input generator (splitmix64 per pair index)                           */
/* ------------------------------------------------------------------------------------ */
static uint64_t g_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static uint64_t g_sm(uint64_t seed, uint64_t k) { return g_mix(seed + (k + 1) * 0x9E3779B97F4A7C15ULL); }

typedef struct { int n; long long npairs, lo, hi; uint64_t seed; uint64_t *w; } gen_job;

static void *gen_worker(void *arg) {
  gen_job *g = (gen_job *)arg;
  static const unsigned posq[8] = {0, 3, 5, 6, 9, 10, 12, 15};
  const int n = g->n;
  const long long half = g->npairs / 2;
  const uint64_t mask = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
  for (long long p = g->lo; p < g->hi; p++) {
    uint64_t cw, dw;
    if (p < half || (n & 1) || n > 42) {
      cw = g_sm(g->seed, 2 * (uint64_t)p) & mask;
      dw = g_sm(g->seed, 2 * (uint64_t)p + 1) & mask;
    } else {
      uint64_t t = 0;
      for (;;) {
        uint64_t r = g_sm(g->seed ^ 0xA5A5A5A5A5A5A5A5ULL, ((uint64_t)p << 20) + t);
        t++;
        cw = dw = 0;
        for (int d = 0; d < n / 2; d++) {
          unsigned q;
          if (d == 0) { q = (unsigned)(r & 15); r >>= 4; }
          else { q = posq[r & 7]; r >>= 3; }
          cw |= (uint64_t)((q >> 3) & 1) << d;
          dw |= (uint64_t)((q >> 2) & 1) << d;
          cw |= (uint64_t)((q >> 1) & 1) << (n - 1 - d);
          dw |= (uint64_t)(q & 1) << (n - 1 - d);
        }
        if (__builtin_popcountll(cw) * 2 == n && __builtin_popcountll(dw) * 2 == n) break;
      }
    }
    g->w[2 * p] = cw;
    g->w[2 * p + 1] = dw;
  }
  return 0;
}

void or_gen_hall_pairs(int n, long long npairs, uint64_t seed, uint64_t *words, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  gen_job jobs[256];
  long long chunk = (npairs + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].n = n; jobs[t].npairs = npairs; jobs[t].seed = seed; jobs[t].w = words;
    jobs[t].lo = t * chunk < npairs ? t * chunk : npairs;
    jobs[t].hi = (t + 1) * chunk < npairs ? (t + 1) * chunk : npairs;
  }
  if (nthreads == 1) { gen_worker(&jobs[0]); return; }
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], 0, gen_worker, &jobs[t]);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], 0);
}
