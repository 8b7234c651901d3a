// firsthit_main.cpp - bs_firsthit: a drop-in for one lane of the reference solver's
// first-hit mode (`WZ_FIRSTHIT=1 wz_match <n> <a> <b> <c> <d>`, src/solver/wz_match.cpp:
// 1343-1391 and 1544-2891), with the C,D stream, the Hall test, the per-cell flattest-k keep
// and the A,B completion running on the GPU through libbsfh.so (include/bsfh.h).
//
// Same argv, same WZ_* environment, same stdout tokens the reference's lane script greps, same
// checkpoint file (CFGSIG line and resume fields) and the same exit codes:
//   0 FOUND, 3 no hit / range exhausted / interrupted, 2 refusal, 1 usage, 5 internal error.
// Not carried over (measurement-only instruments of the reference): FH_TELEM telemetry,
// HALLSTAT adaptive-order statistics, the A2 shadow (WZ_FH_A2=1; the A2 prune, WZ_FH_A2=2,
// runs on the device), LOCATE / ORBIT_AUDIT / OUTER_DUMP / TARGET canaries. WZ_FH_CD_PRUNE prunes the device stream as the reference's DFS does (same stream,
// CDSTAT counts the pruned walk); WZ_FH_HALL_FAST changes no stream and is accepted, and so is
// WZ_FH_MID_SOLVE, which changes only the reference's node statistics (the counts here are
// those without it; verdicts, hits and completion counts are the same either way).
// WZ_FH_WALL_SEC abandons a cell whose stream finds no survivor for that many seconds (its
// partial buffer is still drained, and it counts in cells_walled), and SIGTERM raises the
// context's stop flag, which stops a running stream or completion within one device round.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <csignal>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/bsfh.h"
#include "celllist.h"

using namespace bsfh;
using Clock = std::chrono::steady_clock;

namespace {

volatile sig_atomic_t g_sigterm = 0;
volatile int32_t *g_stop_flag = nullptr;  // the context's mapped stop flag (bs_ctx_stop_flag)
void on_sigterm(int) {
  g_sigterm = 1;
  if (g_stop_flag) *g_stop_flag = 1;  // a plain store to pinned host memory: signal-safe
}

const char *env(const char *k) { return getenv(k); }
long long env_ll(const char *k, long long dflt) {
  const char *e = getenv(k);
  return e ? atoll(e) : dflt;
}
int env_i(const char *k, int dflt) {
  const char *e = getenv(k);
  return e ? atoi(e) : dflt;
}
bool env_on(const char *k) {
  const char *e = getenv(k);
  return e && atoi(e) != 0;
}

double secs_since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

std::vector<int> parse_list(const char *s) {
  std::vector<int> v;
  int val, cnt;
  while (s && sscanf(s, "%d%n", &val, &cnt) == 1) {
    v.push_back(val);
    s += cnt;
    while (*s == ',' || *s == ' ') s++;
  }
  return v;
}

uint64_t pack_seq(const int *x, int L) {
  uint64_t w = 0;
  for (int i = 0; i < L; i++)
    if (x[i] > 0) w |= 1ULL << i;
  return w;
}
void unpack_seq(uint64_t w, int L, int *x) {
  for (int i = 0; i < L; i++) x[i] = ((w >> i) & 1ULL) ? 1 : -1;
}

int npaf_at(const int *A, const int *B, int n1, const int *C, const int *D, int n2, int s) {
  int c = 0;
  if (s < n1)
    for (int i = 0; i < n1 - s; i++) c += A[i] * A[i + s] + B[i] * B[i + s];
  if (s < n2)
    for (int i = 0; i < n2 - s; i++) c += C[i] * C[i + s] + D[i] * D[i + s];
  return c;
}

void print_seq(const char *name, const int *x, int L) {
  printf("%s = {", name);
  for (int i = 0; i < L; i++) printf("%d%s", x[i], i < L - 1 ? "," : "");
  printf("};\n");
}

int fail_gpu(int rc, const char *what) {
  printf("RESULT: GPU ERROR in %s: %s (%d)\n", what, bs_strerror(rc), rc);
  fflush(stdout);
  return 5;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 6) {
    std::cerr << "Usage: " << argv[0] << " <n> <a> <b> <c> <d>\n"
              << "  e.g.  WZ_FIRSTHIT=1 " << argv[0] << " 10 5 1 4 0   (BS(11,10))\n";
    return 1;
  }
  const int n = atoi(argv[1]);
  if (n < 4) { std::cerr << "ERROR: n must be >= 4\n"; return 1; }
  const int n1 = n + 1;
  const int SA = atoi(argv[2]), SB = atoi(argv[3]), SC = atoi(argv[4]), SD = atoi(argv[5]);
  const int sigsum = SA * SA + SB * SB + SC * SC + SD * SD;
  if (sigsum != 4 * n + 2) {
    std::cerr << "ERROR: sig norm = " << sigsum << ", expected " << (4 * n + 2) << "\n";
    return 1;
  }
  if (!env("WZ_FIRSTHIT")) {
    std::cerr << "bs_firsthit runs the first-hit lane only: set WZ_FIRSTHIT=1\n";
    return 1;
  }
  if (n1 > 64) { std::cerr << "ERROR: bs_firsthit supports n <= 63\n"; return 1; }
  bool thm211b = env("WZ_THM211B") != nullptr, thm212 = env("WZ_THM212") != nullptr;
  const bool endpos = env_on("WZ_FH_ENDPOS");
  // the reference applies its outer-lag tables only for K >= 2 (wz_match.cpp:602-603): any
  // smaller K runs without them, as K = 0 does; K > 3 has no table and is refused below
  const int outer_k_env = env_i("WZ_FH_OUTER_K", 3);  // printed as given
  const int outer_k = outer_k_env < 2 ? 0 : outer_k_env;
  const int a2_mode = env_i("WZ_FH_A2", 0);
  if (a2_mode != 0 && a2_mode != 2) {
    printf("RESULT: WZ_FH_A2=%d (the A2 shadow instrument) is not built on the GPU lane — refusing\n", a2_mode);
    return 2;
  }
  if (outer_k > 3) {
    printf("RESULT: WZ_FH_OUTER_K must be at most 3\n");
    return 2;
  }
  const bool cand_log = env_on("WZ_FH_CAND_LOG");
  if (const char *e = env("WZ_FH_TELEMETRY")) {
    if (strcmp(e, "0") && strcmp(e, "1") && strcmp(e, "64")) {
      std::cerr << "WZ_FH_TELEMETRY must be 0, 1 or 64\n";
      return 2;
    }
  }
  // 2.11b and 2.12 are forced at n >= 36 in first-hit mode (wz_match.cpp:1388)
  if (n >= 36) { thm211b = true; thm212 = true; }
  const int early = (env("WZ_FH_EARLY_CHECK") && atoi(env("WZ_FH_EARLY_CHECK")) == 0) ? 0 : 1;
  const int canon = env("WZ_FH_NO_CANON") ? 0 : 1;
  int hall_mode = BS_HALL_TC_FP16;
  if (const char *e = env("BS_HALL_FORM")) {
    if (!strcmp(e, "fp64")) hall_mode = BS_HALL_FP64;
    else if (!strcmp(e, "tc_bf16x2")) hall_mode = BS_HALL_TC_BF16X2;
  }

  printf("========================================================\n");
  printf("  bs_firsthit (GB300) — first-hit BS(%d,%d), sig=(%d,%d,%d,%d)\n", n1, n, SA, SB, SC, SD);
  printf("  device: sm_103a via libbsfh (Hall filter %s)\n",
         hall_mode == BS_HALL_FP64 ? "fp64" : hall_mode == BS_HALL_TC_FP16 ? "tc_fp16" : "tc_bf16x2");
  printf("========================================================\n");
  fflush(stdout);
  const auto G_T0 = Clock::now();

  // ---------------------------------------------------------------- run configuration
  bool fh_m6 = (n >= 36);
  if (const char *e = env("WZ_FH_M6")) fh_m6 = atoi(e) != 0;
  const long long budget = env_ll("WZ_FH_AB_BUDGET", 200000);
  const long long max_cand = env_ll("WZ_FH_MAX_CAND", 0);
  const long long score_max = env_ll("WZ_FH_SCORE_MAX", 0);
  const int prof_order = env_i("WZ_FH_PROF_ORDER", 0);
  const double stream_total = env("WZ_FH_STREAM_TOTAL") ? atof(env("WZ_FH_STREAM_TOTAL")) : 0;
  int fh_shard = env_i("WZ_FH_SHARD", 0), fh_nshard = env_i("WZ_FH_NSHARD", 1);
  if (fh_nshard < 1) fh_nshard = 1;
  if (fh_shard < 0 || fh_shard >= fh_nshard) {
    printf("[firsthit] BAD SHARD %d/%d\n", fh_shard, fh_nshard);
    return 2;
  }

  // ---------------------------------------------------------------- cell list
  ListOptions lopt;
  lopt.m6 = fh_m6;
  lopt.thm211b = thm211b;
  lopt.thm212 = thm212;
  lopt.endpos = endpos;
  lopt.endpos_nocell = env_on("WZ_FH_ENDPOS_NOCELL");
  const bool orbit_canon = env_i("WZ_FH_ORBIT_CANON", 0) != 0;
  lopt.orbit_canon = orbit_canon;
  lopt.orbit_q = env_i("WZ_FH_ORBIT_Q", 0);
  lopt.qprune = env_on("WZ_FH_ORBIT_QPRUNE");
  lopt.prof_order = prof_order;
  lopt.nshard = fh_nshard;
  lopt.qprune_dump = env("WZ_FH_QPRUNE_DUMP");
  CellList list;
  if (build_cell_list(n, SA, SB, SC, SD, lopt, list, stdout) != 0) return 2;
  std::vector<Profile> &cells = list.cells;
  const int fh_m = list.m;
  const bool orbit_q = list.orbit_q, qp_active = list.qp_active;
  const std::string order_digest = list.digest;
  // the canonical orbit representative need not carry the zero-sum pin (wz_match.cpp:1659-1662)
  const bool pins_dropped = orbit_canon && (SC == 0 || SD == 0);
  const bool pinC = (SC == 0) && !orbit_canon, pinD = (SD == 0) && !orbit_canon;
  if (orbit_canon && prof_order == 3) {
    if (const char *e = env("WZ_FH_EXPECT_DIGEST"))
      if (order_digest != e) {
        printf("RESULT: DIGEST MISMATCH (expected %s) — refusing to search or resume\n", e);
        return 2;
      }
    if (env("WZ_FH_LIST_ONLY")) return 0;
    if (!env("WZ_FH_EXPECT_DIGEST") && !env("WZ_FH_LOCATE_C") && !env("WZ_FH_ORBIT_AUDIT") &&
        !env("WZ_FH_CELLSIZE") && !env("WZ_FH_ORD3_NODIGEST_OK")) {
      printf("RESULT: PROF_ORDER=3 search requires WZ_FH_EXPECT_DIGEST (from the manifest)\n");
      return 2;
    }
  }
  if (prof_order == 3 && !orbit_canon) {
    printf("RESULT: PROF_ORDER=3 requires WZ_FH_ORBIT_CANON=1\n");
    return 2;
  }
  printf("[firsthit] profiles=%zu m=%d order=%d ab_budget=%lld max_cand=%lld score_max=%lld shard=%d/%d\n",
         cells.size(), fh_m, prof_order, budget, max_cand, score_max, fh_shard, fh_nshard);
  fflush(stdout);
  // WZ_FH_LIST_CELLS=lo,hi: print raw cells [lo, hi) of the final list (with their orbit-kept
  // flag) and exit; a tool for choosing benchmark and canary cells.
  if (const char *e = env("WZ_FH_LIST_CELLS")) {
    std::vector<int> r = parse_list(e);
    long long lo = r.size() > 0 ? r[0] : 0, hi = r.size() > 1 ? r[1] : (long long)cells.size();
    for (long long pi = std::max(0LL, lo); pi < std::min(hi, (long long)cells.size()); pi++) {
      printf("CELL pi=%lld kept=%d px=", pi, (int)list.kept[pi]);
      for (int c = 0; c < fh_m; c++) printf("%d%s", cells[pi].px[c], c + 1 < fh_m ? "," : "");
      printf(" py=");
      for (int c = 0; c < fh_m; c++) printf("%d%s", cells[pi].py[c], c + 1 < fh_m ? "," : "");
      printf("\n");
    }
    return 0;
  }

  // ---------------------------------------------------------------- lane settings
  long long cand = 0, pre_rej = 0, score_rej = 0, clean_no = 0, aborted_ct = 0;
  long long cells_done = 0, cells_empty = 0, cells_orbit_dup = 0;
  long long cum_done_base = 0, cum_dup_base = 0, cum_dead_base = 0, cum_empty_base = 0;
  long long bt_entered = 0, hit_idx = -1, nodes_total = 0;
  bool fh_stop = false, found = false;
  signal(SIGTERM, on_sigterm);
  const double prog_sec = env("WZ_FH_PROG_SEC") ? atof(env("WZ_FH_PROG_SEC")) : 60;
  const auto T0 = Clock::now();
  const int fh_skip = env_i("WZ_FH_PROF_SKIP", 0);
  const int fh_end = env_i("WZ_FH_PROF_END", 0);
  bool cell_order = fh_m6;
  if (const char *e = env("WZ_FH_CELL_ORDER")) cell_order = atoi(e) != 0;
  bool ab_prof = fh_m6;
  if (const char *e = env("WZ_FH_AB_PROF")) ab_prof = atoi(e) != 0;
  const size_t abp_cap = (size_t)env_ll("WZ_FH_AB_PROF_CAP", 20000);
  const long long buf_cap = env_ll("WZ_FH_BUF_CAP", 500000);
  const long long drain_top = env_ll("WZ_FH_DRAIN_TOP", 0);
  const long long drain_batches = std::max(1LL, env_ll("WZ_FH_DRAIN_BATCHES", 1));
  const bool stream_rev = env_i("WZ_FH_STREAM_REV", 0) != 0;
  const long long wall_sec = std::max(0LL, env_ll("WZ_FH_WALL_SEC", 0));
  std::string ckpt_path;
  if (const char *e = env("WZ_FH_CKPT_DIR")) ckpt_path = std::string(e) + "/arm_" + std::to_string(fh_shard) + ".ckpt";
  bool resume_on = env_i("WZ_FH_RESUME", 1) != 0;
  const long long cellsize = std::max(0LL, env_ll("WZ_FH_CELLSIZE", 0));
  if (cellsize > 0) {
    ckpt_path.clear();
    resume_on = false;
    printf("[cellsize] MEASUREMENT MODE cap=%lld (no completions, no checkpoints)\n", cellsize);
    fflush(stdout);
  }
  const long long test_stop = env_ll("WZ_FH_TEST_STOP_AFTER", 0);
  const bool test_ierr = env("WZ_FH_TEST_INTERNAL_ERROR") != nullptr;
  FILE *dump = nullptr;
  if (const char *e = env("WZ_FH_DUMP")) dump = fopen(e, "w");

  // CFGSIG, wz_match.cpp:2241-2287 (fields appended only when non-default)
  char sigbuf[512];
  snprintf(sigbuf, sizeof sigbuf,
           "n%d.a%d.b%d.c%d.d%d.ns%d.sh%d.ord%d.m%d.co%d.ap%d.sm%lld.cap%lld.sk%d.t1%d.t2%d.oc%d.dt%lld", n, SA,
           SB, SC, SD, fh_nshard, fh_shard, prof_order, fh_m, cell_order ? 1 : 0, ab_prof ? 1 : 0, score_max,
           buf_cap, fh_skip, thm211b ? 1 : 0, thm212 ? 1 : 0, orbit_canon ? 1 : 0, drain_top);
  auto append = [&](const std::string &s) {
    size_t L0 = strlen(sigbuf);
    snprintf(sigbuf + L0, sizeof sigbuf - L0, "%s", s.c_str());
  };
  if (drain_batches > 1) append(".db" + std::to_string(drain_batches));
  if (stream_rev) append(".sr1");
  if (pins_dropped) append(".np1");
  if (wall_sec > 0) append(".ws" + std::to_string(wall_sec));
  if (endpos) append(".ep1");
  if (orbit_canon && orbit_q) append(".oq1");
  if (qp_active) append(".qp1");
  if (prof_order == 3) {
    std::string tail = ".bud" + std::to_string(budget) + ".dg" + (order_digest.empty() ? "none" : order_digest);
    if (strlen(sigbuf) + tail.size() >= sizeof sigbuf) { printf("RESULT: CFGSIG buffer overflow\n"); return 2; }
    append(tail);
  }
  const std::string cfg_sig = sigbuf;
  bool resuming = false;
  long long res_pi = 0, res_batch = 0, res_k = 0, tested_base = 0;
  if (!ckpt_path.empty() && resume_on) {
    if (FILE *cf = fopen(ckpt_path.c_str(), "r")) {
      char line[600], fsig[520] = {0};
      long long rpi = -1, rb = -1, rk = -1, tc = 0, cdc = 0, cdu = 0, cde = 0, cem = 0;
      while (fgets(line, sizeof line, cf)) {
        if (sscanf(line, "CFGSIG=%519s", fsig) == 1) continue;
        if (sscanf(line, "resume_pi=%lld", &rpi) == 1) continue;
        if (sscanf(line, "resume_batch=%lld", &rb) == 1) continue;
        if (sscanf(line, "resume_k=%lld", &rk) == 1) continue;
        if (sscanf(line, "tested_cum=%lld", &tc) == 1) continue;
        if (sscanf(line, "cells_done_cum=%lld", &cdc) == 1) continue;
        if (sscanf(line, "cells_dup_cum=%lld", &cdu) == 1) continue;
        if (sscanf(line, "cells_dead_cum=%lld", &cde) == 1) continue;
        sscanf(line, "cells_empty_cum=%lld", &cem);
      }
      fclose(cf);
      if (cfg_sig == fsig && rpi >= 0 && rb >= 0 && rk >= 0) {
        resuming = true;
        res_pi = rpi; res_batch = rb; res_k = rk; tested_base = tc;
        cum_done_base = cdc; cum_dup_base = cdu; cum_dead_base = cde; cum_empty_base = cem;
        printf("[firsthit ckpt] RESUME pi=%lld batch=%lld k=%lld tested_cum=%lld\n", rpi, rb, rk, tc);
      } else {
        printf("[firsthit ckpt] STALE/MISMATCHED checkpoint IGNORED (%s != %s) — starting FRESH\n", fsig,
               cfg_sig.c_str());
      }
      fflush(stdout);
    }
  }

  // ---- allowed A,B rows per cell invariant (the reference's abpMap) ----
  AbpRows abp;
  if (ab_prof) {
    auto tb0 = Clock::now();
    std::vector<uint64_t> keys;
    for (long long pi = fh_shard + (long long)fh_skip * fh_nshard; pi < (long long)cells.size(); pi += fh_nshard) {
      if (!list.kept[pi]) continue;
      keys.push_back(AbpRows::cell_key_of(cells[pi], n, fh_m));
    }
    abp.build(keys, n, SA, SB, fh_m);
    printf("[abprof] K=%zu R=%zu cell_keys=%zu rows=%lld max_list=%zu cap=%zu build=%gs\n", abp.nK, abp.nR,
           abp.by_key.size(), abp.rows, abp.max_list, abp_cap, secs_since(tb0));
    fflush(stdout);
  }

  // ---- the GPU context ----
  bs_ctx *ctx = nullptr;
  int rc = bs_ctx_create(n, SA, SB, SC, SD, env_i("BS_DEVICE", 0), &ctx);
  if (rc) return fail_gpu(rc, "bs_ctx_create");
  g_stop_flag = bs_ctx_stop_flag(ctx);
  if (g_sigterm) *g_stop_flag = 1;  // a SIGTERM before the context existed
  bs_ab_opts abo;
  memset(&abo, 0, sizeof abo);
  abo.budget = budget;
  abo.outer_k = outer_k;
  abo.early = early;
  abo.canon = canon;
  abo.m = fh_m;
  abo.first_hit = 1;
  abo.a2 = a2_mode;
  abo.max_seconds = 0;

  // ---- complete-only mode (WZ_FH_COMPLETE_C/_D), wz_match.cpp:2403-2455 ----
  if (const char *cc = env("WZ_FH_COMPLETE_C")) {
    std::vector<int> C0 = parse_list(cc), D0 = parse_list(env("WZ_FH_COMPLETE_D"));
    if ((int)C0.size() != n || (int)D0.size() != n) { printf("COMPLETE_ONLY: bad C/D length\n"); return 2; }
    bs_ab_cand one;
    memset(&one, 0, sizeof one);
    one.c = pack_seq(C0.data(), n);
    one.d = pack_seq(D0.data(), n);
    int32_t v = 0;
    long long nd = 0;
    std::vector<int8_t> A8(n1), B8(n1);
    auto t0c = Clock::now();
    rc = bs_complete_ab_batch(ctx, &one, 1, nullptr, 0, &abo, &v, &nd, A8.data(), B8.data());
    if (rc == BS_STOPPED) {
      printf("COMPLETE_ONLY interrupted (SIGTERM)\n");
      fflush(stdout);
      bs_ctx_destroy(ctx);
      return 3;
    }
    if (rc) return fail_gpu(rc, "bs_complete_ab_batch");
    printf("COMPLETE_ONLY r=%d nodes=%lld budget=%lld outer_k=%d a2=%d sec=%g\n", v, nd, budget, outer_k_env, a2_mode,
           secs_since(t0c));
    if (v == 0) {
      std::vector<int> A(n1), B(n1);
      for (int i = 0; i < n1; i++) { A[i] = A8[i]; B[i] = B8[i]; }
      printf("*** BS(%d,%d) FOUND ***  (complete-only)\n", n1, n);
      print_seq("A", A.data(), n1);
      print_seq("B", B.data(), n1);
      print_seq("C", C0.data(), n);
      print_seq("D", D0.data(), n);
    }
    fflush(stdout);
    bs_ctx_destroy(ctx);
    return 0;
  }

  long long cells_prof_dead = 0, cells_prof_uncap = 0, cells_capped = 0, cells_walled = 0;
  long long ck_pi = fh_shard + (long long)fh_skip * fh_nshard, ck_batch = 0, ck_k = 0;
  if (resuming) { ck_pi = res_pi; ck_batch = res_batch; ck_k = res_k; }
  auto write_ckpt = [&]() {
    if (ckpt_path.empty()) return;
    std::string tmp = ckpt_path + ".tmp";
    FILE *cf = fopen(tmp.c_str(), "w");
    if (!cf) return;
    fprintf(cf, "CFGSIG=%s\nresume_pi=%lld\nresume_batch=%lld\nresume_k=%lld\ntested_cum=%lld\n", cfg_sig.c_str(),
            ck_pi, ck_batch, ck_k, tested_base + clean_no + aborted_ct + (hit_idx >= 0 ? 1LL : 0LL));
    fprintf(cf, "cells_done_cum=%lld\ncells_dup_cum=%lld\ncells_dead_cum=%lld\ncells_empty_cum=%lld\n",
            cum_done_base + cells_done, cum_dup_base + cells_orbit_dup, cum_dead_base + cells_prof_dead,
            cum_empty_base + cells_empty);
    fclose(cf);
    rename(tmp.c_str(), ckpt_path.c_str());
  };
  auto last_ckpt = T0;
  long long ck_tick = 0;
  auto maybe_ckpt = [&]() {
    if (ckpt_path.empty()) return;
    if ((++ck_tick & 63) != 0) return;
    if (secs_since(last_ckpt) >= prog_sec) { last_ckpt = Clock::now(); write_ckpt(); }
  };
  long long test_ct = 0;
  auto last_prog = T0;
  const long long pi_end = (fh_end > 0) ? std::min((long long)cells.size(), (long long)fh_shard + (long long)fh_end * fh_nshard)
                                        : (long long)cells.size();
  bs_stream_opts so;
  memset(&so, 0, sizeof so);
  so.m = fh_m;
  so.rev = stream_rev ? 1 : 0;
  so.endpos = endpos ? 1 : 0;
  so.cd_prune = env_i("WZ_FH_CD_PRUNE", 0);
  so.hall_mode = hall_mode;
  so.wall_sec = (double)wall_sec;
  // Front-only lanes use only a cell's first DRAIN_BATCHES x BUF_CAP survivors (the reference
  // stops the cell's DFS there); the device stream stops there too. Score filtering and the
  // unbuffered order see further into the stream, so they stream whole cells.
  if (cell_order && drain_top > 0 && score_max == 0 && cellsize == 0)
    so.limit = drain_batches * buf_cap;
  std::vector<uint64_t> surv;
  std::vector<int32_t> surv_score;
  std::vector<int8_t> empty_rows;

  for (long long pi = fh_shard + (long long)fh_skip * fh_nshard; pi < pi_end && !fh_stop; pi += fh_nshard) {
    if (resuming && pi < res_pi) continue;
    if (resuming && pi > res_pi) resuming = false;
    if (!list.kept[pi]) {
      cells_orbit_dup++;
      if (resuming && pi == res_pi) resuming = false;
      ck_pi = pi + fh_nshard; ck_batch = 0; ck_k = 0;
      continue;
    }
    const std::vector<int8_t> *rows = nullptr;
    if (ab_prof) {
      auto it = abp.by_key.find(AbpRows::cell_key_of(cells[pi], n, fh_m));
      if (it == abp.by_key.end() || it->second.empty()) {
        cells_prof_dead++;
        cells_done++;
        if (resuming && pi == res_pi) resuming = false;
        ck_pi = pi + fh_nshard; ck_batch = 0; ck_k = 0;
        continue;
      }
      if (it->second.size() / 16 <= abp_cap) rows = &it->second;
      else cells_prof_uncap++;
    }
    long long cur_batch = 0, cell_done_ct = 0;
    bool cell_stop = false;
    const long long cs_start = cand;
    const auto cs_t0 = Clock::now();
    double cs_sec_at_buf = -1;
    ck_pi = pi;
    if (!(resuming && pi == res_pi)) { ck_batch = 0; ck_k = 0; }

    // ---- the whole cell's stream on the GPU, in the reference's order ----
    bs_cell cell;
    memset(&cell, 0, sizeof cell);
    for (int c = 0; c < fh_m; c++) { cell.tx[c] = (int8_t)cells[pi].px[c]; cell.ty[c] = (int8_t)cells[pi].py[c]; }
    cell.pinX = pinC;
    cell.pinY = pinD;
    bs_cell_stats cst;
    long long nout = 0;
    if (surv.size() < 2 * (size_t)(1 << 20)) surv.resize(2 * (size_t)(1 << 20));
    rc = bs_cd_stream(ctx, &cell, 1, &so, surv.data(), nullptr, (long long)surv.size() / 2, &nout, &cst);
    for (int retry = 0; rc == BS_ERR_CAP && retry < 3; retry++) {
      // the output or the device survivor buffer was short: grow to the reported size
      surv.resize(std::max(surv.size(), 2 * (size_t)nout));
      so.survivor_cap = std::max(so.survivor_cap, nout);
      rc = bs_cd_stream(ctx, &cell, 1, &so, surv.data(), nullptr, (long long)surv.size() / 2, &nout, &cst);
    }
    // stopped by SIGTERM: the loop below sees g_sigterm and takes nothing of this cell;
    // stopped by the wall: the cell's survivors so far are processed and drained as usual
    const bool walled = rc == BS_WALLED;
    if (walled) cells_walled++;
    if (rc == BS_STOPPED || rc == BS_WALLED) rc = BS_OK;
    if (rc) return fail_gpu(rc, "bs_cd_stream");
    // flat scores of every survivor (stream order), computed on the GPU
    surv_score.assign((size_t)nout, 0);
    if (nout > 0 && (cell_order || score_max > 0) && cellsize == 0) {
      std::vector<int64_t> ord((size_t)nout);
      std::vector<int32_t> sc((size_t)nout);
      long long nk = 0;
      rc = bs_flat_topk(ctx, surv.data(), nout, nout, 0, ord.data(), sc.data(), &nk);
      if (rc) return fail_gpu(rc, "bs_flat_topk");
      for (long long t = 0; t < nk; t++) surv_score[(size_t)ord[t]] = sc[t];
    }

    std::vector<long long> cellbuf;  // survivor indices of the current drain batch
    auto handle_result = [&](const int *Ci, const int *Di, int r, long long nodes, const int8_t *A8,
                             const int8_t *B8, long long rank) {
      if (r == 4 || (r == 0 && test_ierr)) {
        // the first shift whose NPAF is not zero (under the test hook, the first shift), as
        // the reference's check names it (wz_match.cpp:1328-1335)
        int A[64], B[64], bad = 1;
        for (int i = 0; i < n1; i++) { A[i] = A8[i]; B[i] = B8[i]; }
        if (!test_ierr)
          while (bad < n && npaf_at(A, B, n1, Ci, Di, n, bad) == 0) bad++;
        printf("FH_INTERNAL_ERROR: completer FOUND but NPAF[%d] != 0\n", bad);
        printf("RESULT: INTERNAL ERROR at candidate idx=%lld pi=%lld — arm stopped, candidate NOT marked attempted, checkpoint NOT advanced\n",
               cand, pi);
        fflush(stdout);
        exit(5);
      }
      nodes_total += nodes;
      if (cand_log) printf("CAND idx=%lld ci=%lld pi=%lld r=%d nodes=%lld ns=0\n", cand, rank, pi, r, nodes);
      if (r >= 2) bt_entered++;
      if (test_stop > 0 && ++test_ct >= test_stop) { g_sigterm = 1; fh_stop = true; }
      if (r == 1) pre_rej++;
      else if (r == 2) clean_no++;
      else if (r == 3) aborted_ct++;
      else if (r == 0) {
        hit_idx = cand;
        found = true;
        fh_stop = true;
        double t = secs_since(T0);
        int A[64], B[64];
        for (int i = 0; i < n1; i++) { A[i] = A8[i]; B[i] = B8[i]; }
        int sa = 0, sb = 0, sc2 = 0, sd = 0;
        for (int i = 0; i < n1; i++) { sa += A[i]; sb += B[i]; }
        for (int i = 0; i < n; i++) { sc2 += Ci[i]; sd += Di[i]; }
        printf("\n*** BS(%d,%d) FOUND ***  (firsthit probe)\n", n1, n);
        printf("sig = (%d,%d,%d,%d)\n", sa, sb, sc2, sd);
        print_seq("A", A, n1);
        print_seq("B", B, n1);
        print_seq("C", Ci, n);
        print_seq("D", Di, n);
        int maxv = 0;
        for (int s = 1; s <= n; s++) maxv = std::max(maxv, std::abs(npaf_at(A, B, n1, Ci, Di, n, s)));
        printf("VERIFY: max |NPAF[s]| over s=1..%d = %d%s", n, maxv, maxv == 0 ? "  (NPAF==0 confirmed)\n" : "  (NONZERO!)\n");
        long long fsc = 0;
        for (int s = 1; s <= n; s++) {
          int cdv = 0;
          for (int i = 0; i + s < n; i++) cdv += Ci[i] * Ci[i + s] + Di[i] * Di[i + s];
          fsc += std::abs(cdv);
        }
        printf("FIRSTHIT: idx=%lld profile_rank=%lld nodes_this_cand=%lld score=%lld elapsed=%gs", hit_idx, pi,
               nodes, fsc, t);
        if (stream_total > 0) printf("  frac_depth=%g", (double)hit_idx / stream_total);
        printf("\n");
        fflush(stdout);
      }
    };
    // complete survivors `idx` (in this order) on the GPU with first-hit semantics; the
    // callback sees results in order until a stop. `ranks` are drain ranks for the log.
    auto complete_list = [&](const std::vector<long long> &idx, size_t start, size_t stop_at,
                             const std::function<void(size_t)> &after_one) {
      const size_t CH = 8192;
      for (size_t b0 = start; b0 < stop_at && !(found || g_sigterm); b0 += CH) {
        size_t b1 = std::min(stop_at, b0 + CH);
        std::vector<bs_ab_cand> cs(b1 - b0);
        for (size_t t = b0; t < b1; t++) {
          bs_ab_cand &x = cs[t - b0];
          memset(&x, 0, sizeof x);
          x.c = surv[2 * (size_t)idx[t]];
          x.d = surv[2 * (size_t)idx[t] + 1];
          x.row_off = 0;
          x.nrows = rows ? (int32_t)(rows->size() / 16) : 0;
        }
        std::vector<int32_t> v(cs.size());
        std::vector<long long> nd(cs.size());
        std::vector<int8_t> A8(cs.size() * n1), B8(cs.size() * n1);
        int r2 = bs_complete_ab_batch(ctx, cs.data(), (long long)cs.size(), rows ? rows->data() : nullptr,
                                      rows ? (long long)(rows->size() / 16) : 0, &abo, v.data(), nd.data(),
                                      A8.data(), B8.data());
        if (r2 && r2 != BS_STOPPED) exit(fail_gpu(r2, "bs_complete_ab_batch"));
        for (size_t t = b0; t < b1; t++) {
          if (found || g_sigterm) break;
          int Ci[64], Di[64];
          unpack_seq(surv[2 * (size_t)idx[t]], n, Ci);
          unpack_seq(surv[2 * (size_t)idx[t] + 1], n, Di);
          int r = v[t - b0];
          if (r < 0) { printf("RESULT: INTERNAL ERROR: candidate %zu of a batch was not completed (%d)\n", t, r); exit(5); }
          handle_result(Ci, Di, r, nd[t - b0], &A8[(t - b0) * n1], &B8[(t - b0) * n1], (long long)t);
          after_one(t);
        }
      }
    };
    auto drain = [&]() {
      if (resuming && pi == res_pi && cur_batch < res_batch) {
        cur_batch++;
        cellbuf.clear();
        return;
      }
      if (drain_top > 0 && cur_batch >= drain_batches) {
        resuming = false;
        cellbuf.clear();
        if (!cell_stop) { cell_stop = true; cells_capped++; }
        return;
      }
      size_t start = 0;
      if (resuming && pi == res_pi && cur_batch == res_batch) {
        start = (size_t)std::min((long long)cellbuf.size(), res_k);
        resuming = false;
      }
      // stable sort of the batch by flat score on the GPU (bs_flat_topk over the batch)
      std::vector<uint64_t> bw(2 * cellbuf.size());
      for (size_t t = 0; t < cellbuf.size(); t++) {
        bw[2 * t] = surv[2 * (size_t)cellbuf[t]];
        bw[2 * t + 1] = surv[2 * (size_t)cellbuf[t] + 1];
      }
      size_t stop_at = cellbuf.size();
      if (drain_top > 0 && cur_batch < drain_batches) stop_at = std::min(cellbuf.size(), (size_t)drain_top);
      std::vector<int64_t> ord(cellbuf.size());
      long long nk = 0;
      if (!cellbuf.empty()) {
        int r3 = bs_flat_topk(ctx, bw.data(), (long long)cellbuf.size(), (long long)cellbuf.size(),
                              (long long)stop_at, ord.data(), nullptr, &nk);
        if (r3) exit(fail_gpu(r3, "bs_flat_topk"));
      }
      std::vector<long long> sorted((size_t)nk);
      for (long long t = 0; t < nk; t++) sorted[(size_t)t] = cellbuf[(size_t)ord[t]];
      complete_list(sorted, start, (size_t)nk, [&](size_t t) {
        ck_batch = cur_batch;
        ck_k = (long long)t + 1;
        maybe_ckpt();
      });
      if (!(found || g_sigterm)) {
        cur_batch++;
        ck_batch = cur_batch;
        ck_k = 0;
        if (drain_top > 0 && cur_batch >= drain_batches) { cell_stop = true; cells_capped++; }
      }
      cellbuf.clear();
    };

    // ---- the probe sequence of the reference (wz_match.cpp:2715-2808) over the survivors ----
    std::vector<long long> nonbuf;  // eligible survivors of the non-buffered path
    for (long long i = 0; i < nout; i++) {
      if (fh_stop || g_sigterm) { cell_stop = true; break; }
      if (cell_stop) break;
      cand++;
      if ((cand & 255) == 0 && secs_since(last_prog) >= prog_sec) {
        last_prog = Clock::now();
        printf("[firsthit progress] candidates_streamed=%lld  pre_filter_rejected=%lld  score_rejected=%lld  clean_no_AB=%lld  budget_aborted=%lld  total_AB_nodes=%lld  [%gs]\n",
               cand, pre_rej, score_rej, clean_no, aborted_ct, nodes_total, secs_since(T0));
        fflush(stdout);
      }
      if (dump) {
        int Ci[64], Di[64];
        unpack_seq(surv[2 * i], n, Ci);
        unpack_seq(surv[2 * i + 1], n, Di);
        for (int t = 0; t < n; t++) fprintf(dump, "%d ", Ci[t]);
        fprintf(dump, "| ");
        for (int t = 0; t < n; t++) fprintf(dump, "%d ", Di[t]);
        fprintf(dump, "\n");
      }
      if (cellsize > 0) {
        long long c = cand - cs_start;
        if (c == buf_cap) cs_sec_at_buf = secs_since(cs_t0);
        if (c >= cellsize) cell_stop = true;
        continue;
      }
      long long sc = -1;
      if (score_max > 0 || cell_order) sc = surv_score[(size_t)i];
      if (score_max > 0 && sc > score_max) { score_rej++; continue; }
      if (cell_order) {
        cellbuf.push_back(i);
        if ((long long)cellbuf.size() >= buf_cap) drain();
        if (max_cand > 0 && cand >= max_cand) fh_stop = true;
        continue;
      }
      // non-buffered path: completion order = eligible stream order
      if (resuming && pi == res_pi) {
        if (cell_done_ct < res_k) { cell_done_ct++; continue; }
        resuming = false;
      }
      std::vector<long long> one{i};
      complete_list(one, 0, 1, [&](size_t) {
        cell_done_ct++;
        ck_batch = 0;
        ck_k = cell_done_ct;
        maybe_ckpt();
      });
      if (max_cand > 0 && cand >= max_cand) fh_stop = true;
    }
    if (cellsize > 0) {
      long long c = cand - cs_start;
      printf("CELLSIZE pi=%lld cand=%lld capped=%d partial=%d sec=%g sec_at_buf=%g leaves=%lld hall_ok=%lld\n", pi, c,
             c >= cellsize ? 1 : 0, fh_stop ? 1 : 0, secs_since(cs_t0), cs_sec_at_buf, cst.leaves, cst.ok);
      printf("CDSTAT pi=%lld dfs_nodes=%lld cd_prune=%d hall_fast=1\n", pi, cst.nodes, env_i("WZ_FH_CD_PRUNE", 0));
      fflush(stdout);
    }
    if (cell_order && !cellbuf.empty() && (!cell_stop || walled)) drain();
    if (!fh_stop && !g_sigterm) {
      cells_done++;
      if (cand == cs_start) cells_empty++;
      ck_pi = pi + fh_nshard;
      ck_batch = 0;
      ck_k = 0;
      write_ckpt();
    }
  }
  if (g_sigterm) fh_stop = true;
  const double t = secs_since(T0);
  const long long completed_tested = clean_no + aborted_ct + (hit_idx >= 0 ? 1 : 0);
  write_ckpt();
  printf("\n=== FIRSTHIT SUMMARY (n=%d, sig %d,%d,%d,%d, shard %d/%d) ===\n", n, SA, SB, SC, SD, fh_shard, fh_nshard);
  printf("candidates_streamed=%lld  pre_filter_rejected=%lld  score_rejected=%lld\n", cand, pre_rej, score_rej);
  printf("backtracks_entered=%lld  clean_no_AB=%lld  budget_aborted=%lld  total_AB_nodes=%lld  cells_done=%lld (skip=%d)  ab_prof=%d  cells_prof_dead=%lld  cells_prof_uncap=%lld  cells_orbit_dup=%lld  cells_empty=%lld  cum_done=%lld  cum_dup=%lld  cum_dead=%lld  cum_empty=%lld  cells_capped=%lld (drain_top=%lld batches=%lld)  cells_walled=%lld (wall_sec=%lld)  range_end=%d  pins_dropped=%d  tested_cum=%lld  resume_pi=%lld  resume_batch=%lld  resume_k=%lld\n",
         completed_tested, clean_no, aborted_ct, nodes_total, cells_done, fh_skip, ab_prof ? 1 : 0, cells_prof_dead,
         cells_prof_uncap, cells_orbit_dup, cells_empty, cum_done_base + cells_done, cum_dup_base + cells_orbit_dup,
         cum_dead_base + cells_prof_dead, cum_empty_base + cells_empty, cells_capped, drain_top, drain_batches,
         cells_walled, wall_sec, fh_end, pins_dropped ? 1 : 0, tested_base + completed_tested, ck_pi, ck_batch, ck_k);
  if (hit_idx >= 0) printf("RESULT: FOUND at idx=%lld\n", hit_idx);
  else if (g_sigterm) printf("RESULT: INTERRUPTED (SIGTERM) — counts are LOWER BOUNDS, stream NOT exhausted\n");
  else if (fh_end > 0 && !fh_stop) printf("RESULT: RANGE EXHAUSTED — this arm completed its owned cells [skip,end)\n");
  else printf("RESULT: NO HIT within probe budget — NOT a proof of absence\n");
  printf("Time: %gs\n", t);
  fflush(stdout);
  if (dump) fclose(dump);
  bs_ctx_destroy(ctx);
  (void)G_T0;
  return hit_idx >= 0 ? 0 : 3;
}
