/*
 * bsfh.h - C ABI of the GB300 first-hit search library (libbsfh.so).
 *
 * One context per host thread. The context owns its device buffers and a CUDA stream.
 * All entry points return 0 (BS_OK) or a negative BS_ERR_* code; none throws. Sequences are
 * +1/-1. In "packed" form a sequence of length L <= 64 is one uint64 word with bit i set
 * when element i is +1; a (C,D) pair is two consecutive words.
 *
 * Each entry point names the reference interface it replaces, as a path within
 * DanielGord0n/BS45_Quantum_Explorer (file:line).
 */
#ifndef BSFH_H
#define BSFH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  BS_STOPPED = 1,       /* stopped early by the context's stop flag: the results cover the
                           part completed (the reference's SIGTERM path, lower bounds) */
  BS_WALLED = 2,        /* bs_cd_stream stopped by its wall limit (WZ_FH_WALL_SEC): the
                           survivors cover the part streamed */
  BS_OK = 0,
  BS_ERR_ARG = -1,      /* bad argument (size, length, mode, null pointer) */
  BS_ERR_CUDA = -2,     /* a CUDA runtime call failed */
  BS_ERR_NOMEM = -3,    /* device or host allocation failed */
  BS_ERR_TIMEOUT = -4,  /* a device wait ran out of its iteration limit; results invalid */
  BS_ERR_INTERNAL = -5, /* an internal consistency check failed (e.g. NPAF recheck) */
  BS_ERR_CAP = -6,      /* an output capacity was exceeded; the call reports how much it needs */
  BS_ERR_NODEV = -7     /* no CUDA device, or not an sm_103 device */
};

/* Hall (Thm 2.4) filter forms. */
enum {
  BS_HALL_FP64 = 0,      /* CUDA-core FP64 in the reference's expression order (exact) */
  BS_HALL_TC_FP16 = 1,   /* tcgen05 tensor cores, +-1 x fp16 quantised table, FP32 accumulate,
                            proven margin, FP64 recheck of the margin band (exact decisions) */
  BS_HALL_TC_BF16X2 = 2  /* as above with the table split hi+lo in bf16 (narrower band) */
};

typedef struct bs_ctx bs_ctx;

typedef struct {
  long long pairs;          /* pairs tested */
  long long passed;         /* pairs accepted (== the reference's hall_ok_pair_fast count) */
  long long rechecked;      /* pairs inside the tensor-core margin band, decided again by the
                               exact fixed-point test */
  long long fp64_rechecked; /* of those, pairs within the fixed-point test's own (about 1e-6
                               wide) band, decided in FP64 */
  double pass_below;        /* max pair PSD at or below which a pair certainly passes */
  double reject_above;      /* max pair PSD at or above which a pair certainly fails */
  double quant_err;         /* per-sequence |Re|,|Im| quantisation bound e of the table */
  int mode;
} bs_hall_stats;

/* Library identity and error text. */
int bs_version(void);
const char *bs_strerror(int code);

/* Create a context for BS(n+1,n) with signature (a,b,c,d) on CUDA device `device`.
 * Builds the Hall tables on the host with libm exactly as init_hall_tables does
 * (src/solver/wz_match.cpp:106-114) and uploads them. 4 <= n <= 63. */
int bs_ctx_create(int n, int a, int b, int c, int d, int device, bs_ctx **out);
void bs_ctx_destroy(bs_ctx *ctx);
/* Point an existing context at another BS(n+1,n) and signature, keeping its stream and every
 * device buffer (a serving slot reuses one context across jobs instead of allocating, and so
 * synchronising the device, per job). Waits for the context's queued work first. On failure
 * the tables are left half loaded: only another bs_ctx_retarget (which then reloads them all)
 * or bs_ctx_destroy may follow. No counterpart in the reference (one process per lane there). */
int bs_ctx_retarget(bs_ctx *ctx, int n, int a, int b, int c, int d);
/* Use a caller-owned CUDA stream (cudaStream_t) for every later call; NULL = the context's own. */
int bs_ctx_set_stream(bs_ctx *ctx, void *cuda_stream);
/* Last error recorded by the device (timeouts), cleared on read. */
int bs_ctx_device_status(bs_ctx *ctx);
/* The context's stop flag: one int32 of pinned host memory mapped into the device, initially
 * 0. Storing a nonzero value (a plain store, safe in a signal handler) makes the context's
 * running and later bs_cd_stream and bs_complete_ab_batch calls stop within one device round
 * (bs_cd_stream: one launch of at most round_us; bs_complete_ab_batch: the warps poll it every
 * 1,024 search steps and before each candidate) and return BS_STOPPED with the part completed.
 * Store 0 to clear it. Replaces the reference's g_fh_sigterm / cooperative stop
 * (src/solver/wz_match.cpp:640-642, 712-713: a stream-walled arm that ignored SIGTERM hung
 * its lane driver past walltime). */
volatile int32_t *bs_ctx_stop_flag(bs_ctx *ctx);
/* Kernel timing, for measurement: when enabled, the dominant kernel of each call (the Hall
 * kernel) is bracketed by CUDA events on the context stream. _read synchronises, returns the
 * summed duration and launch count since the last read, and the number of kernels this
 * context has launched in total. No reference counterpart (instrumentation). */
int bs_ctx_timing(bs_ctx *ctx, int enable);
int bs_ctx_timing_read(bs_ctx *ctx, double *ms, long long *timed_launches, long long *all_launches);

/* ---- Hall filter --------------------------------------------------------------------
 * Replaces hall_ok_pair_fast(X, L, Y, L) / hall_ok_single && hall_ok
 * (src/solver/wz_match.cpp:117-181) over a batch: pass[i] = 1 exactly when the reference
 * accepts pair i. Host buffers: XY is npairs rows of 2L int8 (C then D), L = n. */
int bs_hall_filter_batch(bs_ctx *ctx, const int8_t *XY, long long npairs, int mode,
                         uint8_t *pass, bs_hall_stats *stats);
/* Same, host packed input (2 words per pair). */
int bs_hall_filter_packed(bs_ctx *ctx, const uint64_t *bits, long long npairs, int mode,
                          uint8_t *pass, bs_hall_stats *stats);
/* Same, device-resident input and output, enqueued on the context stream. stats (host, may
 * be NULL) is filled after a stream synchronise when non-NULL. */
int bs_hall_filter_dev(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                       uint8_t *d_pass, bs_hall_stats *stats);
/* Allocation-free form of bs_hall_filter_dev (tensor-core fp16 form + FP64 recheck of the
 * margin band), for callers that may not allocate device memory: code running under a
 * device-memory budget owned by a scheduler or host framework, or latency-sensitive code in
 * the middle of overlapped multi-stream work, where cudaMalloc / cudaFree would synchronise
 * the device. No counterpart in the reference. It needs no context and allocates nothing:
 * its scratch (screen and band lists, counters, status word, tables) is one fixed static
 * device array of about 8.2 MiB, which every GPU that loads the library keeps until the process
 * exits.
 * n is the sequence length (4 <= n <= 63); d_bits holds 2 words per pair and d_pass
 * receives the decisions, both device memory owned by the caller; at most 1,048,576 pairs
 * per call (BS_ERR_CAP beyond); npairs = 0 only checks the set-up. The work is enqueued on
 * `stream` (a cudaStream_t; NULL is the legacy default stream), and every call ends by
 * synchronising that stream to read the status word back, so no call can be made inside
 * stream capture. The first call on a device, and the first call with a new n, set the
 * scratch up (device symbol address, kernel attributes, tables uploaded from static host
 * arrays).
 * Calls share the one array and keep the last call's tables and band list; the counters are
 * cleared by every call. Calls that overlap on the GPU (other streams, other host threads)
 * race and must be serialised by the caller. */
int bs_hall_filter_noalloc(int n, const uint64_t *d_bits, long long npairs, uint8_t *d_pass,
                           void *stream);
/* Diagnostics: raw tensor-core accumulators for npairs (multiple of 64, <= 65536) pairs,
 * d_acc[row][208] fp32 with row 2p = C of pair p, 2p+1 = D; columns 0..100 are Re at the
 * unique angles j = 1..100, 200 and columns 104..204 the matching Im. */
int bs_hall_tc_dump_dev(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                        float *d_acc);

/* ---- C,D stream ----------------------------------------------------------------------
 * Replaces count_pairs22(n, px, py, false, pinC, pinD, leaves, ok, &sink, m, stop)
 * (src/solver/wz_match.cpp:678-784) for a batch of cells of one context (L = n): every
 * Thm 2.2 mirror-quad (C,D) whose class sums equal the cell's targets and that passes the
 * Thm 2.4 test, in the reference's emission order (cells in the given order, then DFS
 * order), with per-cell counts equal to the reference's CDSTAT dfs_nodes, leaves and
 * hall_ok (CELLSIZE) figures. The subtrees are explored in waves, in stream order: each
 * wave refines the next run of the cell's frontier to as many subtrees as keep the GPU busy,
 * and walks that run long are split further between launches, so cells of more than 10^13
 * nodes (n = 42) stream at full speed and `limit` stops early. */
typedef struct {
  int8_t tx[8], ty[8];  /* class-sum targets of C and D at modulus m (entries >= m unused) */
  int32_t pinX, pinY;   /* zero-sum pins: C[0] = +1 / D[0] = +1 (wz_match.cpp:1526-1527) */
} bs_cell;

typedef struct {
  int32_t m;                 /* class modulus of the cells: 3 or 6 */
  int32_t rev;               /* WZ_FH_STREAM_REV: reversed branch order */
  int32_t endpos;            /* WZ_FH_ENDPOS: positive-product endpoint quad */
  int32_t cd_prune;          /* WZ_FH_CD_PRUNE (wz_match.cpp:655-666, 719-731): bit 1 the root
                                quad's entry sum mod 4, bit 2 exact reachability of each mirror
                                block from depth 1; C,D side, m = 6, even L only (else no-op).
                                The survivors are the same; the node counts are the pruned
                                walk's, as the reference's CDSTAT prints them */
  int32_t hall_mode;         /* BS_HALL_* form of the leaf test */
  int32_t ab_side;           /* 1: stream the A,B side (length n+1, negative-product root quads) */
  long long target_prefixes; /* coarse split of the batch into subtrees (0 = 262144); the
                                waves refine it further as the measured subtree sizes ask */
  long long leaf_chunk;      /* leaves buffered per round (0 = 2^24) */
  long long survivor_cap;    /* device survivor buffer (0 = 2^22) */
  long long limit;           /* > 0: stop once the first `limit` survivors of the batch (in
                                stream order) are known and return only those -- the lane's
                                front-only cut (BUF_CAP x DRAIN_BATCHES survivors per cell,
                                wz_match.cpp:2656-2714, 2782-2790), which stops the
                                reference's DFS; the stats then cover the part explored */
  long long round_us;        /* longest device launch in microseconds (0 = 25,000); walks still
                                running then suspend, and when few remain the host splits them
                                into their remaining subtrees (small values exercise that path) */
  double wall_sec;           /* WZ_FH_WALL_SEC (wz_match.cpp:643-653, 715-718): > 0 abandons
                                the stream once this many seconds pass without a new survivor
                                (counted from the call's start, then from the last launch that
                                found one); the call returns BS_WALLED with the survivors of the
                                waves it completed, which the lane still drains */
  /* work sizes (0 = the defaults; bs45_quantum_explorer_gb300.tune picks them by measuring):
     fine_nodes  the DFS nodes a fine subtree is refined to (default 2e4),
     wave_nodes  the DFS nodes a wave aims at (default 8e9),
     dfs_blocks  DFS blocks per SM: 4 (64 registers), 5 (48) or 6 (40) */
  double fine_nodes;
  double wave_nodes;
  int32_t dfs_blocks;
  int32_t reserved;
} bs_stream_opts;

typedef struct { long long nodes, leaves, ok; } bs_cell_stats;

/* ---- the lane's cell list (host only: no device, no context) -----------------------------
 * Replaces the first-hit lane's cell-list block (src/solver/wz_match.cpp:1388-1886): the
 * mod-3 or mod-6 C,D profile cells surviving 2.11a (+2.11b/2.12), the ENDPOS filter, the
 * profile order (WZ_FH_PROF_ORDER 0..3), orbit canonicalisation with the quad switch and its
 * Q-closure prune, and the ORDER=3 digest "<list>:<kept>". cells[i] is raw cell i of the
 * lane (pins set as the lane sets them), kept[i] = 1 when the lane searches it (its orbit's
 * representative under canon; always 1 without). Nothing is printed. Returns BS_ERR_CAP
 * (with *ncells set) when cap is too small, 2 where the reference refuses (truncated list,
 * duplicate keys). digest (may be NULL) receives up to 40 bytes, "" unless prof_order 3.
 * A call that returns BS_ERR_CAP keeps the list it built (one list, process-wide, until the
 * next bs_cell_list call), so the same call repeated with a large enough buffer copies it
 * instead of building it again. */
typedef struct {
  int32_t m6;           /* WZ_FH_M6 (the lane's default is n >= 36) */
  int32_t thm211b;      /* WZ_THM211B (forced at n >= 36) */
  int32_t thm212;       /* WZ_THM212 (forced at n >= 36) */
  int32_t endpos;       /* WZ_FH_ENDPOS */
  int32_t orbit_canon;  /* WZ_FH_ORBIT_CANON */
  int32_t orbit_q;      /* WZ_FH_ORBIT_Q: 0, 1, 2 */
  int32_t qprune;       /* WZ_FH_ORBIT_QPRUNE */
  int32_t prof_order;   /* WZ_FH_PROF_ORDER: 0..3 */
  int32_t nshard;       /* WZ_FH_NSHARD (only the [order] balance figures use it) */
  int32_t reserved;
} bs_list_opts;

int bs_cell_list(int n, int a, int b, int c, int d, const bs_list_opts *opt, bs_cell *cells,
                 uint8_t *kept, long long cap, long long *ncells, char *digest);

/* Replaces the lane's abpMap build (src/solver/wz_match.cpp:2318-2378): for each given cell,
 * the allowed A,B class-sum rows (16 int8 each: k[8] then r[8]) of its invariant, written
 * back to back; row_off[i] / nrows[i] locate cell i's rows (cells with one invariant share
 * them). nrows[i] = 0 means no allowed row: the cell holds no base sequence and the lane
 * skips it (cells_prof_dead) -- do not pass it on as an unconstrained bs_ab_cand. The lane
 * runs cells with more than WZ_FH_AB_PROF_CAP rows unconstrained. *nrows_total = rows
 * written; BS_ERR_CAP (with *nrows_total = rows needed) when rows_cap is too small. */
int bs_ab_rows(int n, int a, int b, int m, const bs_cell *cells, long long ncells, int8_t *rows,
               long long rows_cap, long long *row_off, int32_t *nrows, long long *nrows_total);

/* out_words: 2 words (C, D) per survivor, out_cell (may be NULL): the survivor's cell index.
 * *nout always receives the survivor count; BS_ERR_CAP when it exceeds out_cap, or when one
 * wave's survivors exceed survivor_cap (then *nout is a lower bound: retry with both at
 * least *nout). */
int bs_cd_stream(bs_ctx *ctx, const bs_cell *cells, int ncells, const bs_stream_opts *opt,
                 uint64_t *out_words, uint32_t *out_cell, long long out_cap, long long *nout,
                 bs_cell_stats *stats);

/* ---- per-cell flattest-k keep -----------------------------------------------------------
 * Replaces flat_score (src/solver/wz_match.cpp:2569-2583) and drain()'s stable_sort by score
 * with its front-only cut (wz_match.cpp:2656-2714): a cell's survivors (2 words each, in
 * stream order) are split into batches of buf_cap; each batch is ordered by flat score, ties
 * in stream order, and its first `keep` entries (keep <= 0: all) are returned as stream
 * indices in `order`, batch after batch, with their scores (may be NULL). *nkept = entries. */
int bs_flat_topk(bs_ctx *ctx, const uint64_t *words, long long nsurv, long long buf_cap,
                 long long keep, int64_t *order, int32_t *scores, long long *nkept);
/* Device-resident form: d_order / d_scores_sorted hold ceil(nsurv/buf_cap) slots of
 * min(keep, buf_cap) entries each (a short last batch leaves its tail unwritten); d_scores
 * (nsurv) receives every survivor's score. Enqueued on the context stream. */
int bs_flat_topk_dev(bs_ctx *ctx, const uint64_t *d_words, long long nsurv, long long buf_cap,
                     long long keep, int64_t *d_order, int32_t *d_scores_sorted,
                     int32_t *d_scores);

/* ---- A,B completion --------------------------------------------------------------------
 * Replaces fh_complete_ab(C, D) (src/solver/wz_match.cpp:1298-1341) with fh_ab_search
 * (:1171-1293) over a batch: for candidate i, verdict[i] and nodes[i] equal the reference's
 * return value and charged node count (the fh_nodes_total delta), and on a hit A,B (n+1
 * int8 each, at A + i*(n+1)) equal its first completion. The cell's allowed A,B class-sum
 * rows (AbpRow, wz_match.cpp:970: k[8] then r[8], int8) are rows[row_off .. row_off+nrows);
 * nrows = 0 runs unconstrained (FH_ABP == nullptr). Verdicts: 0 hit, 1 prefilter, 2 clean
 * no, 3 budget abort, 4 NPAF recheck failed, -1 not run (after an earlier hit in first_hit
 * mode, or stopped), -2 wall limit (max_seconds) reached. */
typedef struct {
  uint64_t c, d;        /* packed C, D (length n) */
  long long row_off;    /* first allowed row of the candidate's cell */
  int32_t nrows;        /* allowed rows (0 = unconstrained), <= 65535 */
  int32_t reserved;
} bs_ab_cand;

typedef struct {
  long long budget;     /* WZ_FH_AB_BUDGET: nodes per candidate, 0 = exact */
  int32_t outer_k;      /* WZ_FH_OUTER_K: 0 | 2 | 3 */
  int32_t early;        /* WZ_FH_EARLY_CHECK (reference default 1) */
  int32_t canon;        /* root + reversal canonicalisation (1 unless WZ_FH_NO_CANON) */
  int32_t m;            /* class modulus of the rows: 3 or 6 */
  int32_t first_hit;    /* 1: candidates after the lowest-index hit are not run */
  int32_t a2;           /* WZ_FH_A2: 0 off, 2 the A2 row-reachability prune (wz_match.cpp:
                           977-1047, 1069-1072); mode 1, the reference's shadow instrument, is
                           not built (BS_ERR_ARG) */
  double max_seconds;   /* per-candidate wall limit on the device (0 = none) */
  int32_t blocks_per_sm; /* resident completer blocks of 8 warps per SM: 1, 2 or 3 (0 = 2) */
  int32_t reserved;
} bs_ab_opts;

int bs_complete_ab_batch(bs_ctx *ctx, const bs_ab_cand *cands, long long ncand,
                         const int8_t *rows, long long nrows_total, const bs_ab_opts *opt,
                         int32_t *verdict, long long *nodes, int8_t *A, int8_t *B);

/* ---- exact verification and the autocorrelation join ------------------------------------
 * bs_npaf_verify_batch replaces npaf_at over s = 1..n+1 (src/solver/wz_match.cpp:184-192;
 * tools/verify_npaf.py:42-53) for a batch: quads are 4 words (A, B of length n+1, C, D of
 * length n); maxabs[i] = max_s |NPAF(s)|, 0 for a base sequence. */
int bs_npaf_verify_batch(bs_ctx *ctx, const uint64_t *quads, long long count, int32_t *maxabs);

/* Replaces the WZ_JOIN22 hash join (src/solver/wz_match.cpp:2894-3104): every (A,B) of
 * ab_words (length n+1) is matched against every (C,D) of cd_words (length n) with the same
 * autocorrelation vector AB[s] = -CD[s], s = 1..n; each match is verified with the exact
 * NPAF on the device and written as a quad (4 words). All matches are returned (the
 * reference keeps one C,D per key). BS_ERR_CAP when more than out_cap; *nout = matches,
 * *key_hits = equal-key pairings examined. */
int bs_join_quads(bs_ctx *ctx, const uint64_t *cd_words, long long ncd, const uint64_t *ab_words,
                  long long nab, uint64_t *out_quads, long long out_cap, long long *nout,
                  long long *key_hits);

/* Pack host int8 sequences (rows of L values) into words. No device work. */
int bs_pack_rows(const int8_t *seq, long long rows, int L, uint64_t *words);

/* Seeded Hall-microbench input on the device (2 words per pair, length ctx n): the first
 * half i.i.d. +-1, the second half mirror-quad pairs with sum C = sum D = 0. No reference
 * counterpart: it generates the synthetic workload the benchmark times. */
int bs_gen_hall_pairs_dev(bs_ctx *ctx, long long npairs, uint64_t seed, uint64_t *d_words);

#ifdef __cplusplus
}
#endif
#endif
