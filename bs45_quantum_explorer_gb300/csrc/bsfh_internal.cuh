// bsfh_internal.cuh - shared definitions of the GB300 first-hit library (not part of the ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>

#include "../../include/bsfh.h"

#define BS_MAXL 64          // longest sequence held in one packed word
#define BS_TC_COLS 208      // tensor-core N: 104 Re columns + 104 Im columns
#define BS_TC_IM0 104       // first Im column of a dumped accumulator row
#define BS_TC_NANG 101      // unique Hall angles (j = 1..100 and 200)

// One tensor-core table image: 208 rows (columns of the DFT) x 64 halves, stored in the
// 128-byte-swizzled K-major layout the UMMA shared-memory descriptor reads. The 101 unique
// angles u sit in 104 slots (3 zero rows); slot order is any permutation, since the test takes
// a maximum over angles. Slots 0..31 hold the screening angles (32 angles spread evenly over
// the grid, u = round(k * 100 / 31)), so that rows [0, 64) -- their cos rows, then their sin
// rows -- are the B operand of the screening MMA (N = 64). The full table is two blocks, each
// a contiguous run of rows one MMA of N = 2 x (slots in the block) reads:
//   block 0 = slots 0..63: rows [cos 0..31][sin 0..31][cos 32..63][sin 32..63] (rows 0..127)
//   block 1 = slots 64..103: rows [cos 64..103][sin 64..103] (rows 128..207)
#define BS_TC_PART_BYTES (BS_TC_COLS * 128)
#define BS_TC_BLK0 64
#define BS_TC_BLK1 40
#define BS_TC_SCREEN 32
static inline __host__ __device__ int bs_tc_screen_u(int k) { return (k * 100 + 15) / 31; }
// slot of angle u: the screening angles first (in order), then the others in increasing u
static inline __host__ __device__ int bs_tc_slot_of(int u) {
  int k = (u * 31 + 50) / 100;  // the screening index u would have
  if (k < BS_TC_SCREEN && bs_tc_screen_u(k) == u) return k;
  int below = 0;  // screening angles below u
  for (int j = 0; j < BS_TC_SCREEN; j++) below += bs_tc_screen_u(j) < u;
  return BS_TC_SCREEN + u - below;
}
static inline __host__ __device__ int bs_tc_row_of_slot(int slot, int sin_part) {
  if (slot < BS_TC_BLK0) return 64 * (slot / 32) + (sin_part ? 32 : 0) + slot % 32;
  return 2 * BS_TC_BLK0 + (sin_part ? BS_TC_BLK1 : 0) + (slot - BS_TC_BLK0);
}
static inline __host__ __device__ int bs_tc_row(int u, int sin_part) {
  return bs_tc_row_of_slot(bs_tc_slot_of(u), sin_part);
}

struct bs_hall_tc_form {
  int nparts;            // 1 (fp16) or 2 (bf16 hi + lo)
  int fmt;               // UMMA operand format: 0 = f16, 1 = bf16
  double quant_err;      // per-sequence bound e on |Re - Re_q|, |Im - Im_q|
  float pass_below;      // certified thresholds on the fp32 max pair PSD
  float reject_above;
  uint8_t *d_image;      // nparts * BS_TC_PART_BYTES
};

// The Hall tables in fixed point for the margin band's second test: T = round(t * 2^30) for
// the 101 unique angles, [cos 101 x L][sin 101 x L][row sums cos 101][row sums sin 101] int64,
// with the certified thresholds of that form (see hall.cu).
#define BS_FIX_WORDS (2 * BS_TC_NANG * BS_MAXL + 2 * BS_TC_NANG)
struct bs_hall_fix_form {
  double err;           // per-sequence bound on |Re - Re_fix|, |Im - Im_fix|
  double pass_below, reject_above;
  int64_t *d_tab;       // BS_FIX_WORDS, laid out for length L
};

struct bs_ctx {
  int n, n1, sig[4], device;
  int num_sms;
  cudaStream_t own_stream, stream;
  double *d_cos, *d_sin;     // FP64 Hall tables, [200][BS_MAXL] for j = 1..200
  double lim;                // 4n + 2 + 0.5
  bs_hall_tc_form tc[3];     // index by mode (0 unused), sequences of length n (C,D)
  bs_hall_tc_form tc_ab[3];  // the same for length n+1 (A,B)
  bs_hall_fix_form fix[2];   // fixed-point band test, lengths n (0) and n+1 (1)
  int *d_status;             // device-side error word
  unsigned long long *d_count;  // [0] band count, [1] pass count, [2] overflow flag,
                                // [3] pairs left for the FP64 test, [4] screen survivors
  // scratch for the host-buffer entry points
  uint64_t *d_bits; long long bits_cap;   // pairs
  uint8_t *d_pass; long long pass_cap;
  int8_t *d_rows; long long rows_cap;     // int8 staging for packing
  unsigned *d_unc; long long unc_cap;     // band pair indices
  unsigned *d_unc2; long long unc2_cap;   // pairs the fixed-point test leaves undecided
  unsigned *d_scr; long long scr_cap;     // pairs the tensor-core screen did not reject
  void *h_pinned; size_t pinned_bytes;
  // kernel timing (bs_ctx_timing): start/stop events around the timed kernel class
  int timing;
  int nev;                  // event pairs recorded since the last read
  cudaEvent_t ev[2 * 512];
  double timed_ms;          // accumulated duration of the timed kernels
  long long timed_launches; // launches of the timed kernels
  long long launches;       // every kernel this context has launched
  volatile int32_t *h_stop;  // the stop flag (bs_ctx_stop_flag): mapped pinned host memory
  int32_t *d_stop;           // its device address
  void *stream_bufs;        // C,D stream buffers (cd_stream.cu)
  void *ab_bufs;            // A,B completion buffers (complete.cu)
};

void bs_stream_free(bs_ctx *ctx);
// Hall filter of pairs of length L (n for C,D, n+1 for A,B), device buffers, no stats.
int bs_hall_dev_len(bs_ctx *ctx, const uint64_t *d_bits, long long npairs, int mode,
                    uint8_t *d_pass, int L);
void bs_ab_free(bs_ctx *ctx);

// Record the start / stop event of one timed kernel launch on the context stream.
void bs_timed_begin(bs_ctx *ctx);
void bs_timed_end(bs_ctx *ctx);

// Internal helpers implemented in capi.cu
int bs_cuda_fail(cudaError_t e);
int bs_ensure_dev(void **ptr, long long *cap, long long need, size_t elem);
int bs_ensure_pinned(bs_ctx *ctx, size_t bytes);

// Device wait limit: a spin or try_wait loop gives up after this many SM clock cycles,
// records BS_ERR_TIMEOUT in the context's status word and returns.
#define BS_WAIT_CYCLES (4000000000ULL)

static inline int bs_grid_for(long long work, int block, int max_blocks) {
  long long g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}
