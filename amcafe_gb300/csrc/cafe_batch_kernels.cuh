// Batched forms of the step kernels: one launch per kernel for every
// realisation of an ensemble (no counterpart in the reference, which runs one
// realisation per MPI job, main1.C:18-101).
//
// Each realisation keeps its own device state (CafeDev, CafeConsts and its
// step parameters at CafeDev::Pd), described in device memory by one
// CafeBatchReal. A batched launch's blocks are divided among the realisations
// by a table of first blocks per kernel (start[kind][r], ascending): block x
// belongs to the realisation r with start[r] <= x < start[r+1] and runs the
// plain kernel's body (the d_* functions of cafe_kernels.cu) as its block
// x - start[r] of start[r+1] - start[r]. So every realisation executes the same
// code on the same launch shape as its plain graphed step, and gets the same
// results; the event loop runs one block per realisation, all at once.
// Realisations without the flag `active` (finished, or stepped on the plain
// path this time) leave their blocks idle.

enum {
  BK_RESET_A = 0,  // CTR_HOT = 0 (before the melt pass)
  BK_MELT,
  BK_PBOX0,
  BK_PBOX1,
  BK_LIST,
  BK_RESET_B,      // CTR_NLIQ = 0 (after the liquid-list pass used it)
  BK_ACOUNT,
  BK_SCAN,
  BK_ASCATTER,
  BK_GATHER,
  BK_LCOUNT,
  BK_SCANP,
  BK_LSCATTER,
  BK_RESET_C,      // CTR_SLOW = CTR_NPAIRS = 0
  BK_PREP,
  BK_GEO,
  BK_ORDER,
  BK_LOOP,
  BK_FINAL,
  BK_WB,
  BK_M2S,
  BK_REPORT,       // CTR_HOT and the error word into the host-visible report
  BK_COUNT
};

struct CafeBatchReal {
  CafeDev D;
  CafeConsts K;
  int act_chunks;   // cafe_sim::act_chunks
  int allow_fast;   // 0: the reference's full per-event scan
  long long nblk_act, nblk_pos;
};

struct CafeBatchArgs {
  const CafeBatchReal *__restrict__ R;  // [n]
  const int *__restrict__ start;        // [BK_COUNT][n + 1]
  const int *__restrict__ active;       // [n]
  int *report;                          // [2 n]: CTR_HOT, error word
  int n;
};

// The realisation r, block b of nb, of this block of a batched launch of
// `kind`; false for blocks of inactive realisations.
__device__ __forceinline__ bool cafe_batch_slot(const CafeBatchArgs &B, int kind, int &r, int &b, int &nb) {
  const int *st = B.start + (long long)kind * (B.n + 1);
  const int x = blockIdx.x;
  int lo = 0, hi = B.n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (st[mid] <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  r = lo;
  b = x - st[r];
  nb = st[r + 1] - st[r];
  return b >= 0 && b < nb && B.active[r];
}

#define CAFE_BATCH_BLOCK(kind)                        \
  int r, b, nb;                                       \
  if (!cafe_batch_slot(B, kind, r, b, nb)) return;    \
  const CafeBatchReal &R = B.R[r]

__global__ void kb_reset_a(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_RESET_A);
  if (threadIdx.x == 0) R.D.ctr[CTR_HOT] = 0;
}
__global__ void kb_melt(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_MELT);
  d_melt(R.D, R.K, R.D.Pd, b, nb);
}
__global__ void kb_solid2mushy_pbox0(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_PBOX0);
  d_solid2mushy_pbox(R.D, R.K, R.D.Pd, 0, b, nb);
}
__global__ void kb_solid2mushy_pbox1(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_PBOX1);
  d_solid2mushy_pbox(R.D, R.K, R.D.Pd, 1, b, nb);
}
__global__ void kb_solid2mushy_list(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_LIST);
  d_solid2mushy_list(R.D, R.K, b, nb);
}
__global__ void kb_reset_b(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_RESET_B);
  if (threadIdx.x == 0) R.D.ctr[CTR_NLIQ] = 0;
}
__global__ void kb_active_count(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_ACOUNT);
  d_active_count(R.D, R.K, R.D.Pd, R.act_chunks, R.nblk_act, b, nb);
}
__global__ void __launch_bounds__(1024) kb_scan_blocks(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_SCAN);
  d_scan_blocks(R.D.blk, R.nblk_act, R.D.ctr + CTR_NA, b, nb);
}
__global__ void kb_active_scatter(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_ASCATTER);
  d_active_scatter(R.D, R.K, R.D.Pd, R.act_chunks, R.nblk_act, b, nb);
}
__global__ void kb_gather(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_GATHER);
  d_gather(R.D, R.K, R.D.Pd, b, nb);
}
__global__ void kb_lists_count(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_LCOUNT);
  d_lists_count(R.D, b, nb);
}
__global__ void __launch_bounds__(1024) kb_scan_pairs(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_SCANP);
  d_scan_pairs(R.D.blk, R.nblk_pos, R.D.ctr + CTR_NA, R.D.ctr + CTR_NVS2, R.D.ctr + CTR_NROWS, b, nb);
}
__global__ void kb_lists_scatter(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_LSCATTER);
  d_lists_scatter(R.D, b, nb);
}
__global__ void kb_reset_c(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_RESET_C);
  if (threadIdx.x == 0) {
    R.D.ctr[CTR_SLOW] = 0;
    R.D.ctr[CTR_NPAIRS] = 0;
    R.D.fill_seq[0] = 0;  // the event loop's fill hand-off (two blocks per realisation)
    R.D.fill_seq[1] = 0;
  }
}
__global__ void kb_rows_prep(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_PREP);
  d_rows_prep(R.D, R.K, b, nb);
}
__global__ void kb_rows_geo(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_GEO);
  d_rows_geo(R.D, R.K, b, nb);
}
__global__ void kb_rows_order(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_ORDER);
  d_rows_order(R.D, R.K, b, nb);
}
__global__ void __launch_bounds__(CAFE_LOOP_THREADS, 1) kb_event_loop(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_LOOP);
  d_event_loop(R.D, R.K, R.D.Pd, R.D.act_cap + 1, R.allow_fast, b, nb);
}
__global__ void kb_rows_finalize(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_FINAL);
  d_rows_finalize(R.D, b, nb);
}
__global__ void kb_writeback(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_WB);
  d_writeback(R.D, R.K, b, nb);
}
__global__ void kb_mushy2solid(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_M2S);
  d_mushy2solid(R.D, R.K, b, nb);
}
__global__ void kb_report(CafeBatchArgs B) {
  CAFE_BATCH_BLOCK(BK_REPORT);
  if (threadIdx.x == 0) {
    B.report[2 * r] = R.D.ctr[CTR_HOT];
    B.report[2 * r + 1] = *R.D.err;
  }
}
#undef CAFE_BATCH_BLOCK
