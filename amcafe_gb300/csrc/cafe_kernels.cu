// CUDA kernels of the CA step (VoxelsCA::UpdateVoxels and TempField::
// AnalyticTempCurr, AMCAFE src/src-mpi/VoxelsCA.C:232-655, TempField.C:139-217)
// and of the per-layer operations (CleanLayer, AddLayer1 Voronoi assignment).
//
// Step pipeline (one realisation, launched by cafe_host.cu on one stream):
//   k_melt          pool box only: SetLiquid3 + BuildjID + "any cell at the
//                   liquidus" flag (VoxelsCA.C:1098-1116, TempField.C:191-206)
//   k_solid2mushy   ConvertSolid1(1) (VoxelsCA.C:780-797), in place
//   k_active_count  \ order-preserving compaction of the active set
//   k_scan_blocks    > (VoxelsCA.C:262-275): mushy, undercooled liquid and
//   k_active_scatter/  their neighbours at/above the liquidus, in index order
//   k_gather        per-position copies, neighbour positions (VoxelsCA.C:
//                   283-335), ruq offsets (VoxelsCA.C:380) by RNG jump-ahead
//   k_lists_*       vs2ind (mushy positions in order) and frontier rows
//   k_rows_*        capture-time numerators per (frontier cell, liquid
//                   neighbour), sorted per cell
//   k_event_loop    the sequential capture/nucleation loop (VoxelsCA.C:
//                   381-610), one thread block
//   k_writeback     VoxelsCA.C:633-643
//   k_mushy2solid   ConvertSolid1(0) (VoxelsCA.C:739-758), in place
// All FP64 arithmetic follows the reference's expression order; the file is
// compiled with --fmad=false so no product is fused into an add.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cafe_device.cuh"

#define CAFE_DENSE_THREADS 256
#define CAFE_CELLS_PER_THREAD 8
#define CAFE_CELLS_PER_BLOCK (CAFE_DENSE_THREADS * CAFE_CELLS_PER_THREAD)
// The active-set compaction takes `chunks` (1..4) 8-cell chunks per thread:
// more per thread on very large grids, where nearly every chunk is decided
// from its state bytes and the number of blocks dominates; one per thread
// otherwise, where the cell-by-cell tests inside the pool box set the pace.
#define CAFE_ACT_MAX_CHUNKS 4
#define CAFE_LOOP_THREADS 512
#ifdef CAFE_DETAIL_CYCLES
// clock read ordered with the surrounding memory operations and barriers
__device__ __forceinline__ long long cafe_clock_ordered() {
  long long t;
  asm volatile("mov.u64 %0, %%clock64;" : "=l"(t)::"memory");
  return t;
}
#endif

// ------------------------------------------------------------------ helpers
// Hint: bring the line holding *a into this SM's L1 (no effect on results).
__device__ __forceinline__ void cafe_prefetch_l1(const void *a) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
}
// Growth velocity of active position p (VoxelsCA.C:405): per temperature class
// with the analytic field, per cell with the EASM field.
__device__ __forceinline__ double cafe_vh(const CafeDev &D, const CafeConsts &K, int p) {
  return K.easm ? D.a_vh[p] : K.vhat_cls[D.a_cls[p]];
}

// Nucleation probability of a capture event that takes active position icap
// (VoxelsCA.C:483): rX, or with the Gaussian-undercooling extension
// rX exp(-.5 x1^2), x1 = ((tL - T) - mean) / sd / sqrt(2), the form of
// VoxelsCA.C:2545-2548, with T the captured cell's temperature.
__device__ __forceinline__ double cafe_nuc_rate(const CafeDev &D, const CafeConsts &K, int icap) {
  if (!K.nuc_gauss) return K.rX;
  double T = K.easm ? D.temp[D.act[icap]] : K.Tcls[D.a_cls[icap]];
  double x1 = ((K.tL - T) - K.nuc_mean) / K.nuc_sd / 1.4142135623730951;
  return K.rX * crm_exp(-.5 * (x1 * x1));
}

__device__ __forceinline__ int cafe_hot(const CafeDev &D, const CafeConsts &K, const CafeStepParams &P,
                                        int i, int j, int k) {
  return K.hot_cls[cafe_cls(D, P, i, j, k)];
}

// Moore neighbours in ascending linear-index order (Grid.C:399-414 + sort at
// Grid.C:375); writes cell indices, returns the count.
__device__ __forceinline__ int cafe_moore(const CafeConsts &K, int i, int j, int k, long long *nb) {
  int n = 0;
  for (int dz = -1; dz <= 1; ++dz) {
    int z = k + dz;
    if (z < 0 || z >= K.nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = j + dy;
      if (y < 0 || y >= K.ny) continue;
      for (int dx = -1; dx <= 1; ++dx) {
        int x = i + dx;
        if (x < 0 || x >= K.nx) continue;
        if (dx == 0 && dy == 0 && dz == 0) continue;
        nb[n++] = (long long)K.nxy * z + (long long)K.nx * y + x;
      }
    }
  }
  return n;
}

// ------------------------------------------------------------------ K: melt
// Over the box where T may reach the liquidus: SetLiquid3 and BuildjID.
__device__ __forceinline__ void d_melt(const CafeDev &D, const CafeConsts &K, const CafeStepParams *__restrict__ Pp, const int cafe_bid, const int cafe_nblk) {
  const CafeStepParams P = *Pp;
  int bx = P.hi[0] - P.lo[0], by = P.hi[1] - P.lo[1], bz = P.hi[2] - P.lo[2];
  long long nbox = (long long)bx * by * bz;
  long long iz1 = (long long)P.ilaserLoc * K.nxy;
  int any = 0;
  for (long long t = cafe_bid * (long long)blockDim.x + threadIdx.x; t < nbox;
       t += (long long)cafe_nblk * blockDim.x) {
    int i = P.lo[0] + (int)(t % bx);
    long long r = t / bx;
    int j = P.lo[1] + (int)(r % by);
    int k = P.lo[2] + (int)(r / by);
    int c = cafe_temp_class_exact(K, P, i, j, k);
    D.tcls[t] = (uint8_t)c;
    long long idx = (long long)K.nxy * k + (long long)K.nx * j + i;
    if (K.gt_cls[c]) D.buildj[idx] = 1;
    if (K.hot_cls[c]) {
      any = 1;
      if (idx < K.nxy) {
        D.state[idx] = 2;
      } else if (idx < iz1) {
        D.state[idx] = 1;
        D.gid[idx] = 0;
      }
      D.ext[idx] = 0.0;
    }
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(&D.ctr[CTR_HOT], 1);
}
__global__ void k_melt(CafeDev D, CafeConsts K, const CafeStepParams *__restrict__ Pp) {
  d_melt(D, K, Pp, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ K: solid -> mushy
// ConvertSolid1(1): solid cells with a liquid neighbour become mushy. In place
// is equivalent to the reference's collect-then-apply: the test reads only
// "neighbour == liquid", which this pass never changes. Liquid cells can only
// be (a) cells listed by the previous step's write-back, (b) cells of the
// previous step's pool box, (c) cells of this step's pool box; the box kernel
// covers (b) and (c) dilated by one cell, the list kernel (a).
__global__ void k_solid2mushy_dense(CafeDev D, CafeConsts K) {
  long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * CAFE_CELLS_PER_THREAD;
  for (int c = 0; c < CAFE_CELLS_PER_THREAD; ++c) {
    long long idx = base + c;
    if (idx >= K.N) return;
    if (D.state[idx] != 3) continue;
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    long long nb[26];
    int n = cafe_moore(K, i, j, k, nb);
    bool liq = false;
    for (int a = 0; a < n && !liq; ++a) liq = (D.state[nb[a]] == 1);
    if (liq) D.state[idx] = 2;
  }
}

// ConvertSolid1(1) over this step's pool box (which = 0) or the previous one
// (1), each dilated by one cell, read from the step parameters in device memory.
__device__ __forceinline__ void d_solid2mushy_pbox(const CafeDev &D, const CafeConsts &K, const CafeStepParams *__restrict__ Pp, int which, const int cafe_bid, const int cafe_nblk) {
  const int *lo = which ? Pp->plo : Pp->lo, *hi = which ? Pp->phi : Pp->hi;
  int x0 = lo[0], x1 = hi[0], y0 = lo[1], y1 = hi[1], z0 = lo[2], z1 = hi[2];
  if (which && !(x1 > x0 && y1 > y0 && z1 > z0)) return;  // no previous box
  x0 = max(x0 - 1, 0); y0 = max(y0 - 1, 0); z0 = max(z0 - 1, 0);
  x1 = min(x1 + 1, K.nx); y1 = min(y1 + 1, K.ny); z1 = min(z1 + 1, K.nz);
  if (x1 <= x0 || y1 <= y0 || z1 <= z0) return;
  long long bx = x1 - x0, by = y1 - y0, nbox = bx * by * (z1 - z0);
  for (long long t = cafe_bid * (long long)blockDim.x + threadIdx.x; t < nbox;
       t += (long long)cafe_nblk * blockDim.x) {
    int i = x0 + (int)(t % bx);
    long long r = t / bx;
    int j = y0 + (int)(r % by), k = z0 + (int)(r / by);
    long long idx = (long long)K.nxy * k + (long long)K.nx * j + i;
    if (D.state[idx] != 3) continue;
    long long nb[26];
    int n = cafe_moore(K, i, j, k, nb);
    bool liq = false;
    for (int a = 0; a < n && !liq; ++a) liq = (D.state[nb[a]] == 1);
    if (liq) D.state[idx] = 2;
  }
}
__global__ void k_solid2mushy_pbox(CafeDev D, CafeConsts K, const CafeStepParams *__restrict__ Pp, int which) {
  d_solid2mushy_pbox(D, K, Pp, which, blockIdx.x, gridDim.x);
}

// The step parameters into device memory (kernel arguments are copied at
// launch, so the host copy may change right after).
__global__ void k_put_params(CafeStepParams *Pd, CafeStepParams P) { *Pd = P; }


__device__ __forceinline__ void d_solid2mushy_list(const CafeDev &D, const CafeConsts &K, const int cafe_bid, const int cafe_nblk) {
  int n = D.ctr[CTR_NLIQ];
  for (int t = cafe_bid * blockDim.x + threadIdx.x; t < n; t += cafe_nblk * blockDim.x) {
    long long idx = D.liq[t];
    if (D.state[idx] != 1) continue;
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    long long nb[26];
    int m = cafe_moore(K, i, j, k, nb);
    for (int a = 0; a < m; ++a)
      if (D.state[nb[a]] == 3) D.state[nb[a]] = 2;
  }
}
__global__ void k_solid2mushy_list(CafeDev D, CafeConsts K) {
  d_solid2mushy_list(D, K, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ active set
__device__ __forceinline__ bool cafe_is_active(const CafeDev &D, const CafeConsts &K,
                                               const CafeStepParams &P, long long idx) {
  uint8_t s = D.state[idx];
  if (s == 2) return true;
  int i, j, k;
  cafe_cell_xyz(K, idx, i, j, k);
  int hot = cafe_hot(D, K, P, i, j, k);
  if (!hot) return s == 1;  // undercooled liquid; a cell below the liquidus is active only as such
  // a cell at/above the liquidus is active when a neighbour is mushy or undercooled liquid
  for (int dz = -1; dz <= 1; ++dz) {
    int z = k + dz;
    if (z < 0 || z >= K.nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = j + dy;
      if (y < 0 || y >= K.ny) continue;
      for (int dx = -1; dx <= 1; ++dx) {
        int x = i + dx;
        if (x < 0 || x >= K.nx || (dx == 0 && dy == 0 && dz == 0)) continue;
        uint8_t t = D.state[(long long)K.nxy * z + (long long)K.nx * y + x];
        if (t == 2) return true;
        if (t == 1 && !cafe_hot(D, K, P, x, y, z)) return true;
      }
    }
  }
  return false;
}

// Cell-index range that can hold active cells this step: the z planes of the
// mushy and liquid cells left by the previous step (k_writeback) and of this
// and the previous pool box, widened by one plane. Every active cell is mushy,
// liquid, or at/above the liquidus (inside the pool box); a cell turns mushy
// this step only next to a liquid cell (ConvertSolid1(1)), and liquid cells
// are those left by the previous step or melted in the pool box; new layers
// bring solid and powder cells only.
__device__ __forceinline__ void cafe_active_range(const CafeDev &D, const CafeConsts &K, const CafeStepParams &P,
                                                  long long &r0, long long &r1) {
  int zlo = D.ctr[CTR_ZLO], zhi = D.ctr[CTR_ZHI];
  if (P.hi[0] > P.lo[0] && P.hi[1] > P.lo[1] && P.hi[2] > P.lo[2]) {
    zlo = min(zlo, P.lo[2]);
    zhi = max(zhi, P.hi[2] - 1);
  }
  if (P.phi[0] > P.plo[0] && P.phi[1] > P.plo[1] && P.phi[2] > P.plo[2]) {
    zlo = min(zlo, P.plo[2]);
    zhi = max(zhi, P.phi[2] - 1);
  }
  zlo = max(zlo - 1, 0);
  zhi = min(zhi + 1, K.nz - 1);
  if (zhi < zlo) {
    r0 = r1 = 0;
    return;
  }
  r0 = (long long)zlo * K.nxy;
  r1 = (long long)(zhi + 1) * K.nxy;
}

// Flags of the eight state bytes of w (bit c for byte c): the byte is 1
// (liquid) or 2 (mushy). Bit arithmetic on the word: a byte is 1 or 2 when
// it is below 4 and its two low bits differ; the eight results, one per
// byte's lowest bit, are gathered into the top byte by one multiplication.
__device__ __forceinline__ uint32_t cafe_liq_or_mushy8(unsigned long long w) {
  const unsigned long long t = w & 0xFCFCFCFCFCFCFCFCULL;
  const unsigned long long u = (t | (t >> 2) | (t >> 4)) & 0x0C0C0C0C0C0C0C0CULL;
  const unsigned long long ge4 = (u | (u >> 1)) & 0x0404040404040404ULL;  // bit 2: the byte is >= 4
  const unsigned long long a = (w ^ (w >> 1)) & ~(ge4 >> 2) & 0x0101010101010101ULL;
  return (uint32_t)((a * 0x0102040810204080ULL) >> 56);
}

// Activity flags of the eight cells i0..i0+7 of row (j, k), i0 and nx multiples
// of 8: cafe_is_active for each. The chunk's own classes come first: when no
// cell of the chunk is at or above the liquidus, each is active exactly when
// liquid or mushy. Otherwise the states of the 3 x 3 rows around the chunk over
// i0-1..i0+8 (an aligned 64-bit word and two bytes per row) and the classes of
// their liquid cells are loaded, all before any test, so that no load waits on
// another's outcome. A neighbour "emits" when it is mushy or liquid below the
// liquidus; a cell at or above the liquidus is active when mushy or when an
// emitter lies among its 26 neighbours, i.e. in the three-wide window of the
// nine rows' emitter masks (the cell itself, at or above the liquidus, emits
// only if mushy, and then it is active anyway).
__device__ __forceinline__ uint32_t cafe_chunk_active_rows(const CafeDev &D, const CafeConsts &K,
                                                           const CafeStepParams &P, int i0, int j, int k) {
  const uint32_t hotmask = (K.hot_cls[0] ? 1u : 0u) | (K.hot_cls[1] ? 2u : 0u) | (K.hot_cls[2] ? 4u : 0u);
  const unsigned long long wown = *(const unsigned long long *)(D.state + (long long)K.nxy * k + (long long)K.nx * j + i0);
  uint32_t own_hot = 0;  // bit c: cell i0 + c at or above the liquidus
#pragma unroll
  for (int c = 0; c < 8; ++c) own_hot |= ((hotmask >> cafe_cls(D, P, i0 + c, j, k)) & 1u) << c;
  const uint32_t own_lm = cafe_liq_or_mushy8(wown);
  if (own_hot == 0) return own_lm;
  uint32_t own_mushy = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) own_mushy |= (((wown >> (8 * c)) & 0xffu) == 2u ? 1u : 0u) << c;
  uint32_t win = 0;  // bit x: an emitter at x - 1..x + 1 (x = 0..9 for i0 - 1 + x) in some row
#pragma unroll
  for (int r = 0; r < 9; ++r) {
    const int y = j + r % 3 - 1, z = k + r / 3 - 1;
    const bool rowin = y >= 0 && y < K.ny && z >= 0 && z < K.nz;
    const long long rb = (long long)K.nxy * (rowin ? z : 0) + (long long)K.nx * (rowin ? y : 0);
    const unsigned long long w = rowin ? *(const unsigned long long *)(D.state + rb + i0) : 0ULL;
    const unsigned int sl = (rowin && i0 > 0) ? D.state[rb + i0 - 1] : 0u;
    const unsigned int sr = (rowin && i0 + 8 < K.nx) ? D.state[rb + i0 + 8] : 0u;
    uint32_t e = 0;
#pragma unroll
    for (int x = 0; x < 10; ++x) {
      const unsigned int s = x == 0 ? sl : (x == 9 ? sr : (unsigned int)(w >> (8 * (x - 1))) & 0xffu);
      // the class of a liquid neighbour
      const int c = s == 1u ? cafe_cls(D, P, i0 - 1 + x, y, z) : 1;
      const bool hot = (hotmask >> c) & 1u;
      e |= (s == 2u || (s == 1u && !hot)) ? 1u << x : 0u;
    }
    win |= e | (e << 1) | (e >> 1);
  }
  // cell i0 + c is bit c + 1 of the window
  const uint32_t nb = (win >> 1) & 0xffu;
  return ((~own_hot & own_lm) | (own_hot & (own_mushy | nb))) & 0xffu;
}

// Activity flags of the 8-cell chunk i0..i0+7 of row (j0, k0) (bit c for
// cell i0 + c). A cell that cannot be at or above the liquidus (outside the
// pool box, or not below the laser plane) is active exactly when it is liquid
// or mushy, so a chunk outside the hot region is decided from its state bytes,
// loaded as one 64-bit word; other chunks take the 3 x 3-row test.
__device__ __forceinline__ uint32_t cafe_chunk_active_row(const CafeDev &D, const CafeConsts &K,
                                                          const CafeStepParams &P, long long base, int i0,
                                                          int j0, int k0) {
  // (with any_hot_full, T0 or tS reaches the liquidus and no class is cold)
  const bool cold = !P.any_hot_full && (k0 >= P.kabove || k0 < P.lo[2] || k0 >= P.hi[2] || j0 < P.lo[1] ||
                                        j0 >= P.hi[1] || i0 + 7 < P.lo[0] || i0 >= P.hi[0]);
  if (cold) return cafe_liq_or_mushy8(*(const unsigned long long *)(D.state + base));
  return cafe_chunk_active_rows(D, K, P, i0, j0, k0);
}

// Activity flags of the CAFE_CELLS_PER_THREAD (8) cells from `base` (bit c
// for cell base + c) for any grid: a chunk lying in one row is decided as in
// cafe_chunk_active_row, others cell by cell.
__device__ __forceinline__ uint32_t cafe_chunk_active(const CafeDev &D, const CafeConsts &K,
                                                      const CafeStepParams &P, long long base) {
  static_assert(CAFE_CELLS_PER_THREAD == 8, "one 64-bit word of states per thread");
  uint32_t flags = 0;
  if (base + 8 <= K.N) {
    int i0, j0, k0, i1, j1, k1;
    cafe_cell_xyz(K, base, i0, j0, k0);
    cafe_cell_xyz(K, base + 7, i1, j1, k1);
    if (j0 == j1 && k0 == k1 && (K.nx & 7) == 0) return cafe_chunk_active_row(D, K, P, base, i0, j0, k0);
    bool cold = false;
    if (!P.any_hot_full && j0 == j1 && k0 == k1)
      cold = k0 >= P.kabove || k0 < P.lo[2] || k0 >= P.hi[2] || j0 < P.lo[1] || j0 >= P.hi[1] || i1 < P.lo[0] ||
             i0 >= P.hi[0];
    if (cold && (base & 7) == 0) return cafe_liq_or_mushy8(*(const unsigned long long *)(D.state + base));
  }
  for (int c = 0; c < CAFE_CELLS_PER_THREAD; ++c) {
    long long idx = base + c;
    if (idx < K.N && cafe_is_active(D, K, P, idx)) flags |= 1u << c;
  }
  return flags;
}

// Activity flags of this thread's `chunks` chunks (bit 8 c + j for cell
// base + 8 c + j), base a multiple of 8. With nx a multiple of 8 every chunk
// lies in one row: the cell coordinates are formed once and stepped from
// chunk to chunk.
__device__ __forceinline__ uint32_t cafe_thread_active(const CafeDev &D, const CafeConsts &K,
                                                       const CafeStepParams &P, long long base, int chunks,
                                                       long long r0, long long r1) {
  uint32_t f = 0;
  if (base >= r1 || base + 8LL * chunks <= r0) return 0;  // no plane that can hold active cells
  if ((K.nx & 7) == 0 && base + 8LL * chunks <= K.N) {
    int i, j, k;
    cafe_cell_xyz(K, base, i, j, k);
#pragma unroll
    for (int c = 0; c < CAFE_ACT_MAX_CHUNKS; ++c)
      if (c < chunks) {
        f |= cafe_chunk_active_row(D, K, P, base + 8 * c, i, j, k) << (8 * c);
        i += 8;
        if (i == K.nx) {
          i = 0;
          if (++j == K.ny) {
            j = 0;
            ++k;
          }
        }
      }
  } else {
#pragma unroll
    for (int c = 0; c < CAFE_ACT_MAX_CHUNKS; ++c)
      if (c < chunks) f |= cafe_chunk_active(D, K, P, base + 8 * c) << (8 * c);
  }
  // cells of the range's edge chunks that lie outside it: keep [r0 - base, r1 - base)
  const long long lo = r0 - base, hi = r1 - base;
  if (lo > 0) f &= lo >= 32 ? 0u : ~((1u << lo) - 1u);
  if (hi < 32) f &= hi <= 0 ? 0u : (1u << hi) - 1u;
  return f;
}

// The compaction runs over "virtual blocks" of CAFE_DENSE_THREADS threads x
// `chunks` 8-cell chunks (nvb of them cover the grid); a persistent grid
// strides over them, writes a zero count for those outside the active range
// (cafe_active_range) without touching their cells, and counts the rest.
__device__ __forceinline__ void d_active_count(const CafeDev &D, const CafeConsts &K, const CafeStepParams *__restrict__ Pp, int chunks, long long nvb, const int cafe_bid, const int cafe_nblk) {
  const CafeStepParams P = *Pp;
  __shared__ int wsum[CAFE_DENSE_THREADS / 32];
  long long r0, r1;
  cafe_active_range(D, K, P, r0, r1);
  const long long per_vb = (long long)CAFE_DENSE_THREADS * CAFE_CELLS_PER_THREAD * chunks;
  for (long long vb = cafe_bid; vb < nvb; vb += cafe_nblk) {
    long long b0 = vb * per_vb;
    if (b0 >= r1 || b0 + per_vb <= r0) {
      if (threadIdx.x == 0) D.blk[vb] = 0;
      continue;
    }
    long long base = b0 + (long long)threadIdx.x * (CAFE_CELLS_PER_THREAD * chunks);
    const uint32_t f = cafe_thread_active(D, K, P, base, chunks, r0, r1);
    D.act_flags[vb * CAFE_DENSE_THREADS + threadIdx.x] = f;
    int cnt = __popc(f);
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      int sum = 0;
      for (int w = 0; w < CAFE_DENSE_THREADS / 32; ++w) sum += wsum[w];
      D.blk[vb] = sum;
    }
    __syncthreads();
  }
}
__global__ void k_active_count(CafeDev D, CafeConsts K, const CafeStepParams *__restrict__ Pp, int chunks, long long nvb) {
  d_active_count(D, K, Pp, chunks, nvb, blockIdx.x, gridDim.x);
}

// Exclusive scan over the block of one value per thread (blockDim.x a multiple
// of 32, at most 1024; every thread must call it): returns this thread's
// prefix and leaves the block total in tot. ws: 33 shared words.
__device__ __forceinline__ long long cafe_block_excl_scan(long long v, long long *ws, long long &tot) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const long long t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[w] = incl;
  __syncthreads();
  if (w == 0) {
    const long long x = lane < nw ? ws[lane] : 0;
    long long xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(FULL, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < nw) ws[lane] = xi - x;
    if (lane == 31) ws[32] = xi;
  }
  __syncthreads();
  tot = ws[32];
  return ws[w] + incl - v;
}

// Exclusive scan of n block counts in place; writes the total to *total.
__device__ __forceinline__ void d_scan_blocks(int32_t *blk, long long n, int *total, const int cafe_bid, const int cafe_nblk) {
  __shared__ long long ws[33];
  // each thread's segment is a multiple of four counts, so that its groups of
  // four are aligned 16-byte loads and stores (a warp's lanes read segments
  // apart, and one vector access serves four counts)
  const long long per = ((n + blockDim.x - 1) / blockDim.x + 3) & ~3LL;
  long long b0 = threadIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
  if (b0 > n) b0 = n;
  long long s = 0;
  for (long long b = b0; b < b1; b += 16) {
    int4 v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long g = b + 4 * i;
      if (g + 4 <= b1)
        v[i] = *(const int4 *)(blk + g);
      else
        v[i] = make_int4(g < b1 ? blk[g] : 0, g + 1 < b1 ? blk[g + 1] : 0, g + 2 < b1 ? blk[g + 2] : 0, 0);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) s += (long long)v[i].x + v[i].y + v[i].z + v[i].w;
  }
  long long tot;
  long long acc = cafe_block_excl_scan(s, ws, tot);
  if (threadIdx.x == 0) *total = (int)tot;
  for (long long b = b0; b < b1; b += 16) {
    int4 v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long g = b + 4 * i;
      if (g + 4 <= b1)
        v[i] = *(const int4 *)(blk + g);
      else
        v[i] = make_int4(g < b1 ? blk[g] : 0, g + 1 < b1 ? blk[g + 1] : 0, g + 2 < b1 ? blk[g + 2] : 0, 0);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long g = b + 4 * i;
      int4 o;
      o.x = (int32_t)acc;
      acc += v[i].x;
      o.y = (int32_t)acc;
      acc += v[i].y;
      o.z = (int32_t)acc;
      acc += v[i].z;
      o.w = (int32_t)acc;
      acc += v[i].w;
      if (g + 4 <= b1) {
        *(int4 *)(blk + g) = o;
      } else {
        if (g < b1) blk[g] = o.x;
        if (g + 1 < b1) blk[g + 1] = o.y;
        if (g + 2 < b1) blk[g + 2] = o.z;
      }
    }
  }
}
__global__ void __launch_bounds__(1024) k_scan_blocks(int32_t *blk, long long n, int *total) {
  d_scan_blocks(blk, n, total, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void d_active_scatter(const CafeDev &D, const CafeConsts &K, const CafeStepParams *__restrict__ Pp, int chunks, long long nvb, const int cafe_bid, const int cafe_nblk) {
  const CafeStepParams P = *Pp;
  __shared__ int wsum[CAFE_DENSE_THREADS / 32];
  long long r0, r1;
  cafe_active_range(D, K, P, r0, r1);
  const long long per_vb = (long long)CAFE_DENSE_THREADS * CAFE_CELLS_PER_THREAD * chunks;
  long long vb_lo = r0 / per_vb, vb_hi = r1 > 0 ? (r1 - 1) / per_vb : -1;
  if (vb_hi >= nvb) vb_hi = nvb - 1;
  for (long long vb = vb_lo + cafe_bid; vb <= vb_hi; vb += cafe_nblk) {
  long long base = vb * per_vb + (long long)threadIdx.x * (CAFE_CELLS_PER_THREAD * chunks);
  const uint32_t flags = D.act_flags[vb * CAFE_DENSE_THREADS + threadIdx.x];  // from k_active_count
  const int cnt = __popc(flags);
  // block-exclusive scan of per-thread counts
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = threadIdx.x < CAFE_DENSE_THREADS / 32 ? wsum[threadIdx.x] : 0;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, inc, o);
      if (threadIdx.x >= o) inc += u;
    }
    if (threadIdx.x < CAFE_DENSE_THREADS / 32) wsum[threadIdx.x] = inc - v;
  }
  __syncthreads();
  long long pos = (long long)D.blk[vb] + wsum[w] + (incl - cnt);
  for (int c = 0; c < CAFE_CELLS_PER_THREAD * chunks; ++c) {
    if (!(flags >> c & 1u)) continue;
    long long idx = base + c;
    if (pos < D.act_cap) {
      D.act[pos] = (int32_t)idx;
      D.pos_of[idx] = (int32_t)pos;
    } else {
      atomicOr(D.err, CAFE_ERR_ACTIVE_CAP);
    }
    ++pos;
  }
  __syncthreads();  // wsum is reused by the next virtual block
  }
}
__global__ void k_active_scatter(CafeDev D, CafeConsts K, const CafeStepParams *__restrict__ Pp, int chunks, long long nvb) {
  d_active_scatter(D, K, Pp, chunks, nvb, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ gather
// Per active position: copies of the cell data, temperature class, neighbour
// positions in ascending index order (-1 = not active), liquid-neighbour count,
// all-neighbours-below-liquidus flag and the ruq offset (VoxelsCA.C:380:
// ruq[p] = (U_p - .5) dX / 100, U_p the p-th uniform of minstd(30 tInd + seed1)).
__device__ __forceinline__ void d_gather(const CafeDev &D, const CafeConsts &K, const CafeStepParams *__restrict__ Pp, const int cafe_bid, const int cafe_nblk) {
  const CafeStepParams P = *Pp;
  int na = D.ctr[CTR_NA];
  if (na > D.act_cap) na = (int)D.act_cap;
  uint32_t seed = cafe_minstd_seed((uint64_t)(uint32_t)(30 * P.tInd + (int)K.seed1));
  if (cafe_bid == 0 && threadIdx.x == 0) {  // rebuilt by k_writeback for the next step
    D.ctr[CTR_ZLO] = 0x7fffffff;
    D.ctr[CTR_ZHI] = -1;
  }
  for (int p = cafe_bid * blockDim.x + threadIdx.x; p < na; p += cafe_nblk * blockDim.x) {
    long long idx = D.act[p];
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    D.a_state[p] = D.state[idx];
    D.a_gid[p] = D.gid[idx];
    D.a_ext[p] = D.ext[idx];
    D.a_cx[p] = D.cx[idx];
    D.a_cy[p] = D.cy[idx];
    D.a_cz[p] = D.cz[idx];
    D.a_cls[p] = (uint8_t)cafe_cls(D, P, i, j, k);
    if (K.easm) {
      // VoxelsCA.C:405: T >= tL ? 0 : Avel pow(tL - T, nvel)
      double T = D.temp[idx];
      D.a_vh[p] = T >= K.tL ? 0.0 : K.Avel * crm_pow_int(K.tL - T, K.nvel_i);
    }
    long long nb[26];
    int n = cafe_moore(K, i, j, k, nb);
    int m = 0, liq = 0, cold = 1;
    for (int a = 0; a < n; ++a) {
      int q = D.pos_of[nb[a]];
      if (q < 0) continue;
      D.a_nbr[(long long)p * CAFE_NSLOT + m] = q;
      ++m;
      if (D.state[nb[a]] == 1) ++liq;
      int ni, nj, nk;
      cafe_cell_xyz(K, nb[a], ni, nj, nk);
      if (cafe_hot(D, K, P, ni, nj, nk)) cold = 0;
    }
    D.a_nn[p] = (uint8_t)m;
    D.a_liq[p] = liq;
    D.a_cold[p] = (uint8_t)cold;
    D.a_frow[p] = -1;
    double U = cafe_uniform_at(seed, (uint64_t)p);
    D.a_ruq[p] = (U - .5) * K.ruq_dx / 100.;
  }
}
__global__ void k_gather(CafeDev D, CafeConsts K, const CafeStepParams *__restrict__ Pp) {
  d_gather(D, K, Pp, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ vs2ind + frontier rows
// Two order-preserving compactions over positions: mushy positions (vs2ind,
// VoxelsCA.C:346-353) and, among them, those with a liquid neighbour and no
// neighbour at the liquidus (the cells that can capture, VoxelsCA.C:396-397).
__device__ __forceinline__ void d_lists_count(const CafeDev &D, const int cafe_bid, const int cafe_nblk) {
  __shared__ int ws[2][CAFE_DENSE_THREADS / 32];
  int na = D.ctr[CTR_NA];
  if (na > D.act_cap) na = (int)D.act_cap;
  long long base = ((long long)cafe_bid * blockDim.x + threadIdx.x) * CAFE_CELLS_PER_THREAD;
  int c2 = 0, cf = 0;
  for (int c = 0; c < CAFE_CELLS_PER_THREAD; ++c) {
    long long p = base + c;
    if (p >= na) break;
    if (D.a_state[p] == 2) {
      ++c2;
      if (D.a_liq[p] > 0 && D.a_cold[p]) ++cf;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    c2 += __shfl_down_sync(0xffffffffu, c2, o);
    cf += __shfl_down_sync(0xffffffffu, cf, o);
  }
  if ((threadIdx.x & 31) == 0) {
    ws[0][threadIdx.x >> 5] = c2;
    ws[1][threadIdx.x >> 5] = cf;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int s2 = 0, sf = 0;
    for (int w = 0; w < CAFE_DENSE_THREADS / 32; ++w) {
      s2 += ws[0][w];
      sf += ws[1][w];
    }
    D.blk[2 * cafe_bid] = s2;
    D.blk[2 * cafe_bid + 1] = sf;
  }
}
__global__ void k_lists_count(CafeDev D) {
  d_lists_count(D, blockIdx.x, gridDim.x);
}

// Exclusive scan of interleaved pairs (blk[2b], blk[2b+1]), b < n, one block.
// Exclusive scan of the (mushy, frontier) count pairs of the position blocks
// that hold active positions (na from *na_ptr); totals to *tot0, *tot1.
__device__ __forceinline__ void d_scan_pairs(int32_t *blk, long long n, const int *na_ptr, int *tot0, int *tot1, const int cafe_bid, const int cafe_nblk) {
  __shared__ long long ws[2][33];
  {
    long long used = ((long long)*na_ptr + CAFE_CELLS_PER_BLOCK - 1) / CAFE_CELLS_PER_BLOCK;
    if (used < n) n = used;
  }
  long long per = (n + blockDim.x - 1) / blockDim.x;
  long long b0 = threadIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
  const int2 *p2 = (const int2 *)blk;  // (count 0, count 1) of block b
  long long s0 = 0, s1 = 0;
  for (long long b = b0; b < b1; b += 8) {
    int2 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = b + i < b1 ? p2[b + i] : make_int2(0, 0);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      s0 += v[i].x;
      s1 += v[i].y;
    }
  }
  long long t0, t1;
  long long a0 = cafe_block_excl_scan(s0, ws[0], t0);
  long long a1 = cafe_block_excl_scan(s1, ws[1], t1);
  if (threadIdx.x == 0) {
    *tot0 = (int)t0;
    *tot1 = (int)t1;
  }
  int2 *q2 = (int2 *)blk;
  for (long long b = b0; b < b1; b += 8) {
    int2 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = b + i < b1 ? q2[b + i] : make_int2(0, 0);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (b + i < b1) {
        q2[b + i] = make_int2((int32_t)a0, (int32_t)a1);
        a0 += v[i].x;
        a1 += v[i].y;
      }
  }
}
__global__ void __launch_bounds__(1024) k_scan_pairs(int32_t *blk, long long n, const int *na_ptr, int *tot0, int *tot1) {
  d_scan_pairs(blk, n, na_ptr, tot0, tot1, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void d_lists_scatter(const CafeDev &D, const int cafe_bid, const int cafe_nblk) {
  __shared__ int ws[2][CAFE_DENSE_THREADS / 32];
  int na = D.ctr[CTR_NA];
  if (na > D.act_cap) na = (int)D.act_cap;
  long long base = ((long long)cafe_bid * blockDim.x + threadIdx.x) * CAFE_CELLS_PER_THREAD;
  int c2 = 0, cf = 0;
  for (int c = 0; c < CAFE_CELLS_PER_THREAD; ++c) {
    long long p = base + c;
    if (p >= na) break;
    if (D.a_state[p] == 2) {
      ++c2;
      if (D.a_liq[p] > 0 && D.a_cold[p]) ++cf;
    }
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int i2 = c2, i_f = cf;
  for (int o = 1; o < 32; o <<= 1) {
    int v2 = __shfl_up_sync(0xffffffffu, i2, o), vf = __shfl_up_sync(0xffffffffu, i_f, o);
    if (lane >= o) {
      i2 += v2;
      i_f += vf;
    }
  }
  if (lane == 31) {
    ws[0][w] = i2;
    ws[1][w] = i_f;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a2 = 0, af = 0;
    for (int q = 0; q < CAFE_DENSE_THREADS / 32; ++q) {
      int v2 = ws[0][q], vf = ws[1][q];
      ws[0][q] = a2;
      ws[1][q] = af;
      a2 += v2;
      af += vf;
    }
  }
  __syncthreads();
  long long j2 = (long long)D.blk[2 * cafe_bid] + ws[0][w] + (i2 - c2);
  long long jf = (long long)D.blk[2 * cafe_bid + 1] + ws[1][w] + (i_f - cf);
  for (int c = 0; c < CAFE_CELLS_PER_THREAD; ++c) {
    long long p = base + c;
    if (p >= na) break;
    if (D.a_state[p] != 2) continue;
    if (j2 < D.vs2_cap)
      D.vs2[j2] = (int32_t)p;
    else
      atomicOr(D.err, CAFE_ERR_MUSHY_CAP);
    if (D.a_liq[p] > 0 && D.a_cold[p]) {
      if (jf < D.row_cap) {
        D.row_pos[jf] = (int32_t)p;
        D.row_j[jf] = (int32_t)j2;
        D.row_alive[jf] = 1;
        D.a_frow[p] = (int32_t)jf;
      } else {
        atomicOr(D.err, CAFE_ERR_ROW_CAP);
      }
      ++jf;
    }
    ++j2;
  }
}
__global__ void k_lists_scatter(CafeDev D) {
  d_lists_scatter(D, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ frontier rows
// Order keys: an unsigned integer order equal to the numeric order of the
// doubles (negative values included); cafe_key_canon maps -0 to +0 first so
// that equal values get equal keys.
#define CAFE_KEY_NONE 0xffffffffffffffffULL
__device__ __forceinline__ unsigned long long cafe_key(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double cafe_unkey(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long cafe_key_canon(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if (b == 0x8000000000000000ULL) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ unsigned long long cafe_shfl_u64(unsigned long long v, int src) {
  return (unsigned long long)__shfl_sync(0xffffffffu, (long long)v, src);
}
__device__ __forceinline__ unsigned long long cafe_shfl_u64_xor(unsigned long long v, int o) {
  return (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)v, o);
}
__device__ __forceinline__ bool cafe_is_nan(double x) { return (crm_bits(x) & CRM_ABS_MASK) > CRM_BITS_INF; }
// x < 0.0 (negative, nonzero, not NaN)
__device__ __forceinline__ bool cafe_is_neg(double x) {
  long long b = crm_bits(x);
  return b < 0 && (b & CRM_ABS_MASK) != 0 && (b & CRM_ABS_MASK) <= CRM_BITS_INF;
}
// e with |x| < 2^e (a large value for inf and NaN)
__device__ __forceinline__ int cafe_exp_ub(double x) {
  int f = (int)((crm_bits(x) >> 52) & 0x7ff);
  return f == 0x7ff ? 4096 : (f == 0 ? -1022 : f - 1022);
}
// e with |x| >= 2^e for a normal x (a small value for zero and subnormals)
__device__ __forceinline__ int cafe_exp_lb(double x) {
  int f = (int)((crm_bits(x) >> 52) & 0x7ff);
  return f == 0 ? -4096 : f - 1023;
}

// Row order, exact best candidate and largest |g| of row r (position p) once
// every lane of the calling warp holds its slot: liv (the neighbour is liquid),
// gv (its numerator g) and q (its position). The live slots are ordered by g
// (NaN last, ties by slot) into row_ord, followed by the other slots. With
// `eval`, the row's exact best candidate at iteration `ev` and time T is stored
// (what cafe_row_best computes, one slot per lane). Returns, in every lane, the
// order key of the largest finite |g| of the live slots, or 0 when none.
// `parts` selects the row order (CAFE_FIN_ORDER) and the rest (CAFE_FIN_BEST:
// row_live, the best candidate, the largest |g|), so that two warps holding
// the same slots can share the work.
#define CAFE_FIN_ORDER 1
#define CAFE_FIN_BEST 2
__device__ unsigned long long cafe_row_finish_warp(const CafeDev &D, const CafeConsts &K, long long r, int p,
                                                   int nn, bool liv, double gv, int q, bool eval, int ev,
                                                   double T, bool have_t = false, double t_pre = 0.0,
                                                   double ruqs_pre = 0.0,
                                                   int parts = CAFE_FIN_ORDER | CAFE_FIN_BEST) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31;
  uint32_t live = __ballot_sync(FULL, liv);
  // rank of this slot in the row order
#ifdef CAFE_DETAIL_CYCLES
  long long fz0 = clock64();
#endif
  const bool gfin = !cafe_is_nan(gv);
  if (parts & CAFE_FIN_ORDER) {
    unsigned long long key = (liv && gfin) ? cafe_key_canon(gv) : CAFE_KEY_NONE;
    int rank = liv ? 0 : __popc(live);
    // (every slot position, so that the shuffles are independent; the bits of
    // live above nn are clear)
#pragma unroll
    for (int t = 0; t < CAFE_NSLOT; ++t) {
      unsigned long long kt = cafe_shfl_u64(key, t);
      bool lt = (live >> t) & 1u;
      if (liv)
        rank += lt && (kt < key || (kt == key && t < lane));
      else
        rank += !lt && t < nn && t < lane;
    }
    if (lane < nn) D.row_ord[r * CAFE_NSLOT + rank] = (uint8_t)lane;
  }
  if (!(parts & CAFE_FIN_BEST)) return 0ULL;
  if (lane == 0) D.row_live[r] = live;
#ifdef CAFE_DETAIL_CYCLES
  long long fz1 = clock64();
#endif
  if (eval) {
    // t and ruqs of each live slot (given by the caller when have_t)
    double t = 0.0, ruqs = 0.0;
    bool cand = false;
    if (liv) {
      if (have_t) {
        t = t_pre;
        ruqs = ruqs_pre;
      } else {
        double E = D.a_ext[p];
        double v = cafe_vh(D, K, p);
        double dr = gv - E;
        t = dr / v;
        ruqs = .5 * (D.a_ruq[p] + D.a_ruq[q]);
      }
      cand = !cafe_is_nan(t);
    }
    // lexicographic (t, ruqs, slot) minimum over the warp (VoxelsCA.C:427-440)
    const unsigned long long tk0 = cand ? cafe_key_canon(t) : CAFE_KEY_NONE;
    unsigned long long tk = tk0;
    unsigned long long rk = cand ? cafe_key_canon(ruqs) : CAFE_KEY_NONE;
    int sl = cand ? lane : 255;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long tk2 = (unsigned long long)__shfl_xor_sync(FULL, (long long)tk, o);
      unsigned long long rk2 = (unsigned long long)__shfl_xor_sync(FULL, (long long)rk, o);
      int sl2 = __shfl_xor_sync(FULL, sl, o);
      if (tk2 < tk || (tk2 == tk && (rk2 < rk || (rk2 == rk && sl2 < sl)))) {
        tk = tk2;
        rk = rk2;
        sl = sl2;
      }
    }
    // the smallest time of the other candidates (the row's time once slot sl
    // is captured by another row)
    unsigned long long k2 = lane == sl ? CAFE_KEY_NONE : tk0;
    for (int o = 16; o > 0; o >>= 1) k2 = min(k2, cafe_shfl_u64_xor(k2, o));
    double bt = __shfl_sync(FULL, t, sl & 31);
    double bruq = __shfl_sync(FULL, ruqs, sl & 31);
    int bq = __shfl_sync(FULL, q, sl & 31);
    if (lane == 0) {
      D.row_stamp[r] = ev + 1;
      if (sl == 255) {
        D.row_key[r] = CAFE_KEY_NONE;
      } else {
        D.row_bt[r] = bt;
        D.row_bruq[r] = bruq;
        D.row_bslot[r] = sl;
        D.row_bq[r] = bq;
        const unsigned long long key = cafe_key(T + bt);
        D.row_key[r] = key;
        D.row_key2[r] = k2 == CAFE_KEY_NONE ? key : cafe_key(T + cafe_unkey(k2));
      }
    }
  }
#ifdef CAFE_DETAIL_CYCLES
  long long fz2 = clock64();
#endif
  unsigned long long ak = (liv && gfin) ? cafe_key(fabs(gv)) : 0ULL;
  for (int o = 16; o > 0; o >>= 1) ak = max(ak, (unsigned long long)__shfl_xor_sync(FULL, (long long)ak, o));
  __syncwarp();
#ifdef CAFE_DETAIL_CYCLES
  if (gridDim.x == 1 && lane == 0) {
    long long fz3 = clock64();
    atomicAdd(&D.stat[STAT_DETAIL + 24], (unsigned long long)(fz1 - fz0));
    atomicAdd(&D.stat[STAT_DETAIL + 25], (unsigned long long)(fz2 - fz1));
    atomicAdd(&D.stat[STAT_DETAIL + 26], (unsigned long long)(fz3 - fz2));
  }
#endif
  return ak;
}

// The captured cell's grain, centre and extent as the capture section just
// stored them, handed to the fill through shared memory.
struct CafeNewCell {
  double c[3], ext;
  int gid;
};
// Per-slot partial results passed between the four warps of cafe_row_fill_quad.
struct CafeQuadScratch {
  double cth[32], sph[32], l[32], d1I[32], dI2[32], d1J[32], dJ3[32], dr[32], ruqs[32];
};
#define CAFE_QUAD_THREADS 128
__device__ __forceinline__ void cafe_bar_quad() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// Fills row r for position p, the cell just captured, with warps 0-3 of the
// block together (all 128 threads must call it): every liquid neighbour slot
// gets its numerator g and capture result (extent, centre), the slots are
// ordered and, with `eval`, the row's exact best candidate at iteration `ev`
// and time T is stored. A warp issues one FP64 instruction at a time whatever its
// active lanes, so the independent chains of each slot's geometry run in
// different warps, lane s of each warp on slot s. First stage:
//   warp 0: cos th and the cell distance l; warp 1: sin ph;
//   warp 2: |R^T dn|_1 and the projection on edge p0-p1;
//   warp 3: the projection on edge p0-p2 and the tie-break ruqs.
// Second stage, after one barrier: warps 0 and 1 form g; warp 0 the capture
// time t = (g - ExtA)/v (with eval) and the row's best candidate, warp 1 the
// slot order; warp 2 the extent and warp 3 the centre a capture from this row
// gives. The return value is valid in warp 0.
__device__ unsigned long long cafe_row_fill_quad(const CafeDev &D, const CafeConsts &K, long long r, int p,
                                                 bool eval, int ev, double T, CafeQuadScratch &S,
                                                 const CafeNewCell *nc = nullptr) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#ifdef CAFE_DETAIL_CYCLES
  long long fq0 = clock64();
#endif
  int nn = D.a_nn[p];
  int gp = nc ? nc->gid : D.a_gid[p];
  bool grain_ok = gp >= 1 && gp <= D.grain_cap;
  bool liv = false;
  int q = 0;
  double dn[3] = {0.0, 0.0, 0.0}, cs[3] = {0.0, 0.0, 0.0};
  int ci = 0, cj = 0, ck = 0, si = 0, sj = 0, sk = 0;
  if (lane < nn) {
    q = D.a_nbr[(long long)p * CAFE_NSLOT + lane];
    liv = D.a_state[q] == 1;
  }
  const bool work = liv && grain_ok;
  double R[9], loc[3], dr = 0.0, pk[3][3];
  double E0 = 0.0, v0 = 1.0;  // warp 0: the row's extent and velocity for t
  int s0i = 0;
  if (work) {
    cafe_cell_xyz(K, D.act[q], ci, cj, ck);
    cafe_cell_xyz(K, D.act[p], si, sj, sk);
    cs[0] = nc ? nc->c[0] : D.a_cx[p];
    cs[1] = nc ? nc->c[1] : D.a_cy[p];
    cs[2] = nc ? nc->c[2] : D.a_cz[p];
    cafe_geo_dn(K, ci, cj, ck, cs, dn);
    if (w == 0) {
      if (eval) {
        E0 = nc ? nc->ext : D.a_ext[p];
        v0 = cafe_vh(D, K, p);
      }
      S.cth[lane] = cafe_geo_costh(dn);
      S.l[lane] = cafe_geo_l(K, ci, cj, ck, si, sj, sk);
    } else if (w == 1) {
      S.sph[lane] = cafe_geo_sinph(dn);
    } else {
      const double *Rg = D.rot + 9LL * (gp - 1);
      for (int a = 0; a < 9; ++a) R[a] = Rg[a];
      dr = cafe_geo_loc(R, dn, loc);
      s0i = cafe_geo_corners(loc, dr, pk);
      if (w == 2) {
        S.dr[lane] = dr;
        cafe_geo_edge(loc, pk[0], pk[1], &S.d1I[lane], &S.dI2[lane]);
      } else {
        cafe_geo_edge(loc, pk[0], pk[2], &S.d1J[lane], &S.dJ3[lane]);
        if (eval) S.ruqs[lane] = .5 * (D.a_ruq[p] + D.a_ruq[q]);
      }
    }
  }
#ifdef CAFE_DETAIL_CYCLES
  long long fq1 = clock64();
#endif
  cafe_bar_quad();
#ifdef CAFE_DETAIL_CYCLES
  long long fq2 = clock64();
#endif
  // second stage, no barrier after it: warp 0 forms g and the capture time
  // and takes the row's best candidate, warp 1 forms g and orders the slots,
  // warps 2 and 3 finish the capture geometry (extent, centre), which only a
  // later capture by this row reads
  double gv = liv ? NAN : 0.0;  // a capturing cell without a grain never captures
  unsigned long long ak = 0ULL;
#ifdef CAFE_DETAIL_CYCLES
  long long fq3 = clock64();
#endif
  if (w <= 1) {
    double f = 0.0;
    if (work) {
      f = crm_pow_half(S.cth[lane] * S.sph[lane]);
      gv = f * S.dr[lane];
    }
    if (w == 0) {
      double t = NAN;
      if (work && eval) {
        double dr2 = gv - E0;
        t = dr2 / v0;
      }
      if (liv) D.row_g[r * CAFE_NSLOT + lane] = gv;
      ak = cafe_row_finish_warp(D, K, r, p, nn, liv, gv, q, eval, ev, T, true, t, work ? S.ruqs[lane] : 0.0,
                                CAFE_FIN_BEST);
    } else {
      // the slot order (read only by later evaluations)
      cafe_row_finish_warp(D, K, r, p, nn, liv, gv, q, false, ev, T, false, 0.0, 0.0, CAFE_FIN_ORDER);
    }
  } else if (work) {
    double Lmud = cafe_geo_lmud(K, S.l[lane], S.d1I[lane], S.dI2[lane], S.d1J[lane], S.dJ3[lane]);
    double *o = D.row_geo + (r * CAFE_NSLOT + lane) * 4;
    if (w == 2) {
      double f = crm_pow_half(S.cth[lane] * S.sph[lane]);
      o[0] = f * Lmud * 1.0;
    } else {
      double cn[3];
      cafe_geo_centre(R, cs, pk[0], s0i, Lmud, cn);
      o[1] = cn[0];
      o[2] = cn[1];
      o[3] = cn[2];
    }
  }
#ifdef CAFE_DETAIL_CYCLES
  if (lane == 0) {
    long long fq4 = clock64();
    atomicAdd(&D.stat[STAT_DETAIL + 16 + w], (unsigned long long)(fq1 - fq0));
    if (w >= 2) atomicAdd(&D.stat[STAT_DETAIL + 18 + w], (unsigned long long)(fq4 - fq3));
    if (w == 0) {
      atomicAdd(&D.stat[STAT_DETAIL + 22], (unsigned long long)(fq4 - fq3));
      atomicAdd(&D.stat[STAT_DETAIL + 23], 1ULL);
    }
  }
#endif
  return ak;
}

// ------------------------------------------------------------------ event loop
// A capture candidate: time t and tie-break ruqs, compared through their
// order keys (equal doubles give equal keys; NaN times are never candidates).
struct CafeCand {
  unsigned long long tk, rk;
  double t, ruqs;
  int j, s;  // vs2 index and neighbour slot of the capturing cell; j < 0 = none
  int r, p, q;  // (not compared) its row, its active position and the captured position
};
__device__ __forceinline__ CafeCand cafe_cand_none() {
  CafeCand c;
  c.tk = c.rk = CAFE_KEY_NONE;
  c.t = c.ruqs = 0.0;
  c.j = -1;
  c.s = 0;
  c.r = c.p = c.q = 0;
  return c;
}
__device__ __forceinline__ bool cafe_cand_better(const CafeCand &a, const CafeCand &b) {
  // lexicographic (t, ruqs, scan position): VoxelsCA.C:427-440 keeps the first
  // scanned candidate among full ties
  if (a.j < 0) return false;
  if (b.j < 0) return true;
  if (a.tk != b.tk) return a.tk < b.tk;
  if (a.rk != b.rk) return a.rk < b.rk;
  if (a.j != b.j) return a.j < b.j;
  return a.s < b.s;
}
__device__ __forceinline__ CafeCand cafe_shfl_cand(const CafeCand &c, int o) {
  CafeCand r;
  r.tk = cafe_shfl_u64_xor(c.tk, o);
  r.rk = cafe_shfl_u64_xor(c.rk, o);
  r.t = __shfl_xor_sync(0xffffffffu, c.t, o);
  r.ruqs = __shfl_xor_sync(0xffffffffu, c.ruqs, o);
  r.j = __shfl_xor_sync(0xffffffffu, c.j, o);
  r.s = __shfl_xor_sync(0xffffffffu, c.s, o);
  r.r = __shfl_xor_sync(0xffffffffu, c.r, o);
  r.p = __shfl_xor_sync(0xffffffffu, c.p, o);
  r.q = __shfl_xor_sync(0xffffffffu, c.q, o);
  return r;
}
// Best candidate of the warp, in every lane.
__device__ __forceinline__ CafeCand cafe_warp_best(CafeCand best) {
  for (int o = 16; o > 0; o >>= 1) {
    CafeCand c = cafe_shfl_cand(best, o);
    if (cafe_cand_better(c, best)) best = c;
  }
  return best;
}
#define CAFE_KEY_1E6 0xc12e848000000000ULL  // cafe_key(1e6)

// Best candidate of frontier row r (VoxelsCA.C:386-445 restricted to one cell)
// with the row cell's current extent. For a positive finite growth velocity the
// capture time fl(fl(g - E)/v) is non-decreasing in g, so the live slots are
// visited in g order and the visit stops at the first time above the row's
// minimum; otherwise every live slot is evaluated. `bounded` applies the
// reference's acceptance limit t <= 1e6 (VoxelsCA.C:383, 427).
__device__ __forceinline__ void cafe_row_best_live(const CafeDev &D, const CafeConsts &K, long long r,
                                                   uint32_t live, CafeCand &best, bool bounded,
                                                   unsigned long long *k2out = nullptr) {
  int p = D.row_pos[r];
  if (!live) return;
  double E = D.row_E[r];
  double v = cafe_vh(D, K, p);
  long long vb = crm_bits(v);
  bool mono = vb > 0 && vb < CRM_BITS_INF;  // 0 < v < inf
  const double *g = D.row_g + r * CAFE_NSLOT;
  const uint8_t *ord = D.row_ord + r * CAFE_NSLOT;
  const int32_t *nbr = D.a_nbr + (long long)p * CAFE_NSLOT;
  int nn = D.a_nn[p];
  int jrow = D.row_j[r];
  double ruq_p = D.a_ruq[p];
  bool have = false;
  unsigned long long tfirst = 0;
  // with k2out (best enters empty): the smallest time key of the candidates
  // other than the best one; in g order the slot that ends the visit has it
  unsigned long long k2 = CAFE_KEY_NONE;
  // visits slot s of order position k with numerator gs and neighbour q:
  // 0 go on, 1 the visit ends
  auto visit = [&](int k, int s, double gs, int q) -> int {
    if (!(live >> s & 1u)) return 0;
    double dr = gs - E;
    double t = dr / v;
    if (cafe_is_nan(t)) return 0;
    unsigned long long tk = cafe_key_canon(t);
    if (bounded && !(tk <= CAFE_KEY_1E6)) return mono ? 1 : 0;
    if (mono && have && tk > tfirst) {
      k2 = min(k2, tk);
      return 1;
    }
    CafeCand c;
    c.t = t;
    c.tk = tk;
    c.ruqs = .5 * (ruq_p + D.a_ruq[q]);
    c.rk = cafe_key_canon(c.ruqs);
    c.j = jrow;
    c.s = s;
    c.r = (int)r;
    c.p = p;
    c.q = q;
    if (cafe_cand_better(c, best)) {
      if (have) k2 = min(k2, best.tk);
      best = c;
    } else {
      k2 = min(k2, tk);
    }
    if (!have) {
      have = true;
      tfirst = tk;
    }
    return 0;
  };
  // the first four slots of the visiting order with their numerators and
  // neighbours, loaded together (a visit usually ends within them)
  int s4[4], q4[4];
  double g4[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) s4[i] = i < nn ? (mono ? (int)ord[i] : i) : 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    g4[i] = i < nn ? g[s4[i]] : 0.0;
    q4[i] = i < nn ? nbr[s4[i]] : 0;
  }
  bool ended = false;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (!ended && i < nn) ended = visit(i, s4[i], g4[i], q4[i]) != 0;
  for (int k = 4; k < nn && !ended; ++k) {
    int s = mono ? ord[k] : k;
    ended = visit(k, s, g[s], nbr[s]) != 0;
  }
  if (k2out) *k2out = k2;
}
__device__ __forceinline__ void cafe_row_best(const CafeDev &D, const CafeConsts &K, long long r,
                                              CafeCand &best, bool bounded = true) {
  cafe_row_best_live(D, K, r, D.row_live[r], best, bounded);
}

// Slot of `target` in q's neighbour list, -1 if absent. All CAFE_NSLOT entries
// are loaded at once (the list storage is always that long) and masked by nn.
__device__ __forceinline__ int cafe_find_slot(const CafeDev &D, int q, int target) {
  int nn = D.a_nn[q];
  const int32_t *nb = D.a_nbr + (long long)q * CAFE_NSLOT;
  int found = -1;
#pragma unroll
  for (int s = CAFE_NSLOT - 1; s >= 0; --s) {
    int v = nb[s];
    if (s < nn && v == target) found = s;
  }
  return found;
}

// ---- keyed rows -------------------------------------------------------------
// Every frontier cell of a step grows by the same fl(v * DtMin) at every capture
// event while it has a liquid neighbour (VoxelsCA.C:511-516), and a row's
// candidate times all fall by about DtMin per event. A row therefore carries a
// key: the absolute time T + t_best of its best candidate when it was last
// evaluated exactly. Between evaluations the key is within a small rounding
// bound of the row's exact current value (or below it once a candidate was
// captured by someone else), so the event needs exact times only for the rows
// whose key lies within twice that bound of the smallest key. When the row's
// best candidate is the one captured elsewhere, the key becomes row_key2, the
// key of the row's next candidate at the same evaluation, which bounds the
// row's exact value the same way. An extent that a
// negative event may clamp at zero (VoxelsCA.C:515) breaks the bound; such rows
// are stamped -1 and evaluated again. The growth is logged once per event and
// replayed per row when the row is evaluated, and for every row at the end of
// the step (k_rows_finalize).
#define CAFE_ALIVE 0x7fffffff   // row_death of a row that is still alive
#define CAFE_M_DONE 0x7fffffff  // row_m of a row whose extent is kept current
#ifndef CAFE_CATCHUP
#define CAFE_CATCHUP 2  // logged events a selecting thread replays per event for its second row
#endif

// Applies the logged growth of events row_m+1 .. min(upto, row_death). A
// nucleation logs +0, which leaves an extent unchanged (extents are never -0).
__device__ __forceinline__ void cafe_row_replay(const CafeDev &D, int r, int upto) {
  int m = D.row_m[r];
  int stop = min(upto, D.row_death[r]);
  if (stop <= m) return;
  double E = D.row_E[r];
  for (int k = m + 1; k <= stop; ++k) {
    E = E + D.ev_vd[k];
    E = cafe_is_neg(E) ? 0.0 : E;  // (E < 0.0) ? 0.0 : E
  }
  D.row_E[r] = E;
  D.row_m[r] = stop;
}

// Exact evaluation of row r (live slots `live`) for the iteration after `ev`
// events at time T.
__device__ __forceinline__ void cafe_row_eval_live(const CafeDev &D, const CafeConsts &K, int r, int ev,
                                                   double T, uint32_t live) {
#ifdef CAFE_DETAIL_CYCLES
  long long rp0 = clock64();
  int rm0 = D.row_m[r];
#endif
  cafe_row_replay(D, r, ev);
#ifdef CAFE_DETAIL_CYCLES
  atomicAdd(&D.stat[STAT_DETAIL + 27], (unsigned long long)(D.row_m[r] - rm0 > 0 ? D.row_m[r] - rm0 : 0));
  atomicAdd(&D.stat[STAT_DETAIL + 28], 1ULL);
  atomicAdd(&D.stat[STAT_DETAIL + 29], (unsigned long long)(clock64() - rp0));
#endif
  CafeCand b = cafe_cand_none();
#ifdef CAFE_DETAIL_CYCLES
  long long be0 = clock64();
#endif
  unsigned long long k2;
  cafe_row_best_live(D, K, r, live, b, false, &k2);
#ifdef CAFE_DETAIL_CYCLES
  atomicAdd(&D.stat[STAT_DETAIL + 30], (unsigned long long)(clock64() - be0));
  atomicAdd(&D.stat[STAT_DETAIL + 31], 1ULL);
#endif
  D.row_stamp[r] = ev + 1;
  if (b.j < 0) {
    D.row_key[r] = CAFE_KEY_NONE;
    return;
  }
  D.row_bt[r] = b.t;
  D.row_bruq[r] = b.ruqs;
  D.row_bslot[r] = b.s;
  D.row_bq[r] = b.q;
  const unsigned long long key = cafe_key(T + b.t);
  D.row_key[r] = key;
  D.row_key2[r] = k2 == CAFE_KEY_NONE ? key : cafe_key(T + cafe_unkey(k2));
}
__device__ __forceinline__ void cafe_row_eval(const CafeDev &D, const CafeConsts &K, int r, int ev,
                                              double T) {
  cafe_row_eval_live(D, K, r, ev, T, D.row_live[r]);
}

// Frontier rows of the step, in three passes so that the capture geometry,
// the expensive part, runs with one (row, slot) pair per lane:
// k_rows_prep (one warp per row) finds each row's liquid neighbours, sets the
// row's extent and growth watermark, and lists the pairs that need geometry;
// k_rows_geo evaluates the listed pairs; k_rows_order (one warp per row)
// orders each row's slots and, when every row grows with the same velocity,
// takes its exact best candidate and key.
__device__ __forceinline__ void d_rows_prep(const CafeDev &D, const CafeConsts &K, const int cafe_bid, const int cafe_nblk) {
  int nrows = D.ctr[CTR_NROWS];
  if (nrows > D.row_cap) nrows = (int)D.row_cap;
  const int warps = (cafe_nblk * blockDim.x) >> 5;
  const int w = (cafe_bid * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  const double V = K.vhat_cls[1];
  for (int r = w; r < nrows; r += warps) {
    int p = D.row_pos[r];
    int nn = D.a_nn[p];
    int gp = D.a_gid[p];
    bool grain_ok = gp >= 1 && gp <= D.grain_cap;
    bool liv = false;
    if (lane < nn) liv = D.a_state[D.a_nbr[(long long)p * CAFE_NSLOT + lane]] == 1;
    if (liv && !grain_ok) D.row_g[(long long)r * CAFE_NSLOT + lane] = NAN;  // never captures
    uint32_t work = __ballot_sync(FULL, liv && grain_ok);
    int base = 0;
    if (lane == 0 && work) base = atomicAdd(&D.ctr[CTR_NPAIRS], __popc(work));
    base = __shfl_sync(FULL, base, 0);
    if (work >> lane & 1u) D.row_pairs[base + __popc(work & ((1u << lane) - 1u))] = r * 32 + lane;
    if (lane == 0) {
      D.row_E[r] = D.a_ext[p];
      D.row_m[r] = 0;
      D.row_death[r] = CAFE_ALIVE;
      if (D.a_cls[p] != 1 || !(V > 0.0 && V < INFINITY)) atomicOr(&D.ctr[CTR_SLOW], 1);
    }
  }
}
__global__ void k_rows_prep(CafeDev D, CafeConsts K) {
  d_rows_prep(D, K, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void d_rows_geo(const CafeDev &D, const CafeConsts &K, const int cafe_bid, const int cafe_nblk) {
  int n = D.ctr[CTR_NPAIRS];
  const long long cap = D.row_cap * CAFE_NSLOT;
  if (n > cap) n = (int)cap;
  for (int i = cafe_bid * blockDim.x + threadIdx.x; i < n; i += cafe_nblk * blockDim.x) {
    int v = D.row_pairs[i];
    int r = v >> 5, sl = v & 31;
    int p = D.row_pos[r];
    int q = D.a_nbr[(long long)p * CAFE_NSLOT + sl];
    const double *Rg = D.rot + 9LL * (D.a_gid[p] - 1);
    double Rm[9];
    for (int a = 0; a < 9; ++a) Rm[a] = Rg[a];
    int i0, j0, k0, si, sj, sk;
    cafe_cell_xyz(K, D.act[q], i0, j0, k0);
    cafe_cell_xyz(K, D.act[p], si, sj, sk);
    double cs[3] = {D.a_cx[p], D.a_cy[p], D.a_cz[p]};
    double g, e, cn[3];
    cafe_capture_geometry(K, i0, j0, k0, si, sj, sk, cs, Rm, &g, &e, cn);
    long long o = (long long)r * CAFE_NSLOT + sl;
    D.row_g[o] = g;
    double *og = D.row_geo + o * 4;
    og[0] = e;
    og[1] = cn[0];
    og[2] = cn[1];
    og[3] = cn[2];
  }
}
__global__ void k_rows_geo(CafeDev D, CafeConsts K) {
  d_rows_geo(D, K, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void d_rows_order(const CafeDev &D, const CafeConsts &K, const int cafe_bid, const int cafe_nblk) {
  int nrows = D.ctr[CTR_NROWS];
  if (nrows > D.row_cap) nrows = (int)D.row_cap;
  const int warps = (cafe_nblk * blockDim.x) >> 5;
  const int w = (cafe_bid * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (int r = w; r < nrows; r += warps) {
    int p = D.row_pos[r];
    int nn = D.a_nn[p];
    int q = 0;
    bool liv = false;
    double gv = 0.0;
    if (lane < nn) {
      q = D.a_nbr[(long long)p * CAFE_NSLOT + lane];
      liv = D.a_state[q] == 1;
      if (liv) gv = D.row_g[(long long)r * CAFE_NSLOT + lane];
    }
    cafe_row_finish_warp(D, K, r, p, nn, liv, gv, q, true, 0, 0.0);
  }
}
__global__ void k_rows_order(CafeDev D, CafeConsts K) {
  d_rows_order(D, K, blockIdx.x, gridDim.x);
}

// ---- event selection by a group of warps ------------------------------------
// Shared scratch of one selecting group (up to 16 warps).
struct CafeSelShared {
  unsigned long long redk[16];
  CafeCand red[16];
  unsigned long long kthr;
  long long evals;  // selection rounds that evaluated rows exactly
#ifdef CAFE_DETAIL_CYCLES
  long long cyc[4], rounds;
#endif
};
// bar.sync on a named barrier, with an OR reduction of v over the n threads.
__device__ __forceinline__ int cafe_bar_or(int id, int n, int v) {
  int r;
  asm volatile(
      "{ .reg .pred p, q;\n\t"
      "setp.ne.s32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.s32 %0, 1, 0, p; }"
      : "=r"(r)
      : "r"(v), "r"(id), "r"(n)
      : "memory");
  return r;
}
__device__ __forceinline__ void cafe_bar_n(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// Smallest and second smallest key (and rows) of a sequence of rows: row r
// with key k enters.
__device__ __forceinline__ void cafe_top2(unsigned long long k, int r, unsigned long long &m, int &mr,
                                          unsigned long long &m2, int &r2) {
  if (k < m) {
    m2 = m;
    r2 = mr;
    m = k;
    mr = r;
  } else if (k < m2) {
    m2 = k;
    r2 = r;
  }
}

// Keyed selection of the best capture among rows [0, nrows) for the iteration
// after `ev` events at time T (VoxelsCA.C:386-480 restricted to the rows that
// can hold the minimum), by the group of gn threads (gtid = 0..gn-1) that
// shares named barrier `bar`. Thread gtid owns rows r = gtid (mod gn) and keeps
// the smallest key among them in my_min, with its row in my_hot, and the
// smallest key of its other rows in my_u2, with its row in my_r2 (-1 none; -2
// not known), all rescanned when dirty[gtid] is set; a forced[gtid] flag makes
// it evaluate its rows stamped -1. Every key change made elsewhere (a row's
// key raised, a row's death, a new row) sets dirty, so between rescans the
// thread's own evaluations are the only changes. The result is left
// in S.red[0] (valid after the group's next barrier; every group thread has
// passed the last barrier when this returns).
__device__ void cafe_select_keyed(const CafeDev &D, const CafeConsts &K, int ev, double T, int nrows, int gtid,
                                  int gn, int bar, unsigned long long &my_min, int &my_hot,
                                  unsigned long long &my_u2, int &my_r2, bool &my_forced, unsigned char *dirty,
                                  unsigned char *forced, CafeSelShared &S, double gmax, double emax, double dsum,
                                  double V) {
  const int lane = gtid & 31, gw = gtid >> 5, ngw = gn >> 5;
#ifdef CAFE_DETAIL_CYCLES
  long long sc0 = cafe_clock_ordered();
#endif
  if (forced[gtid]) {
    forced[gtid] = 0;
    my_forced = true;
  }
  if (dirty[gtid]) {
    dirty[gtid] = 0;
    unsigned long long m = CAFE_KEY_NONE, m2 = CAFE_KEY_NONE;
    int mr = -1, r2 = -1;
    // batches of eight loads in flight together
    for (int r0 = gtid; r0 < nrows; r0 += 8 * gn) {
      unsigned long long kk[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int r = r0 + i * gn;
        kk[i] = r < nrows ? D.row_key[r] : CAFE_KEY_NONE;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) cafe_top2(kk[i], r0 + i * gn, m, mr, m2, r2);
    }
    my_min = m;
    my_hot = mr;
    my_u2 = m2;
    my_r2 = r2;
  }
  CafeCand best;
  // this thread's last scan in this selection: marked rows, the two smallest
  // keys of the others
  bool sc_have = false;
  uint32_t sc_mark = 0;
  unsigned long long sc_u = CAFE_KEY_NONE, sc_u2 = CAFE_KEY_NONE;
  int sc_ur = -1, sc_r2 = -1;
#ifdef CAFE_DETAIL_CYCLES
  long long sc1 = cafe_clock_ordered();
  if (gtid == 0) S.cyc[0] += sc1 - sc0;  // dirty rescan
#endif
  while (true) {
#ifdef CAFE_DETAIL_CYCLES
    long long sr0 = cafe_clock_ordered();
#endif
    unsigned long long km = my_min;
    for (int o = 16; o > 0; o >>= 1) km = min(km, cafe_shfl_u64_xor(km, o));
    if (lane == 0) S.redk[gw] = km;
    cafe_bar_n(bar, gn);
    if (gw == 0) {
      km = lane < ngw ? S.redk[lane] : CAFE_KEY_NONE;
      for (int o = 16; o > 0; o >>= 1) km = min(km, cafe_shfl_u64_xor(km, o));
      if (lane == 0) {
        unsigned long long kt = CAFE_KEY_NONE;
        if (km != CAFE_KEY_NONE) {
          // rows whose exact value may be the minimum: keys within twice the
          // rounding bound delta = (ev+16) 2^-48 (|K*| + |T| + (gmax+emax)/v
          // + 2 sum|dt| + 1e-300); the magnitude is bounded by a power of
          // two from the exponents of its terms (below 8 times the largest)
          double kd = cafe_unkey(km);
          int eg = max(cafe_exp_ub(gmax), cafe_exp_ub(emax)) + 1 - cafe_exp_lb(V);
          int em = max(max(cafe_exp_ub(kd), cafe_exp_ub(T)), max(eg, cafe_exp_ub(dsum) + 1)) + 3;
          int ed = em - 47;  // 2 delta < (ev+16) 2^ed
          if (ed > -126 && ed < 100 && ev < (1 << 24)) {
            float delta2 = (float)(ev + 16) * __int_as_float((ed + 127) << 23);
            double thr = kd + (double)delta2;
            kt = cafe_is_nan(thr) ? CAFE_KEY_NONE : cafe_key(thr);
          } else {
            double magd = fabs(kd) + fabs(T) + (gmax + emax) / V + 2.0 * dsum + 1e-300;
            double thr = kd + 2.0 * ((double)(ev + 16) * 0x1p-48 * magd);
            kt = cafe_is_nan(thr) ? CAFE_KEY_NONE : cafe_key(thr);
          }
        }
        S.kthr = kt;
      }
    }
    cafe_bar_n(bar, gn);
#ifdef CAFE_DETAIL_CYCLES
    long long sr1 = cafe_clock_ordered();
    if (gtid == 0) S.cyc[1] += sr1 - sr0;  // minimum and threshold
#endif
    const unsigned long long kthr = S.kthr;
    int again = 0;
#ifdef CAFE_DETAIL_CYCLES
    long long eval_cyc = 0, phase_a = 0;
    int n_mark = 0;
#endif
    best = cafe_cand_none();
    if (kthr != CAFE_KEY_NONE && (my_min <= kthr || my_forced)) {
      // visits row r: evaluates it when its key may be the minimum and was not
      // evaluated for this iteration (or when it is forced), takes its best
      // candidate when its key is at or below the threshold, returns the key
      auto visit = [&](int r) -> unsigned long long {
        unsigned long long k = D.row_key[r];
        int stamp = D.row_stamp[r];
        // stamp -1: forced after a possible clamp of the row's extent
        if ((k <= kthr && stamp != ev + 1) || (stamp == -1 && D.row_alive[r])) {
#ifdef CAFE_DETAIL_CYCLES
          long long ev0 = cafe_clock_ordered();
#endif
          cafe_row_eval(D, K, r, ev, T);
#ifdef CAFE_DETAIL_CYCLES
          eval_cyc += cafe_clock_ordered() - ev0;
#endif
          k = D.row_key[r];
          again = 1;
        }
        if (k <= kthr) {
          CafeCand c;
          c.t = D.row_bt[r];
          c.ruqs = D.row_bruq[r];
          c.tk = cafe_key_canon(c.t);
          c.rk = cafe_key_canon(c.ruqs);
          c.j = D.row_j[r];
          c.s = D.row_bslot[r];
          c.r = r;
          c.p = D.row_pos[r];
          c.q = D.row_bq[r];
          if (cafe_cand_better(c, best)) best = c;
        }
        return k;
      };
      if (!my_forced && my_r2 != -2 && my_u2 > kthr && my_hot >= 0) {
        // every other row of this thread has a key above the threshold: only
        // the smallest-key row is visited and no other key is loaded
#ifdef CAFE_DETAIL_CYCLES
        n_mark += 1;
#endif
        const unsigned long long k = visit(my_hot);
        if (k <= my_u2) {
          my_min = k;
        } else {
          // the second row is now the smallest; the next one is not known
          my_min = my_u2;
          my_hot = my_r2;
          my_r2 = -2;
        }
      } else {
        unsigned long long m = CAFE_KEY_NONE, m2 = CAFE_KEY_NONE;
        int mr = -1, r2 = -1;
        // this thread's rows r = r0 + i gn, 32 at a time: first their keys,
        // loaded together, mark the rows at or below the threshold (and, when
        // forced, the rows stamped -1); then only the marked rows are visited.
        // Within one selection only this thread changes its rows, and only
        // marked ones: with its rows in one chunk, a later round whose
        // threshold lies below the smallest unmarked key of the last scan
        // visits the same marked rows again without loading the other keys.
        const bool one_chunk = nrows <= 32 * gn;
        for (int r0 = gtid; r0 < nrows; r0 += 32 * gn) {
          uint32_t mark = 0;
          if (one_chunk && sc_have && !my_forced && sc_u > kthr) {
            mark = sc_mark;
            m = sc_u;
            mr = sc_ur;
            m2 = sc_u2;
            r2 = sc_r2;
          } else {
#ifdef CAFE_DETAIL_CYCLES
            long long pa0 = cafe_clock_ordered();
#endif
            // (branch-free batches of eight loads, so that they are in flight
            // together)
#pragma unroll
            for (int b = 0; b < 32; b += 8) {
              if (r0 + b * gn >= nrows) break;
              unsigned long long kk[8];
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                const int r = r0 + (b + i) * gn;
                kk[i] = r < nrows ? D.row_key[r] : CAFE_KEY_NONE;
              }
              uint32_t fm = 0;  // rows stamped -1, visited whatever their key
              if (my_forced) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                  const int r = r0 + (b + i) * gn;
                  fm |= (r < nrows && D.row_stamp[r] == -1) ? 1u << i : 0u;
                }
              }
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                // a visited row's key enters the two smallest after its visit
                if (kk[i] <= kthr || (fm >> i & 1u))
                  mark |= 1u << (b + i);
                else
                  cafe_top2(kk[i], r0 + (b + i) * gn, m, mr, m2, r2);
              }
            }
#ifdef CAFE_DETAIL_CYCLES
            phase_a += cafe_clock_ordered() - pa0;
            n_mark += __popc(mark);
#endif
            if (one_chunk) {
              sc_have = true;
              sc_mark = mark;
              sc_u = m;
              sc_ur = mr;
              sc_u2 = m2;
              sc_r2 = r2;
            }
          }
          while (mark) {
            const int r = r0 + (__ffs(mark) - 1) * gn;
            mark &= mark - 1;
            cafe_top2(visit(r), r, m, mr, m2, r2);
          }
        }
        my_min = m;
        my_hot = mr;
        my_u2 = m2;
        my_r2 = r2;
        my_forced = false;
      }
    }
#ifdef CAFE_DETAIL_CYCLES
    if (again) {
      // scan time of the evaluating threads apart from their evaluations
      atomicAdd(&D.stat[STAT_DETAIL + 10], (unsigned long long)(cafe_clock_ordered() - sr1 - eval_cyc));
      atomicAdd(&D.stat[STAT_DETAIL + 11], 1ULL);
      atomicAdd(&D.stat[STAT_DETAIL + 12], (unsigned long long)eval_cyc);
      atomicAdd(&D.stat[STAT_DETAIL + 14], (unsigned long long)phase_a);
      atomicAdd(&D.stat[STAT_DETAIL + 15], (unsigned long long)n_mark);
    }
#endif
#ifdef CAFE_DETAIL_CYCLES
    long long sr2 = cafe_clock_ordered();
    if (gtid == 0) S.cyc[2] += sr2 - sr1;  // scan and evaluations (this thread)
#endif
    again = cafe_bar_or(bar, gn, again);
#ifdef CAFE_DETAIL_CYCLES
    if (gtid == 0) {
      S.cyc[3] += cafe_clock_ordered() - sr2;  // waiting for the slowest thread's evaluations
      S.rounds++;
    }
#endif
    if (gtid == 0 && again) S.evals++;
    if (!again) break;
  }
  best = cafe_warp_best(best);
  if (lane == 0) S.red[gw] = best;
  cafe_bar_n(bar, gn);
  if (gw == 0) {
    CafeCand b = lane < ngw ? S.red[lane] : cafe_cand_none();
    b = cafe_warp_best(b);
    if (lane == 0) S.red[0] = b;
  }
}

// The capture/nucleation loop of one step (VoxelsCA.C:381-610), one block.
//
// Keyed mode (every frontier row grows with one velocity) pipelines two events:
// after the winner of event e is applied and the captured cell's neighbours are
// updated, warps 0-3 fill the row of the newly captured cell while warps 4-15
// select the best capture of event e+1 among the other rows. The winner of
// e+1 is the better of that selection and the new row's own exact best
// candidate: a row not evaluated by the selection has a key above the
// threshold, so its exact time is above the selected one. Per event: (1)
// thread 0 settles the winner (its candidate carries the row and both cells)
// with the draw made one event ahead and logs the growth; (2) thread 0 applies
// the capture or nucleation, warp 1 updates the captured cell's neighbours and
// their rows (row deaths, second-key promotions), thread 64 draws the next
// event's uniform, and on a negative event the selecting threads flag the rows
// whose extent may clamp; (3) the new-row fill beside the next selection; (4)
// thread 0 merges the two. Exact mode (the reference's per-event scan of every
// row, also the fallback when the rows stop sharing one velocity) evaluates
// every row at every event.
// ---- the fill helper: a second block of the event loop -----------------------
// A warp issues one FP64 instruction per ~64 cycles and each SM sub-partition
// completes one FP64 warp-instruction per ~64 cycles, so the new row's fill
// (its four warps' chains, ~20k cycles) saturates the FP64 pipes of the SM it
// runs on and slows the next event's selection there. With two blocks
// (cooperative launch: both resident), the main block posts the fill of each
// new row as soon as the event's winner is known, and the helper block, on
// another SM, fills the row while the main block applies the capture and
// selects the next event; the main block takes the result at the merge.
// Both sides wait with a wall-clock limit; a wait that runs out sets
// CAFE_ERR_SYNC and ends the step.
#define CAFE_SYNC_WAIT_NS 2000000000ULL
__device__ __forceinline__ unsigned long long cafe_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int cafe_ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void cafe_st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Thread 0: waits until *p != last (or == want when want >= 0); returns the
// value seen, or INT_MIN when the wait ran out (error bit set).
__device__ __forceinline__ int cafe_wait_seq(const CafeDev &D, const int *p, int last, int want) {
  const unsigned long long t0 = cafe_globaltimer();
  unsigned int spins = 0;
  while (true) {
    int v = cafe_ld_acquire(p);
    if (want >= 0 ? v == want : v != last) return v;
    if ((++spins & 255u) == 0 && cafe_globaltimer() - t0 > CAFE_SYNC_WAIT_NS) {
      atomicOr(D.err, CAFE_ERR_SYNC);
      return (int)0x80000000;
    }
  }
}

__device__ __noinline__ void cafe_fill_helper(const CafeDev &D, const CafeConsts &K, CafeQuadScratch &S) {
  __shared__ int s_cmd;
  __shared__ CafeFillReq s_req;
  const int tid = threadIdx.x;
  int last = 0;
  while (true) {
    if (tid == 0) {
      const int v = cafe_wait_seq(D, D.fill_seq, last, -1);
      s_cmd = v;
      if (v > 0) s_req = *D.fill;  // after the acquire: the main block's request
    }
    __syncthreads();
    const int v = s_cmd;
    if (v <= 0) return;  // -1: the main block left the keyed loop; INT_MIN: time-out
    last = v;
    if (tid < CAFE_QUAD_THREADS) {
      CafeNewCell nc;
      nc.c[0] = s_req.c[0];
      nc.c[1] = s_req.c[1];
      nc.c[2] = s_req.c[2];
      nc.ext = s_req.ext;
      nc.gid = s_req.gid;
      unsigned long long gk = cafe_row_fill_quad(D, K, s_req.r, s_req.p, true, s_req.e, s_req.T, S, &nc);
      if (tid == 0) D.fill->gk = gk;
    }
    __syncthreads();
    if (tid == 0) cafe_st_release(D.fill_seq + 1, v);  // orders the row's stores before it
  }
}

__device__ __forceinline__ void d_event_loop(const CafeDev &D, const CafeConsts &K, const CafeStepParams *__restrict__ Pp, long long max_events, int allow_fast, const int cafe_bid, const int cafe_nblk) {
  const CafeStepParams P = *Pp;
  constexpr int NSEL = CAFE_LOOP_THREADS - CAFE_QUAD_THREADS;  // threads of the selecting warps
  __shared__ CafeCand red[CAFE_LOOP_THREADS / 32];
  __shared__ CafeSelShared s_sel;
  __shared__ CafeCand s_best;  // winner of the next event (keyed mode)
  __shared__ double s_tinc, s_dt, s_dsum, s_gmax, s_emax, s_vd, s_vs;
  __shared__ int s_nvs2, s_countS, s_nrows, s_ngrain, s_done, s_nuc, s_icap, s_jspos, s_bslot, s_brow, s_na,
      s_slow, s_ev, s_switch, s_newrow;
  __shared__ unsigned char s_dirty[NSEL];   // a row of selecting thread i changed its key elsewhere
  __shared__ unsigned char s_forced[NSEL];  // a row of selecting thread i was stamped -1
  __shared__ uint32_t s_rng, s_rng_next;  // stream state after the consumed draws, after the next one
  __shared__ double s_unext;               // the next event's draw (VoxelsCA.C:483)
  __shared__ CafeNewCell s_nc;
  __shared__ unsigned int s_sdloc;
  __shared__ long long s_nnuc, s_negdt;
  __shared__ long long s_cyc[4];  // winner, capture + bookkeeping, new row || selection, merge
  __shared__ long long s_t0;
  __shared__ CafeQuadScratch s_quad;
#ifdef CAFE_DETAIL_CYCLES
  // finer event-loop sections, thread 0's clock (profiling builds only)
  __shared__ long long s_dcyc[16], s_dt0;
#define CAFE_DCYC(slot)                          \
  do {                                           \
    if (threadIdx.x == 0) {                      \
      long long _t = cafe_clock_ordered();       \
      s_dcyc[slot] += _t - s_dt0;                \
      s_dt0 = _t;                                \
    }                                            \
  } while (0)
  if (threadIdx.x < 16) s_dcyc[threadIdx.x] = 0;
  __shared__ unsigned long long s_fb0, s_sp0;
  if (threadIdx.x == 0) {
    s_dt0 = cafe_clock_ordered();
    s_fb0 = *(volatile unsigned long long *)&crm_fallback_calls;
    s_sp0 = *(volatile unsigned long long *)&crm_special_calls;
  }
#else
#define CAFE_DCYC(slot) \
  do {                  \
  } while (0)
#endif
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthr = blockDim.x, nwarp = blockDim.x >> 5;
  const int hid = tid - CAFE_QUAD_THREADS;  // index among the selecting warps (>= 0 there)
  if (cafe_bid == 1) {  // the fill helper (two-block launch)
    cafe_fill_helper(D, K, s_quad);
    return;
  }
  const bool use_helper = cafe_nblk == 2;
  __shared__ int s_post, s_seq;  // this event's fill went to the helper; requests posted
  const double V = K.vhat_cls[1];
  unsigned long long my_min = CAFE_KEY_NONE;  // smallest key of this selecting thread's rows
  int my_hot = -1;                            // ... and its row
  unsigned long long my_u2 = CAFE_KEY_NONE;   // smallest key of its other rows
  int my_r2 = -2;                             // ... and its row (-1 none, -2 not known)
  int hot_r = -1;                             // the row whose extent this thread keeps current
  bool hot_ok = false;                        // hot_E is its extent after event e - 1
  double hot_E = 0.0;
  int sec_r = -1;                             // likewise its second-smallest-key row
  bool sec_ok = false;
  double sec_E = 0.0;
  bool my_forced = false;                     // one of them is stamped -1
  if (hid >= 0) {
    s_dirty[hid] = 1;
    s_forced[hid] = 0;
  }
  if (tid == 0) {
    s_na = D.ctr[CTR_NA];
    s_nvs2 = D.ctr[CTR_NVS2];
    s_nrows = D.ctr[CTR_NROWS];
    s_ngrain = D.ctr[CTR_NGRAIN];
    uint32_t seed = cafe_minstd_seed((uint64_t)(uint32_t)(30 * P.tInd + (int)K.seed1));
    s_rng = cafe_minstd_skip(seed, 2ULL * (uint64_t)s_na);
    {
      // the first event's draw; later draws are made one event ahead
      cafe_uniform_stream st;
      st.x = s_rng;
      s_unext = cafe_uniform_next(&st);
      s_rng_next = st.x;
    }
    s_sdloc = K.seed0 + 32u * (unsigned int)P.tInd + 64u * (unsigned int)s_ngrain;
    s_tinc = 0.0;
    s_dsum = 0.0;
    s_vd = 0.0;
    s_vs = 0.0;
    s_countS = s_na;
    s_nnuc = 0;
    s_negdt = 0;
    s_sel.evals = 0;
#ifdef CAFE_DETAIL_CYCLES
    s_sel.cyc[0] = s_sel.cyc[1] = s_sel.cyc[2] = s_sel.cyc[3] = s_sel.rounds = 0;
#endif
    s_ev = 0;
    s_switch = 0;
    s_newrow = -1;
    s_post = 0;
    s_seq = 0;
    s_cyc[0] = s_cyc[1] = s_cyc[2] = s_cyc[3] = 0;
    D.ev_vd[0] = 0.0;
    D.ev_vs[0] = 0.0;
    s_slow = !allow_fast || D.ctr[CTR_SLOW] != 0;
    s_done = (*D.err != 0) || (s_na > D.act_cap) || (s_nvs2 > D.vs2_cap) || (s_nrows > D.row_cap);
    if (s_na + 2 > D.ev_cap) {
      atomicOr(D.err, CAFE_ERR_ITER_CAP);
      s_done = 1;
    }
  }
  __syncthreads();
  // ======================================================== keyed, pipelined
  if (!s_slow && !s_done) {
    // magnitudes for the key rounding bound: largest numerator and extent
    {
      unsigned long long gk = 0, ek = 0;
      for (int r = tid; r < s_nrows; r += nthr) {
        int p = D.row_pos[r];
        uint32_t live = D.row_live[r];
        int nn = D.a_nn[p];
        for (int k = 0; k < nn; ++k)
          if (live >> k & 1u) {
            double gv = fabs(D.row_g[(long long)r * CAFE_NSLOT + k]);
            if (!cafe_is_nan(gv)) gk = max(gk, cafe_key(gv));
          }
        const double er = D.row_E[r];  // NaN extents occur (the reference's 0/0) and are left out
        if (!cafe_is_nan(er)) ek = max(ek, cafe_key(fabs(er)));
      }
      for (int o = 16; o > 0; o >>= 1) {
        gk = max(gk, cafe_shfl_u64_xor(gk, o));
        ek = max(ek, cafe_shfl_u64_xor(ek, o));
      }
      if (lane == 0) {
        red[warp].tk = gk;
        red[warp].rk = ek;
      }
      __syncthreads();
      if (tid == 0) {
        unsigned long long g2 = 0, e2 = 0;
        for (int w = 0; w < nwarp; ++w) {
          g2 = max(g2, red[w].tk);
          e2 = max(e2, red[w].rk);
        }
        s_gmax = g2 ? cafe_unkey(g2) : 0.0;
        s_emax = e2 ? cafe_unkey(e2) : 0.0;
      }
      __syncthreads();
    }
    // selection of the first event
    if (hid >= 0)
      cafe_select_keyed(D, K, 0, 0.0, s_nrows, hid, NSEL, 2, my_min, my_hot, my_u2, my_r2, my_forced, s_dirty,
                        s_forced, s_sel, s_gmax, s_emax, s_dsum, V);
    __syncthreads();
    if (tid == 0) s_best = s_sel.red[0];
    __syncthreads();
    while (true) {
      // ---- (1) the winner of this event (VoxelsCA.C:427-505), thread 0
      if (tid == 0) {
        s_t0 = clock64();
        // while (vSind2 != countS && tinc < DelT)
        const bool tin = !cafe_is_nan(s_tinc) && cafe_key(s_tinc) < cafe_key(K.DelT);
        if (!(s_nvs2 != s_countS && tin)) s_done = 1;
        s_countS = s_nvs2;
        CafeCand b = s_best;
        if (!s_done) {
          if (b.j < 0 || !(b.tk < CAFE_KEY_1E6) || s_ev >= max_events) {
            if (b.j >= 0 && b.tk < CAFE_KEY_1E6) atomicOr(D.err, CAFE_ERR_ITER_CAP);
            s_done = 1;
          } else {
            // the draw made one event ahead from the current stream state
            const double U = s_unext;
            s_rng = s_rng_next;
            // (the candidate carries vs2[j], its row and the captured
            // position a_nbr[vs2[j], s])
            s_jspos = b.p;
            s_bslot = b.s;
            s_brow = b.r;
            s_icap = b.q;
            s_nuc = U < cafe_nuc_rate(D, K, s_icap);
            s_dt = s_nuc ? 0.0 : b.t;
            if (cafe_is_neg(s_dt)) s_negdt++;
            s_ev += 1;
            // log this event's growth of the rows (VoxelsCA.C:514)
            s_vd = s_nuc ? 0.0 : V * s_dt;
            D.ev_vd[s_ev] = s_vd;
            s_vs = s_vs + s_vd;
            D.ev_vs[s_ev] = s_vs;
            s_dsum += fabs(s_dt);
            s_tinc += s_dt;
            // hand the new row's fill to the helper block now when the
            // captured cell will start a row of the shared velocity class
            // (the condition phase 3 tests; the capture changes neither the
            // cell's liquid count nor its neighbours' states)
            s_post = 0;
            const int icp = s_icap;
            if (use_helper && !s_nuc && s_nrows < D.row_cap && D.a_liq[icp] > 0 && D.a_cold[icp] &&
                D.a_cls[icp] == 1) {
              CafeFillReq *F = D.fill;
              const double *gq = D.row_geo + ((long long)s_brow * CAFE_NSLOT + s_bslot) * 4;
              F->r = s_nrows;
              F->p = icp;
              F->e = s_ev;
              F->gid = D.a_gid[s_jspos];
              F->ext = gq[0];
              F->c[0] = gq[1];
              F->c[1] = gq[2];
              F->c[2] = gq[3];
              F->T = s_tinc;
              s_seq += 1;
              cafe_st_release(D.fill_seq, s_seq);
              s_post = 1;
            }
          }
        }
        long long tn = clock64();
        s_cyc[0] += tn - s_t0;
        s_t0 = tn;
      }
      __syncthreads();
      if (s_done) break;
      CAFE_DCYC(0);
      const int e = s_ev, icap = s_icap;
      const int nrows_ev = s_nrows;  // rows before this event's new row
      // ---- (2) the captured cell, its neighbours' rows, clamp flags
      if (tid == 0) {
        // the captured cell (VoxelsCA.C:483-505 and 518-605)
        const int js = s_jspos;
        D.a_state[icap] = 2;
        if (s_nvs2 < D.vs2_cap) {
          D.vs2[s_nvs2] = icap;
        } else {
          atomicOr(D.err, CAFE_ERR_MUSHY_CAP);
          s_done = 1;
        }
        s_nvs2 += 1;
        if (s_nuc) {
          int ci, cj, ck;
          cafe_cell_xyz(K, D.act[icap], ci, cj, ck);
          if (s_ngrain < D.grain_cap) {
            double q4[4];
            cafe_sample_orientation(K, s_sdloc, q4);
            double *c = D.cth + 4LL * s_ngrain;
            for (int a = 0; a < 4; ++a) c[a] = q4[a];
            cafe_rot_from_cth(c, D.rot + 9LL * s_ngrain);
          } else {
            atomicOr(D.err, CAFE_ERR_GRAIN_CAP);
            s_done = 1;
          }
          s_ngrain += 1;
          D.a_gid[icap] = s_ngrain;
          s_nc.gid = s_ngrain;
          D.a_cx[icap] = s_nc.c[0] = ((double)ci + .5) * K.dx[0];
          D.a_cy[icap] = s_nc.c[1] = ((double)cj + .5) * K.dx[1];
          D.a_cz[icap] = s_nc.c[2] = ((double)ck + .5) * K.dx[2];
          s_sdloc += 10u;
          D.a_ext[icap] = s_nc.ext = 0.0;
          s_nnuc++;
        } else {
          // the capture result of this slot, computed when the row was filled
          const int gcap = D.a_gid[js];
          if (gcap >= 1 && gcap <= D.grain_cap) {
            // the grain's rotation, read by the new row's fill
            cafe_prefetch_l1(D.rot + 9LL * (gcap - 1));
            cafe_prefetch_l1(D.rot + 9LL * (gcap - 1) + 8);
          }
          cafe_prefetch_l1(D.act + icap);
          D.a_gid[icap] = s_nc.gid = gcap;
          const double *gq = D.row_geo + ((long long)s_brow * CAFE_NSLOT + s_bslot) * 4;
          D.a_ext[icap] = s_nc.ext = gq[0];
          D.a_cx[icap] = s_nc.c[0] = gq[1];
          D.a_cy[icap] = s_nc.c[1] = gq[2];
          D.a_cz[icap] = s_nc.c[2] = gq[3];
        }
      } else if (warp == 1) {
        // neighbours of the captured cell lose one liquid neighbour
        const int nn = D.a_nn[icap];
        if (lane < nn) {
          int q = D.a_nbr[(long long)icap * CAFE_NSLOT + lane];
          // the new row's fill reads these next (nothing writes them here)
          cafe_prefetch_l1(D.a_state + q);
          cafe_prefetch_l1(D.act + q);
          // every load before the stores, so that the loads of one chain
          // level are in flight together
          const int liq = D.a_liq[q];
          const int r = D.a_frow[q];
          const int sl = cafe_find_slot(D, q, icap);
          const int rr = r >= 0 ? r : 0;
          const bool alive = r >= 0 && D.row_alive[rr];
          const uint32_t lv = D.row_live[rr];
          const int bs = D.row_bslot[rr];
          const unsigned long long k1 = D.row_key[rr], k2 = D.row_key2[rr];
          const int left = liq - 1;
          D.a_liq[q] = left;
          if (alive) {
            if (sl >= 0) D.row_live[r] = lv & ~(1u << sl);
            if (left <= 0) {
              D.row_alive[r] = 0;
              D.row_death[r] = e;  // it grew at this event too
              D.row_key[r] = CAFE_KEY_NONE;
              s_dirty[r % NSEL] = 1;
            } else if (sl >= 0 && sl == bs && k2 > k1) {
              // the row's best candidate is gone: its key rises to that of
              // its next candidate at the same evaluation, which bounds the
              // row's exact value from below as the old key did
              D.row_key[r] = k2;
              s_dirty[r % NSEL] = 1;
            }
          }
        }
      } else if (tid == 64) {
        // the next event's draw, off the winner section's chain (the stream
        // advances by two engine outputs per event whatever the event)
        cafe_uniform_stream st;
        st.x = s_rng;
        s_unext = cafe_uniform_next(&st);
        s_rng_next = st.x;
      } else if (hid >= 0) {
        if (!s_nuc && cafe_is_neg(s_dt)) {
          // a negative event may clamp a small extent at zero (VoxelsCA.C:515),
          // which breaks the key bound of that row: mark the rows whose
          // extrapolated extent comes near zero for re-evaluation
          const double vd = s_vd;
          const double margin = (double)(e + 16) * 0x1p-48 * (s_emax + s_gmax + V * s_dsum + 1e-300);
          const double vs_prev = D.ev_vs[e - 1];
          for (int r = hid; r < nrows_ev; r += NSEL) {
            if (D.row_death[r] < e) continue;
            int m = D.row_m[r];
            if (m >= e) continue;
            double elb = D.row_E[r] + (vs_prev - D.ev_vs[m]);
            if (elb + vd < margin) {
              D.row_stamp[r] = -1;
              s_forced[r % NSEL] = 1;
            }
          }
        }
        // this thread's smallest-key row is the one an exact evaluation of
        // the next selection most likely needs. Once its extent is current
        // (after that evaluation's replay) it is kept current, one addition
        // per event with the logged growth, held in registers and written
        // through, so that the next evaluation replays nothing: the same
        // additions in the same order as the lazy replay, only earlier (and
        // after the clamp check above, which reads the state before this
        // event). Only this thread writes its rows' extents in the keyed loop;
        // a row that dies marks its owner dirty, whose rescan moves my_hot.
        if (my_hot >= 0 && my_hot < nrows_ev) {
          if (hot_r != my_hot) {
            hot_r = my_hot;
            hot_ok = false;
          }
          if (!hot_ok && D.row_m[hot_r] == e - 1 && D.row_death[hot_r] >= e) {
            hot_E = D.row_E[hot_r];
            hot_ok = true;
          }
          if (hot_ok) {
            hot_E = hot_E + s_vd;
            hot_E = cafe_is_neg(hot_E) ? 0.0 : hot_E;  // (E < 0.0) ? 0.0 : E
            D.row_E[hot_r] = hot_E;
            D.row_m[hot_r] = e;
          }
        } else {
          hot_r = -1;
          hot_ok = false;
        }
        // The second-smallest-key row becomes the smallest when the smallest
        // one's key rises (its best candidate captured elsewhere). It is kept
        // current the same way; as it is rarely evaluated, it is first brought
        // up to date by a replay of at most CAFE_CATCHUP logged events per
        // event, in this section where the selecting threads are otherwise
        // idle. A row of this thread that dies marks it dirty, whose rescan
        // moves my_r2.
        if (my_r2 >= 0 && my_r2 < nrows_ev && my_r2 != hot_r) {
          if (sec_r != my_r2) {
            sec_r = my_r2;
            sec_ok = false;
          }
          if (!sec_ok) {
            // one level of loads: the row's death, watermark and extent, then
            // the logged growths (independent of the running extent)
            const int death = D.row_death[sec_r], m0 = D.row_m[sec_r];
            double E = D.row_E[sec_r];
            if (death >= e && m0 <= e - 1) {
              const int stop = min(e - 1, m0 + CAFE_CATCHUP);
#pragma unroll
              for (int i = 1; i <= CAFE_CATCHUP; ++i) {
                const int k = m0 + i;
                if (k <= stop) {
                  E = E + D.ev_vd[k];
                  E = cafe_is_neg(E) ? 0.0 : E;  // (E < 0.0) ? 0.0 : E
                }
              }
              if (stop == e - 1) {
                sec_E = E;
                sec_ok = true;
              } else {
                D.row_E[sec_r] = E;
                D.row_m[sec_r] = stop;
              }
            }
          }
          if (sec_ok) {
            sec_E = sec_E + s_vd;
            sec_E = cafe_is_neg(sec_E) ? 0.0 : sec_E;  // (E < 0.0) ? 0.0 : E
            D.row_E[sec_r] = sec_E;
            D.row_m[sec_r] = e;
          }
        } else {
          sec_r = -1;
          sec_ok = false;
        }
      }
      __syncthreads();
      CAFE_DCYC(1);
      if (tid == 0) {
        long long tn = clock64();
        s_cyc[1] += tn - s_t0;
        s_t0 = tn;
      }
      // ---- (3) the new row (warps 0-3) || selection of the next event (the rest)
      if (warp < CAFE_QUAD_THREADS / 32) {
        if (s_post) {
          // the helper fills this row: its bookkeeping here, its result at (4)
          if (tid == 0) {
            const int r = nrows_ev;
            D.row_pos[r] = icap;
            D.row_j[r] = s_nvs2 - 1;
            D.row_alive[r] = 1;
            D.a_frow[icap] = r;
            D.row_death[r] = CAFE_ALIVE;
            D.row_E[r] = D.a_ext[icap];
            D.row_m[r] = e;
          }
        } else if (D.a_liq[icap] > 0 && D.a_cold[icap] && !s_done) {
          int r = nrows_ev;
          if (r < D.row_cap) {
            if (tid == 0) {
              D.row_pos[r] = icap;
              D.row_j[r] = s_nvs2 - 1;
              D.row_alive[r] = 1;
              D.a_frow[icap] = r;
              D.row_death[r] = CAFE_ALIVE;
              D.row_E[r] = D.a_ext[icap];
              D.row_m[r] = e;
            }
            const bool same_v = D.a_cls[icap] == 1;
            unsigned long long gk = cafe_row_fill_quad(D, K, r, icap, same_v, e, s_tinc, s_quad, &s_nc);
            if (tid == 0) {
              if (!same_v) {
                s_switch = 1;
              } else {
                if (gk != 0ULL) {
                  double gm = cafe_unkey(gk);
                  if (gm > s_gmax) s_gmax = gm;
                }
                double ea = fabs(D.a_ext[icap]);
                if (ea > s_emax) s_emax = ea;
              }
              s_nrows = r + 1;
              s_newrow = r;
            }
          } else if (tid == 0) {
            atomicOr(D.err, CAFE_ERR_ROW_CAP);
            s_done = 1;
          }
        }
      } else {
        cafe_select_keyed(D, K, e, s_tinc, nrows_ev, hid, NSEL, 2, my_min, my_hot, my_u2, my_r2, my_forced, s_dirty,
                          s_forced, s_sel, s_gmax, s_emax, s_dsum, V);
      }
      __syncthreads();
      CAFE_DCYC(2);
      // ---- (4) the winner of the next event: selection or the new row
      if (tid == 0) {
        long long tn = clock64();
        s_cyc[2] += tn - s_t0;
        s_t0 = tn;
        if (s_post) {
          // the helper's fill of this event's new row (bounded wait)
          const int got = cafe_wait_seq(D, D.fill_seq + 1, 0, s_seq);
          if (got != s_seq) {
            s_done = 1;
          } else {
            const int r = nrows_ev;
            const unsigned long long gk = D.fill->gk;
            if (gk != 0ULL) {
              double gm = cafe_unkey(gk);
              if (gm > s_gmax) s_gmax = gm;
            }
            double ea = fabs(D.a_ext[icap]);
            if (ea > s_emax) s_emax = ea;
            s_nrows = r + 1;
            s_newrow = r;
          }
          s_post = 0;
        }
        CafeCand b = s_sel.red[0];
        const int r = s_newrow;
        if (r >= 0) {
          s_newrow = -1;
          s_dirty[r % NSEL] = 1;  // the row joins its owner's set
          if (D.row_key[r] != CAFE_KEY_NONE) {
            CafeCand c;
            c.t = D.row_bt[r];
            c.ruqs = D.row_bruq[r];
            c.tk = cafe_key_canon(c.t);
            c.rk = cafe_key_canon(c.ruqs);
            c.j = D.row_j[r];
            c.s = D.row_bslot[r];
            c.r = r;
            c.p = D.row_pos[r];
            c.q = D.row_bq[r];
            if (cafe_cand_better(c, b)) b = c;
          }
        }
        s_best = b;
        tn = clock64();
        s_cyc[3] += tn - s_t0;
        s_t0 = tn;
      }
      __syncthreads();
      CAFE_DCYC(3);
      if (s_switch) break;
    }
    if (s_switch && !s_done) {
      // a capturing cell with another growth velocity: bring every row up to
      // date and continue with the exact per-event scan
      for (int r = tid; r < s_nrows; r += nthr) {
        cafe_row_replay(D, r, s_ev);
        D.row_m[r] = CAFE_M_DONE;
      }
      __syncthreads();
      if (tid == 0) s_slow = 1;
      __syncthreads();
    }
  } else if (s_slow && !s_done) {
    // exact per-event scan with eager growth: extents are kept current
    for (int r = tid; r < s_nrows; r += nthr) D.row_m[r] = CAFE_M_DONE;
    __syncthreads();
  }
  // the helper block leaves (no request is outstanding here: every posted
  // fill is taken at (4) of its own event)
  if (use_helper && tid == 0) cafe_st_release(D.fill_seq, -1);
  // ======================================================== exact scan
  while (s_slow && !s_done) {
    if (tid == 0) {
      // while (vSind2 != countS && tinc < DelT)
      if (!(s_nvs2 != s_countS && s_tinc < K.DelT)) s_done = 1;
      s_countS = s_nvs2;
    }
    __syncthreads();
    if (s_done) break;
    // ---- every row's best candidate (VoxelsCA.C:386-445)
    CafeCand best = cafe_cand_none();
    for (int r = tid; r < s_nrows; r += nthr)
      if (D.row_alive[r]) cafe_row_best(D, K, r, best);
    best = cafe_warp_best(best);
    if (lane == 0) red[warp] = best;
    __syncthreads();
    if (warp == 0) {
      CafeCand b = lane < nwarp ? red[lane] : cafe_cand_none();
      b = cafe_warp_best(b);
      if (lane == 0) {
        if (b.j < 0 || !(b.tk < CAFE_KEY_1E6) || s_ev >= max_events) {
          if (b.j >= 0 && b.tk < CAFE_KEY_1E6) atomicOr(D.err, CAFE_ERR_ITER_CAP);
          s_done = 1;
        } else {
          cafe_uniform_stream st;
          st.x = s_rng;
          double U = cafe_uniform_next(&st);
          s_rng = st.x;
          int jspos = D.vs2[b.j];
          s_jspos = jspos;
          s_bslot = b.s;
          s_icap = D.a_nbr[(long long)jspos * CAFE_NSLOT + b.s];
          s_nuc = U < cafe_nuc_rate(D, K, s_icap);
          s_dt = s_nuc ? 0.0 : b.t;
          if (s_dt < 0.0) s_negdt++;
          s_ev += 1;
        }
      }
    }
    __syncthreads();
    if (s_done) break;
    // ---- growth of every mushy cell of the list (VoxelsCA.C:511-516)
    if (!s_nuc) {
      double d = s_dt;
      if (isfinite(d)) {
        for (int r = tid; r < s_nrows; r += nthr) {
          if (!D.row_alive[r]) continue;
          int p = D.row_pos[r];
          double e = D.row_E[r] + cafe_vh(D, K, p) * d;
          D.row_E[r] = (e < 0.0) ? 0.0 : e;
        }
      } else {
        // a non-finite DtMin also reaches the cells that have no liquid
        // neighbour (0 * inf)
        for (int j = tid; j < s_countS; j += nthr) {
          int p = D.vs2[j];
          int r = D.a_frow[p];
          double v = (r >= 0 && D.row_alive[r]) ? cafe_vh(D, K, p) : 0.0;
          double *ep = r >= 0 ? &D.row_E[r] : &D.a_ext[p];
          double e = *ep + v * d;
          *ep = (e < 0.0) ? 0.0 : e;
        }
      }
    }
    __syncthreads();
    const int icap = s_icap;
    // ---- the captured cell (VoxelsCA.C:483-505 and 518-605)
    if (tid == 0) {
      const int js = s_jspos;
      D.a_state[icap] = 2;
      if (s_nvs2 < D.vs2_cap) {
        D.vs2[s_nvs2] = icap;
      } else {
        atomicOr(D.err, CAFE_ERR_MUSHY_CAP);
        s_done = 1;
      }
      s_nvs2 += 1;
      if (s_nuc) {
        int ci, cj, ck;
        cafe_cell_xyz(K, D.act[icap], ci, cj, ck);
        if (s_ngrain < D.grain_cap) {
          double q4[4];
          cafe_sample_orientation(K, s_sdloc, q4);
          double *c = D.cth + 4LL * s_ngrain;
          for (int a = 0; a < 4; ++a) c[a] = q4[a];
          cafe_rot_from_cth(c, D.rot + 9LL * s_ngrain);
        } else {
          atomicOr(D.err, CAFE_ERR_GRAIN_CAP);
          s_done = 1;
        }
        s_ngrain += 1;
        D.a_gid[icap] = s_ngrain;
        D.a_cx[icap] = ((double)ci + .5) * K.dx[0];
        D.a_cy[icap] = ((double)cj + .5) * K.dx[1];
        D.a_cz[icap] = ((double)ck + .5) * K.dx[2];
        s_sdloc += 10u;
        D.a_ext[icap] = 0.0;
        s_nnuc++;
      } else {
        D.a_gid[icap] = D.a_gid[js];
        const double *gq = D.row_geo + ((long long)D.a_frow[js] * CAFE_NSLOT + s_bslot) * 4;
        D.a_ext[icap] = gq[0];
        D.a_cx[icap] = gq[1];
        D.a_cy[icap] = gq[2];
        D.a_cz[icap] = gq[3];
      }
      s_tinc += s_dt;
    } else if (warp == 1) {
      // ---- neighbours of the captured cell lose one liquid neighbour
      const int nn = D.a_nn[icap];
      if (lane < nn) {
        int q = D.a_nbr[(long long)icap * CAFE_NSLOT + lane];
        int left = --D.a_liq[q];
        int r = D.a_frow[q];
        if (r >= 0 && D.row_alive[r]) {
          int sl = cafe_find_slot(D, q, icap);
          if (sl >= 0) D.row_live[r] &= ~(1u << sl);
          if (left <= 0) {
            D.row_alive[r] = 0;
            D.row_death[r] = s_ev;
            D.row_key[r] = CAFE_KEY_NONE;
          }
        }
      }
    }
    __syncthreads();
    // ---- the captured cell becomes a capturing cell if it qualifies
    if (warp < CAFE_QUAD_THREADS / 32) {
      if (D.a_liq[icap] > 0 && D.a_cold[icap] && !s_done) {
        int r = s_nrows;
        if (r < D.row_cap) {
          if (tid == 0) {
            D.row_pos[r] = icap;
            D.row_j[r] = s_nvs2 - 1;
            D.row_alive[r] = 1;
            D.a_frow[icap] = r;
            D.row_death[r] = CAFE_ALIVE;
            D.row_E[r] = D.a_ext[icap];
            D.row_m[r] = CAFE_M_DONE;
          }
          cafe_row_fill_quad(D, K, r, icap, false, s_ev, s_tinc, s_quad);
          if (tid == 0) s_nrows = r + 1;
        } else if (tid == 0) {
          atomicOr(D.err, CAFE_ERR_ROW_CAP);
          s_done = 1;
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    D.ctr[CTR_NGRAIN] = s_ngrain;
    D.ctr[CTR_NVS2_END] = s_nvs2;
    D.ctr[CTR_NROWS_END] = s_nrows;
    D.ctr[CTR_NEV] = s_ev;
    D.ctr[CTR_NNUC] = (int)s_nnuc;
    atomicAdd(&D.stat[STAT_EVENTS], (unsigned long long)s_ev);
    atomicAdd(&D.stat[STAT_NUC], (unsigned long long)s_nnuc);
    atomicAdd(&D.stat[STAT_NEGDT], (unsigned long long)s_negdt);
    atomicMax(&D.stat[STAT_MAXNA], (unsigned long long)s_na);
    atomicMax(&D.stat[STAT_MAXROWS], (unsigned long long)s_nrows);
    atomicAdd(&D.stat[STAT_STEPS], 1ULL);
    atomicAdd(&D.stat[STAT_SUMNA], (unsigned long long)s_na);
    atomicAdd(&D.stat[STAT_SUMROWS], (unsigned long long)s_nrows);
    atomicAdd(&D.stat[STAT_EVALS], (unsigned long long)s_sel.evals);
    if (s_slow) atomicAdd(&D.stat[STAT_SLOWSTEPS], 1ULL);
    for (int c = 0; c < 4; ++c) atomicAdd(&D.stat[STAT_CYC_SELECT + c], (unsigned long long)s_cyc[c]);
#ifdef CAFE_DETAIL_CYCLES
    for (int c = 0; c < 16; ++c)
      if (c != 9 && c != 13 && c != 14) atomicAdd(&D.stat[STAT_DETAIL + c], (unsigned long long)s_dcyc[c]);
    atomicAdd(&D.stat[STAT_DETAIL + 9], *(volatile unsigned long long *)&crm_fallback_calls - s_fb0);
    atomicAdd(&D.stat[STAT_DETAIL + 13], *(volatile unsigned long long *)&crm_special_calls - s_sp0);
    for (int c = 0; c < 4; ++c) atomicAdd(&D.stat[STAT_DETAIL + 4 + c], (unsigned long long)s_sel.cyc[c]);
    atomicAdd(&D.stat[STAT_DETAIL + 8], (unsigned long long)s_sel.rounds);
#endif
  }
#undef CAFE_DCYC
}
__global__ void __launch_bounds__(CAFE_LOOP_THREADS, 1)
    k_event_loop(CafeDev D, CafeConsts K, const CafeStepParams *__restrict__ Pp, long long max_events, int allow_fast) {
  d_event_loop(D, K, Pp, max_events, allow_fast, blockIdx.x, gridDim.x);
}

// Brings every row's extent up to the end of the step (the lazily applied
// growth of VoxelsCA.C:511-516), spread over the whole GPU, and copies it back
// to the row cell's active-list position.
__device__ __forceinline__ void d_rows_finalize(const CafeDev &D, const int cafe_bid, const int cafe_nblk) {
  int nrows = D.ctr[CTR_NROWS_END];
  if (nrows > D.row_cap) nrows = (int)D.row_cap;
  int nev = D.ctr[CTR_NEV];
  for (int r = cafe_bid * blockDim.x + threadIdx.x; r < nrows; r += cafe_nblk * blockDim.x) {
    cafe_row_replay(D, r, nev);
    D.a_ext[D.row_pos[r]] = D.row_E[r];
  }
}
__global__ void k_rows_finalize(CafeDev D) {
  d_rows_finalize(D, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ write back
__device__ __forceinline__ void d_writeback(const CafeDev &D, const CafeConsts &K, const int cafe_bid, const int cafe_nblk) {
  int na = D.ctr[CTR_NA];
  if (na > D.act_cap) na = (int)D.act_cap;
  int zlo = 0x7fffffff, zhi = -1;
  for (int p = cafe_bid * blockDim.x + threadIdx.x; p < na; p += cafe_nblk * blockDim.x) {
    long long idx = D.act[p];
    if (D.a_state[p] == 1 || D.a_state[p] == 2) {
      int k = (int)(idx / K.nxy);
      zlo = min(zlo, k);
      zhi = max(zhi, k);
    }
    D.state[idx] = D.a_state[p];
    D.gid[idx] = D.a_gid[p];
    D.ext[idx] = D.a_ext[p];
    D.cx[idx] = D.a_cx[p];
    D.cy[idx] = D.a_cy[p];
    D.cz[idx] = D.a_cz[p];
    D.pos_of[idx] = -1;
    if (D.a_state[p] == 1) {
      int t = atomicAdd(&D.ctr[CTR_NLIQ], 1);
      D.liq[t] = (int32_t)idx;  // t < na <= act_cap = liq capacity
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    zlo = min(zlo, __shfl_down_sync(0xffffffffu, zlo, o));
    zhi = max(zhi, __shfl_down_sync(0xffffffffu, zhi, o));
  }
  if ((threadIdx.x & 31) == 0 && zhi >= 0) {
    atomicMin(&D.ctr[CTR_ZLO], zlo);
    atomicMax(&D.ctr[CTR_ZHI], zhi);
  }
}
__global__ void k_writeback(CafeDev D, CafeConsts K) {
  d_writeback(D, K, blockIdx.x, gridDim.x);
}

// ConvertSolid1(0): mushy cells whose neighbours are all mushy or solid become
// solid with zero extent. Every mushy cell is in this step's active list. In
// place is equivalent to collect-then-apply: 2 -> 3 keeps "neighbour >= 2".
__device__ __forceinline__ void d_mushy2solid(const CafeDev &D, const CafeConsts &K, const int cafe_bid, const int cafe_nblk) {
  int na = D.ctr[CTR_NA];
  if (na > D.act_cap) na = (int)D.act_cap;
  for (int p = cafe_bid * blockDim.x + threadIdx.x; p < na; p += cafe_nblk * blockDim.x) {
    if (D.a_state[p] != 2) continue;
    long long idx = D.act[p];
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    long long nb[26];
    int n = cafe_moore(K, i, j, k, nb);
    bool all = true;
    for (int a = 0; a < n && all; ++a) all = D.state[nb[a]] >= 2;
    if (all) {
      D.state[idx] = 3;
      D.ext[idx] = 0.0;
    }
  }
}
__global__ void k_mushy2solid(CafeDev D, CafeConsts K) {
  d_mushy2solid(D, K, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ grains
__global__ void k_rot_range(CafeDev D, int g0, int g1) {
  for (int g = g0 + blockIdx.x * blockDim.x + threadIdx.x; g < g1; g += gridDim.x * blockDim.x)
    cafe_rot_from_cth(D.cth + 4LL * g, D.rot + 9LL * g);
}

// CleanLayer (VoxelsCA.C:800-839): grain volumes, renumbering, compaction.
__global__ void k_grain_count(CafeDev D, CafeConsts K, int32_t *cnt) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x) {
    int g = D.gid[idx];
    if (g > 0) atomicAdd(&cnt[g - 1], 1);
  }
}
// Single block: newid[g] (1-based, 0 = dropped) and compacted grain tables.
__global__ void k_grain_renumber(CafeDev D, const int32_t *cnt, int32_t *newid, double *cth2,
                                 double *rot2) {
  __shared__ int part[1024];
  int ng = D.ctr[CTR_NGRAIN];
  int per = (ng + blockDim.x - 1) / blockDim.x;
  int b0 = threadIdx.x * per, b1 = min(b0 + per, ng);
  int s = 0;
  for (int g = b0; g < b1; ++g) s += cnt[g] > 0;
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      int v = part[t];
      part[t] = acc;
      acc += v;
    }
    D.ctr[CTR_NVS2_END] = acc;  // scratch: new grain count
  }
  __syncthreads();
  int k = part[threadIdx.x];
  for (int g = b0; g < b1; ++g) {
    if (cnt[g] > 0) {
      newid[g] = k + 1;
      for (int a = 0; a < 4; ++a) cth2[4LL * k + a] = D.cth[4LL * g + a];
      for (int a = 0; a < 9; ++a) rot2[9LL * k + a] = D.rot[9LL * g + a];
      ++k;
    } else {
      newid[g] = 0;
    }
  }
}
__global__ void k_gid_remap(CafeDev D, CafeConsts K, const int32_t *newid) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x) {
    int g = D.gid[idx];
    if (g != 0) D.gid[idx] = newid[g - 1];
  }
}

// ------------------------------------------------------------------ Voronoi
// Nearest site with the reference's distance (dx^2 + dy^2) + dz^2 and its
// first-minimum rule (BasePlate.C:269-272, VoxelsCA.C:925-930). Sites are
// bucketed on a uniform grid; rings of buckets are searched until no unvisited
// bucket can hold a site whose rounded distance could reach the best found.
struct CafeSiteGrid {
  const double *xyz;      // 3 per site
  const int32_t *start;   // bucket CSR
  const int32_t *idx;     // site indices, ascending inside a bucket
  double lo[3], h;
  int nb[3];
};

__device__ int cafe_nearest_site(const CafeSiteGrid &G, double q0, double q1, double q2) {
  double q[3] = {q0, q1, q2};
  int qb[3];
  for (int a = 0; a < 3; ++a) {
    double f = floor((q[a] - G.lo[a]) / G.h);
    int b = f < 0 ? 0 : (f > G.nb[a] - 1 ? G.nb[a] - 1 : (int)f);
    qb[a] = b;
  }
  double best = INFINITY;
  int besti = -1;
  int rmax = max(G.nb[0], max(G.nb[1], G.nb[2]));
  for (int r = 0; r <= rmax; ++r) {
    for (int dz = -r; dz <= r; ++dz) {
      int bz = qb[2] + dz;
      if (bz < 0 || bz >= G.nb[2]) continue;
      for (int dy = -r; dy <= r; ++dy) {
        int by = qb[1] + dy;
        if (by < 0 || by >= G.nb[1]) continue;
        bool edge = (abs(dz) == r || abs(dy) == r);
        for (int dxx = -r; dxx <= r; dxx += (edge ? 1 : (2 * r > 0 ? 2 * r : 1))) {
          int bx = qb[0] + dxx;
          if (bx < 0 || bx >= G.nb[0]) continue;
          int b = (bz * G.nb[1] + by) * G.nb[0] + bx;
          for (int t = G.start[b]; t < G.start[b + 1]; ++t) {
            int i = G.idx[t];
            double a = q0 - G.xyz[3LL * i], bb = q1 - G.xyz[3LL * i + 1], c = q2 - G.xyz[3LL * i + 2];
            double d = a * a + bb * bb + c * c;
            if (d < best || (d == best && i < besti)) {
              best = d;
              besti = i;
            }
          }
          if (r == 0) break;
        }
      }
    }
    // lower bound on the distance to any bucket outside rings 0..r
    double gap = INFINITY;
    bool more = false;
    for (int a = 0; a < 3; ++a) {
      if (qb[a] - r - 1 >= 0) {
        more = true;
        double g = q[a] - (G.lo[a] + (qb[a] - r) * G.h);
        gap = g < gap ? g : gap;
      }
      if (qb[a] + r + 1 < G.nb[a]) {
        more = true;
        double g = (G.lo[a] + (qb[a] + r + 1) * G.h) - q[a];
        gap = g < gap ? g : gap;
      }
    }
    if (!more) break;
    gap -= 1e-9 * G.h;
    if (besti >= 0 && gap > 0 && gap * gap > best * (1.0 + 1e-9)) break;
  }
  return besti;
}

// Baseplate (BasePlate.C:262-273 + VoxelsCA.C:133-141, 148-156): cell centres,
// cells below z = Nzh-1 solid, the top baseplate plane mushy.
__global__ void k_baseplate(CafeDev D, CafeConsts K, CafeSiteGrid G, int Nzh) {
  long long nbp = (long long)Nzh * K.nxy;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nbp;
       idx += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    double x = (i + .5) * K.dx[0], y = (j + .5) * K.dx[1], z = (k + .5) * K.dx[2];
    int s = cafe_nearest_site(G, x, y, z);
    D.gid[idx] = s + 1;
    D.state[idx] = idx < (long long)(Nzh - 1) * K.nxy ? 3 : 2;
    D.cx[idx] = ((double)i + .5) * K.dx[0];
    D.cy[idx] = ((double)j + .5) * K.dx[1];
    D.cz[idx] = ((double)k + .5) * K.dx[2];
  }
}

// AddLayer1 part 1 (VoxelsCA.C:922-936): nearest site (corner coordinates) for
// every cell of the layer slab [iz1, ilaserLoc) (also beyond the box top, as
// the reference does), and the used-site flags.
__global__ void k_layer_voronoi(CafeConsts K, CafeSiteGrid G, int iz1, int ilaser, int32_t *gtmp,
                                int32_t *used) {
  long long nslab = (long long)K.nxy * (ilaser - iz1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nslab;
       t += (long long)gridDim.x * blockDim.x) {
    int k = iz1 + (int)(t / K.nxy);
    long long r = t % K.nxy;
    int j = (int)(r / K.nx), i = (int)(r % K.nx);
    double x = i * K.dx[0], y = j * K.dx[1], z = k * K.dx[2];
    int s = cafe_nearest_site(G, x, y, z);
    gtmp[t] = s;
    used[s] = 1;
  }
}
// AddLayer1 part 2 (VoxelsCA.C:952-981): new grain IDs, solid state, cell
// centres inside the slab; empty state above the laser plane.
__global__ void k_layer_apply(CafeDev D, CafeConsts K, int iz1, int ilaser, const int32_t *gtmp,
                              const int32_t *map, int ngrain0) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    if (k >= iz1 && k < ilaser) {
      long long t = (long long)(k - iz1) * K.nxy + (long long)j * K.nx + i;
      D.gid[idx] = ngrain0 + map[gtmp[t]] + 1;
      D.state[idx] = 3;
      D.cx[idx] = ((double)i + .5) * K.dx[0];
      D.cy[idx] = ((double)j + .5) * K.dx[1];
      D.cz[idx] = ((double)k + .5) * K.dx[2];
    }
    if (idx >= (long long)K.nxy * ilaser) {
      D.state[idx] = 0;
      D.gid[idx] = 0;
    }
  }
}

// TempField::TempCurr for output (the step computes it on the fly).
__global__ void k_temperature(CafeConsts K, CafeStepParams P, double *T) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cafe_cell_xyz(K, idx, i, j, k);
    T[idx] = K.Tcls[cafe_temp_class_exact(K, P, i, j, k)];
  }
}

// ------------------------------------------------------------------ host transfers
// Layout conversions between the device state and the C ABI's host layout
// (int32 vState/BuildjID, interleaved centres), one staging chunk at a time.
__global__ void k_u8_to_i32(const uint8_t *src, int32_t *dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
// Converts and checks 0 <= v <= vmax; a bad value sets bit `bad_bit` of *bad.
__global__ void k_i32_to_u8_check(const int32_t *src, uint8_t *dst, long long n, int vmax, int *bad, int bad_bit) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int v = src[i];
    if (v < 0 || v > vmax) atomicOr(bad, bad_bit);
    dst[i] = (uint8_t)v;
  }
}
__global__ void k_check_range_i32(const int32_t *a, long long n, int vmax, int *bad, int bad_bit) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int v = a[i];
    if (v < 0 || v > vmax) atomicOr(bad, bad_bit);
  }
}
__global__ void k_interleave3(const double *x, const double *y, const double *z, double *dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    dst[3 * i] = x[i];
    dst[3 * i + 1] = y[i];
    dst[3 * i + 2] = z[i];
  }
}
__global__ void k_deinterleave3(const double *src, double *x, double *y, double *z, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    x[i] = src[3 * i];
    y[i] = src[3 * i + 1];
    z[i] = src[3 * i + 2];
  }
}

// ------------------------------------------------------------------ output
// VoxelsCA::Build. InitializeVoxels marks the baseplate cells that carry a
// grain (VoxelsCA.C:156-159); SetBuild (VoxelsCA.C:76-115) marks every cell of
// every grain that has a melted cell (BuildjID = 1) or a Build cell. The
// reference does this in two passes; the grains of its second pass are those
// of the first plus those of the Build cells, so one flag pass over both
// conditions and one marking pass give the same field.
__global__ void k_build_init(CafeDev D, CafeConsts K) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x)
    D.build[idx] = D.gid[idx] != 0;
}
__global__ void k_build_flag(CafeDev D, CafeConsts K, uint8_t *gflag) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x) {
    int g = D.gid[idx];
    if (g > 0 && (D.buildj[idx] == 1 || D.build[idx] == 1)) gflag[g] = 1;
  }
}
__global__ void k_build_mark(CafeDev D, CafeConsts K, const uint8_t *gflag) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < K.N;
       idx += (long long)gridDim.x * blockDim.x) {
    int g = D.gid[idx];
    if (g > 0 && gflag[g]) D.build[idx] = 1;
  }
}

// One direction of the IPF colouring (VoxelsCA.C:1645-1702 for z, 1703-1760
// for x, 1761-1810 for y) for rotation R. With own_hue false the hue starts
// from H as given (the reference's y direction adds to the x direction's hue),
// and the hue fraction is H/6 as the reference writes it.
__device__ void cafe_ipf_dir(const CafeIpfConsts &C, const double R[3][3], int dir, bool own_hue, double &H,
                             float *rgb) {
  const double v[3] = {dir == 1 ? 1.0 : 0.0, dir == 2 ? 1.0 : 0.0, dir == 0 ? 1.0 : 0.0};
  double a = fabs(R[0][0] * v[0] + R[1][0] * v[1] + R[2][0] * v[2]);
  double b = fabs(R[0][1] * v[0] + R[1][1] * v[1] + R[2][1] * v[2]);
  double c = fabs(R[0][2] * v[0] + R[1][2] * v[1] + R[2][2] * v[2]);
  // std::sort of three (libstdc++'s insertion sort, order of comparisons
  // kept), then the swap of the first two
  if (b < a) { double t = a; a = b; b = t; }
  if (c < a) { double t = c; c = b; b = a; a = t; }
  else if (c < b) { double t = c; c = b; b = t; }
  double v0 = b, v1 = a, v2 = (1.0 < c) ? 1.0 : c;
  double xp = 2. * v0 / (1. + v2);
  double yp = 2. * v1 / (1. + v2);
  if (own_hue) {
    H = crm_atan2((yp - C.y0) / (xp - C.x0), 1.0) * 180. / 3.14159265358979323846;
    if (xp < C.x0) H += 180;
  }
  H = H + 240 - C.hoff;
  const double V = 1.;
  double S = crm_pow_half((xp - C.x0) * (xp - C.x0) + (yp - C.y0) * (yp - C.y0));
  S = S / C.sMax * 0.8 + 0.2;
  if (H >= 360.0) H = 0.0;
  int icase = (int)floor(H / 60.0);
  double ff = H / 6.0 - icase;
  double p = V * (1. - S), q = V * (1. - S * ff), tt = V * (1. - (S * (1. - ff)));
  float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
  if (!(S <= 0.0)) {
    switch (icase) {
      case 0: r0 = (float)V; r1 = (float)tt; r2 = (float)p; break;
      case 1: r0 = (float)q; r1 = (float)V; r2 = (float)p; break;
      case 2: r0 = (float)p; r1 = (float)V; r2 = (float)tt; break;
      case 3: r0 = (float)p; r1 = (float)q; r2 = (float)V; break;
      case 4: r0 = (float)tt; r1 = (float)p; r2 = (float)V; break;
      case 5: r0 = (float)V; r1 = (float)p; r2 = (float)q; break;
      default: break;
    }
  }
  rgb[0] = r0;
  rgb[1] = r1;
  rgb[2] = r2;
}
// IPF colours of grains [0, ngrain): 9 floats per grain (z, x, y directions).
__global__ void k_ipf_grains(const double *cth, int ngrain, CafeIpfConsts C, float *out) {
  for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngrain; gi += gridDim.x * blockDim.x) {
    const double *cc = cth + 4LL * gi;
    double omega = cc[0], ax[3] = {cc[1], cc[2], cc[3]};
    double co = crm_cos(omega), so = crm_sin(omega);
    double R[3][3];
    // VoxelsCA.C:1635-1644, with pow(a, 2.0) = a*a
    R[0][0] = co + (ax[0] * ax[0]) * (1 - co);
    R[0][1] = ax[0] * ax[1] * (1 - co) - ax[2] * so;
    R[0][2] = ax[0] * ax[2] * (1 - co) + ax[1] * so;
    R[1][0] = ax[0] * ax[1] * (1 - co) + ax[2] * so;
    R[1][1] = co + (ax[1] * ax[1]) * (1 - co);
    R[1][2] = ax[1] * ax[2] * (1 - co) - ax[0] * so;
    R[2][0] = ax[2] * ax[0] * (1 - co) - ax[1] * so;
    R[2][1] = ax[2] * ax[1] * (1 - co) + ax[0] * so;
    R[2][2] = co + (ax[2] * ax[2]) * (1 - co);
    double H = 0.0;
    float *o = out + 9LL * gi;
    cafe_ipf_dir(C, R, 0, true, H, o);
    cafe_ipf_dir(C, R, 1, true, H, o + 3);
    cafe_ipf_dir(C, R, 2, false, H, o + 6);
  }
}
// Per-cell colours of direction `d` (0 z, 1 x, 2 y) for cells [off, off+n).
__global__ void k_ipf_cells(CafeDev D, const float *gcol, int d, long long off, long long n, float *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int g = D.gid[off + i];
    float r = 0.0f, gg = 0.0f, b = 0.0f;
    if (g >= 1) {
      const float *c = gcol + 9LL * (g - 1) + 3 * d;
      r = c[0];
      gg = c[1];
      b = c[2];
    }
    out[3 * i] = r;
    out[3 * i + 1] = gg;
    out[3 * i + 2] = b;
  }
}
// TempField::TempCurr as float for cells [off, off+n) (WriteToHDF1's TempOut).
__global__ void k_temperature_f(CafeConsts K, CafeStepParams P, long long off, long long n, float *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int a, b, c;
    cafe_cell_xyz(K, off + i, a, b, c);
    out[i] = (float)K.Tcls[cafe_temp_class_exact(K, P, a, b, c)];
  }
}
// Build as int32 for cells [off, off+n).
__global__ void k_build_i32(CafeDev D, long long off, long long n, int32_t *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = D.build[off + i];
}

// ------------------------------------------------------------------ EASM
// TempField::EASM (TempField.C:79-137): per cell below the laser plane the
// damped fixed point of Utilities::EASM_Temp_LG (Utilities.C:128-140) on
// Utilities::Integral (Utilities.C:105-124) = 300 + sum_i w_i f(x_i), f the
// moving-Gaussian-source kernel Temp_Fun_G (Utilities.C:228-249) with the 316L
// properties at the iterate (Utilities.C:39-76). Expressions keep the
// reference's order; pow(x, 2) is x*x, pow(t - x, -0.5) and exp are the
// correctly rounded functions of cafe_crmath.h.
__device__ __forceinline__ void cafe_easm_materials(double T, double M[4]) {
  double rho, cP, k;
  if (T < 1660)
    rho = 8084.2 - 0.42086 * T - 3.8942 * 1e-5 * T * T;
  else if (T >= 1660 && T < 3090)
    rho = 7432.7 + 3.9338 * 1e-2 * T - 1.8007 * 1e-4 * T * T;
  else
    rho = 6124.72;
  if (T < 1660)
    cP = 458.984 + 0.1328 * T;
  else
    cP = 769.855;
  if (T < 1660)
    k = 9.248 + 1.571 * 1e-2 * T;
  else if (T >= 1660 && T < 3090)
    k = 12.41 + 3.279 * 1e-3 * T;
  else
    k = 21.6465;
  M[0] = cP;
  M[1] = k;
  M[2] = rho;
  M[3] = k / (rho * cP);
}
__device__ __forceinline__ double cafe_easm_integral(const CafeEasm &E, const double *Lx, double R0, double R1,
                                                     double R2, double Ly, double Lz, double T) {
  const double sigma = 50.0e-6, eta = 0.56, pi = 3.14159265358979323846;
  double M[4];
  cafe_easm_materials(T, M);
  double C = eta * E.Q / (pi * M[2] * M[0] * sqrt(4 * pi * M[3]));
  double sig2 = sigma * sigma;
  double dy = R1 - Ly, dz = fabs(R2 - Lz);
  double dy2 = dy * dy, dz2 = dz * dz;
  double s = 0.0;
  for (int i = 0; i < CAFE_EASM_NODES; ++i) {
    double tx = E.tx[i];
    double dx = R0 - Lx[i];
    double a = C * E.r[i] / (2 * M[3] * tx + sig2);
    double arg = -1 * (dx * dx + dy2) / (4 * M[3] * tx + 2 * sig2) - dz2 / (4 * M[3] * tx);
    // exp(arg) is exactly 0 below -745.2, and so is this term
    double f = arg < -745.2 ? a * 0.0 : a * crm_exp(arg);
    s += E.qw[i] * f;
  }
  return 300 + s;
}
__global__ void k_set_int(int *p, int v) { *p = v; }
__global__ void k_easm_reset(CafeDev D) {
  int t = threadIdx.x;
  if (t < 3) D.ctr[CTR_EASM_BOX + t] = 0x7fffffff;
  else if (t < 6) D.ctr[CTR_EASM_BOX + t] = -1;
  else if (t == 6) D.ctr[CTR_EASM_COLD] = 0;
  else if (t == 7) *(unsigned long long *)&D.ctr[CTR_EASM_CURSOR] = 0ULL;
  else if (t == 8) D.ctr[CTR_EASM_QN] = 0;
  else if (t == 9) D.ctr[CTR_EASM_QHEAD] = 0;
}
// Cells [0, ncell) (cells above the laser plane keep T = 0). Writes temp,
// BuildjID, the box of the cells at or above the liquidus and the "some cell
// below the liquidus" flag. Cells need 2 to 100 integrals each, so each
// thread takes the next cell from a shared cursor whenever its own has
// converged: the lanes of a warp then run the same 25-node loop together
// instead of idling behind the slowest cell of a fixed assignment.
__global__ void k_easm(CafeDev D, CafeConsts K, CafeStepParams P, CafeEasm E, long long ncell) {
  __shared__ double s_Lx[CAFE_EASM_NODES];
  __shared__ int s_box[6], s_cold;
  __shared__ unsigned long long s_integrals;
  const double t = 80.0e-5;
  if (threadIdx.x < CAFE_EASM_NODES) {
    double x0 = P.lx - E.bmV * t;  // Utilities.C:243-244
    s_Lx[threadIdx.x] = x0 + E.bmV * E.qx[threadIdx.x];
  }
  if (threadIdx.x < 3) {
    s_box[threadIdx.x] = 0x7fffffff;
    s_box[3 + threadIdx.x] = -1;
  }
  if (threadIdx.x == 0) {
    s_cold = 0;
    s_integrals = 0;
  }
  __syncthreads();
  unsigned long long nint = 0;
  int bx0 = 0x7fffffff, by0 = 0x7fffffff, bz0 = 0x7fffffff, bx1 = -1, by1 = -1, bz1 = -1, cold = 0;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  long long idx = -1;  // this lane's cell, -1 when it needs one
  bool exhausted = false;
  int ci = 0, cj = 0, ck = 0, n = 0, done_here = 0;
  bool first = true;
  double xp = 0, yp = 0, zp = 0, Told = 0, Tnew = 0, Tin = 0;
  // warp-synchronous rounds: lanes without a cell take new ones together (one
  // atomic per warp), then every lane evaluates one integral (lanes without a
  // cell on dummy inputs, discarded), so the warp stays converged
  while (true) {
    bool need = idx < 0 && !exhausted;
    unsigned needm = __ballot_sync(FULL, need);
    if (needm) {
      unsigned long long base = 0;
      int leader = __ffs(needm) - 1;
      if (lane == leader) base = atomicAdd((unsigned long long *)&D.ctr[CTR_EASM_CURSOR], (unsigned long long)__popc(needm));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        long long r = (long long)(base + __popc(needm & ((1u << lane) - 1u)));
        // from the top down: the cells just below the laser plane take the most
        // integrals, and handing them out first keeps the end of the pass from
        // waiting on a few long cells
        long long c = ncell - 1 - r;
        if (r >= ncell) {
          exhausted = true;
        } else {
          cafe_cell_xyz(K, c, ci, cj, ck);
          double x0 = ((double)ci + .5) * K.dx[0];
          double y0 = ((double)cj + .5) * K.dx[1];
          zp = ((double)ck + .5) * K.dx[2];
          if (zp > P.lz) {
            // above the laser plane: T stays 0 (TempField.C:99)
          } else if ((x0 > P.lx) && (zp > (P.lz - E.layerT))) {
            double T = .99 * K.T0;
            D.temp[c] = T;
            if (T > K.tL)
              D.buildj[c] = 1;
            else if (T < K.T0)
              D.buildj[c] = 0;
            if (T >= K.tL) {
              bx0 = min(bx0, ci); by0 = min(by0, cj); bz0 = min(bz0, ck);
              bx1 = max(bx1, ci); by1 = max(by1, cj); bz1 = max(bz1, ck);
            } else {
              cold = 1;
            }
          } else {
            xp = P.cg * (x0 - K.hLX0) + P.sg * (y0 - K.hLX1) + K.hLX0;
            yp = -P.sg * (x0 - K.hLX0) + P.cg * (y0 - K.hLX1) + K.hLX1;
            idx = c;
            first = true;
            Told = 0.0;
            Tin = 0.0;
            n = 0;
            done_here = 0;
          }
        }
      }
    }
    const bool work = idx >= 0;
    if (__all_sync(FULL, !work && exhausted)) break;
    if (!__any_sync(FULL, work)) continue;  // only cells without integrals were taken
    // one integral per lane; then the step of Utilities::EASM_Temp_LG's loop
    double Tres = cafe_easm_integral(E, s_Lx, xp, yp, zp, P.ly, P.lz, Tin);
    if (!work) continue;
    ++nint;
    if (first) {
      Tnew = Tres;
      first = false;
    } else {
      Tnew = 0.5 * (Told + Tres);
      n++;
    }
    if (fabs(Told - Tnew) > 10.0 && n < 100) {
      // a long fixed point goes on in the warp-per-cell pass (when the queue
      // has room), from this point of the loop: test passed, next integral due
      if (++done_here >= CAFE_EASM_LANE_INTEGRALS) {
        int slot = atomicAdd(&D.ctr[CTR_EASM_QN], 1);
        if (slot < D.easm_qcap) {
          CafeEasmItem it;
          it.idx = idx;
          it.Told = Told;
          it.Tnew = Tnew;
          it.n = n;
          it.pad = 0;
          D.easm_q[slot] = it;
          idx = -1;
          continue;
        }
      }
      Told = Tnew;
      Tin = Told;
      continue;
    }
    double T = Tnew;
    D.temp[idx] = T;
    if (T > K.tL)
      D.buildj[idx] = 1;
    else if (T < K.T0)
      D.buildj[idx] = 0;
    if (T >= K.tL) {
      bx0 = min(bx0, ci); by0 = min(by0, cj); bz0 = min(bz0, ck);
      bx1 = max(bx1, ci); by1 = max(by1, cj); bz1 = max(bz1, ck);
    } else {
      cold = 1;
    }
    idx = -1;
  }
  if (bx1 >= 0) {
    atomicMin(&s_box[0], bx0); atomicMin(&s_box[1], by0); atomicMin(&s_box[2], bz0);
    atomicMax(&s_box[3], bx1); atomicMax(&s_box[4], by1); atomicMax(&s_box[5], bz1);
  }
  if (cold) s_cold = 1;
  if (nint) atomicAdd(&s_integrals, nint);
  __syncthreads();
  if (threadIdx.x == 0 && s_integrals) atomicAdd(&D.stat[STAT_EASM_INTEGRALS], s_integrals);
  if (threadIdx.x < 3 && s_box[3 + threadIdx.x] >= 0) {
    atomicMin(&D.ctr[CTR_EASM_BOX + threadIdx.x], s_box[threadIdx.x]);
    atomicMax(&D.ctr[CTR_EASM_BOX + 3 + threadIdx.x], s_box[3 + threadIdx.x]);
  }
  if (threadIdx.x == 0 && s_cold) D.ctr[CTR_EASM_COLD] = 1;
}
// Utilities::Integral for one cell with the 25 nodes spread over the lanes of
// a warp; the weighted terms are added in node order on every lane, as the
// quadrature sum does, so the result is that of cafe_easm_integral.
__device__ __forceinline__ double cafe_easm_integral_warp(const CafeEasm &E, const double *Lx, double R0, double R1,
                                                          double R2, double Ly, double Lz, double T, int lane) {
  const unsigned FULL = 0xffffffffu;
  const double sigma = 50.0e-6, eta = 0.56, pi = 3.14159265358979323846;
  double M[4];
  cafe_easm_materials(T, M);
  double C = eta * E.Q / (pi * M[2] * M[0] * sqrt(4 * pi * M[3]));
  double sig2 = sigma * sigma;
  double dy = R1 - Ly, dz = fabs(R2 - Lz);
  double dy2 = dy * dy, dz2 = dz * dz;
  double p = 0.0;
  if (lane < CAFE_EASM_NODES) {
    int i = lane;
    double tx = E.tx[i];
    double dx = R0 - Lx[i];
    double a = C * E.r[i] / (2 * M[3] * tx + sig2);
    double arg = -1 * (dx * dx + dy2) / (4 * M[3] * tx + 2 * sig2) - dz2 / (4 * M[3] * tx);
    double f = arg < -745.2 ? a * 0.0 : a * crm_exp(arg);
    p = E.qw[i] * f;
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < CAFE_EASM_NODES; ++i) s += __shfl_sync(FULL, p, i);
  return 300 + s;
}

// The cells queued by k_easm: one warp per cell until its fixed point ends.
__global__ void k_easm_long(CafeDev D, CafeConsts K, CafeStepParams P, CafeEasm E) {
  __shared__ double s_Lx[CAFE_EASM_NODES];
  __shared__ int s_box[6], s_cold;
  __shared__ unsigned long long s_integrals;
  const double t = 80.0e-5;
  if (threadIdx.x < CAFE_EASM_NODES) {
    double x0 = P.lx - E.bmV * t;
    s_Lx[threadIdx.x] = x0 + E.bmV * E.qx[threadIdx.x];
  }
  if (threadIdx.x < 3) {
    s_box[threadIdx.x] = 0x7fffffff;
    s_box[3 + threadIdx.x] = -1;
  }
  if (threadIdx.x == 0) {
    s_cold = 0;
    s_integrals = 0;
  }
  __syncthreads();
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int nq = D.ctr[CTR_EASM_QN];
  if (nq > D.easm_qcap) nq = (int)D.easm_qcap;
  unsigned long long nint = 0;
  int bx0 = 0x7fffffff, by0 = 0x7fffffff, bz0 = 0x7fffffff, bx1 = -1, by1 = -1, bz1 = -1, cold = 0;
  while (true) {
    int q = 0;
    if (lane == 0) q = atomicAdd(&D.ctr[CTR_EASM_QHEAD], 1);
    q = __shfl_sync(FULL, q, 0);
    if (q >= nq) break;
    CafeEasmItem it = D.easm_q[q];
    int ci, cj, ck;
    cafe_cell_xyz(K, it.idx, ci, cj, ck);
    double x0 = ((double)ci + .5) * K.dx[0];
    double y0 = ((double)cj + .5) * K.dx[1];
    double zp = ((double)ck + .5) * K.dx[2];
    double xp = P.cg * (x0 - K.hLX0) + P.sg * (y0 - K.hLX1) + K.hLX0;
    double yp = -P.sg * (x0 - K.hLX0) + P.cg * (y0 - K.hLX1) + K.hLX1;
    double Told = it.Told, Tnew = it.Tnew;
    int n = it.n;
    // continue Utilities::EASM_Temp_LG's loop where the lane pass left it
    while (fabs(Told - Tnew) > 10.0 && n < 100) {
      Told = Tnew;
      double Tt = cafe_easm_integral_warp(E, s_Lx, xp, yp, zp, P.ly, P.lz, Told, lane);
      Tnew = 0.5 * (Told + Tt);
      n++;
      ++nint;
    }
    if (lane == 0) {
      double T = Tnew;
      D.temp[it.idx] = T;
      if (T > K.tL)
        D.buildj[it.idx] = 1;
      else if (T < K.T0)
        D.buildj[it.idx] = 0;
      if (T >= K.tL) {
        bx0 = min(bx0, ci); by0 = min(by0, cj); bz0 = min(bz0, ck);
        bx1 = max(bx1, ci); by1 = max(by1, cj); bz1 = max(bz1, ck);
      } else {
        cold = 1;
      }
    }
  }
  if (bx1 >= 0) {
    atomicMin(&s_box[0], bx0); atomicMin(&s_box[1], by0); atomicMin(&s_box[2], bz0);
    atomicMax(&s_box[3], bx1); atomicMax(&s_box[4], by1); atomicMax(&s_box[5], bz1);
  }
  if (cold) s_cold = 1;
  if (lane == 0 && nint) atomicAdd(&s_integrals, nint);
  __syncthreads();
  if (threadIdx.x == 0 && s_integrals) atomicAdd(&D.stat[STAT_EASM_INTEGRALS], s_integrals);
  if (threadIdx.x < 3 && s_box[3 + threadIdx.x] >= 0) {
    atomicMin(&D.ctr[CTR_EASM_BOX + threadIdx.x], s_box[threadIdx.x]);
    atomicMax(&D.ctr[CTR_EASM_BOX + 3 + threadIdx.x], s_box[3 + threadIdx.x]);
  }
  if (threadIdx.x == 0 && s_cold) D.ctr[CTR_EASM_COLD] = 1;
}

// SetLiquid3 (VoxelsCA.C:1098-1116) and the class map over the box of the
// cells at or above the liquidus, from the EASM temperatures.
// The Rosenthal field (extension) over cells [0, ncell): temp, BuildjID as
// AnalyticTempCurr sets it (TempField.C:180-185), the box of the cells at or
// above the liquidus and the "some cell below the liquidus" flag, in the slots
// the EASM field uses.
__global__ void k_rosenthal(CafeDev D, CafeConsts K, CafeStepParams P, long long ncell) {
  __shared__ int s_box[6], s_cold;
  if (threadIdx.x < 3) {
    s_box[threadIdx.x] = 0x7fffffff;
    s_box[3 + threadIdx.x] = -1;
  }
  if (threadIdx.x == 0) s_cold = 0;
  __syncthreads();
  int bx0 = 0x7fffffff, by0 = 0x7fffffff, bz0 = 0x7fffffff, bx1 = -1, by1 = -1, bz1 = -1, cold = 0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    int ci, cj, ck;
    cafe_cell_xyz(K, c, ci, cj, ck);
    double T = cafe_rosenthal_T(K, P, ci, cj, ck);
    D.temp[c] = T;
    if (T > K.tL)
      D.buildj[c] = 1;
    else if (T < K.T0)
      D.buildj[c] = 0;
    if (T >= K.tL) {
      bx0 = min(bx0, ci); by0 = min(by0, cj); bz0 = min(bz0, ck);
      bx1 = max(bx1, ci); by1 = max(by1, cj); bz1 = max(bz1, ck);
    } else {
      cold = 1;
    }
  }
  if (bx1 >= 0) {
    atomicMin(&s_box[0], bx0); atomicMin(&s_box[1], by0); atomicMin(&s_box[2], bz0);
    atomicMax(&s_box[3], bx1); atomicMax(&s_box[4], by1); atomicMax(&s_box[5], bz1);
  }
  if (cold) s_cold = 1;
  __syncthreads();
  if (threadIdx.x < 3 && s_box[3 + threadIdx.x] >= 0) {
    atomicMin(&D.ctr[CTR_EASM_BOX + threadIdx.x], s_box[threadIdx.x]);
    atomicMax(&D.ctr[CTR_EASM_BOX + 3 + threadIdx.x], s_box[3 + threadIdx.x]);
  }
  if (threadIdx.x == 0 && s_cold) D.ctr[CTR_EASM_COLD] = 1;
}
__global__ void k_fill_f64(double *p, long long n, double v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}
__global__ void k_melt_easm(CafeDev D, CafeConsts K, CafeStepParams P) {
  int bx = P.hi[0] - P.lo[0], by = P.hi[1] - P.lo[1], bz = P.hi[2] - P.lo[2];
  long long nbox = (long long)bx * by * bz;
  long long iz1 = (long long)P.ilaserLoc * K.nxy;
  int any = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nbox;
       t += (long long)gridDim.x * blockDim.x) {
    int i = P.lo[0] + (int)(t % bx);
    long long r = t / bx;
    int j = P.lo[1] + (int)(r % by);
    int k = P.lo[2] + (int)(r / by);
    long long idx = (long long)K.nxy * k + (long long)K.nx * j + i;
    double zp = ((double)k + .5) * K.dx[2];
    double T = D.temp[idx];
    int c = zp > P.lz ? 0 : (T >= K.tL ? 2 : 1);
    D.tcls[t] = (uint8_t)c;
    if (c == 2) {
      any = 1;
      if (idx < K.nxy) {
        D.state[idx] = 2;
      } else if (idx < iz1) {
        D.state[idx] = 1;
        D.gid[idx] = 0;
      }
      D.ext[idx] = 0.0;
    }
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(&D.ctr[CTR_HOT], 1);
}
// Temperatures of cells [off, off+n) as float (output) from the EASM field.
__global__ void k_temp_copy_f(const double *T, long long off, long long n, float *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)T[off + i];
}

// Sets bit `bit` of *bad if some v[i] > maxv.
__global__ void k_check_range_u8(const uint8_t *v, long long n, int maxv, int *bad, int bit) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    if (v[i] > maxv) atomicOr(bad, bit);
}

// ------------------------------------------------------------------ growth log
// Before k_rows_finalize: every frontier row of the step (those present at
// the start and those created by captures) gets a log entry holding its cell
// and its extent before the step's growth (a_ext still holds it: the start
// value, or the value set at capture). tau temporarily holds that extent.
__global__ void k_glog_begin(CafeDev D, const CafeStepParams *__restrict__ Pp) {
  int nrows = D.ctr[CTR_NROWS_END];
  if (nrows > D.row_cap) nrows = (int)D.row_cap;
  long long base = D.ctr[CTR_GLOG_N];
  if (base + nrows > D.glog_cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) D.ctr[CTR_GLOG_OVER] = 1;
    return;
  }
  const int tind = Pp->tInd;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    int p = D.row_pos[r];
    D.glog_cell[base + r] = (int32_t)D.act[p];
    D.glog_step[base + r] = tind;
    D.glog_tau[base + r] = D.a_ext[p];
  }
}
// After k_rows_finalize: growth time = (final extent - extent before) / v
// (0 for a row that does not grow).
__global__ void k_glog_end(CafeDev D, CafeConsts K) {
  int nrows = D.ctr[CTR_NROWS_END];
  if (nrows > D.row_cap) nrows = (int)D.row_cap;
  long long base = D.ctr[CTR_GLOG_N];
  if (base + nrows > D.glog_cap) return;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    int p = D.row_pos[r];
    double v = cafe_vh(D, K, p);
    double e0 = D.glog_tau[base + r];
    D.glog_tau[base + r] = v > 0.0 ? (D.a_ext[p] - e0) / v : 0.0;
  }
}
__global__ void k_glog_advance(CafeDev D) {
  int nrows = D.ctr[CTR_NROWS_END];
  if (nrows > D.row_cap) nrows = (int)D.row_cap;
  long long base = D.ctr[CTR_GLOG_N];
  if (base + nrows <= D.glog_cap) D.ctr[CTR_GLOG_N] = (int)(base + nrows);
}
