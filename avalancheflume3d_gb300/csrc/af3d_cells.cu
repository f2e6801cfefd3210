// af3d_cells.cu -- the sorted cell list: counting sort of clumps by (cell, id).
//
// Replaces the fixed-capacity slot table of cells.cu (clear_cell / clear_ocup / cell_locate).
// The predictor kernel has already written every clump's bucket key and its atomic arrival rank
// inside the bucket, and counted it in its bucket's scan tile.  Here:
//   1. exclusive scan of the bucket counts  -> start[b]      (one pass: each tile starts from the
//                                                            tile counts before it)
//   2. scatter old slots by arrival          -> tmp_slot
//   3. rank every clump inside its bucket by clump id (buckets hold a handful of clumps), which
//      makes the final order deterministic and equal to the reference's ascending-id insertion
//      order (cells.cu:60-109)                 -> perm[new slot] = old slot
// Integer work only; HBM-bound.
#include "af3d_internal.h"

namespace af3d {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;   // consecutive buckets per thread, moved as four int4
constexpr int kTile = kScanThreads * kScanItems;
static_assert(kTile == kScanTile, "the producers count clumps per kScanTile buckets");

// The kScanItems counts of one thread starting at bucket `base` (a multiple of kScanItems, so
// the vector loads are 16-byte aligned); buckets at or past nb read as zero.
__device__ __forceinline__ void load_counts(const int *__restrict__ count, long base, long nb, int *v) {
  if (base + kScanItems <= nb) {
    const int4 *q = reinterpret_cast<const int4 *>(count + base);
#pragma unroll
    for (int i = 0; i < kScanItems / 4; i++) {
      const int4 x = q[i];
      v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; i++) v[i] = base + i < nb ? count[base + i] : 0;
  }
}

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int u = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v += u;
  }
  return v;
}

// Exclusive scan of one value per thread across the block; returns the block total in *total.
__device__ __forceinline__ int block_excl_scan(int v, int *total) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = warp_incl_scan(v);
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
    int ti = warp_incl_scan(t);
    if (lane < kScanThreads / 32) warp_tot[lane] = ti - t;
    if (lane == kScanThreads / 32 - 1) *total = ti;
  }
  __syncthreads();
  int r = incl - v + warp_tot[wid];
  __syncthreads();
  return r;
}

// Buckets in use: every flume's cells plus one private bucket per clump for the clumps not binned.
__device__ __forceinline__ long n_buckets(const DevScalars *d, long n) { return d->ncell_total + n; }

// Each tile adds the clump counts of the tiles before it (counted at arrival; integer sums are
// exact in any order), then scans its own buckets.
// advance: block 0 also performs k_advance_time's time += dt (steps whose predictor ran in the
// previous force pass start with the sort; nothing before the force pass reads the clock).
__global__ void k_scan_final(const int *__restrict__ count, const int *__restrict__ tile_count,
                             int *start, DevScalars *d, bool advance, long n) {
  if (advance && blockIdx.x == 0 && threadIdx.x == 0) {
    d->time_prev = d->time;
    d->time = d->time + d->flumes[0].sys.dt;
  }
  const long nb = n_buckets(d, n);
  if (blockIdx.x == 0 && threadIdx.x == 0) start[nb] = (int)n;   // every clump has one bucket
  if (blockIdx.x * (long)kTile >= nb) return;   // a tile past the buckets in use
  int part = 0;
  for (long t = threadIdx.x; t < (long)blockIdx.x; t += kScanThreads) part += tile_count[t];
  __shared__ int tile_off;
  block_excl_scan(part, &tile_off);
  const long base = blockIdx.x * (long)kTile + threadIdx.x * (long)kScanItems;
  int v[kScanItems];
  load_counts(count, base, nb, v);
  int sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) sum += v[i];
  __shared__ int tot;
  int e = block_excl_scan(sum, &tot) + tile_off;
  int o[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    o[i] = e;
    e += v[i];
  }
  if (base + kScanItems <= nb) {
    int4 *q = reinterpret_cast<int4 *>(start + base);
#pragma unroll
    for (int i = 0; i < kScanItems / 4; i++) q[i] = make_int4(o[4 * i], o[4 * i + 1], o[4 * i + 2], o[4 * i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
      if (base + i < nb) start[base + i] = o[i];
  }
}

__global__ void k_scatter(const int *__restrict__ key, const int *__restrict__ rank_tmp,
                          const int *__restrict__ start, int *tmp_slot, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  tmp_slot[start[key[s]] + rank_tmp[s]] = (int)s;
}

// Also returns the bucket count and its tile's count to zero, so both arrays are all-zero at the
// next build whatever the grid then is (the scan has consumed them already).
__global__ void k_rank(const int *__restrict__ key, const int *__restrict__ start,
                       const int *__restrict__ tmp_slot, const long long *__restrict__ id, int *perm,
                       const CullRec *__restrict__ cull, float4 *csort, int *count, int *tile_count,
                       DevScalars *d, long ntags, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const long ncell3 = d->ncell_total;
  const int k = key[s];
  count[k] = 0;
  tile_count[k / kTile] = 0;
  const int b = start[k], e = start[k + 1];
  const long long me = id[s];
  int r = 0;
  for (int j = b; j < e; j++) r += id[tmp_slot[j]] < me;
  perm[b + r] = (int)s;
  if (cull) csort[b + r] = cull[s].c;
  // cells.cu:96-102: a cell may hold at most ntags - 1 clumps
  if (ntags > 0 && k < ncell3 && r == 0 && (e - b) >= ntags)
    atomicOr(&d->status, 1 << AF3D_ERR_CELL_CAPACITY);
}

}  // namespace

long scan_tiles(long bucket_cap) { return (bucket_cap + kTile - 1) / kTile; }

void launch_sort(const Launch &L, DevScalars *d, Cells c, const long long *id, long ntags, const CullRec *cull,
                 bool advance) {
  // Launch sizes follow the capacity; the kernels read the bucket count in use from the device,
  // so a captured graph stays valid across device-side re-grids.
  const long ntiles = scan_tiles(c.cap);
  k_scan_final<<<(unsigned)ntiles, kScanThreads, 0, L.st>>>(c.count, c.tile_count, c.start, d, advance, L.n);
  if (L.n <= 0) return;
  const unsigned g = (unsigned)((L.n + 127) / 128);
  k_scatter<<<g, 128, 0, L.st>>>(c.key, c.rank_tmp, c.start, c.tmp_slot, L.n);
  k_rank<<<g, 128, 0, L.st>>>(c.key, c.start, c.tmp_slot, id, c.perm, cull, c.csort, c.count, c.tile_count, d,
                              ntags, L.n);
}

}  // namespace af3d
