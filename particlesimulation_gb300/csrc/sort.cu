// sort.cu - particle ordering for the PM / P3M path.
//
// Two orders are produced on the device:
//   * P3M: the reference's chaining-mesh cell lists (source/chainingMesh.cpp:20-58).  Cell =
//     int(x/HC) per axis, flat x + y*Mx + z*Mx*My; within a cell ascending y with ties by
//     ascending particle index (fillWithYSorting), or descending index (fill).  Particles are
//     sorted by a 64-bit key (cell << 32 | order key) with a stable LSD radix sort, and runs of
//     equal keys are put in index order afterwards, so the result is bit-identical to the
//     reference's lists.
//   * PM: Morton order of 4x4x4-cell bricks, for deposit / interpolation locality only (the
//     density is computed in integer arithmetic, so results do not depend on the order).
//
// The radix sort is our own: per pass a block histogram, a scan of each digit's row of block
// counts (one CTA per digit), and a stable scatter that ranks keys inside a warp with
// __match_any_sync.
#include "common.cuh"

namespace pmgb {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_STRIPS = 16;                          // 32-key strips per warp
static_assert(RS_WARPS * RS_STRIPS * 32 == RS_TILE, "RS_TILE (common.cuh) is the keys per block");

__device__ __forceinline__ u32 lanemask_lt() {
  u32 m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void __launch_bounds__(RS_THREADS) rs_hist_kernel(const u64* __restrict__ keys, int n,
                                                             int shift, u32 mask,
                                                             u32* __restrict__ hist, int nblocks) {
  __shared__ u32 h[256];
  for (int d = threadIdx.x; d < 256; d += RS_THREADS) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
  const int lane = threadIdx.x & 31;
  for (int off = 0; off < RS_TILE; off += RS_THREADS) {
    int i = base + off + threadIdx.x;
    bool valid = i < n;
    u32 d = valid ? (u32)((keys[i] >> shift) & mask) : 0xFFFFFFFFu;
    u32 peers = __match_any_sync(0xFFFFFFFFu, d);
    if (valid && (__ffs(peers) - 1) == lane) atomicAdd(&h[d], (u32)__popc(peers));
  }
  __syncthreads();
  for (int d = threadIdx.x; d <= (int)mask; d += RS_THREADS) hist[d * nblocks + blockIdx.x] = h[d];
}

// ------------------------------------------------------------------ scans --------------
// Exclusive scans of u32 arrays.  One 256-thread CTA scans a tile of SCAN_TILE = 4096 values:
// each warp owns 512 consecutive values, reads them in 16 coalesced rounds of 32 and scans each
// round with shuffles, starting from the sum of the warps before it.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_WARPS = SCAN_THREADS / 32;
constexpr int SCAN_ROUNDS = 16;
constexpr int SCAN_TILE = SCAN_WARPS * SCAN_ROUNDS * 32;

__device__ __forceinline__ u32 warp_incl_scan(u32 v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// out[i] = carry + in[0] + ... + in[i-1] for i < len (len <= SCAN_TILE; in == out allowed: every
// value is read before the CTA's first write).  Returns the sum of in[0, len) to every thread.
// ws: SCAN_WARPS words of shared memory.  Called by all threads of the CTA.
__device__ u32 tile_scan(const u32* in, u32* out, int len, u32 carry, u32* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wb = warp * (SCAN_ROUNDS * 32);
  u32 v[SCAN_ROUNDS];
  u32 s = 0;
#pragma unroll
  for (int r = 0; r < SCAN_ROUNDS; ++r) {
    const int i = wb + r * 32 + lane;
    v[r] = i < len ? in[i] : 0u;
    s += v[r];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if (lane == 0) ws[warp] = s;
  __syncthreads();
  u32 base = carry, tot = 0;
#pragma unroll
  for (int w = 0; w < SCAN_WARPS; ++w) {
    const u32 t = ws[w];
    base += w < warp ? t : 0u;
    tot += t;
  }
  __syncthreads();  // ws may be reused by the caller's next tile
#pragma unroll
  for (int r = 0; r < SCAN_ROUNDS; ++r) {
    const u32 x = warp_incl_scan(v[r], lane);
    const int i = wb + r * 32 + lane;
    if (i < len) out[i] = base + x - v[r];
    base += __shfl_sync(0xFFFFFFFFu, x, 31);
  }
  return tot;
}

// One CTA scans all of in[0, n), tile after tile; total (if given) = the sum.
__global__ void __launch_bounds__(SCAN_THREADS) scan_serial_kernel(const u32* in, u32* out, int n,
                                                                   u32* total) {
  __shared__ u32 ws[SCAN_WARPS];
  u32 carry = 0;
  for (int b = 0; b < n; b += SCAN_TILE) carry += tile_scan(in + b, out + b, min(SCAN_TILE, n - b), carry, ws);
  if (total && threadIdx.x == 0) *total = carry;
}

// partial[t] = sum of tile t.
__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_sums_kernel(const u32* __restrict__ in, int n,
                                                                      u32* __restrict__ partial) {
  __shared__ u32 ws[SCAN_WARPS];
  const int base = blockIdx.x * SCAN_TILE, len = min(SCAN_TILE, n - base);
  u32 s = 0;
  for (int i = threadIdx.x; i < len; i += SCAN_THREADS) s += in[base + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    u32 t = 0;
    for (int w = 0; w < SCAN_WARPS; ++w) t += ws[w];
    partial[blockIdx.x] = t;
  }
}

// Tile t scanned from the exclusive prefix partial[t] of the tile sums.
__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles_kernel(const u32* in, u32* out, int n,
                                                                  const u32* __restrict__ partial) {
  __shared__ u32 ws[SCAN_WARPS];
  const int base = blockIdx.x * SCAN_TILE;
  tile_scan(in + base, out + base, min(SCAN_TILE, n - base), partial[blockIdx.x], ws);
}

// Radix histogram rows: CTA d scans row d (hist[d * nb + b] over the nb blocks) in place and
// stores the row's total in rowtot[d].
__global__ void __launch_bounds__(SCAN_THREADS) rs_rowscan_kernel(u32* hist, int nb, u32* __restrict__ rowtot) {
  __shared__ u32 ws[SCAN_WARPS];
  u32* row = hist + (size_t)blockIdx.x * nb;
  u32 carry = 0;
  for (int b = 0; b < nb; b += SCAN_TILE) carry += tile_scan(row + b, row + b, min(SCAN_TILE, nb - b), carry, ws);
  if (threadIdx.x == 0) rowtot[blockIdx.x] = carry;
}

// hist: each digit row scanned by rs_rowscan_kernel, row totals in rowtot.  A block's first
// slot for digit d = (sum of the row totals of digits below d) + hist[d * nblocks + block].
__global__ void __launch_bounds__(RS_THREADS) rs_scatter_kernel(
    const u64* __restrict__ kin, const u32* __restrict__ vin, u64* __restrict__ kout,
    u32* __restrict__ vout, int n, int shift, u32 mask, const u32* __restrict__ hist,
    const u32* __restrict__ rowtot, int nblocks) {
  static_assert(RS_THREADS == 256, "one thread per digit");
  __shared__ u32 wh[RS_WARPS][256];
  __shared__ u32 gb[256];
  __shared__ u32 wsum[RS_WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&wh[0][0])[i] = 0;
  {
    const int d = threadIdx.x;
    const u32 t = d <= (int)mask ? rowtot[d] : 0u;
    const u32 x = warp_incl_scan(t, lane);
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    u32 base = x - t;
    for (int w = 0; w < warp; ++w) base += wsum[w];
    if (d <= (int)mask) gb[d] = base + hist[(size_t)d * nblocks + blockIdx.x];
  }
  __syncthreads();
  u64 k[RS_STRIPS];
  u32 v[RS_STRIPS], r[RS_STRIPS];
  const int wbase = blockIdx.x * RS_TILE + warp * (RS_STRIPS * 32);
  const u32 lt = lanemask_lt();
#pragma unroll
  for (int s = 0; s < RS_STRIPS; ++s) {
    int i = wbase + s * 32 + lane;
    bool valid = i < n;
    k[s] = valid ? kin[i] : 0ull;
    v[s] = valid ? vin[i] : 0u;
    u32 d = valid ? (u32)((k[s] >> shift) & mask) : 0xFFFFFFFFu;
    u32 peers = __match_any_sync(0xFFFFFFFFu, d);
    u32 rank = __popc(peers & lt);
    u32 pre = valid ? wh[warp][d] : 0u;
    __syncwarp();
    if (valid && rank == 0) wh[warp][d] = pre + __popc(peers);
    __syncwarp();
    r[s] = pre + rank;
  }
  __syncthreads();
  for (int d = threadIdx.x; d <= (int)mask; d += RS_THREADS) {
    u32 run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      u32 t = wh[w][d];
      wh[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int s = 0; s < RS_STRIPS; ++s) {
    int i = wbase + s * 32 + lane;
    if (i < n) {
      u32 d = (u32)((k[s] >> shift) & mask);
      u32 dest = gb[d] + wh[warp][d] + r[s];
      kout[dest] = k[s];
      vout[dest] = v[s];
    }
  }
}

int radix_hist_blocks(int n) { return (n + RS_TILE - 1) / RS_TILE; }
size_t radix_hist_words(int n) { return (size_t)256 * radix_hist_blocks(n) + 256; }

// Sorts (keys, vals) by key bits [0, nbits).  Ping-pongs with the alternates; on return
// *keys / *vals point at the sorted data (the pointers may have been swapped).  hist holds
// radix_hist_words(n) words: the 256 x blocks digit counts, then the 256 row totals.
int radix_sort_pairs(u64** keys, u32** vals, u64** keys_alt, u32** vals_alt, u32* hist, int n,
                     int nbits, cudaStream_t st) {
  if (n <= 0) return PMGB_OK;
  const int nb = radix_hist_blocks(n);
  u32* rowtot = hist + (size_t)256 * nb;
  for (int shift = 0; shift < nbits; shift += 8) {
    int bits = nbits - shift < 8 ? nbits - shift : 8;
    u32 mask = (1u << bits) - 1u;
    rs_hist_kernel<<<nb, RS_THREADS, 0, st>>>(*keys, n, shift, mask, hist, nb);
    rs_rowscan_kernel<<<mask + 1, SCAN_THREADS, 0, st>>>(hist, nb, rowtot);
    rs_scatter_kernel<<<nb, RS_THREADS, 0, st>>>(*keys, *vals, *keys_alt, *vals_alt, n, shift,
                                                 mask, hist, rowtot, nb);
    PMGB_LAUNCH_CHECK();
    count_launches(3);
    u64* tk = *keys;
    *keys = *keys_alt;
    *keys_alt = tk;
    u32* tv = *vals;
    *vals = *vals_alt;
    *vals_alt = tv;
  }
  return PMGB_OK;
}

int scan_scratch_words(int n) { return n / SCAN_TILE + 2; }

// out = exclusive scan of in[0, n) (in == out allowed), *total = the sum.  Up to 8 tiles one
// CTA walks the array; beyond, tile sums, their scan and the tiles run as three launches with
// the tile sums in scratch (scan_scratch_words(n) words).
int exclusive_scan(const u32* in, u32* out, int n, u32* total, u32* scratch, cudaStream_t st) {
  n = n < 0 ? 0 : n;
  const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles <= 8) {
    scan_serial_kernel<<<1, SCAN_THREADS, 0, st>>>(in, out, n, total);
    PMGB_LAUNCH_CHECK();
    count_launches(1);
    return PMGB_OK;
  }
  scan_tile_sums_kernel<<<tiles, SCAN_THREADS, 0, st>>>(in, n, scratch);
  scan_serial_kernel<<<1, SCAN_THREADS, 0, st>>>(scratch, scratch, tiles, total);
  scan_tiles_kernel<<<tiles, SCAN_THREADS, 0, st>>>(in, out, n, scratch);
  PMGB_LAUNCH_CHECK();
  count_launches(3);
  return PMGB_OK;
}

// ------------------------------------------------------------------ keys --------------
// Chaining-mesh cell of a code-unit position (ChainingMesh::tripleToFlatIndex); -1 outside.
__device__ __forceinline__ int chain_cell(const ChainDims& c, float x, float y, float z) {
  int cx = (int)__fdiv_rn(x, c.HCx), cy = (int)__fdiv_rn(y, c.HCy), cz = (int)__fdiv_rn(z, c.HCz);
  if (cx < 0 || cy < 0 || cz < 0 || cx >= c.Mx || cy >= c.My || cz >= c.Mz) return -1;
  return cx + cy * c.Mx + cz * c.Mx * c.My;
}

__global__ void chain_keys_kernel(const float4* __restrict__ pm, const float4* __restrict__ vi,
                                  int n, ChainDims c, int ysort, int ncells,
                                  const int* __restrict__ stop, u64* __restrict__ keys,
                                  u32* __restrict__ vals) {
  if (stop && *stop) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pm[i];
  int cell = chain_cell(c, p.x, p.y, p.z);
  const int sub2 = c.sub * c.sub;
  if (cell < 0) {
    cell = ncells * sub2;  // outside the chaining mesh: last bucket, no pair forces
  } else if (c.sub > 1) {  // sub-column of the cell (clamped: x / HCs and x / HC round apart)
    const int cx = cell % c.Mx, cz = cell / (c.Mx * c.My);
    const int sx = min(max((int)__fdiv_rn(p.x, c.HCsx) - cx * c.sub, 0), c.sub - 1);
    const int sz = min(max((int)__fdiv_rn(p.z, c.HCsz) - cz * c.sub, 0), c.sub - 1);
    cell = (cell * c.sub + sz) * c.sub + sx;
  }
  u32 lo;
  if (ysort) {
    lo = float_key(p.y);
  } else {
    int orig = __float_as_int(vi[i].w);
    lo = 0xFFFFFFFFu - (u32)orig;  // ChainingMesh::fill inserts at the head: descending id
  }
  keys[i] = ((u64)(u32)cell << 32) | lo;
  vals[i] = (u32)i;
}

// Runs of equal (cell, y) keys are ordered by original particle id, as the reference's
// insertion keeps earlier particles first among equal y (chainingMesh.cpp:33-38).
__global__ void fix_ties_kernel(const u64* __restrict__ keys, u32* __restrict__ vals,
                                const float4* __restrict__ vi, int n, const int* __restrict__ stop) {
  if (stop && *stop) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 >= n) return;
  u64 k = keys[i];
  if (keys[i + 1] != k) return;
  if (i > 0 && keys[i - 1] == k) return;
  int e = i + 1;
  while (e + 1 < n && keys[e + 1] == k) ++e;
  for (int a = i + 1; a <= e; ++a) {  // insertion sort of vals[i..e] by original id
    u32 v = vals[a];
    int ov = __float_as_int(vi[v].w);
    int b = a - 1;
    while (b >= i && __float_as_int(vi[vals[b]].w) > ov) {
      vals[b + 1] = vals[b];
      --b;
    }
    vals[b + 1] = v;
  }
}

__device__ __forceinline__ u32 spread3(u32 x) {  // 10 bits -> every third bit
  x &= 0x3FF;
  x = (x | (x << 16)) & 0x030000FF;
  x = (x | (x << 8)) & 0x0300F00F;
  x = (x | (x << 4)) & 0x030C30C3;
  x = (x | (x << 2)) & 0x09249249;
  return x;
}

__global__ void brick_keys_kernel(const float4* __restrict__ pm, int n, MeshDims m, int bshift,
                                  const int* __restrict__ stop, u64* __restrict__ keys,
                                  u32* __restrict__ vals) {
  if (stop && *stop) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pm[i];
  int ix = wrapi((int)floorf(p.x), m.nx) >> bshift;
  int iy = wrapi((int)floorf(p.y), m.ny) >> bshift;
  int iz = wrapi((int)floorf(p.z), m.nz) >> bshift;
  keys[i] = (u64)(spread3(ix) | (spread3(iy) << 1) | (spread3(iz) << 2));
  vals[i] = (u32)i;
}

// Permute particles into sorted order.
__global__ void gather_kernel(const u32* __restrict__ vals, int n, const float4* __restrict__ pm_in,
                              const float4* __restrict__ vi_in, float4* __restrict__ pm_out,
                              float4* __restrict__ vi_out, const int* __restrict__ stop) {
  if (stop && *stop) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  u32 s = vals[i];
  pm_out[i] = pm_in[s];
  vi_out[i] = vi_in[s];
}

// Cell start offsets of the P3M order: cell_start[c] = first sorted slot whose cell (key >> 32)
// is at least c, for c = 0 .. ncells_total (so cell_start[ncells_total] = n when every key is
// below it).  One binary search per cell, so long runs of empty cells cost no thread more than
// the others.
__global__ void cell_start_kernel(const u64* __restrict__ keys, int n, int* __restrict__ cell_start,
                                  int ncells_total, const int* __restrict__ stop) {
  if (stop && *stop) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncells_total) return;
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((int)(__ldg(&keys[mid]) >> 32) < c) lo = mid + 1;
    else hi = mid;
  }
  cell_start[c] = lo;
}

__global__ void fill_int_kernel(int* p, int n, int v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// ------------------------------------------------------------------ host side ---------
int launch_chain_keys(const float4* pm, const float4* vi, int n, ChainDims c, int ysort,
                      const int* stop, u64* keys, u32* vals, cudaStream_t st) {
  int ncells = c.Mx * c.My * c.Mz;  // keys hold sub-column ids (cells x sub^2, then the bucket)
  chain_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(pm, vi, n, c, ysort, ncells, stop, keys, vals);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

int launch_fix_ties(const u64* keys, u32* vals, const float4* vi, int n, const int* stop,
                    cudaStream_t st) {
  fix_ties_kernel<<<(n + 255) / 256, 256, 0, st>>>(keys, vals, vi, n, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

int launch_brick_keys(const float4* pm, int n, MeshDims m, int bshift, const int* stop, u64* keys,
                      u32* vals, cudaStream_t st) {
  brick_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(pm, n, m, bshift, stop, keys, vals);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

int launch_gather(const u64* keys, const u32* vals, int n, const float4* pm_in,
                  const float4* vi_in, float4* pm_out, float4* vi_out, int* cell_start,
                  int ncells_total, const int* stop, cudaStream_t st) {
  if (n == 0) {
    if (cell_start) {
      fill_int_kernel<<<(ncells_total + 256) / 256, 256, 0, st>>>(cell_start, ncells_total + 1, 0);
      PMGB_LAUNCH_CHECK();
    }
    return PMGB_OK;
  }
  gather_kernel<<<(n + 255) / 256, 256, 0, st>>>(vals, n, pm_in, vi_in, pm_out, vi_out, stop);
  if (cell_start)
    cell_start_kernel<<<(ncells_total + 256) / 256, 256, 0, st>>>(keys, n, cell_start, ncells_total, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(cell_start ? 2 : 1);
  return PMGB_OK;
}

}  // namespace pmgb
