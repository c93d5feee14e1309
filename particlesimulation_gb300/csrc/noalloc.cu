// noalloc.cu - chaining-mesh cell lists without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need cell lists: a host
// application that hands this library device buffers from its own pre-sized pool and forbids
// further allocation, or a time-step loop that must not call cudaMalloc (it synchronises the
// device and can fail mid-run when memory is fragmented).  This entry point builds the same
// cell lists as a P3M force evaluation (cell by cell, y ascending with ties by particle index,
// or descending index) from caller-owned device input and output buffers, using only scratch
// that lives in file-scope __device__ arrays of fixed size:
//
//   at most kNoAllocMaxParticles = 262,144 particles and kNoAllocMaxCells - 2 = 262,142 cells;
//   about 7.1 MiB (7.4 MB) of device memory: sort keys 4 MiB, values 2 MiB, cell starts 1 MiB,
//   radix histogram 66 KB.  Under CUDA's lazy module loading (the default) the module holding
//   them, and so the scratch, is loaded on the first call on each device and then held until
//   the process exits.
//
// Host code cannot use those arrays' names as device addresses (on the host they are stand-in
// symbols), so on the first call on each device, with that device current, the device
// addresses are looked up with cudaGetSymbolAddress.  That first call is where the module and
// its scratch get loaded, so it should come before any CUDA graph capture and before any
// section of the caller's that must not allocate.  All calls share the same arrays: calls that may overlap on the
// GPU (different streams, or host threads calling concurrently) race and must be serialised by
// the caller.  Every call overwrites all of the scratch it reads, so nothing from a previous
// call leaks into the next.
#include <mutex>

#include "common.cuh"

namespace pmgb {

constexpr int kNoAllocMaxParticles = 262144;
constexpr int kNoAllocMaxCells = 262144;
// radix_sort_pairs writes radix_hist_words(n) = 256 radix_hist_blocks(n) + 256 histogram words,
// one block per RS_TILE keys (the constant the sort itself is built with)
constexpr int kNoAllocHistBlocks = (kNoAllocMaxParticles + RS_TILE - 1) / RS_TILE;

static __device__ __align__(256) u64 g_na_keys[2][kNoAllocMaxParticles];
static __device__ __align__(256) u32 g_na_vals[2][kNoAllocMaxParticles];
static __device__ __align__(256) u32 g_na_hist[256 * kNoAllocHistBlocks + 256];  // + row totals
static __device__ __align__(256) int g_na_cell_start[kNoAllocMaxCells + 2];

int radix_hist_blocks(int n);
int radix_sort_pairs(u64** keys, u32** vals, u64** keys_alt, u32** vals_alt, u32* hist, int n,
                     int nbits, cudaStream_t st);

struct NoAllocScratch {
  u64* keys[2] = {nullptr, nullptr};
  u32* vals[2] = {nullptr, nullptr};
  u32* hist = nullptr;
  int* cell_start = nullptr;
};

// Device addresses of the scratch arrays, per device (looked up once per device).
static int scratch_for_current_device(NoAllocScratch* out) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static NoAllocScratch table[kMaxDevices];
  static bool ready[kMaxDevices] = {};
  int dev = 0;
  PMGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error("device index out of range"), PMGB_EINVAL;
  std::lock_guard<std::mutex> lock(mu);
  if (!ready[dev]) {
    NoAllocScratch s;
    void* p = nullptr;
    PMGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_na_keys));
    s.keys[0] = static_cast<u64*>(p);
    s.keys[1] = s.keys[0] + kNoAllocMaxParticles;
    PMGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_na_vals));
    s.vals[0] = static_cast<u32*>(p);
    s.vals[1] = s.vals[0] + kNoAllocMaxParticles;
    PMGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_na_hist));
    s.hist = static_cast<u32*>(p);
    PMGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_na_cell_start));
    s.cell_start = static_cast<int*>(p);
    table[dev] = s;
    ready[dev] = true;
  }
  *out = table[dev];
  return PMGB_OK;
}

// Same cell rule as ChainingMesh (reference source/chainingMesh.cpp:20-30, 79-84).
__global__ void na_keys_kernel(const float* __restrict__ pos, int n, ChainDims c, int ysort,
                               int ncells, u64* __restrict__ keys, u32* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
  const int cx = (int)__fdiv_rn(x, c.HCx), cy = (int)__fdiv_rn(y, c.HCy), cz = (int)__fdiv_rn(z, c.HCz);
  int cell = ncells;  // outside the mesh: last bucket, not listed
  if (cx >= 0 && cy >= 0 && cz >= 0 && cx < c.Mx && cy < c.My && cz < c.Mz)
    cell = cx + cy * c.Mx + cz * c.Mx * c.My;
  // input is in particle order and the radix sort is stable: equal y keep index order
  const u32 lo = ysort ? float_key(y) : 0xFFFFFFFFu - (u32)i;
  keys[i] = ((u64)(u32)cell << 32) | lo;
  vals[i] = (u32)i;
}

__global__ void na_starts_kernel(const u64* __restrict__ keys, int n, int ncells_total,
                                 int* __restrict__ cell_start) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (n == 0) {
    for (int c = i; c <= ncells_total; c += gridDim.x * blockDim.x) cell_start[c] = 0;
    return;
  }
  if (i >= n) return;
  const int c = (int)(keys[i] >> 32);
  const int prev = i == 0 ? -1 : (int)(keys[i - 1] >> 32);
  for (int cc = prev + 1; cc <= c; ++cc) cell_start[cc] = i;
  if (i == n - 1)
    for (int cc = c + 1; cc <= ncells_total; ++cc) cell_start[cc] = n;
}

__global__ void na_output_kernel(const u32* __restrict__ vals, const int* __restrict__ cell_start,
                                 int n, int ncells, int* __restrict__ order,
                                 int* __restrict__ counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncells) counts[i] = cell_start[i + 1] - cell_start[i];
  if (i < n && i < cell_start[ncells]) order[i] = (int)vals[i];
}

}  // namespace pmgb

extern "C" int pmgb_chaining_mesh_fill_noalloc(const float* d_pos, int n,
                                               const pmgb_p3m_config* cfg, float H,
                                               int* d_order, int* d_counts, int* dims3,
                                               void* stream) {
  using namespace pmgb;
  if (!cfg || !dims3 || (n > 0 && (!d_pos || !d_order)) || !d_counts)
    return set_error("null argument"), PMGB_EINVAL;
  if (!(cfg->cutoff > 0) || !(H > 0)) return set_error("cutoff radius and H must be positive"), PMGB_EINVAL;
  if (n < 0 || n > kNoAllocMaxParticles)
    return set_error("pmgb_chaining_mesh_fill_noalloc: particle count " + std::to_string(n) +
                     " outside [0, " + std::to_string(kNoAllocMaxParticles) + "]"),
           PMGB_EINVAL;
  ChainDims c;
  c.sub = 1;
  c.Mx = (int)(cfg->comp_box[0] / cfg->cutoff);
  c.My = (int)(cfg->comp_box[1] / cfg->cutoff);
  c.Mz = (int)(cfg->comp_box[2] / cfg->cutoff);
  if (c.Mx < 1 || c.My < 1 || c.Mz < 1)
    return set_error("computational box smaller than the cutoff radius"), PMGB_EINVAL;
  const long long ncells = (long long)c.Mx * c.My * c.Mz;
  if (ncells + 2 > kNoAllocMaxCells)
    return set_error("pmgb_chaining_mesh_fill_noalloc: " + std::to_string(ncells) +
                     " cells exceed the maximum of " + std::to_string(kNoAllocMaxCells - 2)),
           PMGB_EINVAL;
  c.HCx = (cfg->comp_box[0] / c.Mx) / H;
  c.HCy = (cfg->comp_box[1] / c.My) / H;
  c.HCz = (cfg->comp_box[2] / c.Mz) / H;
  dims3[0] = c.Mx;
  dims3[1] = c.My;
  dims3[2] = c.Mz;
  NoAllocScratch s;
  int rc = scratch_for_current_device(&s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nc = (int)ncells;
  u64* keys = s.keys[0];
  u64* keys_alt = s.keys[1];
  u32* vals = s.vals[0];
  u32* vals_alt = s.vals[1];
  if (n > 0) {
    na_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_pos, n, c, cfg->y_sorting, nc, keys, vals);
    PMGB_LAUNCH_CHECK();
    count_launches(1);
    int bits = 32;
    while ((1ll << (bits - 32)) < ncells + 2) ++bits;
    rc = radix_sort_pairs(&keys, &vals, &keys_alt, &vals_alt, s.hist, n, bits, st);
    if (rc) return rc;
  }
  const int tpb = 256;
  na_starts_kernel<<<(n > 0 ? (n + tpb - 1) / tpb : (nc + tpb) / tpb), tpb, 0, st>>>(keys, n, nc + 1, s.cell_start);
  PMGB_LAUNCH_CHECK();
  const int m = n > nc ? n : nc;
  na_output_kernel<<<(m + tpb - 1) / tpb, tpb, 0, st>>>(vals, s.cell_start, n, nc, d_order, d_counts);
  PMGB_LAUNCH_CHECK();
  count_launches(2);
  return PMGB_OK;
}
