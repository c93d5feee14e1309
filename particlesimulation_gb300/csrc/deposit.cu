// deposit.cu - mass assignment (PMMethod::spreadMass, reference source/pmMethod.cpp:200-277).
//
// Each particle's NGP / CIC / TSC contributions are computed with exactly the reference's float
// operations (no FMA contraction), then converted to 64-bit fixed point with a power-of-two
// scale (exact: w * 2^k is representable, so the conversion only drops bits below 2^-k) and
// summed with integer atomics.  Integer addition is associative, so the density mesh is
// bit-identical run to run whatever the order of particles or atomics.
//
// A CTA takes a chunk of consecutive (spatially sorted) particles, reduces the bounding box of
// their stencils and, when it fits, accumulates into a shared-memory tile that is flushed with
// one global atomic per touched cell; chunks whose box is too large (sparse or unsorted
// regions) add straight into global memory.  The tile holds 4,096 cells (32 KB as two 32-bit
// planes, see tile_add; a 64 KB tile, which would also take the 17^3-cell chunks of uniform
// regions, measured slower: fewer resident CTAs) and is flushed a mesh row per warp.  Where a
// chunk holds few particles per tile cell the direct path is the cheaper one: chunks cut at
// aligned 16 x 16 x 8-cell blocks, whose boxes all fit, measured slower with every chunk on
// the tile and no faster with the tile kept for chunks of at most 8 cells per particle.  Mesh
// indices wrap periodically (the reference leaves them unwrapped, undefined beyond the mesh
// edge).
#include "deposit_body.cuh"

namespace pmgb {

constexpr int DEP_TILE_PM = DEP_TILE;

template <int IS>
__global__ void __launch_bounds__(DEP_THREADS) deposit_kernel(const float4* __restrict__ pm,
                                                              int n, MeshDims m, float scale,
                                                              u64* __restrict__ rho,
                                                              const int* __restrict__ stop) {
  if (stop && *stop) return;
  extern __shared__ u64 dep_tile[];
  __shared__ int red[DEP_RED_WORDS];
  deposit_block<IS, DEP_PPT, DEP_TILE_PM>(pm, blockIdx.x * DEP_CHUNK, n, m, scale, rho, dep_tile, red);
}

int launch_deposit(int is, const float4* pm, int n, MeshDims m, float scale, u64* rho,
                   const int* stop, cudaStream_t st) {
  if (n <= 0) return PMGB_OK;
  int blocks = (n + DEP_CHUNK - 1) / DEP_CHUNK;
  constexpr int smem = DEP_TILE_PM * (int)sizeof(u64);
  if (is == 0) {
    PMGB_CUDA_TRY(cudaFuncSetAttribute(deposit_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    deposit_kernel<0><<<blocks, DEP_THREADS, smem, st>>>(pm, n, m, scale, rho, stop);
  } else if (is == 1) {
    PMGB_CUDA_TRY(cudaFuncSetAttribute(deposit_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    deposit_kernel<1><<<blocks, DEP_THREADS, smem, st>>>(pm, n, m, scale, rho, stop);
  } else {
    PMGB_CUDA_TRY(cudaFuncSetAttribute(deposit_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    deposit_kernel<2><<<blocks, DEP_THREADS, smem, st>>>(pm, n, m, scale, rho, stop);
  }
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

}  // namespace pmgb
