// direct.cu - FP64 direct-sum accelerations of sampled target particles.
//
// Restates ppMethod's pairwise force (reference source/ppMethod.cpp:23-36):
//   a_i = sum_{j != i} -G m_j (x_i - x_j) / (|x_i - x_j|^2 + eps^2)^(3/2)
// in double precision, for a list of target particles against all n sources.  It is the
// accuracy yardstick of the force error reports (plain P3M, the learned closure, periodic PM);
// the reference's PP integrator plays the same role in its accuracy scenarios
// (source/demos.cpp:390-396, 617-621).  With periodic_L > 0 the minimum-image separation in a
// cube of side periodic_L is used (an approximation of the periodic force: no Ewald sum).
//
// Layout: targets in blocks of DS_TILE threads (one target each), sources split into `chunks`
// slices along grid.y so that a few thousand targets still fill the GPU; each block walks its
// slice in shared-memory tiles of double4 (x, y, z, m).  Partial sums per (slice, target) go to
// a buffer that a second kernel adds in slice order, so the result does not depend on timing.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace pmgb {

constexpr int DS_TILE = 128;

__global__ void __launch_bounds__(DS_TILE) direct_partial_kernel(
    const float* __restrict__ pos, const float* __restrict__ mass, int n,
    const int* __restrict__ idx, int m, double G, double eps2, double L, int chunk,
    double* __restrict__ part) {
  __shared__ double4 src[DS_TILE];
  const int k = blockIdx.x * DS_TILE + threadIdx.x;
  const int i = k < m ? idx[k] : -1;
  double xi = 0, yi = 0, zi = 0;
  if (i >= 0) {
    xi = pos[3 * i];
    yi = pos[3 * i + 1];
    zi = pos[3 * i + 2];
  }
  const int j0 = blockIdx.y * chunk;
  const int j1 = min(n, j0 + chunk);
  double ax = 0, ay = 0, az = 0;
  for (int jb = j0; jb < j1; jb += DS_TILE) {
    const int j = jb + threadIdx.x;
    if (j < j1)
      src[threadIdx.x] = make_double4(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2], mass[j]);
    __syncthreads();
    const int cnt = min(DS_TILE, j1 - jb);
    for (int s = 0; s < cnt; ++s) {
      const double4 q = src[s];
      double dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
      if (L > 0) {
        dx -= L * rint(dx / L);
        dy -= L * rint(dy / L);
        dz -= L * rint(dz / L);
      }
      const double r2 = dx * dx + dy * dy + dz * dz + eps2;
      // the target itself (j == i) is skipped, as in the reference's pair loop
      const double w = (jb + s == i || r2 == 0.0) ? 0.0 : -G * q.w / (r2 * sqrt(r2));
      ax += w * dx;
      ay += w * dy;
      az += w * dz;
    }
    __syncthreads();
  }
  if (k < m) {
    double* o = part + ((size_t)blockIdx.y * m + k) * 3;
    o[0] = ax;
    o[1] = ay;
    o[2] = az;
  }
}

__global__ void direct_reduce_kernel(const double* __restrict__ part, int m, int chunks,
                                     double* __restrict__ acc) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * m) return;
  double s = 0;
  for (int c = 0; c < chunks; ++c) s += part[(size_t)c * 3 * m + t];
  acc[t] = s;
}

}  // namespace pmgb

using namespace pmgb;

extern "C" int pmgb_direct_sum_fp64(int n, const float* pos, const float* masses, double G,
                                    double eps, int m, const int* idx, double periodic_L,
                                    double* acc) {
  if (n < 0 || m < 0 || (n > 0 && (!pos || !masses)) || (m > 0 && (!idx || !acc)))
    return set_error("pmgb_direct_sum_fp64: bad arguments"), PMGB_EINVAL;
  for (int k = 0; k < m; ++k)
    if (idx[k] < 0 || idx[k] >= n) return set_error("pmgb_direct_sum_fp64: target out of range"), PMGB_EINVAL;
  if (m == 0) return PMGB_OK;
  int dev = 0, sms = 0;
  PMGB_CUDA_TRY(cudaGetDevice(&dev));
  PMGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int tblocks = (m + DS_TILE - 1) / DS_TILE;
  // enough source slices for about 8 blocks per SM, each slice at least 4 tiles long
  int chunks = (8 * sms + tblocks - 1) / tblocks;
  chunks = std::max(1, std::min(chunks, (n + 4 * DS_TILE - 1) / (4 * DS_TILE)));
  const int chunk = (n + chunks - 1) / chunks;
  float *dpos = nullptr, *dmass = nullptr;
  int* didx = nullptr;
  double *dpart = nullptr, *dacc = nullptr;
  cudaStream_t st = nullptr;
  int rc = PMGB_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&dpos, sizeof(float) * 3 * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&dmass, sizeof(float) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&didx, sizeof(int) * (size_t)m);
  if (e == cudaSuccess) e = cudaMalloc(&dpart, sizeof(double) * 3 * (size_t)m * chunks);
  if (e == cudaSuccess) e = cudaMalloc(&dacc, sizeof(double) * 3 * (size_t)m);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dpos, pos, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dmass, masses, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(didx, idx, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    direct_partial_kernel<<<dim3(tblocks, chunks), DS_TILE, 0, st>>>(dpos, dmass, n, didx, m, G, eps * eps,
                                                                      periodic_L, chunk, dpart);
    direct_reduce_kernel<<<(3 * m + 255) / 256, 256, 0, st>>>(dpart, m, chunks, dacc);
    count_launches(2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(acc, dacc, sizeof(double) * 3 * (size_t)m, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_error(std::string("pmgb_direct_sum_fp64: ") + cudaGetErrorString(e));
    rc = e == cudaErrorMemoryAllocation ? PMGB_ENOMEM : PMGB_ECUDA;
  }
  cudaFree(dpos);
  cudaFree(dmass);
  cudaFree(didx);
  cudaFree(dpart);
  cudaFree(dacc);
  if (st) cudaStreamDestroy(st);
  return rc;
}
