// fft.cu - the Poisson solve: forward 3D real-to-complex FFT of the density, multiplication by
// the influence function, inverse complex-to-real FFT to the potential.
//
// The reference (Grid::fftDensity -> FFTAdapter::fft, findFourierPotential, invFftPotential ->
// FFTAdapter::ifft; source/grid.cpp:50-56, source/pmMethod.cpp:340-350) transforms the real
// density with a complex-to-complex FFT and keeps the real part of the inverse.  For a real
// density that is the same as a real-to-complex / complex-to-real pair with the influence
// function replaced by its symmetric part (G(k) + G(-k))/2, which is what is stored (green.cu).
//
// Layout.  Density / potential: nx*ny*nz, x fastest.  Half spectrum: rows of nxp complex
// (nx/2+1 used), then y, then z.  Five kernels, each one read + one write of the mesh:
//   fft_x_r2c   two real rows per complex FFT (the row pair trick); reads the fixed-point
//               density, converts it to float and clears it for the next deposit
//   fft_cols(y) columns of TX consecutive kx along y, forward
//   fft_cols(z) along z: forward, * G, inverse in the same shared-memory tile
//   fft_cols(y) inverse
//   fft_x_c2r   two rows per complex FFT, writes the potential (1/N is folded into G)
// Inside a CTA the transforms run in shared memory in steps of up to 4 bits (radix 16, the 16
// points of a butterfly group in registers, fft_body.cuh): decimation in time on bit-reversed
// input for forward transforms, decimation in frequency (bit-reversed output) for inverse ones,
// with twiddles computed in double on the host.  Each thread issues its global loads in
// batches of 8 before using them, so a CTA keeps enough loads in flight to stream from HBM.
#include "fft_body.cuh"

namespace pmgb {

__global__ void __launch_bounds__(FFT_THREADS) fft_x_r2c_kernel(u64* __restrict__ rho,
                                                                float2* __restrict__ spec,
                                                                MeshDims m, int pairs,
                                                                float fx_inv,
                                                                const float2* __restrict__ twg,
                                                                int nmax,
                                                                const int* __restrict__ stop,
                                                                float* __restrict__ rho_copy) {
  if (stop && *stop) return;
  extern __shared__ float2 sm[];
  fft_x_r2c_body(sm, rho, spec, m, pairs, fx_inv, twg, nmax, 2ll * blockIdx.x * pairs, rho_copy);
}

__global__ void __launch_bounds__(FFT_THREADS) fft_x_c2r_kernel(const float2* __restrict__ spec,
                                                                float* __restrict__ phi,
                                                                MeshDims m, int pairs,
                                                                const float2* __restrict__ twg,
                                                                int nmax,
                                                                const int* __restrict__ stop) {
  if (stop && *stop) return;
  extern __shared__ float2 sm[];
  fft_x_c2r_body(sm, spec, phi, m, pairs, twg, nmax, 2ll * blockIdx.x * pairs);
}

__global__ void __launch_bounds__(FFT_THREADS) fft_cols_kernel(float2* __restrict__ spec,
                                                               MeshDims m, int axis, int mode,
                                                               const float* __restrict__ ghat,
                                                               const float2* __restrict__ twg,
                                                               int nmax,
                                                               const int* __restrict__ stop) {
  if (stop && *stop) return;
  extern __shared__ float2 sm[];
  fft_cols_body(sm, spec, m, axis, mode, ghat, twg, nmax, blockIdx.x * COL_TX, blockIdx.y);
}

// ---------------------------------------------------------------- host side ----------
static int x_pairs(const MeshDims& m) { return x_pairs_default(m); }

int fft_smem_bytes_max(const MeshDims& m) {
  int a = x_smem_elems(m.nx, x_pairs(m)) * (int)sizeof(float2);
  int ny = col_smem_elems(m.ny) * (int)sizeof(float2);
  int nz = col_smem_elems(m.nz) * (int)sizeof(float2);
  return a > ny ? (a > nz ? a : nz) : (ny > nz ? ny : nz);
}

int fft_configure(const MeshDims& m) {
  int bytes = fft_smem_bytes_max(m);
  if (bytes > 48 * 1024) {
    PMGB_CUDA_TRY(cudaFuncSetAttribute(fft_x_r2c_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(fft_x_c2r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(fft_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  }
  return PMGB_OK;
}

// density (fixed point, cleared) -> potential; rho_copy (optional) receives the float density
int launch_poisson(u64* rho, float2* spec, float* phi, const float* ghat, const float2* tw,
                   int nmax, MeshDims m, float fx_inv, const int* stop, cudaStream_t st,
                   float* rho_copy) {
  const int pairs = x_pairs(m);
  const int xblocks = (int)((long long)m.ny * m.nz / 2 / pairs);
  const int xsmem = x_smem_elems(m.nx, pairs) * (int)sizeof(float2);
  const int ctiles = (m.nxp + COL_TX - 1) / COL_TX;
  const int ysmem = col_smem_elems(m.ny) * (int)sizeof(float2);
  const int zsmem = col_smem_elems(m.nz) * (int)sizeof(float2);
  fft_x_r2c_kernel<<<xblocks, FFT_THREADS, xsmem, st>>>(rho, spec, m, pairs, fx_inv, tw, nmax, stop, rho_copy);
  fft_cols_kernel<<<dim3(ctiles, m.nz), FFT_THREADS, ysmem, st>>>(spec, m, 1, 0, nullptr, tw, nmax, stop);
  fft_cols_kernel<<<dim3(ctiles, m.ny), FFT_THREADS, zsmem, st>>>(spec, m, 2, 2, ghat, tw, nmax, stop);
  fft_cols_kernel<<<dim3(ctiles, m.nz), FFT_THREADS, ysmem, st>>>(spec, m, 1, 1, nullptr, tw, nmax, stop);
  fft_x_c2r_kernel<<<xblocks, FFT_THREADS, xsmem, st>>>(spec, phi, m, pairs, tw, nmax, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(5);
  return PMGB_OK;
}

}  // namespace pmgb
