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

// 4 CTAs per SM (64 registers, no spills; the 75 it would take otherwise allow 3): the pass
// streams the fixed-point density and measured ~1.5 % faster at 256^3
template <int LOGN>
__global__ void __launch_bounds__(FFT_THREADS, 4) fft_x_r2c_kernel(u64* __restrict__ rho,
                                                                float2* __restrict__ spec,
                                                                MeshDims m, int pairs,
                                                                float fx_inv,
                                                                const float2* __restrict__ twg,
                                                                int nmax,
                                                                const int* __restrict__ stop,
                                                                float* __restrict__ rho_copy) {
  if (stop && *stop) return;
  extern __shared__ float2 sm[];
  x_r2c_t<LOGN>(sm, rho, spec, m, pairs, fx_inv, twg, nmax, 2ll * blockIdx.x * pairs, rho_copy);
}

template <int LOGN>
__global__ void __launch_bounds__(FFT_THREADS) fft_x_c2r_kernel(const float2* __restrict__ spec,
                                                                float* __restrict__ phi,
                                                                MeshDims m, int pairs,
                                                                const float2* __restrict__ twg,
                                                                int nmax,
                                                                const int* __restrict__ stop) {
  if (stop && *stop) return;
  extern __shared__ float2 sm[];
  x_c2r_t<LOGN>(sm, spec, phi, m, pairs, twg, nmax, 2ll * blockIdx.x * pairs);
}

template <int LOGN>
__global__ void __launch_bounds__(FFT_THREADS) fft_cols_kernel(float2* __restrict__ spec,
                                                               MeshDims m, int axis, int mode,
                                                               const float* __restrict__ ghat,
                                                               const float2* __restrict__ twg,
                                                               int nmax,
                                                               const int* __restrict__ stop) {
  if (stop && *stop) return;
  extern __shared__ float2 sm[];
  cols_t<LOGN>(sm, spec, m, axis, mode, ghat, twg, nmax, blockIdx.x * COL_TX, blockIdx.y);
}

// The kernels of one transform length, picked on the host.
struct FftKernels {
  void (*r2c)(u64*, float2*, MeshDims, int, float, const float2*, int, const int*, float*);
  void (*c2r)(const float2*, float*, MeshDims, int, const float2*, int, const int*);
  void (*cols)(float2*, MeshDims, int, int, const float*, const float2*, int, const int*);
};
template <int LOGN>
constexpr FftKernels fft_kernels_t() {
  return {fft_x_r2c_kernel<LOGN>, fft_x_c2r_kernel<LOGN>, fft_cols_kernel<LOGN>};
}
static const FftKernels kFft[10] = {{}, {}, {}, fft_kernels_t<3>(), fft_kernels_t<4>(), fft_kernels_t<5>(),
                                    fft_kernels_t<6>(), fft_kernels_t<7>(), fft_kernels_t<8>(), fft_kernels_t<9>()};

// ---------------------------------------------------------------- host side ----------
static int x_pairs(const MeshDims& m) { return x_pairs_default(m); }

int fft_configure(const MeshDims& m) {
  const int xs = x_smem_elems(m.nx, x_pairs(m)) * (int)sizeof(float2);
  const int ys = col_smem_elems(m.ny) * (int)sizeof(float2), zs = col_smem_elems(m.nz) * (int)sizeof(float2);
  if (xs > 48 * 1024) {
    PMGB_CUDA_TRY(cudaFuncSetAttribute(kFft[m.lx].r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, xs));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(kFft[m.lx].c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, xs));
  }
  if (ys > 48 * 1024)
    PMGB_CUDA_TRY(cudaFuncSetAttribute(kFft[m.ly].cols, cudaFuncAttributeMaxDynamicSharedMemorySize, ys));
  if (zs > 48 * 1024)
    PMGB_CUDA_TRY(cudaFuncSetAttribute(kFft[m.lz].cols, cudaFuncAttributeMaxDynamicSharedMemorySize, zs));
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
  const FftKernels& kx = kFft[m.lx];
  const FftKernels& ky = kFft[m.ly];
  const FftKernels& kz = kFft[m.lz];
  kx.r2c<<<xblocks, FFT_THREADS, xsmem, st>>>(rho, spec, m, pairs, fx_inv, tw, nmax, stop, rho_copy);
  ky.cols<<<dim3(ctiles, m.nz), FFT_THREADS, ysmem, st>>>(spec, m, 1, 0, nullptr, tw, nmax, stop);
  kz.cols<<<dim3(ctiles, m.ny), FFT_THREADS, zsmem, st>>>(spec, m, 2, 2, ghat, tw, nmax, stop);
  ky.cols<<<dim3(ctiles, m.nz), FFT_THREADS, ysmem, st>>>(spec, m, 1, 1, nullptr, tw, nmax, stop);
  kx.c2r<<<xblocks, FFT_THREADS, xsmem, st>>>(spec, phi, m, pairs, tw, nmax, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(5);
  return PMGB_OK;
}

}  // namespace pmgb
