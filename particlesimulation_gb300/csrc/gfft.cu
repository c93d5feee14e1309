// gfft.cu - 3D FFTs of any transform length (mixed radix), for meshes whose sides are not
// powers of two, and the complex-to-complex transforms of the FFT adapter (pmgb_fft3d).
//
// The reference takes any gridPoints: its FFT plug-ins (FFTW, kissfft) are mixed-radix
// (include/FFTAdapter.h:6-15, include/kissFFTAdapter.h:8-51), and its accuracy scenarios run
// (2Ng, 2Ng, Ng) meshes for Ng = 30, 34, ..., 70 (source/demos.cpp:361-428).  The Poisson solve
// of fft.cu is specialised for powers of two (compile-time radix-16 steps over a half
// spectrum); every other mesh takes this path, which follows the reference's own formulation:
// the real density as a complex mesh, complex-to-complex transforms along x, y and z, the
// influence function applied to the full spectrum, the inverse transforms, the real part as the
// potential.  The influence function is read from the symmetric half spectrum green.cu stores
// (G(k) = G(-k) there), so the potential is the one the reference's real part gives.
//
// Transforms.  One CTA takes a tile of up to GF_TX lines of one axis (lines along x: whole
// rows; along y or z: GF_TX neighbouring x columns, so global loads stay coalesced) into shared
// memory and runs a self-sorting (Stockham) decimation-in-frequency transform over the factors
// of n (4, 2, 3, 5, 7, then any remaining primes): in a stage of radix r over sub-transforms of
// length ncur = r m with stride s,
//   y[q + s (r p + u)] = W_ncur^(p u) sum_t x[q + s (p + t m)] W_r^(t u),
// one output per thread, reading its r inputs from the other buffer.  Twiddles W_n^k come from
// a table computed in double on the host.  Inverse transforms are unnormalised (the 1/N of the
// Poisson solve is folded into the influence function; pmgb_fft3d scales by 1/N like the
// reference's ifft).
#include <algorithm>
#include <cmath>
#include <vector>

#include "handles.cuh"

namespace pmgb {

constexpr int GF_THREADS = 256;
constexpr int GF_TX = 16;          // lines per tile
constexpr int GF_TILE = 8192;      // points per tile buffer (64 KB)
constexpr int GF_MAXF = 24;        // factors of a length

struct GPlan {
  int n = 0;
  int nf = 0;
  int f[GF_MAXF] = {};
  float2* tw = nullptr;  // device: W_n^k, k < n
};

static void factorize(int n, GPlan& p) {
  p.n = n;
  p.nf = 0;
  while (n % 4 == 0) p.f[p.nf++] = 4, n /= 4;
  for (int r : {2, 3, 5, 7})
    while (n % r == 0) p.f[p.nf++] = r, n /= r;
  for (int r = 11; n > 1; r += 2)
    while (n % r == 0) p.f[p.nf++] = r, n /= r;
}

static int make_plan(int n, GPlan& p) {
  factorize(n, p);
  std::vector<float2> w(n);
  const double PI = 3.14159265358979323846;
  for (int k = 0; k < n; ++k) {
    const double a = -2.0 * PI * (double)k / (double)n;
    w[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  PMGB_CUDA_TRY(cudaMalloc(&p.tw, sizeof(float2) * n));
  PMGB_CUDA_TRY(cudaMemcpy(p.tw, w.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  return PMGB_OK;
}

static int tile_lines(int n) { return std::max(1, std::min(GF_TX, GF_TILE / n)); }

// axis 0: lines are rows (contiguous); axis 1: stride nx, lines indexed by (x, z); axis 2:
// stride nx*ny, lines by (x, y).  Tile b of axis 0 = rows b*tl ..; of axes 1, 2 = columns
// x0 = (b % xt) * tl .. at other coordinate o = b / xt.
__global__ void __launch_bounds__(GF_THREADS) gfft_kernel(float2* __restrict__ data, int nx, int ny,
                                                          int nz, int axis, GPlan plan, int inverse,
                                                          const int* __restrict__ stop) {
  if (stop && *stop) return;
  extern __shared__ float2 gsm[];
  const int n = plan.n;
  const int tl = max(1, min(GF_TX, GF_TILE / n));
  float2* buf0 = gsm;
  float2* buf1 = gsm + tl * n;
  float2* tw = gsm + 2 * tl * n;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const float2 w = plan.tw[k];
    tw[k] = make_float2(w.x, inverse ? -w.y : w.y);
  }
  long long base = 0, estride = 1, lstride = 1;
  int nlines = tl;
  if (axis == 0) {
    const long long rows = (long long)ny * nz;
    const long long r0 = (long long)blockIdx.x * tl;
    nlines = (int)min((long long)tl, rows - r0);
    base = r0 * nx;
    estride = 1;
    lstride = nx;
  } else {
    const int xt = (nx + tl - 1) / tl;
    const int x0 = (blockIdx.x % xt) * tl;
    const long long o = blockIdx.x / xt;
    nlines = min(tl, nx - x0);
    estride = axis == 1 ? nx : (long long)nx * ny;
    base = x0 + o * (axis == 1 ? (long long)nx * ny : (long long)nx);
    lstride = 1;
  }
  // load: point-major layout buf[p * tl + l]
  for (int e = threadIdx.x; e < tl * n; e += blockDim.x) {
    int l, p;
    if (axis == 0) {
      l = e / n;
      p = e % n;
    } else {
      p = e / tl;
      l = e % tl;
    }
    if (l < nlines) buf0[p * tl + l] = data[base + l * lstride + p * estride];
  }
  __syncthreads();
  float2* x = buf0;
  float2* y = buf1;
  int ncur = n, s = 1;
  for (int f = 0; f < plan.nf; ++f) {
    const int r = plan.f[f];
    const int m = ncur / r;
    const int wr = n / r, wc = n / ncur;
    for (int e = threadIdx.x; e < tl * n; e += blockDim.x) {
      const int l = e % tl;
      const int o = e / tl;  // output index q + s (r p + u)
      const int q = o % s;
      const int rest = o / s;  // r p + u
      const int u = rest % r, p = rest / r;
      float ax = 0.f, ay = 0.f;
      for (int t = 0; t < r; ++t) {
        const float2 v = x[(q + s * (p + t * m)) * tl + l];
        const float2 w = tw[((t * u) % r) * wr];
        ax = fmaf(v.x, w.x, fmaf(-v.y, w.y, ax));
        ay = fmaf(v.x, w.y, fmaf(v.y, w.x, ay));
      }
      const float2 w = tw[p * u * wc];
      y[o * tl + l] = make_float2(ax * w.x - ay * w.y, ax * w.y + ay * w.x);
    }
    __syncthreads();
    float2* t = x;
    x = y;
    y = t;
    ncur = m;
    s *= r;
  }
  for (int e = threadIdx.x; e < tl * n; e += blockDim.x) {
    int l, p;
    if (axis == 0) {
      l = e / n;
      p = e % n;
    } else {
      p = e / tl;
      l = e % tl;
    }
    if (l < nlines) data[base + l * lstride + p * estride] = x[p * tl + l];
  }
}

// fixed-point density -> complex mesh (real part), cleared for the next deposit
__global__ void gfft_load_density_kernel(u64* __restrict__ rho, float2* __restrict__ data, long long L,
                                         float fx_inv, float* __restrict__ rho_copy,
                                         const int* __restrict__ stop) {
  if (stop && *stop) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x) {
    const float d = __ll2float_rn((long long)rho[i]) * fx_inv;
    rho[i] = 0ull;
    data[i] = make_float2(d, 0.f);
    if (rho_copy) rho_copy[i] = d;
  }
}

// spectrum x symmetric influence function (half spectrum, row stride nxp)
__global__ void gfft_green_kernel(float2* __restrict__ data, const float* __restrict__ ghat, MeshDims m,
                                  const int* __restrict__ stop) {
  if (stop && *stop) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m.L;
       i += (long long)gridDim.x * blockDim.x) {
    int kx = (int)(i % m.nx);
    const long long r = i / m.nx;
    int ky = (int)(r % m.ny), kz = (int)(r / m.ny);
    if (kx >= m.nxh) {  // G(k) = G(-k)
      kx = m.nx - kx;
      ky = (m.ny - ky) % m.ny;
      kz = (m.nz - kz) % m.nz;
    }
    const float g = ghat[((long long)kz * m.ny + ky) * m.nxp + kx];
    const float2 v = data[i];
    data[i] = make_float2(v.x * g, v.y * g);
  }
}

__global__ void gfft_store_potential_kernel(const float2* __restrict__ data, float* __restrict__ phi,
                                            long long L, const int* __restrict__ stop) {
  if (stop && *stop) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x)
    phi[i] = data[i].x;
}

struct GfftPlans {
  GPlan p[3];
};

static int gfft_smem(int n) { return (2 * tile_lines(n) * n + n) * (int)sizeof(float2); }

static int gfft_axis(float2* data, int nx, int ny, int nz, int axis, const GPlan& plan, int inverse,
                     const int* stop, cudaStream_t st) {
  const int n = plan.n;
  if (n == 1) return PMGB_OK;
  const int tl = tile_lines(n);
  long long blocks;
  if (axis == 0)
    blocks = ((long long)ny * nz + tl - 1) / tl;
  else
    blocks = (long long)((nx + tl - 1) / tl) * (axis == 1 ? nz : ny);
  const int sm = gfft_smem(n);
  PMGB_CUDA_TRY(cudaFuncSetAttribute(gfft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  gfft_kernel<<<(unsigned)blocks, GF_THREADS, sm, st>>>(data, nx, ny, nz, axis, plan, inverse, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

static int gfft_3d(float2* data, int nx, int ny, int nz, const GfftPlans& pl, int inverse,
                   const int* stop, cudaStream_t st) {
  const int order[3] = {0, 1, 2};
  for (int k = 0; k < 3; ++k) {
    const int a = inverse ? order[2 - k] : order[k];
    int rc = gfft_axis(data, nx, ny, nz, a, pl.p[a], inverse, stop, st);
    if (rc) return rc;
  }
  return PMGB_OK;
}

bool gfft_supported(int n) { return n >= 1 && n <= GF_TILE; }

int gfft_plans_create(const int dims[3], void** out) {
  auto* pl = new GfftPlans();
  for (int a = 0; a < 3; ++a) {
    int rc = make_plan(dims[a], pl->p[a]);
    if (rc) {
      gfft_plans_destroy(pl);
      return rc;
    }
  }
  *out = pl;
  return PMGB_OK;
}

void gfft_plans_destroy(void* plans) {
  auto* pl = static_cast<GfftPlans*>(plans);
  if (!pl) return;
  for (auto& p : pl->p)
    if (p.tw) cudaFree(p.tw);
  delete pl;
}

int launch_poisson_generic(u64* rho, float2* data, float* phi, const float* ghat, void* plans,
                           MeshDims m, float fx_inv, const int* stop, cudaStream_t st,
                           float* rho_copy) {
  const GfftPlans& pl = *static_cast<GfftPlans*>(plans);
  const int grid = 152 * 8;
  gfft_load_density_kernel<<<grid, 256, 0, st>>>(rho, data, m.L, fx_inv, rho_copy, stop);
  int rc = gfft_3d(data, m.nx, m.ny, m.nz, pl, 0, stop, st);
  if (rc) return rc;
  gfft_green_kernel<<<grid, 256, 0, st>>>(data, ghat, m, stop);
  rc = gfft_3d(data, m.nx, m.ny, m.nz, pl, 1, stop, st);
  if (rc) return rc;
  gfft_store_potential_kernel<<<grid, 256, 0, st>>>(data, phi, m.L, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(3);
  return PMGB_OK;
}

__global__ void gfft_scale_kernel(float2* __restrict__ data, long long L, float s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 v = data[i];
    data[i] = make_float2(v.x * s, v.y * s);
  }
}

}  // namespace pmgb

using namespace pmgb;

extern "C" int pmgb_fft3d(int nx, int ny, int nz, const float* in, float* out, int inverse) {
  if (nx < 1 || ny < 1 || nz < 1 || !in || !out)
    return set_error("pmgb_fft3d: bad arguments"), PMGB_EINVAL;
  if (!gfft_supported(nx) || !gfft_supported(ny) || !gfft_supported(nz))
    return set_error("pmgb_fft3d: transform lengths must be in [1, 8192]"), PMGB_EINVAL;
  const long long L = (long long)nx * ny * nz;
  const int dims[3] = {nx, ny, nz};
  void* plans = nullptr;
  int rc = gfft_plans_create(dims, &plans);
  if (rc) return rc;
  float2* d = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(float2) * L);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, in, sizeof(float2) * L, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    rc = gfft_3d(d, nx, ny, nz, *static_cast<GfftPlans*>(plans), inverse ? 1 : 0, nullptr, st);
    if (!rc && inverse) {
      gfft_scale_kernel<<<152 * 4, 256, 0, st>>>(d, L, (float)(1.0 / (double)L));
      count_launches(1);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess && !rc) e = cudaMemcpyAsync(out, d, sizeof(float2) * L, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && !rc) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess && !rc) {
    set_error(std::string("pmgb_fft3d: ") + cudaGetErrorString(e));
    rc = e == cudaErrorMemoryAllocation ? PMGB_ENOMEM : PMGB_ECUDA;
  }
  if (d) cudaFree(d);
  if (st) cudaStreamDestroy(st);
  gfft_plans_destroy(plans);
  return rc;
}
