// fft_body.cuh - the shared-memory FFT passes of the Poisson solve as device bodies (shared by
// the single-system and the ensemble kernels, so both compute bit-identical potentials).
// See fft.cu for the method.
#pragma once
#include "common.cuh"

namespace pmgb {

constexpr int FFT_THREADS = 256;
constexpr int COL_TX = 16;  // columns (complex) per column-pass tile

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ int brev(int v, int logn) {
  return logn == 0 ? 0 : (int)(__brev((u32)v) >> (32 - logn));
}

// Radix-2 passes over `nlines` lines of length n = 2^logn held in shared memory; element p of
// line l is buf[p*ps + l*ls].  tw[j] = exp(-2 pi i j / n), j < n/2.  DIT expects bit-reversed
// input and produces natural order; DIF the reverse.  inv conjugates the twiddles.
template <bool DIT>
__device__ void smem_fft(float2* buf, int logn, int nlines, int ps, int ls, const float2* tw,
                         bool inv, bool line_fastest) {
  const int n = 1 << logn;
  const int hn = n >> 1;
  const int nb = nlines * hn;
  for (int st = 0; st < logn; ++st) {
    const int s = DIT ? st : logn - 1 - st;
    const int half = 1 << s;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      int l, b;
      if (line_fastest) {
        l = t % nlines;
        b = t / nlines;
      } else {
        b = t & (hn - 1);
        l = t >> (logn - 1);
      }
      const int j = b & (half - 1);
      const int i0 = ((b >> s) << (s + 1)) + j;
      const int i1 = i0 + half;
      float2 w = tw[j << (logn - 1 - s)];
      if (inv) w.y = -w.y;
      float2* p0 = buf + i0 * ps + l * ls;
      float2* p1 = buf + i1 * ps + l * ls;
      float2 a = *p0, c = *p1;
      if (DIT) {
        float2 v = cmul(c, w);
        *p0 = make_float2(a.x + v.x, a.y + v.y);
        *p1 = make_float2(a.x - v.x, a.y - v.y);
      } else {
        *p0 = make_float2(a.x + c.x, a.y + c.y);
        *p1 = cmul(make_float2(a.x - c.x, a.y - c.y), w);
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void load_twiddles(float2* tws, const float2* twg, int n, int nmax) {
  const int stride = nmax / n;
  for (int j = threadIdx.x; j < n / 2; j += blockDim.x) tws[j] = twg[j * stride];
}

// ---------------------------------------------------------------- x pass, forward ----
// rho_copy != nullptr also keeps the float density (the run diagnostics' mesh energy).
__device__ __forceinline__ void fft_x_r2c_body(float2* sm, u64* __restrict__ rho,
                                               float2* __restrict__ spec, const MeshDims& m,
                                               int pairs, float fx_inv,
                                               const float2* __restrict__ twg, int nmax,
                                               long long row0,
                                               float* __restrict__ rho_copy = nullptr) {
  const int nx = m.nx;
  float2* tw = sm + pairs * nx;
  load_twiddles(tw, twg, nx, nmax);
  for (int idx = threadIdx.x; idx < pairs * nx; idx += blockDim.x) {
    const int p = idx / nx, j = idx - p * nx;
    const size_t a = (size_t)(row0 + 2 * p) * nx + j;
    const long long va = (long long)rho[a], vb = (long long)rho[a + nx];
    rho[a] = 0ull;
    rho[a + nx] = 0ull;
    const float2 d = make_float2(__ll2float_rn(va) * fx_inv, __ll2float_rn(vb) * fx_inv);
    if (rho_copy) {
      rho_copy[a] = d.x;
      rho_copy[a + nx] = d.y;
    }
    sm[p * nx + brev(j, m.lx)] = d;
  }
  __syncthreads();
  smem_fft<true>(sm, m.lx, pairs, 1, nx, tw, false, false);
  for (int idx = threadIdx.x; idx < pairs * m.nxh; idx += blockDim.x) {
    const int p = idx / m.nxh, k = idx - p * m.nxh;
    const float2 zk = sm[p * nx + k], znk = sm[p * nx + ((nx - k) & (nx - 1))];
    const float2 A = make_float2(0.5f * (zk.x + znk.x), 0.5f * (zk.y - znk.y));
    const float2 B = make_float2(0.5f * (zk.y + znk.y), -0.5f * (zk.x - znk.x));
    const size_t r = (size_t)(row0 + 2 * p);
    spec[r * m.nxp + k] = A;
    spec[(r + 1) * m.nxp + k] = B;
  }
}

// ---------------------------------------------------------------- x pass, inverse ----
__device__ __forceinline__ void fft_x_c2r_body(float2* sm, const float2* __restrict__ spec,
                                               float* __restrict__ phi, const MeshDims& m,
                                               int pairs, const float2* __restrict__ twg, int nmax,
                                               long long row0) {
  const int nx = m.nx, hn = nx >> 1;
  float2* tw = sm + pairs * nx;
  load_twiddles(tw, twg, nx, nmax);
  for (int idx = threadIdx.x; idx < pairs * nx; idx += blockDim.x) {
    const int p = idx / nx, k = idx - p * nx;
    const size_t r = (size_t)(row0 + 2 * p);
    float2 A, B;
    if (k <= hn) {
      A = spec[r * m.nxp + k];
      B = spec[(r + 1) * m.nxp + k];
      if (k == 0 || k == hn) {  // self-conjugate bins: keep the real part
        A.y = 0.f;
        B.y = 0.f;
      }
    } else {
      A = spec[r * m.nxp + (nx - k)];
      B = spec[(r + 1) * m.nxp + (nx - k)];
      A.y = -A.y;
      B.y = -B.y;
    }
    sm[p * nx + k] = make_float2(A.x - B.y, A.y + B.x);  // A + i B
  }
  __syncthreads();
  smem_fft<false>(sm, m.lx, pairs, 1, nx, tw, true, false);
  for (int idx = threadIdx.x; idx < pairs * nx; idx += blockDim.x) {
    const int p = idx / nx, j = idx - p * nx;
    const float2 z = sm[p * nx + brev(j, m.lx)];
    const size_t a = (size_t)(row0 + 2 * p) * nx + j;
    phi[a] = z.x;
    phi[a + nx] = z.y;
  }
}

// ---------------------------------------------------------------- column passes ------
// axis 1: along y, blockIdx.y = z plane.  axis 2: along z, blockIdx.y = y row.
// mode 0: forward, 1: inverse, 2: forward * G then inverse (axis 2 only).
__device__ __forceinline__ void fft_cols_body(float2* sm, float2* __restrict__ spec,
                                              const MeshDims& m, int axis, int mode,
                                              const float* __restrict__ ghat,
                                              const float2* __restrict__ twg, int nmax, int kx0,
                                              int other) {
  const int logn = axis == 1 ? m.ly : m.lz;
  const int n = 1 << logn;
  float2* tw = sm + n * COL_TX;
  load_twiddles(tw, twg, n, nmax);
  // global index of (point p, column c)
  auto gidx = [&](int p, int c) -> size_t {
    if (axis == 1) return ((size_t)other * m.ny + p) * m.nxp + kx0 + c;
    return ((size_t)p * m.ny + other) * m.nxp + kx0 + c;
  };
  const int ncols = min(COL_TX, m.nxp - kx0);
  const bool forward_first = mode != 1;
  for (int idx = threadIdx.x; idx < n * COL_TX; idx += blockDim.x) {
    const int p = idx / COL_TX, c = idx - p * COL_TX;
    float2 v = c < ncols ? spec[gidx(p, c)] : make_float2(0.f, 0.f);
    sm[(forward_first ? brev(p, logn) : p) * COL_TX + c] = v;
  }
  __syncthreads();
  if (mode == 0) {
    smem_fft<true>(sm, logn, COL_TX, COL_TX, 1, tw, false, true);
  } else if (mode == 1) {
    smem_fft<false>(sm, logn, COL_TX, COL_TX, 1, tw, true, true);
  } else {
    smem_fft<true>(sm, logn, COL_TX, COL_TX, 1, tw, false, true);
    for (int idx = threadIdx.x; idx < n * COL_TX; idx += blockDim.x) {
      const int p = idx / COL_TX, c = idx - p * COL_TX;
      const float g = c < ncols ? ghat[gidx(p, c)] : 0.f;
      sm[idx].x *= g;
      sm[idx].y *= g;
    }
    __syncthreads();
    smem_fft<false>(sm, logn, COL_TX, COL_TX, 1, tw, true, true);
  }
  const bool bitrev_out = mode != 0;
  for (int idx = threadIdx.x; idx < n * COL_TX; idx += blockDim.x) {
    const int p = idx / COL_TX, c = idx - p * COL_TX;
    if (c < ncols) spec[gidx(p, c)] = sm[(bitrev_out ? brev(p, logn) : p) * COL_TX + c];
  }
}


// rows pairs per CTA of the x passes by default (2048 complex points of shared memory)
inline int x_pairs_default(const MeshDims& m) {
  int pairs = 2048 / m.nx;
  if (pairs < 1) pairs = 1;
  const long long rowpairs = (long long)m.ny * m.nz / 2;
  if (pairs > rowpairs) pairs = (int)rowpairs;
  return pairs;
}

}  // namespace pmgb
