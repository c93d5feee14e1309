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
__host__ __device__ constexpr int brev_c(int v, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((v >> b) & 1) << (bits - 1 - b);
  return r;
}
__host__ __device__ constexpr int log2_c(int v) { return v <= 1 ? 0 : 1 + log2_c(v >> 1); }

// cos / sin of 2 pi k / 16, k = 0..7 (the twiddles of the in-register DFTs, all powers of W16)
__device__ __forceinline__ float2 w16(int k, bool inv) {
  constexpr float c[8] = {1.0f, 0.923879532511286756f, 0.707106781186547524f, 0.382683432365089772f,
                          0.0f, -0.382683432365089772f, -0.707106781186547524f, -0.923879532511286756f};
  constexpr float s[8] = {0.0f, 0.382683432365089772f, 0.707106781186547524f, 0.923879532511286756f,
                          1.0f, 0.923879532511286756f, 0.707106781186547524f, 0.382683432365089772f};
  return make_float2(c[k], inv ? s[k] : -s[k]);  // exp(-+ 2 pi i k / 16)
}

// R-point DFT (R = 2, 4, 8, 16) of v in registers, natural order in and out, exponent sign
// -1 (forward) or +1 (INV); radix-2 decimation in time with the multiplications by 1 and -+i
// left out.
template <int R, bool INV>
__device__ __forceinline__ void reg_dft(float2 (&v)[R]) {
  constexpr int LR = log2_c(R);
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = brev_c(i, LR);
    if (i < j) {
      const float2 t = v[i];
      v[i] = v[j];
      v[j] = t;
    }
  }
#pragma unroll
  for (int half = 1; half < R; half <<= 1) {
#pragma unroll
    for (int b = 0; b < R; b += 2 * half) {
#pragma unroll
      for (int j = 0; j < half; ++j) {
        const int k = j * (8 / half);  // W_{2 half}^j = W16^k
        float2 c = v[b + j + half];
        if (k == 4) {
          c = INV ? make_float2(-c.y, c.x) : make_float2(c.y, -c.x);
        } else if (k != 0) {
          c = cmul(c, w16(k, INV));
        }
        const float2 a = v[b + j];
        v[b + j] = make_float2(a.x + c.x, a.y + c.y);
        v[b + j + half] = make_float2(a.x - c.x, a.y - c.y);
      }
    }
  }
}

// Shared-memory layouts of `nlines` lines of n points.  Element p of line l lives at addr(p, l).
// Rows (x passes): line-major with one pad element per 16, so that the strided accesses of the
// first DIT / last DIF step spread over the banks.  Columns (y / z passes): point-major with the
// COL_TX columns of a tile side by side.
struct RowLayout {
  int ls;  // n + n / 16
  __device__ __forceinline__ int operator()(int p, int l) const { return l * ls + p + (p >> 4); }
};
struct ColLayout {
  __device__ __forceinline__ int operator()(int p, int l) const { return p * COL_TX + l; }
};
__host__ __device__ inline int row_stride(int n) { return n + (n >> 4); }

// One step of a radix-2^r FFT over all lines, covering bits [s, s + r) of the index (R = 2^r
// elements per thread in registers).  DIT: input in bit-reversed order, the step equals the r
// radix-2 decimation-in-time stages s .. s+r-1: the R elements base + m 2^s (j = base mod 2^s)
// are multiplied by W_L^(j rho), rho = bitrev_r(m), L = 2^(s+r), and transformed by an R-point
// DFT over rho, giving outputs base + q 2^s.  DIF (natural order in, bit-reversed out): the
// transpose, equal to the r radix-2 decimation-in-frequency stages s+r-1 .. s.  Each thread
// reads and writes its own R elements, so the step is in place.  tw = W_n^k for k < n.
template <int R, bool DIT, bool INV, class Layout>
__device__ __forceinline__ void fft_step(float2* buf, int logn, int s, int nlines,
                                         const float2* tw, Layout addr, bool line_fastest) {
  constexpr int LR = log2_c(R);
  const int gpl = (1 << logn) >> LR;  // groups per line
  const int total = nlines * gpl;
  const int twsh = logn - s - LR;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int l, g;
    if (line_fastest) {
      l = t % nlines;
      g = t / nlines;
    } else {
      g = t & (gpl - 1);
      l = t >> (logn - LR);
    }
    const int j = g & ((1 << s) - 1);
    const int base = ((g >> s) << (s + LR)) + j;
    float2 v[R];
    if (DIT) {
#pragma unroll
      for (int m = 0; m < R; ++m) v[brev_c(m, LR)] = buf[addr(base + (m << s), l)];
#pragma unroll
      for (int rho = 1; rho < R; ++rho) {
        float2 w = tw[(j * rho) << twsh];
        if (INV) w.y = -w.y;
        v[rho] = cmul(v[rho], w);
      }
      reg_dft<R, INV>(v);
#pragma unroll
      for (int q = 0; q < R; ++q) buf[addr(base + (q << s), l)] = v[q];
    } else {
#pragma unroll
      for (int q = 0; q < R; ++q) v[q] = buf[addr(base + (q << s), l)];
      reg_dft<R, INV>(v);
#pragma unroll
      for (int rho = 1; rho < R; ++rho) {
        float2 w = tw[(j * rho) << twsh];
        if (INV) w.y = -w.y;
        v[rho] = cmul(v[rho], w);
      }
#pragma unroll
      for (int rho = 0; rho < R; ++rho) buf[addr(base + (brev_c(rho, LR) << s), l)] = v[rho];
    }
  }
}

template <bool DIT, bool INV, class Layout>
__device__ __forceinline__ void fft_step_r(int r, float2* buf, int logn, int s, int nlines,
                                           const float2* tw, Layout addr, bool line_fastest) {
  switch (r) {
    case 1: fft_step<2, DIT, INV>(buf, logn, s, nlines, tw, addr, line_fastest); break;
    case 2: fft_step<4, DIT, INV>(buf, logn, s, nlines, tw, addr, line_fastest); break;
    case 3: fft_step<8, DIT, INV>(buf, logn, s, nlines, tw, addr, line_fastest); break;
    default: fft_step<16, DIT, INV>(buf, logn, s, nlines, tw, addr, line_fastest); break;
  }
}

// FFT of `nlines` lines of n = 2^logn points in shared memory, in place.  DIT: bit-reversed
// input, natural output; DIF: natural input, bit-reversed output.  INV flips the exponent sign
// (no scaling).  Steps of up to 4 bits (radix 16): two shared-memory round trips for n = 256.
template <bool DIT, bool INV, class Layout>
__device__ void smem_fft(float2* buf, int logn, int nlines, const float2* tw, Layout addr,
                         bool line_fastest) {
  if (DIT) {
    for (int s = 0; s < logn;) {
      const int r = min(4, logn - s);
      fft_step_r<DIT, INV>(r, buf, logn, s, nlines, tw, addr, line_fastest);
      __syncthreads();
      s += r;
    }
  } else {
    for (int s = logn; s > 0;) {
      const int r = min(4, s);
      s -= r;
      fft_step_r<DIT, INV>(r, buf, logn, s, nlines, tw, addr, line_fastest);
      __syncthreads();
    }
  }
}

// W_n^k for k < n from the global half-circle table twg (W_nmax^j, j <= nmax/2).
__device__ __forceinline__ void load_twiddles(float2* tws, const float2* twg, int n, int nmax) {
  const int stride = nmax / n, hn = n >> 1;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const float2 w = twg[(k < hn ? k : k - hn) * stride];
    tws[k] = k < hn ? w : make_float2(-w.x, -w.y);
  }
}

// Shared-memory elements (float2) of an x-pass tile of `pairs` row pairs and of a column tile.
__host__ __device__ inline int x_smem_elems(int nx, int pairs) { return pairs * row_stride(nx) + nx; }
__host__ __device__ inline int col_smem_elems(int n) { return n * COL_TX + n; }

// ---------------------------------------------------------------- x pass, forward ----
// rho_copy != nullptr also keeps the float density (the run diagnostics' mesh energy).
__device__ __forceinline__ void fft_x_r2c_body(float2* sm, u64* __restrict__ rho,
                                               float2* __restrict__ spec, const MeshDims& m,
                                               int pairs, float fx_inv,
                                               const float2* __restrict__ twg, int nmax,
                                               long long row0,
                                               float* __restrict__ rho_copy = nullptr) {
  const int nx = m.nx;
  const RowLayout L{row_stride(nx)};
  float2* tw = sm + pairs * L.ls;
  load_twiddles(tw, twg, nx, nmax);
  // all loads of a batch first (they would otherwise wait one by one behind the clearing
  // stores to the same array), then the clears, the conversion and the bit-reversed scatter
  constexpr int XB = 8;
  const int total = pairs * nx;
  for (int i0 = 0; i0 < total; i0 += XB * blockDim.x) {
    u64 va[XB], vb[XB];
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * blockDim.x + threadIdx.x;
      if (idx < total) {
        const size_t a = (size_t)(row0 + 2 * (idx >> m.lx)) * nx + (idx & (nx - 1));
        va[u] = rho[a];
        vb[u] = rho[a + nx];
      }
    }
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * blockDim.x + threadIdx.x;
      if (idx < total) {
        const int p = idx >> m.lx, j = idx & (nx - 1);
        const size_t a = (size_t)(row0 + 2 * p) * nx + j;
        rho[a] = 0ull;
        rho[a + nx] = 0ull;
        const float2 d = make_float2(__ll2float_rn((long long)va[u]) * fx_inv,
                                     __ll2float_rn((long long)vb[u]) * fx_inv);
        if (rho_copy) {
          rho_copy[a] = d.x;
          rho_copy[a + nx] = d.y;
        }
        sm[L(brev(j, m.lx), p)] = d;
      }
    }
  }
  __syncthreads();
  smem_fft<true, false>(sm, m.lx, pairs, tw, L, false);
  for (int idx = threadIdx.x; idx < pairs * m.nxh; idx += blockDim.x) {
    const int p = idx / m.nxh, k = idx - p * m.nxh;
    const float2 zk = sm[L(k, p)], znk = sm[L((nx - k) & (nx - 1), p)];
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
  const RowLayout L{row_stride(nx)};
  float2* tw = sm + pairs * L.ls;
  load_twiddles(tw, twg, nx, nmax);
  constexpr int XB = 8;  // loads of a batch issued together
  const int total = pairs * nx;
  for (int i0 = 0; i0 < total; i0 += XB * blockDim.x) {
    float2 A[XB], B[XB];
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * blockDim.x + threadIdx.x;
      if (idx < total) {
        const int p = idx >> m.lx, k = idx & (nx - 1);
        const size_t r = (size_t)(row0 + 2 * p);
        const int kk = k <= hn ? k : nx - k;
        A[u] = spec[r * m.nxp + kk];
        B[u] = spec[(r + 1) * m.nxp + kk];
      }
    }
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * blockDim.x + threadIdx.x;
      if (idx < total) {
        const int p = idx >> m.lx, k = idx & (nx - 1);
        float2 a = A[u], b = B[u];
        if (k == 0 || k == hn) {  // self-conjugate bins: keep the real part
          a.y = 0.f;
          b.y = 0.f;
        } else if (k > hn) {
          a.y = -a.y;
          b.y = -b.y;
        }
        sm[L(k, p)] = make_float2(a.x - b.y, a.y + b.x);  // A + i B
      }
    }
  }
  __syncthreads();
  smem_fft<false, true>(sm, m.lx, pairs, tw, L, false);
  for (int idx = threadIdx.x; idx < pairs * nx; idx += blockDim.x) {
    const int p = idx >> m.lx, j = idx & (nx - 1);
    const float2 z = sm[L(brev(j, m.lx), p)];
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
  constexpr int CB = 8;  // loads of a batch issued together
  for (int i0 = 0; i0 < n * COL_TX; i0 += CB * blockDim.x) {
    float2 v[CB];
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const int idx = i0 + u * blockDim.x + threadIdx.x;
      const int p = idx / COL_TX, c = idx - p * COL_TX;
      v[u] = (idx < n * COL_TX && c < ncols) ? spec[gidx(p, c)] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < CB; ++u) {
      const int idx = i0 + u * blockDim.x + threadIdx.x;
      if (idx < n * COL_TX) {
        const int p = idx / COL_TX, c = idx - p * COL_TX;
        sm[(forward_first ? brev(p, logn) : p) * COL_TX + c] = v[u];
      }
    }
  }
  __syncthreads();
  const ColLayout L;
  if (mode == 0) {
    smem_fft<true, false>(sm, logn, COL_TX, tw, L, true);
  } else if (mode == 1) {
    smem_fft<false, true>(sm, logn, COL_TX, tw, L, true);
  } else {
    smem_fft<true, false>(sm, logn, COL_TX, tw, L, true);
    for (int i0 = 0; i0 < n * COL_TX; i0 += CB * blockDim.x) {
      float g[CB];
#pragma unroll
      for (int u = 0; u < CB; ++u) {
        const int idx = i0 + u * blockDim.x + threadIdx.x;
        const int p = idx / COL_TX, c = idx - p * COL_TX;
        g[u] = (idx < n * COL_TX && c < ncols) ? ghat[gidx(p, c)] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < CB; ++u) {
        const int idx = i0 + u * blockDim.x + threadIdx.x;
        if (idx < n * COL_TX) {
          sm[idx].x *= g[u];
          sm[idx].y *= g[u];
        }
      }
    }
    __syncthreads();
    smem_fft<false, true>(sm, logn, COL_TX, tw, L, true);
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
