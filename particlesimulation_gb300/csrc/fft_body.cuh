// fft_body.cuh - the shared-memory FFT passes of the Poisson solve as device bodies (shared by
// the single-system and the ensemble kernels, so both compute bit-identical potentials).
// See fft.cu for the method.
//
// Every body is instantiated per transform length (2^3 .. 2^9, the mesh sizes the handles
// accept) and dispatched on the mesh's log2 size at entry, so the steps of a transform, their
// strides and twiddle spacings are compile-time constants: a thread's R elements of a radix-R
// group are one base address plus immediate offsets.
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
__device__ __forceinline__ int ilog2_dev(int v) { return 31 - __clz(v); }
__device__ __forceinline__ int ceil_log2_dev(int v) { return v <= 1 ? 0 : 32 - __clz(v - 1); }

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

// Shared-memory layouts of lines of n points.  Element p of line l lives at addr(p, l).
// Rows (x passes): line-major with one pad element per 16, so that the strided accesses of the
// first DIT / last DIF step spread over the banks.  Columns (y / z passes): point-major with the
// COL_TX columns of a tile side by side.  off(d) = addr(base + d, l) - addr(base, l) for the
// strides d = m 2^s of an FFT step (base has no bits where d has any).
struct RowLayout {
  int ls;  // n + n / 16
  __device__ __forceinline__ int operator()(int p, int l) const { return l * ls + p + (p >> 4); }
  static constexpr int off(int d) { return d + (d >> 4); }
};
struct ColLayout {
  __device__ __forceinline__ int operator()(int p, int l) const { return p * COL_TX + l; }
  static constexpr int off(int d) { return d * COL_TX; }
};
__host__ __device__ inline int row_stride(int n) { return n + (n >> 4); }

// One step of a radix-R FFT (R = 2^LR) over 2^lnl lines of 2^LOGN points, covering bits
// [S, S + LR) of the index.  DIT: input in bit-reversed order, the step equals the LR radix-2
// decimation-in-time stages S .. S+LR-1: the R elements base + m 2^S (j = base mod 2^S) are
// multiplied by W_L^(j rho), rho = bitrev(m), L = 2^(S+LR), and transformed by an R-point DFT
// over rho, giving outputs base + q 2^S.  DIF (natural order in, bit-reversed out): the
// transpose, equal to the radix-2 decimation-in-frequency stages S+LR-1 .. S.  Each thread
// reads and writes its own R elements, so the step is in place; the step with S = 0 has only
// unit twiddles.  tw = W_n^k for k < n.  LF: consecutive threads take consecutive lines (column
// tiles), else consecutive groups of one line (rows).
template <int R, int S, int LOGN, bool DIT, bool INV, bool LF, class Layout>
__device__ __forceinline__ void fft_step(float2* buf, int lnl, const float2* tw, Layout addr) {
  constexpr int LR = log2_c(R);
  constexpr int LGPL = LOGN - LR;  // log2 of the groups per line
  constexpr int TWSH = LOGN - S - LR;
  const int total = 1 << (lnl + LGPL);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int l, g;
    if (LF) {
      l = t & ((1 << lnl) - 1);
      g = t >> lnl;
    } else {
      g = t & ((1 << LGPL) - 1);
      l = t >> LGPL;
    }
    const int j = g & ((1 << S) - 1);
    const int base = ((g >> S) << (S + LR)) + j;
    float2* b0 = buf + addr(base, l);
    float2 v[R];
    if (DIT) {
#pragma unroll
      for (int m = 0; m < R; ++m) v[brev_c(m, LR)] = b0[Layout::off(m << S)];
      if (S > 0) {
        const int jt = j << TWSH;
#pragma unroll
        for (int rho = 1; rho < R; ++rho) {
          float2 w = tw[jt * rho];
          if (INV) w.y = -w.y;
          v[rho] = cmul(v[rho], w);
        }
      }
      reg_dft<R, INV>(v);
#pragma unroll
      for (int q = 0; q < R; ++q) b0[Layout::off(q << S)] = v[q];
    } else {
#pragma unroll
      for (int q = 0; q < R; ++q) v[q] = b0[Layout::off(q << S)];
      reg_dft<R, INV>(v);
      if (S > 0) {
        const int jt = j << TWSH;
#pragma unroll
        for (int rho = 1; rho < R; ++rho) {
          float2 w = tw[jt * rho];
          if (INV) w.y = -w.y;
          v[rho] = cmul(v[rho], w);
        }
      }
#pragma unroll
      for (int rho = 0; rho < R; ++rho) b0[Layout::off(brev_c(rho, LR) << S)] = v[rho];
    }
  }
}

// The steps of up to 4 bits (radix 16) of a transform.  DIT: S = bits already done, from 0 up;
// DIF: S = bits not yet done, from LOGN down.  A barrier follows every step.
template <int LOGN, int S, bool DIT, bool INV, bool LF, class Layout>
__device__ __forceinline__ void fft_steps(float2* buf, int lnl, const float2* tw, Layout addr) {
  if constexpr (DIT) {
    if constexpr (S < LOGN) {
      constexpr int r = (LOGN - S) < 4 ? (LOGN - S) : 4;
      fft_step<(1 << r), S, LOGN, true, INV, LF>(buf, lnl, tw, addr);
      __syncthreads();
      fft_steps<LOGN, S + r, true, INV, LF>(buf, lnl, tw, addr);
    }
  } else {
    if constexpr (S > 0) {
      constexpr int r = S < 4 ? S : 4;
      fft_step<(1 << r), S - r, LOGN, false, INV, LF>(buf, lnl, tw, addr);
      __syncthreads();
      fft_steps<LOGN, S - r, false, INV, LF>(buf, lnl, tw, addr);
    }
  }
}

// FFT of 2^lnl lines of 2^LOGN points in shared memory, in place.  DIT: bit-reversed input,
// natural output; DIF: natural input, bit-reversed output.  INV flips the exponent sign (no
// scaling).  Two shared-memory round trips for n = 256.
template <int LOGN, bool DIT, bool INV, bool LF, class Layout>
__device__ __forceinline__ void smem_fft(float2* buf, int lnl, const float2* tw, Layout addr) {
  fft_steps<LOGN, DIT ? 0 : LOGN, DIT, INV, LF>(buf, lnl, tw, addr);
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

// Calls f.template operator()<LOGN>() for the transform length 2^logn (3 <= logn <= 9).
template <class F>
__device__ __forceinline__ void with_logn(int logn, F&& f) {
  switch (logn) {
    case 3: f.template operator()<3>(); break;
    case 4: f.template operator()<4>(); break;
    case 5: f.template operator()<5>(); break;
    case 6: f.template operator()<6>(); break;
    case 7: f.template operator()<7>(); break;
    case 8: f.template operator()<8>(); break;
    default: f.template operator()<9>(); break;
  }
}

// ---------------------------------------------------------------- x pass, forward ----
// Rows row0 .. row0 + 2 pairs - 1, two real rows per complex FFT.  rho_copy != nullptr also
// keeps the float density (the run diagnostics' mesh energy).
template <int LOGN>
__device__ __forceinline__ void x_r2c_t(float2* sm, u64* __restrict__ rho, float2* __restrict__ spec,
                                        const MeshDims& m, int pairs, float fx_inv,
                                        const float2* __restrict__ twg, int nmax, long long row0,
                                        float* __restrict__ rho_copy) {
  constexpr int NX = 1 << LOGN, NXH = NX / 2 + 1;
  const RowLayout L{row_stride(NX)};
  float2* tw = sm + pairs * L.ls;
  load_twiddles(tw, twg, NX, nmax);
  u64* rb = rho + row0 * NX;
  float* cb = rho_copy ? rho_copy + row0 * NX : nullptr;
  float2* sb = spec + row0 * m.nxp;
  // all loads of a batch first (they would otherwise wait one by one behind the clearing
  // stores to the same array), then the clears, the conversion and the bit-reversed scatter
  constexpr int XB = 8;
  const int total = pairs * NX;
  for (int i0 = 0; i0 < total; i0 += XB * FFT_THREADS) {
    u64 va[XB], vb[XB];
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * FFT_THREADS + threadIdx.x;
      if (idx < total) {
        const int a = ((idx >> LOGN) << (LOGN + 1)) + (idx & (NX - 1));
        va[u] = rb[a];
        vb[u] = rb[a + NX];
      }
    }
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * FFT_THREADS + threadIdx.x;
      if (idx < total) {
        const int p = idx >> LOGN, j = idx & (NX - 1);
        const int a = (p << (LOGN + 1)) + j;
        rb[a] = 0ull;
        rb[a + NX] = 0ull;
        const float2 d = make_float2(__ll2float_rn((long long)va[u]) * fx_inv,
                                     __ll2float_rn((long long)vb[u]) * fx_inv);
        if (cb) {
          cb[a] = d.x;
          cb[a + NX] = d.y;
        }
        sm[L(brev(j, LOGN), p)] = d;
      }
    }
  }
  __syncthreads();
  smem_fft<LOGN, true, false, false>(sm, ilog2_dev(pairs), tw, L);
  const int nxp = m.nxp;
  for (int idx = threadIdx.x; idx < pairs * NXH; idx += FFT_THREADS) {
    const int p = idx / NXH, k = idx - p * NXH;
    const float2 zk = sm[L(k, p)], znk = sm[L((NX - k) & (NX - 1), p)];
    const float2 A = make_float2(0.5f * (zk.x + znk.x), 0.5f * (zk.y - znk.y));
    const float2 B = make_float2(0.5f * (zk.y + znk.y), -0.5f * (zk.x - znk.x));
    float2* o = sb + 2 * p * nxp + k;
    o[0] = A;
    o[nxp] = B;
  }
}

__device__ __forceinline__ void fft_x_r2c_body(float2* sm, u64* __restrict__ rho,
                                               float2* __restrict__ spec, const MeshDims& m,
                                               int pairs, float fx_inv,
                                               const float2* __restrict__ twg, int nmax,
                                               long long row0,
                                               float* __restrict__ rho_copy = nullptr) {
  with_logn(m.lx, [&]<int LOGN>() { x_r2c_t<LOGN>(sm, rho, spec, m, pairs, fx_inv, twg, nmax, row0, rho_copy); });
}

// ---------------------------------------------------------------- x pass, inverse ----
template <int LOGN>
__device__ __forceinline__ void x_c2r_t(float2* sm, const float2* __restrict__ spec,
                                        float* __restrict__ phi, const MeshDims& m, int pairs,
                                        const float2* __restrict__ twg, int nmax, long long row0) {
  constexpr int NX = 1 << LOGN, HN = NX / 2;
  const RowLayout L{row_stride(NX)};
  float2* tw = sm + pairs * L.ls;
  load_twiddles(tw, twg, NX, nmax);
  const float2* sb = spec + row0 * m.nxp;
  float* pb = phi + row0 * NX;
  const int nxp = m.nxp;
  constexpr int XB = 8;  // loads of a batch issued together
  const int total = pairs * NX;
  for (int i0 = 0; i0 < total; i0 += XB * FFT_THREADS) {
    float2 A[XB], B[XB];
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * FFT_THREADS + threadIdx.x;
      if (idx < total) {
        const int p = idx >> LOGN, k = idx & (NX - 1);
        const int kk = k <= HN ? k : NX - k;
        const float2* r = sb + 2 * p * nxp + kk;
        A[u] = r[0];
        B[u] = r[nxp];
      }
    }
#pragma unroll
    for (int u = 0; u < XB; ++u) {
      const int idx = i0 + u * FFT_THREADS + threadIdx.x;
      if (idx < total) {
        const int p = idx >> LOGN, k = idx & (NX - 1);
        float2 a = A[u], b = B[u];
        if (k == 0 || k == HN) {  // self-conjugate bins: keep the real part
          a.y = 0.f;
          b.y = 0.f;
        } else if (k > HN) {
          a.y = -a.y;
          b.y = -b.y;
        }
        sm[L(k, p)] = make_float2(a.x - b.y, a.y + b.x);  // A + i B
      }
    }
  }
  __syncthreads();
  smem_fft<LOGN, false, true, false>(sm, ilog2_dev(pairs), tw, L);
  for (int idx = threadIdx.x; idx < pairs * NX; idx += FFT_THREADS) {
    const int p = idx >> LOGN, j = idx & (NX - 1);
    const float2 z = sm[L(brev(j, LOGN), p)];
    const int a = (p << (LOGN + 1)) + j;
    pb[a] = z.x;
    pb[a + NX] = z.y;
  }
}

__device__ __forceinline__ void fft_x_c2r_body(float2* sm, const float2* __restrict__ spec,
                                               float* __restrict__ phi, const MeshDims& m,
                                               int pairs, const float2* __restrict__ twg, int nmax,
                                               long long row0) {
  with_logn(m.lx, [&]<int LOGN>() { x_c2r_t<LOGN>(sm, spec, phi, m, pairs, twg, nmax, row0); });
}

// ---------------------------------------------------------------- column passes ------
// axis 1: along y, `other` = z plane.  axis 2: along z, `other` = y row.
// mode 0: forward, 1: inverse, 2: forward * G then inverse (axis 2 only).
// Thread t handles column c = t mod COL_TX of the tile and points p = t / COL_TX + 16 k.
template <int LOGN>
__device__ __forceinline__ void cols_t(float2* sm, float2* __restrict__ spec, const MeshDims& m,
                                       int axis, int mode, const float* __restrict__ ghat,
                                       const float2* __restrict__ twg, int nmax, int kx0, int other) {
  constexpr int N = 1 << LOGN;
  constexpr int PSTEP = FFT_THREADS / COL_TX;
  constexpr int NK = (N + PSTEP - 1) / PSTEP;  // points per thread
  constexpr int CB = NK < 8 ? NK : 8;          // loads of a batch issued together
  float2* tw = sm + N * COL_TX;
  load_twiddles(tw, twg, N, nmax);
  // columns kx >= nxh are row padding: neither read nor written, and only the first 2^lnl
  // columns of a partial tile are transformed
  const int ncols = min(COL_TX, m.nxh - kx0);
  if (ncols <= 0) return;
  const int lnl = ceil_log2_dev(ncols);
  const int c = threadIdx.x & (COL_TX - 1), p0 = threadIdx.x / COL_TX;
  const bool cin = c < ncols;
  const size_t pstride = axis == 1 ? (size_t)m.nxp : (size_t)m.ny * m.nxp;
  const size_t cbase = (axis == 1 ? (size_t)other * m.ny * m.nxp : (size_t)other * m.nxp) + kx0 + c;
  float2* gcol = spec + cbase;
  const bool forward_first = mode != 1;
#pragma unroll 1
  for (int k0 = 0; k0 < NK; k0 += CB) {
    float2 v[CB];
#pragma unroll
    for (int k = 0; k < CB; ++k) {
      const int p = p0 + (k0 + k) * PSTEP;
      v[k] = (cin && p < N) ? gcol[p * pstride] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < CB; ++k) {
      const int p = p0 + (k0 + k) * PSTEP;
      if (p < N) sm[(forward_first ? brev(p, LOGN) : p) * COL_TX + c] = v[k];
    }
  }
  __syncthreads();
  const ColLayout L;
  if (mode == 0) {
    smem_fft<LOGN, true, false, true>(sm, lnl, tw, L);
  } else if (mode == 1) {
    smem_fft<LOGN, false, true, true>(sm, lnl, tw, L);
  } else {
    smem_fft<LOGN, true, false, true>(sm, lnl, tw, L);
    const float* gg = ghat + cbase;
#pragma unroll 1
    for (int k0 = 0; k0 < NK; k0 += CB) {
      float g[CB];
#pragma unroll
      for (int k = 0; k < CB; ++k) {
        const int p = p0 + (k0 + k) * PSTEP;
        g[k] = (cin && p < N) ? gg[p * pstride] : 0.f;
      }
#pragma unroll
      for (int k = 0; k < CB; ++k) {
        const int p = p0 + (k0 + k) * PSTEP;
        if (p < N) {
          float2& s = sm[p * COL_TX + c];
          s.x *= g[k];
          s.y *= g[k];
        }
      }
    }
    __syncthreads();
    smem_fft<LOGN, false, true, true>(sm, lnl, tw, L);
  }
  const bool bitrev_out = mode != 0;
#pragma unroll 8
  for (int k = 0; k < NK; ++k) {
    const int p = p0 + k * PSTEP;
    if (cin && p < N) gcol[p * pstride] = sm[(bitrev_out ? brev(p, LOGN) : p) * COL_TX + c];
  }
}

__device__ __forceinline__ void fft_cols_body(float2* sm, float2* __restrict__ spec,
                                              const MeshDims& m, int axis, int mode,
                                              const float* __restrict__ ghat,
                                              const float2* __restrict__ twg, int nmax, int kx0,
                                              int other) {
  with_logn(axis == 1 ? m.ly : m.lz, [&]<int LOGN>() {
    cols_t<LOGN>(sm, spec, m, axis, mode, ghat, twg, nmax, kx0, other);
  });
}

// rows pairs per CTA of the x passes by default (4096 complex points of shared memory: one
// radix-16 group per thread and step for n >= 16)
inline int x_pairs_default(const MeshDims& m) {
  int pairs = 4096 / m.nx;
  if (pairs < 1) pairs = 1;
  const long long rowpairs = (long long)m.ny * m.nz / 2;
  if (pairs > rowpairs) pairs = (int)rowpairs;
  return pairs;
}

}  // namespace pmgb
