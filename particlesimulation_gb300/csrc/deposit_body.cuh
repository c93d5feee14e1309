// deposit_body.cuh - the deposit of one chunk of particles by one CTA (shared by the
// single-system and the ensemble kernels, so both compute bit-identical densities).
// See deposit.cu for the method.
#pragma once
#include "common.cuh"

namespace pmgb {

constexpr int DEP_THREADS = 256;
constexpr int DEP_PPT = 2;                               // particles per thread
constexpr int DEP_CHUNK = DEP_THREADS * DEP_PPT;
constexpr int DEP_TILE = 4096;                           // u64 cells in the shared tile (32 KB)

template <int IS>
struct Stencil;
template <>
struct Stencil<0> { static constexpr int lo = 0, hi = 0; };
template <>
struct Stencil<1> { static constexpr int lo = 0, hi = 1; };
template <>
struct Stencil<2> { static constexpr int lo = 1, hi = 1; };

__device__ __forceinline__ long long to_fixed(float w, float scale) {
  return __float2ll_rn(__fmul_rn(w, scale));
}

// Calls emit(ix, iy, iz, fixed_value) for every stencil cell of particle p.
template <int IS, typename F>
__device__ __forceinline__ void stencil(const float4 p, float scale, F&& emit) {
  const float d = p.w;
  if (IS == 0) {
    int x = (int)roundf(p.x), y = (int)roundf(p.y), z = (int)roundf(p.z);
    emit(x, y, z, to_fixed(d, scale));
  } else if (IS == 1) {
    int x = (int)p.x, y = (int)p.y, z = (int)p.z;
    float dx = fsub(p.x, (float)x), dy = fsub(p.y, (float)y), dz = fsub(p.z, (float)z);
    float tx = fsub(1.0f, dx), ty = fsub(1.0f, dy), tz = fsub(1.0f, dz);
    emit(x, y, z, to_fixed(fmul(fmul(fmul(d, tx), ty), tz), scale));
    emit(x + 1, y, z, to_fixed(fmul(fmul(fmul(d, dx), ty), tz), scale));
    emit(x, y + 1, z, to_fixed(fmul(fmul(fmul(d, tx), dy), tz), scale));
    emit(x, y, z + 1, to_fixed(fmul(fmul(fmul(d, tx), ty), dz), scale));
    emit(x + 1, y + 1, z, to_fixed(fmul(fmul(fmul(d, dx), dy), tz), scale));
    emit(x + 1, y, z + 1, to_fixed(fmul(fmul(fmul(d, dx), ty), dz), scale));
    emit(x, y + 1, z + 1, to_fixed(fmul(fmul(fmul(d, tx), dy), dz), scale));
    emit(x + 1, y + 1, z + 1, to_fixed(fmul(fmul(fmul(d, dx), dy), dz), scale));
  } else {
    int x = (int)p.x, y = (int)p.y, z = (int)p.z;
    float dx = fsub(p.x, (float)x), dy = fsub(p.y, (float)y), dz = fsub(p.z, (float)z);
    const float d8 = __fdiv_rn(d, 8.0f);
#pragma unroll
    for (int t1 = -1; t1 <= 1; ++t1) {
      float T1 = fmul(d8, tsc_w(dx, t1));
#pragma unroll
      for (int t2 = -1; t2 <= 1; ++t2) {
        float T2 = fmul(T1, tsc_w(dy, t2));
#pragma unroll
        for (int t3 = -1; t3 <= 1; ++t3) {
          float T3 = fmul(T2, tsc_w(dz, t3));
          emit(x + t1, y + t2, z + t3, to_fixed(T3, scale));
        }
      }
    }
  }
}

template <int IS>
__device__ __forceinline__ void base_cell(const float4 p, int& x, int& y, int& z) {
  if (IS == 0) {
    x = (int)roundf(p.x);
    y = (int)roundf(p.y);
    z = (int)roundf(p.z);
  } else {
    x = (int)p.x;
    y = (int)p.y;
    z = (int)p.z;
  }
}

constexpr int DEP_WARPS = DEP_THREADS / 32;
constexpr int DEP_RED_WORDS = 6 * DEP_WARPS;             // shared ints of block_min6

// CTA-wide minima of six values in one pass (one barrier pair instead of one per value).
// red: DEP_RED_WORDS shared ints; the leading barrier lets a previous call's readers finish.
__device__ __forceinline__ void block_min6(int (&v)[6], int* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int j = 0; j < 6; ++j) v[j] = min(v[j], __shfl_xor_sync(0xFFFFFFFFu, v[j], o));
  }
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int j = 0; j < 6; ++j) red[j * DEP_WARPS + w] = v[j];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    int r = red[j * DEP_WARPS];
#pragma unroll
    for (int i = 1; i < DEP_WARPS; ++i) r = min(r, red[j * DEP_WARPS + i]);
    v[j] = r;
  }
}

// Shared tile cell c as two 32-bit planes: low words at t[c], high words at t[tile + c].  A
// 64-bit add is a 32-bit add of the low word, whose carry out (the old value plus the addend
// wraps) goes with the high word's add; modulo 2^64 the planes then hold exactly the 64-bit
// sum, in any order of the adds.  Shared 32-bit atomics are native, the 64-bit ones are not:
// with a 64-bit tile the deposit of 4,194,304 particles on a 256^3 mesh took 155 us, with the
// two planes 130 us.
__device__ __forceinline__ void tile_add(u32* t, int c, int tile, long long v) {
  const u32 lo = (u32)(u64)v, hi = (u32)((u64)v >> 32);
  const u32 old = atomicAdd(&t[c], lo);
  const u32 hc = hi + (u32)(old + lo < old);
  if (hc != 0u) atomicAdd(&t[tile + c], hc);
}

// Deposits particles [base, end) (at most PPT * DEP_THREADS of them).  tile: TILE u64 cells of
// shared memory.
template <int IS, int PPT, int TILE = DEP_TILE>
__device__ __forceinline__ void deposit_block(const float4* __restrict__ pm, int base, int end,
                                              const MeshDims& m, float scale, u64* __restrict__ rho,
                                              u64* tile, int* red) {
  float4 p[PPT];
  bool valid[PPT];
  int mnx = 1 << 30, mny = 1 << 30, mnz = 1 << 30, mxx = -(1 << 30), mxy = -(1 << 30), mxz = -(1 << 30);
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    int i = base + k * DEP_THREADS + threadIdx.x;
    valid[k] = i < end;
    if (valid[k]) {
      p[k] = pm[i];
      int x, y, z;
      base_cell<IS>(p[k], x, y, z);
      mnx = min(mnx, x); mny = min(mny, y); mnz = min(mnz, z);
      mxx = max(mxx, x); mxy = max(mxy, y); mxz = max(mxz, z);
    }
  }
  {
    int b6[6] = {mnx, mny, mnz, -mxx, -mxy, -mxz};
    block_min6(b6, red);
    mnx = b6[0]; mny = b6[1]; mnz = b6[2];
    mxx = -b6[3]; mxy = -b6[4]; mxz = -b6[5];
  }
  const int ox = mnx - Stencil<IS>::lo, oy = mny - Stencil<IS>::lo, oz = mnz - Stencil<IS>::lo;
  const int ex = mxx - mnx + Stencil<IS>::lo + Stencil<IS>::hi + 1;
  const int ey = mxy - mny + Stencil<IS>::lo + Stencil<IS>::hi + 1;
  const int ez = mxz - mnz + Stencil<IS>::lo + Stencil<IS>::hi + 1;
  const long long vol = (long long)ex * ey * ez;
  const bool use_tile = vol <= TILE && ex <= m.nx && ey <= m.ny && ez <= m.nz;
  const size_t sxy = (size_t)m.nx * m.ny;

  if (use_tile) {
    u32* t32 = reinterpret_cast<u32*>(tile);
    for (int c = threadIdx.x; c < (int)vol; c += DEP_THREADS) {
      t32[c] = 0u;
      t32[TILE + c] = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      if (!valid[k]) continue;
      stencil<IS>(p[k], scale, [&](int x, int y, int z, long long v) {
        tile_add(t32, (x - ox) + ex * ((y - oy) + ey * (z - oz)), TILE, v);
      });
    }
    __syncthreads();
    // one mesh row (y, z) of the tile per warp, x across the lanes
    const int lane = threadIdx.x & 31;
    for (int r = threadIdx.x >> 5; r < ey * ez; r += DEP_THREADS / 32) {
      const int tz = r / ey, ty = r - tz * ey;
      u64* row = rho + (size_t)wrapi(oz + tz, m.nz) * sxy + (size_t)wrapi(oy + ty, m.ny) * m.nx;
      const u32* trow = t32 + r * ex;
      for (int tx = lane; tx < ex; tx += 32) {
        const u64 v = ((u64)trow[TILE + tx] << 32) + trow[tx];
        if (v != 0ull) fx_add_global(&row[wrapi(ox + tx, m.nx)], (long long)v);
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      if (!valid[k]) continue;
      stencil<IS>(p[k], scale, [&](int x, int y, int z, long long v) {
        fx_add_global(&rho[(size_t)wrapi(z, m.nz) * sxy + (size_t)wrapi(y, m.ny) * m.nx + wrapi(x, m.nx)], v);
      });
    }
  }
}


}  // namespace pmgb
