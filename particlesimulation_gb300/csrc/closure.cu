// closure.cu - learned short-range closure for P3M (no counterpart in the reference).
//
// The plain P3M pair pass (reference source/p3mMethod.cpp:168-322) sums the short-range force
// of every pair closer than the cutoff re.  The closure runs the pair pass with a reduced
// cutoff re' (< re, same particle shape, same table function) and predicts the missing part,
//   residual_i = sum_{re' <= |r_ij| < re} m_j F(|r_ij|) r_ij,
// with a small MLP from the particle's neighbourhood on the reduced chaining mesh:
//   inputs  (67)  the 4 x 4 x 4 patch of cell masses around the particle (cells of side >= re',
//                 the patch chosen so the particle sits in its central 2 x 2 x 2 block) divided
//                 by the patch mass S, and the particle's offset from the patch centre in cell
//                 units (3)
//   network       67 -> 64 -> 64 -> 64 -> 3, GELU, BF16 weights and activations, FP32
//                 accumulation (mma.sync m16n8k16 bf16 tensor-core tiles, one warp per 16
//                 particles; layer outputs stay in registers as the next layer's operands)
//   output  (3)   residual / (S * c), c = 1 / (4 pi HC'^2)  (the residual is linear in the
//                 masses, so scaling by S makes the map scale free)
// Training pairs are the exact residual from the plain P3M itself (full-cutoff force minus
// reduced-cutoff force, both on the GPU; their PM parts are bit-identical and cancel).  Training
// (forward, backward, Adam) runs on the GPU in the kernels below.  The full-cutoff P3M is the
// judge: every judge_interval steps it recomputes the force, and if the median relative error
// of the closure force exceeds the bound the run falls back to plain P3M.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <numbers>
#include <random>
#include <vector>

#include "handles.cuh"

namespace pmgb {

typedef __nv_bfloat16 bf16;

constexpr int CL_IN = 67, CL_K0 = 80, CL_H = 64, CL_NO = 8;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + CL_H * CL_K0, OFF_W2 = OFF_B1 + CL_H,
              OFF_B2 = OFF_W2 + CL_H * CL_H, OFF_W3 = OFF_B2 + CL_H,
              OFF_B3 = OFF_W3 + CL_H * CL_H, OFF_W4 = OFF_B3 + CL_H,
              OFF_B4 = OFF_W4 + CL_NO * CL_H, CL_NPARAM = OFF_B4 + CL_NO;
// bf16 weight image in shared memory, row strides padded against bank conflicts
constexpr int S80 = 88, S64 = 72, S16 = 24;
constexpr int IMG_W1 = 0, IMG_W2 = IMG_W1 + CL_H * S80, IMG_W3 = IMG_W2 + CL_H * S64,
              IMG_W4 = IMG_W3 + CL_H * S64, IMG_W2T = IMG_W4 + CL_NO * S64,
              IMG_W3T = IMG_W2T + CL_H * S64, IMG_W4T = IMG_W3T + CL_H * S64,
              IMG_SIZE = IMG_W4T + CL_H * S16;  // bf16 elements
constexpr int CL_WARPS = 4, CL_THREADS = CL_WARPS * 32;

// ------------------------------------------------------------------ helpers -----------
__device__ __forceinline__ u32 ld32(const bf16* p) { return *reinterpret_cast<const u32*>(p); }
__device__ __forceinline__ u32 pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<u32*>(&v);
}
__device__ __forceinline__ u32 pack_raw(bf16 lo, bf16 hi) {
  return (u32)__bfloat16_as_ushort(lo) | ((u32)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ void mma16816(float c[4], const u32 a[4], const u32 b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// Fragments of m16n8k16 (g = lane / 4, t = lane % 4):
//   A (16x16, row-major): a0 (g, 2t..2t+1), a1 (g+8, 2t..), a2 (g, 2t+8..), a3 (g+8, 2t+8..)
//   B (16x8, k x n):      b0 (k = 2t..2t+1, n = g), b1 (k = 2t+8.., n = g)
//   C (16x8):             c0, c1 (g, 2t..2t+1), c2, c3 (g+8, 2t..2t+1)
// A[r][k] = M[r0 + r][k0 + k], M row-major with stride S
__device__ __forceinline__ void ld_a(u32 a[4], const bf16* M, int S, int r0, int k0, int g, int t) {
  a[0] = ld32(M + (r0 + g) * S + k0 + 2 * t);
  a[1] = ld32(M + (r0 + g + 8) * S + k0 + 2 * t);
  a[2] = ld32(M + (r0 + g) * S + k0 + 8 + 2 * t);
  a[3] = ld32(M + (r0 + g + 8) * S + k0 + 8 + 2 * t);
}
// A[r][k] = M[k0 + k][r0 + r]
__device__ __forceinline__ void ld_a_t(u32 a[4], const bf16* M, int S, int r0, int k0, int g, int t) {
  a[0] = pack_raw(M[(k0 + 2 * t) * S + r0 + g], M[(k0 + 2 * t + 1) * S + r0 + g]);
  a[1] = pack_raw(M[(k0 + 2 * t) * S + r0 + g + 8], M[(k0 + 2 * t + 1) * S + r0 + g + 8]);
  a[2] = pack_raw(M[(k0 + 2 * t + 8) * S + r0 + g], M[(k0 + 2 * t + 9) * S + r0 + g]);
  a[3] = pack_raw(M[(k0 + 2 * t + 8) * S + r0 + g + 8], M[(k0 + 2 * t + 9) * S + r0 + g + 8]);
}
// B[k][n] = W[n0 + n][k0 + k], W row-major with stride S (a weight matrix stored out x in)
__device__ __forceinline__ void ld_b(u32 b[2], const bf16* W, int S, int n0, int k0, int g, int t) {
  b[0] = ld32(W + (n0 + g) * S + k0 + 2 * t);
  b[1] = ld32(W + (n0 + g) * S + k0 + 8 + 2 * t);
}
// B[k][n] = M[k0 + k][n0 + n]
__device__ __forceinline__ void ld_b_rm(u32 b[2], const bf16* M, int S, int n0, int k0, int g, int t) {
  b[0] = pack_raw(M[(k0 + 2 * t) * S + n0 + g], M[(k0 + 2 * t + 1) * S + n0 + g]);
  b[1] = pack_raw(M[(k0 + 2 * t + 8) * S + n0 + g], M[(k0 + 2 * t + 9) * S + n0 + g]);
}

// One dense layer for a warp's 16 rows: out[nt] (C fragments, NT tiles of 8 columns) =
// A (KS k-slices of 16) x W^T + bias.
template <int NT, int KS>
__device__ __forceinline__ void dense(float out[NT][4], const u32 a[KS][4], const bf16* W, int S,
                                      const float* bias, int g, int t) {
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const float b0 = bias[nt * 8 + 2 * t], b1 = bias[nt * 8 + 2 * t + 1];
    out[nt][0] = b0;
    out[nt][1] = b1;
    out[nt][2] = b0;
    out[nt][3] = b1;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
      u32 b[2];
      ld_b(b, W, S, nt * 8, ks * 16, g, t);
      mma16816(out[nt], a[ks], b);
    }
  }
}

// GELU of 8 C tiles (16 x 64) into 4 A k-slices (register-only chaining).
__device__ __forceinline__ void act_to_a(u32 a[4][4], const float z[8][4]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    a[j][0] = pack_bf16(gelu(z[2 * j][0]), gelu(z[2 * j][1]));
    a[j][1] = pack_bf16(gelu(z[2 * j][2]), gelu(z[2 * j][3]));
    a[j][2] = pack_bf16(gelu(z[2 * j + 1][0]), gelu(z[2 * j + 1][1]));
    a[j][3] = pack_bf16(gelu(z[2 * j + 1][2]), gelu(z[2 * j + 1][3]));
  }
}

struct SmemMLP {
  bf16 img[IMG_SIZE];
  float bias[CL_H * 3 + CL_NO];  // b1, b2, b3, b4
};

__device__ void load_mlp_smem(SmemMLP& s, const bf16* __restrict__ img, const float* __restrict__ p) {
  const u32* src = reinterpret_cast<const u32*>(img);
  u32* dst = reinterpret_cast<u32*>(s.img);
  for (int i = threadIdx.x; i < IMG_SIZE / 2; i += blockDim.x) dst[i] = src[i];
  for (int i = threadIdx.x; i < CL_H; i += blockDim.x) {
    s.bias[i] = p[OFF_B1 + i];
    s.bias[CL_H + i] = p[OFF_B2 + i];
    s.bias[2 * CL_H + i] = p[OFF_B3 + i];
  }
  for (int i = threadIdx.x; i < CL_NO; i += blockDim.x) s.bias[3 * CL_H + i] = p[OFF_B4 + i];
}

// Forward pass of a warp's 16 rows held as A fragments x0 (5 k-slices); returns the output tile
// and, for training, the pre-activations.
template <bool KEEP>
__device__ __forceinline__ void mlp_forward(const SmemMLP& s, const u32 x0[5][4], float y[4],
                                            float z1[8][4], float z2[8][4], float z3[8][4],
                                            u32 a1[4][4], u32 a2[4][4], u32 a3[4][4], int g, int t) {
  dense<8, 5>(z1, x0, s.img + IMG_W1, S80, s.bias, g, t);
  act_to_a(a1, z1);
  dense<8, 4>(z2, a1, s.img + IMG_W2, S64, s.bias + CL_H, g, t);
  act_to_a(a2, z2);
  dense<8, 4>(z3, a2, s.img + IMG_W3, S64, s.bias + 2 * CL_H, g, t);
  act_to_a(a3, z3);
  float out[1][4];
  dense<1, 4>(out, a3, s.img + IMG_W4, S64, s.bias + 3 * CL_H, g, t);
  y[0] = out[0][0];
  y[1] = out[0][1];
  y[2] = out[0][2];
  y[3] = out[0][3];
}

// ------------------------------------------------------------------ occupancy --------
struct ReducedMesh {
  int Mx, My, Mz;
  float HCx, HCy, HCz;
  float fx_scale, fx_inv;
  float out_scale;  // 1 / (4 pi HC^2), code units
};

__global__ void occ_deposit_kernel(const float4* __restrict__ pm, int n, ReducedMesh rm,
                                   u64* __restrict__ occ_fx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int cell = -1;
  long long q = 0;
  if (i < n) {
    const float4 p = pm[i];
    const int cx = (int)__fdiv_rn(p.x, rm.HCx), cy = (int)__fdiv_rn(p.y, rm.HCy),
              cz = (int)__fdiv_rn(p.z, rm.HCz);
    if (cx >= 0 && cy >= 0 && cz >= 0 && cx < rm.Mx && cy < rm.My && cz < rm.Mz) {
      cell = cx + cy * rm.Mx + cz * rm.Mx * rm.My;
      q = __float2ll_rn(__fmul_rn(p.w, rm.fx_scale));
    }
  }
  // one atomic per distinct cell of the warp (sorted particles share cells); integer sums are
  // order independent
  const u32 peers = __match_any_sync(0xFFFFFFFFu, cell);
  const int leader = __ffs(peers) - 1;
  long long sum = q;
  for (int o = 0; o < 32; ++o) {
    const long long v = __shfl_sync(0xFFFFFFFFu, q, o);
    if (o != (threadIdx.x & 31) && ((peers >> o) & 1)) sum += v;
  }
  if (cell >= 0 && (threadIdx.x & 31) == leader) atomicAdd(&occ_fx[cell], (u64)sum);
}

__global__ void occ_finalize_kernel(u64* __restrict__ occ_fx, float* __restrict__ occ, int ncells,
                                    float fx_inv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  occ[c] = __ll2float_rn((long long)occ_fx[c]) * fx_inv;
  occ_fx[c] = 0ull;
}

// Features of one particle: 64 patch masses / S, offset (3), zero padding to 80.  Written as
// floats into f[0..79]; returns S.
__device__ __forceinline__ float features(const ReducedMesh& rm, const float* __restrict__ occ,
                                          float x, float y, float z, float f[CL_K0]) {
  int o[3];
  float off[3];
  const float u[3] = {__fdiv_rn(x, rm.HCx), __fdiv_rn(y, rm.HCy), __fdiv_rn(z, rm.HCz)};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int c = (int)floorf(u[a]);
    const float fr = u[a] - (float)c;
    const int up = fr >= 0.5f ? 1 : 0;
    o[a] = c - 2 + up;
    off[a] = fr - (float)up;
  }
  float S = 0.f;
#pragma unroll
  for (int k = 0; k < 64; ++k) {
    const int cx = o[0] + (k & 3), cy = o[1] + ((k >> 2) & 3), cz = o[2] + (k >> 4);
    float m = 0.f;
    if (cx >= 0 && cy >= 0 && cz >= 0 && cx < rm.Mx && cy < rm.My && cz < rm.Mz)
      m = __ldg(&occ[cx + cy * rm.Mx + cz * rm.Mx * rm.My]);
    f[k] = m;
    S += m;
  }
  const float inv = S > 0.f ? 1.0f / S : 0.f;
#pragma unroll
  for (int k = 0; k < 64; ++k) f[k] *= inv;
  f[64] = off[0];
  f[65] = off[1];
  f[66] = off[2];
#pragma unroll
  for (int k = CL_IN; k < CL_K0; ++k) f[k] = 0.f;
  return S;
}

// ------------------------------------------------------------------ inference --------
// acc[i] += MLP(features(i)) * S * c, for the particles of this handle (sorted order).
__global__ void __launch_bounds__(CL_THREADS) closure_infer_kernel(
    const float4* __restrict__ pm, int n, ReducedMesh rm, const float* __restrict__ occ,
    const bf16* __restrict__ img, const float* __restrict__ params, float4* __restrict__ acc,
    const int* __restrict__ stop) {
  if (*stop) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemMLP& s = *reinterpret_cast<SmemMLP*>(smem_raw);
  bf16* xs_all = reinterpret_cast<bf16*>(smem_raw + sizeof(SmemMLP));
  float* sp_all = reinterpret_cast<float*>(smem_raw + sizeof(SmemMLP) + CL_WARPS * 16 * S80 * sizeof(bf16));
  load_mlp_smem(s, img, params);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  bf16* xs = xs_all + warp * 16 * S80;
  float* spatch = sp_all + warp * 16;
  const int tiles = (n + 15) / 16;
  for (int tile = blockIdx.x * CL_WARPS + warp; tile < tiles; tile += gridDim.x * CL_WARPS) {
    const int r0 = tile * 16;
    // features: lane r < 16 builds row r
    if (lane < 16) {
      const int i = r0 + lane;
      float f[CL_K0];
      float S = 0.f;
      if (i < n) {
        const float4 p = pm[i];
        S = features(rm, occ, p.x, p.y, p.z, f);
      } else {
#pragma unroll
        for (int k = 0; k < CL_K0; ++k) f[k] = 0.f;
      }
#pragma unroll
      for (int c = 0; c < CL_K0; c += 2)
        *reinterpret_cast<u32*>(xs + lane * S80 + c) = pack_bf16(f[c], f[c + 1]);
      spatch[lane] = S;
    }
    __syncwarp();
    u32 x0[5][4];
#pragma unroll
    for (int ks = 0; ks < 5; ++ks) ld_a(x0[ks], xs, S80, 0, ks * 16, g, t);
    float y[4], z1[8][4], z2[8][4], z3[8][4];
    u32 a1[4][4], a2[4][4], a3[4][4];
    mlp_forward<false>(s, x0, y, z1, z2, z3, a1, a2, a3, g, t);
    // y: rows g, g+8; columns 2t, 2t+1 (outputs 0..2 live in t = 0, 1)
    if (t < 2) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = g + 8 * h, i = r0 + r;
        if (i < n) {
          const float sc = spatch[r] * rm.out_scale;
          float* a = reinterpret_cast<float*>(&acc[i]);
          a[2 * t] += y[2 * h] * sc;
          if (t == 0) a[1] += y[2 * h + 1] * sc;
        }
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ training ---------
// Per warp: 16 training rows (by permutation), forward, loss, backward; per-warp partial
// gradients go to gw[warp][CL_NPARAM] (reduced deterministically by grad_reduce_kernel).
struct TrainSmemWarp {
  bf16 x[16 * S80];
  bf16 a1[16 * S64], a2[16 * S64], a3[16 * S64];
  bf16 d[16 * S64];
  bf16 dy[16 * S16];
};

__global__ void __launch_bounds__(CL_THREADS) closure_train_kernel(
    const bf16* __restrict__ X, const float* __restrict__ T, const int* __restrict__ perm,
    int batch_off, int batch, float inv_batch, const bf16* __restrict__ img,
    const float* __restrict__ params, float* __restrict__ gw, float* __restrict__ lossw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemMLP& s = *reinterpret_cast<SmemMLP*>(smem_raw);
  TrainSmemWarp* tw_all = reinterpret_cast<TrainSmemWarp*>(smem_raw + sizeof(SmemMLP));
  load_mlp_smem(s, img, params);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  TrainSmemWarp& w = tw_all[warp];
  const int gwarp = blockIdx.x * CL_WARPS + warp;
  const int r0 = gwarp * 16;
  float* G = gw + (size_t)gwarp * CL_NPARAM;
  // stage inputs
  for (int e = lane; e < 16 * (CL_K0 / 2); e += 32) {
    const int r = e / (CL_K0 / 2), c2 = e % (CL_K0 / 2);
    const int row = r0 + r;
    u32 v = 0u;
    if (row < batch) v = reinterpret_cast<const u32*>(X + (size_t)perm[batch_off + row] * CL_K0)[c2];
    *reinterpret_cast<u32*>(w.x + r * S80 + 2 * c2) = v;
  }
  __syncwarp();
  u32 x0[5][4];
#pragma unroll
  for (int ks = 0; ks < 5; ++ks) ld_a(x0[ks], w.x, S80, 0, ks * 16, g, t);
  float y[4], z1[8][4], z2[8][4], z3[8][4];
  u32 a1[4][4], a2[4][4], a3[4][4];
  mlp_forward<true>(s, x0, y, z1, z2, z3, a1, a2, a3, g, t);
  // activations to shared memory (for the weight gradients)
  auto store_act = [&](bf16* dst, const u32 a[4][4]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      *reinterpret_cast<u32*>(dst + g * S64 + 16 * j + 2 * t) = a[j][0];
      *reinterpret_cast<u32*>(dst + (g + 8) * S64 + 16 * j + 2 * t) = a[j][1];
      *reinterpret_cast<u32*>(dst + g * S64 + 16 * j + 8 + 2 * t) = a[j][2];
      *reinterpret_cast<u32*>(dst + (g + 8) * S64 + 16 * j + 8 + 2 * t) = a[j][3];
    }
  };
  store_act(w.a1, a1);
  store_act(w.a2, a2);
  store_act(w.a3, a3);
  // dY and loss
  float loss = 0.f;
  float dy[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int r = g + 8 * (e >> 1), o = 2 * t + (e & 1), row = r0 + r;
    float d = 0.f;
    if (row < batch && o < 3) {
      const float diff = y[e] - T[(size_t)perm[batch_off + row] * 4 + o];
      loss += diff * diff;
      d = 2.0f * diff * inv_batch;
    }
    dy[e] = d;
  }
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, o);
  if (lane == 0) lossw[gwarp] = loss;
  // dY tile (16 x 16, columns 8..15 zero)
  *reinterpret_cast<u32*>(w.dy + g * S16 + 2 * t) = pack_bf16(dy[0], dy[1]);
  *reinterpret_cast<u32*>(w.dy + (g + 8) * S16 + 2 * t) = pack_bf16(dy[2], dy[3]);
  *reinterpret_cast<u32*>(w.dy + g * S16 + 8 + 2 * t) = 0u;
  *reinterpret_cast<u32*>(w.dy + (g + 8) * S16 + 8 + 2 * t) = 0u;
  __syncwarp();

  // bias gradient of a C-tile column pair: sum over rows g, g+8 and over g
  auto col_sums = [&](float c0, float c1, float& s0, float& s1) {
    s0 = c0;
    s1 = c1;
    for (int o = 4; o < 32; o <<= 1) {
      s0 += __shfl_xor_sync(0xFFFFFFFFu, s0, o);
      s1 += __shfl_xor_sync(0xFFFFFFFFu, s1, o);
    }
  };
  // ---- layer 4: dW4 = dY^T A3 (16 padded outputs x 64), db4, dA3 = dY W4
  {
    u32 aT[4];
    ld_a_t(aT, w.dy, S16, 0, 0, g, t);  // A[o][b] = dY[b][o]
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      u32 b[2];
      ld_b_rm(b, w.a3, S64, nt * 8, 0, g, t);  // B[b][j] = A3[b][j]
      mma16816(c, aT, b);
      if (g < CL_NO) {
        G[OFF_W4 + g * CL_H + nt * 8 + 2 * t] = c[0];
        G[OFF_W4 + g * CL_H + nt * 8 + 2 * t + 1] = c[1];
      }
    }
    float s0, s1;
    col_sums(dy[0] + dy[2], dy[1] + dy[3], s0, s1);
    if (g == 0) {
      G[OFF_B4 + 2 * t] = s0;
      G[OFF_B4 + 2 * t + 1] = s1;
    }
  }
  float dz[8][4];
  {
    u32 ad[4];
    ld_a(ad, w.dy, S16, 0, 0, g, t);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      dz[nt][0] = dz[nt][1] = dz[nt][2] = dz[nt][3] = 0.f;
      u32 b[2];
      ld_b(b, s.img + IMG_W4T, S16, nt * 8, 0, g, t);  // B[o][j] = W4[o][j] = W4T[j][o]
      mma16816(dz[nt], ad, b);
    }
  }
  // ---- hidden layers 3, 2, 1
  auto hidden_backward = [&](float z[8][4], const bf16* a_in, int a_stride, int kin, int off_w,
                             int off_b, const bf16* wt, bool need_dx) {
    // dZ = dA * gelu'(Z)  (in place in dz), bias gradient, dZ to shared memory
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
      for (int e = 0; e < 4; ++e) dz[nt][e] *= gelu_grad(z[nt][e]);
      float s0, s1;
      col_sums(dz[nt][0] + dz[nt][2], dz[nt][1] + dz[nt][3], s0, s1);
      if (g == 0) {
        G[off_b + nt * 8 + 2 * t] = s0;
        G[off_b + nt * 8 + 2 * t + 1] = s1;
      }
      *reinterpret_cast<u32*>(w.d + g * S64 + nt * 8 + 2 * t) = pack_bf16(dz[nt][0], dz[nt][1]);
      *reinterpret_cast<u32*>(w.d + (g + 8) * S64 + nt * 8 + 2 * t) = pack_bf16(dz[nt][2], dz[nt][3]);
    }
    __syncwarp();
    // dW[j][i] = sum_b dZ[b][j] A_in[b][i]: 4 m-tiles (j) x kin/8 n-tiles (i), K = 16 rows
#pragma unroll
    for (int mt = 0; mt < 4; ++mt) {
      u32 aT[4];
      ld_a_t(aT, w.d, S64, mt * 16, 0, g, t);
      for (int nt = 0; nt < kin / 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        u32 b[2];
        ld_b_rm(b, a_in, a_stride, nt * 8, 0, g, t);
        mma16816(c, aT, b);
        const int j0 = mt * 16 + g, i0 = nt * 8 + 2 * t;
        G[off_w + j0 * kin + i0] = c[0];
        G[off_w + j0 * kin + i0 + 1] = c[1];
        G[off_w + (j0 + 8) * kin + i0] = c[2];
        G[off_w + (j0 + 8) * kin + i0 + 1] = c[3];
      }
    }
    if (need_dx) {
      // dA_in = dZ W  (W stored out x in; B[j][i] = W[j][i] = WT[i][j])
      u32 ad[4][4];
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) ld_a(ad[ks], w.d, S64, 0, ks * 16, g, t);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        dz[nt][0] = dz[nt][1] = dz[nt][2] = dz[nt][3] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          u32 b[2];
          ld_b(b, wt, S64, nt * 8, ks * 16, g, t);
          mma16816(dz[nt], ad[ks], b);
        }
      }
    }
    __syncwarp();
  };
  hidden_backward(z3, w.a2, S64, CL_H, OFF_W3, OFF_B3, s.img + IMG_W3T, true);
  hidden_backward(z2, w.a1, S64, CL_H, OFF_W2, OFF_B2, s.img + IMG_W2T, true);
  hidden_backward(z1, w.x, S80, CL_K0, OFF_W1, OFF_B1, nullptr, false);
}

__global__ void grad_reduce_kernel(const float* __restrict__ gw, int nwarps, float* __restrict__ grad,
                                   const float* __restrict__ lossw, float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < CL_NPARAM) {
    float s = 0.f;
    for (int w = 0; w < nwarps; ++w) s += gw[(size_t)w * CL_NPARAM + p];
    grad[p] = s;
  }
  if (p == 0) {
    float s = 0.f;
    for (int w = 0; w < nwarps; ++w) s += lossw[w];
    *loss = s;
  }
}

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ grad, float lr, float b1, float b2, float eps,
                            float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= CL_NPARAM) return;
  const float gr = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * gr;
  const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// bf16 weight image (and transposes) from the fp32 parameters
__global__ void image_kernel(const float* __restrict__ p, bf16* __restrict__ img) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < IMG_SIZE; e += gridDim.x * blockDim.x) {
    float v = 0.f;
    if (e < IMG_W2) {
      const int r = e / S80, c = e % S80;
      v = c < CL_K0 ? p[OFF_W1 + r * CL_K0 + c] : 0.f;
    } else if (e < IMG_W3) {
      const int r = (e - IMG_W2) / S64, c = (e - IMG_W2) % S64;
      v = c < CL_H ? p[OFF_W2 + r * CL_H + c] : 0.f;
    } else if (e < IMG_W4) {
      const int r = (e - IMG_W3) / S64, c = (e - IMG_W3) % S64;
      v = c < CL_H ? p[OFF_W3 + r * CL_H + c] : 0.f;
    } else if (e < IMG_W2T) {
      const int r = (e - IMG_W4) / S64, c = (e - IMG_W4) % S64;
      v = c < CL_H ? p[OFF_W4 + r * CL_H + c] : 0.f;
    } else if (e < IMG_W3T) {
      const int r = (e - IMG_W2T) / S64, c = (e - IMG_W2T) % S64;  // W2T[i][j] = W2[j][i]
      v = c < CL_H ? p[OFF_W2 + c * CL_H + r] : 0.f;
    } else if (e < IMG_W4T) {
      const int r = (e - IMG_W3T) / S64, c = (e - IMG_W3T) % S64;
      v = c < CL_H ? p[OFF_W3 + c * CL_H + r] : 0.f;
    } else {
      const int r = (e - IMG_W4T) / S16, c = (e - IMG_W4T) % S16;  // W4T[j][o] = W4[o][j]
      v = c < CL_NO ? p[OFF_W4 + c * CL_H + r] : 0.f;
    }
    img[e] = __float2bfloat16_rn(v);
  }
}

// training rows from the current state: X (bf16 features), T (targets, 4 floats per row)
__global__ void collect_kernel(const float* __restrict__ pos /*code units, original order*/,
                               const float* __restrict__ accF, const float* __restrict__ accR, int n,
                               ReducedMesh rm, const float* __restrict__ occ, int stride, int phase,
                               int row0, int cap, bf16* __restrict__ X, float* __restrict__ T) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = k * stride + phase;
  if (i >= n) return;
  const int row = row0 + k;
  if (row >= cap) return;
  float f[CL_K0];
  const float S = features(rm, occ, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], f);
  for (int c = 0; c < CL_K0; ++c) X[(size_t)row * CL_K0 + c] = __float2bfloat16_rn(f[c]);
  const float inv = S > 0.f ? 1.0f / (S * rm.out_scale) : 0.f;
  for (int a = 0; a < 3; ++a) T[(size_t)row * 4 + a] = (accF[3 * i + a] - accR[3 * i + a]) * inv;
  T[(size_t)row * 4 + 3] = 0.f;
}

// features of given rows (host test support), float output
__global__ void features_kernel(const float* __restrict__ pos, int n, ReducedMesh rm,
                                const float* __restrict__ occ, float* __restrict__ out,
                                float* __restrict__ spatch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float f[CL_K0];
  const float S = features(rm, occ, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], f);
  for (int c = 0; c < CL_IN; ++c) out[(size_t)i * CL_IN + c] = f[c];
  spatch[i] = S;
}

// MLP on given inputs (test support): X float [n][67] -> Y [n][3]
__global__ void __launch_bounds__(CL_THREADS) mlp_eval_kernel(const float* __restrict__ X, int n,
                                                              const bf16* __restrict__ img,
                                                              const float* __restrict__ params,
                                                              float* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemMLP& s = *reinterpret_cast<SmemMLP*>(smem_raw);
  bf16* xs_all = reinterpret_cast<bf16*>(smem_raw + sizeof(SmemMLP));
  load_mlp_smem(s, img, params);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  bf16* xs = xs_all + warp * 16 * S80;
  const int tiles = (n + 15) / 16;
  for (int tile = blockIdx.x * CL_WARPS + warp; tile < tiles; tile += gridDim.x * CL_WARPS) {
    const int r0 = tile * 16;
    for (int e = lane; e < 16 * CL_K0; e += 32) {
      const int r = e / CL_K0, c = e % CL_K0, i = r0 + r;
      xs[r * S80 + c] = __float2bfloat16_rn(i < n && c < CL_IN ? X[(size_t)i * CL_IN + c] : 0.f);
    }
    __syncwarp();
    u32 x0[5][4];
#pragma unroll
    for (int ks = 0; ks < 5; ++ks) ld_a(x0[ks], xs, S80, 0, ks * 16, g, t);
    float y[4], z1[8][4], z2[8][4], z3[8][4];
    u32 a1[4][4], a2[4][4], a3[4][4];
    mlp_forward<false>(s, x0, y, z1, z2, z3, a1, a2, a3, g, t);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = g + 8 * (e >> 1), o = 2 * t + (e & 1), i = r0 + r;
      if (i < n && o < 3) Y[(size_t)i * 3 + o] = y[e];
    }
    __syncwarp();
  }
}

constexpr size_t kInferSmem = sizeof(SmemMLP) + CL_WARPS * 16 * S80 * sizeof(bf16) + CL_WARPS * 16 * sizeof(float);
constexpr size_t kTrainSmem = sizeof(SmemMLP) + CL_WARPS * sizeof(TrainSmemWarp);

static int configure_closure_kernels() {
  static bool done = false;
  if (done) return PMGB_OK;
  PMGB_CUDA_TRY(cudaFuncSetAttribute(closure_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
  PMGB_CUDA_TRY(cudaFuncSetAttribute(closure_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
  PMGB_CUDA_TRY(cudaFuncSetAttribute(mlp_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
  done = true;
  return PMGB_OK;
}

// Host-side parameter initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and
// biases of each layer (fan_in counts real inputs: 67 for the first layer), zero padding.
static std::vector<float> init_params(unsigned long long seed) {
  std::vector<float> p(CL_NPARAM, 0.f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off_w, int rows, int cols_real, int cols, int off_b, int rows_real, int fan_in) {
    std::uniform_real_distribution<float> u(-1.0f / std::sqrt((float)fan_in), 1.0f / std::sqrt((float)fan_in));
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c)
        p[off_w + r * cols + c] = (r < rows_real && c < cols_real) ? u(rng) : 0.f;
    for (int r = 0; r < rows; ++r) p[off_b + r] = r < rows_real ? u(rng) : 0.f;
  };
  fill(OFF_W1, CL_H, CL_IN, CL_K0, OFF_B1, CL_H, CL_IN);
  fill(OFF_W2, CL_H, CL_H, CL_H, OFF_B2, CL_H, CL_H);
  fill(OFF_W3, CL_H, CL_H, CL_H, OFF_B3, CL_H, CL_H);
  fill(OFF_W4, CL_NO, CL_H, CL_H, OFF_B4, 3, CL_H);
  return p;
}

}  // namespace pmgb

using namespace pmgb;

struct pmgb_closure {
  pmgb_pm* pm = nullptr;
  pmgb_p3m* full = nullptr;     // plain full-cutoff P3M (judge, fallback, training targets)
  pmgb_p3m* reduced = nullptr;  // reduced-cutoff pair pass
  int mode = 0;                 // PMGB_CLOSURE_FULL / _LEARNED / _REDUCED_ONLY
  ReducedMesh rm{};
  int ncells = 0;
  u64* occ_fx = nullptr;
  float* occ = nullptr;
  float* params = nullptr;      // fp32 master
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* grad = nullptr;
  float* gw = nullptr;          // per-warp partial gradients
  float* lossw = nullptr;
  float* loss = nullptr;
  bf16* img = nullptr;
  int gw_warps = 0;
  bf16* X = nullptr;            // training inputs
  float* T = nullptr;           // training targets (4 per row)
  int cap = 0, count = 0;
  float* accF = nullptr;        // scratch: 3n floats each
  float* accR = nullptr;
  int adam_t = 0;
  unsigned long long seed = 0;
};

namespace pmgb {
int p3m_create_internal(pmgb_pm* pm, const pmgb_p3m_config* cfg, pmgb_p3m** out, bool attach);

static int occupancy(pmgb_closure* c, const float4* pm, int n) {
  cudaStream_t st = c->pm->st;
  occ_deposit_kernel<<<(n + 255) / 256, 256, 0, st>>>(pm, n, c->rm, c->occ_fx);
  occ_finalize_kernel<<<(c->ncells + 255) / 256, 256, 0, st>>>(c->occ_fx, c->occ, c->ncells, c->rm.fx_inv);
  PMGB_LAUNCH_CHECK();
  count_launches(2);
  return PMGB_OK;
}

int closure_apply(pmgb_pm* h) {
  pmgb_closure* c = h->closure;
  if (!c || c->mode != PMGB_CLOSURE_LEARNED) return PMGB_OK;
  int rc = occupancy(c, h->pm[h->cur], h->n);
  if (rc) return rc;
  const int tiles = (h->n + 15) / 16;
  const int blocks = std::min((tiles + CL_WARPS - 1) / CL_WARPS, h->num_sms * 4);
  if (blocks > 0) {
    closure_infer_kernel<<<blocks, CL_THREADS, kInferSmem, h->st>>>(h->pm[h->cur], h->n, c->rm, c->occ, c->img,
                                                                    c->params, h->acc_pm, h->flags);
    PMGB_LAUNCH_CHECK();
    count_launches(1);
  }
  return PMGB_OK;
}

static void set_mode(pmgb_closure* c, int mode) {
  c->mode = mode;
  pmgb_pm* h = c->pm;
  h->p3m = mode == PMGB_CLOSURE_FULL ? c->full : c->reduced;
  h->closure = c;
}

// force at the current positions in `mode`, accelerations to dst (3n floats, original order)
static int force_into(pmgb_closure* c, int mode, float* dst) {
  pmgb_pm* h = c->pm;
  const int keep = c->mode;
  set_mode(c, mode);
  int rc = pmgb_pm_method_step(h);
  set_mode(c, keep);
  if (rc) return rc;
  const size_t n = (size_t)h->n;
  rc = launch_unpack(h->pm[h->cur], h->vi[h->cur], h->acc, h->n, h->cfg.H, h->cfg.DT, 0, h->stage,
                     h->stage + 3 * n, h->stage + 6 * n, h->st);
  if (rc) return rc;
  PMGB_CUDA_TRY(cudaMemcpyAsync(dst, h->stage + 6 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToDevice, h->st));
  return PMGB_OK;
}

}  // namespace pmgb

template <typename T>
static int cl_alloc(T** p, size_t count) {
  if (cudaMalloc((void**)p, count * sizeof(T) + 16) != cudaSuccess) {
    set_error("cudaMalloc failed (closure)");
    return PMGB_ENOMEM;
  }
  return PMGB_OK;
}

extern "C" {

int pmgb_closure_create(pmgb_pm* pm, const pmgb_p3m_config* full_cfg, float reduced_cutoff,
                        int capacity, unsigned long long seed, pmgb_closure** out) {
  if (!pm || !full_cfg || !out) return set_error("null argument"), PMGB_EINVAL;
  *out = nullptr;
  if (pm->p3m || pm->closure) return set_error("the PM handle already has a P3M handle"), PMGB_EINVAL;
  if (!(reduced_cutoff > 0) || !(reduced_cutoff < full_cfg->cutoff))
    return set_error("reduced cutoff must be in (0, cutoff)"), PMGB_EINVAL;
  int rc = configure_closure_kernels();
  if (rc) return rc;
  pmgb_closure* c = new pmgb_closure();
  c->pm = pm;
  c->seed = seed;
  pmgb_p3m_config rcfg = *full_cfg;
  rcfg.cutoff = reduced_cutoff;
  if ((rc = p3m_create_internal(pm, full_cfg, &c->full, false)) ||
      (rc = p3m_create_internal(pm, &rcfg, &c->reduced, false))) {
    pmgb_closure_destroy(c);
    return rc;
  }
  const ChainDims& cd = c->reduced->cd;
  c->rm.Mx = cd.Mx;
  c->rm.My = cd.My;
  c->rm.Mz = cd.Mz;
  c->rm.HCx = cd.HCx;
  c->rm.HCy = cd.HCy;
  c->rm.HCz = cd.HCz;
  c->rm.fx_scale = pm->sp.fx_scale;
  c->rm.fx_inv = pm->sp.fx_inv;
  const float hc = std::min(cd.HCx, std::min(cd.HCy, cd.HCz));
  c->rm.out_scale = 1.0f / (4.0f * std::numbers::pi_v<float> * hc * hc);
  c->ncells = cd.Mx * cd.My * cd.Mz;
  c->cap = std::max(capacity, 0);
  const size_t n = (size_t)std::max(pm->n, 1);
  c->gw_warps = 4096 / 16;  // largest batch
  if ((rc = cl_alloc(&c->occ_fx, c->ncells)) || (rc = cl_alloc(&c->occ, c->ncells)) ||
      (rc = cl_alloc(&c->params, CL_NPARAM)) || (rc = cl_alloc(&c->adam_m, CL_NPARAM)) ||
      (rc = cl_alloc(&c->adam_v, CL_NPARAM)) || (rc = cl_alloc(&c->grad, CL_NPARAM)) ||
      (rc = cl_alloc(&c->gw, (size_t)c->gw_warps * CL_NPARAM)) || (rc = cl_alloc(&c->lossw, c->gw_warps)) ||
      (rc = cl_alloc(&c->loss, 1)) || (rc = cl_alloc(&c->img, IMG_SIZE)) ||
      (rc = cl_alloc(&c->X, (size_t)std::max(c->cap, 1) * CL_K0)) ||
      (rc = cl_alloc(&c->T, (size_t)std::max(c->cap, 1) * 4)) || (rc = cl_alloc(&c->accF, 3 * n)) ||
      (rc = cl_alloc(&c->accR, 3 * n))) {
    pmgb_closure_destroy(c);
    return rc;
  }
  std::vector<float> p0 = init_params(seed);
  cudaStream_t st = pm->st;
  if (cudaMemsetAsync(c->occ_fx, 0, c->ncells * sizeof(u64), st) != cudaSuccess ||
      cudaMemcpyAsync(c->params, p0.data(), CL_NPARAM * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(c->adam_m, 0, CL_NPARAM * sizeof(float), st) != cudaSuccess ||
      cudaMemsetAsync(c->adam_v, 0, CL_NPARAM * sizeof(float), st) != cudaSuccess) {
    pmgb_closure_destroy(c);
    return set_error("closure initialisation failed"), PMGB_ECUDA;
  }
  image_kernel<<<64, 256, 0, st>>>(c->params, c->img);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    pmgb_closure_destroy(c);
    return set_error("closure initialisation failed"), PMGB_ECUDA;
  }
  set_mode(c, PMGB_CLOSURE_FULL);
  pm->since_sort = 1 << 30;
  *out = c;
  return PMGB_OK;
}

int pmgb_closure_destroy(pmgb_closure* c) {
  if (!c) return PMGB_OK;
  if (c->pm) {
    cudaStreamSynchronize(c->pm->st);
    if (c->pm->closure == c) {
      c->pm->closure = nullptr;
      c->pm->p3m = nullptr;
    }
  }
  if (c->full) pmgb_p3m_destroy(c->full);
  if (c->reduced) pmgb_p3m_destroy(c->reduced);
  void* ptrs[] = {c->occ_fx, c->occ, c->params, c->adam_m, c->adam_v, c->grad, c->gw, c->lossw,
                  c->loss, c->img, c->X, c->T, c->accF, c->accR};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete c;
  return PMGB_OK;
}

int pmgb_closure_set_mode(pmgb_closure* c, int mode) {
  if (!c || mode < PMGB_CLOSURE_FULL || mode > PMGB_CLOSURE_REDUCED_ONLY)
    return set_error("bad closure mode"), PMGB_EINVAL;
  set_mode(c, mode);
  return PMGB_OK;
}

int pmgb_closure_get_mode(pmgb_closure* c, int* mode) {
  if (!c || !mode) return set_error("null argument"), PMGB_EINVAL;
  *mode = c->mode;
  return PMGB_OK;
}

int pmgb_closure_collect(pmgb_closure* c, int stride, int* total) {
  if (!c) return set_error("null handle"), PMGB_EINVAL;
  if (stride < 1) stride = 1;
  pmgb_pm* h = c->pm;
  int rc = force_into(c, PMGB_CLOSURE_FULL, c->accF);
  if (rc) return rc;
  rc = force_into(c, PMGB_CLOSURE_REDUCED_ONLY, c->accR);
  if (rc) return rc;
  // positions (code units, original order) are in the staging buffer after force_into
  rc = occupancy(c, h->pm[h->cur], h->n);
  if (rc) return rc;
  const int phase = (int)(c->seed + c->count) % stride;
  const int rows = (h->n - phase + stride - 1) / stride;
  if (rows > 0 && c->count < c->cap) {
    collect_kernel<<<(rows + 255) / 256, 256, 0, h->st>>>(h->stage, c->accF, c->accR, h->n, c->rm, c->occ, stride,
                                                          phase, c->count, c->cap, c->X, c->T);
    PMGB_LAUNCH_CHECK();
    count_launches(1);
    c->count = std::min(c->cap, c->count + rows);
  }
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  if (total) *total = c->count;
  return PMGB_OK;
}

int pmgb_closure_train(pmgb_closure* c, int epochs, int batch, float lr, float* final_loss) {
  if (!c) return set_error("null handle"), PMGB_EINVAL;
  if (batch < 16 || batch > 4096 || batch % 64) return set_error("batch must be a multiple of 64 in [64, 4096]"), PMGB_EINVAL;
  if (c->count < batch) return set_error("not enough training rows"), PMGB_EINVAL;
  cudaStream_t st = c->pm->st;
  int* perm = nullptr;
  PMGB_CUDA_TRY(cudaMalloc(&perm, (size_t)c->count * sizeof(int)));
  std::vector<int> hp(c->count);
  std::mt19937_64 rng(c->seed * 7919 + 17);
  const int steps_per_epoch = c->count / batch;
  const int total_steps = epochs * steps_per_epoch;
  float last = 0.f;
  double epoch_loss = 0.0;
  int step = 0;
  for (int e = 0; e < epochs; ++e) {
    for (int i = 0; i < c->count; ++i) hp[i] = i;
    std::shuffle(hp.begin(), hp.end(), rng);
    if (cudaMemcpyAsync(perm, hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      cudaFree(perm);
      return set_error("permutation upload failed"), PMGB_ECUDA;
    }
    epoch_loss = 0.0;
    for (int b = 0; b < steps_per_epoch; ++b, ++step) {
      const int nw = batch / 16;
      closure_train_kernel<<<nw / CL_WARPS, CL_THREADS, kTrainSmem, st>>>(
          c->X, c->T, perm, b * batch, batch, 1.0f / batch, c->img, c->params, c->gw, c->lossw);
      grad_reduce_kernel<<<(CL_NPARAM + 255) / 256, 256, 0, st>>>(c->gw, nw, c->grad, c->lossw, c->loss);
      ++c->adam_t;
      // cosine decay to 5% of lr
      const float frac = total_steps > 1 ? (float)step / (float)(total_steps - 1) : 1.f;
      const float lr_t = lr * (0.05f + 0.95f * 0.5f * (1.0f + std::cos(std::numbers::pi_v<float> * frac)));
      const float b1 = 0.9f, b2 = 0.999f;
      adam_kernel<<<(CL_NPARAM + 255) / 256, 256, 0, st>>>(c->params, c->adam_m, c->adam_v, c->grad, lr_t, b1, b2,
                                                           1e-8f, 1.f - std::pow(b1, (float)c->adam_t),
                                                           1.f - std::pow(b2, (float)c->adam_t));
      image_kernel<<<64, 256, 0, st>>>(c->params, c->img);
      count_launches(4);
      if (b == steps_per_epoch - 1 || b % 64 == 0) {
        float l = 0.f;
        cudaMemcpyAsync(&l, c->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        last = l / batch;
      }
    }
  }
  cudaError_t err = cudaStreamSynchronize(st);
  cudaFree(perm);
  if (err != cudaSuccess) return set_error(std::string("training: ") + cudaGetErrorString(err)), PMGB_ECUDA;
  if (final_loss) *final_loss = last;
  return PMGB_OK;
}

int pmgb_closure_get_params(pmgb_closure* c, float* params, int count) {
  if (!c || !params || count != CL_NPARAM) return set_error("params buffer must hold pmgb_closure_param_count() floats"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaMemcpyAsync(params, c->params, CL_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, c->pm->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(c->pm->st));
  return PMGB_OK;
}

int pmgb_closure_set_params(pmgb_closure* c, const float* params, int count) {
  if (!c || !params || count != CL_NPARAM) return set_error("params buffer must hold pmgb_closure_param_count() floats"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaMemcpyAsync(c->params, params, CL_NPARAM * sizeof(float), cudaMemcpyHostToDevice, c->pm->st));
  image_kernel<<<64, 256, 0, c->pm->st>>>(c->params, c->img);
  PMGB_LAUNCH_CHECK();
  PMGB_CUDA_TRY(cudaStreamSynchronize(c->pm->st));
  return PMGB_OK;
}

int pmgb_closure_param_count(void) { return CL_NPARAM; }

// median relative error of the closure force vs the full-cutoff P3M force, over every
// `stride`-th particle, at the current positions
int pmgb_closure_judge(pmgb_closure* c, int stride, float* median_rel_err) {
  if (!c || !median_rel_err) return set_error("null argument"), PMGB_EINVAL;
  if (stride < 1) stride = 1;
  pmgb_pm* h = c->pm;
  int rc = force_into(c, PMGB_CLOSURE_LEARNED, c->accR);
  if (rc) return rc;
  rc = force_into(c, PMGB_CLOSURE_FULL, c->accF);
  if (rc) return rc;
  const size_t n = (size_t)h->n;
  std::vector<float> a(3 * n), b(3 * n);
  PMGB_CUDA_TRY(cudaMemcpyAsync(a.data(), c->accR, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(b.data(), c->accF, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  std::vector<float> e;
  for (size_t i = 0; i < n; i += (size_t)stride) {
    const double dx = a[3 * i] - b[3 * i], dy = a[3 * i + 1] - b[3 * i + 1], dz = a[3 * i + 2] - b[3 * i + 2];
    const double nb = std::sqrt((double)b[3 * i] * b[3 * i] + (double)b[3 * i + 1] * b[3 * i + 1] +
                                (double)b[3 * i + 2] * b[3 * i + 2]);
    if (nb > 0) e.push_back((float)(std::sqrt(dx * dx + dy * dy + dz * dz) / nb));
  }
  if (e.empty()) {
    *median_rel_err = 0.f;
    return PMGB_OK;
  }
  std::nth_element(e.begin(), e.begin() + e.size() / 2, e.end());
  *median_rel_err = e[e.size() / 2];
  return PMGB_OK;
}

// Runs n_steps loop iterations (pmgb_pm_advance) in the learned mode with the judge every
// judge_interval steps (0 = never): if its median relative error exceeds `bound`, the rest of
// the run uses plain full-cutoff P3M (*fallback_step = the step, else -1).
int pmgb_closure_run(pmgb_closure* c, int n_steps, float bound, int judge_interval,
                     int judge_stride, int* steps_done, int* fallback_step, float* device_ms) {
  if (!c) return set_error("null handle"), PMGB_EINVAL;
  if (fallback_step) *fallback_step = -1;
  float total_ms = 0.f;
  int done = 0;
  for (int s = 0; s < n_steps; ++s) {
    if (c->mode == PMGB_CLOSURE_LEARNED && judge_interval > 0 && s % judge_interval == 0) {
      float err = 0.f;
      int rc = pmgb_closure_judge(c, judge_stride, &err);
      if (rc) return rc;
      if (err > bound) {
        set_mode(c, PMGB_CLOSURE_FULL);
        if (fallback_step) *fallback_step = s;
      }
    }
    float ms = 0.f;
    int d = 0;
    int rc = pmgb_pm_advance(c->pm, 1, &d, &ms);
    total_ms += ms;
    if (rc == PMGB_EESCAPED) {
      if (steps_done) *steps_done = done;
      if (device_ms) *device_ms = total_ms;
      return rc;
    }
    if (rc) return rc;
    ++done;
  }
  if (steps_done) *steps_done = done;
  if (device_ms) *device_ms = total_ms;
  return PMGB_OK;
}

// test support: features (67 floats per particle, original order) and patch masses
int pmgb_closure_features(pmgb_closure* c, float* x, float* spatch) {
  if (!c || !x || !spatch) return set_error("null argument"), PMGB_EINVAL;
  pmgb_pm* h = c->pm;
  const size_t n = (size_t)h->n;
  int rc = launch_unpack(h->pm[h->cur], h->vi[h->cur], h->acc, h->n, h->cfg.H, h->cfg.DT, 0, h->stage,
                         h->stage + 3 * n, h->stage + 6 * n, h->st);
  if (rc) return rc;
  rc = occupancy(c, h->pm[h->cur], h->n);
  if (rc) return rc;
  float *dx = nullptr, *ds = nullptr;
  PMGB_CUDA_TRY(cudaMalloc(&dx, n * CL_IN * sizeof(float) + 16));
  PMGB_CUDA_TRY(cudaMalloc(&ds, n * sizeof(float) + 16));
  features_kernel<<<((int)n + 255) / 256, 256, 0, h->st>>>(h->stage, h->n, c->rm, c->occ, dx, ds);
  cudaMemcpyAsync(x, dx, n * CL_IN * sizeof(float), cudaMemcpyDeviceToHost, h->st);
  cudaMemcpyAsync(spatch, ds, n * sizeof(float), cudaMemcpyDeviceToHost, h->st);
  cudaError_t err = cudaStreamSynchronize(h->st);
  cudaFree(dx);
  cudaFree(ds);
  if (err != cudaSuccess) return set_error(cudaGetErrorString(err)), PMGB_ECUDA;
  return PMGB_OK;
}

int pmgb_closure_scales(pmgb_closure* c, float* out_scale, int* dims3) {
  if (!c) return set_error("null handle"), PMGB_EINVAL;
  if (out_scale) *out_scale = c->rm.out_scale;
  if (dims3) {
    dims3[0] = c->rm.Mx;
    dims3[1] = c->rm.My;
    dims3[2] = c->rm.Mz;
  }
  return PMGB_OK;
}

// test support: the MLP (our kernels) on host inputs; and the training gradients of one batch
int pmgb_mlp_eval(const float* params, int n, const float* x, float* y) {
  if (!params || (n > 0 && (!x || !y))) return set_error("null argument"), PMGB_EINVAL;
  int rc = configure_closure_kernels();
  if (rc) return rc;
  float *dp = nullptr, *dx = nullptr, *dy = nullptr;
  bf16* img = nullptr;
  const size_t nn = (size_t)std::max(n, 1);
  PMGB_CUDA_TRY(cudaMalloc(&dp, CL_NPARAM * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&img, IMG_SIZE * sizeof(bf16)));
  PMGB_CUDA_TRY(cudaMalloc(&dx, nn * CL_IN * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&dy, nn * 3 * sizeof(float)));
  cudaMemcpy(dp, params, CL_NPARAM * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x, (size_t)n * CL_IN * sizeof(float), cudaMemcpyHostToDevice);
  image_kernel<<<64, 256>>>(dp, img);
  mlp_eval_kernel<<<std::max(1, std::min(1024, (n + 63) / 64)), CL_THREADS, kInferSmem>>>(dx, n, img, dp, dy);
  cudaMemcpy(y, dy, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaError_t err = cudaDeviceSynchronize();
  cudaFree(dp);
  cudaFree(img);
  cudaFree(dx);
  cudaFree(dy);
  if (err != cudaSuccess) return set_error(cudaGetErrorString(err)), PMGB_ECUDA;
  return PMGB_OK;
}

int pmgb_mlp_gradients(const float* params, int n, const float* x, const float* t, float* grad,
                       float* loss) {
  if (!params || !x || !t || !grad || n < 16 || n > 4096 || n % 64)
    return set_error("n must be a multiple of 64 in [64, 4096]"), PMGB_EINVAL;
  int rc = configure_closure_kernels();
  if (rc) return rc;
  float *dp = nullptr, *dt = nullptr, *gw = nullptr, *g = nullptr, *lw = nullptr, *l = nullptr;
  bf16 *img = nullptr, *dx = nullptr;
  int* perm = nullptr;
  const int nw = n / 16;
  PMGB_CUDA_TRY(cudaMalloc(&dp, CL_NPARAM * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&img, IMG_SIZE * sizeof(bf16)));
  PMGB_CUDA_TRY(cudaMalloc(&dx, (size_t)n * CL_K0 * sizeof(bf16)));
  PMGB_CUDA_TRY(cudaMalloc(&dt, (size_t)n * 4 * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&gw, (size_t)nw * CL_NPARAM * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&g, CL_NPARAM * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&lw, nw * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&l, sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&perm, n * sizeof(int)));
  std::vector<bf16> hx((size_t)n * CL_K0);
  std::vector<float> ht((size_t)n * 4, 0.f);
  std::vector<int> hp(n);
  for (int i = 0; i < n; ++i) {
    hp[i] = i;
    for (int c = 0; c < CL_K0; ++c) hx[(size_t)i * CL_K0 + c] = __float2bfloat16(c < CL_IN ? x[(size_t)i * CL_IN + c] : 0.f);
    for (int o = 0; o < 3; ++o) ht[(size_t)i * 4 + o] = t[(size_t)i * 3 + o];
  }
  cudaMemcpy(dp, params, CL_NPARAM * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(dx, hx.data(), hx.size() * sizeof(bf16), cudaMemcpyHostToDevice);
  cudaMemcpy(dt, ht.data(), ht.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(perm, hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice);
  image_kernel<<<64, 256>>>(dp, img);
  closure_train_kernel<<<nw / CL_WARPS, CL_THREADS, kTrainSmem>>>(dx, dt, perm, 0, n, 1.0f / n, img, dp, gw, lw);
  grad_reduce_kernel<<<(CL_NPARAM + 255) / 256, 256>>>(gw, nw, g, lw, l);
  cudaMemcpy(grad, g, CL_NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
  float lh = 0.f;
  cudaMemcpy(&lh, l, sizeof(float), cudaMemcpyDeviceToHost);
  cudaError_t err = cudaDeviceSynchronize();
  if (loss) *loss = lh / n;
  void* ptrs[] = {dp, dt, gw, g, lw, l, img, dx, perm};
  for (void* p : ptrs) cudaFree(p);
  if (err != cudaSuccess) return set_error(cudaGetErrorString(err)), PMGB_ECUDA;
  return PMGB_OK;
}

}  // extern "C"
