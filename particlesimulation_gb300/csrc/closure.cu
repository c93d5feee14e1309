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
//                 accumulation.  Inference: tcgen05.mma from shared memory into TMEM, 128
//                 particles per CTA (the tcgen05 forward below).  Training (forward,
//                 backward): tcgen05.mma too, 128 rows per CTA, pre-activations kept in TMEM
//                 and the weight gradients as M = 128 products over the batch tile
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
// BF16 image of the weights (rows out x in, padded strides) and of the transposes the backward
// pass multiplies by; the kernels copy it into their canonical shared-memory operands
constexpr int S80 = 88, S64 = 72;
constexpr int IMG_W1 = 0, IMG_W2 = IMG_W1 + CL_H * S80, IMG_W3 = IMG_W2 + CL_H * S64,
              IMG_W4 = IMG_W3 + CL_H * S64, IMG_W2T = IMG_W4 + CL_NO * S64,
              IMG_W3T = IMG_W2T + CL_H * S64, IMG_SIZE = IMG_W3T + CL_H * S64;  // bf16 elements

// ------------------------------------------------------------------ helpers -----------
__device__ __forceinline__ u32 pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<u32*>(&v);
}
__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
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

// ------------------------------------------------------------------ tcgen05 forward --
// Inference runs on the 5th-generation tensor cores: a CTA of 128 threads takes tiles of 128
// particles (thread r = row r = TMEM lane r = the accumulator row of an M = 128 MMA).  Per
// layer one thread issues tcgen05.mma.kind::f16 (BF16 operands from shared memory, FP32
// accumulator in 64 TMEM columns) over the K slices of 16 and commits to an mbarrier; every
// thread then reads its row from TMEM (tcgen05.ld 32x32b), adds the bias, applies GELU and
// writes the BF16 activations back to shared memory as the next layer's A operand.  The output
// layer is padded to N = 16 (M = 128 takes N in multiples of 16).  Operands are in the
// no-swizzle K-major layout: 8-row x 16-byte core matrices, the core matrix of row group g and
// K group j at j * kstride + g * 128 bytes; the matrix descriptor's leading byte offset is the
// K-group stride, the stride byte offset the row-group stride.  Every wait on the mbarrier is
// bounded (1 s of %globaltimer, and a poll count); a wait that gives up sets err[0], the thread
// waits no more and thread 0 issues no more MMAs, while the barriers stay where they are, so
// the kernel reaches its end (and frees its TMEM) and the host reports PMGB_ETIMEOUT.
constexpr int TC_ROWS = 128;
constexpr int TC_THREADS = 128;
constexpr int TC_N4 = 16;                   // output layer, padded
constexpr int TC_COLS = 64;                 // TMEM columns (power of two >= 32)
constexpr u32 TC_KX = TC_ROWS * 16;         // K-group stride of the 128-row A operands (bytes)
constexpr u32 TC_KW = CL_H * 16;            // K-group stride of the 64-row weight operands
constexpr u32 TC_KW4 = TC_N4 * 16;          // K-group stride of the output layer's weights
constexpr int TC_WAIT_SPINS = 1 << 24;      // backstop of an mbarrier wait's polls
constexpr unsigned long long TC_WAIT_NS = 1000000000ull;  // bound of an mbarrier wait: 1 s

struct TcSmem {
  alignas(16) bf16 w1[CL_H * CL_K0];
  alignas(16) bf16 w2[CL_H * CL_H];
  alignas(16) bf16 w3[CL_H * CL_H];
  alignas(16) bf16 w4[TC_N4 * CL_H];
  alignas(16) bf16 x[TC_ROWS * CL_K0];     // layer-1 inputs
  alignas(16) bf16 h[TC_ROWS * CL_H];      // hidden activations (one layer at a time)
  float bias[3 * CL_H + TC_N4];
  float spatch[TC_ROWS];
  u64 mbar;
  u32 tmem;
};

__device__ __forceinline__ u32 smem_addr(const void* p) { return (u32)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in the canonical layout with K-group stride kstride
__device__ __forceinline__ u32 canon(int r, int k, u32 kstride) {
  return (u32)(k >> 3) * kstride + (u32)(r >> 3) * 128u + (u32)(r & 7) * 16u + (u32)(k & 7) * 2u;
}

// shared-memory matrix descriptor: start, leading byte offset (K-group stride), stride byte
// offset (row-group stride, 128), the fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ u64 tc_desc(u32 saddr, u32 kstride) {
  return (u64)((saddr >> 4) & 0x3FFFu) | ((u64)((kstride >> 4) & 0x3FFFu) << 16) |
         ((u64)(128u >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr u32 tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((u32)(N >> 3) << 17) | ((u32)(M >> 4) << 24);
}

// D (TMEM) = A x B^T over nks K slices of 16 (one thread; no fence, no commit)
__device__ __forceinline__ void tc_mmas(u32 tmem, u32 a, u32 akstride, u32 b, u32 bkstride, int nks,
                                        u32 idesc) {
  for (int ks = 0; ks < nks; ++ks) {
    const u64 ad = tc_desc(a + 2u * ks * akstride, akstride);
    const u64 bd = tc_desc(b + 2u * ks * bkstride, bkstride);
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(ks > 0 ? 1u : 0u) : "memory");
  }
}

// the mbarrier completes a phase once every MMA this thread issued so far has finished
__device__ __forceinline__ void tc_commit(u32 mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(mbar) : "memory");
}

// D (TMEM) = A x B^T over nks K slices of 16, then a commit to the mbarrier (one thread)
__device__ __forceinline__ void tc_mma_layer(u32 tmem, u32 a, u32 akstride, u32 b, u32 bkstride,
                                             int nks, u32 idesc, u32 mbar) {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  tc_mmas(tmem, a, akstride, b, bkstride, nks, idesc);
  tc_commit(mbar);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the mbarrier phase of the given parity, for at most TC_WAIT_NS nanoseconds and
// `spins` polls; false if it gave up.
__device__ __forceinline__ bool tc_wait(u32 mbar, u32 parity, int spins = TC_WAIT_SPINS) {
  u32 done = 0;
  const unsigned long long t0 = globaltimer_ns();
  for (int it = 0; it < spins && !done; ++it) {
    if ((it & 255) == 255 && globaltimer_ns() - t0 > TC_WAIT_NS) break;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  return done != 0;
}

// this thread's TMEM lane (its warp's 32-lane block), columns 0..63 / 0..15
__device__ __forceinline__ void tc_ld64(u32 taddr, float (&v)[64]) {
  u32 r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
      "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
      "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 64; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tc_ld16(u32 taddr, float (&v)[16]) {
  u32 r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// row r of a canonical operand from 8 K groups of 8 values (16-byte stores)
template <int KG>
__device__ __forceinline__ void tc_store_row(unsigned char* base, int r, u32 kstride, const float* v) {
#pragma unroll
  for (int j = 0; j < KG; ++j) {
    uint4 q;
    q.x = pack_bf16(v[8 * j + 0], v[8 * j + 1]);
    q.y = pack_bf16(v[8 * j + 2], v[8 * j + 3]);
    q.z = pack_bf16(v[8 * j + 4], v[8 * j + 5]);
    q.w = pack_bf16(v[8 * j + 6], v[8 * j + 7]);
    *reinterpret_cast<uint4*>(base + canon(r, 8 * j, kstride)) = q;
  }
}

// Prologue of a CTA: weights (from the BF16 image) and biases into shared memory, the
// mbarrier, 64 TMEM columns (warp 0).  Ends with a barrier.
__device__ void tc_setup(TcSmem& s, const bf16* __restrict__ img, const float* __restrict__ p) {
  unsigned char* w1 = reinterpret_cast<unsigned char*>(s.w1);
  unsigned char* w2 = reinterpret_cast<unsigned char*>(s.w2);
  unsigned char* w3 = reinterpret_cast<unsigned char*>(s.w3);
  unsigned char* w4 = reinterpret_cast<unsigned char*>(s.w4);
  for (int e = threadIdx.x; e < CL_H * CL_K0; e += blockDim.x) {
    const int n = e / CL_K0, k = e % CL_K0;
    *reinterpret_cast<bf16*>(w1 + canon(n, k, TC_KW)) = img[IMG_W1 + n * S80 + k];
  }
  for (int e = threadIdx.x; e < CL_H * CL_H; e += blockDim.x) {
    const int n = e / CL_H, k = e % CL_H;
    *reinterpret_cast<bf16*>(w2 + canon(n, k, TC_KW)) = img[IMG_W2 + n * S64 + k];
    *reinterpret_cast<bf16*>(w3 + canon(n, k, TC_KW)) = img[IMG_W3 + n * S64 + k];
  }
  for (int e = threadIdx.x; e < TC_N4 * CL_H; e += blockDim.x) {
    const int n = e / CL_H, k = e % CL_H;
    *reinterpret_cast<bf16*>(w4 + canon(n, k, TC_KW4)) =
        n < CL_NO ? img[IMG_W4 + n * S64 + k] : __float2bfloat16_rn(0.f);
  }
  for (int i = threadIdx.x; i < CL_H; i += blockDim.x) {
    s.bias[i] = p[OFF_B1 + i];
    s.bias[CL_H + i] = p[OFF_B2 + i];
    s.bias[2 * CL_H + i] = p[OFF_B3 + i];
  }
  for (int i = threadIdx.x; i < TC_N4; i += blockDim.x) s.bias[3 * CL_H + i] = i < CL_NO ? p[OFF_B4 + i] : 0.f;
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&s.mbar)) : "memory");
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(&s.tmem)), "r"(TC_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Forward pass of one tile whose inputs are in s.x: returns this thread's row of the output
// layer (3 values).  phase: the mbarrier parity of the next commit (advanced by 4).  live: false
// once one of this thread's waits gave up; from then on the thread waits no more (thread 0 also
// issues no more MMAs), so a failed launch ends within about one wait bound, err[0] set.
__device__ __forceinline__ void tc_forward(TcSmem& s, u32& phase, bool& live, int* __restrict__ err,
                                           float y[3]) {
  const u32 tmem = s.tmem;
  const u32 taddr = tmem + ((u32)(threadIdx.x & ~31) << 16);
  const u32 mbar = smem_addr(&s.mbar);
  const u32 xa = smem_addr(s.x), ha = smem_addr(s.h);
  const u32 wa[3] = {smem_addr(s.w1), smem_addr(s.w2), smem_addr(s.w3)};
  unsigned char* hb = reinterpret_cast<unsigned char*>(s.h);
  // inputs written by every thread: make them visible to the tensor cores
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
#pragma unroll 1
  for (int l = 0; l < 3; ++l) {
    if (threadIdx.x == 0 && live)
      tc_mma_layer(tmem, l == 0 ? xa : ha, TC_KX, wa[l], TC_KW, l == 0 ? CL_K0 / 16 : CL_H / 16,
                   tc_idesc(TC_ROWS, CL_H), mbar);
    if (live && !tc_wait(mbar, phase & 1u)) {
      live = false;
      atomicExch(err, 1);
    }
    ++phase;
    float z[64];
    tc_ld64(taddr, z);
    const float* b = s.bias + l * CL_H;
#pragma unroll
    for (int j = 0; j < 64; ++j) z[j] = gelu(z[j] + b[j]);
    tc_store_row<CL_H / 8>(hb, threadIdx.x, TC_KX, z);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (threadIdx.x == 0 && live)
    tc_mma_layer(tmem, ha, TC_KX, smem_addr(s.w4), TC_KW4, CL_H / 16, tc_idesc(TC_ROWS, TC_N4), mbar);
  if (live && !tc_wait(mbar, phase & 1u)) {
    live = false;
    atomicExch(err, 1);
  }
  ++phase;
  float o[16];
  tc_ld16(taddr, o);
  const float* b4 = s.bias + 3 * CL_H;
  y[0] = o[0] + b4[0];
  y[1] = o[1] + b4[1];
  y[2] = o[2] + b4[2];
  // the next tile rewrites s.x and TMEM only after every thread is past its loads
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
}

// Epilogue of a CTA: every thread is past its TMEM reads, warp 0 frees the columns.
__device__ __forceinline__ void tc_free(u32 tmem, u32 cols) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_teardown(TcSmem& s) { tc_free(s.tmem, TC_COLS); }

// ------------------------------------------------------------------ inference --------
// acc[i] += MLP(features(i)) * S * c, for the particles of this handle (sorted order).
__global__ void __launch_bounds__(TC_THREADS) closure_infer_kernel(
    const float4* __restrict__ pm, int n, ReducedMesh rm, const float* __restrict__ occ,
    const bf16* __restrict__ img, const float* __restrict__ params, float4* __restrict__ acc,
    const int* __restrict__ stop, int* __restrict__ err) {
  if (*stop) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TcSmem& s = *reinterpret_cast<TcSmem*>(smem_raw);
  tc_setup(s, img, params);
  unsigned char* xb = reinterpret_cast<unsigned char*>(s.x);
  u32 phase = 0;
  bool live = true;
  const int tiles = (n + TC_ROWS - 1) / TC_ROWS;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i = tile * TC_ROWS + threadIdx.x;
    float f[CL_K0];
    float S = 0.f;
    if (i < n) {
      const float4 p = pm[i];
      S = features(rm, occ, p.x, p.y, p.z, f);
    } else {
#pragma unroll
      for (int k = 0; k < CL_K0; ++k) f[k] = 0.f;
    }
    tc_store_row<CL_K0 / 8>(xb, threadIdx.x, TC_KX, f);
    float y[3];
    tc_forward(s, phase, live, err, y);
    if (i < n) {
      const float sc = S * rm.out_scale;
      float4 a = acc[i];
      a.x += y[0] * sc;
      a.y += y[1] * sc;
      a.z += y[2] * sc;
      acc[i] = a;
    }
  }
  tc_teardown(s);
}

// ------------------------------------------------------------------ training ---------
// Training runs on the tensor cores too: one CTA of 128 threads per 128 training rows (thread
// r = row r = TMEM lane r), every MMA with M = 128.  The forward pass is the inference one,
// except that each layer's pre-activations stay in their own TMEM columns (the backward pass
// reads them for GELU') and each layer's BF16 activations are also stored transposed (rows =
// features, K = the 128 rows of the batch tile) as the B operand of the next weight gradient.
// Backward, for layer l with input activations A (the features x for l = 1):
//   dW_l  (rows j = the layer's outputs, N = 80) = dZ_l^T (rows j, K = rows b) x A^T (rows i,
//         K = b).  Row 64 of the hidden A^T operands (row 67 of the input's) is all ones, so
//         column 64 (67) of the product is the bias gradient sum_b dZ_l[b][j]; rows j >= 64 of
//         dZ^T are zero and their products are not read
//   dA    (rows b, N = 64) = dZ_l (rows b, K = j) x W_l, the B operand being W_l^T (rows i,
//         K = j)
// and dZ = dA * GELU'(Z) per row in FP32, stored in BF16 both ways.  The output layer's dY (16
// columns, 3 non-zero) stands in for dZ_4.  TMEM columns (512 allocated):
//   Z1 0, Z2 64, Z3 128, Y 192 | dW4 256, dA3 336 | dW3 400, dA2 192 | dW2 256, dA1 336 | dW1 400
// (each region is reused only after every thread has read what it held).  The CTA's partial
// gradient goes to gw[cta][CL_NPARAM] and its loss to lossw[cta]; grad_reduce_kernel sums them
// in a fixed order.  Waits are bounded as in the inference kernel (err[0] on a timeout).
constexpr int TT_N = 80;                 // rows of the transposed activation operands
constexpr u32 TT_K = TT_N * 16;          // their K-group stride (K = the batch tile's rows)
constexpr u32 TD_K = TC_ROWS * 16;       // K-group stride of dZ^T (128 rows)
constexpr u32 TT_COLS = 512;

struct TcTrainSmem {
  alignas(16) bf16 w1[CL_H * CL_K0];
  alignas(16) bf16 w2[CL_H * CL_H];
  alignas(16) bf16 w3[CL_H * CL_H];
  alignas(16) bf16 w4[TC_N4 * CL_H];
  alignas(16) bf16 w2t[CL_H * CL_H];        // rows i, K = j: W2[j][i]
  alignas(16) bf16 w3t[CL_H * CL_H];
  alignas(16) bf16 w4t[CL_H * TC_N4];       // rows j, K = o: W4[o][j] (zero for o >= 8)
  alignas(16) bf16 x[TC_ROWS * CL_K0];      // rows b, K = input features
  alignas(16) bf16 h[TC_ROWS * CL_H];       // rows b, K = j: activations, then dZ
  alignas(16) bf16 dy[TC_ROWS * TC_N4];     // rows b, K = o
  alignas(16) bf16 xt[TT_N * TC_ROWS];      // rows = input features (ones at 67), K = b
  alignas(16) bf16 at[3][TT_N * TC_ROWS];   // rows = hidden features (ones at 64), K = b
  alignas(16) bf16 dzt[TC_ROWS * TC_ROWS];  // rows j (dY^T in rows 0..15, then dZ^T), K = b
  float bias[3 * CL_H + TC_N4];
  float lsum[TC_THREADS / 32];
  u64 mbar;
  u32 tmem;
};

// column b of a canonical operand whose K dimension is the batch row: rows 0..n-1 from v
template <int N>
__device__ __forceinline__ void tc_store_col(bf16* base, int b, u32 kstride, const float* v) {
  unsigned char* p = reinterpret_cast<unsigned char*>(base);
#pragma unroll
  for (int r = 0; r < N; ++r) *reinterpret_cast<bf16*>(p + canon(r, b, kstride)) = __float2bfloat16_rn(v[r]);
}

__device__ __forceinline__ void tc_put(bf16* base, int r, int k, u32 kstride, bf16 v) {
  *reinterpret_cast<bf16*>(reinterpret_cast<unsigned char*>(base) + canon(r, k, kstride)) = v;
}

// The training kernel's per-row work goes 16 columns at a time in loops that are not unrolled:
// the whole epilogue of a layer unrolled runs once per launch, so its straight-line code was
// always cold in the instruction cache (the kernel spent most of its time on instruction
// fetch).  Columns k0 .. k0 + 15 of row r of a canonical operand (two 16-byte stores):
__device__ __forceinline__ void tc_store_row16(bf16* base, int r, int k0, u32 kstride, const float (&v)[16]) {
  unsigned char* p = reinterpret_cast<unsigned char*>(base);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    uint4 q;
    q.x = pack_bf16(v[8 * j + 0], v[8 * j + 1]);
    q.y = pack_bf16(v[8 * j + 2], v[8 * j + 3]);
    q.z = pack_bf16(v[8 * j + 4], v[8 * j + 5]);
    q.w = pack_bf16(v[8 * j + 6], v[8 * j + 7]);
    *reinterpret_cast<uint4*>(p + canon(r, k0 + 8 * j, kstride)) = q;
  }
}
// rows r0 .. r0 + 15 of column b of a canonical operand whose K dimension is the batch row
__device__ __forceinline__ void tc_store_col16(bf16* base, int b, int r0, u32 kstride, const float (&v)[16]) {
  unsigned char* p = reinterpret_cast<unsigned char*>(base);
#pragma unroll
  for (int r = 0; r < 16; ++r) *reinterpret_cast<bf16*>(p + canon(r0 + r, b, kstride)) = __float2bfloat16_rn(v[r]);
}

__global__ void __launch_bounds__(TC_THREADS) closure_train_kernel(
    const bf16* __restrict__ X, const float* __restrict__ T, const int* __restrict__ perm,
    int batch_off, int batch, float inv_batch, const bf16* __restrict__ img,
    const float* __restrict__ params, float* __restrict__ gw, float* __restrict__ lossw,
    int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TcTrainSmem& s = *reinterpret_cast<TcTrainSmem*>(smem_raw);
  const int tid = threadIdx.x;
  const bf16 zero = __float2bfloat16_rn(0.f), one = __float2bfloat16_rn(1.f);
  // weights, their transposes, biases; the constant rows of the transposed operands
  for (int e = tid; e < CL_H * CL_K0; e += TC_THREADS)
    tc_put(s.w1, e / CL_K0, e % CL_K0, TC_KW, img[IMG_W1 + (e / CL_K0) * S80 + e % CL_K0]);
  for (int e = tid; e < CL_H * CL_H; e += TC_THREADS) {
    const int n = e / CL_H, k = e % CL_H;
    tc_put(s.w2, n, k, TC_KW, img[IMG_W2 + n * S64 + k]);
    tc_put(s.w3, n, k, TC_KW, img[IMG_W3 + n * S64 + k]);
    tc_put(s.w2t, n, k, TC_KW, img[IMG_W2T + n * S64 + k]);
    tc_put(s.w3t, n, k, TC_KW, img[IMG_W3T + n * S64 + k]);
  }
  for (int e = tid; e < TC_N4 * CL_H; e += TC_THREADS) {
    const int o = e / CL_H, j = e % CL_H;
    const bf16 v = o < CL_NO ? img[IMG_W4 + o * S64 + j] : zero;
    tc_put(s.w4, o, j, TC_KW4, v);
    tc_put(s.w4t, j, o, TC_KW, v);
  }
  for (int i = tid; i < CL_H; i += TC_THREADS) {
    s.bias[i] = params[OFF_B1 + i];
    s.bias[CL_H + i] = params[OFF_B2 + i];
    s.bias[2 * CL_H + i] = params[OFF_B3 + i];
  }
  for (int i = tid; i < TC_N4; i += TC_THREADS) s.bias[3 * CL_H + i] = i < CL_NO ? params[OFF_B4 + i] : 0.f;
  for (int e = tid; e < (TT_N - CL_IN) * TC_ROWS; e += TC_THREADS) {
    const int r = CL_IN + e / TC_ROWS;
    tc_put(s.xt, r, e % TC_ROWS, TT_K, r == CL_IN ? one : zero);
  }
  for (int e = tid; e < (TT_N - CL_H) * TC_ROWS; e += TC_THREADS) {
    const int r = CL_H + e / TC_ROWS;
#pragma unroll
    for (int l = 0; l < 3; ++l) tc_put(s.at[l], r, e % TC_ROWS, TT_K, r == CL_H ? one : zero);
  }
  for (int e = tid; e < TC_ROWS * TC_ROWS / 8; e += TC_THREADS)
    reinterpret_cast<uint4*>(s.dzt)[e] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&s.mbar)) : "memory");
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(&s.tmem)), "r"(TT_COLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // this thread's training row: BF16 features to x (rows b) and xt (column b)
  const int row = blockIdx.x * TC_ROWS + tid;
  const bool valid = row < batch;
  const int src = valid ? perm[batch_off + row] : 0;
  {
    const uint4* xr = reinterpret_cast<const uint4*>(X + (size_t)src * CL_K0);
#pragma unroll 1
    for (int j = 0; j < CL_K0 / 8; ++j) {
      const uint4 q = valid ? xr[j] : make_uint4(0u, 0u, 0u, 0u);
      *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(s.x) + canon(tid, 8 * j, TC_KX)) = q;
      const u32 w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int h = 0; h < 8; ++h) {  // the input features (rows < CL_IN) of column tid of xt
        const int r = 8 * j + h;
        if (r < CL_IN) {
          const u32 bits = (h & 1) ? (w[h >> 1] >> 16) : (w[h >> 1] & 0xFFFFu);
          tc_put(s.xt, r, tid, TT_K, __ushort_as_bfloat16((unsigned short)bits));
        }
      }
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  const u32 tmem = s.tmem;
  const u32 lane = tmem + ((u32)(tid & ~31) << 16);
  const u32 mbar = smem_addr(&s.mbar);
  const u32 xa = smem_addr(s.x), ha = smem_addr(s.h), dya = smem_addr(s.dy), dzta = smem_addr(s.dzt);
  const u32 xta = smem_addr(s.xt);
  const u32 ata[3] = {smem_addr(s.at[0]), smem_addr(s.at[1]), smem_addr(s.at[2])};
  const u32 wa[3] = {smem_addr(s.w1), smem_addr(s.w2), smem_addr(s.w3)};
  const bool issuer = tid == 0;
  u32 phase = 0;
  bool live = true;
  auto wait = [&]() {
    if (live && !tc_wait(mbar, phase & 1u)) {
      live = false;
      atomicExch(err, 1);
    }
    ++phase;
  };
  // shared-memory operands written by every thread, TMEM reads done: next MMAs may start
  auto publish = [&]() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  };
  float* G = gw + (size_t)blockIdx.x * CL_NPARAM;

  // ---- forward: Z_l into TMEM columns 64 l, activations to h (rows b) and at[l] (column b)
  constexpr u32 colZ[3] = {0u, 64u, 128u};
#pragma unroll 1
  for (int l = 0; l < 3; ++l) {
    if (issuer && live) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      tc_mmas(tmem + colZ[l], l == 0 ? xa : ha, TC_KX, wa[l], TC_KW, l == 0 ? CL_K0 / 16 : CL_H / 16,
              tc_idesc(TC_ROWS, CL_H));
      tc_commit(mbar);
    }
    wait();
#pragma unroll 1
    for (int c = 0; c < CL_H / 16; ++c) {
      float z[16];
      tc_ld16(lane + colZ[l] + 16u * c, z);
      const float* b = s.bias + l * CL_H + 16 * c;
#pragma unroll
      for (int j = 0; j < 16; ++j) z[j] = gelu(z[j] + b[j]);
      tc_store_row16(s.h, tid, 16 * c, TC_KX, z);
      tc_store_col16(s.at[l], tid, 16 * c, TT_K, z);
    }
    publish();
  }
  if (issuer && live) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tc_mmas(tmem + 192u, ha, TC_KX, smem_addr(s.w4), TC_KW4, CL_H / 16, tc_idesc(TC_ROWS, TC_N4));
    tc_commit(mbar);
  }
  wait();
  // ---- loss and dY = 2 (y - t) / batch
  {
    float o[16], dy[TC_N4];
    tc_ld16(lane + 192u, o);
    float loss = 0.f;
#pragma unroll
    for (int k = 0; k < TC_N4; ++k) dy[k] = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (valid) {
        const float diff = o[k] + s.bias[3 * CL_H + k] - T[(size_t)src * 4 + k];
        loss += diff * diff;
        dy[k] = 2.0f * diff * inv_batch;
      }
    }
    tc_store_row<TC_N4 / 8>(reinterpret_cast<unsigned char*>(s.dy), tid, TC_KX, dy);
    tc_store_col<TC_N4>(s.dzt, tid, TD_K, dy);
    for (int d = 16; d > 0; d >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, d);
    if ((tid & 31) == 0) s.lsum[tid >> 5] = loss;
  }
  publish();
  if (tid == 0) lossw[blockIdx.x] = (s.lsum[0] + s.lsum[1]) + (s.lsum[2] + s.lsum[3]);

  // rows j < rows of the weight gradient in TMEM columns col..col+79: W (kin columns) and the
  // bias (column bcol; a W column at bcol is the gradient of a zero input and is written 0)
  auto store_dw = [&](u32 col, int rows, int kin, int off_w, int off_b, int bcol) {
    if ((tid & ~31) < rows) {  // whole warps: tcgen05.ld is warp-wide
      float* gr = G + off_w + (size_t)tid * kin;
#pragma unroll 1
      for (int c = 0; c < TT_N / 16; ++c) {
        float a[16];
        tc_ld16(lane + col + 16u * c, a);
        if (tid < rows) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int i = 16 * c + j;
            if (i == bcol) G[off_b + tid] = a[j];
            if (i < kin) gr[i] = (i == bcol) ? 0.f : a[j];
          }
        }
      }
    }
  };
  // dZ = dA * GELU'(Z + b) of this row, to dzt (column b) and, when `rows`, to h (row b)
  auto make_dz = [&](u32 col_da, u32 col_z, const float* b, bool rows) {
#pragma unroll 1
    for (int c = 0; c < CL_H / 16; ++c) {
      float da[16], z[16];
      tc_ld16(lane + col_da + 16u * c, da);
      tc_ld16(lane + col_z + 16u * c, z);
#pragma unroll
      for (int j = 0; j < 16; ++j) da[j] *= gelu_grad(z[j] + b[16 * c + j]);
      if (rows) tc_store_row16(s.h, tid, 16 * c, TC_KX, da);
      tc_store_col16(s.dzt, tid, 16 * c, TD_K, da);
    }
  };
  auto issue_pair = [&](u32 col_dw, u32 bt, u32 col_da, u32 wt, int nks_da, u32 a_da, u32 akstride, u32 n_da) {
    if (issuer && live) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      tc_mmas(tmem + col_dw, dzta, TD_K, bt, TT_K, TC_ROWS / 16, tc_idesc(TC_ROWS, TT_N));
      if (nks_da > 0) tc_mmas(tmem + col_da, a_da, akstride, wt, TC_KW, nks_da, tc_idesc(TC_ROWS, n_da));
      tc_commit(mbar);
    }
    wait();
  };
  // ---- output layer: dW4 (+ db4), dA3 = dY W4
  issue_pair(256u, ata[2], 336u, smem_addr(s.w4t), TC_N4 / 16, dya, TC_KX, CL_H);
  store_dw(256u, CL_NO, CL_H, OFF_W4, OFF_B4, CL_H);
  make_dz(336u, colZ[2], s.bias + 2 * CL_H, true);
  publish();
  // ---- layer 3: dW3 (+ db3), dA2 = dZ3 W3
  issue_pair(400u, ata[1], 192u, smem_addr(s.w3t), CL_H / 16, ha, TC_KX, CL_H);
  store_dw(400u, CL_H, CL_H, OFF_W3, OFF_B3, CL_H);
  make_dz(192u, colZ[1], s.bias + CL_H, true);
  publish();
  // ---- layer 2: dW2 (+ db2), dA1 = dZ2 W2
  issue_pair(256u, ata[0], 336u, smem_addr(s.w2t), CL_H / 16, ha, TC_KX, CL_H);
  store_dw(256u, CL_H, CL_H, OFF_W2, OFF_B2, CL_H);
  make_dz(336u, colZ[0], s.bias, false);
  publish();
  // ---- layer 1: dW1 (+ db1 from the ones row 67 of xt)
  issue_pair(400u, xta, 0u, 0u, 0, 0u, 0u, CL_H);
  store_dw(400u, CL_H, CL_K0, OFF_W1, OFF_B1, CL_IN);
  tc_free(tmem, TT_COLS);
}

__global__ void grad_reduce_kernel(const float* __restrict__ gw, int nparts, float* __restrict__ grad,
                                   const float* __restrict__ lossw, float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < CL_NPARAM) {
    float s = 0.f;
    for (int w = 0; w < nparts; ++w) s += gw[(size_t)w * CL_NPARAM + p];
    grad[p] = s;
  }
  if (p == 0) {
    float s = 0.f;
    for (int w = 0; w < nparts; ++w) s += lossw[w];
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
    } else {
      const int r = (e - IMG_W3T) / S64, c = (e - IMG_W3T) % S64;
      v = c < CL_H ? p[OFF_W3 + c * CL_H + r] : 0.f;
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

// MLP on given inputs (test support, the inference path): X float [n][67] -> Y [n][3]
__global__ void __launch_bounds__(TC_THREADS) mlp_eval_kernel(const float* __restrict__ X, int n,
                                                              const bf16* __restrict__ img,
                                                              const float* __restrict__ params,
                                                              float* __restrict__ Y, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TcSmem& s = *reinterpret_cast<TcSmem*>(smem_raw);
  tc_setup(s, img, params);
  unsigned char* xb = reinterpret_cast<unsigned char*>(s.x);
  u32 phase = 0;
  bool live = true;
  const int tiles = (n + TC_ROWS - 1) / TC_ROWS;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int i = tile * TC_ROWS + threadIdx.x;
    float f[CL_K0];
#pragma unroll
    for (int k = 0; k < CL_K0; ++k) f[k] = (i < n && k < CL_IN) ? X[(size_t)i * CL_IN + k] : 0.f;
    tc_store_row<CL_K0 / 8>(xb, threadIdx.x, TC_KX, f);
    float y[3];
    tc_forward(s, phase, live, err, y);
    if (i < n) {
      Y[(size_t)i * 3 + 0] = y[0];
      Y[(size_t)i * 3 + 1] = y[1];
      Y[(size_t)i * 3 + 2] = y[2];
    }
  }
  tc_teardown(s);
}

constexpr size_t kInferSmem = sizeof(TcSmem);
constexpr size_t kTrainSmem = sizeof(TcTrainSmem);
static_assert(kTrainSmem <= 227 * 1024, "training tile exceeds the shared memory of a CTA");

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
  float* gw = nullptr;          // per-CTA partial gradients
  float* lossw = nullptr;
  float* loss = nullptr;
  bf16* img = nullptr;
  int gw_parts = 0;
  bf16* X = nullptr;            // training inputs
  float* T = nullptr;           // training targets (4 per row)
  int cap = 0, count = 0;
  float* accF = nullptr;        // scratch: 3n floats each
  float* accR = nullptr;
  unsigned char* judged = nullptr;  // n flags: particles a sampled judge pass covered
  float* jerr = nullptr;        // the judge's relative differences (n), their count
  unsigned* jcount = nullptr;
  float* jerr_host = nullptr;   // pinned copy of the differences (n)
  float4* save_pm = nullptr;    // a judged step's start state (n each), to take it again
  float4* save_vi = nullptr;
  unsigned char* save_diag = nullptr;  // and its diagnostics' running state (32 bytes)
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
  // 128-particle tiles; ~67 KB of shared memory and 64 TMEM columns per CTA: 3 CTAs per SM
  const int tiles = (h->n + TC_ROWS - 1) / TC_ROWS;
  const int blocks = std::min(tiles, h->num_sms * 3);
  if (blocks > 0) {
    closure_infer_kernel<<<blocks, TC_THREADS, kInferSmem, h->st>>>(h->pm[h->cur], h->n, c->rm, c->occ, c->img,
                                                                    c->params, h->acc_pm, h->flags,
                                                                    h->flags + kFlagTimeout);
    PMGB_LAUNCH_CHECK();
    count_launches(1);
  }
  return PMGB_OK;
}

int closure_mode(const pmgb_pm* h) { return h->closure ? h->closure->mode : 3; }

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
  c->gw_parts = 4096 / TC_ROWS;  // largest batch
  if ((rc = cl_alloc(&c->occ_fx, c->ncells)) || (rc = cl_alloc(&c->occ, c->ncells)) ||
      (rc = cl_alloc(&c->params, CL_NPARAM)) || (rc = cl_alloc(&c->adam_m, CL_NPARAM)) ||
      (rc = cl_alloc(&c->adam_v, CL_NPARAM)) || (rc = cl_alloc(&c->grad, CL_NPARAM)) ||
      (rc = cl_alloc(&c->gw, (size_t)c->gw_parts * CL_NPARAM)) || (rc = cl_alloc(&c->lossw, c->gw_parts)) ||
      (rc = cl_alloc(&c->loss, 1)) || (rc = cl_alloc(&c->img, IMG_SIZE)) ||
      (rc = cl_alloc(&c->X, (size_t)std::max(c->cap, 1) * CL_K0)) ||
      (rc = cl_alloc(&c->T, (size_t)std::max(c->cap, 1) * 4)) || (rc = cl_alloc(&c->accF, 3 * n)) ||
      (rc = cl_alloc(&c->accR, 3 * n)) || (rc = cl_alloc(&c->judged, n)) || (rc = cl_alloc(&c->jerr, n)) ||
      (rc = cl_alloc(&c->jcount, 1))) {
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
                  c->loss, c->img, c->X, c->T, c->accF, c->accR, c->judged, c->save_pm, c->save_vi,
                  c->save_diag, c->jerr, c->jcount};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->jerr_host) cudaFreeHost(c->jerr_host);
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
  int rc = configure_closure_kernels();
  if (rc) return rc;
  PMGB_CUDA_TRY(cudaMemsetAsync(c->pm->flags + kFlagTimeout, 0, sizeof(int), st));
  int* perm = nullptr;
  PMGB_CUDA_TRY(cudaMalloc(&perm, (size_t)c->count * sizeof(int)));
  std::vector<int> hp(c->count);
  std::mt19937_64 rng(c->seed * 7919 + 17);
  const int steps_per_epoch = c->count / batch;
  const int total_steps = epochs * steps_per_epoch;
  float last = 0.f;
  int step = 0;
  for (int e = 0; e < epochs; ++e) {
    for (int i = 0; i < c->count; ++i) hp[i] = i;
    std::shuffle(hp.begin(), hp.end(), rng);
    if (cudaMemcpyAsync(perm, hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      cudaFree(perm);
      return set_error("permutation upload failed"), PMGB_ECUDA;
    }
    for (int b = 0; b < steps_per_epoch; ++b, ++step) {
      const int parts = (batch + TC_ROWS - 1) / TC_ROWS;
      closure_train_kernel<<<parts, TC_THREADS, kTrainSmem, st>>>(c->X, c->T, perm, b * batch, batch,
                                                                  1.0f / batch, c->img, c->params, c->gw,
                                                                  c->lossw, c->pm->flags + kFlagTimeout);
      grad_reduce_kernel<<<(CL_NPARAM + 255) / 256, 256, 0, st>>>(c->gw, parts, c->grad, c->lossw, c->loss);
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
  int timed_out = 0;
  cudaMemcpyAsync(&timed_out, c->pm->flags + kFlagTimeout, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t err = cudaStreamSynchronize(st);
  cudaFree(perm);
  if (err != cudaSuccess) return set_error(std::string("training: ") + cudaGetErrorString(err)), PMGB_ECUDA;
  if (timed_out) return set_error("training: a bounded device wait gave up"), PMGB_ETIMEOUT;
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

namespace pmgb {
// |aR - aF| / |aF| of the judged particles (flags[i] set; without flags every stride-th index),
// appended in any order to err (count): the components' differences in float, the rest in
// double without contraction, as the host computed them.
__global__ void judge_err_kernel(const float* __restrict__ accR, const float* __restrict__ accF,
                                 const unsigned char* __restrict__ flags, int stride, int n, float* __restrict__ err,
                                 unsigned* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !(flags ? flags[i] != 0 : i % stride == 0)) return;
  const float b0 = accF[3 * i], b1 = accF[3 * i + 1], b2 = accF[3 * i + 2];
  const double dx = __fsub_rn(accR[3 * i], b0), dy = __fsub_rn(accR[3 * i + 1], b1),
               dz = __fsub_rn(accR[3 * i + 2], b2);
  const double nb = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(b0, b0), __dmul_rn(b1, b1)), __dmul_rn(b2, b2)));
  if (!(nb > 0)) return;
  const double d = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
  err[atomicAdd(count, 1u)] = (float)__ddiv_rn(d, nb);
}
}  // namespace pmgb

// median relative error of the closure force vs the full-cutoff P3M force, over every
// `stride`-th particle, at the current positions
int pmgb_closure_judge(pmgb_closure* c, int stride, float* median_rel_err) {
  if (!c || !median_rel_err) return set_error("null argument"), PMGB_EINVAL;
  if (stride < 1) stride = 1;
  pmgb_pm* h = c->pm;
  const size_t n = (size_t)h->n;
  int rc;
  // the learned force at the current positions: the one the last step left when it was a
  // learned step, else a fresh evaluation
  if (h->acc_mode == PMGB_CLOSURE_LEARNED) {
    rc = launch_unpack(h->pm[h->cur], h->vi[h->cur], h->acc, h->n, h->cfg.H, h->cfg.DT, 0, h->stage,
                       h->stage + 3 * n, h->stage + 6 * n, h->st);
    if (rc) return rc;
    PMGB_CUDA_TRY(cudaMemcpyAsync(c->accR, h->stage + 6 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToDevice,
                                  h->st));
  } else if ((rc = force_into(c, PMGB_CLOSURE_LEARNED, c->accR))) {
    return rc;
  }
  // the plain P3M force on the particles of every stride-th slice of its pair pass (a sampled
  // pass, about 1/stride of its cost), or on every stride-th particle where the pass cannot be
  // sampled (the direct formula with softening)
  const bool sampled = stride > 1 && pair_pass_sampleable(c->full->pp);
  c->full->unit_stride = sampled ? stride : 1;
  rc = force_into(c, PMGB_CLOSURE_FULL, c->accF);
  c->full->unit_stride = 1;
  if (rc) return rc;
  if (sampled && n) {
    PMGB_CUDA_TRY(cudaMemsetAsync(c->judged, 0, n, h->st));
    rc = launch_mark_sampled(c->full->cell_start, c->full->items, c->full->nitems, c->full->nitems_max, stride,
                             h->vi[h->cur], c->judged, h->st);
    if (rc) return rc;
  }
  // the judged particles' relative differences, on the device; only they come back
  if (!c->jerr_host && cudaMallocHost(&c->jerr_host, std::max(n, (size_t)1) * sizeof(float)) != cudaSuccess) {
    c->jerr_host = nullptr;
    cudaGetLastError();
    return set_error("cudaMallocHost failed (judge)"), PMGB_ENOMEM;
  }
  unsigned count = 0;
  PMGB_CUDA_TRY(cudaMemsetAsync(c->jcount, 0, sizeof(unsigned), h->st));
  if (n) {
    judge_err_kernel<<<(unsigned)((n + 255) / 256), 256, 0, h->st>>>(c->accR, c->accF, sampled ? c->judged : nullptr,
                                                                     stride, (int)n, c->jerr, c->jcount);
    PMGB_LAUNCH_CHECK();
    count_launches(1);
  }
  PMGB_CUDA_TRY(cudaMemcpyAsync(&count, c->jcount, sizeof(unsigned), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  if (count == 0) {
    *median_rel_err = 0.f;
    return PMGB_OK;
  }
  PMGB_CUDA_TRY(cudaMemcpyAsync(c->jerr_host, c->jerr, count * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  // the median of the multiset: the same whatever order the kernel appended them in
  std::nth_element(c->jerr_host, c->jerr_host + count / 2, c->jerr_host + count);
  *median_rel_err = c->jerr_host[count / 2];
  return PMGB_OK;
}

// Runs n_steps loop iterations (pmgb_pm_advance, one at a time).  In the learned mode every
// judge_interval-th step (s = 0, judge_interval, ...) is judged after it ran: the learned force it
// used, at the positions it drifted to, against plain P3M there (pmgb_closure_judge).  If the
// median relative difference exceeds `bound`, the step is taken again from its saved start state
// (positions, velocities, particle order, diagnostics' running state) with plain full-cutoff P3M,
// and so is the rest of the run (*fallback_step = the step, else -1): no step keeps a force the
// judge rejected.  device_ms counts both attempts of a rejected step.
int pmgb_closure_run(pmgb_closure* c, int n_steps, float bound, int judge_interval,
                     int judge_stride, int* steps_done, int* fallback_step, float* device_ms) {
  if (!c) return set_error("null handle"), PMGB_EINVAL;
  if (fallback_step) *fallback_step = -1;
  pmgb_pm* h = c->pm;
  const size_t n = (size_t)h->n;
  if (c->mode == PMGB_CLOSURE_LEARNED && judge_interval > 0 && !c->save_pm) {
    if (cudaMalloc(&c->save_pm, std::max(n, (size_t)1) * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&c->save_vi, std::max(n, (size_t)1) * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&c->save_diag, 32) != cudaSuccess) {
      cudaGetLastError();
      return set_error("cudaMalloc failed (closure step state)"), PMGB_ENOMEM;
    }
  }
  float total_ms = 0.f;
  int done = 0;
  auto finish = [&](int rc) {
    if (steps_done) *steps_done = done;
    if (device_ms) *device_ms = total_ms;
    return rc;
  };
  for (int s = 0; s < n_steps; ++s) {
    const bool judge = c->mode == PMGB_CLOSURE_LEARNED && judge_interval > 0 && s % judge_interval == 0;
    const int cur0 = h->cur, since0 = h->since_sort;
    if (judge) {
      PMGB_CUDA_TRY(cudaMemcpyAsync(c->save_pm, h->pm[cur0], n * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
      PMGB_CUDA_TRY(cudaMemcpyAsync(c->save_vi, h->vi[cur0], n * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
      int rc = diag_save(h, c->save_diag);
      if (rc) return rc;
    }
    float ms = 0.f;
    int d = 0;
    int rc = pmgb_pm_advance(h, 1, &d, &ms);
    total_ms += ms;
    if (rc == PMGB_EESCAPED) return finish(rc);
    if (rc) return rc;
    if (judge) {
      float err = 0.f;
      rc = pmgb_closure_judge(c, judge_stride, &err);  // the learned force this step left
      if (rc) return rc;
      if (err > bound) {
        h->cur = cur0;
        h->since_sort = since0;
        h->acc_mode = -1;
        PMGB_CUDA_TRY(cudaMemcpyAsync(h->pm[cur0], c->save_pm, n * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
        PMGB_CUDA_TRY(cudaMemcpyAsync(h->vi[cur0], c->save_vi, n * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
        if ((rc = diag_restore(h, c->save_diag))) return rc;
        set_mode(c, PMGB_CLOSURE_FULL);
        if (fallback_step) *fallback_step = s;
        rc = pmgb_pm_advance(h, 1, &d, &ms);
        total_ms += ms;
        if (rc == PMGB_EESCAPED) return finish(rc);
        if (rc) return rc;
      }
    }
    ++done;
  }
  return finish(PMGB_OK);
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
  int* derr = nullptr;
  const size_t nn = (size_t)std::max(n, 1);
  PMGB_CUDA_TRY(cudaMalloc(&dp, CL_NPARAM * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&img, IMG_SIZE * sizeof(bf16)));
  PMGB_CUDA_TRY(cudaMalloc(&dx, nn * CL_IN * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&dy, nn * 3 * sizeof(float)));
  PMGB_CUDA_TRY(cudaMalloc(&derr, sizeof(int)));
  cudaMemcpy(dp, params, CL_NPARAM * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x, (size_t)n * CL_IN * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(derr, 0, sizeof(int));
  image_kernel<<<64, 256>>>(dp, img);
  mlp_eval_kernel<<<std::max(1, std::min(1024, (n + TC_ROWS - 1) / TC_ROWS)), TC_THREADS, kInferSmem>>>(
      dx, n, img, dp, dy, derr);
  cudaMemcpy(y, dy, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost);
  int timed_out = 0;
  cudaMemcpy(&timed_out, derr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaError_t err = cudaDeviceSynchronize();
  cudaFree(dp);
  cudaFree(img);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(derr);
  if (err != cudaSuccess) return set_error(cudaGetErrorString(err)), PMGB_ECUDA;
  if (timed_out) return set_error("a tensor-core wait gave up"), PMGB_ETIMEOUT;
  return PMGB_OK;
}

// Test support: the tensor-core path's bounded mbarrier wait on a barrier of one expected
// arrival that gets it (arrive = 1) or never does (arrive = 0).
__global__ void tc_wait_probe_kernel(int arrive, int spins, int* __restrict__ err) {
  __shared__ __align__(8) u64 mbar;
  const u32 a = smem_addr(&mbar);
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(a) : "memory");
  __syncthreads();
  if (threadIdx.x == 0 && arrive)
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" :: "r"(a) : "memory");
  if (!tc_wait(a, 0u, spins)) atomicExch(err, 1);
}

int pmgb_tc_wait_probe(int arrive, int spins) {
  if (spins < 1) return set_error("spins must be positive"), PMGB_EINVAL;
  int* derr = nullptr;
  PMGB_CUDA_TRY(cudaMalloc(&derr, sizeof(int)));
  int gave_up = 0;
  cudaMemset(derr, 0, sizeof(int));
  tc_wait_probe_kernel<<<1, TC_THREADS>>>(arrive, spins, derr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&gave_up, derr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(derr);
  if (e != cudaSuccess) return set_error(cudaGetErrorString(e)), PMGB_ECUDA;
  if (gave_up) return set_error("a bounded device wait gave up"), PMGB_ETIMEOUT;
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
  int *perm = nullptr, *derr = nullptr;
  const int parts = (n + TC_ROWS - 1) / TC_ROWS;
  auto release = [&]() {
    void* all[] = {dp, dt, gw, g, lw, l, img, dx, perm, derr};
    for (void* p : all) cudaFree(p);
  };
  if (cudaMalloc(&dp, CL_NPARAM * sizeof(float)) || cudaMalloc(&img, IMG_SIZE * sizeof(bf16)) ||
      cudaMalloc(&dx, (size_t)n * CL_K0 * sizeof(bf16)) || cudaMalloc(&dt, (size_t)n * 4 * sizeof(float)) ||
      cudaMalloc(&gw, (size_t)parts * CL_NPARAM * sizeof(float)) || cudaMalloc(&g, CL_NPARAM * sizeof(float)) ||
      cudaMalloc(&lw, parts * sizeof(float)) || cudaMalloc(&l, sizeof(float)) ||
      cudaMalloc(&perm, n * sizeof(int)) || cudaMalloc(&derr, sizeof(int))) {
    release();
    return set_error("device allocation failed"), PMGB_ECUDA;
  }
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
  cudaMemset(derr, 0, sizeof(int));
  image_kernel<<<64, 256>>>(dp, img);
  closure_train_kernel<<<parts, TC_THREADS, kTrainSmem>>>(dx, dt, perm, 0, n, 1.0f / n, img, dp, gw, lw, derr);
  grad_reduce_kernel<<<(CL_NPARAM + 255) / 256, 256>>>(gw, parts, g, lw, l);
  count_launches(3);
  cudaMemcpy(grad, g, CL_NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
  float lh = 0.f;
  int timed_out = 0;
  cudaMemcpy(&lh, l, sizeof(float), cudaMemcpyDeviceToHost);
  cudaMemcpy(&timed_out, derr, sizeof(int), cudaMemcpyDeviceToHost);
  cudaError_t err = cudaDeviceSynchronize();
  if (loss) *loss = lh / n;
  release();
  if (err != cudaSuccess) return set_error(cudaGetErrorString(err)), PMGB_ECUDA;
  if (timed_out) return set_error("a bounded device wait gave up"), PMGB_ETIMEOUT;
  return PMGB_OK;
}

}  // extern "C"
