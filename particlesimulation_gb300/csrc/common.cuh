// common.cuh - shared device state and helpers of the PM / P3M kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/pmgb.h"

namespace pmgb {

typedef unsigned long long u64;
typedef unsigned int u32;

// ---------------------------------------------------------------- error plumbing ----
void set_error(const std::string& msg);
// Host-side tally of kernels launched through this library (pmgb_kernel_launches).
void count_launches(int k);
#define PMGB_CUDA_TRY(expr)                                                        \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) {                                                       \
      ::pmgb::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));       \
      return PMGB_ECUDA;                                                           \
    }                                                                              \
  } while (0)
#define PMGB_LAUNCH_CHECK()                                                        \
  do {                                                                             \
    cudaError_t _e = cudaGetLastError();                                           \
    if (_e != cudaSuccess) {                                                       \
      ::pmgb::set_error(std::string("kernel launch: ") + cudaGetErrorString(_e));  \
      return PMGB_ECUDA;                                                           \
    }                                                                              \
  } while (0)

// Keys per block of the LSD radix sort (sort.cu): its histogram holds 256 words per block of
// RS_TILE keys plus 256 row totals (radix_hist_words).
constexpr int RS_TILE = 4096;

// ---------------------------------------------------------------- parameters --------
// Everything a kernel needs about one system, passed by value.
struct MeshDims {
  int nx, ny, nz;
  int lx, ly, lz;     // log2 of the above
  int nxh;            // nx/2 + 1 complex bins kept along x
  int nxp;            // row stride of the half spectrum (nxh rounded up to a multiple of 4)
  long long L;        // nx*ny*nz
};

struct ExtField {
  int kind;
  float cx, cy, cz, R, M, G;
};

struct StepParams {
  MeshDims m;
  int is;             // 0 NGP 1 CIC 2 TSC
  int fds;            // 0 two-point 1 four-point
  float H, DT;        // for the unit round trip and the external field
  float box_x, box_y, box_z;  // escape test, original units
  ExtField ext;
  float fx_scale;     // 2^k: float -> fixed-point density
  float fx_inv;       // 2^-k
  int step_tag;       // run iteration whose drift this launch performs (escape bookkeeping)
  int periodic;       // wrap positions into the mesh after a drift instead of the escape test
};

// Entry test of a kernel that may drift.  A drift that escapes sets stop[0] while other blocks
// of the same launch may not have started yet, so such a kernel must not test stop[0]: it
// stops only if an earlier iteration escaped (stop[1] holds the smallest escaping iteration,
// INT_MAX at the start of a run).  Every other kernel tests stop[0].
__device__ __forceinline__ bool stopped_before(const int* stop, bool drifts, int tag) {
  return drifts ? stop[1] < tag : stop[0] != 0;
}

// Kick, drift, the reference's unit round trip (stateToOriginalUnits / stateToCodeUnits,
// source/pmMethod.cpp:87-113) and the escapedComputationalBox test (146-156) of one particle,
// dt = 1 in code units (source/leapfrog.cpp:5-24).  An escape sets stop[0] and records the
// iteration in stop[1].
__device__ __forceinline__ void kick_drift(const StepParams& sp, float4& p, float4& v, float3 a,
                                           float kick, int drift, int* stop) {
  if (kick != 0.f) {
    v.x = v.x + kick * a.x;
    v.y = v.y + kick * a.y;
    v.z = v.z + kick * a.z;
  }
  if (!drift) return;
  p.x = p.x + v.x;
  p.y = p.y + v.y;
  p.z = p.z + v.z;
  if (sp.periodic) {
    const float nx = (float)sp.m.nx, ny = (float)sp.m.ny, nz = (float)sp.m.nz;
    p.x = p.x < 0.f ? p.x + nx : (p.x >= nx ? p.x - nx : p.x);
    p.y = p.y < 0.f ? p.y + ny : (p.y >= ny ? p.y - ny : p.y);
    p.z = p.z < 0.f ? p.z + nz : (p.z >= nz ? p.z - nz : p.z);
  }
  const float xo = __fmul_rn(sp.H, p.x), yo = __fmul_rn(sp.H, p.y), zo = __fmul_rn(sp.H, p.z);
  const float vxo = __fdiv_rn(__fmul_rn(sp.H, v.x), sp.DT);
  const float vyo = __fdiv_rn(__fmul_rn(sp.H, v.y), sp.DT);
  const float vzo = __fdiv_rn(__fmul_rn(sp.H, v.z), sp.DT);
  if (!sp.periodic) {
    const bool inside = xo >= 0 && xo <= sp.box_x && yo >= 0 && yo <= sp.box_y && zo >= 0 && zo <= sp.box_z;
    if (!inside) {
      atomicExch(stop, 1);
      atomicMin(stop + 1, sp.step_tag);
    }
  }
  p.x = __fdiv_rn(xo, sp.H);
  p.y = __fdiv_rn(yo, sp.H);
  p.z = __fdiv_rn(zo, sp.H);
  v.x = __fdiv_rn(__fmul_rn(sp.DT, vxo), sp.H);
  v.y = __fdiv_rn(__fmul_rn(sp.DT, vyo), sp.H);
  v.z = __fdiv_rn(__fmul_rn(sp.DT, vzo), sp.H);
}

// Chaining mesh geometry (ChainingMesh ctor, reference source/chainingMesh.cpp:6-18).
struct ChainDims {
  int Mx, My, Mz;
  float HCx, HCy, HCz;  // cell side, code units (lengthToCodeUnits(compBox/M, H))
  // Sub-columns: each cell is split into sub x sub columns along x and z (the particles of a
  // column sorted by y), so the pair pass can skip the columns of a neighbour cell that are out
  // of reach in x and z.  sub = 1: plain cells.  Sub-column id = (cell * sub + sz) * sub + sx.
  int sub;
  float HCsx, HCsz;  // sub-column widths (HCx / sub, HCz / sub)
};

// Short-range pair pass parameters, code units.
struct PairParams {
  float re2;       // cutoff^2
  float re;        // cutoff
  float inv_d2;    // 1 / delta^2 of the table
  int use_table;
  int ysort;       // y-window pruning (cell lists are y-sorted)
  int shape;       // 0 S1, 1 S2 (direct formula)
  float a;         // particle diameter
  float eps2;      // softening^2
};

// Fixed-point density: signed 64-bit sums stored in unsigned slots (two's complement adds).
__device__ __forceinline__ void fx_add_global(u64* p, long long v) {
  atomicAdd(p, (u64)v);
}

// powers of two only: one AND, exact for any a (the interpolation's potential reads, where the
// general form below measured 30 % slower at 256^3)
__device__ __forceinline__ int wrapi_p2(int a, int n) { return a & (n - 1); }

__device__ __forceinline__ int wrapi(int a, int n) {
  // a mesh index wrapped into [0, n).  Powers of two: one AND, exact for any a.  Other sizes
  // (the mixed-radix meshes): a is at most a stencil width outside the mesh for particles inside
  // it; an index further out (a particle that left the box, whose run stops) is clamped so that
  // every access stays inside the mesh.
  if ((n & (n - 1)) == 0) return a & (n - 1);
  a += a < 0 ? n : 0;
  a -= a >= n ? n : 0;
  return min(max(a, 0), n - 1);
}

// Exact product chain of the reference, with no contraction into FMA.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// PMMethod::TSCAssignmentFunc (reference source/pmMethod.cpp:187-198), evaluated without FMA
// contraction so every weight is the reference's float value.
__device__ __forceinline__ float tsc_w(float x, int t) {
  if (t == 1) {
    float a = fadd(0.5f, x);
    return fmul(a, a);
  }
  if (t == 0) return fsub(1.5f, fmul(fmul(2.0f, x), x));
  float a = fsub(0.5f, x);
  return fmul(a, a);
}

// Order-preserving key of a float (for the y-sorted cell lists); -0 is folded onto +0 so
// that equal floats get equal keys, as the reference's `>` comparison treats them.
__device__ __forceinline__ u32 float_key(float f) {
  if (f == 0.0f) f = 0.0f;
  u32 b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

}  // namespace pmgb
