// pair.cu - the P3M short-range pair pass on the chaining mesh.
//
// Restates P3MMethod::calculateShortRangeForces / updateSRForces / correctAccelerations
// (reference source/p3mMethod.cpp:50-57, 168-192, 247-273, 296-322): every particle pair closer
// than the cutoff in the same or adjacent chaining cells (non-periodic) adds
//   F_ij = m_i m_j (T[t] + (xi - t) (T[t+1] - T[t])) r_ij,   xi = |r_ij|^2 / delta^2, t = int(xi)
// from the 500-entry table (initSRForceTable, 275-294), or the direct S1/S2 formula
// (shortRangeForce, 220-238) when the table is off; the acceleration gains F_i / m_i.
//
// GPU formulation.  The reference walks 13 half-shell neighbour cells and scatters -F_ij into
// per-neighbour slots of j.  Here each particle gathers from all 27 cells (each pair is
// evaluated twice, once per side), so no scatter, no atomics and a deterministic result, except
// for the dense sub-column pairs of equal-mass systems, which the slotted pass evaluates once,
// both sides into slots of their own (the symmetric part, below).
// Two kernels: pair_slot_kernel (below; the table pass and the exact formula of every run,
// finer work items and fewer instructions per pair) and pair_kernel, described here, which also
// counts pairs and evaluates the softened table-free formula.
// Work items are 32-particle slices of one cell (the cells are y-sorted, so a slice spans a
// narrow y range); a warp takes items from a global counter (dense cells cost more, the counter
// balances).  For each neighbour cell a lane binary-searches the y window
// [y_min - re, y_max + re] of the slice in that cell's y-sorted list (pairs outside it fail the
// cutoff test anyway, as the reference's early break assumes); candidate j particles are loaded
// 32 at a time, one per lane, and broadcast with shuffles.  Sums are FP32 per 32-particle chunk,
// chunks are added with Kahan compensation.
//
// The epilogue adds the PM acceleration and, in a run, applies the kick, the drift, the unit
// round trip and the escape test, writing the new state to separate buffers (other warps still
// read the old positions).
#include <algorithm>

#include "handles.cuh"

namespace pmgb {

struct ChainDimsP {
  int Mx, My, Mz;
  int ncells;
  int sub;            // sub-columns per cell along x and z
  float HCsx, HCsz;   // sub-column widths
};

constexpr int PAIR_THREADS = 256;
constexpr int PAIR_WARPS = PAIR_THREADS / 32;

// referenceForceS1 / S2 (p3mMethod.cpp:194-218) and the direct short-range force magnitude
// per unit r (shortRangeForce, 220-238): F = mi mj (-G/(r^2+eps^2) + R(r)) / r.
__device__ float ref_force(int shape, float r, float a) {
  const float G = 1.0f / (4.0f * 3.14159265f);
  if (shape == 0) {
    if (r >= a) return G / (r * r);
    const float q = r / a;
    return G / (a * a) * (8.0f * q - 9.0f * q * q + 2.0f * q * q * q * q);
  }
  const float u = 2.0f * r / a;
  const float u2 = u * u, u3 = u2 * u, u4 = u2 * u2, u5 = u4 * u, u6 = u3 * u3;
  if (u <= 1.0f)
    return G / (35.0f * a * a) * (224.0f * u - 224.0f * u3 + 70.0f * u4 + 48.0f * u5 - 21.0f * u6);
  if (u <= 2.0f)
    return G / (35.0f * a * a) *
           (12.0f / u2 - 224.0f + 896.0f * u - 840.0f * u2 + 224.0f * u3 + 70.0f * u4 - 48.0f * u5 + 7.0f * u6);
  return G / (r * r);
}

__device__ __forceinline__ float direct_f(const PairParams& pp, float r2) {
  const float G = 1.0f / (4.0f * 3.14159265f);
  const float r = sqrtf(r2);
  return (-G / (r2 + pp.eps2) + ref_force(pp.shape, r, pp.a)) / r;
}

// first index in [lo, hi) whose y >= v (lower) / > v (upper)
__device__ __forceinline__ int y_lower(const float4* __restrict__ pm, int lo, int hi, float v) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&pm[mid].y) < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int y_upper(const float4* __restrict__ pm, int lo, int hi, float v) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&pm[mid].y) <= v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}


constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: adding it rounds to an integer

template <bool TABLE, bool COUNT>
__global__ void __launch_bounds__(PAIR_THREADS) pair_kernel(
    const float4* __restrict__ pm, const float4* __restrict__ vi, const float4* __restrict__ acc_pm,
    const int* __restrict__ cell_start, const int2* __restrict__ items, const u32* __restrict__ nitems_p,
    u32* __restrict__ counter, ChainDimsP cd, PairParams pp, const float* __restrict__ table,
    StepParams sp, float kick, int drift, int kdk, float4* __restrict__ pm_out,
    float4* __restrict__ vi_out, float4* __restrict__ acc_out, unsigned long long* __restrict__ npairs,
    int* stop) {
  if (stopped_before(stop, kdk && drift, sp.step_tag)) return;
  // (T[t], T[t+1] - T[t]); entry 499 = (T[499], 0) so that t = 499 at the cutoff is in range
  __shared__ float2 tab[500];
  __shared__ float4 jbuf[PAIR_WARPS][32];
  for (int t = threadIdx.x; t < 500; t += PAIR_THREADS) {
    const float a = table[t], b = t < 499 ? table[t + 1] : a;
    tab[t] = make_float2(a, b - a);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const u32 nitems = *nitems_p;
  unsigned long long my_pairs = 0;
  for (;;) {
    u32 it = 0;
    if (lane == 0) it = atomicAdd(counter, 1u);
    it = __shfl_sync(0xFFFFFFFFu, it, 0);
    if (it >= nitems) break;
    const int2 item = items[it];
    const int sub2 = cd.sub * cd.sub;
    const int cell = item.x / sub2;
    const int cend = cell_start[item.x + 1];
    const int i = item.y + lane;
    const bool valid = i < cend;
    const int last = min(item.y + 31, cend - 1);
    const float4 pi = pm[valid ? i : last];
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;

    if (cell < cd.ncells) for (int qs = 0; qs < sub2; ++qs) {
      const int gx = cell % cd.Mx, gy = (cell / cd.Mx) % cd.My, gz = cell / (cd.Mx * cd.My);
      // y range of the slice: lane 0 holds its first particle, lane 31 its last (lanes past
      // the end of the cell load the last particle)
      const float ylo = __shfl_sync(0xFFFFFFFFu, pi.y, 0) - pp.re;
      const float yhi = __shfl_sync(0xFFFFFFFFu, pi.y, 31) + pp.re;
      // lane k < 27 resolves neighbour k = (dx, dy, dz) in {-1,0,1}^3
      int jb = 0, je = 0;
      if (lane < 27) {
        const int nx = gx + lane % 3 - 1, ny = gy + (lane / 3) % 3 - 1, nz = gz + lane / 9 - 1;
        if (nx >= 0 && ny >= 0 && nz >= 0 && nx < cd.Mx && ny < cd.My && nz < cd.Mz) {
          const int cn = (nx + ny * cd.Mx + nz * cd.Mx * cd.My) * sub2 + qs;
          jb = cell_start[cn];
          je = cell_start[cn + 1];
          if (pp.ysort && je > jb) {
            jb = y_lower(pm, jb, je, ylo);
            je = y_upper(pm, jb, je, yhi);
          }
        }
      }
      for (int k = 0; k < 27; ++k) {
        const int b = __shfl_sync(0xFFFFFFFFu, jb, k);
        const int e = __shfl_sync(0xFFFFFFFFu, je, k);
        for (int j0 = b; j0 < e; j0 += 32) {
          // stage 32 candidates in this warp's shared buffer; every lane then reads each one
          // with a broadcast load
          const int jj = j0 + lane;
          jbuf[warp][lane] = jj < e ? pm[jj] : make_float4(3.0e30f, 3.0e30f, 3.0e30f, 0.f);
          __syncwarp();
          const int cnt = min(32, e - j0);
          float px = 0.f, py = 0.f, pz = 0.f;
#pragma unroll 4
          for (int s = 0; s < cnt; ++s) {
            const float4 q = jbuf[warp][s];
            const float dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            float f;
            if (TABLE) {
              // t = floor(xi) from the float's mantissa (full-rate ops instead of two
              // quarter-rate conversions); at an exact integer xi it may give xi - 1 with
              // frac = 1, the same point of the piecewise-linear table
              const float xi = fminf(r2, pp.re2) * pp.inv_d2;
              const float tf = (xi - 0.5f) + kMagic;
              const int t = __float_as_int(tf) - __float_as_int(kMagic);
              const float frac = xi - (tf - kMagic);
              const float2 tv = tab[t];
              f = fmaf(frac, tv.y, tv.x);
            } else {
              f = r2 > 0.f ? direct_f(pp, r2) : 0.f;
            }
            const bool in = r2 < pp.re2;
            f = in ? f * q.w : 0.f;
            px = fmaf(f, dx, px);
            py = fmaf(f, dy, py);
            pz = fmaf(f, dz, pz);
            if (COUNT) my_pairs += (in && r2 > 0.f && valid) ? 1ull : 0ull;
          }
          __syncwarp();
          kahan_add(sx, cx, px);
          kahan_add(sy, cy, py);
          kahan_add(sz, cz, pz);
        }
      }
    }
    if (valid) {
      const float4 ap = acc_pm[i];
      const float3 a = make_float3(ap.x + sx, ap.y + sy, ap.z + sz);
      if (kdk) {
        float4 p = pi, v = vi[i];
        kick_drift(sp, p, v, a, kick, drift, stop);
        pm_out[i] = p;
        vi_out[i] = v;
      }
      acc_out[i] = make_float4(a.x, a.y, a.z, 0.f);
    }
  }
  if (COUNT) {
    for (int o = 16; o > 0; o >>= 1) my_pairs += __shfl_xor_sync(0xFFFFFFFFu, my_pairs, o);
    if (lane == 0 && my_pairs) atomicAdd(npairs, my_pairs);
  }
}

// ------------------------------------------------------- table pair pass, slotted ----
// The table path without pair counting.  Work is split finer than one item per slice so that
// the dense cells of clustered inputs do not leave a long tail: a work item is one 64-particle
// slice of a cell against ONE of its 27 neighbour cells, and it writes the slice's partial
// short-range acceleration from that neighbour into slot k of each particle
// (slots[k * n + i], k = 0..26, zero for a neighbour outside the mesh).  An epilogue kernel adds
// the 27 slots in a fixed order (so the result is deterministic), the PM acceleration, and in a
// run the kick and drift.  Fewer instructions per candidate pair than pair_kernel:
//  * each lane holds two i particles, so every staged candidate is read once from shared
//    memory for two pairs;
//  * the table is kept in intercept form per segment, f(xi) = A[t] + xi S[t] with
//    S[t] = T[t+1] - T[t] (float, as the reference forms it) and A[t] = T[t] - t S[t] (double,
//    rounded once): one FMA instead of forming xi - t;
//  * positions enter in units of sqrt(512) table spacings delta, relative to the slice's first
//    particle (so differences keep code-unit precision): |r|^2 is xs = xi / 512, and the last
//    multiply-add of |r|^2 saturates it to [0, 1] (fma.sat, no extra instruction), which is the
//    bound check of the lookup; 512 is folded into S and 1/delta into the table;
//  * t = floor(512 xs) is one round-down multiply-add of xs by 512 plus 1.5 * 2^23 (FFMA.RM,
//    exact: 512 xs is a power-of-two scaling), whose bits give the lane's table entry by one
//    32-bit multiply-add into a shared-memory address;
//  * the cutoff test is folded into the table: segments 499 <= t <= 512 (xi >= 499, i.e.
//    r^2 >= re^2) are zero;
//  * with equal masses (every benchmark workload) the mass is folded into the table;
//  * the table is replicated 16 times, copy (lane mod 16) for each lane, so the per-lane lookups
//    of a half warp fall into 16 distinct bank pairs whatever their segments (an 8-byte load
//    of a warp then takes the minimum of two shared-memory wavefronts instead of about four);
//    64 KB of shared memory;
//  * one 512-thread CTA per SM with the whole register file, 128 registers per thread
//    (SLOT_CTAS_PER_SM): two CTAs of 64 registers (32 warps per SM) spilled and took 6.42 ms on
//    the 262,144-particle disk; one CTA (16 warps, enough to keep issue busy with the 16-deep
//    candidate loop) took 6.51 ms at 80 registers, 6.23 at 96, 6.36 at 112, 6.18 at 128.
// The y window of the slice in the neighbour's y-sorted list is found by a warp-cooperative
// search (32 probes per round).  Per-chunk partial sums are added with Kahan compensation.
constexpr int SLOT_IPL = 2;                  // i particles per lane
constexpr int SLOT_SLICE = 32 * SLOT_IPL;    // particles per work item
constexpr int SLOT_TAB = 513;                // segments 0..512 (499..512 = zero)
constexpr int SLOT_REP = 16;                 // table copies (lane mod 16)
constexpr int NNB = 27;                      // neighbour cells (and slots) per particle
constexpr int SLOT_THREADS = 512;
constexpr int SLOT_WARPS = SLOT_THREADS / 32;
constexpr int SLOT_CTAS_PER_SM = 1;         // resident CTAs per SM (128 registers per thread)
// staging (SLOT_WARPS x 32 float4) + CTA partial sums (SLOT_WARPS x SLOT_SLICE float4) + table
constexpr int SLOT_PART = 128;              // partial sums per warp (the symmetric slices' 128)
constexpr int SLOT_SMEM = SLOT_WARPS * 32 * 16 + SLOT_WARPS * SLOT_PART * 16 + SLOT_TAB * SLOT_REP * 8;
// Units whose estimated cost reaches 1/SLOT_HEAVY_DIV of a warp's share of the pass (and at
// least SLOT_HEAVY_MIN) are taken by whole CTAs.
constexpr int SLOT_HEAVY_DIV = 4;
constexpr int SLOT_REST_BATCH = 1;  // one-sided units a warp claims per fetch in the last loop (4: -1 % on
                                     // the reduced pass, +1 % elsewhere; 32: +3-5 %)
// symmetric sub-column pairs: L = sub^2 sub-columns per cell (9, 16 or 25), one slot per
// (direction, neighbour sub-column) and particle; mask words per sub-column: 27 L mark bits
// (bit k L + q: neighbour sub-column q of direction k), then one word of dead directions (bit k:
// nothing one-sided is left toward neighbour cell k)
__host__ __device__ constexpr int sym_mark_words(int local) { return (NNB * local + 31) / 32; }
// counter words of the slotted pass (see SLOT_COUNTER_WORDS)
// symmetric units in cost buckets (longest first): 0..3 for CTAs (|p| |q| >= 8, 2, 1, 1/2 heavy
// thresholds), 4..8 for warps (>= 1/4, 1/8, 1/16, 1/32 of the threshold, below)
constexpr int SYM_NB = 9, SYM_NB_CTA = 4;
constexpr int SLOT_SYM_COUNT = 10, SLOT_SYM_TAKEN = SLOT_SYM_COUNT + SYM_NB, SLOT_SYM_TOTAL = SLOT_SYM_TAKEN + SYM_NB;
static_assert(SLOT_SYM_TOTAL == kSlotSymTotalWord, "counter layout shared with api.cu");
constexpr unsigned long long SLOT_HEAVY_MIN = 64ull * 1024;

struct SlotI {
  float4 p;
  float sx, sy, sz, cx, cy, cz;
  float px, py, pz;
};

// tab_base: shared-memory address of this lane's table copy minus bits(kMagic) * SLOT_REP * 8,
// so that segment t = bits(kMagic + t) - bits(kMagic) is at bits(kMagic + t) * SLOT_REP * 8 +
// tab_base (32-bit arithmetic modulo 2^32): one multiply-add per lookup.
// Positions are in units of sqrt(512) delta (relative to the slice's first particle), so |r|^2
// is xs = xi / 512, saturated to [0, 1]; the table holds f / (sqrt(512) delta) for the scaled
// difference vector, with the slopes times 512.
// EXACT (the reference's table-free short-range force, useSRForceTable = false, softening 0):
// positions in units of the cutoff, so xs = |r|^2 / re^2 saturated to [0, 1]; the smooth part
// R(r)/r of the force comes from a 499-segment table in xs, the Newton part -G/r^3 exactly from
// rsqrt: f = A[t] + xs S[t] + cn rsqrt(xs)^3, cn = -G m / re^2.  Segment 499 (xs = 1: at or
// beyond the cutoff) holds A = -cn r3(1) with r3(1) computed by the same instructions, so the
// two parts cancel there; |r|^2 starts from 1e-20 (not 0) so that the self pair (dx = dy = dz
// = 0) has a finite f.
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <bool EQM, bool EXACT>
__device__ __forceinline__ void slot_pair(SlotI& I, const float4& q, u32 tab_base, float cn) {
  const float dx = I.p.x - q.x, dy = I.p.y - q.y, dz = I.p.z - q.z;
  float xs;
  asm("fma.rn.sat.f32 %0, %1, %1, %2;" : "=f"(xs)
      : "f"(dz), "f"(fmaf(dy, dy, EXACT ? fmaf(dx, dx, 1e-20f) : dx * dx)));
  // kMagic + floor(512 xs) (table) or kMagic + floor(499 xs) (exact): one rounding of the exact
  // product, so the floor is exact
  const u32 bits = __float_as_uint(__fmaf_rd(xs, EXACT ? 499.0f : 512.0f, kMagic));
  float2 ab;
  asm("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(ab.x), "=f"(ab.y) : "r"(bits * (SLOT_REP * 8) + tab_base));
  float f = fmaf(xs, ab.y, ab.x);
  if (EXACT) {
    const float ri = rsqrt_approx(xs);
    f = fmaf(cn, ri * ri * ri, f);
  }
  if (!EQM) f *= q.w;
  I.px = fmaf(f, dx, I.px);
  I.py = fmaf(f, dy, I.py);
  I.pz = fmaf(f, dz, I.pz);
}

// First index in [lo, hi) whose y is >= v (UPPER = false) or > v (UPPER = true), found by the
// whole warp: each round probes 32 evenly spaced entries and keeps the one gap that holds the
// boundary, so a list of n entries takes about log32(n) rounds of loads.
template <bool UPPER>
__device__ __forceinline__ int warp_y_bound(const float4* __restrict__ pm, int lo, int hi, float v,
                                            int lane) {
  while (hi - lo > 32) {
    const int step = (hi - lo + 31) >> 5;
    const int idx = lo + lane * step;
    bool below = false;
    if (idx < hi) {
      const float y = __ldg(&pm[idx].y);
      below = UPPER ? (y <= v) : (y < v);
    }
    const int c = __popc(__ballot_sync(0xFFFFFFFFu, below));
    const int nlo = c > 0 ? lo + (c - 1) * step + 1 : lo;
    hi = min(hi, lo + c * step);
    lo = nlo;
  }
  const int idx = lo + lane;
  bool below = false;
  if (idx < hi) {
    const float y = __ldg(&pm[idx].y);
    below = UPPER ? (y <= v) : (y < v);
  }
  return lo + __popc(__ballot_sync(0xFFFFFFFFu, below));
}

// Estimated time of a unit for its warp: SLOT_SLICE times the neighbour cell's particles (the
// lanes run every candidate of the window whether or not all of them hold a particle, so a
// partial slice costs as much as a full one).  On the disk workloads a unit against the bulge
// can come close to a warp's whole share of the pass, and a warp holding one at the end leaves
// the GPU idle.
__device__ __forceinline__ unsigned long long slot_cost(const int* __restrict__ cell_start,
                                                        const ChainDimsP& cd, int2 item, int k) {
  const int sub2 = cd.sub * cd.sub;
  const int cell = item.x / sub2;
  if (cell >= cd.ncells) return 0;
  const int gx = cell % cd.Mx, gy = (cell / cd.Mx) % cd.My, gz = cell / (cd.Mx * cd.My);
  const int nx = gx + k % 3 - 1, ny = gy + (k / 3) % 3 - 1, nz = gz + k / 9 - 1;
  if (nx < 0 || ny < 0 || nz < 0 || nx >= cd.Mx || ny >= cd.My || nz >= cd.Mz) return 0;
  const int nb = nx + ny * cd.Mx + nz * cd.Mx * cd.My;
  return (unsigned long long)SLOT_SLICE *
         (unsigned long long)(__ldg(&cell_start[(nb + 1) * sub2]) - __ldg(&cell_start[nb * sub2]));
}

// rsqrt.approx of 1 and its cube as the exact-mode pass computes them (rsqrt_approx, then two
// multiplies).
__global__ void rsqrt_one_kernel(float* out) {
  const float r1 = rsqrt_approx(1.0f);
  out[0] = r1;
  out[1] = r1 * r1 * r1;
}

// Per-launch constants of the table pass.
struct SlotCtx {
  const float4* __restrict__ pm;
  const int* __restrict__ cell_start;
  const int2* __restrict__ items;
  float4* __restrict__ slots;
  int n;
  ChainDimsP cd;
  float re2, sc, gap_margin;
  int ysort;
  float cn;  // EXACT: Newton coefficient -G m / re^2 in the scaled coordinates
  // symmetric part of the pass (null when off): bit k sub^2 + q of sub-column a's sym_words
  // words marks neighbour sub-column q of direction k as evaluated by the symmetric units instead
  const u32* __restrict__ sym_masks;
  int sym_words;
};

// One work unit: the slice items[it / 27] against neighbour cell it % 27, into slot k of the
// slice's particles.  COOP: every warp of the CTA takes the unit, warp w the candidate chunks
// c = w, w + SLOT_WARPS, ... (chunks of 32 counted across the neighbour's sub-columns), and the
// warps' partial sums are added in warp order through shared memory (part: SLOT_WARPS x
// SLOT_SLICE), so the result does not depend on timing.
template <bool EQM, bool EXACT, bool COOP>
__device__ __forceinline__ void slot_unit(const SlotCtx& c, u32 it, float4 (*jbuf)[32], float4* part,
                                          u32 tab_base, int lane, int warp) {
  const ChainDimsP& cd = c.cd;
  const int sub = cd.sub, sub2 = sub * sub;
  const int2 item = c.items[it / NNB];
  const int k = (int)(it % NNB);
  const int cell = item.x / sub2;
  const int cend = c.cell_start[item.x + 1];
  const int last = min(item.y + SLOT_SLICE - 1, cend - 1);
  SlotI I[SLOT_IPL];
#pragma unroll
  for (int u = 0; u < SLOT_IPL; ++u) {
    const int i = item.y + 32 * u + lane;
    I[u].p = c.pm[i < cend ? i : last];
    I[u].sx = I[u].sy = I[u].sz = I[u].cx = I[u].cy = I[u].cz = 0.f;
  }
  if (cell < cd.ncells) {
    const int gx = cell % cd.Mx, gy = (cell / cd.Mx) % cd.My, gz = cell / (cd.Mx * cd.My);
    const int nx = gx + k % 3 - 1, ny = gy + (k / 3) % 3 - 1, nz = gz + k / 9 - 1;
    // the slice's sub-column: x and z ranges in code units
    const int isx = item.x % sub, isz = (item.x / sub) % sub;
    const float ix0 = (gx * sub + isx) * cd.HCsx, iz0 = (gz * sub + isz) * cd.HCsz;
    // y range of the slice: its first particle (lane 0, u = 0) and its last one
    const float ys0 = __shfl_sync(0xFFFFFFFFu, I[0].p.y, 0);
    const float ys1 = __ldg(&c.pm[last].y);
    // origin of the scaled coordinates: the slice's first particle (near every pair's ends, so
    // the differences keep the precision of code-unit differences)
    const float ox = __shfl_sync(0xFFFFFFFFu, I[0].p.x, 0), oz = __shfl_sync(0xFFFFFFFFu, I[0].p.z, 0);
    const float sc = c.sc;
#pragma unroll
    for (int u = 0; u < SLOT_IPL; ++u) {
      I[u].p.x = (I[u].p.x - ox) * sc;
      I[u].p.y = (I[u].p.y - ys0) * sc;
      I[u].p.z = (I[u].p.z - oz) * sc;
    }
    int chunk = 0;  // COOP: candidate chunks met so far in this unit
    const bool nin = nx >= 0 && ny >= 0 && nz >= 0 && nx < cd.Mx && ny < cd.My && nz < cd.Mz;
    // the candidates [b, e) of neighbour sub-column qs (false: out of reach or taken by the
    // symmetric units); a warp-collective search
    auto qwin = [&](int qs, int& b, int& e) -> bool {
      const int jsx = qs % sub, jsz = qs / sub;
      const float jx0 = (nx * sub + jsx) * cd.HCsx, jz0 = (nz * sub + jsz) * cd.HCsz;
      const float gxs = fmaxf(fmaxf(jx0 - (ix0 + cd.HCsx), ix0 - (jx0 + cd.HCsx)) - c.gap_margin, 0.f);
      const float gzs = fmaxf(fmaxf(jz0 - (iz0 + cd.HCsz), iz0 - (jz0 + cd.HCsz)) - c.gap_margin, 0.f);
      const float g2 = gxs * gxs + gzs * gzs;
      if (g2 >= c.re2) return false;
      if (c.sym_masks) {
        const int sb = k * sub2 + qs;
        if ((__ldg(&c.sym_masks[(size_t)item.x * c.sym_words + (sb >> 5)]) >> (sb & 31)) & 1u) return false;
      }
      // a pair in range has |dy|^2 < re^2 - (its x-z distance)^2 <= re^2 - g2: the y window
      // of this sub-column is the chord of the cutoff sphere at the sub-column's x-z gap, widened
      // by 1e-5 of the coordinates' size against float rounding of the comparisons
      const float h = sqrtf(c.re2 - g2) + 1e-5f * (1.f + fabsf(ys1));
      const int cn = (nx + ny * cd.Mx + nz * cd.Mx * cd.My) * sub2 + qs;
      b = c.cell_start[cn];
      e = c.cell_start[cn + 1];
      if (c.ysort && e > b) {
        b = warp_y_bound<false>(c.pm, b, e, ys0 - h, lane);
        e = warp_y_bound<true>(c.pm, b, e, ys1 + h, lane);
      }
      return true;
    };
    // COOP: the warps find the sub-columns' windows once for the CTA (warp w those of sub-columns
    // w, w + SLOT_WARPS), instead of every warp searching all of them
    __shared__ int2 s_qwin[32];
    if (COOP && nin) {
      for (int qs = warp; qs < sub2; qs += SLOT_WARPS) {
        int b = 0, e = 0;
        if (!qwin(qs, b, e)) b = e = 0;
        if (lane == 0) s_qwin[qs] = make_int2(b, e);
      }
      __syncthreads();
    }
    if (nin)
    for (int qs = 0; qs < sub2; ++qs) {
      int b, e;
      if (COOP) {
        const int2 w = s_qwin[qs];
        b = w.x;
        e = w.y;
        if (e <= b) continue;
      } else if (!qwin(qs, b, e)) {
        continue;
      }
      // COOP: this warp's chunks of the window are c = first, first + SLOT_WARPS, ... where
      // chunk + first = warp (mod SLOT_WARPS)
      int j0 = b, jstep = 32;
      if (COOP) {
        j0 = b + 32 * ((warp - chunk) & (SLOT_WARPS - 1));
        jstep = 32 * SLOT_WARPS;
        chunk += (e - b + 31) >> 5;
      }
      for (; j0 < e; j0 += jstep) {
        const int jj = j0 + lane;
        float4 qj = jj < e ? c.pm[jj] : make_float4(3.0e30f, 3.0e30f, 3.0e30f, 0.f);
        qj.x = (qj.x - ox) * sc;
        qj.y = (qj.y - ys0) * sc;
        qj.z = (qj.z - oz) * sc;
        jbuf[warp][lane] = qj;
        __syncwarp();
        const int cnt = min(32, e - j0);
#pragma unroll
        for (int u = 0; u < SLOT_IPL; ++u) I[u].px = I[u].py = I[u].pz = 0.f;
        // 4 candidates per iteration: the kernel also holds the symmetric units' code, and
        // shorter loop bodies keep the instruction cache warm (1,048,576-particle disk, reduced / full
        // cutoff: 28.0 / 76.7 ms at 16, 27.8 / 75.6 at 8, 27.3 / 75.3 at 4, 27.7 / 75.7 at 2;
        // 262,144-particle disk 5.97 / 5.92 / 5.97 / 6.06 ms; 4 deep already with the tail
        // group of the symmetric windows run as a full group)
        if constexpr (!EXACT) {
          // the table: whole groups of 4 (no remainder loop), the staged entries past the
          // window being far-away points whose |r|^2 saturates to the zero segments (or whose
          // mass is 0): they add exactly nothing (262,144-particle disk 5.72 -> 5.60 ms)
          const int cnt4 = (cnt + 3) & ~3;
#pragma unroll 1
          for (int s = 0; s < cnt4; s += 4) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              const float4 q = jbuf[warp][s + t];
#pragma unroll
              for (int u = 0; u < SLOT_IPL; ++u) slot_pair<EQM, EXACT>(I[u], q, tab_base, c.cn);
            }
          }
        } else {
#pragma unroll 4
          for (int s = 0; s < cnt; ++s) {
            const float4 q = jbuf[warp][s];
#pragma unroll
            for (int u = 0; u < SLOT_IPL; ++u) slot_pair<EQM, EXACT>(I[u], q, tab_base, c.cn);
          }
        }
        __syncwarp();
#pragma unroll
        for (int u = 0; u < SLOT_IPL; ++u) {
          kahan_add(I[u].sx, I[u].cx, I[u].px);
          kahan_add(I[u].sy, I[u].cy, I[u].py);
          kahan_add(I[u].sz, I[u].cz, I[u].pz);
        }
      }
    }
  }
  if (!COOP) {
#pragma unroll
    for (int u = 0; u < SLOT_IPL; ++u) {
      const int i = item.y + 32 * u + lane;
      if (i < cend) c.slots[(size_t)k * c.n + i] = make_float4(I[u].sx, I[u].sy, I[u].sz, 0.f);
    }
  } else {
#pragma unroll
    for (int u = 0; u < SLOT_IPL; ++u)
      part[warp * SLOT_SLICE + 32 * u + lane] = make_float4(I[u].sx, I[u].sy, I[u].sz, 0.f);
    __syncthreads();
    if (threadIdx.x < SLOT_SLICE) {
      float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll 4
      for (int w = 0; w < SLOT_WARPS; ++w) {
        const float4 v = part[w * SLOT_SLICE + threadIdx.x];
        kahan_add(sx, cx, v.x);
        kahan_add(sy, cy, v.y);
        kahan_add(sz, cz, v.z);
      }
      const int i = item.y + (int)threadIdx.x;
      if (i < cend) c.slots[(size_t)k * c.n + i] = make_float4(sx, sy, sz, 0.f);
    }
    __syncthreads();
  }
}

// ------------------------------------------------ symmetric sub-column pairs ------------
// The reference evaluates each pair once (half shell of 13 neighbour cells, the j side written
// to per-neighbour slots of j: source/p3mMethod.cpp:247-273, 296-322).  Here the same holds for
// the dense sub-column pairs (p, q): both lists non-empty, the larger at least SYM_MIN_BIG
// particles and the smaller SYM_MIN_SMALL, x-z gap below the cutoff, |p| |q| below
// SYM_CTA_MUL heavy thresholds of the one-sided pass (denser pairs stay one-sided, where whole
// CTAs share their units).  One unit per such pair (listed from its upper-half side: direction
// k > 13, or k = 13 and the higher local index); its i side p is the larger list, its j side q.
// The unit runs p's 128-particle slices (4 per lane) against their y windows in q and writes
//   * the i side into slot (k, local index of q) of p's particles (one store per slice), and
//   * the j side into slot (26 - k, local index of p) of q's particles: the lanes' products for
//     4 candidates are summed across the warp by a transposing butterfly of 18 shuffles (no
//     selects: the lanes visit the 4 candidates of a group in an order swizzled by lane bits 4
//     and 3, so that every lane sends and keeps the same registers), each lane keeping one
//     candidate's total per chunk of 32, added to the slot (cleared at the unit's start;
//     read-modify-written by one warp at a time, in slice order).
// Units of cost |p| |q| >= 1/2 of the heavy threshold are taken by whole CTAs (the warps split each
// window's chunks, the i sides added in warp order through shared memory), the rest by warps.
// Every slot has one writer at a time and a fixed summation order: the result is deterministic.
// The one-sided pass skips the pairs marked in the sub-column's mask and the epilogue adds the
// marked slots after each direction's one-sided slot.  Equal masses only (the mass is folded in
// the table); sampled passes stay one-sided.
constexpr int SYM_IPL = 4;                // i particles per lane
constexpr int SYM_SLICE = 32 * SYM_IPL;   // particles per slice of a unit's i side
constexpr int SYM_MIN_BIG = 128;          // the larger list of a symmetric pair, at least
constexpr int SYM_MIN_SMALL = 8;          // the smaller one, at least
constexpr unsigned long long SYM_CTA_MUL = 16;  // |p| |q| below 16 heavy thresholds

struct SymI {
  float x, y, z;
  float sx, sy, sz, cx, cy, cz;
  float px, py, pz;
};

// Squared x-z gap between sub-columns (cell x gx, z gz, local ca) and (nx, nz, cb), computed the
// same way in either order (min / max, no contraction), so that the marks are symmetric.
__device__ __forceinline__ float sym_gap2(const ChainDimsP& cd, int gx, int gz, int ca, int nx, int nz, int cb,
                                          float margin) {
  const float ax = (float)(gx * cd.sub + ca % cd.sub) * cd.HCsx, az = (float)(gz * cd.sub + ca / cd.sub) * cd.HCsz;
  const float bx = (float)(nx * cd.sub + cb % cd.sub) * cd.HCsx, bz = (float)(nz * cd.sub + cb / cd.sub) * cd.HCsz;
  const float gxs = fmaxf(__fsub_rn(__fsub_rn(fmaxf(ax, bx), __fadd_rn(fminf(ax, bx), cd.HCsx)), margin), 0.f);
  const float gzs = fmaxf(__fsub_rn(__fsub_rn(fmaxf(az, bz), __fadd_rn(fminf(az, bz), cd.HCsz)), margin), 0.f);
  return __fadd_rn(__fmul_rn(gxs, gxs), __fmul_rn(gzs, gzs));
}

// The L mark bits of direction k (bits k L .. k L + L - 1) in the mask words w.
template <int L>
__device__ __forceinline__ u32 sym_field(const u32 (&w)[sym_mark_words(L) + 1], int k) {
  static_assert(L < 32, "a direction's marks must fit one word");
  const int lo = k * L, t = lo >> 5, off = lo & 31;
  u32 field = w[t] >> off;
  if (off + L > 32 && t + 1 < sym_mark_words(L)) field |= w[t + 1] << (32 - off);
  return field & ((1u << L) - 1u);
}

// True if nothing one-sided is left between sub-column a and neighbour cell k (every one of its
// sub-columns empty, out of reach in x-z or taken by the symmetric units): the one-sided unit is
// skipped and its slot not read.
__device__ __forceinline__ bool sym_dead(const u32* __restrict__ masks, int words, int a, int k) {
  return (__ldg(&masks[(size_t)a * words + words - 1]) >> k) & 1u;
}

// Marks and units, one warp at a time per sub-column a (a = nsub: the bucket outside the mesh, no
// marks; the warps stride over the sub-columns, most of which are empty or sparse); lane l of
// round t looks at mark bit 32 t + l (direction k, neighbour sub-column cb), so a round's ballot
// is one mask word.
// Each unit is staged as (p, q, bucket, position in its bucket); sym_scatter_kernel then lays
// the buckets out one after the other in units.  If more than cap units are listed, the pass
// runs one-sided.
__device__ __forceinline__ int sym_bucket(unsigned long long c, unsigned long long thr) {
  if (2 * c >= thr) return c >= 8 * thr ? 0 : c >= 2 * thr ? 1 : c >= thr ? 2 : 3;
  return 4 * c >= thr ? 4 : 8 * c >= thr ? 5 : 16 * c >= thr ? 6 : 32 * c >= thr ? 7 : 8;
}

template <int L>
__global__ void sym_plan_kernel(const int* __restrict__ cs, ChainDimsP cd, int nsub, float re2, float margin,
                                u32* __restrict__ masks, uint4* __restrict__ stage, u32 cap,
                                u32* __restrict__ counter, const int* __restrict__ stop) {
  constexpr int MW = sym_mark_words(L) + 1;
  static_assert(MW <= 32, "one mask word per lane");
  if (*stop) return;
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int a = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); a <= nsub; a += nwarps) {
    const int pa = a < nsub ? __ldg(&cs[a + 1]) - __ldg(&cs[a]) : 0;
    u32 word = 0u;  // lane t < MW - 1: mark word t; lane MW - 1: the dead directions
    if (pa >= SYM_MIN_SMALL) {
      const unsigned long long thr = __ldcg(reinterpret_cast<const unsigned long long*>(counter + 6));
      const int cell = a / L, ca = a % L;
      const int gx = cell % cd.Mx, gy = (cell / cd.Mx) % cd.My, gz = cell / (cd.Mx * cd.My);
      u32 alive = 0u;  // bit k: something one-sided left toward neighbour cell k (this lane's bits)
#pragma unroll 1
      for (int t = 0; t < MW - 1; ++t) {
        const int sb = 32 * t + lane;
        bool marked = false;
        if (sb < NNB * L) {
          const int k = sb / L, cb = sb % L;
          const int nx = gx + k % 3 - 1, ny = gy + (k / 3) % 3 - 1, nz = gz + k / 9 - 1;
          if (nx >= 0 && ny >= 0 && nz >= 0 && nx < cd.Mx && ny < cd.My && nz < cd.Mz) {
            const int b = (nx + ny * cd.Mx + nz * cd.Mx * cd.My) * L + cb;
            const int pb = b == a ? 0 : __ldg(&cs[b + 1]) - __ldg(&cs[b]);
            if (b == a) {
              alive |= 1u << k;
            } else if (pb > 0 && sym_gap2(cd, gx, gz, ca, nx, nz, cb, margin) < re2) {
              const unsigned long long cost = (unsigned long long)pa * (unsigned long long)pb;
              if (pb < SYM_MIN_SMALL || max(pa, pb) < SYM_MIN_BIG || cost >= thr * SYM_CTA_MUL) {
                alive |= 1u << k;
              } else {
                marked = true;
                if (k > 13 || (k == 13 && cb > ca)) {
                  const int bk = sym_bucket(cost, thr);
                  const u32 pos = atomicAdd(&counter[SLOT_SYM_COUNT + bk], 1u);
                  const u32 idx = atomicAdd(&counter[SLOT_SYM_TOTAL], 1u);
                  if (idx < cap)
                    stage[idx] = pa >= pb ? make_uint4((u32)a, (u32)b, (u32)bk, pos)
                                          : make_uint4((u32)b, (u32)a, (u32)bk, pos);
                }
              }
            }
          }
        }
        const u32 bits = __ballot_sync(0xFFFFFFFFu, marked);
        if (lane == t) word = bits;
      }
      // a direction with nothing one-sided left (out of the mesh, or every sub-column empty, out
      // of reach or marked) is dead
      const u32 alive_all = __reduce_or_sync(0xFFFFFFFFu, alive);
      if (lane == MW - 1) word = ~alive_all & ((1u << NNB) - 1u);
    }
    if (lane < MW) masks[(size_t)a * MW + lane] = word;
  }
}

// subcol[i] = the sub-column (or the outside bucket) of sorted particle i.
__global__ void subcol_kernel(const int* __restrict__ cs, const int2* __restrict__ items,
                              const u32* __restrict__ nitems_p, int* __restrict__ subcol,
                              const int* __restrict__ stop) {
  if (*stop) return;
  const u32 it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= *nitems_p) return;
  const int2 item = items[it];
  const int end = min(item.y + SLOT_SLICE, cs[item.x + 1]);
  for (int i = item.y; i < end; ++i) subcol[i] = item.x;
}

// Start of each bucket in the laid-out unit list (exclusive prefix of the bucket counts).
__device__ __forceinline__ u32 sym_bucket_start(const u32* __restrict__ counter, int b) {
  u32 off = 0;
#pragma unroll
  for (int i = 0; i < SYM_NB; ++i)
    if (i < b) off += __ldcg(&counter[SLOT_SYM_COUNT + i]);
  return off;
}

// Lays the staged units out bucket after bucket (positions within a bucket as staged).
__global__ void sym_scatter_kernel(const uint4* __restrict__ stage, uint2* __restrict__ units, u32 cap,
                                   const u32* __restrict__ counter, const int* __restrict__ stop) {
  if (*stop) return;
  const u32 total = __ldcg(&counter[SLOT_SYM_TOTAL]);
  if (total > cap) return;
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const uint4 e = stage[i];
    units[sym_bucket_start(counter, (int)e.z) + e.w] = make_uint2(e.x, e.y);
  }
}

// One candidate q against the lane's SYM_IPL i particles: their sums accumulate as in slot_pair;
// v = the sum of the pair forces f d, the candidate's share of its j side (negated later).
// MASKED: each force is multiplied by w[u] (0 for lanes past a slice's end, which hold copies
// of its last particle and may not reach a sum).
template <bool EXACT, bool MASKED>
__device__ __forceinline__ void sym_pair(SymI (&I)[SYM_IPL], const float4& q, u32 tab_base, float cn,
                                         const float (&w)[SYM_IPL], float (&v)[3]) {
#pragma unroll
  for (int u = 0; u < SYM_IPL; ++u) {
    const float dx = I[u].x - q.x, dy = I[u].y - q.y, dz = I[u].z - q.z;
    float xs;
    asm("fma.rn.sat.f32 %0, %1, %1, %2;" : "=f"(xs)
        : "f"(dz), "f"(fmaf(dy, dy, EXACT ? fmaf(dx, dx, 1e-20f) : dx * dx)));
    const u32 bits = __float_as_uint(__fmaf_rd(xs, EXACT ? 499.0f : 512.0f, kMagic));
    float2 ab;
    asm("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(ab.x), "=f"(ab.y) : "r"(bits * (SLOT_REP * 8) + tab_base));
    float f = fmaf(xs, ab.y, ab.x);
    if (EXACT) {
      const float ri = rsqrt_approx(xs);
      f = fmaf(cn, ri * ri * ri, f);
    }
    if (MASKED) f *= w[u];
    I[u].px = fmaf(f, dx, I[u].px);
    I[u].py = fmaf(f, dy, I[u].py);
    I[u].pz = fmaf(f, dz, I[u].pz);
    if (u == 0) {
      v[0] = f * dx;
      v[1] = f * dy;
      v[2] = f * dz;
    } else {
      v[0] = fmaf(f, dx, v[0]);
      v[1] = fmaf(f, dy, v[1]);
      v[2] = fmaf(f, dz, v[2]);
    }
  }
}

// The candidates [jb, je) of q against the slice in I (scaled coordinates, origin (ox, ys0, oz)):
// i sides into I's sums, j sides read-modified-written in sj.  COOP: this warp takes the chunks
// warp, warp + SLOT_WARPS, ... of the window.
template <bool EXACT, bool MASKED, bool COOP>
__device__ __forceinline__ void sym_window(const SlotCtx& c, SymI (&I)[SYM_IPL], const float (&w)[SYM_IPL],
                                           int jb, int je, float ox, float ys0, float oz, float4* __restrict__ sj,
                                           float4 (*jbuf)[32], u32 tab_base, int lane, int warp) {
  const int swz = (lane >> 3) & 3;     // candidate order within a group of 4: m ^ swz
  const int own = 4 * (lane & 7) + swz;  // this lane's candidate total of each chunk
  const float sc = c.sc;
  const int jstep = COOP ? 32 * SLOT_WARPS : 32;
  for (int j0 = jb + (COOP ? 32 * warp : 0); j0 < je; j0 += jstep) {
    const int jj = j0 + lane;
    float4 qj = jj < je ? c.pm[jj] : make_float4(3.0e30f, 3.0e30f, 3.0e30f, 0.f);
    qj.x = (qj.x - ox) * sc;
    qj.y = (qj.y - ys0) * sc;
    qj.z = (qj.z - oz) * sc;
    jbuf[warp][lane] = qj;
    const int jo = j0 + own;
    const float4 old = jo < je ? sj[jo] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    const int cnt = min(32, je - j0);
#pragma unroll
    for (int u = 0; u < SYM_IPL; ++u) I[u].px = I[u].py = I[u].pz = 0.f;
    float tx = 0.f, ty = 0.f, tz = 0.f;
    // a partial last group runs as a full one: the staged entries past the window are far-away
    // points (3e30), whose |r|^2 saturates to the table's last segment, where the force is
    // exactly 0 (the table: segments 499.. are zero; exact mode: the Newton term and segment
    // 499's constant cancel exactly, which the handle checks before it enables this part), so
    // they add nothing to the i sides, and their j sides are never stored
#pragma unroll 1
    for (int g = 0; 4 * g < cnt; ++g) {
      float v[4][3];
#pragma unroll
      for (int m = 0; m < 4; ++m)
        sym_pair<EXACT, MASKED>(I, jbuf[warp][4 * g + (m ^ swz)], tab_base, c.cn, w, v[m]);
      // lanes l and l ^ 16 hold each other's slots 2, 3 in their slots 0, 1 (swz differs in bit
      // 1), lanes l and l ^ 8 each other's slot 1 in their slot 0 (bit 0); then bits 2..0
      float x[3];
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        const float w0 = v[0][cc] + __shfl_xor_sync(0xFFFFFFFFu, v[2][cc], 16);
        const float w1 = v[1][cc] + __shfl_xor_sync(0xFFFFFFFFu, v[3][cc], 16);
        float t = w0 + __shfl_xor_sync(0xFFFFFFFFu, w1, 8);
        t += __shfl_xor_sync(0xFFFFFFFFu, t, 4);
        t += __shfl_xor_sync(0xFFFFFFFFu, t, 2);
        t += __shfl_xor_sync(0xFFFFFFFFu, t, 1);
        x[cc] = t;
      }
      if ((lane & 7) == g) {
        tx = x[0];
        ty = x[1];
        tz = x[2];
      }
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < SYM_IPL; ++u) {
      kahan_add(I[u].sx, I[u].cx, I[u].px);
      kahan_add(I[u].sy, I[u].cy, I[u].py);
      kahan_add(I[u].sz, I[u].cz, I[u].pz);
    }
    if (jo < je) sj[jo] = make_float4(old.x - tx, old.y - ty, old.z - tz, 0.f);
    __syncwarp();
  }
}

// One symmetric unit (i side p, j side q) by one warp, or by the whole CTA (COOP; part:
// SLOT_WARPS x SYM_SLICE partial sums).
template <bool EXACT, bool COOP>
__device__ __forceinline__ void sym_unit(const SlotCtx& c, float4* __restrict__ sym_slots, uint2 unit,
                                         float4 (*jbuf)[32], float4* part, u32 tab_base, int lane, int warp) {
  const ChainDimsP& cd = c.cd;
  const int p = (int)unit.x, q = (int)unit.y;
  const int L = cd.sub * cd.sub;
  const int cp = p / L, ca = p % L, cq = q / L, cb = q % L;
  const int gx = cp % cd.Mx, gy = (cp / cd.Mx) % cd.My, gz = cp / (cd.Mx * cd.My);
  const int nx = cq % cd.Mx, ny = (cq / cd.Mx) % cd.My, nz = cq / (cd.Mx * cd.My);
  const int k = (nx - gx + 1) + 3 * (ny - gy + 1) + 9 * (nz - gz + 1);
  float4* __restrict__ si = sym_slots + (size_t)(k * L + cb) * c.n;
  float4* __restrict__ sj = sym_slots + (size_t)((NNB - 1 - k) * L + ca) * c.n;
  const float h0 = sqrtf(c.re2 - sym_gap2(cd, gx, gz, ca, nx, nz, cb, c.gap_margin));
  const int bb = c.cell_start[q], be = c.cell_start[q + 1];
  const int p0 = c.cell_start[p], cend = c.cell_start[p + 1];
  // the y window in q of the slice starting at i0: the cutoff chord at the sub-columns' gap
  // around the slice's y range, widened by 1e-5 of the coordinates' size against float rounding
  auto window = [&](int i0, int& jb, int& je) {
    const float ys0 = __ldg(&c.pm[i0].y), ys1 = __ldg(&c.pm[min(i0 + SYM_SLICE - 1, cend - 1)].y);
    const float h = h0 + 1e-5f * (1.f + fabsf(ys1));
    jb = bb;
    je = be;
    if (c.ysort && je > jb) {
      jb = warp_y_bound<false>(c.pm, jb, je, ys0 - h, lane);
      je = warp_y_bound<true>(c.pm, jb, je, ys1 + h, lane);
    }
  };
  // COOP: one warp finds each slice's window for the whole CTA (the first before the unit's
  // barrier, the next while four other warps add up the current slice's i sides) instead of
  // every warp searching the same one
  __shared__ int s_win[2];
  constexpr int WIN_WARP = SLOT_WARPS - 1;
  if (COOP) {
    for (int j = bb + (int)threadIdx.x; j < be; j += SLOT_THREADS) sj[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (warp == WIN_WARP) {
      int jb, je;
      window(p0, jb, je);
      if (lane == 0) {
        s_win[0] = jb;
        s_win[1] = je;
      }
    }
    __syncthreads();
  } else {
    for (int j = bb + lane; j < be; j += 32) sj[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
  }
  const float sc = c.sc;
  for (int i0 = p0; i0 < cend; i0 += SYM_SLICE) {
    const int last = min(i0 + SYM_SLICE - 1, cend - 1);
    SymI I[SYM_IPL];
    float w[SYM_IPL];
#pragma unroll
    for (int u = 0; u < SYM_IPL; ++u) {
      const int i = i0 + 32 * u + lane;
      const float4 pi = c.pm[i < cend ? i : last];
      I[u].x = pi.x;
      I[u].y = pi.y;
      I[u].z = pi.z;
      I[u].sx = I[u].sy = I[u].sz = I[u].cx = I[u].cy = I[u].cz = 0.f;
      w[u] = i < cend ? 1.f : 0.f;
    }
    const float ys0 = __shfl_sync(0xFFFFFFFFu, I[0].y, 0);
    const float ys1 = __ldg(&c.pm[last].y);
    const float ox = __shfl_sync(0xFFFFFFFFu, I[0].x, 0), oz = __shfl_sync(0xFFFFFFFFu, I[0].z, 0);
#pragma unroll
    for (int u = 0; u < SYM_IPL; ++u) {
      I[u].x = (I[u].x - ox) * sc;
      I[u].y = (I[u].y - ys0) * sc;
      I[u].z = (I[u].z - oz) * sc;
    }
    int jb, je;
    if (COOP) {
      jb = s_win[0];
      je = s_win[1];
    } else {
      window(i0, jb, je);
    }
    if (i0 + SYM_SLICE <= cend)
      sym_window<EXACT, false, COOP>(c, I, w, jb, je, ox, ys0, oz, sj, jbuf, tab_base, lane, warp);
    else
      sym_window<EXACT, true, COOP>(c, I, w, jb, je, ox, ys0, oz, sj, jbuf, tab_base, lane, warp);
    if (!COOP) {
#pragma unroll
      for (int u = 0; u < SYM_IPL; ++u) {
        const int i = i0 + 32 * u + lane;
        if (i < cend) si[i] = make_float4(I[u].sx, I[u].sy, I[u].sz, 0.f);
      }
    } else {
#pragma unroll
      for (int u = 0; u < SYM_IPL; ++u)
        part[warp * SYM_SLICE + 32 * u + lane] = make_float4(I[u].sx, I[u].sy, I[u].sz, 0.f);
      __syncthreads();
      if (warp == WIN_WARP && i0 + SYM_SLICE < cend) {  // the next slice's window
        int jb2, je2;
        window(i0 + SYM_SLICE, jb2, je2);
        if (lane == 0) {
          s_win[0] = jb2;
          s_win[1] = je2;
        }
      }
      if (threadIdx.x < SYM_SLICE) {
        float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll 4
        for (int ww = 0; ww < SLOT_WARPS; ++ww) {
          const float4 v = part[ww * SYM_SLICE + threadIdx.x];
          kahan_add(sx, cx, v.x);
          kahan_add(sy, cy, v.y);
          kahan_add(sz, cz, v.z);
        }
        const int i = i0 + (int)threadIdx.x;
        if (i < cend) si[i] = make_float4(sx, sy, sz, 0.f);
      }
      __syncthreads();
    }
  }
}

// The lane-replicated force table of the slotted passes, in shared memory (tab_all, SLOT_TAB x
// SLOT_REP float2), with the coordinate scale sc and, exact mode, the Newton coefficient cn.
template <bool EQM, bool EXACT>
__device__ __forceinline__ void slot_table_setup(const float4* __restrict__ pm, const PairParams& pp,
                                                 const float* __restrict__ table, float2* tab_all,
                                                 float& sc_out, float& cn_out) {
  // table: coordinates are scaled by sc = 1/(sqrt(512) delta) (512 sc^2 = 1/delta^2 to float
  // rounding); exact: by sc = 1/re
  const float sc = EXACT ? 1.0f / pp.re : (float)sqrt((double)pp.inv_d2 / 512.0);
  const double mj = EQM ? (double)__ldg(&pm[0].w) : 1.0;
  float cn = 0.f;
  if (!EXACT) {
    // every particle has the same mass when EQM: fold it into the table, with 1/sc
    const double mjs = mj / (double)sc;
    for (int t = threadIdx.x; t < SLOT_TAB; t += (int)blockDim.x) {
      float2 ab = make_float2(0.f, 0.f);
      if (t < 499) {
        const float a = table[t];
        const float s = table[t + 1] - a;
        const double A = (double)a - (double)t * (double)s;
        ab = make_float2((float)(A * mjs), (float)((double)s * 512.0 * mjs));
      }
#pragma unroll
      for (int c = 0; c < SLOT_REP; ++c) tab_all[t * SLOT_REP + c] = ab;
    }
  } else {
    // smooth part g = R(r)/r at r^2 = t delta (table[500 + t], double-computed on the host),
    // times m re, linear in xs = t / 499 per segment; segment 499 cancels the Newton part
    const double G = 1.0 / (4.0 * 3.14159265358979323846), re = pp.re;
    cn = (float)(-G * mj / (re * re));
    const float r1 = rsqrt_approx(1.0f);
    const float c499 = -(cn * (r1 * r1 * r1));
    const double w = mj * re;
    for (int t = threadIdx.x; t < SLOT_TAB; t += (int)blockDim.x) {
      float2 ab = make_float2(0.f, 0.f);
      if (t < 499) {
        const double g0 = table[500 + t], g1 = table[500 + t + 1];
        ab = make_float2((float)((g0 - (double)t * (g1 - g0)) * w), (float)((g1 - g0) * 499.0 * w));
      } else if (t == 499) {
        ab = make_float2(c499, 0.f);
      }
#pragma unroll
      for (int c = 0; c < SLOT_REP; ++c) tab_all[t * SLOT_REP + c] = ab;
    }
  }
  sc_out = sc;
  cn_out = cn;
}

// The slotted pass, one persistent CTA per SM.  The heavy one-sided units listed by
// plan_heavy_kernel (heavy[0, counter[2]), cost at least the threshold thr in counter[6..7]) are
// taken first, each by a whole CTA (counter[0]), so that no single warp is left with a unit of
// tens of thousands of candidates per particle while the others idle; then (equal masses, when
// the symmetric part is on) the symmetric units of CTAs, longest bucket first; then every warp
// takes the two longest buckets of symmetric warp units, the medium one-sided units (cost in
// [thr / 4, thr), listed from the far end of the heavy buffer, counter[1]), the other symmetric
// units, and the rest of the one-sided units in unit order (counter[8]).  If the heavy lists
// overflowed their buffer, every one-sided unit is taken by the last loop; if the symmetric
// list overflowed, the pass is one-sided.
template <bool EQM, bool EXACT>
__global__ void __maxnreg__(128) pair_slot_kernel(
    const float4* __restrict__ pm, int n, const int* __restrict__ cell_start,
    const int2* __restrict__ items, const u32* __restrict__ nitems_p, const u32* __restrict__ heavy,
    u32 heavy_cap, u32* __restrict__ counter, ChainDimsP cd, PairParams pp, const float* __restrict__ table,
    float4* __restrict__ slots, u32 unit_stride, const u32* __restrict__ sym_masks, int sym_words, u32 sym_cap,
    float4* __restrict__ sym_slots, const uint2* __restrict__ sym_units, const int* __restrict__ stop) {
  static_assert(SLOT_PART >= SLOT_SLICE && SLOT_PART >= SYM_SLICE, "partial-sum buffer too small");
  if (*stop) return;
  extern __shared__ float4 slot_smem[];
  __shared__ u32 s_unit;
  float4 (*jbuf)[32] = reinterpret_cast<float4 (*)[32]>(slot_smem);
  float4* part = slot_smem + SLOT_WARPS * 32;
  float2* tab_all = reinterpret_cast<float2*>(part + SLOT_WARPS * SLOT_PART);
  float sc, cn;
  slot_table_setup<EQM, EXACT>(pm, pp, table, tab_all, sc, cn);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const u32 tab_base = (u32)__cvta_generic_to_shared(tab_all + (lane & (SLOT_REP - 1))) -
                       __float_as_uint(kMagic) * (u32)(SLOT_REP * 8);
  // a neighbour sub-column is skipped when its x-z distance from the slice's sub-column is at
  // least the cutoff (with a margin far above the rounding of the sub-column assignment)
  const bool sym_on = EQM && sym_masks && __ldcg(&counter[SLOT_SYM_TOTAL]) <= sym_cap;
  const SlotCtx c{pm, cell_start, items, slots, n, cd, pp.re2, sc, 1e-3f * fminf(cd.HCsx, cd.HCsz), pp.ysort, cn,
                  sym_on ? sym_masks : nullptr, sym_words};
  const u32 nall = *nitems_p * NNB;  // every slice once per neighbour cell
  const u32 nh = __ldcg(&counter[2]), nm = __ldcg(&counter[3]);
  const bool listed = (unsigned long long)nh + nm <= heavy_cap;  // both lists complete
  const u32 nheavy = listed ? nh : 0u, nmedium = listed ? nm : 0u;
  const unsigned long long thr = __ldcg(reinterpret_cast<const unsigned long long*>(counter + 6));
  for (;;) {
    if (threadIdx.x == 0) s_unit = atomicAdd(&counter[0], 1u);
    __syncthreads();
    const u32 h = s_unit;
    __syncthreads();
    if (h >= nheavy) break;
    slot_unit<EQM, EXACT, true>(c, __ldg(&heavy[h]), jbuf, part, tab_base, lane, warp);
  }
  if constexpr (EQM) {
    if (sym_on) {  // the symmetric units of CTAs, longest bucket first
      for (int b = 0; b < SYM_NB_CTA; ++b) {
        const u32 cnt = __ldcg(&counter[SLOT_SYM_COUNT + b]), off = sym_bucket_start(counter, b);
        for (;;) {
          if (threadIdx.x == 0) s_unit = atomicAdd(&counter[SLOT_SYM_TAKEN + b], 1u);
          __syncthreads();
          const u32 h = s_unit;
          __syncthreads();
          if (h >= cnt) break;
          sym_unit<EXACT, true>(c, sym_slots, __ldg(&sym_units[off + h]), jbuf, part, tab_base, lane, warp);
        }
      }
    }
  }
  // warps: one loop with one call site per kind of unit, so that each unit's code is in the
  // kernel once (the instruction cache holds less).  Phases: 0 the two longest buckets of
  // symmetric units, 1 the medium one-sided units, 2 the other symmetric buckets, 3 the rest of
  // the one-sided units, SLOT_REST_BATCH per fetch (each lane tests one: sampled slice, not
  // listed, not a dead direction of the symmetric part), the live ones in unit order.
  const bool wsym = EQM && sym_on;
  int ph = wsym ? 0 : 1, b = SYM_NB_CTA;
  u32 live_m = 0u, base = 0u;
#pragma unroll 1
  for (;;) {
    if (ph == 0 || ph == 2) {
      if (b == (ph == 0 ? SYM_NB_CTA + 2 : SYM_NB)) {
        ++ph;
        continue;
      }
      u32 m = 0;
      if (lane == 0) m = atomicAdd(&counter[SLOT_SYM_TAKEN + b], 1u);
      m = __shfl_sync(0xFFFFFFFFu, m, 0);
      if (m >= __ldcg(&counter[SLOT_SYM_COUNT + b])) {
        ++b;
        continue;
      }
      if constexpr (EQM)
        sym_unit<EXACT, false>(c, sym_slots, __ldg(&sym_units[sym_bucket_start(counter, b) + m]), jbuf, part,
                               tab_base, lane, warp);
      continue;
    }
    u32 unit;
    if (ph == 1) {
      u32 m = 0;
      if (lane == 0) m = atomicAdd(&counter[1], 1u);
      m = __shfl_sync(0xFFFFFFFFu, m, 0);
      if (m >= nmedium) {
        ph = wsym ? 2 : 3;
        continue;
      }
      unit = __ldg(&heavy[heavy_cap - 1 - m]);
    } else {
      if (!live_m) {
        if (lane == 0) base = atomicAdd(&counter[8], (u32)SLOT_REST_BATCH);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= nall) break;
        const u32 it = base + lane;
        bool live = lane < SLOT_REST_BATCH && it < nall && (it / NNB) % unit_stride == 0;  // sampled: every stride-th slice
        if (live && listed) live = slot_cost(cell_start, cd, items[it / NNB], (int)(it % NNB)) < thr / 4;
        if (live && c.sym_masks) live = !sym_dead(c.sym_masks, c.sym_words, items[it / NNB].x, (int)(it % NNB));
        live_m = __ballot_sync(0xFFFFFFFFu, live);
        if (!live_m) continue;
      }
      unit = base + (u32)(__ffs(live_m) - 1);
      live_m &= live_m - 1;
    }
    slot_unit<EQM, EXACT, false>(c, unit, jbuf, part, tab_base, lane, warp);
  }
}

// Sum of the 27 slots in slot order (Kahan), each direction's one-sided slot followed by its
// symmetric slots in sub-column order (when the pass had a symmetric part: sym_slots non-null and
// the unit list complete), plus the PM acceleration; in a run the kick, the drift, the unit round
// trip and the escape test, writing the new state to the other buffers.  L: the symmetric
// part's sub-columns per cell.
template <int L>
__global__ void __launch_bounds__(256) pair_epilogue_kernel(
    const float4* __restrict__ pm, const float4* __restrict__ vi, const float4* __restrict__ acc_pm,
    const float4* __restrict__ slots, int n, StepParams sp, float kick, int drift, int kdk,
    float4* __restrict__ pm_out, float4* __restrict__ vi_out, float4* __restrict__ acc_out,
    const float4* __restrict__ sym_slots, const u32* __restrict__ sym_masks, const int* __restrict__ subcol,
    const u32* __restrict__ counter, u32 sym_cap, int* stop) {
  if (stopped_before(stop, kdk && drift, sp.step_tag)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  if (sym_slots && __ldcg(&counter[SLOT_SYM_TOTAL]) <= sym_cap) {
    constexpr int MW = sym_mark_words(L) + 1;
    const u32* mw = sym_masks + (size_t)subcol[i] * MW;
    u32 w[MW];
#pragma unroll
    for (int t = 0; t < MW; ++t) w[t] = mw[t];
#pragma unroll
    for (int k = 0; k < NNB; ++k) {
      // bits k L .. k L + L - 1 (constants once k is unrolled); a dead direction has no
      // one-sided slot (its units were skipped)
      u32 field = sym_field<L>(w, k);
      const int lo = k * L;
      if (!((w[MW - 1] >> k) & 1u)) {
        const float4 v = slots[(size_t)k * n + i];
        kahan_add(sx, cx, v.x);
        kahan_add(sy, cy, v.y);
        kahan_add(sz, cz, v.z);
      }
      while (field) {
        const int q = __ffs(field) - 1;
        field &= field - 1u;
        const float4 e = sym_slots[(size_t)(lo + q) * n + i];
        kahan_add(sx, cx, e.x);
        kahan_add(sy, cy, e.y);
        kahan_add(sz, cz, e.z);
      }
    }
  } else {
#pragma unroll 9
    for (int k = 0; k < NNB; ++k) {
      const float4 v = slots[(size_t)k * n + i];
      kahan_add(sx, cx, v.x);
      kahan_add(sy, cy, v.y);
      kahan_add(sz, cz, v.z);
    }
  }
  const float4 ap = acc_pm[i];
  const float3 a = make_float3(ap.x + sx, ap.y + sy, ap.z + sz);
  if (kdk) {
    float4 p = pm[i], v = vi[i];
    kick_drift(sp, p, v, a, kick, drift, stop);
    pm_out[i] = p;
    vi_out[i] = v;
  }
  acc_out[i] = make_float4(a.x, a.y, a.z, 0.f);
}

// ------------------------------------------------------------------ work items ---------
// One item (sub-column id, slice start) per slice of `slice` particles of a sub-column; the
// table pass takes each item once per neighbour cell (item index * 27 + k).
__global__ void item_count_kernel(const int* __restrict__ cell_start, int ncells_total,
                                  u32* __restrict__ cnt, int slice, const int* stop) {
  if (*stop) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells_total) return;
  const int n = cell_start[c + 1] - cell_start[c];
  cnt[c] = (u32)((n + slice - 1) / slice);
}

__global__ void item_build_kernel(const int* __restrict__ cell_start, const u32* __restrict__ off,
                                  int ncells_total, int2* __restrict__ items, int slice,
                                  const int* stop) {
  if (*stop) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells_total) return;
  const int b = cell_start[c], e = cell_start[c + 1];
  u32 o = off[c];
  for (int s = b; s < e; s += slice) items[o++] = make_int2(c, s);
}

// counter words of the table pass: [0] heavy units taken (by CTAs), [1] medium units taken,
// [2] heavy units listed, [3] medium units listed, [4..5] u64 total estimated cost, [6..7] u64
// heavy threshold, [8] other units taken, [10, 19) symmetric units per cost bucket, [19, 28) taken
// per bucket, [28] symmetric units listed.
constexpr int SLOT_COUNTER_WORDS = 32;

// Total estimated cost of all units (one thread per item, its 27 neighbour cells).
__global__ void plan_cost_kernel(const int* __restrict__ cell_start, const int2* __restrict__ items,
                                 const u32* __restrict__ nitems_p, ChainDimsP cd, u32* __restrict__ counter,
                                 u32 unit_stride, const int* stop) {
  if (*stop) return;
  const u32 item = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long s = 0;
  if (item < *nitems_p && item % unit_stride == 0) {
    const int2 it = items[item];
    for (int k = 0; k < NNB; ++k) s += slot_cost(cell_start, cd, it, k);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(reinterpret_cast<unsigned long long*>(counter + 4), s);
}

// Sets the threshold thr (a 1/SLOT_HEAVY_DIV share of one of `warps` warps, at least
// SLOT_HEAVY_MIN) and lists the heavy units (cost >= thr) from the front of `heavy`, the medium
// ones (thr / 4 <= cost < thr) from its back.  If the two lists do not fit in `cap` entries
// together, the table pass uses neither.
__global__ void plan_heavy_kernel(const int* __restrict__ cell_start, const int2* __restrict__ items,
                                  const u32* __restrict__ nitems_p, ChainDimsP cd,
                                  u32* __restrict__ heavy, u32 cap, u32* __restrict__ counter,
                                  unsigned long long warps, u32 unit_stride, const int* stop) {
  if (*stop) return;
  const unsigned long long total = __ldcg(reinterpret_cast<const unsigned long long*>(counter + 4));
  const unsigned long long t = total / (warps * SLOT_HEAVY_DIV);
  const unsigned long long thr = t > SLOT_HEAVY_MIN ? t : SLOT_HEAVY_MIN;
  const u32 item = blockIdx.x * blockDim.x + threadIdx.x;
  if (item == 0) *reinterpret_cast<unsigned long long*>(counter + 6) = thr;
  if (item >= *nitems_p || item % unit_stride) return;
  const int2 it = items[item];
  for (int k = 0; k < NNB; ++k) {
    const unsigned long long cost = slot_cost(cell_start, cd, it, k);
    if (cost >= thr) {
      const u32 h = atomicAdd(&counter[2], 1u);
      if (h < cap) heavy[h] = item * NNB + k;
    } else if (cost >= thr / 4) {
      const u32 m = atomicAdd(&counter[3], 1u);
      if (m < cap) heavy[cap - 1 - m] = item * NNB + k;
    }
  }
}

// The particles a sampled pass (unit_stride > 1) covers: those of every unit_stride-th slice,
// flagged in original index order (flags cleared by the caller).
__global__ void mark_sampled_kernel(const int* __restrict__ cell_start, const int2* __restrict__ items,
                                    const u32* __restrict__ nitems_p, u32 unit_stride,
                                    const float4* __restrict__ vi, unsigned char* __restrict__ flags) {
  const u32 k = (blockIdx.x * blockDim.x + threadIdx.x) * unit_stride;
  if (k >= *nitems_p) return;
  const int2 it = items[k];
  const int end = min(it.y + SLOT_SLICE, cell_start[it.x + 1]);
  for (int i = it.y; i < end; ++i) flags[__float_as_int(vi[i].w)] = 1;
}

int launch_mark_sampled(const int* cell_start, const int2* items, const u32* nitems, int nitems_max,
                        int unit_stride, const float4* vi, unsigned char* flags, cudaStream_t st) {
  const int nk = (nitems_max + unit_stride - 1) / unit_stride;
  if (nk > 0) mark_sampled_kernel<<<(nk + 255) / 256, 256, 0, st>>>(cell_start, items, nitems, (u32)unit_stride,
                                                                    vi, flags);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

bool pair_pass_sampleable(const PairParams& pp) { return pp.use_table || pp.eps2 == 0.f; }

int slot_counter_words() { return SLOT_COUNTER_WORDS; }

int slot_heavy_capacity(int nitems_max) {
  const long long units = (long long)nitems_max * NNB;
  return (int)(units < (1 << 22) ? units : (1 << 22));
}

bool sym_supported(int sub) { return sub >= 3 && sub <= 5; }

// The symmetric part's padded candidates (sym_window) add exactly nothing in exact mode only if
// the Newton term at |r| = re, cn r1^3, is exactly the value segment 499 cancels, which holds
// when rsqrt.approx(1) and its cube are exactly 1 (GB300: they are).  Checked once per process.
int exact_mode_pads_vanish(cudaStream_t st, bool* vanish) {
  static int known = -1;
  if (known < 0) {
    float* d = nullptr;
    float h[2] = {0.f, 0.f};
    PMGB_CUDA_TRY(cudaMalloc(&d, 2 * sizeof(float)));
    rsqrt_one_kernel<<<1, 1, 0, st>>>(d);
    const cudaError_t e1 = cudaGetLastError();
    const cudaError_t e2 = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, st);
    const cudaError_t e3 = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
      return set_error("rsqrt probe failed"), PMGB_ECUDA;
    count_launches(1);
    known = h[0] == 1.0f && h[1] == 1.0f ? 1 : 0;
  }
  *vanish = known == 1;
  return PMGB_OK;
}

int sym_mask_words(int sub) { return sym_mark_words(sub * sub) + 1; }

// Units a symmetric pass can list: up to 13 L upper-half neighbours and L - 1 within the cell per
// sub-column of at least SYM_MIN_SMALL particles (L = sub^2 sub-columns per cell), at most 2^24.
int sym_unit_capacity(int nsub, int n, int sub) {
  const long long per_sub = 13LL * sub * sub + sub * sub - 1;
  const long long units = per_sub * (long long)std::max(std::min(nsub, n / SYM_MIN_SMALL), 1);
  return (int)(units < (1 << 24) ? units : (1 << 24));
}

int exclusive_scan(const u32* in, u32* out, int n, u32* total, u32* scratch, cudaStream_t st);

int launch_pair(const float4* pm, const float4* vi, const float4* acc_pm, const int* cell_start,
                const ChainDims& chd, u32* item_cnt, u32* item_off, u32* scan_tmp, u32* nitems, int2* items,
                int nitems_max, u32* heavy, u32* counter, const PairParams& pp, const float* table,
                const StepParams& sp, float kick, int drift, int kdk, float4* pm_out, float4* vi_out,
                float4* acc_out, unsigned long long* npairs, int* stop, int num_sms, cudaEvent_t ev_pair,
                cudaStream_t st, int equal_mass, float4* slots, int n, int unit_stride,
                const SymPass* sym) {
  const u32 ustride = unit_stride > 1 ? (u32)unit_stride : 1u;
  const int ncells = chd.Mx * chd.My * chd.Mz;
  const int ntot = ncells * chd.sub * chd.sub + 1;  // sub-columns + the bucket outside the mesh
  // the slotted pass: the table, or the exact table-free force without softening
  const bool exact = !pp.use_table && pp.eps2 == 0.f;
  const bool slotted = (pp.use_table || exact) && !npairs && slots;
  const int slice = slotted ? SLOT_SLICE : 32;
  // the symmetric part: equal masses, 3 x 3 to 5 x 5 y-sorted sub-columns, every slice (not
  // sampled)
  const bool sym_on = slotted && sym && sym->enabled && sym->slots && equal_mass && sym_supported(chd.sub) &&
                      pp.ysort && ustride == 1 && nitems_max > 0 && n > 0;
  item_count_kernel<<<(ntot + 255) / 256, 256, 0, st>>>(cell_start, ntot, item_cnt, slice, stop);
  int rc = exclusive_scan(item_cnt, item_off, ntot, nitems, scan_tmp, st);
  if (rc) return rc;
  item_build_kernel<<<(ntot + 255) / 256, 256, 0, st>>>(cell_start, item_off, ntot, items, slice, stop);
  PMGB_CUDA_TRY(cudaMemsetAsync(counter, 0, SLOT_COUNTER_WORDS * sizeof(u32), st));
  if (npairs) PMGB_CUDA_TRY(cudaMemsetAsync(npairs, 0, sizeof(unsigned long long), st));
  ChainDimsP cd{chd.Mx, chd.My, chd.Mz, ncells, chd.sub, chd.HCsx, chd.HCsz};
  const u32 heavy_cap = (u32)slot_heavy_capacity(nitems_max);
  if (slotted && nitems_max > 0) {
    const int pb = (nitems_max + 255) / 256;
    plan_cost_kernel<<<pb, 256, 0, st>>>(cell_start, items, nitems, cd, counter, ustride, stop);
    plan_heavy_kernel<<<pb, 256, 0, st>>>(cell_start, items, nitems, cd, heavy, heavy_cap, counter,
                                          (unsigned long long)num_sms * SLOT_CTAS_PER_SM * SLOT_WARPS, ustride,
                                          stop);
    if (sym_on) {
      const int nsub = ncells * chd.sub * chd.sub;
      // units buffer: 2 cap uint2 of staging (as cap uint4), then the laid-out list
      uint4* stage = reinterpret_cast<uint4*>(sym->units);
      auto plan = chd.sub == 5 ? sym_plan_kernel<25> : chd.sub == 4 ? sym_plan_kernel<16> : sym_plan_kernel<9>;
      plan<<<std::min((nsub + 1 + 7) / 8, num_sms * 16), 256, 0, st>>>(
          cell_start, cd, nsub, pp.re2, 1e-3f * fminf(cd.HCsx, cd.HCsz), sym->masks, stage, sym->cap, counter, stop);
      sym_scatter_kernel<<<num_sms * 4, 256, 0, st>>>(stage, sym->units + 2 * (size_t)sym->cap, sym->cap, counter,
                                                       stop);
      subcol_kernel<<<pb, 256, 0, st>>>(cell_start, items, nitems, sym->subcol, stop);
    }
  }
  if (ev_pair) PMGB_CUDA_TRY(cudaEventRecord(ev_pair, st));
  const dim3 grid(num_sms * 8), block(PAIR_THREADS);
  if (slotted) {  // table, staging and partial sums: 104.6 KB of dynamic shared memory
    PMGB_CUDA_TRY(cudaFuncSetAttribute(pair_slot_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SLOT_SMEM));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(pair_slot_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SLOT_SMEM));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(pair_slot_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SLOT_SMEM));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(pair_slot_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SLOT_SMEM));
  }
#define PMGB_PAIR_ARGS pm, vi, acc_pm, cell_start, items, nitems, counter, cd, pp, table, sp, kick, \
                       drift, kdk, pm_out, vi_out, acc_out, npairs, stop
  int launches = 3;  // item count, item build, pair pass (the scan counts itself)
  if (slotted) {
    if (nitems_max > 0) launches += 2;  // the two planning kernels
    if (sym_on) launches += 3;  // symmetric planning, unit lay-out, sub-column ids
    auto kern = equal_mass ? (exact ? pair_slot_kernel<true, true> : pair_slot_kernel<true, false>)
                           : (exact ? pair_slot_kernel<false, true> : pair_slot_kernel<false, false>);
    kern<<<num_sms * SLOT_CTAS_PER_SM, SLOT_THREADS, SLOT_SMEM, st>>>(
        pm, n, cell_start, items, nitems, heavy, heavy_cap, counter, cd, pp, table, slots, ustride,
        sym_on ? sym->masks : nullptr, sym_mask_words(chd.sub), sym_on ? sym->cap : 0u,
        sym_on ? sym->slots : nullptr, sym_on ? sym->units + 2 * (size_t)sym->cap : nullptr, stop);
    auto epilogue = !sym_on || chd.sub == 3 ? pair_epilogue_kernel<9>
                    : chd.sub == 4          ? pair_epilogue_kernel<16>
                                            : pair_epilogue_kernel<25>;
    if (n > 0)
      epilogue<<<(n + 255) / 256, 256, 0, st>>>(
          pm, vi, acc_pm, slots, n, sp, kick, drift, kdk, pm_out, vi_out, acc_out,
          sym_on ? sym->slots : nullptr, sym_on ? sym->masks : nullptr, sym_on ? sym->subcol : nullptr, counter,
          sym_on ? sym->cap : 0u, stop);
    ++launches;
  } else if (pp.use_table) {
    if (npairs) pair_kernel<true, true><<<grid, block, 0, st>>>(PMGB_PAIR_ARGS);
    else pair_kernel<true, false><<<grid, block, 0, st>>>(PMGB_PAIR_ARGS);
  } else {
    if (npairs) pair_kernel<false, true><<<grid, block, 0, st>>>(PMGB_PAIR_ARGS);
    else pair_kernel<false, false><<<grid, block, 0, st>>>(PMGB_PAIR_ARGS);
  }
#undef PMGB_PAIR_ARGS
  PMGB_LAUNCH_CHECK();
  count_launches(launches);
  return PMGB_OK;
}

}  // namespace pmgb
