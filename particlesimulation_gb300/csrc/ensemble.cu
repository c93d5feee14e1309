// ensemble.cu - an ensemble of independent PM systems (uneven particle counts and meshes)
// advanced together: every stage of the step is ONE launch over all systems.
//
// No counterpart in the reference (it runs one system per process).  Each system is what a
// pmgb_pm handle would be (same unit conversions, fixed-point scale, influence function, FFT
// passes, interpolation and fused leapfrog; the kernels call the same device bodies, so a system
// of the ensemble and the same system run alone give bit-identical results), laid out in
// concatenated particle and mesh pools.  A table of systems and tables of work items (particle
// chunks, x-pass row groups, column tiles) drive persistent kernels: a grid sized to the GPU
// loops over the items of all systems.  The seven launches of a step are captured once into a
// CUDA graph per (kick, drift) variant and replayed every step.  Tile shapes that do not change
// the arithmetic (particles per deposit thread, rows per x-pass CTA) are picked at creation by
// timing the candidates on the actual ensemble (the autotuner).  Particles are put in brick
// (Morton) order per system once at creation; the order only affects locality.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numbers>
#include <vector>

#include "deposit_body.cuh"
#include "fft_body.cuh"
#include "handles.cuh"
#include "interp_body.cuh"

namespace pmgb {

struct EnsSys {
  int n, p_off;
  long long rho_off, spec_off;
  int pairs;  // x-pass row pairs per work item (autotuned)
  StepParams sp;
};

// Escape flags, 4 ints per system: [0] committed stop, [1] unused, [2] pending stop and [3] its
// iteration, written by kick_drift in the interpolation kernel.  A drifting launch tests only the
// committed word, so an escape in one of its blocks does not make the blocks that start later
// skip their particles; every other kernel tests both words, and the next step's deposit
// commits the pending word.
__device__ __forceinline__ bool ens_stopped(const int* flags, int s) {
  return (flags[4 * s] | flags[4 * s + 2]) != 0;
}

template <int IS, int PPT>
__global__ void __launch_bounds__(DEP_THREADS) ens_deposit_kernel(const EnsSys* __restrict__ sys,
                                                                  const int2* __restrict__ items,
                                                                  int nitems, const float4* __restrict__ pm,
                                                                  u64* __restrict__ rho,
                                                                  int* __restrict__ flags) {
  __shared__ u64 tile[DEP_TILE];
  __shared__ int red[DEP_RED_WORDS];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int2 w = items[it];
    if (ens_stopped(flags, w.x)) {
      if (threadIdx.x == 0) flags[4 * w.x] = 1;
      continue;
    }
    const EnsSys s = sys[w.x];
    deposit_block<IS, PPT>(pm + s.p_off, w.y, s.n, s.sp.m, s.sp.fx_scale, rho + s.rho_off, tile, red);
    __syncthreads();
  }
}

// The FFT passes of all systems' meshes share one kernel each (a switch on the transform length
// inside): capped at 80 registers, 3 CTAs per SM, so the largest length's code sets no lower
// occupancy for the rest.
__global__ void __launch_bounds__(FFT_THREADS, 3) ens_fft_x_r2c_kernel(const EnsSys* __restrict__ sys,
                                                                    const int2* __restrict__ items,
                                                                    int nitems, u64* __restrict__ rho,
                                                                    float2* __restrict__ spec,
                                                                    const float2* __restrict__ tw,
                                                                    int nmax, const int* __restrict__ flags) {
  extern __shared__ float2 sm[];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int2 w = items[it];
    if (ens_stopped(flags, w.x)) continue;
    const EnsSys s = sys[w.x];
    fft_x_r2c_body(sm, rho + s.rho_off, spec + s.spec_off, s.sp.m, s.pairs, s.sp.fx_inv, tw, nmax, w.y);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(FFT_THREADS, 3) ens_fft_x_c2r_kernel(const EnsSys* __restrict__ sys,
                                                                    const int2* __restrict__ items,
                                                                    int nitems,
                                                                    const float2* __restrict__ spec,
                                                                    float* __restrict__ phi,
                                                                    const float2* __restrict__ tw,
                                                                    int nmax, const int* __restrict__ flags) {
  extern __shared__ float2 sm[];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int2 w = items[it];
    if (ens_stopped(flags, w.x)) continue;
    const EnsSys s = sys[w.x];
    fft_x_c2r_body(sm, spec + s.spec_off, phi + s.rho_off, s.sp.m, s.pairs, tw, nmax, w.y);
    __syncthreads();
  }
}

// items: (system, kx0, other) for one axis
__global__ void __launch_bounds__(FFT_THREADS, 3) ens_fft_cols_kernel(const EnsSys* __restrict__ sys,
                                                                   const int4* __restrict__ items,
                                                                   int nitems, float2* __restrict__ spec,
                                                                   int axis, int mode,
                                                                   const float* __restrict__ ghat,
                                                                   const float2* __restrict__ tw,
                                                                   int nmax, const int* __restrict__ flags) {
  extern __shared__ float2 sm[];
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 w = items[it];
    if (ens_stopped(flags, w.x)) continue;
    const EnsSys s = sys[w.x];
    fft_cols_body(sm, spec + s.spec_off, s.sp.m, axis, mode, ghat ? ghat + s.spec_off : nullptr, tw, nmax,
                  w.y, w.z);
    __syncthreads();
  }
}

template <int IS, int FDS>
__global__ void __launch_bounds__(256) ens_interp_kernel(const EnsSys* __restrict__ sys,
                                                         const int2* __restrict__ items, int nitems,
                                                         float4* __restrict__ pm, float4* __restrict__ vi,
                                                         float4* __restrict__ acc,
                                                         const float* __restrict__ phi, float kick,
                                                         int drift, int kdk, int* flags) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int2 w = items[it];
    if (kdk && drift ? flags[4 * w.x] != 0 : ens_stopped(flags, w.x)) continue;
    int* stop = flags + 4 * w.x + 2;
    const EnsSys s = sys[w.x];
    const int i = w.y + threadIdx.x;
    if (i < s.n) {
      if (kdk)
        interp_particle<IS, FDS, true>(pm + s.p_off, vi + s.p_off, acc + s.p_off, i, phi + s.rho_off, s.sp,
                                       kick, drift, stop);
      else
        interp_particle<IS, FDS, false>(pm + s.p_off, vi + s.p_off, acc + s.p_off, i, phi + s.rho_off, s.sp,
                                        kick, drift, stop);
    }
  }
}

inline float host_mass_to_code(float m, float H, float DT, float G) {
  volatile float c = DT * DT * 4 * std::numbers::pi_v<float> * G / (H * H * H);
  return c * m;
}

static u32 morton_host(u32 x, u32 y, u32 z) {
  auto spread = [](u32 v) {
    v &= 0x3FF;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
  };
  return spread(x) | (spread(y) << 1) | (spread(z) << 2);
}

}  // namespace pmgb

using namespace pmgb;

struct pmgb_ensemble {
  int S = 0;
  long long N = 0;
  int is = 0, fds = 0;
  std::vector<pmgb_pm_config> cfg;
  std::vector<EnsSys> hsys;
  EnsSys* sys = nullptr;
  cudaStream_t st = nullptr;
  int num_sms = 0;
  float4 *pm = nullptr, *vi = nullptr, *acc = nullptr;
  u64* rho = nullptr;
  float2* spec = nullptr;
  float* phi = nullptr;
  float* ghat = nullptr;
  float2* tw = nullptr;
  int nmax = 0;
  int* flags = nullptr;  // 4 per system (ens_stopped)
  float* stage = nullptr;
  long long rho_total = 0, spec_total = 0;
  int2* part_items = nullptr;
  int n_part_items = 0;
  int2* interp_items = nullptr;
  int n_interp_items = 0;
  int2* x_items = nullptr;
  int n_x_items = 0;
  int4* y_items = nullptr;
  int n_y_items = 0;
  int4* z_items = nullptr;
  int n_z_items = 0;
  int ppt = 2;        // tuned: particles per deposit thread
  int pair_mult = 1;  // tuned: x-pass rows per CTA relative to the default (x 1/2, 1, 2)
  size_t x_smem = 0, col_smem = 0;
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};  // (0.5, drift), (1, drift), (1, none)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float tune_ms[6] = {0, 0, 0, 0, 0, 0};
};

namespace {

template <typename T>
int ens_alloc(T** p, size_t count) {
  if (cudaMalloc((void**)p, count * sizeof(T) + 16) != cudaSuccess) {
    set_error("cudaMalloc failed (ensemble)");
    return PMGB_ENOMEM;
  }
  return PMGB_OK;
}

void ens_free(pmgb_ensemble* e) {
  if (!e) return;
  for (auto& g : e->graph)
    if (g) cudaGraphExecDestroy(g);
  void* ptrs[] = {e->sys, e->pm, e->vi, e->acc, e->rho, e->spec, e->phi, e->ghat, e->tw, e->flags, e->stage,
                  e->part_items, e->interp_items, e->x_items, e->y_items, e->z_items};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
}

int upload_tables(pmgb_ensemble* e) {
  // particle chunks for the deposit (DEP_THREADS * ppt particles) and the interpolation (256)
  std::vector<int2> part, interp, xi;
  std::vector<int4> yi, zi;
  const int chunk = DEP_THREADS * e->ppt;
  for (int s = 0; s < e->S; ++s) {
    const EnsSys& q = e->hsys[s];
    for (int b = 0; b < q.n; b += chunk) part.push_back(make_int2(s, b));
    for (int b = 0; b < q.n; b += 256) interp.push_back(make_int2(s, b));
    const MeshDims& m = q.sp.m;
    const long long rowpairs = (long long)m.ny * m.nz / 2;
    for (long long r = 0; r < rowpairs; r += q.pairs) xi.push_back(make_int2(s, (int)(2 * r)));
    const int ctiles = (m.nxp + COL_TX - 1) / COL_TX;
    for (int o = 0; o < m.nz; ++o)
      for (int c = 0; c < ctiles; ++c) yi.push_back(make_int4(s, c * COL_TX, o, 0));
    for (int o = 0; o < m.ny; ++o)
      for (int c = 0; c < ctiles; ++c) zi.push_back(make_int4(s, c * COL_TX, o, 0));
  }
  auto up = [&](auto** dst, auto& v, int* count) -> int {
    if (*dst) cudaFree(*dst);
    *dst = nullptr;
    int rc = ens_alloc(dst, std::max<size_t>(v.size(), 1));
    if (rc) return rc;
    PMGB_CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice));
    *count = (int)v.size();
    return PMGB_OK;
  };
  int rc;
  if ((rc = up(&e->part_items, part, &e->n_part_items)) || (rc = up(&e->interp_items, interp, &e->n_interp_items)) ||
      (rc = up(&e->x_items, xi, &e->n_x_items)) || (rc = up(&e->y_items, yi, &e->n_y_items)) ||
      (rc = up(&e->z_items, zi, &e->n_z_items)))
    return rc;
  PMGB_CUDA_TRY(cudaMemcpy(e->sys, e->hsys.data(), e->S * sizeof(EnsSys), cudaMemcpyHostToDevice));
  return PMGB_OK;
}

int grid_for(const pmgb_ensemble* e, int items, int per_sm) {
  return std::max(1, std::min(items, e->num_sms * per_sm));
}

// the launches of one step (force + kick + drift); stage selects what to launch (all = -1)
int launch_step(pmgb_ensemble* e, float kick, int drift, int kdk, int stage = -1) {
  cudaStream_t st = e->st;
  if (stage < 0 || stage == 0) {
    const int g = grid_for(e, e->n_part_items, 8);
    if (e->is == 0) {
      if (e->ppt == 1) ens_deposit_kernel<0, 1><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
      else if (e->ppt == 2) ens_deposit_kernel<0, 2><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
      else ens_deposit_kernel<0, 4><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
    } else if (e->is == 1) {
      if (e->ppt == 1) ens_deposit_kernel<1, 1><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
      else if (e->ppt == 2) ens_deposit_kernel<1, 2><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
      else ens_deposit_kernel<1, 4><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
    } else {
      if (e->ppt == 1) ens_deposit_kernel<2, 1><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
      else if (e->ppt == 2) ens_deposit_kernel<2, 2><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
      else ens_deposit_kernel<2, 4><<<g, DEP_THREADS, 0, st>>>(e->sys, e->part_items, e->n_part_items, e->pm, e->rho, e->flags);
    }
  }
  if (stage < 0 || stage == 1) {
    ens_fft_x_r2c_kernel<<<grid_for(e, e->n_x_items, 4), FFT_THREADS, e->x_smem, st>>>(
        e->sys, e->x_items, e->n_x_items, e->rho, e->spec, e->tw, e->nmax, e->flags);
  }
  if (stage < 0 || stage == 2) {
    ens_fft_cols_kernel<<<grid_for(e, e->n_y_items, 4), FFT_THREADS, e->col_smem, st>>>(
        e->sys, e->y_items, e->n_y_items, e->spec, 1, 0, nullptr, e->tw, e->nmax, e->flags);
    ens_fft_cols_kernel<<<grid_for(e, e->n_z_items, 4), FFT_THREADS, e->col_smem, st>>>(
        e->sys, e->z_items, e->n_z_items, e->spec, 2, 2, e->ghat, e->tw, e->nmax, e->flags);
    ens_fft_cols_kernel<<<grid_for(e, e->n_y_items, 4), FFT_THREADS, e->col_smem, st>>>(
        e->sys, e->y_items, e->n_y_items, e->spec, 1, 1, nullptr, e->tw, e->nmax, e->flags);
  }
  if (stage < 0 || stage == 3) {
    ens_fft_x_c2r_kernel<<<grid_for(e, e->n_x_items, 4), FFT_THREADS, e->x_smem, st>>>(
        e->sys, e->x_items, e->n_x_items, e->spec, e->phi, e->tw, e->nmax, e->flags);
  }
  if (stage < 0 || stage == 4) {
    const int g = grid_for(e, e->n_interp_items, 8);
    const int code = e->is * 2 + e->fds;
#define ENS_INTERP(IS_, FDS_)                                                                    \
  ens_interp_kernel<IS_, FDS_><<<g, 256, 0, st>>>(e->sys, e->interp_items, e->n_interp_items, e->pm, \
                                                  e->vi, e->acc, e->phi, kick, drift, kdk, e->flags)
    switch (code) {
      case 0: ENS_INTERP(0, 0); break;
      case 1: ENS_INTERP(0, 1); break;
      case 2: ENS_INTERP(1, 0); break;
      case 3: ENS_INTERP(1, 1); break;
      case 4: ENS_INTERP(2, 0); break;
      default: ENS_INTERP(2, 1); break;
    }
#undef ENS_INTERP
  }
  PMGB_LAUNCH_CHECK();
  count_launches(stage < 0 ? 7 : (stage == 2 ? 3 : 1));
  return PMGB_OK;
}

int set_pairs(pmgb_ensemble* e, int mult) {
  size_t smem = 0;
  for (auto& q : e->hsys) {
    int p = x_pairs_default(q.sp.m);
    const long long rowpairs = (long long)q.sp.m.ny * q.sp.m.nz / 2;
    if (mult == 0) p = std::max(1, p / 2);
    if (mult == 2) p = (int)std::min<long long>(rowpairs, 2ll * p);
    q.pairs = p;
    smem = std::max(smem, (size_t)x_smem_elems(q.sp.m.nx, p) * sizeof(float2));
  }
  e->pair_mult = mult;
  e->x_smem = smem;
  if (smem > 48 * 1024) {
    PMGB_CUDA_TRY(cudaFuncSetAttribute(ens_fft_x_r2c_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    PMGB_CUDA_TRY(cudaFuncSetAttribute(ens_fft_x_c2r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  return PMGB_OK;
}

// time `stage` of the step (reps launches), ms per launch
float time_stage(pmgb_ensemble* e, int stage, int reps) {
  cudaEventRecord(e->ev0, e->st);
  for (int r = 0; r < reps; ++r) launch_step(e, 1.0f, 0, 0, stage);
  cudaEventRecord(e->ev1, e->st);
  cudaEventSynchronize(e->ev1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e->ev0, e->ev1);
  return ms / reps;
}

// The autotuner: particles per deposit thread (1, 2, 4) and rows per x-pass CTA (x 1/2, 1, 2);
// neither changes the arithmetic.  The deposit candidates add into the density mesh, so the
// mesh is cleared afterwards.
int autotune(pmgb_ensemble* e) {
  float best = 1e30f;
  int best_ppt = 2;
  for (int ppt : {1, 2, 4}) {
    e->ppt = ppt;
    int rc = upload_tables(e);
    if (rc) return rc;
    launch_step(e, 1.f, 0, 0, 0);
    const float ms = time_stage(e, 0, 3);
    e->tune_ms[ppt == 1 ? 0 : (ppt == 2 ? 1 : 2)] = ms;
    if (ms < best) {
      best = ms;
      best_ppt = ppt;
    }
  }
  e->ppt = best_ppt;
  best = 1e30f;
  int best_mult = 1;
  for (int mult : {0, 1, 2}) {
    int rc = set_pairs(e, mult);
    if (rc) return rc;
    rc = upload_tables(e);
    if (rc) return rc;
    launch_step(e, 1.f, 0, 0, 1);
    launch_step(e, 1.f, 0, 0, 3);
    const float ms = time_stage(e, 1, 2) + time_stage(e, 3, 2);
    e->tune_ms[3 + mult] = ms;
    if (ms < best) {
      best = ms;
      best_mult = mult;
    }
  }
  int rc = set_pairs(e, best_mult);
  if (rc) return rc;
  rc = upload_tables(e);
  if (rc) return rc;
  PMGB_CUDA_TRY(cudaMemsetAsync(e->rho, 0, e->rho_total * sizeof(u64), e->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return PMGB_OK;
}

int capture_graphs(pmgb_ensemble* e) {
  const float kicks[3] = {0.5f, 1.0f, 1.0f};
  const int drifts[3] = {1, 1, 0};
  for (int v = 0; v < 3; ++v) {
    cudaGraph_t g = nullptr;
    PMGB_CUDA_TRY(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
    int rc = launch_step(e, kicks[v], drifts[v], 1);
    cudaError_t ce = cudaStreamEndCapture(e->st, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) return set_error(std::string("graph capture: ") + cudaGetErrorString(ce)), PMGB_ECUDA;
    ce = cudaGraphInstantiate(&e->graph[v], g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return set_error(std::string("graph instantiate: ") + cudaGetErrorString(ce)), PMGB_ECUDA;
  }
  return PMGB_OK;
}

}  // namespace

extern "C" {

int pmgb_ensemble_create(int n_systems, const pmgb_pm_config* cfgs, const int* counts,
                         const float* const* states, const float* const* masses,
                         pmgb_ensemble** out) {
  if (!out || !cfgs || !counts || !states || !masses || n_systems < 1)
    return set_error("null argument or empty ensemble"), PMGB_EINVAL;
  *out = nullptr;
  for (int s = 0; s < n_systems; ++s) {
    const pmgb_pm_config& c = cfgs[s];
    for (int i = 0; i < 3; ++i)
      if (c.grid[i] < 8 || c.grid[i] > 512 || (c.grid[i] & (c.grid[i] - 1)))
        return set_error("grid points must be powers of two in [8, 512]"), PMGB_EINVAL;
    if (c.interpolation != cfgs[0].interpolation || c.finite_diff != cfgs[0].finite_diff)
      return set_error("all systems of an ensemble share the interpolation and difference schemes"), PMGB_EINVAL;
    if (c.interpolation < 0 || c.interpolation > 2 || c.finite_diff < 0 || c.finite_diff > 1 || c.greens < 0 ||
        c.greens > 3 || !(c.H > 0) || !(c.DT > 0) || counts[s] < 0)
      return set_error("bad system configuration"), PMGB_EINVAL;
    if ((c.greens == PMGB_S1_OPTIMAL || c.greens == PMGB_S2_OPTIMAL) && !(c.particle_diameter > 0))
      return set_error("optimal Green's functions need a positive particle diameter"), PMGB_EINVAL;
  }
  pmgb_ensemble* e = new pmgb_ensemble();
  e->S = n_systems;
  e->is = cfgs[0].interpolation;
  e->fds = cfgs[0].finite_diff;
  e->cfg.assign(cfgs, cfgs + n_systems);
  auto fail = [&](int rc) {
    ens_free(e);
    return rc;
  };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess)
    return set_error("CUDA set-up failed"), fail(PMGB_ECUDA);
  // system table, host particle arrays (code units, brick order per system)
  e->hsys.resize(n_systems);
  std::vector<float4> hp, hv;
  long long rho_off = 0, spec_off = 0;
  for (int s = 0; s < n_systems; ++s) {
    const pmgb_pm_config& c = cfgs[s];
    EnsSys& q = e->hsys[s];
    MeshDims& m = q.sp.m;
    m.nx = c.grid[0];
    m.ny = c.grid[1];
    m.nz = c.grid[2];
    auto lg = [](int v) {
      int l = 0;
      while ((1 << l) < v) ++l;
      return l;
    };
    m.lx = lg(m.nx);
    m.ly = lg(m.ny);
    m.lz = lg(m.nz);
    m.nxh = m.nx / 2 + 1;
    m.nxp = (m.nxh + 3) & ~3;
    m.L = (long long)m.nx * m.ny * m.nz;
    e->nmax = std::max(e->nmax, std::max(m.nx, std::max(m.ny, m.nz)));
    StepParams& sp = q.sp;
    sp.is = c.interpolation;
    sp.fds = c.finite_diff;
    sp.H = c.H;
    sp.DT = c.DT;
    sp.box_x = c.box[0];
    sp.box_y = c.box[1];
    sp.box_z = c.box[2];
    sp.ext.kind = c.ext.kind;
    sp.ext.cx = c.ext.center[0];
    sp.ext.cy = c.ext.center[1];
    sp.ext.cz = c.ext.center[2];
    sp.ext.R = c.ext.R;
    sp.ext.M = c.ext.M;
    sp.ext.G = c.ext.G;
    sp.step_tag = 0;
    sp.periodic = c.periodic ? 1 : 0;
    q.n = counts[s];
    q.p_off = (int)e->N;
    q.rho_off = rho_off;
    q.spec_off = spec_off;
    rho_off += m.L;
    spec_off += (long long)m.nxp * m.ny * m.nz;
    const float H = c.H, DT = c.DT, G = c.G;
    const int n = counts[s];
    std::vector<int> order(n);
    std::vector<u32> key(n);
    double msum = 0.0;
    for (int i = 0; i < n; ++i) {
      order[i] = i;
      const float* x = states[s] + 3 * i;
      auto b = [](float v, int nm) {
        int c0 = (int)std::floor(v);
        c0 = ((c0 % nm) + nm) % nm;
        return (u32)(c0 >> 2);
      };
      key[i] = morton_host(b(x[0] / H, m.nx), b(x[1] / H, m.ny), b(x[2] / H, m.nz));
      msum += std::fabs((double)host_mass_to_code(masses[s][i], H, DT, G));
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    for (int k = 0; k < n; ++k) {
      const int i = order[k];
      const float* x = states[s] + 3 * i;
      const float* v = states[s] + 3 * (n + i);
      hp.push_back(make_float4(x[0] / H, x[1] / H, x[2] / H, host_mass_to_code(masses[s][i], H, DT, G)));
      float idf;
      std::memcpy(&idf, &i, 4);
      hv.push_back(make_float4((DT * v[0]) / H, (DT * v[1]) / H, (DT * v[2]) / H, idf));
    }
    int k = msum > 0 ? (int)std::floor(62.0 - std::log2(4.0 * msum)) : 62;
    k = std::min(k, 100);
    sp.fx_scale = std::ldexp(1.0f, k);
    sp.fx_inv = std::ldexp(1.0f, -k);
    e->N += n;
  }
  e->rho_total = rho_off;
  e->spec_total = spec_off;
  const size_t NN = (size_t)std::max<long long>(e->N, 1);
  int rc;
  if ((rc = ens_alloc(&e->sys, n_systems)) || (rc = ens_alloc(&e->pm, NN)) || (rc = ens_alloc(&e->vi, NN)) ||
      (rc = ens_alloc(&e->acc, NN)) || (rc = ens_alloc(&e->rho, rho_off)) || (rc = ens_alloc(&e->spec, spec_off)) ||
      (rc = ens_alloc(&e->phi, rho_off)) || (rc = ens_alloc(&e->ghat, spec_off)) ||
      (rc = ens_alloc(&e->tw, e->nmax / 2 + 1)) || (rc = ens_alloc(&e->flags, 4 * n_systems)) ||
      (rc = ens_alloc(&e->stage, 9 * NN)))
    return fail(rc);
  if (cudaMemcpy(e->pm, hp.data(), hp.size() * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->vi, hv.data(), hv.size() * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(e->acc, 0, NN * sizeof(float4)) != cudaSuccess ||
      cudaMemset(e->rho, 0, rho_off * sizeof(u64)) != cudaSuccess ||
      cudaMemset(e->spec, 0, spec_off * sizeof(float2)) != cudaSuccess ||
      cudaMemset(e->flags, 0, 4 * n_systems * sizeof(int)) != cudaSuccess)
    return set_error("ensemble upload failed"), fail(PMGB_ECUDA);
  {
    std::vector<float2> tw(e->nmax / 2 + 1);
    for (int j = 0; j <= e->nmax / 2; ++j) {
      const double a = -2.0 * 3.14159265358979323846 * j / e->nmax;
      tw[j] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    if (cudaMemcpy(e->tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
      return set_error("twiddle upload failed"), fail(PMGB_ECUDA);
  }
  for (int s = 0; s < n_systems; ++s) {
    const pmgb_pm_config& c = cfgs[s];
    rc = launch_green(e->ghat + e->hsys[s].spec_off, e->hsys[s].sp.m, c.greens, c.interpolation, c.finite_diff,
                      (double)c.particle_diameter / (double)c.H, e->st);
    if (rc) return fail(rc);
  }
  size_t col_smem = 0;
  for (auto& q : e->hsys)
    col_smem = std::max(col_smem, (size_t)col_smem_elems(std::max(q.sp.m.ny, q.sp.m.nz)) * sizeof(float2));
  e->col_smem = col_smem;
  if (col_smem > 48 * 1024 &&
      cudaFuncSetAttribute(ens_fft_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)col_smem) != cudaSuccess)
    return set_error("shared memory configuration failed"), fail(PMGB_ECUDA);
  if ((rc = set_pairs(e, 1)) || (rc = upload_tables(e)) || (rc = autotune(e)) || (rc = capture_graphs(e)))
    return fail(rc);
  if (cudaStreamSynchronize(e->st) != cudaSuccess) return set_error("ensemble set-up failed"), fail(PMGB_ECUDA);
  *out = e;
  return PMGB_OK;
}

int pmgb_ensemble_destroy(pmgb_ensemble* e) {
  if (!e) return PMGB_OK;
  cudaStreamSynchronize(e->st);
  ens_free(e);
  return PMGB_OK;
}

// PMMethod::run for every system at once (initial force, half kick, sim_length + 1 loop
// iterations; a system whose particle leaves its box stops there, the others go on).
int pmgb_ensemble_run(pmgb_ensemble* e, int sim_length, int* escaped, float* device_ms) {
  if (!e || sim_length < 0) return set_error("bad argument"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaMemsetAsync(e->flags, 0, 4 * e->S * sizeof(int), e->st));
  PMGB_CUDA_TRY(cudaEventRecord(e->ev0, e->st));
  PMGB_CUDA_TRY(cudaGraphLaunch(e->graph[0], e->st));
  for (int t = 0; t <= sim_length; ++t) PMGB_CUDA_TRY(cudaGraphLaunch(e->graph[t < sim_length ? 1 : 2], e->st));
  count_launches(7 * (sim_length + 2));
  PMGB_CUDA_TRY(cudaEventRecord(e->ev1, e->st));
  std::vector<int> flags(4 * e->S);
  PMGB_CUDA_TRY(cudaMemcpyAsync(flags.data(), e->flags, flags.size() * sizeof(int), cudaMemcpyDeviceToHost, e->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  if (device_ms) cudaEventElapsedTime(device_ms, e->ev0, e->ev1);
  bool any = false;
  for (int s = 0; s < e->S; ++s) {
    const int esc = (flags[4 * s] | flags[4 * s + 2]) != 0;
    if (escaped) escaped[s] = esc;
    any = any || esc;
  }
  return any ? PMGB_EESCAPED : PMGB_OK;
}

// n_steps more loop iterations (drift, force, kick) for every system, continuing from run().
int pmgb_ensemble_advance(pmgb_ensemble* e, int n_steps, float* device_ms) {
  if (!e || n_steps < 0) return set_error("bad argument"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  PMGB_CUDA_TRY(cudaEventRecord(e->ev0, e->st));
  if (n_steps > 0) {
    // the loop body's first drift is the previous step's closing drift: replay (1, drift)
    // graphs and finish with (1, no drift); the extra leading drift comes from a drift-only
    // interpolation pass
    int rc = launch_step(e, 0.f, 1, 1, 4);  // drift only (kick 0 leaves velocities)
    if (rc) return rc;
    for (int t = 0; t < n_steps; ++t) PMGB_CUDA_TRY(cudaGraphLaunch(e->graph[t + 1 < n_steps ? 1 : 2], e->st));
    count_launches(7 * n_steps);
  }
  PMGB_CUDA_TRY(cudaEventRecord(e->ev1, e->st));
  PMGB_CUDA_TRY(cudaEventSynchronize(e->ev1));
  if (device_ms) cudaEventElapsedTime(device_ms, e->ev0, e->ev1);
  return PMGB_OK;
}

int pmgb_ensemble_get_particles(pmgb_ensemble* e, int system, float* pos, float* vel, float* acc,
                                int units) {
  if (!e || system < 0 || system >= e->S) return set_error("bad system index"), PMGB_EINVAL;
  const EnsSys& q = e->hsys[system];
  const size_t n = (size_t)q.n;
  if (n == 0) return PMGB_OK;
  int rc = launch_unpack(e->pm + q.p_off, e->vi + q.p_off, e->acc + q.p_off, q.n, q.sp.H, q.sp.DT,
                         units == PMGB_UNITS_ORIGINAL, e->stage, e->stage + 3 * n, e->stage + 6 * n, e->st);
  if (rc) return rc;
  if (pos) PMGB_CUDA_TRY(cudaMemcpyAsync(pos, e->stage, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, e->st));
  if (vel) PMGB_CUDA_TRY(cudaMemcpyAsync(vel, e->stage + 3 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, e->st));
  if (acc) PMGB_CUDA_TRY(cudaMemcpyAsync(acc, e->stage + 6 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, e->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return PMGB_OK;
}

int pmgb_ensemble_tuning(pmgb_ensemble* e, int* deposit_ppt, int* x_rows_mult, float* timings6) {
  if (!e) return set_error("null handle"), PMGB_EINVAL;
  if (deposit_ppt) *deposit_ppt = e->ppt;
  if (x_rows_mult) *x_rows_mult = e->pair_mult;
  if (timings6)
    for (int i = 0; i < 6; ++i) timings6[i] = e->tune_ms[i];
  return PMGB_OK;
}

int pmgb_ensemble_size(pmgb_ensemble* e, int* n_systems, long long* total_particles) {
  if (!e) return set_error("null handle"), PMGB_EINVAL;
  if (n_systems) *n_systems = e->S;
  if (total_particles) *total_particles = e->N;
  return PMGB_OK;
}

}  // extern "C"
