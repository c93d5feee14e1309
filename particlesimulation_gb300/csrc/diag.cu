// diag.cu - FP64 run diagnostics on the device.
//
// The reference's PMMethod::run / P3MMethod::run with collectDiagnostics record, once per loop
// iteration right after its drift, what SimInfo computes (source/simInfo.cpp:50-127; call sites
// source/pmMethod.cpp:66-106, source/p3mMethod.cpp:69-130, source/PMMethodGPU.cu:86-139):
//   potential energy   0.5 H^3 sum_cells rho_orig * phi_orig + sum_i m_i Phi_ext(x_i)
//   kinetic energy     sum_i 0.5 m_i |v_i|^2       (v = the half-step velocity)
//   momentum           sum_i m_i u_i                (u = integer-step velocity v + a/2)
//   angular momentum   sum_i m_i x_i cross u_i
//   expected momentum  initial momentum + DT * sum over iterations of sum_i m_i g_ext(x_i)
// in original units (massToOriginalUnits, densityToOriginalUnits, potentialToOriginalUnits,
// include/unitConversions.h:8-50), with the density and potential of the force evaluation
// before the drift.  The reference sums in float on the host (its GPU path copies particles
// and both meshes to the host every iteration); here every sum is in double on the device and
// the records stay in device memory until the caller asks for them.
//
// The per-particle values are formed in float exactly as the reference forms them (u = v +
// 0.5f * a, then H * u / DT; x_orig = H * x; m_orig = c * m) and then summed in double.
// collectDiagnostics also converts the masses to original units and back every iteration,
// which can move a code-unit mass by one ulp: the particle kernel writes that round-tripped
// mass back, so a run with diagnostics follows the reference's trajectory.
//
// Kernels (fixed grids, fixed reduction order: the records are deterministic and independent
// of the SM count):
//   diag_particles  DIAG_BLOCKS x 256 threads, grid-stride over particles; per-block partial
//                   sums of the 11 particle quantities (warp shuffles, then shared memory)
//   diag_mesh       DIAG_BLOCKS x 256, sum of rho * phi over the mesh, float4 loads
//   diag_finalize   one warp: sums the partials in block order, composes the record, advances
//                   the expected momentum, appends the record
// Bytes per record: 44 per particle (position + mass, velocity, acceleration; 4 more for the
// mass write) and 8 per mesh cell, plus the 4 bytes per cell the x pass writes for the density
// copy: a few microseconds at the benchmark sizes.
#include <algorithm>
#include <climits>
#include <cmath>
#include <numbers>

#include "handles.cuh"

struct pmgb_diag {
  int cap = 0;
  float* rho = nullptr;     // float density of the last force evaluation (code units)
  double* part = nullptr;   // DIAG_BLOCKS x 12 particle partials
  double* mpart = nullptr;  // DIAG_BLOCKS mesh partials
  double* state = nullptr;  // expected momentum (3)
  double* rec = nullptr;    // cap x PMGB_DIAG_WIDTH records
  int* count = nullptr;     // records taken (may exceed cap: the excess is dropped)
  bool rho_valid = false;
};

namespace pmgb {

namespace {

constexpr int DIAG_BLOCKS = 256;
constexpr int DIAG_THREADS = 256;
constexpr int DIAG_NP = 11;  // ke, P xyz, L xyz, F_ext xyz, U_ext

struct DiagConsts {
  float H, DT;
  float m_to_orig, m_to_code;  // float factors of massToOriginalUnits / massToCodeUnits
  ExtField ext;
  int n;
  int record;      // 0: initial momentum only (velocity as integer-step velocity)
  int round_trip;  // write back the round-tripped mass
  int tag;
};

__device__ __forceinline__ bool diag_skip(const int* stop, int tag) {
  return stop[0] != 0 && stop[1] < tag;  // an earlier iteration escaped: no record
}

// sphRadDecrField / sphRadDecrFieldPotential (reference source/externalFields.cpp:4-28), double.
__device__ __forceinline__ void ext_field_pot(const ExtField& e, double x, double y, double z,
                                              double g[3], double& phi) {
  g[0] = g[1] = g[2] = 0.0;
  phi = 0.0;
  if (e.kind != PMGB_EXT_SPH_RAD_DECR) return;
  const double dx = x - (double)e.cx, dy = y - (double)e.cy, dz = z - (double)e.cz;
  const double r = sqrt(dx * dx + dy * dy + dz * dz);
  const double R = e.R, GM = (double)e.G * (double)e.M;
  const double gm = r > R ? -GM / (r * r) : -(GM / (R * R * R)) * r * (4.0 - 3.0 * r / R);
  if (r > 0.0) {
    g[0] = gm * dx / r;
    g[1] = gm * dy / r;
    g[2] = gm * dz / r;
  }
  const double u = r / R;
  phi = r > R ? -GM / r : GM / R * (-2.0 + u * u * (2.0 - u));
}

template <int K>
__device__ __forceinline__ void block_sums(double (&v)[K], double* __restrict__ out) {
  __shared__ double sm[DIAG_THREADS / 32][K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double a = v[k];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xFFFFFFFFu, a, o);
    if (lane == 0) sm[warp][k] = a;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double a = 0.0;
    for (int w = 0; w < DIAG_THREADS / 32; ++w) a += sm[w][threadIdx.x];
    out[threadIdx.x] = a;
  }
}

__global__ void __launch_bounds__(DIAG_THREADS) diag_particles_kernel(
    float4* __restrict__ pm, const float4* __restrict__ vi, const float4* __restrict__ acc,
    DiagConsts c, const int* __restrict__ stop, double* __restrict__ part) {
  if (c.record && diag_skip(stop, c.tag)) return;
  double s[DIAG_NP];
#pragma unroll
  for (int k = 0; k < DIAG_NP; ++k) s[k] = 0.0;
  for (int i = blockIdx.x * DIAG_THREADS + threadIdx.x; i < c.n; i += DIAG_BLOCKS * DIAG_THREADS) {
    float4 p = pm[i];
    const float4 v = vi[i];
    const float mo = __fmul_rn(c.m_to_orig, p.w);
    if (c.round_trip) {
      p.w = __fmul_rn(c.m_to_code, mo);
      pm[i] = p;
    }
    float ux = v.x, uy = v.y, uz = v.z;
    if (c.record) {  // setIntegerStepVelocities (source/leapfrog.cpp:10-15), dt = 1
      const float4 a = acc[i];
      ux = __fadd_rn(v.x, __fmul_rn(0.5f, a.x));
      uy = __fadd_rn(v.y, __fmul_rn(0.5f, a.y));
      uz = __fadd_rn(v.z, __fmul_rn(0.5f, a.z));
    }
    // velocityToOriginalUnits H * v / DT, positionToOriginalUnits H * x
    const double uxo = __fdiv_rn(__fmul_rn(c.H, ux), c.DT);
    const double uyo = __fdiv_rn(__fmul_rn(c.H, uy), c.DT);
    const double uzo = __fdiv_rn(__fmul_rn(c.H, uz), c.DT);
    const double m = mo;
    s[1] += m * uxo;
    s[2] += m * uyo;
    s[3] += m * uzo;
    if (c.record) {
      const double vxo = __fdiv_rn(__fmul_rn(c.H, v.x), c.DT);
      const double vyo = __fdiv_rn(__fmul_rn(c.H, v.y), c.DT);
      const double vzo = __fdiv_rn(__fmul_rn(c.H, v.z), c.DT);
      const double x = __fmul_rn(c.H, p.x), y = __fmul_rn(c.H, p.y), z = __fmul_rn(c.H, p.z);
      s[0] += 0.5 * m * (vxo * vxo + vyo * vyo + vzo * vzo);
      s[4] += m * (y * uzo - z * uyo);
      s[5] += m * (z * uxo - x * uzo);
      s[6] += m * (x * uyo - y * uxo);
      double g[3], phi;
      ext_field_pot(c.ext, x, y, z, g, phi);
      s[7] += m * g[0];
      s[8] += m * g[1];
      s[9] += m * g[2];
      s[10] += m * phi;
    }
  }
  block_sums<DIAG_NP>(s, part + 12 * blockIdx.x);
}

__global__ void __launch_bounds__(DIAG_THREADS) diag_mesh_kernel(const float* __restrict__ rho,
                                                                 const float* __restrict__ phi,
                                                                 long long L, int tag,
                                                                 const int* __restrict__ stop,
                                                                 double* __restrict__ mpart) {
  if (diag_skip(stop, tag)) return;
  double s[1] = {0.0};
  const long long L4 = L >> 2;
  const float4* r4 = reinterpret_cast<const float4*>(rho);
  const float4* p4 = reinterpret_cast<const float4*>(phi);
  for (long long k = blockIdx.x * (long long)DIAG_THREADS + threadIdx.x; k < L4;
       k += (long long)DIAG_BLOCKS * DIAG_THREADS) {
    const float4 a = r4[k], b = p4[k];
    s[0] += (double)a.x * b.x + (double)a.y * b.y + (double)a.z * b.z + (double)a.w * b.w;
  }
  for (long long k = 4 * L4 + blockIdx.x * (long long)DIAG_THREADS + threadIdx.x; k < L;
       k += (long long)DIAG_BLOCKS * DIAG_THREADS)
    s[0] += (double)rho[k] * phi[k];
  block_sums<1>(s, mpart + blockIdx.x);
}

__global__ void diag_finalize_kernel(const double* __restrict__ part,
                                     const double* __restrict__ mpart, DiagConsts c,
                                     double kmesh, const int* __restrict__ stop,
                                     double* __restrict__ state, double* __restrict__ rec,
                                     int cap, int* __restrict__ count) {
  if (c.record && diag_skip(stop, c.tag)) return;
  __shared__ double s[12];
  const int k = threadIdx.x;
  if (k < DIAG_NP) {
    double a = 0.0;
    for (int b = 0; b < DIAG_BLOCKS; ++b) a += part[12 * b + k];
    s[k] = a;
  } else if (k == DIAG_NP) {
    double a = 0.0;
    if (c.record)
      for (int b = 0; b < DIAG_BLOCKS; ++b) a += mpart[b];
    s[k] = a;
  }
  __syncthreads();
  if (k != 0) return;
  if (!c.record) {  // setInitialMomentum
    state[0] = s[1];
    state[1] = s[2];
    state[2] = s[3];
    return;
  }
  // updateExpectedMomentum(totalExternalForceOrigUnits(), DT)
  const double DT = c.DT;
  const double e0 = state[0] + DT * s[7], e1 = state[1] + DT * s[8], e2 = state[2] + DT * s[9];
  state[0] = e0;
  state[1] = e1;
  state[2] = e2;
  const int slot = *count;
  *count = slot + 1;
  if (slot >= cap) return;
  double* r = rec + (size_t)PMGB_DIAG_WIDTH * slot;
  r[PMGB_DIAG_POTENTIAL] = kmesh * s[11] + s[10];
  r[PMGB_DIAG_KINETIC] = s[0];
  r[PMGB_DIAG_MOMENTUM] = s[1];
  r[PMGB_DIAG_MOMENTUM + 1] = s[2];
  r[PMGB_DIAG_MOMENTUM + 2] = s[3];
  r[PMGB_DIAG_ANGULAR_MOMENTUM] = s[4];
  r[PMGB_DIAG_ANGULAR_MOMENTUM + 1] = s[5];
  r[PMGB_DIAG_ANGULAR_MOMENTUM + 2] = s[6];
  r[PMGB_DIAG_EXPECTED_MOMENTUM] = e0;
  r[PMGB_DIAG_EXPECTED_MOMENTUM + 1] = e1;
  r[PMGB_DIAG_EXPECTED_MOMENTUM + 2] = e2;
  r[PMGB_DIAG_EXTERNAL_POTENTIAL] = s[10];
}

// Fixed-point density (the deposit's mesh) to float, clearing it like the x pass does.
__global__ void fx_to_float_kernel(u64* __restrict__ rho, float* __restrict__ out, long long L,
                                   float fx_inv) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < L;
       k += (long long)gridDim.x * blockDim.x) {
    const long long v = (long long)rho[k];
    rho[k] = 0ull;
    out[k] = __ll2float_rn(v) * fx_inv;
  }
}

// massToOriginalUnits / massToCodeUnits factors as the reference's float expressions
// (include/unitConversions.h:42-47).
float mass_to_orig_factor(float H, float DT, float G) {
  volatile float c = (H * H * H) / (DT * DT * 4 * std::numbers::pi_v<float> * G);
  return c;
}
float mass_to_code_factor(float H, float DT, float G) {
  volatile float c = DT * DT * 4 * std::numbers::pi_v<float> * G / (H * H * H);
  return c;
}

DiagConsts consts(const pmgb_pm* h, int record, int tag) {
  DiagConsts c;
  c.H = h->cfg.H;
  c.DT = h->cfg.DT;
  c.m_to_orig = mass_to_orig_factor(h->cfg.H, h->cfg.DT, h->cfg.G);
  c.m_to_code = mass_to_code_factor(h->cfg.H, h->cfg.DT, h->cfg.G);
  c.ext = h->sp.ext;
  c.n = h->n;
  c.record = record;
  c.round_trip = record;
  c.tag = tag;
  return c;
}

int launch_records(pmgb_pm* h, int record, int tag) {
  pmgb_diag* d = h->diag;
  const DiagConsts c = consts(h, record, tag);
  diag_particles_kernel<<<DIAG_BLOCKS, DIAG_THREADS, 0, h->st>>>(h->pm[h->cur], h->vi[h->cur],
                                                                 h->acc, c, h->flags, d->part);
  int k = 2;
  double kmesh = 0.0;
  if (record) {
    diag_mesh_kernel<<<DIAG_BLOCKS, DIAG_THREADS, 0, h->st>>>(d->rho, h->phi, h->m.L, tag,
                                                              h->flags, d->mpart);
    ++k;
    // 0.5 * vol * densityToOriginalUnits * potentialToOriginalUnits, in double
    const double H = h->cfg.H, DT = h->cfg.DT, G = h->cfg.G;
    kmesh = 0.5 * (H * H * H) / (DT * DT * 4.0 * std::numbers::pi * G) * (H * H / (DT * DT));
  }
  diag_finalize_kernel<<<1, 32, 0, h->st>>>(d->part, d->mpart, c, kmesh, h->flags, d->state,
                                            d->rec, d->cap, d->count);
  PMGB_LAUNCH_CHECK();
  count_launches(k);
  return PMGB_OK;
}

template <typename T>
int dmalloc(T** p, size_t count) {
  if (cudaMalloc((void**)p, count * sizeof(T) + 16) != cudaSuccess) {
    set_error("cudaMalloc failed (diagnostics)");
    return PMGB_ENOMEM;
  }
  return PMGB_OK;
}

}  // namespace

float* diag_density(pmgb_pm* h) {
  if (!h->diag) return nullptr;
  h->diag->rho_valid = true;  // the caller's Poisson solve fills it
  return h->diag->rho;
}

int diag_run_begin(pmgb_pm* h) {
  if (!h->diag) return PMGB_OK;
  PMGB_CUDA_TRY(cudaMemsetAsync(h->diag->count, 0, sizeof(int), h->st));
  return launch_records(h, 0, 0);
}

int diag_before_drift(pmgb_pm* h) {
  pmgb_diag* d = h->diag;
  if (!d || d->rho_valid || h->n == 0) return PMGB_OK;
  int rc = launch_deposit(h->cfg.interpolation, h->pm[h->cur], h->n, h->m, h->sp.fx_scale, h->rho,
                          h->flags, h->st);
  if (rc) return rc;
  fx_to_float_kernel<<<4 * h->num_sms, 256, 0, h->st>>>(h->rho, d->rho, h->m.L, h->sp.fx_inv);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  d->rho_valid = true;
  return PMGB_OK;
}

int diag_after_drift(pmgb_pm* h, int tag) {
  if (!h->diag) return PMGB_OK;
  return launch_records(h, 1, tag);
}

int diag_capacity(const pmgb_pm* h) { return h->diag ? h->diag->cap : 0; }

int diag_save(pmgb_pm* h, unsigned char* save) {
  pmgb_diag* d = h->diag;
  if (!d) return PMGB_OK;
  PMGB_CUDA_TRY(cudaMemcpyAsync(save, d->state, 3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(save + 3 * sizeof(double), d->count, sizeof(int), cudaMemcpyDeviceToDevice, h->st));
  return PMGB_OK;
}

int diag_restore(pmgb_pm* h, const unsigned char* save) {
  pmgb_diag* d = h->diag;
  if (!d) return PMGB_OK;
  PMGB_CUDA_TRY(cudaMemcpyAsync(d->state, save, 3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(d->count, save + 3 * sizeof(double), sizeof(int), cudaMemcpyDeviceToDevice, h->st));
  d->rho_valid = false;  // the density buffer holds the abandoned step's
  return PMGB_OK;
}

void diag_free(pmgb_pm* h) {
  pmgb_diag* d = h->diag;
  if (!d) return;
  void* ptrs[] = {d->rho, d->part, d->mpart, d->state, d->rec, d->count};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete d;
  h->diag = nullptr;
}

}  // namespace pmgb

using namespace pmgb;

extern "C" {

int pmgb_pm_set_diagnostics(pmgb_pm* h, int capacity) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  if (capacity < 0) return set_error("negative diagnostics capacity"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  diag_free(h);
  if (capacity == 0) return PMGB_OK;
  pmgb_diag* d = new pmgb_diag();
  h->diag = d;
  d->cap = capacity;
  int rc;
  if ((rc = dmalloc(&d->rho, (size_t)h->m.L)) || (rc = dmalloc(&d->part, (size_t)12 * DIAG_BLOCKS)) ||
      (rc = dmalloc(&d->mpart, (size_t)DIAG_BLOCKS)) || (rc = dmalloc(&d->state, 3)) ||
      (rc = dmalloc(&d->rec, (size_t)PMGB_DIAG_WIDTH * capacity)) || (rc = dmalloc(&d->count, 1))) {
    diag_free(h);
    return rc;
  }
  if (cudaMemsetAsync(d->rho, 0, (size_t)h->m.L * sizeof(float), h->st) != cudaSuccess) {
    diag_free(h);
    return set_error("cudaMemset failed"), PMGB_ECUDA;
  }
  // the expected momentum starts at the current momentum (setInitialMomentum)
  rc = diag_run_begin(h);
  if (rc) {
    diag_free(h);
    return rc;
  }
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  return PMGB_OK;
}

int pmgb_pm_get_diagnostics(pmgb_pm* h, double* records, int max_records, int* count) {
  if (!h || !count) return set_error("null argument"), PMGB_EINVAL;
  if (max_records < 0 || (max_records > 0 && !records)) return set_error("bad record buffer"), PMGB_EINVAL;
  *count = 0;
  if (!h->diag) return PMGB_OK;
  int taken = 0;
  PMGB_CUDA_TRY(cudaMemcpyAsync(&taken, h->diag->count, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  const int k = std::min(std::min(taken, h->diag->cap), max_records);
  if (k > 0)
    PMGB_CUDA_TRY(cudaMemcpyAsync(records, h->diag->rec, (size_t)k * PMGB_DIAG_WIDTH * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  *count = taken;
  return PMGB_OK;
}

}  // extern "C"
