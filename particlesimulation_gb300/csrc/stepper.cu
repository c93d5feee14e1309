// stepper.cu - the reference's leapfrog free functions and totalExternalForceOrigUnits as
// entry points of their own.
//
// The run loops fuse the leapfrog into the interpolation / pair epilogues (common.cuh
// kick_drift); these entry points expose the four operations of source/leapfrog.cpp:5-24 by
// themselves, for callers that step a particle set the way the reference's callers do:
//   setHalfStepVelocities     v += 0.5 dt a
//   updatePositions           x += dt v
//   updateVelocities          v += dt a
//   setIntegerStepVelocities  u = v + 0.5 dt a   (integerStepVelocity, include/particle.h:10)
// either on host arrays (the reference's std::vector<Particle> argument) or on a PM handle's
// particles on the device (code units, the accelerations of its last force evaluation), and
// PMMethod::totalExternalForceOrigUnits (source/pmMethod.cpp:158-162): sum m g(x) over the
// particles in original units, summed in double in a fixed order.
#include <algorithm>
#include <vector>

#include "handles.cuh"

namespace pmgb {

// the float arithmetic of leapfrog.cpp: 0.5f * dt * a (left to right), then the add
__device__ __forceinline__ float half_dt(float dt) { return __fmul_rn(0.5f, dt); }

__global__ void leapfrog_arrays_kernel(int op, int n, float* __restrict__ pos, float* __restrict__ vel,
                                       const float* __restrict__ acc, float* __restrict__ ivel, float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  switch (op) {
    case PMGB_LEAPFROG_HALF_KICK: vel[i] = __fadd_rn(vel[i], __fmul_rn(half_dt(dt), acc[i])); break;
    case PMGB_LEAPFROG_DRIFT: pos[i] = __fadd_rn(pos[i], __fmul_rn(dt, vel[i])); break;
    case PMGB_LEAPFROG_KICK: vel[i] = __fadd_rn(vel[i], __fmul_rn(dt, acc[i])); break;
    default: ivel[i] = __fadd_rn(vel[i], __fmul_rn(half_dt(dt), acc[i])); break;
  }
}

// on a handle's particles (sorted order); integer-step velocities go to ivel in original order
__global__ void leapfrog_handle_kernel(int op, int n, float4* __restrict__ pm, float4* __restrict__ vi,
                                       const float4* __restrict__ acc, float4* __restrict__ ivel, float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 v = vi[i];
  const float4 a = acc[i];
  if (op == PMGB_LEAPFROG_DRIFT) {
    float4 p = pm[i];
    p.x = __fadd_rn(p.x, __fmul_rn(dt, v.x));
    p.y = __fadd_rn(p.y, __fmul_rn(dt, v.y));
    p.z = __fadd_rn(p.z, __fmul_rn(dt, v.z));
    pm[i] = p;
    return;
  }
  const float k = op == PMGB_LEAPFROG_KICK ? dt : half_dt(dt);
  const float ux = __fadd_rn(v.x, __fmul_rn(k, a.x));
  const float uy = __fadd_rn(v.y, __fmul_rn(k, a.y));
  const float uz = __fadd_rn(v.z, __fmul_rn(k, a.z));
  if (op == PMGB_LEAPFROG_INTEGER_STEP) {
    const int id = __float_as_int(v.w);
    ivel[id] = make_float4(ux, uy, uz, 0.f);
    return;
  }
  v.x = ux;
  v.y = uy;
  v.z = uz;
  vi[i] = v;
}

constexpr int EXT_THREADS = 256, EXT_BLOCKS = 304;

// sum over particles of m g(H x) in original units: per-block double sums, added on the host
// in block order
__global__ void __launch_bounds__(EXT_THREADS) ext_force_kernel(const float4* __restrict__ pm, int n,
                                                               float H, float m_code_per_orig, ExtField e,
                                                               double* __restrict__ part) {
  double s[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * EXT_THREADS + threadIdx.x; i < n; i += EXT_BLOCKS * EXT_THREADS) {
    const float4 p = pm[i];
    const double m = __fdiv_rn(p.w, m_code_per_orig);  // massToOriginalUnits
    const double x = __fmul_rn(H, p.x), y = __fmul_rn(H, p.y), z = __fmul_rn(H, p.z);
    const double dx = x - (double)e.cx, dy = y - (double)e.cy, dz = z - (double)e.cz;
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    const double R = e.R, GM = (double)e.G * (double)e.M;
    const double g = r > R ? -GM / (r * r) : -(GM / (R * R * R)) * r * (4.0 - 3.0 * r / R);
    if (r > 0.0) {
      s[0] += m * g * dx / r;
      s[1] += m * g * dy / r;
      s[2] += m * g * dz / r;
    }
  }
  __shared__ double sm[EXT_THREADS / 32][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 3; ++k) {
    double a = s[k];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xFFFFFFFFu, a, o);
    if (lane == 0) sm[warp][k] = a;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double a = 0.0;
    for (int w = 0; w < EXT_THREADS / 32; ++w) a += sm[w][threadIdx.x];
    part[3 * blockIdx.x + threadIdx.x] = a;
  }
}

}  // namespace pmgb

using namespace pmgb;

extern "C" int pmgb_leapfrog(int op, int n, float* pos, float* vel, const float* acc, float* int_vel,
                             float dt) {
  if (op < PMGB_LEAPFROG_HALF_KICK || op > PMGB_LEAPFROG_INTEGER_STEP || n < 0)
    return set_error("pmgb_leapfrog: bad operation or count"), PMGB_EINVAL;
  const bool need_pos = op == PMGB_LEAPFROG_DRIFT;
  const bool need_acc = op != PMGB_LEAPFROG_DRIFT;
  const bool need_ivel = op == PMGB_LEAPFROG_INTEGER_STEP;
  if (n > 0 && (!vel || (need_pos && !pos) || (need_acc && !acc) || (need_ivel && !int_vel)))
    return set_error("pmgb_leapfrog: null array"), PMGB_EINVAL;
  if (n == 0) return PMGB_OK;
  const size_t bytes = sizeof(float) * 3 * (size_t)n;
  float *dp = nullptr, *dv = nullptr, *da = nullptr, *du = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess && need_pos) e = cudaMalloc(&dp, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&dv, bytes);
  if (e == cudaSuccess && need_acc) e = cudaMalloc(&da, bytes);
  if (e == cudaSuccess && need_ivel) e = cudaMalloc(&du, bytes);
  if (e == cudaSuccess && need_pos) e = cudaMemcpyAsync(dp, pos, bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dv, vel, bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && need_acc) e = cudaMemcpyAsync(da, acc, bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    leapfrog_arrays_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(op, n, dp, dv, da, du, dt);
    count_launches(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    if (op == PMGB_LEAPFROG_DRIFT) e = cudaMemcpyAsync(pos, dp, bytes, cudaMemcpyDeviceToHost, st);
    else if (need_ivel) e = cudaMemcpyAsync(int_vel, du, bytes, cudaMemcpyDeviceToHost, st);
    else e = cudaMemcpyAsync(vel, dv, bytes, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int rc = PMGB_OK;
  if (e != cudaSuccess) {
    set_error(std::string("pmgb_leapfrog: ") + cudaGetErrorString(e));
    rc = e == cudaErrorMemoryAllocation ? PMGB_ENOMEM : PMGB_ECUDA;
  }
  cudaFree(dp);
  cudaFree(dv);
  cudaFree(da);
  cudaFree(du);
  if (st) cudaStreamDestroy(st);
  return rc;
}

extern "C" int pmgb_pm_leapfrog(pmgb_pm* h, int op, float dt) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  if (op < PMGB_LEAPFROG_HALF_KICK || op > PMGB_LEAPFROG_INTEGER_STEP)
    return set_error("pmgb_pm_leapfrog: bad operation"), PMGB_EINVAL;
  if (h->n == 0) return PMGB_OK;
  if (op == PMGB_LEAPFROG_INTEGER_STEP && !h->ivel) {
    PMGB_CUDA_TRY(cudaMalloc(&h->ivel, sizeof(float4) * (size_t)h->n));
    PMGB_CUDA_TRY(cudaMemsetAsync(h->ivel, 0, sizeof(float4) * (size_t)h->n, h->st));
  }
  if (op == PMGB_LEAPFROG_DRIFT) h->acc_mode = -1;  // accelerations of the old positions
  leapfrog_handle_kernel<<<(h->n + 255) / 256, 256, 0, h->st>>>(op, h->n, h->pm[h->cur], h->vi[h->cur],
                                                                h->acc, h->ivel, dt);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  return PMGB_OK;
}

extern "C" int pmgb_pm_get_integer_step_velocities(pmgb_pm* h, float* vel, int units) {
  if (!h || !vel) return set_error("null argument"), PMGB_EINVAL;
  const size_t n = (size_t)h->n;
  std::vector<float> u(4 * n, 0.f);
  if (h->ivel && n) {
    PMGB_CUDA_TRY(cudaMemcpyAsync(u.data(), h->ivel, sizeof(float4) * n, cudaMemcpyDeviceToHost, h->st));
    PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  }
  const float H = h->cfg.H, DT = h->cfg.DT;
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const float c = u[4 * i + k];
      vel[3 * i + k] = units == PMGB_UNITS_ORIGINAL ? H * c / DT : c;  // velocityToOriginalUnits
    }
  return PMGB_OK;
}

extern "C" int pmgb_pm_total_external_force(pmgb_pm* h, float* force3) {
  if (!h || !force3) return set_error("null argument"), PMGB_EINVAL;
  force3[0] = force3[1] = force3[2] = 0.f;
  if (h->sp.ext.kind != PMGB_EXT_SPH_RAD_DECR || h->n == 0) return PMGB_OK;
  // the float factor m_code / m_orig = DT^2 4 pi G / H^3 (include/unitConversions.h)
  const float c = mass_code_factor(h->cfg.H, h->cfg.DT, h->cfg.G);
  double* part = nullptr;
  PMGB_CUDA_TRY(cudaMalloc(&part, sizeof(double) * 3 * EXT_BLOCKS));
  ext_force_kernel<<<EXT_BLOCKS, EXT_THREADS, 0, h->st>>>(h->pm[h->cur], h->n, h->cfg.H, c, h->sp.ext, part);
  count_launches(1);
  std::vector<double> hp(3 * EXT_BLOCKS);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  cudaFree(part);
  if (e != cudaSuccess) return set_error(cudaGetErrorString(e)), PMGB_ECUDA;
  double s[3] = {0, 0, 0};
  for (int b = 0; b < EXT_BLOCKS; ++b)
    for (int k = 0; k < 3; ++k) s[k] += hp[3 * b + k];
  for (int k = 0; k < 3; ++k) force3[k] = (float)s[k];
  return PMGB_OK;
}
