// interp.cu - finite-difference field + force interpolation + leapfrog, fused.
//
// Restates, per particle, the reference's findFieldInCells + interpolateField +
// updateAccelerations (source/pmMethod.cpp:279-338, 352-390): the field of each stencil cell is
// computed on the fly from the potential by the 2- or 4-point difference with periodically
// wrapped reads (Grid::getPotential, source/grid.cpp:66-68) instead of being stored as a mesh;
// the external field is added in code units.
//
// Modes:
//   ACC   write the acceleration (pmMethodStep; also the PM part of a P3M step)
//   KDK   PM-only run step: v += kick * a, then (if drift) x += v, the reference's unit round
//         trip (stateToOriginalUnits / stateToCodeUnits, source/pmMethod.cpp:87-113), and the
//         escapedComputationalBox test on original-unit positions.  An escaped particle sets
//         *stop, which every later kernel checks first, so nothing after the escaping drift
//         runs: the state is left exactly where the reference's loop breaks.
#include "common.cuh"

namespace pmgb {

__device__ __forceinline__ float phi_at(const float* __restrict__ phi, const MeshDims& m, int x,
                                        int y, int z) {
  return __ldg(&phi[((size_t)wrapi(z, m.nz) * m.ny + wrapi(y, m.ny)) * m.nx + wrapi(x, m.nx)]);
}

template <int FDS>
__device__ __forceinline__ float3 field_at(const float* __restrict__ phi, const MeshDims& m, int x,
                                           int y, int z) {
  float3 f;
  if (FDS == 0) {
    f.x = -0.5f * (phi_at(phi, m, x + 1, y, z) - phi_at(phi, m, x - 1, y, z));
    f.y = -0.5f * (phi_at(phi, m, x, y + 1, z) - phi_at(phi, m, x, y - 1, z));
    f.z = -0.5f * (phi_at(phi, m, x, y, z + 1) - phi_at(phi, m, x, y, z - 1));
  } else {
    const float c = -1.0f / 12;
    f.x = c * (-phi_at(phi, m, x + 2, y, z) + 8 * phi_at(phi, m, x + 1, y, z) -
               8 * phi_at(phi, m, x - 1, y, z) + phi_at(phi, m, x - 2, y, z));
    f.y = c * (-phi_at(phi, m, x, y + 2, z) + 8 * phi_at(phi, m, x, y + 1, z) -
               8 * phi_at(phi, m, x, y - 1, z) + phi_at(phi, m, x, y - 2, z));
    f.z = c * (-phi_at(phi, m, x, y, z + 2) + 8 * phi_at(phi, m, x, y, z + 1) -
               8 * phi_at(phi, m, x, y, z - 1) + phi_at(phi, m, x, y, z - 2));
  }
  return f;
}

template <int IS, int FDS>
__device__ __forceinline__ float3 interpolate(const float* __restrict__ phi, const MeshDims& m,
                                              float x, float y, float z) {
  float3 r = make_float3(0.f, 0.f, 0.f);
  if (IS == 0) {
    return field_at<FDS>(phi, m, (int)roundf(x), (int)roundf(y), (int)roundf(z));
  } else if (IS == 1) {
    const int xi = (int)x, yi = (int)y, zi = (int)z;
    const float dx = x - xi, dy = y - yi, dz = z - zi;
    const float tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
    const float w[8] = {tx * ty * tz, dx * ty * tz, tx * dy * tz, tx * ty * dz,
                        dx * dy * tz, dx * ty * dz, tx * dy * dz, dx * dy * dz};
    const int ox[8] = {0, 1, 0, 0, 1, 1, 0, 1}, oy[8] = {0, 0, 1, 0, 1, 0, 1, 1},
              oz[8] = {0, 0, 0, 1, 0, 1, 1, 1};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      float3 f = field_at<FDS>(phi, m, xi + ox[c], yi + oy[c], zi + oz[c]);
      r.x += w[c] * f.x;
      r.y += w[c] * f.y;
      r.z += w[c] * f.z;
    }
  } else {
    const int xi = (int)x, yi = (int)y, zi = (int)z;
    const float dx = x - xi, dy = y - yi, dz = z - zi;
#pragma unroll
    for (int t1 = -1; t1 <= 1; ++t1) {
      const float T1 = tsc_w(dx, t1);
#pragma unroll
      for (int t2 = -1; t2 <= 1; ++t2) {
        const float T2 = T1 * tsc_w(dy, t2);
#pragma unroll
        for (int t3 = -1; t3 <= 1; ++t3) {
          const float w = 0.125f * (T2 * tsc_w(dz, t3));
          float3 f = field_at<FDS>(phi, m, xi + t1, yi + t2, zi + t3);
          r.x += w * f.x;
          r.y += w * f.y;
          r.z += w * f.z;
        }
      }
    }
  }
  return r;
}

// sphRadDecrField (reference source/externalFields.cpp:4-15) at H*x, in code units
// (accelerationToCodeUnits: DT*DT*a/H).
__device__ __forceinline__ float3 external_field(const StepParams& sp, float x, float y, float z) {
  if (sp.ext.kind != PMGB_EXT_SPH_RAD_DECR) return make_float3(0.f, 0.f, 0.f);
  const float px = sp.H * x - sp.ext.cx, py = sp.H * y - sp.ext.cy, pz = sp.H * z - sp.ext.cz;
  const float r = sqrtf(px * px + py * py + pz * pz);
  const float R = sp.ext.R;
  const float g = r > R ? -sp.ext.G * sp.ext.M / (r * r)
                        : -(sp.ext.G * sp.ext.M / (R * R * R)) * r * (4 - 3 * r / R);
  const float s = (sp.DT * sp.DT) * g / r / sp.H;
  return make_float3(s * px, s * py, s * pz);
}


template <int IS, int FDS, bool KDK>
__global__ void __launch_bounds__(256) interp_kernel(float4* __restrict__ pm, float4* __restrict__ vi,
                                                     float4* __restrict__ acc, int n,
                                                     const float* __restrict__ phi, StepParams sp,
                                                     float kick, int drift, int* stop) {
  if (*stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pm[i];
  float3 a = interpolate<IS, FDS>(phi, sp.m, p.x, p.y, p.z);
  const float3 e = external_field(sp, p.x, p.y, p.z);
  a.x += e.x;
  a.y += e.y;
  a.z += e.z;
  acc[i] = make_float4(a.x, a.y, a.z, 0.f);
  if (KDK) {
    float4 v = vi[i];
    kick_drift(sp, p, v, a, kick, drift, stop);
    pm[i] = p;
    vi[i] = v;
  }
}

template <int IS, int FDS>
static void launch_interp_t(bool kdk, float4* pm, float4* vi, float4* acc, int n, const float* phi,
                            const StepParams& sp, float kick, int drift, int* stop, cudaStream_t st) {
  const int blocks = (n + 255) / 256;
  if (kdk)
    interp_kernel<IS, FDS, true><<<blocks, 256, 0, st>>>(pm, vi, acc, n, phi, sp, kick, drift, stop);
  else
    interp_kernel<IS, FDS, false><<<blocks, 256, 0, st>>>(pm, vi, acc, n, phi, sp, kick, drift, stop);
}

int launch_interp(bool kdk, float4* pm, float4* vi, float4* acc, int n, const float* phi,
                  const StepParams& sp, float kick, int drift, int* stop, cudaStream_t st) {
  if (n <= 0) return PMGB_OK;
  switch (sp.is * 2 + sp.fds) {
    case 0: launch_interp_t<0, 0>(kdk, pm, vi, acc, n, phi, sp, kick, drift, stop, st); break;
    case 1: launch_interp_t<0, 1>(kdk, pm, vi, acc, n, phi, sp, kick, drift, stop, st); break;
    case 2: launch_interp_t<1, 0>(kdk, pm, vi, acc, n, phi, sp, kick, drift, stop, st); break;
    case 3: launch_interp_t<1, 1>(kdk, pm, vi, acc, n, phi, sp, kick, drift, stop, st); break;
    case 4: launch_interp_t<2, 0>(kdk, pm, vi, acc, n, phi, sp, kick, drift, stop, st); break;
    default: launch_interp_t<2, 1>(kdk, pm, vi, acc, n, phi, sp, kick, drift, stop, st); break;
  }
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

// Kick / drift only (the P3M epilogue when the pair pass is skipped, and the initial half kick).
__global__ void kick_drift_kernel(float4* __restrict__ pm, float4* __restrict__ vi,
                                  const float4* __restrict__ acc, int n, StepParams sp, float kick,
                                  int drift, int* stop) {
  if (*stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pm[i], v = vi[i];
  const float4 a = acc[i];
  kick_drift(sp, p, v, make_float3(a.x, a.y, a.z), kick, drift, stop);
  pm[i] = p;
  vi[i] = v;
}

int launch_kick_drift(float4* pm, float4* vi, const float4* acc, int n, const StepParams& sp,
                      float kick, int drift, int* stop, cudaStream_t st) {
  if (n <= 0) return PMGB_OK;
  kick_drift_kernel<<<(n + 255) / 256, 256, 0, st>>>(pm, vi, acc, n, sp, kick, drift, stop);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

}  // namespace pmgb
