// interp_body.cuh - finite-difference field, interpolation and the fused leapfrog for one
// particle (shared by the single-system and the ensemble kernels).  See interp.cu.
#pragma once
#include "common.cuh"

namespace pmgb {

template <bool POW2>
__device__ __forceinline__ float phi_at(const float* __restrict__ phi, const MeshDims& m, int x,
                                        int y, int z) {
  if (POW2)
    return __ldg(&phi[((size_t)wrapi_p2(z, m.nz) * m.ny + wrapi_p2(y, m.ny)) * m.nx + wrapi_p2(x, m.nx)]);
  return __ldg(&phi[((size_t)wrapi(z, m.nz) * m.ny + wrapi(y, m.ny)) * m.nx + wrapi(x, m.nx)]);
}

// Where the potential is read: the mesh in global memory, indices wrapped periodically as in
// Grid::getPotential (reference source/grid.cpp:66-68); POW2: every side a power of two.
template <bool POW2>
struct PhiGlobal {
  const float* __restrict__ phi;
  MeshDims m;
  __device__ __forceinline__ float operator()(int x, int y, int z) const { return phi_at<POW2>(phi, m, x, y, z); }
};

template <int FDS, class Phi>
__device__ __forceinline__ float3 field_at(const Phi& phi_at, int x, int y, int z) {
  float3 f;
  if (FDS == 0) {
    f.x = -0.5f * (phi_at(x + 1, y, z) - phi_at(x - 1, y, z));
    f.y = -0.5f * (phi_at(x, y + 1, z) - phi_at(x, y - 1, z));
    f.z = -0.5f * (phi_at(x, y, z + 1) - phi_at(x, y, z - 1));
  } else {
    const float c = -1.0f / 12;
    f.x = c * (-phi_at(x + 2, y, z) + 8 * phi_at(x + 1, y, z) - 8 * phi_at(x - 1, y, z) + phi_at(x - 2, y, z));
    f.y = c * (-phi_at(x, y + 2, z) + 8 * phi_at(x, y + 1, z) - 8 * phi_at(x, y - 1, z) + phi_at(x, y - 2, z));
    f.z = c * (-phi_at(x, y, z + 2) + 8 * phi_at(x, y, z + 1) - 8 * phi_at(x, y, z - 1) + phi_at(x, y, z - 2));
  }
  return f;
}

template <int IS, int FDS, class Phi>
__device__ __forceinline__ float3 interpolate(const Phi& phi, float x, float y, float z) {
  float3 r = make_float3(0.f, 0.f, 0.f);
  if (IS == 0) {
    return field_at<FDS>(phi, (int)roundf(x), (int)roundf(y), (int)roundf(z));
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
      float3 f = field_at<FDS>(phi, xi + ox[c], yi + oy[c], zi + oz[c]);
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
          float3 f = field_at<FDS>(phi, xi + t1, yi + t2, zi + t3);
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


// One particle: interpolated field + external field -> acc[i]; with KDK also kick / drift.
template <int IS, int FDS, bool KDK, class Phi>
__device__ __forceinline__ void interp_particle_p(float4* __restrict__ pm, float4* __restrict__ vi,
                                                  float4* __restrict__ acc, int i, float4 p,
                                                  const Phi& phi, const StepParams& sp, float kick,
                                                  int drift, int* stop) {
  float3 a = interpolate<IS, FDS>(phi, p.x, p.y, p.z);
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

template <int IS, int FDS, bool KDK, bool POW2 = true>
__device__ __forceinline__ void interp_particle(float4* __restrict__ pm, float4* __restrict__ vi,
                                                float4* __restrict__ acc, int i,
                                                const float* __restrict__ phi, const StepParams& sp,
                                                float kick, int drift, int* stop) {
  interp_particle_p<IS, FDS, KDK>(pm, vi, acc, i, pm[i], PhiGlobal<POW2>{phi, sp.m}, sp, kick, drift, stop);
}

}  // namespace pmgb
