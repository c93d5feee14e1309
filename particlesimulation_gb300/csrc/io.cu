// io.cu - particle state in and out of a handle, in the caller's index order and units.
//
// The device keeps particles in sorted order with their original id in vi.w; these kernels
// scatter / gather by that id and apply the reference's unit conversions
// (include/unitConversions.h:8-50: positionToOriginalUnits H*x, velocityToOriginalUnits H*v/DT,
// accelerationToOriginalUnits H*a/DT^2, and the inverses x/H, DT*v/H) so that host transfers are
// single contiguous copies.
#include "common.cuh"

namespace pmgb {

__global__ void unpack_kernel(const float4* __restrict__ pm, const float4* __restrict__ vi,
                              const float4* __restrict__ acc, int n, float H, float DT, int orig,
                              float* __restrict__ pos, float* __restrict__ vel,
                              float* __restrict__ aout) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float4 p = pm[k], v = vi[k], a = acc[k];
  const int i = __float_as_int(v.w);
  if (i < 0 || i >= n) return;
  if (orig) {
    pos[3 * i] = __fmul_rn(H, p.x);
    pos[3 * i + 1] = __fmul_rn(H, p.y);
    pos[3 * i + 2] = __fmul_rn(H, p.z);
    vel[3 * i] = __fdiv_rn(__fmul_rn(H, v.x), DT);
    vel[3 * i + 1] = __fdiv_rn(__fmul_rn(H, v.y), DT);
    vel[3 * i + 2] = __fdiv_rn(__fmul_rn(H, v.z), DT);
    const float dt2 = __fmul_rn(DT, DT);
    aout[3 * i] = __fdiv_rn(__fmul_rn(H, a.x), dt2);
    aout[3 * i + 1] = __fdiv_rn(__fmul_rn(H, a.y), dt2);
    aout[3 * i + 2] = __fdiv_rn(__fmul_rn(H, a.z), dt2);
  } else {
    pos[3 * i] = p.x;
    pos[3 * i + 1] = p.y;
    pos[3 * i + 2] = p.z;
    vel[3 * i] = v.x;
    vel[3 * i + 1] = v.y;
    vel[3 * i + 2] = v.z;
    aout[3 * i] = a.x;
    aout[3 * i + 1] = a.y;
    aout[3 * i + 2] = a.z;
  }
}

__global__ void pack_kernel(const float* __restrict__ pos, const float* __restrict__ vel,
                            const float* __restrict__ mass_code, int n, float H, float DT,
                            int orig, float4* __restrict__ pm, float4* __restrict__ vi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
  float vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
  if (orig) {
    x = __fdiv_rn(x, H);
    y = __fdiv_rn(y, H);
    z = __fdiv_rn(z, H);
    vx = __fdiv_rn(__fmul_rn(DT, vx), H);
    vy = __fdiv_rn(__fmul_rn(DT, vy), H);
    vz = __fdiv_rn(__fmul_rn(DT, vz), H);
  }
  pm[i] = make_float4(x, y, z, mass_code[i]);
  vi[i] = make_float4(vx, vy, vz, __int_as_float(i));
}

int launch_unpack(const float4* pm, const float4* vi, const float4* acc, int n, float H, float DT,
                  int orig, float* pos, float* vel, float* aout, cudaStream_t st) {
  if (n <= 0) return PMGB_OK;
  unpack_kernel<<<(n + 255) / 256, 256, 0, st>>>(pm, vi, acc, n, H, DT, orig, pos, vel, aout);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

int launch_pack(const float* pos, const float* vel, const float* mass_code, int n, float H,
                float DT, int orig, float4* pm, float4* vi, cudaStream_t st) {
  if (n <= 0) return PMGB_OK;
  pack_kernel<<<(n + 255) / 256, 256, 0, st>>>(pos, vel, mass_code, n, H, DT, orig, pm, vi);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

}  // namespace pmgb
