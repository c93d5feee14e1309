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
#include "interp_body.cuh"

namespace pmgb {

template <int IS, int FDS, bool KDK, bool POW2>
__global__ void __launch_bounds__(256) interp_kernel(float4* __restrict__ pm, float4* __restrict__ vi,
                                                     float4* __restrict__ acc, int n,
                                                     const float* __restrict__ phi, StepParams sp,
                                                     float kick, int drift, int* stop) {
  if (stopped_before(stop, KDK && drift, sp.step_tag)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  interp_particle<IS, FDS, KDK, POW2>(pm, vi, acc, i, phi, sp, kick, drift, stop);
}

template <int IS, int FDS>
static void launch_interp_t(bool kdk, float4* pm, float4* vi, float4* acc, int n, const float* phi,
                            const StepParams& sp, float kick, int drift, int* stop, cudaStream_t st) {
  const int blocks = (n + 255) / 256;
  const MeshDims& m = sp.m;
  const bool p2 = !(m.nx & (m.nx - 1)) && !(m.ny & (m.ny - 1)) && !(m.nz & (m.nz - 1));
  auto k = kdk ? (p2 ? interp_kernel<IS, FDS, true, true> : interp_kernel<IS, FDS, true, false>)
               : (p2 ? interp_kernel<IS, FDS, false, true> : interp_kernel<IS, FDS, false, false>);
  k<<<blocks, 256, 0, st>>>(pm, vi, acc, n, phi, sp, kick, drift, stop);
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
  if (stopped_before(stop, drift != 0, sp.step_tag)) return;
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
