// samplers.cu - initial conditions on the device: the reference's PlummerSampler
// (source/plummerSampler.cpp:11-83) and DiskSamplerLinear (source/diskSamplerLinear.cpp:10-74),
// one thread per particle, with the same random stream.
//
// The reference draws from std::default_random_engine(seed) (libstdc++: minstd_rand0,
// x <- 16807 x mod (2^31 - 1), x0 = seed mod (2^31 - 1), 1 if that is 0) through
// uniform_real_distribution<float>(0, 1), i.e. generate_canonical<float, 24>: one engine draw
// per number, u = float(x - 1) / float(2^31 - 2) (that divisor rounds to 2^31), clamped below 1.
// Particle i of a Plummer sample uses draws 6i+1 .. 6i+6 (position: phi, r, theta; velocity:
// cdf, phi, theta), of a linear disk draws 3i+1 .. 3i+3 (phi, cdf of r, z); a thread jumps to
// its draws by modular exponentiation (x_k = 16807^k x0 mod m), so the sample is the
// reference's sequence, not merely the same distribution.  The arithmetic follows the
// reference's float expressions (CUDA's libm may differ from the host's by an ulp; Newton
// iterations then land within the solver tolerance's square of the same root).
#include <cmath>
#include <numbers>

#include "handles.cuh"

namespace pmgb {

namespace {

constexpr unsigned long long kLcgM = 2147483647ull;  // 2^31 - 1
constexpr unsigned long long kLcgA = 16807ull;

__host__ __device__ inline unsigned long long lcg_pow(unsigned long long k) {
  unsigned long long r = 1, b = kLcgA;
  while (k) {
    if (k & 1) r = r * b % kLcgM;
    b = b * b % kLcgM;
    k >>= 1;
  }
  return r;
}

struct Lcg {
  unsigned long long x;
  __device__ float next() {
    x = x * kLcgA % kLcgM;
    float u = __fdiv_rn(__uint2float_rn((unsigned)(x - 1)), 2147483648.0f);
    return u >= 1.0f ? 0.99999994f : u;  // nextafter(1, 0)
  }
};

__device__ __forceinline__ Lcg lcg_at(unsigned long long x0, unsigned long long draws) {
  return Lcg{lcg_pow(draws) * x0 % kLcgM};
}

// reference utils.cpp newton(): x -= f(x) / df(x) until |x - xPrev| <= tol or maxIter
template <class F, class D>
__device__ float newton(F f, D df, float guess, int max_iter, float tol) {
  int i = 0;
  float err = tol + 1;
  float x = guess;
  while (err > tol && i < max_iter) {
    ++i;
    const float prev = x;
    x = x - f(x) / df(x);
    err = fabsf(x - prev);
  }
  return x;
}

struct PlummerArgs {
  float cx, cy, cz, a, r_max, M, G;
  int n;
  unsigned long long x0, offset;
};

__global__ void plummer_kernel(PlummerArgs p, float* __restrict__ state) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  Lcg g = lcg_at(p.x0, p.offset + 6ull * i);
  const float pi = std::numbers::pi_v<float>;
  // getPosition
  const float phi = 2 * pi * g.next();
  float r = p.a * powf(powf(g.next(), -2.0f / 3) - 1, (float)(-1.0 / 2));
  if (r > p.r_max) r = p.r_max;
  const float theta = acosf(1 - 2 * g.next());
  state[3 * i] = p.cx + r * sinf(theta) * cosf(phi);
  state[3 * i + 1] = p.cy + r * sinf(theta) * sinf(phi);
  state[3 * i + 2] = p.cz + r * cosf(theta);
  // getVelocity
  const float norm = 512.0f / (7 * pi);
  const float potential = -p.G * p.M / sqrtf(r * r + p.a * p.a);
  const float v_esc = sqrtf(-2 * potential);
  const float cdf = g.next();
  auto cdf_f = [&](float x) {
    const float sq = sqrtf(1 - x * x);
    const float at = atanf(x / sq);
    const float num = x * sq * (-105 + 1210 * x * x - 2104 * powf(x, 4) + 1488 * powf(x, 6) -
                                384 * powf(x, 8)) + 105 * at;
    return (num / 3840.0f) * norm - cdf;
  };
  auto pdf = [&](float x) { return x * x * powf(1 - x * x, 3.5f) * norm; };
  const float q = newton(cdf_f, pdf, 0.5f, 100, 1e-3f);
  const float v = q * v_esc;
  const float vphi = 2 * pi * g.next();
  const float vtheta = acosf(1 - 2 * g.next());
  float* vel = state + 3 * (size_t)p.n;
  vel[3 * i] = v * sinf(vtheta) * cosf(vphi);
  vel[3 * i + 1] = v * sinf(vtheta) * sinf(vphi);
  vel[3 * i + 2] = v * cosf(vtheta);
}

struct DiskArgs {
  float cx, cy, cz, rb, mb, rd, md, thickness, G, r0;
  int n;
  unsigned long long x0, offset;
};

__global__ void disk_linear_kernel(DiskArgs p, float* __restrict__ state) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  Lcg g = lcg_at(p.x0, p.offset + 3ull * i);
  const float pi = std::numbers::pi_v<float>;
  const float phi = g.next() * 2 * pi;
  // sampleFromLinear: root of the implicit inverse CDF (diskSamplerLinear.h:31-37)
  const float cdf = g.next();
  const float rd = p.rd, r0 = p.r0;
  auto f = [&](float r) {
    return 2 * powf(r, 3) - 3 * rd * r * r + cdf * powf(rd - r0, 2) * (2 * r0 + rd) - 2 * powf(r0, 3) +
           3 * rd * r0 * r0;
  };
  auto df = [&](float r) { return 6 * r * r - 6 * rd * r; };
  const float r = newton(f, df, rd / 2.0f, 100, 0.01f);
  const float x = r * cosf(phi), y = r * sinf(phi);
  const float z = (p.thickness / 2) * (2 * g.next() - 1);
  const float px = p.cx + x, py = p.cy + y, pz = p.cz + z;
  state[3 * i] = px;
  state[3 * i + 1] = py;
  state[3 * i + 2] = pz;
  // getVelocity (diskSamplerLinear.cpp:37-65)
  const float rx = px - p.cx, ry = py - p.cy, rz = pz - p.cz;
  const float rr = sqrtf(rx * rx + ry * ry + rz * rz);
  const float rho = sqrtf(rx * rx + ry * ry);
  const float ra = rr / rd;
  const float sigma0 = 3 * p.md / (pi * rd * rd);
  const float k = 2.5f, h = 0.66f;
  const float aa = -k / (h * h);
  const float gd_val = -p.G * sigma0 * (aa * (ra - h) * (ra - h) + k);
  // sphRadDecrField(pos, center, rb, mb, G) (externalFields.cpp:4-15)
  float gbx, gby, gbz;
  {
    const float dir_x = rx / rr, dir_y = ry / rr, dir_z = rz / rr;
    const float gg = rr > p.rb ? -p.G * p.mb / (rr * rr)
                               : -(p.G * p.mb / powf(p.rb, 3)) * rr * (4 - 3 * rr / p.rb);
    gbx = gg * dir_x;
    gby = gg * dir_y;
    gbz = gg * dir_z;
  }
  const float gx = gbx + gd_val * rx / rho, gy = gby + gd_val * ry / rho, gz = gbz + gd_val * 0.0f / rho;
  const float g_val = sqrtf(gx * gx + gy * gy + gz * gz);
  const float v = sqrtf(g_val * rho * rho / rr);
  float* vel = state + 3 * (size_t)p.n;
  vel[3 * i] = -v * ry / rho;
  vel[3 * i + 1] = v * rx / rho;
  vel[3 * i + 2] = 0.0f;
}

unsigned long long seed_state(unsigned int seed) {
  const unsigned long long s = seed % kLcgM;
  return s == 0 ? 1ull : s;
}

int run_sampler(int n, float* state_host, void (*launch)(float*, cudaStream_t, const void*),
                const void* args) {
  if (n <= 0) return PMGB_OK;
  float* d = nullptr;
  cudaStream_t st = nullptr;
  PMGB_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  if (cudaMalloc((void**)&d, (size_t)6 * n * sizeof(float)) != cudaSuccess) {
    cudaStreamDestroy(st);
    return set_error("cudaMalloc failed (sampler)"), PMGB_ENOMEM;
  }
  launch(d, st, args);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(state_host, d, (size_t)6 * n * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  cudaStreamDestroy(st);
  if (e != cudaSuccess) return set_error(std::string("sampler: ") + cudaGetErrorString(e)), PMGB_ECUDA;
  count_launches(1);
  return PMGB_OK;
}

}  // namespace

}  // namespace pmgb

using namespace pmgb;

extern "C" {

int pmgb_sample_plummer(unsigned int seed, unsigned long long offset, const float* center, float a,
                        float r_max, float M, float G, int n, float* state) {
  if (n < 0 || (n > 0 && (!state || !center))) return set_error("bad sampler arguments"), PMGB_EINVAL;
  PlummerArgs p{center ? center[0] : 0.f, center ? center[1] : 0.f, center ? center[2] : 0.f,
                a, r_max, M, G, n, seed_state(seed), offset};
  return run_sampler(n, state, [](float* d, cudaStream_t st, const void* args) {
    const PlummerArgs& q = *static_cast<const PlummerArgs*>(args);
    plummer_kernel<<<(q.n + 255) / 256, 256, 0, st>>>(q, d);
  }, &p);
}

int pmgb_sample_disk_linear(unsigned int seed, unsigned long long offset, const float* center,
                            float rb, float mb, float rd, float md, float thickness, float G, int n,
                            float r0, float* state) {
  if (n < 0 || (n > 0 && (!state || !center))) return set_error("bad sampler arguments"), PMGB_EINVAL;
  DiskArgs p{center ? center[0] : 0.f, center ? center[1] : 0.f, center ? center[2] : 0.f,
             rb, mb, rd, md, thickness, G, r0, n, seed_state(seed), offset};
  return run_sampler(n, state, [](float* d, cudaStream_t st, const void* args) {
    const DiskArgs& q = *static_cast<const DiskArgs*>(args);
    disk_linear_kernel<<<(q.n + 255) / 256, 256, 0, st>>>(q, d);
  }, &p);
}

}  // extern "C"
