// green.cu - influence function, once per run, in FP64 on the device.
//
// Restates the reference's Green's function options (source/greensFunctions.cpp:8-221, chosen in
// PMMethod::initGreensFunction, source/pmMethod.cpp:164-185):
//   DISCRETE_LAPLACIAN  -1 / (4 sum sin^2(pi k_i / N_i))
//   POOR_MAN            -1 / |k|^2 with k wrapped to [-N/2, N/2]
//   S1/S2_OPTIMAL       Hockney-Eastwood optimal influence function: alias sum over
//                       n in [-2, 2]^3 of U^2(k_n) R(k_n), projected on the FD operator D(k),
//                       divided by |D|^2 (sum U^2)^2 with the closed-form alias sums.
// k = 0 is 0.  The stored value is the symmetric part (G(k) + G(-k)) / 2 over the kept half
// spectrum (the truncated alias sum is not exactly symmetric; the reference's real part of a
// complex inverse FFT applies exactly this symmetric part), times 1/(nx*ny*nz), the inverse
// FFT normalisation.  For the optimal function the 7 non-zero modes whose components are all 0
// or N/2 get 0: there D(k) = 0 and the reference divides float rounding noise by rounding
// noise; the finite-difference field annihilates these modes, so forces do not see them.
// S1(u), S2(u) use their Taylor series below u = 0.05, where the closed forms cancel.
#include "common.cuh"

namespace pmgb {

__device__ double d_sinc(double x) { return x == 0.0 ? 1.0 : sin(x) / x; }

__device__ double d_assign_fourier(int is, const double k[3]) {
  double prod = 1.0;
  for (int i = 0; i < 3; ++i) {
    double s = d_sinc(k[i] / 2);
    prod *= is == 2 ? s * s * s : (is == 1 ? s * s : s);
  }
  return prod;
}

__device__ double d_alias_sum(int is, const double k[3]) {
  if (is == 2) {
    double sum = 1.0;
    for (int i = 0; i < 3; ++i) {
      double s = sin(k[i] / 2), s2 = s * s;
      sum *= 1.0 - s2 + 2.0 / 15.0 * s2 * s2;
    }
    return sum;
  }
  if (is == 1) {
    double sum = 1.0;
    for (int i = 0; i < 3; ++i) {
      double c = cos(k[i] / 2);
      sum *= 1.0 + 2.0 * c * c;
    }
    return sum / 27.0;
  }
  return 1.0;
}

__device__ double d_shape(int cs, double k, double a) {
  double u = k * a / 2;
  double u2 = u * u;
  if (cs == 0) {
    if (u < 0.05) return 1.0 - u2 / 10.0 + u2 * u2 / 280.0;
    return -3.0 / (u2 * u) * (u * cos(u) - sin(u));
  }
  if (u < 0.05) return 1.0 - u2 / 15.0 + u2 * u2 / 560.0;
  return 12.0 / (u2 * u2) * (2.0 - 2.0 * cos(u) - u * sin(u));
}

__device__ double d_green(int gf, int is, int fds, int cs, double a, int kx, int ky, int kz,
                          const MeshDims& m) {
  const double PI = 3.14159265358979323846;
  if (kx == 0 && ky == 0 && kz == 0) return 0.0;
  if (gf == PMGB_DISCRETE_LAPLACIAN) {
    double sx = sin(PI * kx / m.nx), sy = sin(PI * ky / m.ny), sz = sin(PI * kz / m.nz);
    return -0.25 / (sx * sx + sy * sy + sz * sz);
  }
  if (gf == PMGB_POOR_MAN) {
    int ki = kx <= m.nx / 2 ? kx : kx - m.nx;
    int kj = ky <= m.ny / 2 ? ky : ky - m.ny;
    int kk = kz <= m.nz / 2 ? kz : kz - m.nz;
    double fx = 2 * PI * ki / m.nx, fy = 2 * PI * kj / m.ny, fz = 2 * PI * kk / m.nz;
    return -1.0 / (fx * fx + fy * fy + fz * fz);
  }
  auto edge = [](int k, int n) { return k == 0 || 2 * k == n; };
  if (edge(kx, m.nx) && edge(ky, m.ny) && edge(kz, m.nz)) return 0.0;
  const double k[3] = {2 * PI * kx / m.nx, 2 * PI * ky / m.ny, 2 * PI * kz / m.nz};
  const double denomSum = d_alias_sum(is, k);
  // D(k) = i d, d real
  double d[3];
  for (int i = 0; i < 3; ++i)
    d[i] = fds == 0 ? sin(k[i]) : (4.0 / 3.0) * sin(k[i]) + (1.0 - 4.0 / 3.0) * sin(2 * k[i]) / 2.0;
  const double dn2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  // R(k_n) = -i k_n S^2 / |k_n|^2; numerator = D . conj(sum U^2 R) = sum_i d_i * sum U^2 k_n,i S^2/|k_n|^2 * (-1)
  double acc[3] = {0.0, 0.0, 0.0};
  for (int n1 = -2; n1 <= 2; ++n1)
    for (int n2 = -2; n2 <= 2; ++n2)
      for (int n3 = -2; n3 <= 2; ++n3) {
        const double kn[3] = {k[0] + 2 * PI * n1, k[1] + 2 * PI * n2, k[2] + 2 * PI * n3};
        const double u = d_assign_fourier(is, kn);
        const double kl2 = kn[0] * kn[0] + kn[1] * kn[1] + kn[2] * kn[2];
        const double s = d_shape(cs, sqrt(kl2), a);
        const double f = u * u * s * s / kl2;
        acc[0] += f * kn[0];
        acc[1] += f * kn[1];
        acc[2] += f * kn[2];
      }
  // (i d) . conj(-i acc) = (i d)(i acc) = -d . acc
  const double num = -(d[0] * acc[0] + d[1] * acc[1] + d[2] * acc[2]);
  return num / (dn2 * denomSum * denomSum);
}

__global__ void green_kernel(float* __restrict__ ghat, MeshDims m, int gf, int is, int fds,
                             int cs, double a) {
  const long long total = (long long)m.nxp * m.ny * m.nz;
  const double invL = 1.0 / (double)m.L;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % m.nxp);
    const long long r = idx / m.nxp;
    const int ky = (int)(r % m.ny), kz = (int)(r / m.ny);
    if (kx >= m.nxh) {
      ghat[idx] = 0.f;
      continue;
    }
    const double g1 = d_green(gf, is, fds, cs, a, kx, ky, kz, m);
    const double g2 = d_green(gf, is, fds, cs, a, (m.nx - kx) % m.nx, (m.ny - ky) % m.ny,
                              (m.nz - kz) % m.nz, m);
    ghat[idx] = (float)(0.5 * (g1 + g2) * invL);
  }
}

int launch_green(float* ghat, MeshDims m, int gf, int is, int fds, double a, cudaStream_t st) {
  const int cs = gf == PMGB_S1_OPTIMAL ? 0 : 1;
  green_kernel<<<152 * 8, 256, 0, st>>>(ghat, m, gf, is, fds, cs, a);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  return PMGB_OK;
}

}  // namespace pmgb
