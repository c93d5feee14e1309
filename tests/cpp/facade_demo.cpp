// facade_demo.cpp - the reference's P3M accuracy-demo call sequence written against the C++
// facade (include/pmgb/pmgb.hpp): construct PMMethodGPU + P3MMethod with the reference's
// argument lists, evaluate one force, run a few steps, print the first particle.  Built and
// linked by tests/test_facade.py (CPU) and run by its GPU test.
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "pmgb/pmgb.hpp"

int main() {
  using namespace pmgb;
  const int n = 2000;
  std::mt19937 rng(3);
  std::normal_distribution<float> g(15.0f, 3.0f);
  std::vector<Vec3> state(2 * n);
  std::vector<float> masses(n, 1.0f / n);
  for (int i = 0; i < n; ++i) {
    auto c = [&] { return std::fmin(26.0f, std::fmax(4.0f, g(rng))); };
    state[i] = {c(), c(), c()};
    state[n + i] = {0, 0, 0};
  }
  const auto box = std::make_tuple(30.0f, 30.0f, 30.0f);
  const float H = 30.0f / 16, a = 3 * H;
  PMMethodGPU pm(state, masses, box, ExternalField::none(), H, 0.05f, 1.0f,
                 InterpolationScheme::TSC, FiniteDiffScheme::TWO_POINT,
                 GreensFunction::S2_OPTIMAL, a, std::make_tuple(32, 32, 32));
  P3MMethod p3m(pm, box, a, a, H, 0.0f, CloudShape::S2);
  p3m.force();
  const auto& p = pm.getParticles()[0];
  std::printf("acc0 %.9e %.9e %.9e\n", p.acceleration.x, p.acceleration.y, p.acceleration.z);
  p3m.run(3);
  const auto& q = pm.getParticles()[0];
  std::printf("pos0 %.9e %.9e %.9e\n", q.position.x, q.position.y, q.position.z);
  // the reference's stepper, FFT plug-in and grid surfaces
  {
    Grid grid = pm.getGrid();
    auto [gx, gy, gz] = grid.getGridPoints();
    double rho = 0;
    for (int i = 0; i < grid.getLength(); ++i) {
      auto [x, y, z] = grid.indexTripleFromFlat(i);
      rho += grid.getDensity(x, y, z);
    }
    Vec3 f = grid.getField(16, 16, 16);
    std::printf("grid %d %d %d %.6e %.6e\n", gx, gy, gz, rho, f.x);
    std::vector<Particle> ps = pm.getParticles();
    LeapfrogStepper stepper(pm);
    stepper.doStep(ps, 1.0f);
    setIntegerStepVelocities(ps);
    std::printf("step %.9e %.9e\n", ps[0].position.x, ps[0].integerStepVelocity.x);
    std::printf("extforce %.3e\n", pm.totalExternalForceOrigUnits().x);
    std::printf("extpot %.3e\n", pm.getExternalPotential()(Vec3{1, 2, 3}));
    CudaFFTAdapter fft({6, 10, 15});
    std::vector<std::complex<float>> a(900), b, c;
    for (int i = 0; i < 900; ++i) a[i] = {std::sin(0.1f * i), std::cos(0.3f * i)};
    fft.fft(a, b);
    fft.ifft(b, c);
    double err = 0;
    for (int i = 0; i < 900; ++i) err = std::fmax(err, std::abs(c[i] - a[i]));
    std::printf("fftroundtrip %.3e\n", err);
  }
  try {
    PMMethodGPU bad(state, masses, box, ExternalField::none(), H, 0.05f, 1.0f,
                    InterpolationScheme::TSC, FiniteDiffScheme::TWO_POINT,
                    GreensFunction::S1_OPTIMAL, 0.0f, std::make_tuple(32, 32, 32));
    std::printf("no exception\n");
    return 1;
  } catch (const std::invalid_argument&) {
    std::printf("invalid_argument ok\n");
  }
  return 0;
}
