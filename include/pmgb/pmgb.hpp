// pmgb.hpp - C++ facade with the reference's PM / P3M class surface over the C ABI (pmgb.h).
//
// Drop-in for the reference's PMMethodGPU / PMMethod and P3MMethod in code such as its demos
// (reference source/demos.cpp): same class names, constructor argument order and meaning, same
// member functions (include/pmMethod.h:12-46, include_gpu/PMMethodGPU.h:12-55,
// include/p3mMethod.h:11-31), same enums (include/pmConfig.h:3-5, include/greensFunctions.h:7),
// and the same error behaviour (std::invalid_argument for bad enums / arguments, a printed
// message and an early return when a particle leaves the box), plus the reference's
// StateRecorder, PlummerSampler and DiskSamplerLinear.  One difference a device path needs: the
// external field is described by `ExternalField` (sphRadDecrField parameters, or none) instead
// of a host std::function.
#pragma once

#include <cmath>
#include <complex>
#include <cstdio>
#include <functional>
#include <iostream>
#include <stdexcept>
#include <string>
#include <array>
#include <tuple>
#include <vector>

#include "../pmgb.h"

namespace pmgb {

struct Vec3 {
  float x{}, y{}, z{};
};
static_assert(sizeof(Vec3) == 3 * sizeof(float), "Vec3 is three packed floats");

enum class InterpolationScheme { NGP = PMGB_NGP, CIC = PMGB_CIC, TSC = PMGB_TSC };
enum class FiniteDiffScheme { TWO_POINT = PMGB_TWO_POINT, FOUR_POINT = PMGB_FOUR_POINT };
enum class GreensFunction {
  DISCRETE_LAPLACIAN = PMGB_DISCRETE_LAPLACIAN,
  S1_OPTIMAL = PMGB_S1_OPTIMAL,
  S2_OPTIMAL = PMGB_S2_OPTIMAL,
  POOR_MAN = PMGB_POOR_MAN
};
enum class CloudShape { S1 = PMGB_S1, S2 = PMGB_S2 };

// One record of the run diagnostics (PMGB_DIAG_* layout of pmgb.h): what SimInfo computes
// (reference source/simInfo.cpp:50-127) after each drift of a run with collectDiagnostics.
struct DiagnosticsRecord {
  double potentialEnergy;
  double kineticEnergy;
  double momentum[3];
  double angularMomentum[3];
  double expectedMomentum[3];
  double externalPotentialEnergy;
};
static_assert(sizeof(DiagnosticsRecord) == PMGB_DIAG_WIDTH * sizeof(double), "record layout");

// PlummerSampler / DiskSamplerLinear with the reference's interface (include/plummerSampler.h,
// include/diskSamplerLinear.h): the state of n particles (n positions then n velocities),
// sampled on the device from the reference's own random stream; successive sample() calls
// continue the stream like the reference's engine.
class PlummerSampler {
 public:
  explicit PlummerSampler(unsigned int seed = 0) : seed(seed) {}
  std::vector<Vec3> sample(Vec3 center, float a, float rMax, float M, float G, int n) {
    std::vector<Vec3> state(2 * size_t(n));
    const float c[3] = {center.x, center.y, center.z};
    int rc = pmgb_sample_plummer(seed, draws, c, a, rMax, M, G, n, reinterpret_cast<float*>(state.data()));
    if (rc != PMGB_OK) throw std::invalid_argument(pmgb_last_error());
    draws += 6ull * (unsigned long long)n;
    return state;
  }

 private:
  unsigned int seed;
  unsigned long long draws = 0;
};

class DiskSamplerLinear {
 public:
  explicit DiskSamplerLinear(unsigned int seed = 0) : seed(seed) {}
  std::vector<Vec3> sample(Vec3 center, float rb, float mb, float rd, float md, float thickness,
                           float G, int n, float r0 = 0.0f) {
    std::vector<Vec3> state(2 * size_t(n));
    const float c[3] = {center.x, center.y, center.z};
    int rc = pmgb_sample_disk_linear(seed, draws, c, rb, mb, rd, md, thickness, G, n, r0,
                                     reinterpret_cast<float*>(state.data()));
    if (rc != PMGB_OK) throw std::invalid_argument(pmgb_last_error());
    draws += 3ull * (unsigned long long)n;
    return state;
  }

 private:
  unsigned int seed;
  unsigned long long draws = 0;
};

// StateRecorder with the reference's constructor (include/stateRecorder.h:10-21); the files
// and their formats are the reference's.  maxRecords (the reference's write-batch size) has no
// counterpart: frames are written from device buffers as they fill.
class StateRecorder {
 public:
  StateRecorder(int particlesCnt, int framesCnt, const std::string& outputDirPath,
                const char* positionsFile = "positions.dat", const char* energyFile = "energy.txt",
                const char* momentumFile = "momentum.txt",
                const char* expectedMomentumFile = "expected_momentum.txt",
                const char* angularMomentumFile = "angular_momentum.txt",
                const char* fieldFile = "field.dat", int /*maxRecords*/ = 500) {
    const char* names[6] = {positionsFile, energyFile, momentumFile, expectedMomentumFile,
                            angularMomentumFile, fieldFile};
    int rc = pmgb_recorder_create(particlesCnt, framesCnt, outputDirPath.c_str(), names, 1, &h);
    if (rc != PMGB_OK) throw std::invalid_argument(pmgb_last_error());
  }
  ~StateRecorder() { pmgb_recorder_destroy(h); }
  StateRecorder(const StateRecorder&) = delete;
  StateRecorder& operator=(const StateRecorder&) = delete;

  std::string flush() {
    char buf[4096];
    if (pmgb_recorder_flush(h, buf, sizeof buf) != PMGB_OK) throw std::runtime_error(pmgb_last_error());
    return buf;
  }
  pmgb_recorder* handle() { return h; }

 private:
  pmgb_recorder* h = nullptr;
};

// The reference's Particle (include/particle.h:5-15) without the per-neighbour P3M slots,
// which the device path does not need.
struct Particle {
  Vec3 position, velocity, acceleration;
  float mass{};
  Vec3 integerStepVelocity;  // set by setIntegerStepVelocities (include/particle.h:10)
};

// sphRadDecrField(pos, center, R, M, G) (reference source/externalFields.cpp:4-15), or none.
struct ExternalField {
  bool enabled = false;
  Vec3 center;
  float R = 0, M = 0, G = 0;
  static ExternalField none() { return {}; }
  static ExternalField sphRadDecr(Vec3 c, float R, float M, float G) {
    ExternalField f;
    f.enabled = true;
    f.center = c;
    f.R = R;
    f.M = M;
    f.G = G;
    return f;
  }
};

inline void check(int rc) {
  if (rc == PMGB_OK || rc == PMGB_EESCAPED) return;
  if (rc == PMGB_EINVAL) throw std::invalid_argument(pmgb_last_error());
  throw std::runtime_error(pmgb_last_error());
}

// The reference's FFT plug-in interface (include/FFTAdapter.h:6-15) and a device
// implementation of it: 3D complex-to-complex transforms of x-fastest meshes of any size; ifft
// includes the 1/N scale (source/FFTWAdapter.cpp:34-43).  dims = (nz, ny, nx), the order the
// reference passes to its adapters (source/demos.cpp:758).
template <typename T>
class FFTAdapter {
 public:
  virtual ~FFTAdapter() {}
  virtual std::vector<std::complex<T>>& fft(std::vector<std::complex<T>>& in,
                                            std::vector<std::complex<T>>& out) = 0;
  virtual std::vector<std::complex<T>>& ifft(std::vector<std::complex<T>>& in,
                                             std::vector<std::complex<T>>& out) = 0;
};

class CudaFFTAdapter : public FFTAdapter<float> {
 public:
  explicit CudaFFTAdapter(std::array<int, 3> dims) : dims(dims) {}
  std::vector<std::complex<float>>& fft(std::vector<std::complex<float>>& in,
                                        std::vector<std::complex<float>>& out) override {
    return run(in, out, 0);
  }
  std::vector<std::complex<float>>& ifft(std::vector<std::complex<float>>& in,
                                         std::vector<std::complex<float>>& out) override {
    return run(in, out, 1);
  }

 private:
  std::vector<std::complex<float>>& run(std::vector<std::complex<float>>& in,
                                        std::vector<std::complex<float>>& out, int inverse) {
    const size_t L = size_t(dims[0]) * dims[1] * dims[2];
    if (in.size() != L) throw std::invalid_argument("input size differs from the adapter's dims");
    out.resize(L);
    check(pmgb_fft3d(dims[2], dims[1], dims[0], reinterpret_cast<const float*>(in.data()),
                     reinterpret_cast<float*>(out.data()), inverse));
    return out;
  }
  static void check(int rc) {
    if (rc == PMGB_EINVAL) throw std::invalid_argument(pmgb_last_error());
    if (rc != PMGB_OK) throw std::runtime_error(pmgb_last_error());
  }
  std::array<int, 3> dims;
};

// Read-only copy of a PM handle's meshes with the reference Grid's getters (include/grid.h:10-
// 70): x-fastest layout, density and field reads unwrapped, potential reads wrapped.  The field
// is not kept on the device (the interpolation differences the potential on the fly); getField
// differences the potential the same way (source/pmMethod.cpp:352-382).
class Grid {
 public:
  Grid(int nx, int ny, int nz, FiniteDiffScheme fds)
      : gridPointsX(nx), gridPointsY(ny), gridPointsZ(nz), length(nx * ny * nz), fds(fds),
        density(size_t(length)), potential(size_t(length)),
        greenHalf(size_t(nx / 2 + 1) * ny * nz) {}
  std::tuple<int, int, int> indexTripleFromFlat(int flatIndex) const {
    return std::make_tuple(flatIndex % gridPointsX, (flatIndex / gridPointsX) % gridPointsY,
                           flatIndex / (gridPointsX * gridPointsY));
  }
  int getLength() const { return length; }
  std::tuple<int, int, int> getGridPoints() const {
    return std::make_tuple(gridPointsX, gridPointsY, gridPointsZ);
  }
  float getDensity(int x, int y, int z) const { return density[size_t(getIndx(x, y, z))]; }
  float getPotential(int i, int j, int k) const { return potential[size_t(getWrappedIndx(i, j, k))]; }
  // G(k) as the reference stores it (not divided by the mesh size), symmetrised over k and -k
  std::complex<float> getGreensFunction(int i, int j, int k) const {
    const int nxh = gridPointsX / 2 + 1;
    if (i >= nxh) {
      i = gridPointsX - i;
      j = (gridPointsY - j) % gridPointsY;
      k = (gridPointsZ - k) % gridPointsZ;
    }
    return {greenHalf[(size_t(k) * gridPointsY + j) * nxh + i] * float(length), 0.0f};
  }
  Vec3 getField(int x, int y, int z) const {
    auto phi = [&](int a, int b, int c) { return getPotential(a, b, c); };
    if (fds == FiniteDiffScheme::TWO_POINT)
      return {-0.5f * (phi(x + 1, y, z) - phi(x - 1, y, z)), -0.5f * (phi(x, y + 1, z) - phi(x, y - 1, z)),
              -0.5f * (phi(x, y, z + 1) - phi(x, y, z - 1))};
    const float c = -1.0f / 12;
    return {c * (-phi(x + 2, y, z) + 8 * phi(x + 1, y, z) - 8 * phi(x - 1, y, z) + phi(x - 2, y, z)),
            c * (-phi(x, y + 2, z) + 8 * phi(x, y + 1, z) - 8 * phi(x, y - 1, z) + phi(x, y - 2, z)),
            c * (-phi(x, y, z + 2) + 8 * phi(x, y, z + 1) - 8 * phi(x, y, z - 1) + phi(x, y, z - 2))};
  }

 private:
  friend class PMMethodGPU;
  static int mod(int a, int b) { return (a % b + b) % b; }
  int getWrappedIndx(int i, int j, int k) const {
    return mod(i, gridPointsX) + mod(j, gridPointsY) * gridPointsX +
           mod(k, gridPointsZ) * gridPointsX * gridPointsY;
  }
  int getIndx(int i, int j, int k) const { return i + j * gridPointsX + k * gridPointsX * gridPointsY; }
  int gridPointsX, gridPointsY, gridPointsZ, length;
  FiniteDiffScheme fds;
  std::vector<float> density, potential, greenHalf;
};

class PMMethodGPU {
 public:
  PMMethodGPU(const std::vector<Vec3>& state, const std::vector<float>& masses,
              const std::tuple<float, float, float> effectiveBoxSize,
              const ExternalField externalField, const float H, const float DT, const float G,
              const InterpolationScheme is, const FiniteDiffScheme fds,
              const GreensFunction gFunc, const float particleDiameter,
              std::tuple<int, int, int> gridPoints)
      : N(int(masses.size())), H(H), DT(DT), G(G), fds(fds), ext(externalField) {
    if (state.size() != 2 * masses.size())
      throw std::invalid_argument("state must hold N positions followed by N velocities");
    pmgb_pm_config c{};
    c.grid[0] = std::get<0>(gridPoints);
    c.grid[1] = std::get<1>(gridPoints);
    c.grid[2] = std::get<2>(gridPoints);
    c.box[0] = std::get<0>(effectiveBoxSize);
    c.box[1] = std::get<1>(effectiveBoxSize);
    c.box[2] = std::get<2>(effectiveBoxSize);
    c.H = H;
    c.DT = DT;
    c.G = G;
    c.interpolation = int(is);
    c.finite_diff = int(fds);
    c.greens = int(gFunc);
    c.particle_diameter = particleDiameter;
    if (externalField.enabled) {
      c.ext.kind = PMGB_EXT_SPH_RAD_DECR;
      c.ext.center[0] = externalField.center.x;
      c.ext.center[1] = externalField.center.y;
      c.ext.center[2] = externalField.center.z;
      c.ext.R = externalField.R;
      c.ext.M = externalField.M;
      c.ext.G = externalField.G;
    }
    check(pmgb_pm_create(&c, N, reinterpret_cast<const float*>(state.data()), masses.data(), &h));
    particles.resize(N);
    for (int i = 0; i < N; ++i) particles[i].mass = masses[i];
  }
  ~PMMethodGPU() { pmgb_pm_destroy(h); }
  PMMethodGPU(const PMMethodGPU&) = delete;
  PMMethodGPU& operator=(const PMMethodGPU&) = delete;

  // PMMethod::run without StateRecorder; returns "" (the reference returns the recorder's
  // output directory).  collectDiagnostics records the per-iteration diagnostics, read with
  // diagnostics().
  std::string run(const int simLength, bool collectDiagnostics = false) {
    if (collectDiagnostics) ensureDiagnostics(simLength + 1);
    int done = 0;
    int rc = pmgb_pm_run(h, simLength, &done);
    check(rc);
    if (rc == PMGB_EESCAPED) std::cout << "Particle moved outside the computational box.\n";
    copyParticlesDeviceToHost();
    return std::string();
  }

  // PMMethod::run(stateRecorder, simLength, collectDiagnostics, recordField)
  // (source/pmMethod.cpp:62-135): the reference's output files; returns the output directory.
  std::string run(StateRecorder& stateRecorder, const int simLength, bool collectDiagnostics = false,
                  bool recordField = false) {
    if (collectDiagnostics) ensureDiagnostics(simLength + 1);
    int done = 0;
    int rc = pmgb_pm_run_recorded(h, stateRecorder.handle(), simLength, collectDiagnostics ? 1 : 0,
                                  recordField ? 1 : 0, &done);
    check(rc);
    if (rc == PMGB_EESCAPED) std::cout << "Particle moved outside the computational box.\n";
    copyParticlesDeviceToHost();
    return stateRecorder.flush();
  }

  void pmMethodStep() { check(pmgb_pm_method_step(h)); }
  void initGreensFunction() { check(pmgb_pm_init_greens_function(h)); }

  // Particles as last copied from the device, code units (as the reference holds them
  // during a run).
  std::vector<Particle>& getParticles() { return particles; }

  void copyParticlesDeviceToHost() {
    std::vector<float> pos(3 * size_t(N)), vel(3 * size_t(N)), acc(3 * size_t(N));
    check(pmgb_pm_get_particles(h, pos.data(), vel.data(), acc.data(), PMGB_UNITS_CODE));
    for (int i = 0; i < N; ++i) {
      particles[i].position = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
      particles[i].velocity = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
      particles[i].acceleration = {acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]};
    }
  }
  void copyParticlesHostToDevice() {
    std::vector<float> pos(3 * size_t(N)), vel(3 * size_t(N));
    for (int i = 0; i < N; ++i) {
      pos[3 * i] = particles[i].position.x;
      pos[3 * i + 1] = particles[i].position.y;
      pos[3 * i + 2] = particles[i].position.z;
      vel[3 * i] = particles[i].velocity.x;
      vel[3 * i + 1] = particles[i].velocity.y;
      vel[3 * i + 2] = particles[i].velocity.z;
    }
    check(pmgb_pm_set_particles(h, pos.data(), vel.data(), PMGB_UNITS_CODE));
  }

  float getH() const { return H; }
  float getDT() const { return DT; }
  float getG() const { return G; }

  bool escapedComputationalBox() {
    int e = 0;
    check(pmgb_pm_escaped(h, &e));
    return e != 0;
  }

  std::vector<float> getGridDensity() {
    int n = 0, g[3];
    check(pmgb_pm_size(h, &n, g));
    std::vector<float> d(size_t(g[0]) * g[1] * g[2]);
    check(pmgb_pm_get_density(h, d.data()));
    return d;
  }
  std::vector<float> getGridPotential() {
    int n = 0, g[3];
    check(pmgb_pm_size(h, &n, g));
    std::vector<float> d(size_t(g[0]) * g[1] * g[2]);
    check(pmgb_pm_get_potential(h, d.data()));
    return d;
  }

  // Records of the last run with collectDiagnostics (or since setDiagnostics), in original
  // units and double precision.
  std::vector<DiagnosticsRecord> diagnostics() {
    std::vector<DiagnosticsRecord> r(static_cast<size_t>(diagCapacity));
    int taken = 0;
    check(pmgb_pm_get_diagnostics(h, reinterpret_cast<double*>(r.data()), diagCapacity, &taken));
    r.resize(size_t(taken < diagCapacity ? taken : diagCapacity));
    return r;
  }
  void setDiagnostics(int capacity) {
    check(pmgb_pm_set_diagnostics(h, capacity));
    diagCapacity = capacity;
  }
  void ensureDiagnostics(int capacity) {
    if (diagCapacity < capacity) setDiagnostics(capacity);
  }

  // PMMethod::getGrid (include/pmMethod.h:37): the meshes of the last force evaluation, copied
  // from the device into a read-only Grid with the reference's getters.
  Grid getGrid() {
    int n = 0, g[3];
    check(pmgb_pm_size(h, &n, g));
    Grid grid(g[0], g[1], g[2], fds);
    check(pmgb_pm_get_density(h, grid.density.data()));
    check(pmgb_pm_get_potential(h, grid.potential.data()));
    check(pmgb_pm_get_greens_function(h, grid.greenHalf.data()));
    return grid;
  }

  // PMMethod::getExternalPotential (include/pmMethod.h:38): the potential of the external field
  // at a position in original units (sphRadDecrFieldPotential, source/externalFields.cpp:17-28).
  std::function<float(Vec3)> getExternalPotential() const {
    const ExternalField f = ext;
    return [f](Vec3 pos) -> float {
      if (!f.enabled) return 0.0f;
      const float dx = pos.x - f.center.x, dy = pos.y - f.center.y, dz = pos.z - f.center.z;
      const float r = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (r > f.R) return -f.G * f.M / r;
      const float u = r / f.R;
      return f.G * f.M / f.R * (-2 + u * u * (2 - u));
    };
  }

  // PMMethod::totalExternalForceOrigUnits (source/pmMethod.cpp:158-162), on the device.
  Vec3 totalExternalForceOrigUnits() {
    Vec3 f;
    check(pmgb_pm_total_external_force(h, &f.x));
    return f;
  }

  pmgb_pm* handle() { return h; }

 private:
  pmgb_pm* h = nullptr;
  int diagCapacity = 0;
  int N;
  float H, DT, G;
  FiniteDiffScheme fds = FiniteDiffScheme::TWO_POINT;
  ExternalField ext;
  std::vector<Particle> particles;
};

// The reference's CPU class name maps to the same device implementation.
using PMMethod = PMMethodGPU;

class P3MMethod {
 public:
  P3MMethod(PMMethodGPU& pmMethod, std::tuple<float, float, float> compBoxSize,
            float cutoffRadius, float particleDiameter, float H, float softeningLength,
            CloudShape cloudShape, bool useSRForceTable = true, bool enableYSorting = true)
      : pm(pmMethod) {
    if (H != pmMethod.getH()) throw std::invalid_argument("H differs from the PM method's H");
    pmgb_p3m_config c{};
    c.comp_box[0] = std::get<0>(compBoxSize);
    c.comp_box[1] = std::get<1>(compBoxSize);
    c.comp_box[2] = std::get<2>(compBoxSize);
    c.cutoff = cutoffRadius;
    c.particle_diameter = particleDiameter;
    c.softening = softeningLength;
    c.cloud_shape = int(cloudShape);
    c.use_table = useSRForceTable ? 1 : 0;
    c.y_sorting = enableYSorting ? 1 : 0;
    check(pmgb_p3m_create(pm.handle(), &c, &h));
  }
  ~P3MMethod() { pmgb_p3m_destroy(h); }
  P3MMethod(const P3MMethod&) = delete;
  P3MMethod& operator=(const P3MMethod&) = delete;

  void run(const int simLength, bool collectDiagnostics = false) {
    if (collectDiagnostics) pm.ensureDiagnostics(simLength + 1);
    int done = 0;
    int rc = pmgb_p3m_run(h, simLength, &done);
    check(rc);
    if (rc == PMGB_EESCAPED) std::cout << "Particle moved outside the computational box.\n";
    pm.copyParticlesDeviceToHost();
  }

  // P3MMethod::run(stateRecorder, simLength, collectDiagnostics, recordField)
  // (source/p3mMethod.cpp:59-166).
  std::string run(StateRecorder& stateRecorder, const int simLength, bool collectDiagnostics = false,
                  bool recordField = false) {
    return pm.run(stateRecorder, simLength, collectDiagnostics, recordField);
  }

  // One force evaluation (pmMethodStep + short-range forces + correctAccelerations).
  void force() {
    check(pmgb_p3m_force(h));
    pm.copyParticlesDeviceToHost();
  }

  pmgb_p3m* handle() { return h; }

 private:
  PMMethodGPU& pm;
  pmgb_p3m* h = nullptr;
};

// The leapfrog free functions (include/leapfrog.h:6-12, source/leapfrog.cpp:5-24) on the
// reference's particle vectors, computed on the device in the reference's float arithmetic ...
namespace detail {
inline void leapfrog(int op, std::vector<Particle>& particles, float dt) {
  const size_t n = particles.size();
  std::vector<float> pos(3 * n), vel(3 * n), acc(3 * n), u(3 * n);
  for (size_t i = 0; i < n; ++i) {
    const Particle& p = particles[i];
    float* q[3] = {&pos[3 * i], &vel[3 * i], &acc[3 * i]};
    const Vec3* v[3] = {&p.position, &p.velocity, &p.acceleration};
    for (int k = 0; k < 3; ++k) {
      q[k][0] = v[k]->x;
      q[k][1] = v[k]->y;
      q[k][2] = v[k]->z;
    }
  }
  check(pmgb_leapfrog(op, int(n), pos.data(), vel.data(), acc.data(), u.data(), dt));
  for (size_t i = 0; i < n; ++i) {
    Particle& p = particles[i];
    if (op == PMGB_LEAPFROG_DRIFT) p.position = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    else if (op == PMGB_LEAPFROG_INTEGER_STEP) p.integerStepVelocity = {u[3 * i], u[3 * i + 1], u[3 * i + 2]};
    else p.velocity = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
  }
}
}  // namespace detail

inline void setHalfStepVelocities(std::vector<Particle>& particles, float dt = 1.0f) {
  detail::leapfrog(PMGB_LEAPFROG_HALF_KICK, particles, dt);
}
inline void setIntegerStepVelocities(std::vector<Particle>& particles, float dt = 1.0f) {
  detail::leapfrog(PMGB_LEAPFROG_INTEGER_STEP, particles, dt);
}
inline void updateVelocities(std::vector<Particle>& particles, float dt = 1.0f) {
  detail::leapfrog(PMGB_LEAPFROG_KICK, particles, dt);
}
inline void updatePositions(std::vector<Particle>& particles, float dt = 1.0f) {
  detail::leapfrog(PMGB_LEAPFROG_DRIFT, particles, dt);
}

// ... and on a PM handle's own particles on the device (code units, the accelerations of its
// last force evaluation); getParticles() reflects them after copyParticlesDeviceToHost().
inline void setHalfStepVelocities(PMMethodGPU& pm, float dt = 1.0f) {
  check(pmgb_pm_leapfrog(pm.handle(), PMGB_LEAPFROG_HALF_KICK, dt));
}
inline void setIntegerStepVelocities(PMMethodGPU& pm, float dt = 1.0f) {
  check(pmgb_pm_leapfrog(pm.handle(), PMGB_LEAPFROG_INTEGER_STEP, dt));
}
inline void updateVelocities(PMMethodGPU& pm, float dt = 1.0f) {
  check(pmgb_pm_leapfrog(pm.handle(), PMGB_LEAPFROG_KICK, dt));
}
inline void updatePositions(PMMethodGPU& pm, float dt = 1.0f) {
  check(pmgb_pm_leapfrog(pm.handle(), PMGB_LEAPFROG_DRIFT, dt));
}

// Accelerations of every particle by the pairwise gravitational sum of ppMethod
// (source/ppMethod.cpp:23-36), evaluated in FP64 on the device and rounded to float (the
// reference sums in float); positions and result in the caller's units.
inline std::vector<Vec3> ppAccelerations(const std::vector<Vec3>& positions, const std::vector<float>& masses,
                                         float G, float softeningLength) {
  const int n = int(masses.size());
  if (positions.size() < masses.size()) throw std::invalid_argument("fewer positions than masses");
  std::vector<int> idx(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) idx[size_t(i)] = i;
  std::vector<double> acc(3 * static_cast<size_t>(n));
  check(pmgb_direct_sum_fp64(n, &positions[0].x, masses.data(), G, softeningLength, n, idx.data(), 0.0,
                             acc.data()));
  std::vector<Vec3> out(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i)
    out[size_t(i)] = {float(acc[3 * size_t(i)]), float(acc[3 * size_t(i) + 1]), float(acc[3 * size_t(i) + 2])};
  return out;
}

// AbstractStepper (include/abstractStepper.h:4-9) and a leapfrog stepper over a PM method: one
// kick-drift-kick step of the particles in code units, the force from the PM (or P3M, when a
// P3MMethod is attached to it) on the device.
template <typename T>
class AbstractStepper {
 public:
  virtual ~AbstractStepper() {}
  virtual void doStep(std::vector<T>& x, float dt) = 0;
};

class LeapfrogStepper : public AbstractStepper<Particle> {
 public:
  explicit LeapfrogStepper(PMMethodGPU& pm) : pm(pm) {}
  void doStep(std::vector<Particle>& x, float dt) override {
    std::vector<Particle>& own = pm.getParticles();
    if (x.size() != own.size()) throw std::invalid_argument("particle count differs from the PM method's");
    own = x;
    pm.copyParticlesHostToDevice();
    pm.pmMethodStep();        // accelerations at x
    setHalfStepVelocities(pm, dt);
    updatePositions(pm, dt);
    pm.pmMethodStep();        // accelerations at the new positions
    setHalfStepVelocities(pm, dt);
    pm.copyParticlesDeviceToHost();
    x = own;
  }

 private:
  PMMethodGPU& pm;
};

}  // namespace pmgb
