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

#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <string>
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

class PMMethodGPU {
 public:
  PMMethodGPU(const std::vector<Vec3>& state, const std::vector<float>& masses,
              const std::tuple<float, float, float> effectiveBoxSize,
              const ExternalField externalField, const float H, const float DT, const float G,
              const InterpolationScheme is, const FiniteDiffScheme fds,
              const GreensFunction gFunc, const float particleDiameter,
              std::tuple<int, int, int> gridPoints)
      : N(int(masses.size())), H(H), DT(DT), G(G) {
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

  pmgb_pm* handle() { return h; }

 private:
  pmgb_pm* h = nullptr;
  int diagCapacity = 0;
  int N;
  float H, DT, G;
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

}  // namespace pmgb
