// pmgb_demos.cpp - the reference's PM / P3M simulation scenarios (source/demos.cpp, selected by
// the command line of source/main.cpp:23-62) on the GB300 path, written against the drop-in
// facade (include/pmgb/pmgb.hpp) exactly as the reference's demos are written against its
// classes: same samplers and seeds, same settings, same StateRecorder output files.
//
//   pmgb_demos <option> [output dir]
//
// Options: galaxy-sim-pm, galaxy-sim-p3m, galaxy-collision-sim-pm, galaxy-collision-sim-p3m,
// cluster-sim-pm, cluster-sim-p3m, galaxy-sim-pm-timing, galaxy-sim-p3m-timing, and the PM field
// sweeps anisotropy, finite-diff-err, assignment-schemes, poor-man-vs-laplacian, pm-optimal,
// pm-optimal-var-diameter, pm-optimal-assignments, and the accuracy scenarios pm-accuracy-soft,
// pm-accuracy-no-soft, p3m-accuracy-assignments and p3m-accuracy-shapes.  Their direct-sum
// reference forces (the reference's ppMethodLeapfrog with simLength 0: the accelerations of the
// initial state and the positions after one drift) are computed in FP64 on the device and
// rounded to float (the reference sums in float).  The Barnes-Hut scenarios are out of scope.
// Differences from the reference's scenarios, all deliberate: the external field is passed as a
// description (the GPU path has no host callbacks); galaxy-sim-p3m uses the reference's CPU
// settings (S1-optimal influence function, a = 3H), which its CUDA build replaced by the
// discrete Laplacian; cluster-sim-p3m runs P3M (the reference builds the P3MMethod and then
// runs the plain PM method).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "pmgb/pmgb.hpp"

using namespace pmgb;

namespace {

Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }

// galaxy-sim-pm (galaxySimulationPM, source/demos.cpp:729-777): linear disk + external bulge
void galaxySimulationPM(const std::string& out, int n = 50000, int simLength = 200, bool timing = false) {
  const Vec3 center = v3(30, 30, 15);
  const float rb = 3.0f, mb = 60.0f, rd = 15.0f, md = 15.0f, thickness = 0.3f, G = 4.5e-3f;
  DiskSamplerLinear diskSampler(42);
  std::vector<Vec3> state = diskSampler.sample(center, rb, mb, rd, md, thickness, G, n);
  std::vector<float> masses(n, md / n);
  const auto gridPoints = std::make_tuple(128, 128, 64);
  const auto box = std::make_tuple(60.0f, 60.0f, 30.0f);
  const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2), DT = 1;
  PMMethodGPU pm(state, masses, box, ExternalField::sphRadDecr(center, rb, mb, G), H, DT, G,
                 InterpolationScheme::TSC, FiniteDiffScheme::TWO_POINT,
                 GreensFunction::DISCRETE_LAPLACIAN, 0, gridPoints);
  StateRecorder stateRecorder(n, simLength + 1, out);
  const auto t0 = std::chrono::high_resolution_clock::now();
  pm.run(stateRecorder, simLength, true /*diagnostics*/);
  const std::chrono::duration<double> dt = std::chrono::high_resolution_clock::now() - t0;
  if (timing) std::cout << n << ' ' << dt.count() << std::endl;
}

// galaxy-sim-p3m (galaxySimulationP3M, source/demos.cpp:897-951)
void galaxySimulationP3M(const std::string& out, int n = 50000, int simLength = 200, bool timing = false) {
  const Vec3 center = v3(30, 30, 15);
  const float rb = 3.0f, mb = 60.0f, rd = 15.0f, md = 15.0f, thickness = 0.3f, G = 4.5e-3f;
  DiskSamplerLinear diskSampler(42);
  std::vector<Vec3> state = diskSampler.sample(center, rb, mb, rd, md, thickness, G, n);
  std::vector<float> masses(n, md / n);
  const auto gridPoints = std::make_tuple(128, 128, 64);
  const auto box = std::make_tuple(60.0f, 60.0f, 30.0f);
  const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2), DT = 1;
  const float a = 3 * H;
  PMMethodGPU pm(state, masses, box, ExternalField::sphRadDecr(center, rb, mb, G), H, DT, G,
                 InterpolationScheme::TSC, FiniteDiffScheme::TWO_POINT, GreensFunction::S1_OPTIMAL, a,
                 gridPoints);
  const float re = 0.7f * a, softeningLength = 1.5f;
  P3MMethod p3m(pm, box, re, a, H, softeningLength, CloudShape::S1);
  StateRecorder stateRecorder(n, simLength + 1, out);
  const auto t0 = std::chrono::high_resolution_clock::now();
  p3m.run(stateRecorder, simLength, true /*diagnostics*/);
  const std::chrono::duration<double> dt = std::chrono::high_resolution_clock::now() - t0;
  if (timing) std::cout << n << ' ' << dt.count() << std::endl;
}

// Two disks, the second scaled down by 1.5, each with a central point mass
// (galaxyCollisionPM / galaxyCollisionP3M, source/demos.cpp:838-895, 1018-1080).
void collisionState(std::vector<Vec3>& state, std::vector<float>& masses, int n) {
  const Vec3 c1 = v3(40, 30, 15), c2 = v3(80, 30, 15);
  const float rb = 3.0f, mb = 60.0f, rd = 15.0f, md = 15.0f, thickness = 0.3f, G = 4.5e-3f;
  DiskSamplerLinear diskSampler(42);
  std::vector<Vec3> s1 = diskSampler.sample(c1, rb, mb, rd, md, thickness, G, n, rb);
  std::vector<float> m1(n, md / n);
  s1[0] = c1;
  s1[n] = v3(0, 0, 0);
  m1[0] = 60.0f;
  std::vector<Vec3> s2 = diskSampler.sample(c2, rb / 1.5f, mb / 1.5f, rd / 1.5f, md / 1.5f, thickness,
                                            G, n, rb / 1.5f);
  std::vector<float> m2(n, md / n);
  s2[0] = c2;
  s2[n] = v3(0, 0, 0);
  m2[0] = 60.0f / 1.5f;
  state.assign(4 * size_t(n), Vec3{});
  masses.assign(2 * size_t(n), 0.f);
  for (int i = 0; i < n; ++i) {
    state[i] = s1[i];
    state[i + 2 * n] = s1[i + n];
    masses[i] = m1[i];
    state[i + n] = s2[i];
    state[i + 3 * n] = s2[i + n];
    masses[i + n] = m2[i];
  }
}

void galaxyCollision(const std::string& out, bool p3mRun) {
  const int n = 30000, simLength = 400;
  const float G = 4.5e-3f;
  std::vector<Vec3> state;
  std::vector<float> masses;
  collisionState(state, masses, n);
  const auto gridPoints = std::make_tuple(128, 128, 64);
  const auto box = std::make_tuple(120.0f, 120.0f, 60.0f);
  const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2), DT = 1;
  const float a = 3 * H;
  PMMethodGPU pm(state, masses, box, ExternalField::none(), H, DT, G, InterpolationScheme::TSC,
                 FiniteDiffScheme::TWO_POINT,
                 p3mRun ? GreensFunction::S1_OPTIMAL : GreensFunction::DISCRETE_LAPLACIAN,
                 p3mRun ? a : 0.0f, gridPoints);
  StateRecorder stateRecorder(2 * n, simLength + 1, out);
  if (p3mRun) {
    P3MMethod p3m(pm, box, 0.7f * a, a, H, 1.5f, CloudShape::S1);
    p3m.run(stateRecorder, simLength, true /*diagnostics*/);
  } else {
    pm.run(stateRecorder, simLength, true /*diagnostics*/);
  }
}

// cluster-sim-pm / cluster-sim-p3m (plummerPM / plummerP3M, source/demos.cpp:1369-1452)
void plummer(const std::string& out, bool p3mRun) {
  const Vec3 center = v3(30, 30, 30);
  const float a = 2, rMax = 15, M = 1.0f, G = 4.5e-3f;
  const int n = 10000, simLength = 200;
  PlummerSampler sampler(42);
  std::vector<Vec3> state = sampler.sample(center, a, rMax, M, G, n);
  std::vector<float> masses(n, M / n);
  const auto gridPoints = std::make_tuple(128, 128, 128);
  const auto box = std::make_tuple(60.0f, 60.0f, 60.0f);
  const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2), DT = 1;
  const float particleDiam = 3 * H;
  PMMethodGPU pm(state, masses, box, ExternalField::none(), H, DT, G, InterpolationScheme::TSC,
                 FiniteDiffScheme::TWO_POINT,
                 p3mRun ? GreensFunction::S1_OPTIMAL : GreensFunction::DISCRETE_LAPLACIAN,
                 p3mRun ? particleDiam : 0.0f, gridPoints);
  StateRecorder stateRecorder(n, simLength + 1, out);
  if (p3mRun) {
    P3MMethod p3m(pm, box, 0.7f * a, particleDiam, H, 0.5f, CloudShape::S1);
    p3m.run(stateRecorder, simLength, true /*diagnostics*/);
  } else {
    pm.run(stateRecorder, simLength, true /*diagnostics*/);
  }
}

// The PM field sweeps (anisotropy, finiteDiffRelError, assignmentSchemes, poorLaplace,
// pmOptimal, pmOptimalVaryingDiameter, pmOptimalAssignments; source/demos.cpp:109-591): one
// particle of mass 1 at `center` and 399 massless tracers every 0.075 along `dir`, 64 x 64 x 32
// mesh over a 60 x 60 x 30 box (H = 60 / 32), G = 4.5e-3, DT = 1, one iteration with the
// positions and the field (the acceleration each tracer feels) recorded.
std::vector<Vec3> linearSpacing(int n, float dx, Vec3 center, Vec3 dir) {
  std::vector<Vec3> state(2 * size_t(n), Vec3{});
  for (int i = 0; i < n; ++i)
    state[i] = v3(center.x + i * dx * dir.x, center.y + i * dx * dir.y, center.z + i * dx * dir.z);
  return state;
}

void fieldSweep(const std::string& out, const char* positionsFile, const char* fieldFile, Vec3 center,
                Vec3 dir, InterpolationScheme is, FiniteDiffScheme fds, GreensFunction gf,
                float particleDiameter) {
  const int n = 400, simLength = 1;
  const float G = 4.5e-3f;
  std::vector<float> masses(n, 0.0f);
  masses[0] = 1.0f;
  const auto gridPoints = std::make_tuple(64, 64, 32);
  const auto box = std::make_tuple(60.0f, 60.0f, 30.0f);
  const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2), DT = 1;
  StateRecorder stateRecorder(n, simLength + 1, out, positionsFile, "", "", "", "", fieldFile);
  PMMethodGPU pm(linearSpacing(n, 0.075f, center, dir), masses, box, ExternalField::none(), H, DT, G, is,
                 fds, gf, particleDiameter, gridPoints);
  pm.run(stateRecorder, simLength, false /*diagnostics*/, true /*field*/);
}

constexpr float kSweepH = 60.0f / 32;  // H of the field sweeps

void anisotropy(const std::string& out) {
  const auto T = InterpolationScheme::TSC;
  const auto F2 = FiniteDiffScheme::TWO_POINT;
  const auto L = GreensFunction::DISCRETE_LAPLACIAN;
  fieldSweep(out, "positions.dat", "field.dat", v3(30, 30, 15), v3(1, 0, 0), T, F2, L, 0);
  fieldSweep(out, "positions_offset.dat", "field_offset.dat", v3(30 - kSweepH / 2, 30, 15), v3(1, 0, 0), T,
             F2, L, 0);
  const float s = 1 / std::sqrt(2.0f);
  fieldSweep(out, "positions_diag.dat", "field_diag.dat", v3(30, 30, 15), v3(s, s, 0), T, F2, L, 0);
}

void finiteDiffRelError(const std::string& out) {
  const auto T = InterpolationScheme::TSC;
  const auto L = GreensFunction::DISCRETE_LAPLACIAN;
  fieldSweep(out, "positions-2.dat", "field-2.dat", v3(30, 30, 15), v3(1, 0, 0), T,
             FiniteDiffScheme::TWO_POINT, L, 0);
  fieldSweep(out, "positions-4.dat", "field-4.dat", v3(30, 30, 15), v3(1, 0, 0), T,
             FiniteDiffScheme::FOUR_POINT, L, 0);
}

void assignmentSchemes(const std::string& out) {
  const auto F4 = FiniteDiffScheme::FOUR_POINT;
  const auto L = GreensFunction::DISCRETE_LAPLACIAN;
  fieldSweep(out, "positions-tsc.dat", "field-tsc.dat", v3(30, 30, 15), v3(1, 0, 0),
             InterpolationScheme::TSC, F4, L, 0);
  fieldSweep(out, "positions-cic.dat", "field-cic.dat", v3(30, 30, 15), v3(1, 0, 0),
             InterpolationScheme::CIC, F4, L, 0);
  fieldSweep(out, "positions-ngp.dat", "field-ngp.dat", v3(30, 30, 15), v3(1, 0, 0),
             InterpolationScheme::NGP, F4, L, 0);
}

void poorLaplace(const std::string& out) {
  const auto T = InterpolationScheme::TSC;
  const auto F4 = FiniteDiffScheme::FOUR_POINT;
  fieldSweep(out, "positions-poor-man.dat", "field-poor-man.dat", v3(30, 30, 15), v3(1, 0, 0), T, F4,
             GreensFunction::POOR_MAN, 0);
  fieldSweep(out, "positions-discrete-lap.dat", "field-discrete-lap.dat", v3(30, 30, 15), v3(1, 0, 0), T,
             F4, GreensFunction::DISCRETE_LAPLACIAN, 0);
}

void pmOptimal(const std::string& out) {
  const auto T = InterpolationScheme::TSC;
  const auto F4 = FiniteDiffScheme::FOUR_POINT;
  fieldSweep(out, "positions-s1.dat", "field-s1.dat", v3(30, 30, 15), v3(1, 0, 0), T, F4,
             GreensFunction::S1_OPTIMAL, 4 * kSweepH);
  fieldSweep(out, "positions-s2.dat", "field-s2.dat", v3(30, 30, 15), v3(1, 0, 0), T, F4,
             GreensFunction::S2_OPTIMAL, 4 * kSweepH);
}

void pmOptimalVaryingDiameter(const std::string& out) {
  const auto T = InterpolationScheme::TSC;
  const auto F4 = FiniteDiffScheme::FOUR_POINT;
  for (const auto gf : {GreensFunction::S1_OPTIMAL, GreensFunction::S2_OPTIMAL}) {
    const std::string tag = gf == GreensFunction::S1_OPTIMAL ? "s1" : "s2";
    for (int i = 5; i <= 30; ++i) {
      const std::string positions = "positions-" + tag + ".dat";
      const std::string field = "field-" + tag + "-" + std::to_string(i) + ".dat";
      fieldSweep(out, positions.c_str(), field.c_str(), v3(30, 30, 15), v3(1, 0, 0), T, F4, gf,
                 0.2f * i * kSweepH);
    }
  }
}

void pmOptimalAssignments(const std::string& out) {
  const std::pair<InterpolationScheme, const char*> schemes[] = {
      {InterpolationScheme::NGP, "NGP"}, {InterpolationScheme::CIC, "CIC"}, {InterpolationScheme::TSC, "TSC"}};
  for (const auto& [is, name] : schemes) {
    const std::string field = std::string("field-s1-") + name + ".dat";
    fieldSweep(out, "positions-s1.dat", field.c_str(), v3(30, 30, 15), v3(1, 0, 0), is,
               FiniteDiffScheme::FOUR_POINT, GreensFunction::S1_OPTIMAL, 4 * kSweepH);
  }
}

// One-frame StateRecorder file (int32 particle count, int32 frame count, float triplets;
// source/stateRecorder.cpp:5-44, 109-119).
void writeFrame(const std::string& out, const std::string& name, const std::vector<Vec3>& v) {
  const std::string path = out + "/" + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  const int hdr[2] = {int(v.size()), 1};
  std::fwrite(hdr, sizeof(int), 2, f);
  std::fwrite(v.data(), sizeof(Vec3), v.size(), f);
  std::fclose(f);
}

// ppMethodLeapfrog(state, masses, 0, DT = 1, G, eps, recorder, recordField = true)
// (source/ppMethod.cpp:88-125): the field file holds the initial accelerations, the positions
// file the positions after the first drift (half kick, then drift, dt = 1).
void ppReference(const std::string& out, const std::vector<Vec3>& state, const std::vector<float>& masses,
                 float G, float eps, const std::string& positionsFile, const std::string& forceFile) {
  const size_t n = masses.size();
  std::vector<Vec3> pos(state.begin(), state.begin() + long(n));
  std::vector<Vec3> acc = ppAccelerations(pos, masses, G, eps);
  std::vector<Particle> ps(n);
  for (size_t i = 0; i < n; ++i) {
    ps[i].position = pos[i];
    ps[i].velocity = state[n + i];
    ps[i].acceleration = acc[i];
    ps[i].mass = masses[i];
  }
  setHalfStepVelocities(ps);
  updatePositions(ps);
  for (size_t i = 0; i < n; ++i) pos[i] = ps[i].position;
  writeFrame(out, forceFile, acc);
  writeFrame(out, positionsFile, pos);
}

// The disk of the accuracy scenarios (source/demos.cpp:361-373, 593-605)
void accuracyDisk(std::vector<Vec3>& state, std::vector<float>& masses, float& G) {
  const int n = 10000;
  G = 4.5e-3f;
  DiskSamplerLinear diskSampler(42);
  state = diskSampler.sample(v3(30, 30, 15), 3.0f, 60.0f, 15.0f, 15.0f, 0.3f, G, n);
  masses.assign(size_t(n), 15.0f / n);
}

const char* name(InterpolationScheme is) {
  return is == InterpolationScheme::NGP ? "NGP" : is == InterpolationScheme::CIC ? "CIC" : "TSC";
}
// the reference's toString names in its file names (source/demos.cpp:63-96)
const char* name(FiniteDiffScheme f) { return f == FiniteDiffScheme::TWO_POINT ? "2-point" : "4-point"; }
const char* name(GreensFunction g) {
  return g == GreensFunction::S1_OPTIMAL ? "S1" : g == GreensFunction::S2_OPTIMAL ? "S2" : "Unknown";
}

// pm-accuracy-soft / pm-accuracy-no-soft (pmAccuracy, source/demos.cpp:361-428): PM forces of
// the disk on (2 Ng, 2 Ng, Ng) meshes, Ng = 30, 34, ..., 70, every interpolation and difference
// scheme; direct-sum forces with softening box / Ng (soft) or one without (no-soft)
void pmAccuracy(const std::string& out, bool ppSoftening) {
  std::vector<Vec3> state;
  std::vector<float> masses;
  float G;
  accuracyDisk(state, masses, G);
  const int n = int(masses.size());
  const auto box = std::make_tuple(60.0f, 60.0f, 30.0f);
  const int NgStart = 30, NgEnd = 70, NgStep = 4;
  if (ppSoftening) {
    for (int Ng = NgStart; Ng <= NgEnd; Ng += NgStep)
      ppReference(out, state, masses, G, std::get<0>(box) / Ng, "positions-pp.dat",
                  "force-pp-" + std::to_string(Ng) + ".dat");
  } else {
    ppReference(out, state, masses, G, 0.0f, "positions-pp.dat", "force-pp-0.dat");
  }
  for (auto is : {InterpolationScheme::NGP, InterpolationScheme::CIC, InterpolationScheme::TSC})
    for (auto fds : {FiniteDiffScheme::TWO_POINT, FiniteDiffScheme::FOUR_POINT})
      for (int Ng = NgStart; Ng <= NgEnd; Ng += NgStep) {
        const auto gridPoints = std::make_tuple(2 * Ng, 2 * Ng, Ng);
        const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2);
        const std::string forceFile =
            std::string("force-pm-") + name(is) + "-" + name(fds) + "-" + std::to_string(Ng) + ".dat";
        std::cout << forceFile << '\n';
        StateRecorder stateRecorder(n, 1, out, "positions-pm.dat", "", "", "", "", forceFile.c_str());
        PMMethodGPU pm(state, masses, box, ExternalField::none(), H, 1.0f, G, is, fds,
                       GreensFunction::DISCRETE_LAPLACIAN, 0.0f, gridPoints);
        pm.run(stateRecorder, 0, false, true);
      }
}

// p3m-accuracy-assignments / p3m-accuracy-shapes (source/demos.cpp:593-727): P3M forces of the
// disk on the 128 x 128 x 64 mesh for particle diameters a = 0.2 aMul H, aMul = 5 .. 25,
// cutoff re = a, table-free short-range force, unsorted chaining mesh
void p3mAccuracy(const std::string& out, bool shapes) {
  std::vector<Vec3> state;
  std::vector<float> masses;
  float G;
  accuracyDisk(state, masses, G);
  const int n = int(masses.size());
  const auto box = std::make_tuple(60.0f, 60.0f, 30.0f);
  ppReference(out, state, masses, G, 0.0f, "positions-pp.dat", "force-pp.dat");
  const auto gridPoints = std::make_tuple(128, 128, 64);
  const float H = std::get<0>(box) / (std::get<0>(gridPoints) / 2);
  auto one = [&](InterpolationScheme is, FiniteDiffScheme fds, GreensFunction gf, int aMul,
                 const std::string& forceFile) {
    const float a = 0.2f * aMul * H;
    std::cout << forceFile << '\n';
    StateRecorder stateRecorder(n, 1, out, "positions-pm.dat", "", "", "", "", forceFile.c_str());
    PMMethodGPU pm(state, masses, box, ExternalField::none(), H, 1.0f, G, is, fds, gf, a, gridPoints);
    P3MMethod p3m(pm, box, a, a, H, 0.0f,
                  gf == GreensFunction::S2_OPTIMAL ? CloudShape::S2 : CloudShape::S1, false, false);
    p3m.run(stateRecorder, 0, false, true);
  };
  if (!shapes) {
    for (auto is : {InterpolationScheme::NGP, InterpolationScheme::CIC, InterpolationScheme::TSC})
      for (auto fds : {FiniteDiffScheme::TWO_POINT, FiniteDiffScheme::FOUR_POINT})
        for (int aMul = 5; aMul <= 25; ++aMul)
          one(is, fds, GreensFunction::S1_OPTIMAL, aMul,
              std::string("force-p3m-") + name(is) + "-" + name(fds) + "-" + std::to_string(aMul) + ".dat");
  } else {
    for (auto gf : {GreensFunction::S1_OPTIMAL, GreensFunction::S2_OPTIMAL})
      for (auto fds : {FiniteDiffScheme::TWO_POINT, FiniteDiffScheme::FOUR_POINT})
        for (int aMul = 5; aMul <= 25; ++aMul)
          one(InterpolationScheme::TSC, fds, gf, aMul,
              std::string("force-p3m-TSC-") + name(fds) + "-" + name(gf) + "-" + std::to_string(aMul) + ".dat");
  }
}

}  // namespace

int main(int argc, char* argv[]) {
  try {
    if (argc < 2) throw std::runtime_error("Unknown option");
    std::cout << "running " << argv[1] << " with arguments: ";
    for (int i = 2; i < argc; ++i) std::cout << argv[i] << (i < argc - 1 ? ", " : "");
    std::cout << '\n';
    const std::string option(argv[1]);
    const std::string out = argc > 2 && argv[2][0] ? argv[2] : ".";
    const std::map<std::string, std::function<void()>> handlers = {
        {"galaxy-sim-pm", [&] { galaxySimulationPM(out); }},
        {"galaxy-sim-p3m", [&] { galaxySimulationP3M(out); }},
        {"galaxy-collision-sim-pm", [&] { galaxyCollision(out, false); }},
        {"galaxy-collision-sim-p3m", [&] { galaxyCollision(out, true); }},
        {"cluster-sim-pm", [&] { plummer(out, false); }},
        {"cluster-sim-p3m", [&] { plummer(out, true); }},
        {"anisotropy", [&] { anisotropy(out); }},
        {"finite-diff-err", [&] { finiteDiffRelError(out); }},
        {"assignment-schemes", [&] { assignmentSchemes(out); }},
        {"poor-man-vs-laplacian", [&] { poorLaplace(out); }},
        {"pm-optimal", [&] { pmOptimal(out); }},
        {"pm-optimal-var-diameter", [&] { pmOptimalVaryingDiameter(out); }},
        {"pm-optimal-assignments", [&] { pmOptimalAssignments(out); }},
        {"pm-accuracy-soft", [&] { pmAccuracy(out, true); }},
        {"pm-accuracy-no-soft", [&] { pmAccuracy(out, false); }},
        {"p3m-accuracy-assignments", [&] { p3mAccuracy(out, false); }},
        {"p3m-accuracy-shapes", [&] { p3mAccuracy(out, true); }},
        // galaxySimulationPMTiming / P3MTiming (source/demos.cpp:779-836, 953-1016): "n seconds"
        {"galaxy-sim-pm-timing",
         [&] {
           for (int n = 10000; n <= 50000; n += 5000) galaxySimulationPM(out, n, 100, true);
         }},
        {"galaxy-sim-p3m-timing",
         [&] {
           for (int n = 10000; n <= 50000; n += 5000) galaxySimulationP3M(out, n, 25, true);
         }},
    };
    const auto it = handlers.find(option);
    if (it == handlers.end()) throw std::runtime_error("Unknown option: " + option);
    it->second();
  } catch (const std::exception& e) {
    std::cerr << e.what() << '\n';
    return 1;
  }
  return 0;
}
