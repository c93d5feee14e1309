/*
 * ref_shim.cpp - drives the reference's own CPU PMMethod / P3MMethod / ChainingMesh / ppMethod
 * code (compiled from the reference sources by oracle/Makefile) through the C functions
 * declared in oracle/oracle_api.h.  TEST INFRASTRUCTURE ONLY: it is the pin of the oracle
 * port and the source of the golden fixtures in tests/golden/; nothing in the product
 * links it.
 *
 * Each function follows the reference's own call sequence:
 *   forces   : PMMethod ctor -> stateToCodeUnits / massToCodeUnits -> initGreensFunction ->
 *              pmMethodStep  (reference source/pmMethod.cpp:30-75, 137-144)
 *   P3M      : + calculateShortRangeForces -> correctAccelerations (source/p3mMethod.cpp:59-73)
 *   run      : PMMethod::run / P3MMethod::run with a StateRecorder in a scratch directory
 *   cells    : ChainingMesh::fill / fillWithYSorting, walked cell by cell through
 *              getParticlesInCell (source/chainingMesh.cpp:20-58)
 *   pp       : the FP32 pairwise updateAccelerations of source/ppMethod.cpp:23-36
 */
#include <algorithm>
#include <array>
#include <complex>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iostream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

// P3MMethod keeps calculateShortRangeForces private and Grid keeps its potential mesh
// private; the shim needs both to read single force evaluations.
#define private public
#include "chainingMesh.h"
#include "grid.h"
#include "kissFFTAdapter.h"
#include "p3mMethod.h"
#include "pmMethod.h"
#include "ppMethod.h"
#include "stateRecorder.h"
#include "unitConversions.h"
#include "externalFields.h"
#undef private

#include "oracle_api.h"

// Defined with external linkage in the reference sources (p3mMethod.cpp:50, ppMethod.cpp:23).
void correctAccelerations(std::vector<Particle>& particles);
void updateAccelerations(std::vector<Particle>& particles, float G, float eps);

namespace {

std::vector<Vec3> toState(int n, const float* state) {
  std::vector<Vec3> st(2 * n);
  for (int i = 0; i < 2 * n; ++i) {
    st[i].x = state[3 * i];
    st[i].y = state[3 * i + 1];
    st[i].z = state[3 * i + 2];
  }
  return st;
}

std::function<Vec3(Vec3)> makeField(const orc_pm_params* p) {
  if (p->ext_kind == 1) {
    Vec3 c;
    c.x = p->ext_cx;
    c.y = p->ext_cy;
    c.z = p->ext_cz;
    float R = p->ext_R, M = p->ext_M, G = p->ext_G;
    return [c, R, M, G](Vec3 pos) -> Vec3 { return sphRadDecrField(pos, c, R, M, G); };
  }
  return [](Vec3) -> Vec3 { return Vec3::zero(); };
}

std::function<float(Vec3)> makePotential(const orc_pm_params* p) {
  if (p->ext_kind == 1) {
    Vec3 c;
    c.x = p->ext_cx;
    c.y = p->ext_cy;
    c.z = p->ext_cz;
    float R = p->ext_R, M = p->ext_M, G = p->ext_G;
    return [c, R, M, G](Vec3 pos) -> float { return sphRadDecrFieldPotential(pos, c, R, M, G); };
  }
  return [](Vec3) -> float { return 0.0f; };
}

struct PMBundle {
  std::array<int, 3> dims;
  std::unique_ptr<KissFFTAdapter<float>> fft;
  std::unique_ptr<Grid> grid;
  std::unique_ptr<PMMethod> pm;
};

PMBundle makePM(const orc_pm_params* p, int n, const float* state, const float* masses) {
  PMBundle b;
  // The reference passes the FFT dimensions reversed (z, y, x) to match its x-fastest
  // storage (source/demos.cpp:757-758).
  b.dims = {p->nz, p->ny, p->nx};
  b.fft = std::make_unique<KissFFTAdapter<float>>(b.dims.data(), 3);
  b.grid = std::make_unique<Grid>(std::make_tuple(p->nx, p->ny, p->nz), *b.fft);
  std::vector<float> ms(masses, masses + n);
  b.pm = std::make_unique<PMMethod>(
      toState(n, state), ms, std::make_tuple(p->box_x, p->box_y, p->box_z), makeField(p),
      makePotential(p), p->H, p->DT, p->G, static_cast<InterpolationScheme>(p->is),
      static_cast<FiniteDiffScheme>(p->fds), static_cast<GreensFunction>(p->gf), p->diameter,
      *b.grid);
  return b;
}

bool outside(const Vec3& v, const orc_pm_params* p) {
  return !(v.x >= 0 && v.x <= p->box_x && v.y >= 0 && v.y <= p->box_y && v.z >= 0 &&
           v.z <= p->box_z);
}

// After run() the particles are in code units, unless the loop stopped on an escaped
// particle, in which case they were left in original units (pmMethod.cpp:94-111).  The
// last frame of positions.dat tells which.
void exportRunState(const std::vector<Particle>& parts, const orc_pm_params* p,
                    const std::string& outdir, int n, float* state_out, int* escaped) {
  std::ifstream f(std::filesystem::path(outdir) / "positions.dat", std::ios::binary);
  std::vector<char> all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  bool esc = false;
  size_t frame = size_t(n) * sizeof(Vec3);
  if (all.size() >= 8 + frame) {
    size_t frames = (all.size() - 8) / frame;
    const Vec3* last = reinterpret_cast<const Vec3*>(all.data() + 8 + (frames - 1) * frame);
    for (int i = 0; i < n && !esc; ++i) esc = outside(last[i], p);
  }
  *escaped = esc ? 1 : 0;
  for (int i = 0; i < n; ++i) {
    Vec3 x = parts[i].position, v = parts[i].velocity;
    if (!esc) {
      x = positionToOriginalUnits(x, p->H);
      v = velocityToOriginalUnits(v, p->H, p->DT);
    }
    state_out[3 * i] = x.x;
    state_out[3 * i + 1] = x.y;
    state_out[3 * i + 2] = x.z;
    state_out[3 * (n + i)] = v.x;
    state_out[3 * (n + i) + 1] = v.y;
    state_out[3 * (n + i) + 2] = v.z;
  }
}

}  // namespace

extern "C" {

int ref_pm_accel(const orc_pm_params* p, int n, const float* state, const float* masses,
                 float* acc, float* density, float* potential, float* green) {
  try {
    PMBundle b = makePM(p, n, state, masses);
    auto& parts = b.pm->getParticles();
    stateToCodeUnits(parts, p->H, p->DT);
    massToCodeUnits(parts, p->H, p->DT, p->G);
    b.pm->initGreensFunction();
    b.pm->pmMethodStep();
    for (int i = 0; i < n; ++i) {
      acc[3 * i] = parts[i].acceleration.x;
      acc[3 * i + 1] = parts[i].acceleration.y;
      acc[3 * i + 2] = parts[i].acceleration.z;
    }
    int L = p->nx * p->ny * p->nz;
    for (int idx = 0; idx < L; ++idx) {
      if (density) density[idx] = b.grid->density[idx].real();
      if (potential) potential[idx] = b.grid->potential[idx].real();
      if (green) green[idx] = b.grid->greensFunction[idx].real();
    }
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_pm_accel: %s\n", e.what());
    return 1;
  }
}

int ref_p3m_accel(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
                  const float* masses, float* acc) {
  try {
    PMBundle b = makePM(p, n, state, masses);
    P3MMethod p3m(*b.pm, std::make_tuple(q->comp_x, q->comp_y, q->comp_z), q->cutoff,
                  q->diameter, p->H, q->softening, static_cast<CloudShape>(q->cloud_shape),
                  q->use_table != 0, q->y_sorting != 0);
    auto& parts = b.pm->getParticles();
    stateToCodeUnits(parts, p->H, p->DT);
    massToCodeUnits(parts, p->H, p->DT, p->G);
    b.pm->initGreensFunction();
    b.pm->pmMethodStep();
    p3m.calculateShortRangeForces(parts);
    correctAccelerations(parts);
    for (int i = 0; i < n; ++i) {
      acc[3 * i] = parts[i].acceleration.x;
      acc[3 * i + 1] = parts[i].acceleration.y;
      acc[3 * i + 2] = parts[i].acceleration.z;
    }
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_p3m_accel: %s\n", e.what());
    return 1;
  }
}

int ref_pm_run(const orc_pm_params* p, int n, const float* state, const float* masses,
               int sim_length, const char* outdir, float* state_out, int* escaped,
               int collect_diagnostics) {
  try {
    PMBundle b = makePM(p, n, state, masses);
    {
      StateRecorder rec(n, sim_length + 1, outdir);
      std::streambuf* old = std::cout.rdbuf();
      std::ostringstream sink;
      std::cout.rdbuf(sink.rdbuf());
      b.pm->run(rec, sim_length, (collect_diagnostics & 1) != 0, (collect_diagnostics & 2) != 0);
      std::cout.rdbuf(old);
    }
    exportRunState(b.pm->getParticles(), p, outdir, n, state_out, escaped);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_pm_run: %s\n", e.what());
    return 1;
  }
}

int ref_p3m_run(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
                const float* masses, int sim_length, const char* outdir, float* state_out,
                int* escaped, int collect_diagnostics) {
  try {
    PMBundle b = makePM(p, n, state, masses);
    P3MMethod p3m(*b.pm, std::make_tuple(q->comp_x, q->comp_y, q->comp_z), q->cutoff,
                  q->diameter, p->H, q->softening, static_cast<CloudShape>(q->cloud_shape),
                  q->use_table != 0, q->y_sorting != 0);
    {
      StateRecorder rec(n, sim_length + 1, outdir);
      std::streambuf* old = std::cout.rdbuf();
      std::ostringstream sink;
      std::cout.rdbuf(sink.rdbuf());
      p3m.run(rec, sim_length, (collect_diagnostics & 1) != 0, (collect_diagnostics & 2) != 0);
      std::cout.rdbuf(old);
    }
    exportRunState(b.pm->getParticles(), p, outdir, n, state_out, escaped);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_p3m_run: %s\n", e.what());
    return 1;
  }
}

int ref_chaining_mesh(const orc_p3m_params* q, float H, int n, const float* pos_code,
                      int y_sorting, int* order, int* counts, int* dims) {
  std::vector<Particle> parts;
  parts.reserve(n);
  for (int i = 0; i < n; ++i) {
    Vec3 x;
    x.x = pos_code[3 * i];
    x.y = pos_code[3 * i + 1];
    x.z = pos_code[3 * i + 2];
    parts.emplace_back(x, Vec3::zero(), 1.0f);
  }
  ChainingMesh cm(std::make_tuple(q->comp_x, q->comp_y, q->comp_z), q->cutoff, H, n);
  if (y_sorting)
    cm.fillWithYSorting(parts);
  else
    cm.fill(parts);
  auto [Mx, My, Mz] = cm.getLength();
  dims[0] = Mx;
  dims[1] = My;
  dims[2] = Mz;
  if (!order) return 0;
  int k = 0;
  for (int c = 0; c < cm.getSize(); ++c) {
    int cnt = 0;
    for (auto node = cm.getParticlesInCell(c); node != nullptr; node = node->next) {
      order[k++] = node->particleId;
      ++cnt;
    }
    counts[c] = cnt;
  }
  return 0;
}

int ref_pp_accel(int n, const float* pos, const float* masses, float G, float eps, float* acc) {
  std::vector<Particle> parts;
  parts.reserve(n);
  for (int i = 0; i < n; ++i) {
    Vec3 x;
    x.x = pos[3 * i];
    x.y = pos[3 * i + 1];
    x.z = pos[3 * i + 2];
    parts.emplace_back(x, Vec3::zero(), masses[i]);
  }
  updateAccelerations(parts, G, eps);
  for (int i = 0; i < n; ++i) {
    acc[3 * i] = parts[i].acceleration.x;
    acc[3 * i + 1] = parts[i].acceleration.y;
    acc[3 * i + 2] = parts[i].acceleration.z;
  }
  return 0;
}

int ref_sr_table(const orc_p3m_params* q, float H, float* table, float* delta_sq) {
  orc_pm_params p{};
  p.nx = p.ny = p.nz = 8;
  p.box_x = p.box_y = p.box_z = q->comp_x;
  p.H = H;
  p.DT = 1;
  p.G = 1;
  float st[6] = {1, 1, 1, 0, 0, 0}, ms[1] = {1};
  PMBundle b = makePM(&p, 1, st, ms);
  P3MMethod p3m(*b.pm, std::make_tuple(q->comp_x, q->comp_y, q->comp_z), q->cutoff, q->diameter,
                H, q->softening, static_cast<CloudShape>(q->cloud_shape), true, q->y_sorting != 0);
  for (int i = 0; i < 500; ++i) table[i] = p3m.FTable[i];
  *delta_sq = p3m.deltaSquared;
  return 0;
}

}  // extern "C"

/* ---- samplers: PlummerSampler(seed).sample(center, a, rMax, M, G, n) (the parameter order of
 * its definition, source/plummerSampler.cpp:11-16) and DiskSamplerLinear(seed).sample(...)
 * (source/diskSamplerLinear.cpp:10-33); state_out = 2n xyz triplets (positions, velocities). */
#include "diskSamplerLinear.h"
#include "plummerSampler.h"

extern "C" int ref_sample_plummer(unsigned int seed, const float* c, float a, float r_max, float M,
                                  float G, int n, float* state_out) {
  PlummerSampler s(seed);
  Vec3 center;
  center.x = c[0];
  center.y = c[1];
  center.z = c[2];
  auto st = s.sample(center, a, r_max, M, G, n);
  for (int i = 0; i < 2 * n; ++i) {
    state_out[3 * i] = st[i].x;
    state_out[3 * i + 1] = st[i].y;
    state_out[3 * i + 2] = st[i].z;
  }
  return 0;
}

extern "C" int ref_sample_disk_linear(unsigned int seed, const float* c, float rb, float mb, float rd,
                                      float md, float thickness, float G, int n, float r0,
                                      float* state_out) {
  DiskSamplerLinear s(seed);
  Vec3 center;
  center.x = c[0];
  center.y = c[1];
  center.z = c[2];
  auto st = s.sample(center, rb, mb, rd, md, thickness, G, n, r0);
  for (int i = 0; i < 2 * n; ++i) {
    state_out[3 * i] = st[i].x;
    state_out[3 * i + 1] = st[i].y;
    state_out[3 * i + 2] = st[i].z;
  }
  return 0;
}
