// api.cu - handles and the C ABI declared in include/pmgb.h.
//
// A pmgb_pm owns, on one CUDA stream:
//   particles  SoA float4 x 2 buffers: (x, y, z, m) and (vx, vy, vz, original id bits), code
//              units, kept in the last sorted order; accelerations (final and PM part)
//   mesh       fixed-point density (u64), half spectrum (float2, rows of nxp), potential (f32),
//              influence function (f32, half spectrum, 1/N folded in), twiddles
//   sort       64-bit keys / 32-bit values x 2 and the radix histogram
//   flags      [0] stop (a particle escaped: every later kernel returns at once),
//              [1] iteration whose drift escaped
// A pmgb_p3m adds the chaining mesh (cell starts, work items) and the short-range table, and
// makes every force evaluation of its PM handle a P3M one.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numbers>
#include <string>
#include <vector>

#include "handles.cuh"

namespace pmgb {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
static std::atomic<long long> g_launches{0};
void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

static int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}
static bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

float mass_code_factor(float H, float DT, float G) {
  volatile float c = DT * DT * 4 * std::numbers::pi_v<float> * G / (H * H * H);
  return c;
}

}  // namespace pmgb

using namespace pmgb;

namespace {

template <typename T>
int dalloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T) + 16);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return PMGB_ENOMEM;
  }
  return PMGB_OK;
}

void free_pm(pmgb_pm* h) {
  if (!h) return;
  diag_free(h);
  void* ptrs[]= {h->pm[0], h->pm[1], h->vi[0], h->vi[1], h->acc,  h->acc_pm, h->keys, h->keys_alt,
                  h->vals,  h->vals_alt, h->hist, h->rho, h->spec, h->phi, h->ghat, h->tw, h->flags,
                  h->stage, h->mass_code};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->gplans) gfft_plans_destroy(h->gplans);
  if (h->ivel) cudaFree(h->ivel);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
}

// float arithmetic of include/unitConversions.h (reference), evaluated on the host
inline float f_mass_to_code(float m, float H, float DT, float G) { return mass_code_factor(H, DT, G) * m; }

int check_cfg(const pmgb_pm_config* c, int n) {
  if (!c) return set_error("null config"), PMGB_EINVAL;
  if (n < 0) return set_error("negative particle count"), PMGB_EINVAL;
  for (int i = 0; i < 3; ++i)
    if (c->grid[i] < 4 || c->grid[i] > 4096)
      return set_error("grid points must be in [4, 4096]"), PMGB_EINVAL;
  if (c->interpolation < 0 || c->interpolation > 2)
    return set_error("Unkown interpolation scheme"), PMGB_EINVAL;
  if (c->finite_diff < 0 || c->finite_diff > 1)
    return set_error("Unknown finite difference type."), PMGB_EINVAL;
  if (c->greens < 0 || c->greens > 3) return set_error("not implemented"), PMGB_EINVAL;
  if (!(c->H > 0) || !(c->DT > 0)) return set_error("H and DT must be positive"), PMGB_EINVAL;
  if ((c->greens == PMGB_S1_OPTIMAL || c->greens == PMGB_S2_OPTIMAL) && !(c->particle_diameter > 0))
    return set_error("optimal Green's functions need a positive particle diameter"), PMGB_EINVAL;
  return PMGB_OK;
}

int upload_state(pmgb_pm* h, const float* pos, const float* vel, int units) {
  const size_t n = (size_t)h->n;
  h->acc_mode = -1;
  if (n == 0) return PMGB_OK;
  PMGB_CUDA_TRY(cudaMemcpyAsync(h->stage, pos, 3 * n * sizeof(float), cudaMemcpyHostToDevice, h->st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(h->stage + 3 * n, vel, 3 * n * sizeof(float), cudaMemcpyHostToDevice, h->st));
  int rc = launch_pack(h->stage, h->stage + 3 * n, h->mass_code, h->n, h->cfg.H, h->cfg.DT,
                       units == PMGB_UNITS_ORIGINAL, h->pm[h->cur], h->vi[h->cur], h->st);
  if (rc) return rc;
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  h->since_sort = 1 << 30;
  return PMGB_OK;
}

// Sort particles (P3M: chaining-mesh order every evaluation; PM: brick order every
// sort_interval evaluations) and permute them into the other buffer.
int sort_particles(pmgb_pm* h) {
  const int n = h->n;
  // The sort only permutes particles, so it runs even after an escape (the stop flag): the
  // buffer flips below then stay consistent with what is in memory.
  const int* stop = nullptr;
  pmgb_p3m* q = h->p3m;
  int rc;
  if (q) {
    rc = launch_chain_keys(h->pm[h->cur], h->vi[h->cur], n, q->cd, q->cfg.y_sorting, stop, h->keys, h->vals, h->st);
    if (rc) return rc;
    const int bits = 32 + ilog2(q->nsub + 2);
    rc = radix_sort_pairs(&h->keys, &h->vals, &h->keys_alt, &h->vals_alt, h->hist, n, bits, h->st);
    if (rc) return rc;
    if (q->cfg.y_sorting) {
      rc = launch_fix_ties(h->keys, h->vals, h->vi[h->cur], n, stop, h->st);
      if (rc) return rc;
    }
    rc = launch_gather(h->keys, h->vals, n, h->pm[h->cur], h->vi[h->cur], h->pm[1 - h->cur],
                       h->vi[1 - h->cur], q->cell_start, q->nsub + 1, stop, h->st);
    if (rc) return rc;
    h->cur = 1 - h->cur;
    return PMGB_OK;
  }
  // default 16: a brick sort of 4M particles costs ~0.25 ms, and on the benchmark workloads
  // particles move well under a brick (4 cells) in 16 steps (deposit and interpolation times
  // measured unchanged between re-sorts every 4, 8, 16 and 32 steps)
  const int interval = h->cfg.sort_interval > 0 ? h->cfg.sort_interval : 16;
  if (h->since_sort < interval) {
    ++h->since_sort;
    return PMGB_OK;
  }
  const int bshift = 2;
  int maxb = std::max(h->m.nx, std::max(h->m.ny, h->m.nz)) >> bshift;
  const int bits = 3 * std::max(1, ilog2(maxb));
  rc = launch_brick_keys(h->pm[h->cur], n, h->m, bshift, stop, h->keys, h->vals, h->st);
  if (rc) return rc;
  rc = radix_sort_pairs(&h->keys, &h->vals, &h->keys_alt, &h->vals_alt, h->hist, n, bits, h->st);
  if (rc) return rc;
  rc = launch_gather(h->keys, h->vals, n, h->pm[h->cur], h->vi[h->cur], h->pm[1 - h->cur],
                     h->vi[1 - h->cur], nullptr, 0, stop, h->st);
  if (rc) return rc;
  h->cur = 1 - h->cur;
  h->since_sort = 1;
  return PMGB_OK;
}

// One force evaluation.  kdk = 0: accelerations only.  kdk = 1: then kick by `kick` and, if
// `drift`, drift (tagging an escape with `tag`).
int force(pmgb_pm* h, int kdk, float kick, int drift, int tag, bool timed) {
  const int n = h->n;
  int* stop = h->flags;
  int rc;
  if (timed) cudaEventRecord(h->ev[0], h->st);
  rc = sort_particles(h);
  if (rc) return rc;
  if (timed) cudaEventRecord(h->ev[1], h->st);
  rc = launch_deposit(h->cfg.interpolation, h->pm[h->cur], n, h->m, h->sp.fx_scale, h->rho, stop, h->st);
  if (rc) return rc;
  if (timed) cudaEventRecord(h->ev[2], h->st);
  if (h->generic)
    rc = launch_poisson_generic(h->rho, h->spec, h->phi, h->ghat, h->gplans, h->m, h->sp.fx_inv, stop,
                                h->st, diag_density(h));
  else
    rc = launch_poisson(h->rho, h->spec, h->phi, h->ghat, h->tw, h->nmax, h->m, h->sp.fx_inv, stop, h->st,
                        diag_density(h));
  if (rc) return rc;
  if (timed) cudaEventRecord(h->ev[3], h->st);
  StepParams sp = h->sp;
  sp.step_tag = tag;
  pmgb_p3m* q = h->p3m;
  if (!q) {
    rc = launch_interp(kdk != 0, h->pm[h->cur], h->vi[h->cur], h->acc, n, h->phi, sp, kick, drift, stop, h->st);
    if (rc) return rc;
    if (timed) {
      cudaEventRecord(h->ev[4], h->st);
      cudaEventRecord(h->ev[5], h->st);
    }
    h->acc_mode = (kdk && drift) ? -1 : closure_mode(h);
    return PMGB_OK;
  }
  rc = launch_interp(false, h->pm[h->cur], h->vi[h->cur], h->acc_pm, n, h->phi, sp, kick, drift, stop, h->st);
  if (rc) return rc;
  if (h->closure) {
    rc = closure_apply(h);
    if (rc) return rc;
  }
  // ev[4] is recorded just before the pair kernel (after its work-item setup)
  rc = launch_pair(h->pm[h->cur], h->vi[h->cur], h->acc_pm, q->cell_start, q->cd,
                   q->item_cnt, q->item_off, q->scan_tmp, q->nitems, q->items, q->nitems_max, q->heavy,
                   q->counter, q->pp, q->table, sp,
                   kick, drift, kdk, h->pm[1 - h->cur], h->vi[1 - h->cur], h->acc,
                   q->count_pairs ? q->npairs : nullptr, stop,
                   h->num_sms, timed ? h->ev[4] : nullptr, h->st, h->equal_mass, q->slots, n,
                   q->unit_stride, &q->sym);
  if (rc) return rc;
  if (kdk) {
    h->cur = 1 - h->cur;
    // acc was written in the order of the particles just moved into h->cur: same slots
  }
  if (timed) cudaEventRecord(h->ev[5], h->st);
  // a drift after the force leaves accelerations that belong to the old positions; a sampled
  // pair pass leaves most of them incomplete
  h->acc_mode = (kdk && drift) || q->unit_stride > 1 ? -1 : closure_mode(h);
  return PMGB_OK;
}

// What a run records right after the drift of the iteration tagged `tag`.
int after_drift(pmgb_pm* h, int tag) {
  int rc = diag_after_drift(h, tag);
  if (rc) return rc;
  return rec_after_drift(h, tag);
}

// Run start: the stop and timeout words cleared, the escape iteration at INT_MAX.
int clear_run_flags(pmgb_pm* h) {
  PMGB_CUDA_TRY(cudaMemsetAsync(h->flags, 0, 3 * sizeof(int), h->st));
  const int big = 0x7FFFFFFF;
  PMGB_CUDA_TRY(cudaMemcpyAsync(h->flags + 1, &big, sizeof(int), cudaMemcpyHostToDevice, h->st));
  return PMGB_OK;
}

// Run end (after the stream synchronised): flags[0..2] read back; a bounded wait that gave up
// comes first, then an escape.
int run_status(const int flags[3], int* steps_done, int done_steps) {
  if (flags[kFlagTimeout]) return set_error("a bounded device wait gave up"), PMGB_ETIMEOUT;
  if (flags[0]) {
    if (steps_done) *steps_done = flags[1];
    set_error("Particle moved outside the computational box.");
    return PMGB_EESCAPED;
  }
  if (steps_done) *steps_done = done_steps;
  return PMGB_OK;
}

int run_loop(pmgb_pm* h, int sim_length, int* steps_done) {
  int rc = clear_run_flags(h);
  if (rc) return rc;
  rc = diag_run_begin(h);
  if (rc) return rc;
  // initial force, half kick (setHalfStepVelocities) and the drift of iteration 0
  rc = force(h, 1, 0.5f, 1, 0, false);
  if (rc) return rc;
  rc = after_drift(h, 0);
  if (rc) return rc;
  for (int t = 0; t <= sim_length; ++t) {
    rc = force(h, 1, 1.0f, t < sim_length ? 1 : 0, t + 1, false);
    if (rc) return rc;
    if (t < sim_length && (rc = after_drift(h, t + 1))) return rc;
  }
  int flags[3];
  PMGB_CUDA_TRY(cudaMemcpyAsync(flags, h->flags, 3 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  rc = run_status(flags, steps_done, sim_length + 1);
  if (rc) h->acc_mode = -1;  // stopped after a drift whose force was skipped
  return rc;
}

}  // namespace

extern "C" {

const char* pmgb_last_error(void) { return g_last_error.c_str(); }
const char* pmgb_version(void) { return "pmgb 0.1 sm_103a"; }

int pmgb_kernel_launches(long long* count) {
  if (!count) return set_error("null argument"), PMGB_EINVAL;
  *count = g_launches.load();
  return PMGB_OK;
}

int pmgb_pm_create(const pmgb_pm_config* cfg, int n, const float* state, const float* masses,
                   pmgb_pm** out) {
  if (!out) return set_error("null output handle"), PMGB_EINVAL;
  *out = nullptr;
  int rc = check_cfg(cfg, n);
  if (rc) return rc;
  if (n > 0 && (!state || !masses)) return set_error("null state or masses"), PMGB_EINVAL;
  pmgb_pm* h = new pmgb_pm();
  h->cfg = *cfg;
  h->n = n;
  MeshDims& m = h->m;
  m.nx = cfg->grid[0];
  m.ny = cfg->grid[1];
  m.nz = cfg->grid[2];
  m.lx = ilog2(m.nx);
  m.ly = ilog2(m.ny);
  m.lz = ilog2(m.nz);
  m.nxh = m.nx / 2 + 1;
  m.nxp = (m.nxh + 3) & ~3;
  m.L = (long long)m.nx * m.ny * m.nz;
  h->nmax = std::max(m.nx, std::max(m.ny, m.nz));
  StepParams& sp = h->sp;
  sp.m = m;
  sp.is = cfg->interpolation;
  sp.fds = cfg->finite_diff;
  sp.H = cfg->H;
  sp.DT = cfg->DT;
  sp.box_x = cfg->box[0];
  sp.box_y = cfg->box[1];
  sp.box_z = cfg->box[2];
  sp.ext.kind = cfg->ext.kind;
  sp.ext.cx = cfg->ext.center[0];
  sp.ext.cy = cfg->ext.center[1];
  sp.ext.cz = cfg->ext.center[2];
  sp.ext.R = cfg->ext.R;
  sp.ext.M = cfg->ext.M;
  sp.ext.G = cfg->ext.G;
  sp.step_tag = 0;
  sp.periodic = cfg->periodic ? 1 : 0;

  auto fail = [&](int code) {
    free_pm(h);
    return code;
  };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    set_error("no CUDA device");
    return fail(PMGB_ECUDA);
  }
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return fail(PMGB_ECUDA);
  }
  for (auto& e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return set_error("cudaEventCreate failed"), fail(PMGB_ECUDA);
  const size_t N = std::max(n, 1);
  const size_t half = (size_t)m.nxp * m.ny * m.nz;
  // powers of two in [8, 512] take the specialised half-spectrum Poisson solve (fft.cu); other
  // meshes the mixed-radix one over a full complex mesh (gfft.cu)
  for (int i = 0; i < 3; ++i)
    if (!pow2(cfg->grid[i]) || cfg->grid[i] < 8 || cfg->grid[i] > 512) h->generic = true;
  const size_t spec_elems = h->generic ? std::max(half, (size_t)m.L) : half;
  if ((rc = dalloc(&h->pm[0], N)) || (rc = dalloc(&h->pm[1], N)) || (rc = dalloc(&h->vi[0], N)) ||
      (rc = dalloc(&h->vi[1], N)) || (rc = dalloc(&h->acc, N)) || (rc = dalloc(&h->acc_pm, N)) ||
      (rc = dalloc(&h->keys, N)) || (rc = dalloc(&h->keys_alt, N)) || (rc = dalloc(&h->vals, N)) ||
      (rc = dalloc(&h->vals_alt, N)) || (rc = dalloc(&h->hist, radix_hist_words((int)N))) ||
      (rc = dalloc(&h->rho, (size_t)m.L)) || (rc = dalloc(&h->spec, spec_elems)) || (rc = dalloc(&h->phi, (size_t)m.L)) ||
      (rc = dalloc(&h->ghat, half)) || (rc = dalloc(&h->tw, (size_t)h->nmax / 2 + 1)) || (rc = dalloc(&h->flags, 4)) ||
      (rc = dalloc(&h->stage, 9 * N)) || (rc = dalloc(&h->mass_code, N)))
    return fail(rc);
  if (cudaMemsetAsync(h->rho, 0, (size_t)m.L * sizeof(u64), h->st) != cudaSuccess ||
      cudaMemsetAsync(h->spec, 0, spec_elems * sizeof(float2), h->st) != cudaSuccess ||
      cudaMemsetAsync(h->phi, 0, (size_t)m.L * sizeof(float), h->st) != cudaSuccess ||
      cudaMemsetAsync(h->acc, 0, N * sizeof(float4), h->st) != cudaSuccess ||
      cudaMemsetAsync(h->flags, 0, 4 * sizeof(int), h->st) != cudaSuccess) {
    set_error("cudaMemset failed");
    return fail(PMGB_ECUDA);
  }
  if (h->generic) {
    const int dims[3] = {m.nx, m.ny, m.nz};
    rc = gfft_plans_create(dims, &h->gplans);
  } else {
    rc = fft_configure(m);
  }
  if (rc) return fail(rc);
  {
    std::vector<float2> tw(h->nmax / 2 + 1);
    for (int j = 0; j <= h->nmax / 2; ++j) {
      double a = -2.0 * 3.14159265358979323846 * j / h->nmax;
      tw[j] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    if (cudaMemcpyAsync(h->tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, h->st) != cudaSuccess) {
      set_error("twiddle upload failed");
      return fail(PMGB_ECUDA);
    }
  }
  // particles: code units (stateToCodeUnits, massToCodeUnits), original ids in vi.w
  std::vector<float4> hp(N), hv(N);
  double msum = 0.0;
  const float H = cfg->H, DT = cfg->DT, G = cfg->G;
  for (int i = 0; i < n; ++i) {
    const float* x = state + 3 * i;
    const float* v = state + 3 * (n + i);
    const float mc = f_mass_to_code(masses[i], H, DT, G);
    hp[i] = make_float4(x[0] / H, x[1] / H, x[2] / H, mc);
    float idf;
    int id = i;
    std::memcpy(&idf, &id, 4);
    hv[i] = make_float4((DT * v[0]) / H, (DT * v[1]) / H, (DT * v[2]) / H, idf);
    msum += std::fabs((double)mc);
  }
  // fixed-point scale 2^k with 4 * sum|m| * 2^k <= 2^62 (TSC weights sum to at most 3.375 in
  // magnitude per particle, the reference's floor-offset quirk included)
  int k = msum > 0 ? (int)std::floor(62.0 - std::log2(4.0 * msum)) : 62;
  k = std::min(k, 100);
  sp.fx_scale = std::ldexp(1.0f, k);
  sp.fx_inv = std::ldexp(1.0f, -k);
  if (n > 0 &&
      (cudaMemcpyAsync(h->pm[0], hp.data(), n * sizeof(float4), cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
       cudaMemcpyAsync(h->vi[0], hv.data(), n * sizeof(float4), cudaMemcpyHostToDevice, h->st) != cudaSuccess)) {
    set_error("particle upload failed");
    return fail(PMGB_ECUDA);
  }
  {
    std::vector<float> mc(N, 0.f);
    for (int i = 0; i < n; ++i) mc[i] = hp[i].w;
    h->equal_mass = n > 0 && std::all_of(mc.begin(), mc.begin() + n, [&](float m) { return m == mc[0]; });
    if (cudaMemcpyAsync(h->mass_code, mc.data(), N * sizeof(float), cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
        cudaStreamSynchronize(h->st) != cudaSuccess) {
      set_error("mass upload failed");
      return fail(PMGB_ECUDA);
    }
  }
  rc = pmgb_pm_init_greens_function(h);
  if (rc) return fail(rc);
  if (cudaStreamSynchronize(h->st) != cudaSuccess) {
    set_error(std::string("create: ") + cudaGetErrorString(cudaGetLastError()));
    return fail(PMGB_ECUDA);
  }
  *out = h;
  return PMGB_OK;
}

int pmgb_pm_destroy(pmgb_pm* h) {
  if (!h) return PMGB_OK;
  if (h->p3m) return set_error("destroy the P3M handle borrowing this PM handle first"), PMGB_EINVAL;
  cudaStreamSynchronize(h->st);
  free_pm(h);
  return PMGB_OK;
}

int pmgb_pm_init_greens_function(pmgb_pm* h) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  const double a = (double)h->cfg.particle_diameter / (double)h->cfg.H;
  int rc = launch_green(h->ghat, h->m, h->cfg.greens, h->cfg.interpolation, h->cfg.finite_diff, a, h->st);
  if (rc) return rc;
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  return PMGB_OK;
}

int pmgb_pm_method_step(pmgb_pm* h) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaMemsetAsync(h->flags, 0, sizeof(int), h->st));
  PMGB_CUDA_TRY(cudaMemsetAsync(h->flags + kFlagTimeout, 0, sizeof(int), h->st));
  int rc = force(h, 0, 0.f, 0, 0, true);
  if (rc) return rc;
  int timed_out = 0;
  if (h->closure)  // the closure's tensor-core kernel is the one with bounded waits
    PMGB_CUDA_TRY(cudaMemcpyAsync(&timed_out, h->flags + kFlagTimeout, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  for (int s = 0; s < 5; ++s) cudaEventElapsedTime(&h->stage_ms[s], h->ev[s], h->ev[s + 1]);
  if (timed_out) return set_error("a bounded device wait gave up"), PMGB_ETIMEOUT;
  return PMGB_OK;
}

int pmgb_pm_advance(pmgb_pm* h, int n_steps, int* steps_done, float* device_ms) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  if (n_steps < 0) return set_error("negative step count"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  int rc0 = clear_run_flags(h);
  if (rc0) return rc0;
  PMGB_CUDA_TRY(cudaEventRecord(h->ev[0], h->st));
  if (n_steps > 0) {
    // the first drift of the loop body, then (force, kick, drift) with the last drift left out
    StepParams sp = h->sp;
    sp.step_tag = 0;
    int rc = diag_before_drift(h);
    if (rc) return rc;
    rc = launch_kick_drift(h->pm[h->cur], h->vi[h->cur], h->acc, h->n, sp, 0.f, 1, h->flags, h->st);
    if (rc) return rc;
    if ((rc = after_drift(h, 0))) return rc;
    for (int t = 0; t < n_steps; ++t) {
      rc = force(h, 1, 1.0f, t + 1 < n_steps ? 1 : 0, t + 1, false);
      if (rc) return rc;
      if (t + 1 < n_steps && (rc = after_drift(h, t + 1))) return rc;
    }
  }
  PMGB_CUDA_TRY(cudaEventRecord(h->ev[5], h->st));
  int flags[3];
  PMGB_CUDA_TRY(cudaMemcpyAsync(flags, h->flags, 3 * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  if (device_ms) cudaEventElapsedTime(device_ms, h->ev[0], h->ev[5]);
  rc0 = run_status(flags, steps_done, n_steps);
  if (rc0) h->acc_mode = -1;  // stopped after a drift whose force was skipped
  return rc0;
}

int pmgb_pm_run_recorded(pmgb_pm* h, pmgb_recorder* rec, int sim_length, int collect_diagnostics,
                         int record_field, int* steps_done) {
  if (!h || !rec) return set_error("null handle"), PMGB_EINVAL;
  if (sim_length < 0) return set_error("negative simLength"), PMGB_EINVAL;
  if (collect_diagnostics && diag_capacity(h) < sim_length + 1) {
    int rc = pmgb_pm_set_diagnostics(h, sim_length + 1);
    if (rc) return rc;
  }
  h->rec = rec;
  h->rec_field = record_field ? 1 : 0;
  int rc = rec_begin_run(h, h->rec_field);
  const int rc_run = rc ? rc : run_loop(h, sim_length, steps_done);
  rc = rc_run == PMGB_OK || rc_run == PMGB_EESCAPED ? rec_end_run(h, collect_diagnostics) : PMGB_OK;
  h->rec = nullptr;
  if (rc) return rc;
  if (rc_run != PMGB_OK && rc_run != PMGB_EESCAPED) return rc_run;
  rc = pmgb_recorder_flush(rec, nullptr, 0);
  if (rc) return rc;
  if (rc_run == PMGB_EESCAPED) set_error("Particle moved outside the computational box.");
  return rc_run;
}

int pmgb_pm_run(pmgb_pm* h, int sim_length, int* steps_done) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  if (sim_length < 0) return set_error("negative simLength"), PMGB_EINVAL;
  return run_loop(h, sim_length, steps_done);
}

int pmgb_pm_get_particles(pmgb_pm* h, float* pos, float* vel, float* acc, int units) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  const size_t n = (size_t)h->n;
  if (n == 0) return PMGB_OK;
  int rc = launch_unpack(h->pm[h->cur], h->vi[h->cur], h->acc, h->n, h->cfg.H, h->cfg.DT,
                         units == PMGB_UNITS_ORIGINAL, h->stage, h->stage + 3 * n, h->stage + 6 * n, h->st);
  if (rc) return rc;
  if (pos) PMGB_CUDA_TRY(cudaMemcpyAsync(pos, h->stage, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  if (vel) PMGB_CUDA_TRY(cudaMemcpyAsync(vel, h->stage + 3 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  if (acc) PMGB_CUDA_TRY(cudaMemcpyAsync(acc, h->stage + 6 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  return PMGB_OK;
}

int pmgb_pm_set_particles(pmgb_pm* h, const float* pos, const float* vel, int units) {
  if (!h || !pos || !vel) return set_error("null argument"), PMGB_EINVAL;
  return upload_state(h, pos, vel, units);
}

int pmgb_pm_escaped(pmgb_pm* h, int* escaped) {
  if (!h || !escaped) return set_error("null argument"), PMGB_EINVAL;
  std::vector<float> pos(3 * (size_t)std::max(h->n, 1));
  int rc = pmgb_pm_get_particles(h, pos.data(), nullptr, nullptr, PMGB_UNITS_ORIGINAL);
  if (rc) return rc;
  *escaped = 0;
  for (int i = 0; i < h->n; ++i) {
    const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    if (!(x >= 0 && x <= h->cfg.box[0] && y >= 0 && y <= h->cfg.box[1] && z >= 0 && z <= h->cfg.box[2])) {
      *escaped = 1;
      break;
    }
  }
  return PMGB_OK;
}

int pmgb_pm_get_density(pmgb_pm* h, float* density) {
  if (!h || !density) return set_error("null argument"), PMGB_EINVAL;
  // the forward FFT consumes the fixed-point mesh: deposit again into it and read it out
  PMGB_CUDA_TRY(cudaMemsetAsync(h->flags, 0, sizeof(int), h->st));
  int rc = launch_deposit(h->cfg.interpolation, h->pm[h->cur], h->n, h->m, h->sp.fx_scale, h->rho, h->flags, h->st);
  if (rc) return rc;
  std::vector<unsigned long long> fx((size_t)h->m.L);
  PMGB_CUDA_TRY(cudaMemcpyAsync(fx.data(), h->rho, fx.size() * sizeof(u64), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaMemsetAsync(h->rho, 0, fx.size() * sizeof(u64), h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  for (size_t i = 0; i < fx.size(); ++i) density[i] = (float)(long long)fx[i] * h->sp.fx_inv;
  return PMGB_OK;
}

int pmgb_pm_get_potential(pmgb_pm* h, float* potential) {
  if (!h || !potential) return set_error("null argument"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaMemcpyAsync(potential, h->phi, (size_t)h->m.L * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  return PMGB_OK;
}

int pmgb_pm_get_greens_function(pmgb_pm* h, float* ghat) {
  if (!h || !ghat) return set_error("null argument"), PMGB_EINVAL;
  const MeshDims& m = h->m;
  std::vector<float> g((size_t)m.nxp * m.ny * m.nz);
  PMGB_CUDA_TRY(cudaMemcpyAsync(g.data(), h->ghat, g.size() * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  for (int z = 0; z < m.nz; ++z)
    for (int y = 0; y < m.ny; ++y)
      for (int x = 0; x < m.nxh; ++x)
        ghat[((size_t)z * m.ny + y) * m.nxh + x] = g[((size_t)z * m.ny + y) * m.nxp + x];
  return PMGB_OK;
}

int pmgb_pm_stage_times(pmgb_pm* h, float* ms5) {
  if (!h || !ms5) return set_error("null argument"), PMGB_EINVAL;
  for (int s = 0; s < 5; ++s) ms5[s] = h->stage_ms[s];
  return PMGB_OK;
}

int pmgb_pm_size(pmgb_pm* h, int* n, int* grid3) {
  if (!h) return set_error("null handle"), PMGB_EINVAL;
  if (n) *n = h->n;
  if (grid3) {
    grid3[0] = h->m.nx;
    grid3[1] = h->m.ny;
    grid3[2] = h->m.nz;
  }
  return PMGB_OK;
}

int pmgb_pm_get_stream(pmgb_pm* h, void** stream) {
  if (!h || !stream) return set_error("null argument"), PMGB_EINVAL;
  *stream = (void*)h->st;
  return PMGB_OK;
}

// ------------------------------------------------------------------------- P3M -------
int pmgb_p3m_create(pmgb_pm* pm, const pmgb_p3m_config* cfg, pmgb_p3m** out) {
  if (!pm || !cfg || !out) return set_error("null argument"), PMGB_EINVAL;
  *out = nullptr;
  if (pm->p3m || pm->closure) return set_error("this PM handle already has a P3M handle"), PMGB_EINVAL;
  return pmgb::p3m_create_internal(pm, cfg, out, true);
}

}  // extern "C"

namespace pmgb {
// P3M handle over `pm`; attach = make it the PM handle's pair pass now (a closure keeps two
// detached handles and switches between them).
int p3m_create_internal(pmgb_pm* pm, const pmgb_p3m_config* cfg, pmgb_p3m** out, bool attach) {
  if (!(cfg->cutoff > 0)) return set_error("cutoff radius must be positive"), PMGB_EINVAL;
  if (cfg->cloud_shape != PMGB_S1 && cfg->cloud_shape != PMGB_S2) return set_error("not implemented"), PMGB_EINVAL;
  pmgb_p3m* q = new pmgb_p3m();
  q->pm = pm;
  q->cfg = *cfg;
  const float H = pm->cfg.H;
  // ChainingMesh ctor (source/chainingMesh.cpp:6-18): M = int(box / cutoff), HC = (box/M)/H
  q->cd.Mx = (int)(cfg->comp_box[0] / cfg->cutoff);
  q->cd.My = (int)(cfg->comp_box[1] / cfg->cutoff);
  q->cd.Mz = (int)(cfg->comp_box[2] / cfg->cutoff);
  if (q->cd.Mx < 1 || q->cd.My < 1 || q->cd.Mz < 1) {
    delete q;
    return set_error("computational box smaller than the cutoff radius"), PMGB_EINVAL;
  }
  q->cd.HCx = (cfg->comp_box[0] / q->cd.Mx) / H;
  q->cd.HCy = (cfg->comp_box[1] / q->cd.My) / H;
  q->cd.HCz = (cfg->comp_box[2] / q->cd.Mz) / H;
  q->ncells = q->cd.Mx * q->cd.My * q->cd.Mz;
  // Sub-columns per cell axis when the lists are y-sorted (the pair pass prunes by x-z gap and y
  // window per sub-column, and its symmetric part pairs sub-columns): 5 where the particles
  // average at least 96 per cell, 4 from 32, else 3.  Pair pass on the disk workloads, 3 / 4 / 5
  // sub-columns, by mean particles per cell: 14: 26.3 / 27.0 / 29.1 ms; 28: 5.59 / 5.63 / 6.07;
  // 39: 43.8 / 42.4 / 43.5; 60: 56.9 / 52.9 / 53.6; 113: 87.6 / 74.2 / 73.8 (2 x 2 was slower
  // throughout).  A finer split only where its symmetric slots (27 sub^2 x 16 B per particle)
  // stay within a quarter of the free device memory (the rule the allocation below applies).
  // The reference's unsorted fill order keeps whole cells.
  q->cd.sub = 1;
  if (cfg->y_sorting) {
    const long long n = pm->n, nc = q->ncells;
    q->cd.sub = n >= 96 * nc ? 5 : n >= 32 * nc ? 4 : 3;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      free_b = 0;
      cudaGetLastError();
    }
    while (q->cd.sub > 3 && 27ull * q->cd.sub * q->cd.sub * sizeof(float4) * (size_t)n > free_b / 4) --q->cd.sub;
  }
  q->cd.HCsx = q->cd.HCx / q->cd.sub;
  q->cd.HCsz = q->cd.HCz / q->cd.sub;
  q->nsub = q->ncells * q->cd.sub * q->cd.sub;
  // initSRForceTable (source/p3mMethod.cpp:275-294) in the reference's float arithmetic
  const float re = cfg->cutoff / H, a = cfg->particle_diameter / H, eps = cfg->softening / H;
  q->delta2 = re * re / (500 - 1);
  const float Gc = 1 / (4 * std::numbers::pi_v<float>);
  auto refS1 = [&](float r) -> float {
    if (r >= a) return Gc / (r * r);
    return Gc / (a * a) * (8 * r / a - 9 * r * r / (a * a) + 2 * std::pow(r / a, 4.0f));
  };
  auto refS2 = [&](float r) -> float {
    const float u = 2 * r / a;
    if (u <= 1)
      return Gc / (35 * std::pow(a, 2.0f)) *
             (224 * u - 224 * std::pow(u, 3.0f) + 70 * std::pow(u, 4.0f) + 48 * std::pow(u, 5.0f) - 21 * std::pow(u, 6.0f));
    if (u <= 2)
      return Gc / (35 * std::pow(a, 2.0f)) *
             (12 / std::pow(u, 2.0f) - 224 + 896 * u - 840 * std::pow(u, 2.0f) + 224 * std::pow(u, 3.0f) +
              70 * std::pow(u, 4.0f) - 48 * std::pow(u, 5.0f) + 7 * std::pow(u, 6.0f));
    return Gc / (r * r);
  };
  for (int i = 0; i < 500; ++i) {
    volatile float rSquared = i * q->delta2;
    const float r = std::sqrt((float)rSquared);
    const float R = cfg->cloud_shape == PMGB_S1 ? -refS1(r) : -refS2(r);
    const float totalForce = -Gc / (r * r + eps * eps);
    q->table_h[i] = r == 0 ? 0.0f : (totalForce - R) / std::sqrt(r * r + eps * eps);
  }
  // the smooth part R(r)/r of the table-free force (shortRangeForce, source/p3mMethod.cpp:
  // 220-238: (-G/r^2 + R(r)) / r per unit r_ij) at r^2 = i delta, in double, for the slotted
  // pass's exact mode (pair.cu), which adds the Newton part -G/r^3 itself; its limit at r = 0
  {
    const double ad = a, Gd = 1.0 / (4.0 * std::numbers::pi), d2 = (double)re * re / 499.0;
    auto Rd = [&](double r) -> double {
      if (cfg->cloud_shape == PMGB_S1) {
        if (r >= ad) return Gd / (r * r);
        const double q1 = r / ad;
        return Gd / (ad * ad) * (8 * q1 - 9 * q1 * q1 + 2 * q1 * q1 * q1 * q1);
      }
      const double u = 2 * r / ad;
      if (u <= 1)
        return Gd / (35 * ad * ad) * (224 * u - 224 * std::pow(u, 3) + 70 * std::pow(u, 4) + 48 * std::pow(u, 5) - 21 * std::pow(u, 6));
      if (u <= 2)
        return Gd / (35 * ad * ad) *
               (12 / (u * u) - 224 + 896 * u - 840 * u * u + 224 * std::pow(u, 3) + 70 * std::pow(u, 4) -
                48 * std::pow(u, 5) + 7 * std::pow(u, 6));
      return Gd / (r * r);
    };
    const double g0 = cfg->cloud_shape == PMGB_S1 ? 8 * Gd / (ad * ad * ad) : 448 * Gd / (35 * ad * ad * ad);
    for (int i = 0; i < 500; ++i) {
      const double r = std::sqrt(i * d2);
      q->table_h[500 + i] = (float)(i == 0 ? g0 : Rd(r) / r);
    }
  }
  q->pp.re2 = re * re;
  q->pp.re = re;
  q->pp.inv_d2 = 1.0f / q->delta2;
  q->pp.use_table = cfg->use_table;
  q->pp.ysort = cfg->y_sorting;
  q->pp.shape = cfg->cloud_shape;
  q->pp.a = a;
  q->pp.eps2 = eps * eps;
  const size_t ntot = (size_t)q->nsub + 1;  // sub-columns + the bucket outside the mesh
  int rc;
  // slices of sub-columns (32 particles for pair counting / the direct formula, 64 for the
  // table pass, which takes each slice once per neighbour cell), the table pass's list of heavy
  // units, and its 27 partial-force slots per particle
  q->nitems_max = (int)((size_t)pm->n / 32 + ntot + 32);
  if ((rc = dalloc(&q->cell_start, ntot + 1)) || (rc = dalloc(&q->item_cnt, ntot)) ||
      (rc = dalloc(&q->item_off, ntot)) || (rc = dalloc(&q->nitems, 1)) || (rc = dalloc(&q->counter, (size_t)slot_counter_words())) ||
      (rc = dalloc(&q->scan_tmp, (size_t)scan_scratch_words((int)ntot))) ||
      (rc = dalloc(&q->items, (size_t)q->nitems_max)) ||
      (rc = dalloc(&q->heavy, (size_t)slot_heavy_capacity(q->nitems_max))) ||
      (rc = dalloc(&q->table, 1000)) || (rc = dalloc(&q->npairs, 1)) ||
      (rc = dalloc(&q->slots, 27 * (size_t)std::max(pm->n, 1)))) {
    pmgb_p3m_destroy(q);
    return rc;
  }
  // the symmetric part of the pair pass (y-sorted lists): 27 sub^2 slots per particle (3.9, 6.9
  // or 10.8 KB), the mask words per sub-column, the unit list; left off if it would take more
  // than a quarter of the free device memory or the allocation fails
  bool pads_vanish = true;  // exact mode: the symmetric part's padded candidates add exactly 0
  if (!cfg->use_table && cfg->softening == 0.f && (rc = exact_mode_pads_vanish(pm->st, &pads_vanish))) {
    pmgb_p3m_destroy(q);
    return rc;
  }
  if (sym_supported(q->cd.sub) && pm->n > 0 && pads_vanish) {
    const size_t n = (size_t)pm->n, nslot = 27 * (size_t)q->cd.sub * q->cd.sub;
    q->sym.cap = (u32)sym_unit_capacity(q->nsub, pm->n, q->cd.sub);
    void* ptr[4] = {nullptr, nullptr, nullptr, nullptr};
    const size_t bytes[4] = {nslot * n * sizeof(float4), ((size_t)q->nsub + 1) * sym_mask_words(q->cd.sub) * sizeof(u32),
                             3 * (size_t)q->sym.cap * sizeof(uint2), n * sizeof(int)};
    size_t free_b = 0, total_b = 0;
    bool ok = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
              bytes[0] + bytes[1] + bytes[2] + bytes[3] <= free_b / 4;
    for (int i = 0; i < 4 && ok; ++i)
      if (cudaMalloc(&ptr[i], bytes[i]) != cudaSuccess) {
        ptr[i] = nullptr;
        ok = false;
      }
    if (ok) {
      q->sym.slots = (float4*)ptr[0];
      q->sym.masks = (u32*)ptr[1];
      q->sym.units = (uint2*)ptr[2];
      q->sym.subcol = (int*)ptr[3];
      q->sym.enabled = 1;
    } else {
      for (void* p : ptr)
        if (p) cudaFree(p);
      cudaGetLastError();
      q->sym = SymPass{};
    }
  }
  if (cudaMemcpyAsync(q->table, q->table_h, 1000 * sizeof(float), cudaMemcpyHostToDevice, pm->st) != cudaSuccess ||
      cudaMemsetAsync(q->npairs, 0, sizeof(unsigned long long), pm->st) != cudaSuccess ||
      cudaStreamSynchronize(pm->st) != cudaSuccess) {
    pmgb_p3m_destroy(q);
    return set_error("P3M table upload failed"), PMGB_ECUDA;
  }
  if (attach) pm->p3m = q;
  *out = q;
  return PMGB_OK;
}
}  // namespace pmgb

extern "C" {

int pmgb_p3m_destroy(pmgb_p3m* q) {
  if (!q) return PMGB_OK;
  if (q->pm) {
    cudaStreamSynchronize(q->pm->st);
    if (q->pm->p3m == q) q->pm->p3m = nullptr;
    q->pm->since_sort = 1 << 30;
  }
  void* ptrs[] = {q->cell_start, q->item_cnt, q->item_off, q->scan_tmp, q->nitems, q->counter, q->items, q->table,
                  q->npairs, q->slots, q->heavy, q->sym.slots, q->sym.masks, q->sym.units, q->sym.subcol};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete q;
  return PMGB_OK;
}

int pmgb_p3m_force(pmgb_p3m* q) {
  if (!q) return set_error("null handle"), PMGB_EINVAL;
  return pmgb_pm_method_step(q->pm);
}

int pmgb_p3m_run(pmgb_p3m* q, int sim_length, int* steps_done) {
  if (!q) return set_error("null handle"), PMGB_EINVAL;
  return pmgb_pm_run(q->pm, sim_length, steps_done);
}

int pmgb_p3m_get_cell_lists(pmgb_p3m* q, int* order, int* counts, int* dims3) {
  if (!q) return set_error("null handle"), PMGB_EINVAL;
  if (dims3) {
    dims3[0] = q->cd.Mx;
    dims3[1] = q->cd.My;
    dims3[2] = q->cd.Mz;
  }
  if (!order && !counts) return PMGB_OK;
  pmgb_pm* h = q->pm;
  const int n = h->n;
  const int sub2 = q->cd.sub * q->cd.sub;
  std::vector<int> cs(q->nsub + 2);
  std::vector<float4> hv(n), hp(n);
  PMGB_CUDA_TRY(cudaMemcpyAsync(cs.data(), q->cell_start, cs.size() * sizeof(int), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(hv.data(), h->vi[h->cur], n * sizeof(float4), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(hp.data(), h->pm[h->cur], n * sizeof(float4), cudaMemcpyDeviceToHost, h->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(h->st));
  if (counts)
    for (int c = 0; c < q->ncells; ++c) counts[c] = cs[(c + 1) * sub2] - cs[c * sub2];
  if (order) {
    // A cell's particles are stored sub-column by sub-column; the reference's list
    // (fillWithYSorting) is the whole cell by ascending y, ties by index, which is the order of
    // the device sort key (y as an order-preserving integer, -0 folded onto +0) then the id.
    auto ykey = [](float y) {
      uint32_t u;
      std::memcpy(&u, &y, 4);
      if (u == 0x80000000u) u = 0;
      return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    };
    std::vector<std::pair<uint64_t, int>> tmp;
    int k = 0;
    for (int c = 0; c < q->ncells; ++c) {
      tmp.clear();
      for (int s = cs[c * sub2]; s < cs[(c + 1) * sub2]; ++s) {
        int id;
        std::memcpy(&id, &hv[s].w, 4);
        tmp.emplace_back(((uint64_t)ykey(hp[s].y) << 32) | (uint32_t)id, id);
      }
      if (q->cfg.y_sorting) std::sort(tmp.begin(), tmp.end());
      for (auto& t : tmp) order[k++] = t.second;
    }
  }
  return PMGB_OK;
}

int pmgb_p3m_set_pair_counting(pmgb_p3m* q, int enable) {
  if (!q) return set_error("null handle"), PMGB_EINVAL;
  q->count_pairs = enable ? 1 : 0;
  return PMGB_OK;
}

int pmgb_p3m_set_symmetric(pmgb_p3m* q, int enable) {
  if (!q) return set_error("null handle"), PMGB_EINVAL;
  q->sym.enabled = enable && q->sym.slots ? 1 : 0;
  return PMGB_OK;
}

int pmgb_p3m_get_symmetric(pmgb_p3m* q, int* enabled, unsigned int* units_last_pass) {
  if (!q || !enabled) return set_error("null argument"), PMGB_EINVAL;
  *enabled = q->sym.enabled;
  if (units_last_pass) {
    PMGB_CUDA_TRY(cudaMemcpyAsync(units_last_pass, q->counter + kSlotSymTotalWord, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                  q->pm->st));
    PMGB_CUDA_TRY(cudaStreamSynchronize(q->pm->st));
  }
  return PMGB_OK;
}

int pmgb_p3m_get_subcolumns(const pmgb_p3m* q, int* per_axis) {
  if (!q || !per_axis) return set_error("null argument"), PMGB_EINVAL;
  *per_axis = q->cd.sub;
  return PMGB_OK;
}

int pmgb_p3m_pair_count(pmgb_p3m* q, unsigned long long* ordered_pairs) {
  if (!q || !ordered_pairs) return set_error("null argument"), PMGB_EINVAL;
  PMGB_CUDA_TRY(cudaMemcpyAsync(ordered_pairs, q->npairs, sizeof(unsigned long long), cudaMemcpyDeviceToHost, q->pm->st));
  PMGB_CUDA_TRY(cudaStreamSynchronize(q->pm->st));
  return PMGB_OK;
}

int pmgb_p3m_get_sr_table(pmgb_p3m* q, float* table500, float* delta_sq) {
  if (!q) return set_error("null handle"), PMGB_EINVAL;
  if (table500) std::memcpy(table500, q->table_h, 500 * sizeof(float));
  if (delta_sq) *delta_sq = q->delta2;
  return PMGB_OK;
}

}  // extern "C"
