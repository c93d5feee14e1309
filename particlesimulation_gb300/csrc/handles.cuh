// handles.cuh - the handle structures behind the C ABI and the launchers shared between
// translation units.
#pragma once
#include "common.cuh"

namespace pmgb {

int radix_hist_blocks(int n);
size_t radix_hist_words(int n);  // size of radix_sort_pairs' hist buffer
int radix_sort_pairs(u64** keys, u32** vals, u64** keys_alt, u32** vals_alt, u32* hist, int n,
                     int nbits, cudaStream_t st);
int scan_scratch_words(int n);   // size of exclusive_scan's scratch buffer
int slot_heavy_capacity(int nitems_max);  // entries of the pair pass's heavy-unit list
int slot_counter_words();                 // words of the pair pass's counter buffer
int exclusive_scan(const u32* in, u32* out, int n, u32* total, u32* scratch, cudaStream_t st);
int launch_chain_keys(const float4* pm, const float4* vi, int n, ChainDims c, int ysort,
                      const int* stop, u64* keys, u32* vals, cudaStream_t st);
int launch_fix_ties(const u64* keys, u32* vals, const float4* vi, int n, const int* stop,
                    cudaStream_t st);
int launch_brick_keys(const float4* pm, int n, MeshDims m, int bshift, const int* stop, u64* keys,
                      u32* vals, cudaStream_t st);
int launch_gather(const u64* keys, const u32* vals, int n, const float4* pm_in,
                  const float4* vi_in, float4* pm_out, float4* vi_out, int* cell_start,
                  int ncells_total, const int* stop, cudaStream_t st);
int launch_deposit(int is, const float4* pm, int n, MeshDims m, float scale, u64* rho,
                   const int* stop, cudaStream_t st);
int fft_configure(const MeshDims& m);
int launch_poisson(u64* rho, float2* spec, float* phi, const float* ghat, const float2* tw,
                   int nmax, MeshDims m, float fx_inv, const int* stop, cudaStream_t st,
                   float* rho_copy = nullptr);
int launch_green(float* ghat, MeshDims m, int gf, int is, int fds, double a, cudaStream_t st);
// m_code / m_orig in the float arithmetic of the reference's massToCodeUnits (api.cu)
float mass_code_factor(float H, float DT, float G);
// Mixed-radix Poisson solve for meshes whose sides are not powers of two in [8, 512] (gfft.cu):
// plans (twiddle tables per axis) made once per handle; data = a full complex mesh.
bool gfft_supported(int n);
int gfft_plans_create(const int dims[3], void** out);
void gfft_plans_destroy(void* plans);
int launch_poisson_generic(u64* rho, float2* data, float* phi, const float* ghat, void* plans,
                           MeshDims m, float fx_inv, const int* stop, cudaStream_t st,
                           float* rho_copy);
int launch_interp(bool kdk, float4* pm, float4* vi, float4* acc, int n, const float* phi,
                  const StepParams& sp, float kick, int drift, int* stop, cudaStream_t st);
int launch_kick_drift(float4* pm, float4* vi, const float4* acc, int n, const StepParams& sp,
                      float kick, int drift, int* stop, cudaStream_t st);
int launch_unpack(const float4* pm, const float4* vi, const float4* acc, int n, float H, float DT,
                  int orig, float* pos, float* vel, float* aout, cudaStream_t st);
int launch_pack(const float* pos, const float* vel, const float* mass_code, int n, float H,
                float DT, int orig, float4* pm, float4* vi, cudaStream_t st);
// Buffers of the pair pass's symmetric part (pair.cu): dense sub-column pairs below a cost
// bound are evaluated once per pair, each side's partial force going to a slot of its own
// (direction, neighbour sub-column); the rest stays one-sided.
struct SymPass {
  float4* slots = nullptr;  // 27 L x n partial accelerations (L = sub-columns per cell), slot =
                            // direction * L + sub-column
  u32* masks = nullptr;     // sym_mask_words(sub) per sub-column (nsub + 1): slots used, dead directions
  uint2* units = nullptr;   // 3 cap: staged units (cap x 16 B), then the list (i side, j side)
  u32 cap = 0;              // units a pass can list
  int* subcol = nullptr;    // sub-column of each particle (sorted order)
  int enabled = 0;          // the handle's switch (pmgb_p3m_set_symmetric)
};
int sym_unit_capacity(int nsub, int n, int sub);
constexpr int kSlotSymTotalWord = 28;  // counter word of the symmetric units a pass listed
int sym_mask_words(int sub);  // mask words per sub-column with sub x sub sub-columns per cell
bool sym_supported(int sub);  // sub-column counts the symmetric part is built for
int exact_mode_pads_vanish(cudaStream_t st, bool* vanish);  // the symmetric part's exact-mode condition

int launch_pair(const float4* pm, const float4* vi, const float4* acc_pm, const int* cell_start,
                const ChainDims& cd, u32* item_cnt, u32* item_off, u32* scan_tmp, u32* nitems, int2* items,
                int nitems_max, u32* heavy, u32* counter, const PairParams& pp, const float* table,
                const StepParams& sp, float kick, int drift, int kdk, float4* pm_out, float4* vi_out,
                float4* acc_out, unsigned long long* npairs, int* stop, int num_sms, cudaEvent_t ev_pair,
                cudaStream_t st, int equal_mass, float4* slots, int n, int unit_stride = 1,
                const SymPass* sym = nullptr);
// Sampled pair passes (unit_stride > 1, slotted passes only: pair_pass_sampleable): flags[id] = 1
// for the particles of the slices such a pass covered (original index order).
bool pair_pass_sampleable(const PairParams& pp);
int launch_mark_sampled(const int* cell_start, const int2* items, const u32* nitems, int nitems_max,
                        int unit_stride, const float4* vi, unsigned char* flags, cudaStream_t st);

}  // namespace pmgb

namespace pmgb {
// word of pmgb_pm::flags that a kernel sets when a bounded device wait gave up (the run then
// returns PMGB_ETIMEOUT)
constexpr int kFlagTimeout = 2;
}  // namespace pmgb

struct pmgb_p3m;
struct pmgb_closure;
struct pmgb_diag;
struct pmgb_recorder;

struct pmgb_pm {
  pmgb_pm_config cfg{};
  int n = 0;
  pmgb::MeshDims m{};
  pmgb::StepParams sp{};
  cudaStream_t st = nullptr;
  int num_sms = 0;
  float4* pm[2] = {nullptr, nullptr};
  float4* vi[2] = {nullptr, nullptr};
  float4* acc = nullptr;
  float4* acc_pm = nullptr;
  int cur = 0;
  pmgb::u64 *keys = nullptr, *keys_alt = nullptr;
  pmgb::u32 *vals = nullptr, *vals_alt = nullptr, *hist = nullptr;
  pmgb::u64* rho = nullptr;
  float2* spec = nullptr;
  float* phi = nullptr;
  float* ghat = nullptr;
  float2* tw = nullptr;
  int nmax = 0;
  int* flags = nullptr;  // device: [0] stop, [1] escape iteration, [kFlagTimeout] a wait gave up
  pmgb_p3m* p3m = nullptr;
  pmgb_closure* closure = nullptr;  // learned short-range closure applied after interpolation
  int since_sort = 1 << 30;
  cudaEvent_t ev[6] = {};
  float stage_ms[5] = {0, 0, 0, 0, 0};
  float* stage = nullptr;      // 9 n floats: positions, velocities, accelerations (original order)
  float* mass_code = nullptr;  // n floats, code-unit masses in original order
  pmgb_diag* diag = nullptr;   // run diagnostics (diag.cu), null when off
  int equal_mass = 0;          // every particle has the same mass (pair pass folds it)
  pmgb_recorder* rec = nullptr;  // recorder of the current pmgb_pm_run_recorded, else null
  int rec_field = 0;
  float4* ivel = nullptr;  // integer-step velocities, original order (pmgb_pm_leapfrog), lazily
  // the closure mode whose force h->acc holds at the current positions (-1: none; 3: no closure)
  int acc_mode = -1;
  bool generic = false;    // mesh not all powers of two in [8, 512]: mixed-radix Poisson solve
  void* gplans = nullptr;  // its plans (gfft.cu)
};

struct pmgb_p3m {
  pmgb_pm* pm = nullptr;
  pmgb_p3m_config cfg{};
  pmgb::ChainDims cd{};
  int ncells = 0;
  int nsub = 0;               // sub-columns: ncells * cd.sub^2
  int* cell_start = nullptr;  // nsub + 2: sub-column starts, the bucket outside the mesh, n
  pmgb::u32 *item_cnt = nullptr, *item_off = nullptr, *nitems = nullptr, *counter = nullptr;
  pmgb::u32* scan_tmp = nullptr;  // scratch of the item-count scan (scan_scratch_words)
  int2* items = nullptr;
  int nitems_max = 0;             // capacity of items
  pmgb::u32* heavy = nullptr;     // heavy units of the table pass (slot_heavy_capacity entries)
  float* table = nullptr;
  float table_h[1000];  // [0, 500): initSRForceTable; [500, 1000): R(r)/r for the exact mode
  float delta2 = 0;
  pmgb::PairParams pp{};
  unsigned long long* npairs = nullptr;
  int count_pairs = 0;  // count in-range pairs during force evaluations (pmgb_p3m_set_pair_counting)
  float4* slots = nullptr;  // 27 x n partial short-range accelerations (pair.cu, table pass)
  int unit_stride = 1;      // > 1: the next passes cover every unit_stride-th slice only (judge)
  pmgb::SymPass sym{};      // symmetric sub-column pairs (y-sorted lists only)
};

namespace pmgb {
// Adds the closure's predicted residual short-range acceleration to h->acc_pm (sorted order of
// h->pm[h->cur]); defined in closure.cu.
int closure_apply(pmgb_pm* h);
// The closure mode of h's force evaluations (PMGB_CLOSURE_*), 3 without a closure (closure.cu).
int closure_mode(const pmgb_pm* h);
// P3M handle over pm; attach = make it pm's pair pass (api.cu).
int p3m_create_internal(pmgb_pm* pm, const pmgb_p3m_config* cfg, pmgb_p3m** out, bool attach);

// Run diagnostics (diag.cu).  diag_density: the float density buffer the Poisson solve fills
// while diagnostics are on (else null).  diag_run_begin: the start of a run (records cleared,
// expected momentum = current momentum).  diag_after_drift: one record of the state just
// drifted by the iteration tagged `tag`; skipped on device if an earlier iteration escaped.
// diag_before_drift: makes sure the density of the current positions is available for the
// next record (advance() starts with a drift whose force may predate the diagnostics).
float* diag_density(pmgb_pm* h);
int diag_run_begin(pmgb_pm* h);
int diag_before_drift(pmgb_pm* h);
int diag_after_drift(pmgb_pm* h, int tag);
void diag_free(pmgb_pm* h);
int diag_capacity(const pmgb_pm* h);
// The records' running state (expected momentum, record count: 28 bytes into the device buffer
// `save`) saved before a step and put back to take the step again (the density then recomputed).
int diag_save(pmgb_pm* h, unsigned char* save);
int diag_restore(pmgb_pm* h, const unsigned char* save);

// StateRecorder output (recorder.cu): frame of the iteration tagged `tag`, run start / end.
int rec_begin_run(pmgb_pm* h, int record_field);
int rec_after_drift(pmgb_pm* h, int tag);
int rec_end_run(pmgb_pm* h, int with_diagnostics);
}  // namespace pmgb
