// recorder.cu - the reference's StateRecorder output (source/stateRecorder.cpp:5-137) from a
// run on the device.
//
// Files, byte for byte the reference's formats (so its scripts, e.g. script/load_data.py,
// read them unchanged):
//   positions.dat / field.dat   int32 N, int32 frames (the count given at construction), then
//                               per recorded iteration N float32 xyz triplets in the particles'
//                               original order (positions in original units; field = the
//                               acceleration of the iteration in original units, H a / DT^2)
//   energy.txt                  "pe ke" per iteration, std::to_string of the float values
//   momentum.txt, expected_momentum.txt, angular_momentum.txt
//                               "%.6e %.6e %.6e" per iteration (Vec3::toString)
// An empty file name leaves that output out.
//
// GB300 path.  Every iteration of a recorded run packs its frame (positions, and the field when
// asked) in original order into a device buffer of K frames; when a buffer is full it is copied
// to pinned host memory on the run's stream and a writer thread appends it to the files once
// the copy's event completes, while the device fills the other buffer.  No synchronisation of
// the run loop per frame; the host waits only if the writer falls two buffers behind.  The
// energy and momentum lines come from the FP64 run diagnostics (diag.cu), rounded to float and
// printed as the reference prints its float sums.
#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <filesystem>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "handles.cuh"

struct pmgb_recorder {
  int n = 0;
  int frames = 0;
  std::string dir;
  std::string names[6];  // positions, energy, momentum, expected momentum, angular momentum, field
  FILE* fpos = nullptr;
  FILE* ffield = nullptr;
  std::string text[4];  // energy, momentum, expected momentum, angular momentum
  // device frame buffers (K frames of n xyz positions, then n xyz fields) and their counts
  int K = 0;
  int with_field = 0;
  float* dbuf[2] = {nullptr, nullptr};
  int* dcount[2] = {nullptr, nullptr};
  float* hbuf[2] = {nullptr, nullptr};
  int* hcount[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int cur = 0;
  int slot = 0;
  bool busy[2] = {false, false};
  // writer thread
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int> queue;
  bool quit = false;
  std::string werr;
  long long frames_written = 0;
};

namespace pmgb {

namespace {

__global__ void pack_frame_kernel(const float4* __restrict__ pm, const float4* __restrict__ vi,
                                  const float4* __restrict__ acc, int n, float H, float DT,
                                  int with_field, float* __restrict__ frame,
                                  int* __restrict__ count, const int* __restrict__ stop, int tag) {
  if (stop[0] && stop[1] < tag) return;  // an earlier iteration escaped: nothing recorded
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0) atomicAdd(count, 1);
  if (k >= n) return;
  const float4 p = pm[k];
  const int i = __float_as_int(vi[k].w);
  if (i < 0 || i >= n) return;
  // positionToOriginalUnits H * x (include/unitConversions.h:11-13)
  frame[3 * i] = __fmul_rn(H, p.x);
  frame[3 * i + 1] = __fmul_rn(H, p.y);
  frame[3 * i + 2] = __fmul_rn(H, p.z);
  if (with_field) {  // accelerationToOriginalUnits H * a / (DT * DT) (unitConversions.h:27-29)
    const float4 a = acc[k];
    const float dt2 = __fmul_rn(DT, DT);
    float* f = frame + 3 * (size_t)n;
    f[3 * i] = __fdiv_rn(__fmul_rn(H, a.x), dt2);
    f[3 * i + 1] = __fdiv_rn(__fmul_rn(H, a.y), dt2);
    f[3 * i + 2] = __fdiv_rn(__fmul_rn(H, a.z), dt2);
  }
}

size_t frame_floats(const pmgb_recorder* r) { return (size_t)3 * r->n * (r->with_field ? 2 : 1); }

void writer_loop(pmgb_recorder* r) {
  for (;;) {
    int b;
    {
      std::unique_lock<std::mutex> lk(r->mu);
      r->cv.wait(lk, [&] { return r->quit || !r->queue.empty(); });
      if (r->queue.empty()) return;
      b = r->queue.front();
      r->queue.pop_front();
    }
    std::string err;
    if (cudaEventSynchronize(r->ev[b]) != cudaSuccess) {
      err = "frame copy failed";
    } else {
      const int cnt = std::min(*r->hcount[b], r->K);
      const size_t ff = frame_floats(r), np = (size_t)3 * r->n;
      for (int f = 0; f < cnt && err.empty(); ++f) {
        const float* base = r->hbuf[b] + (size_t)f * ff;
        if (r->fpos && std::fwrite(base, sizeof(float), np, r->fpos) != np) err = "positions write failed";
        if (r->ffield && r->with_field && std::fwrite(base + np, sizeof(float), np, r->ffield) != np)
          err = "field write failed";
      }
      r->frames_written += cnt;
    }
    {
      std::lock_guard<std::mutex> lk(r->mu);
      r->busy[b] = false;
      if (!err.empty() && r->werr.empty()) r->werr = err;
    }
    r->cv.notify_all();
  }
}

// Hands the current device buffer to the writer (copy + event on the run's stream) and makes
// the other one current, waiting for the writer if that one is still being written.
int swap_buffers(pmgb_recorder* r, cudaStream_t st) {
  const int b = r->cur;
  {
    // the pinned buffer of b must be free before the copy into it is queued
    std::unique_lock<std::mutex> lk(r->mu);
    r->cv.wait(lk, [&] { return !r->busy[b]; });
    r->busy[b] = true;
  }
  PMGB_CUDA_TRY(cudaMemcpyAsync(r->hbuf[b], r->dbuf[b], (size_t)r->slot * frame_floats(r) * sizeof(float),
                                cudaMemcpyDeviceToHost, st));
  PMGB_CUDA_TRY(cudaMemcpyAsync(r->hcount[b], r->dcount[b], sizeof(int), cudaMemcpyDeviceToHost, st));
  PMGB_CUDA_TRY(cudaEventRecord(r->ev[b], st));
  {
    std::lock_guard<std::mutex> lk(r->mu);
    r->queue.push_back(b);
  }
  r->cv.notify_all();
  r->cur = 1 - b;
  r->slot = 0;
  // the device counter of the new buffer restarts (ordered after the earlier copy of it)
  PMGB_CUDA_TRY(cudaMemsetAsync(r->dcount[r->cur], 0, sizeof(int), st));
  return PMGB_OK;
}

void wait_writer(pmgb_recorder* r) {
  std::unique_lock<std::mutex> lk(r->mu);
  r->cv.wait(lk, [&] { return r->queue.empty() && !r->busy[0] && !r->busy[1]; });
}

// std::to_string(float) and Vec3::toString of the reference
std::string fmt_f(double v) { return std::to_string((float)v); }
std::string fmt_e3(const double* v) {
  char buf[160];
  std::snprintf(buf, sizeof buf, "%.6e %.6e %.6e", (double)(float)v[0], (double)(float)v[1],
                (double)(float)v[2]);
  return buf;
}

void free_recorder(pmgb_recorder* r) {
  if (!r) return;
  if (r->th.joinable()) {
    {
      std::lock_guard<std::mutex> lk(r->mu);
      r->quit = true;
    }
    r->cv.notify_all();
    r->th.join();
  }
  for (int b = 0; b < 2; ++b) {
    if (r->dbuf[b]) cudaFree(r->dbuf[b]);
    if (r->dcount[b]) cudaFree(r->dcount[b]);
    if (r->hbuf[b]) cudaFreeHost(r->hbuf[b]);
    if (r->hcount[b]) cudaFreeHost(r->hcount[b]);
    if (r->ev[b]) cudaEventDestroy(r->ev[b]);
  }
  if (r->fpos) std::fclose(r->fpos);
  if (r->ffield) std::fclose(r->ffield);
  delete r;
}

FILE* open_binary(const pmgb_recorder* r, const std::string& name) {
  if (name.empty()) return nullptr;
  const std::string path = (std::filesystem::path(r->dir) / name).string();
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return nullptr;
  const int hdr[2] = {r->n, r->frames};
  std::fwrite(hdr, sizeof(int), 2, f);
  return f;
}

}  // namespace

int rec_begin_run(pmgb_pm* h, int record_field) {
  pmgb_recorder* r = h->rec;
  if (!r) return PMGB_OK;
  if (r->n != h->n) return set_error("recorder particle count differs from the method's"), PMGB_EINVAL;
  if (record_field && !r->with_field) return set_error("recorder was created without a field buffer"), PMGB_EINVAL;
  r->slot = 0;
  PMGB_CUDA_TRY(cudaMemsetAsync(r->dcount[r->cur], 0, sizeof(int), h->st));
  return PMGB_OK;
}

int rec_after_drift(pmgb_pm* h, int tag) {
  pmgb_recorder* r = h->rec;
  if (!r) return PMGB_OK;
  float* frame = r->dbuf[r->cur] + (size_t)r->slot * frame_floats(r);
  const int blocks = std::max(1, (h->n + 255) / 256);
  pack_frame_kernel<<<blocks, 256, 0, h->st>>>(h->pm[h->cur], h->vi[h->cur], h->acc, h->n, h->cfg.H,
                                               h->cfg.DT, h->rec_field, frame, r->dcount[r->cur],
                                               h->flags, tag);
  PMGB_LAUNCH_CHECK();
  count_launches(1);
  if (++r->slot == r->K) return swap_buffers(r, h->st);
  return PMGB_OK;
}

int rec_end_run(pmgb_pm* h, int with_diagnostics) {
  pmgb_recorder* r = h->rec;
  if (!r) return PMGB_OK;
  if (r->slot > 0) {
    int rc = swap_buffers(r, h->st);
    if (rc) return rc;
  }
  if (with_diagnostics) {
    int taken = 0;
    int rc = pmgb_pm_get_diagnostics(h, nullptr, 0, &taken);
    if (rc) return rc;
    std::vector<double> rec((size_t)std::max(taken, 1) * PMGB_DIAG_WIDTH);
    rc = pmgb_pm_get_diagnostics(h, rec.data(), taken, &taken);
    if (rc) return rc;
    for (int k = 0; k < taken; ++k) {
      const double* d = rec.data() + (size_t)k * PMGB_DIAG_WIDTH;
      r->text[0] += fmt_f(d[PMGB_DIAG_POTENTIAL]) + ' ' + fmt_f(d[PMGB_DIAG_KINETIC]) + '\n';
      r->text[1] += fmt_e3(d + PMGB_DIAG_MOMENTUM) + '\n';
      r->text[2] += fmt_e3(d + PMGB_DIAG_EXPECTED_MOMENTUM) + '\n';
      r->text[3] += fmt_e3(d + PMGB_DIAG_ANGULAR_MOMENTUM) + '\n';
    }
  }
  return PMGB_OK;
}

}  // namespace pmgb

using namespace pmgb;

extern "C" {

int pmgb_recorder_create(int n, int frames, const char* output_dir, const char* const* names,
                         int with_field, pmgb_recorder** out) {
  if (!out) return set_error("null output handle"), PMGB_EINVAL;
  *out = nullptr;
  if (n < 0 || frames < 0 || !output_dir) return set_error("bad recorder arguments"), PMGB_EINVAL;
  pmgb_recorder* r = new pmgb_recorder();
  r->n = n;
  r->frames = frames;
  r->dir = output_dir;
  static const char* defaults[6] = {"positions.dat", "energy.txt", "momentum.txt",
                                    "expected_momentum.txt", "angular_momentum.txt", "field.dat"};
  for (int k = 0; k < 6; ++k) r->names[k] = names ? (names[k] ? names[k] : "") : defaults[k];
  r->with_field = with_field ? 1 : 0;
  std::error_code ec;
  std::filesystem::create_directories(r->dir, ec);
  r->fpos = open_binary(r, r->names[0]);
  r->ffield = open_binary(r, r->names[5]);
  if ((!r->names[0].empty() && !r->fpos) || (!r->names[5].empty() && !r->ffield)) {
    free_recorder(r);
    return set_error("cannot open the recorder's output files"), PMGB_EINVAL;
  }
  // K frames per device buffer: about 128 MB per buffer, at most 64 frames
  const size_t fb = frame_floats(r) * sizeof(float);
  r->K = (int)std::max<size_t>(1, std::min<size_t>(64, fb ? ((size_t)128 << 20) / fb : 64));
  for (int b = 0; b < 2; ++b) {
    const size_t bytes = std::max<size_t>(1, (size_t)r->K * fb);
    if (cudaMalloc((void**)&r->dbuf[b], bytes) != cudaSuccess || cudaMalloc((void**)&r->dcount[b], sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void**)&r->hbuf[b], bytes) != cudaSuccess ||
        cudaMallocHost((void**)&r->hcount[b], sizeof(int)) != cudaSuccess ||
        cudaEventCreateWithFlags(&r->ev[b], cudaEventDisableTiming) != cudaSuccess ||
        cudaMemset(r->dcount[b], 0, sizeof(int)) != cudaSuccess) {
      free_recorder(r);
      return set_error("recorder buffer allocation failed"), PMGB_ENOMEM;
    }
  }
  r->th = std::thread(writer_loop, r);
  *out = r;
  return PMGB_OK;
}

int pmgb_recorder_flush(pmgb_recorder* r, char* dir_out, int cap) {
  if (!r) return set_error("null handle"), PMGB_EINVAL;
  wait_writer(r);
  if (r->fpos) std::fflush(r->fpos);
  if (r->ffield) std::fflush(r->ffield);
  for (int k = 0; k < 4; ++k) {
    const std::string& name = r->names[1 + k];
    if (name.empty()) continue;
    const std::string path = (std::filesystem::path(r->dir) / name).string();
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return set_error("cannot write " + path), PMGB_EINVAL;
    std::fwrite(r->text[k].data(), 1, r->text[k].size(), f);
    std::fclose(f);
  }
  if (dir_out && cap > 0) {
    std::strncpy(dir_out, r->dir.c_str(), (size_t)cap - 1);
    dir_out[cap - 1] = '\0';
  }
  std::lock_guard<std::mutex> lk(r->mu);
  if (!r->werr.empty()) return set_error(r->werr), PMGB_EINVAL;
  return PMGB_OK;
}

int pmgb_recorder_frames_written(pmgb_recorder* r, long long* frames) {
  if (!r || !frames) return set_error("null argument"), PMGB_EINVAL;
  wait_writer(r);
  *frames = r->frames_written;
  return PMGB_OK;
}

int pmgb_recorder_destroy(pmgb_recorder* r) {
  if (!r) return PMGB_OK;
  wait_writer(r);
  free_recorder(r);
  return PMGB_OK;
}

}  // extern "C"
