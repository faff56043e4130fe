// gb_internal.h -- host-side state shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/itk_gb300.h"

namespace gb {

struct EvalConsts;  // per-evaluation transform constants (gb_kernels.cuh)

// Image geometry (start index 0, x fastest), as ImageBase holds it.
struct Geom {
  int64_t size[3] = {0, 0, 0};
  double spacing[3] = {1, 1, 1};
  double origin[3] = {0, 0, 0};
  double dir[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  double i2p[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // direction * diag(spacing)
  double p2i[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // inverse of i2p
  bool set = false;
  int64_t voxels() const { return size[0] * size[1] * size[2]; }
};

int geom_init(Geom& g, const int64_t size[3], const double spacing[3], const double origin[3], const double dir[9]);

// Owning device buffer from the stream-ordered allocator: allocated and freed
// in the order of the stream it is bound to, so growing or dropping a buffer
// never waits for the whole device (a plain cudaFree does, stalling every other
// stream -- other registrations' iterations included).  Without a stream:
// cudaMalloc / cudaFree.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t st = nullptr;
  bool ordered = false;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) {
      if (ordered) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    reset();
    ordered = false;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
  // stream-ordered: usable on `stream` at once, on other streams once `stream` has been synchronized
  cudaError_t alloc_on(cudaStream_t stream, size_t count) {
    if (count <= n && p) return cudaSuccess;
    reset();
    st = stream;
    ordered = true;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), stream);
    if (e == cudaSuccess) n = count;
    else p = nullptr;
    return e;
  }
};

cudaError_t sort_pairs_u64(const uint64_t* keys_in, uint64_t* keys_out, const uint32_t* vals_in, uint32_t* vals_out,
                           int64_t n, int end_bit, cudaStream_t stream);

// Per-thread last-error text (gb_last_error()).  While an entry point that takes a
// metric handle runs, an ErrorScope names that handle, and fail() records the text
// on the handle as well (gb_metric_last_error).  The scope is also an NVTX range
// named after the entry point, so a timeline (Nsight Systems, ncu's NVTX filters)
// shows every C-ABI call; without an attached tool a range costs a few nanoseconds.
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
gb_metric* error_scope();
void set_error_scope(gb_metric* m);

struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

struct ErrorScope {
  gb_metric* prev;
  NvtxRange range;
  ErrorScope(gb_metric* m, const char* name) : prev(error_scope()), range(name) { set_error_scope(m); }
  ~ErrorScope() { set_error_scope(prev); }
  ErrorScope(const ErrorScope&) = delete;
  ErrorScope& operator=(const ErrorScope&) = delete;
};

// Device image filters (gb_filters.cu).
int smooth_rg_device(cudaStream_t st, const float* in, float* out, float* t1, float* t2, const int64_t size[3],
                     const double spacing[3], const double sigma[3]);
int gradient_rg_device(cudaStream_t st, const float* in, const int64_t size[3], const double spacing[3],
                       const double direction[9], double sigma, bool normalize_across_scale, bool use_direction,
                       float4* out4, float* out3);
void shrink_geometry(const int64_t size[3], const double spacing[3], const double origin[3], const double dir[9],
                     const int64_t factors[3], int64_t out_size[3], double out_spacing[3], double out_origin[3]);

struct OptState;  // device optimizer state (gb_optimizer.cu)

// body(k0, k1) over [0, n) split across the host's threads (at most 16, at least
// `grain` items each); the caller's thread runs whatever no new thread could take.
inline unsigned host_threads() {
  static const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));  // queried once
  return hw;
}

template <typename F>
void parallel_ranges(int64_t n, F body, int64_t grain = 16384) {
  if (n < 2 * grain) {  // small: no thread, no query
    body(0, n);
    return;
  }
  const int64_t T = std::max<int64_t>(1, std::min<int64_t>(host_threads(), n / grain));
  if (T == 1) {
    body(0, n);
    return;
  }
  std::vector<std::thread> th;
  int64_t started = 0;
  try {
    for (; started < T; ++started) th.emplace_back(body, n * started / T, n * (started + 1) / T);
  } catch (...) {  // no more threads: the rest runs here
  }
  for (std::thread& x : th) x.join();
  if (started < T) body(n * started / T, n);
}

// memcpy split across the host's threads for large buffers (a displacement
// field's parameters and derivative are tens to hundreds of MB per call).
inline void copy_parallel(void* dst, const void* src, size_t bytes) {
  parallel_ranges((int64_t)bytes, [&](int64_t a, int64_t b) {
    std::memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, (size_t)(b - a));
  }, (int64_t)4 << 20);
}

}  // namespace gb

// Enqueues one metric evaluation on the handle's stream (gb_metric.cu); results
// land in d_out = [value, nvalid, derivative...] and the handle's status word.
namespace gb {
int enqueue_eval(gb_metric* m, const double* d_params, double* d_out, bool deriv, bool device_params,
                 bool acc_cleared = false);
struct EvalArgs;
void batch_eval_args(gb_metric* m, EvalArgs& a);
}

struct gb_ctx {
  int device = 0;
  int sm_count = 0;
};

struct gb_metric {
  gb_ctx* ctx = nullptr;
  int kind = GB_METRIC_MEAN_SQUARES;
  int64_t bins = 50;
  cudaStream_t stream = nullptr;

  gb::Geom fixed, moving, virt;
  bool virt_user = false;
  gb::DevBuf<float> d_fixed, d_moving;
  // per-level set-up (gb_metric_set_level_smoothing / _shrink)
  double level_sigma = 0.0;
  bool level_sigma_physical = true;
  int64_t level_shrink[3] = {1, 1, 1};
  gb::DevBuf<float> d_fixed_s, d_moving_s;  // the level's smoothed images
  const float* fixed_img() const { return level_sigma > 0.0 ? d_fixed_s.p : d_fixed.p; }
  const float* moving_img() const { return level_sigma > 0.0 ? d_moving_s.p : d_moving.p; }
  gb::DevBuf<double> d_grad_in;  // caller-supplied gradient image (xyz doubles)
  int grad_source = GB_GRADIENT_IMAGE;
  bool grad_set = false;

  std::vector<float> h_points;
  bool points_virtual = true;
  bool use_sampled = false;

  int tkind = -1;
  std::vector<double> tparams, tfixed;
  int64_t nper = 0;  // B-spline nodes per dimension

  // set by Initialize
  bool initialized = false;
  int64_t ndomain = 0;   // candidate points (samples or virtual voxels)
  int64_t nsamples = 0;  // samples with a valid fixed value, sorted
  gb::DevBuf<float4> d_mov4;     // packed moving image: (value, gx, gy, gz)
  gb::DevBuf<float4> d_samples;  // (x, y, z, fixed value | fixed Parzen bin)
  gb::DevBuf<float4> d_cache;    // per-sample pass-1 result for the derivative pass
  gb::DevBuf<float4> d_sup;      // per-sample B-spline support (tx, ty, tz, packed start | valid)
  gb::DevBuf<int4> d_chunks;     // (first sample, end sample, cell, 0) of same-cell sample runs
  gb::DevBuf<int> d_node_first;    // per node: first entry in d_node_entries (nper + 1)
  gb::DevBuf<int> d_node_entries;  // chunk * 192 + support position of each (node, chunk) pair
  gb::DevBuf<float> d_chunk_part;  // nchunks x 192 Jacobian partial sums
  gb::DevBuf<float4> d_nodes;    // B-spline coefficients as float4 nodes
  gb::DevBuf<uint32_t> d_voff;   // displacement field on a point set: each sample's nearest virtual voxel
  double jhmi_variance = 1.5;    // joint-histogram MI: variance of the joint-PDF smoothing
  double fp_res = 0.0;           // UseFloatingPointCorrection resolution, 0 = off
  gb::DevBuf<unsigned char> d_jhmi;  // joint-histogram MI constants (JhmiConsts)
  int64_t nchunks = 0;
  int64_t node_entries_count = 0;  // (node, chunk) pairs: chooses the parameter gather's shape
  int grid[3] = {0, 0, 0};       // B-spline control grid
  double mstate[8] = {0, 0, 0, 0, 0, 0, 0, 0};

  // evaluation buffers
  gb::DevBuf<double> d_params;
  gb::DevBuf<unsigned char> d_acc;  // accumulators, cleared per evaluation
  size_t acc_bytes = 0;
  gb::DevBuf<double> d_scratch;     // per-block / per-group partials, overwritten per evaluation
  gb::DevBuf<double> d_out;         // [value, nvalid, derivative...]
  gb::DevBuf<int> d_status;
  gb::DevBuf<float> d_pratio;       // bins*bins log(p/pm) table
  gb::DevBuf<double> d_pdf;         // normalized joint PDF of the last evaluation
  gb::DevBuf<gb::EvalConsts> d_consts;  // per-evaluation transform constants
  gb::EvalConsts* h_consts = nullptr;   // pinned staging of the constants
  double* h_params = nullptr;       // pinned staging
  double* h_out = nullptr;          // pinned staging, 2 + P doubles
  int* h_status = nullptr;
  uint64_t last_nvalid = 0;
  int last_status = GB_OK;

  // device optimizer (gb_metric_optimize_regular_step)
  const int* eval_halt = nullptr;   // while set, evaluation kernels return at once once it reads nonzero
  gb::DevBuf<unsigned char> d_opt;  // optimizer state
  gb::DevBuf<double> d_opt_vec;     // previous gradient, scaled gradient, best parameters, 1 / scales (4 x P)
  unsigned char* h_opt = nullptr;   // pinned copy of the state
  int* h_halt = nullptr;            // pinned halt flags, one per batch slot
  bool opt_graphs = true;           // capture each iteration in a CUDA graph

  // the host call's device work as CUDA graphs, [value only, with derivative]
  cudaGraphExec_t host_exec[2] = {nullptr, nullptr};
  bool host_graph_tried[2] = {false, false};
  void drop_host_graphs();

  size_t device_bytes() const;  // all device buffers of the handle (gb_metric.cu)
  void release_buffers();       // frees them in the handle's stream order (gb_metric.cu)
  size_t h_cap = 0;             // doubles held by h_params and h_out (pinned, reused across levels)

  int inject_fault = GB_FAULT_NONE;  // gb_metric_set_fault_injection
  std::string last_error;            // text of the last error raised by a call on this handle

  // per-kernel event timing (gb_metric_set_profiling)
  bool profiling = false;
  static constexpr int kMaxEvents = 8;
  cudaEvent_t events[kMaxEvents] = {};
  int nevents = 0;
  void mark() {
    if (!profiling || nevents >= kMaxEvents) return;
    if (!events[nevents]) cudaEventCreate(&events[nevents]);
    cudaEventRecord(events[nevents], stream);
    ++nevents;
  }
};
