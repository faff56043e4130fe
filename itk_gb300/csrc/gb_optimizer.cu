// gb_optimizer.cu -- RegularStepGradientDescentOptimizerv4 with its whole loop
// in device memory.
//
// Reference semantics (paths relative to ITK's Modules/):
//   StartOptimization / AdvanceOneStep       Numerics/Optimizersv4/include/itkRegularStepGradientDescentOptimizerv4.hxx:39-229
//   ResumeOptimization loop, best value      Numerics/Optimizersv4/include/itkGradientDescentOptimizerv4.hxx:59-169
//   scales validation and identity test      Numerics/Optimizersv4/src/itkObjectToObjectOptimizerBase.cxx:102-142
//   Transform::UpdateTransformParameters     Core/Transform/include/itkTransform.hxx:69-121
//
// One iteration is the metric evaluation (its kernels read the parameters from
// device memory) followed by two small kernels:
//   k_step_reduce  g = derivative / scales and g_prev / scales per parameter,
//                  ||g||^2 and g . g_prev as compensated FP64 sums (per block,
//                  then by the last block in a fixed order); the last block
//                  takes the optimizer's decisions (metric error, gradient
//                  tolerance, relaxation, minimum step, best value);
//   k_step_apply   params += (g * relaxation * rate) * (1 / ||g||) per
//                  parameter, or the return-best restore when the loop stopped.
// After a stop the state's halt word is set, and every kernel of the later
// iterations that the host has already enqueued returns at once.  The host
// enqueues iterations in batches (each one a CUDA graph launch when capture
// works) and reads the halt word between batches, one batch behind the GPU.
//
// The sums run over the parameters in a fixed tree of two-sum pairs instead of
// the reference's sequential Kahan loop: both are exact to about one rounding
// of the result, so the two can differ in the last bit of ||g|| and g . g_prev.
// Every other operation is the reference's, rounding for rounding (FP64, no
// contraction).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gb_device.cuh"
#include "gb_internal.h"
#include "gb_step.cuh"

namespace gb {

constexpr int kMaxBatch = 16;  // iterations enqueued between reads of the halt word

__global__ void __launch_bounds__(kStepBlock) k_step_reduce(StepArgs s) {
  griddep_wait();
  OptState* S = s.st;
  if (__ldcg(&S->halt)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) S->action = kActNone;
    return;
  }
  griddep_launch_dependents();
  const int status = __ldcg(s.status);
  const bool err = metric_error(s, status);
  DD q = {0.0, 0.0}, r = {0.0, 0.0};
  if (!err) {
    // one parameter per thread up to the grid's size, a grid-stride run of them beyond
    // (a displacement field's millions); each thread's terms added by two-sum
    const long long stride = (long long)gridDim.x * kStepBlock;
    for (long long j = (long long)blockIdx.x * kStepBlock + threadIdx.x; j < s.P; j += stride) {
      double qq, rr;
      step_terms(s, j, qq, rr);
      q = dd_add(q, DD{qq, 0.0});
      r = dd_add(r, DD{rr, 0.0});
    }
  }
  block_dd2(q, r);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    S->part[blockIdx.x][0] = q.hi;
    S->part[blockIdx.x][1] = q.lo;
    S->part[blockIdx.x][2] = r.hi;
    S->part[blockIdx.x][3] = r.lo;
    __threadfence();
    last = atomicAdd(&S->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x >= 32) return;
  __threadfence();
  const int lane = threadIdx.x;
  DD x = {0.0, 0.0}, y = {0.0, 0.0};
  for (int b = lane; b < (int)gridDim.x; b += 32) {
    x = dd_add(x, DD{__ldcg(&S->part[b][0]), __ldcg(&S->part[b][1])});
    y = dd_add(y, DD{__ldcg(&S->part[b][2]), __ldcg(&S->part[b][3])});
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const DD ox = dd_shfl_down(x, off), oy = dd_shfl_down(y, off);
    if (lane < off) {
      x = dd_add(x, ox);
      y = dd_add(y, oy);
    }
  }
  if (lane != 0) return;
  S->ticket = 0u;
  step_decide(s, S, status, x, y);
}

__global__ void __launch_bounds__(kStepBlock) k_step_apply(StepArgs s) {
  griddep_wait();
  griddep_launch_dependents();
  const OptState* S = s.st;
  const int act = __ldcg(&S->action);
  const long long stride = (long long)gridDim.x * kStepBlock;
  for (long long j = (long long)blockIdx.x * kStepBlock + threadIdx.x; j < s.P; j += stride) step_apply(s, S, act, j);
}

// The whole step of a registration with at most 32 parameters in one warp
// (reduce, decide and apply in one launch).
__global__ void __launch_bounds__(32) k_step_single(StepArgs s) {
  griddep_wait();
  griddep_launch_dependents();
  step_block<32>(s);
}

// The loop ran out of iterations without another stop: MAXIMUM_NUMBER_OF_ITERATIONS.
__global__ void __launch_bounds__(kStepBlock) k_opt_finish(StepArgs s) {
  griddep_wait();
  OptState* S = s.st;
  const bool was_halted = __ldcg(&S->halt) != 0;
  __syncthreads();
  if (was_halted) return;
  if (s.return_best)
    for (long long j = threadIdx.x; j < s.P; j += blockDim.x) s.params[j] = __ldcg(s.best + j);
  if (threadIdx.x == 0) {
    S->stop = GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS;
    S->halt = 1;
    if (s.return_best) S->value = S->best_value;
  }
}

static int cuda_fail(cudaError_t e, const char* where) {
  return fail(GB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GB_OPT_CUDA(call)                               \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

template <typename... KArgs, typename... Args>
static cudaError_t launch_dependent(cudaStream_t st, void (*kernel)(KArgs...), unsigned grid, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kStepBlock);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// One optimizer iteration: the evaluation, then the step (one warp for at most 32
// parameters, else the multi-block reduce and apply).
static int enqueue_iteration(gb_metric* m, const StepArgs& a, unsigned blocks) {
  int rc = enqueue_eval(m, m->d_params.p, m->d_out.p, true, true);
  if (rc) return rc;
  if (a.P <= 32) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(32);
    cfg.stream = m->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_OPT_CUDA(cudaLaunchKernelEx(&cfg, k_step_single, a));
    return GB_OK;
  }
  GB_OPT_CUDA(launch_dependent(m->stream, k_step_reduce, blocks, a));
  GB_OPT_CUDA(launch_dependent(m->stream, k_step_apply, blocks, a));
  return GB_OK;
}

// Restores the handle's evaluation settings however the loop ends.
struct LoopGuard {
  gb_metric* m;
  bool profiling;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~LoopGuard() {
    m->eval_halt = nullptr;
    m->profiling = profiling;
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};

// StartOptimization for one registration: validates the settings and scales,
// allocates the handle's optimizer buffers and enqueues their initial state on
// the handle's stream (synchronized before returning); fills the step arguments.
int opt_setup(gb_metric* m, const gb_regular_step_settings* cfg, const double* scales, int64_t nscales,
              StepArgs& a) {
  if (!m || !cfg) return fail(GB_ERR_BAD_ARG, "null argument");
  if (!m->initialized) return fail(GB_ERR_NOT_INITIALIZED, "call gb_metric_initialize first");
  const int64_t P = (int64_t)m->tparams.size();
  if (P <= 0) return fail(GB_ERR_BAD_ARG, "the moving transform has no parameters");
  if (P > (int64_t)0x7fffffff) return fail(GB_ERR_UNSUPPORTED, "more than 2^31-1 parameters in the device optimizer");
  if (cfg->number_of_iterations < 0) return fail(GB_ERR_BAD_ARG, "number of iterations must be >= 0");
  if (cfg->gradient_magnitude_tolerance < 0.0)
    return fail(GB_ERR_BAD_ARG, "Gradient magnitude tolerance must be greater or equal 0.0. Current value is " +
                                    std::to_string(cfg->gradient_magnitude_tolerance));
  if (cfg->relaxation_factor < 0.0)
    return fail(GB_ERR_BAD_ARG,
                "Relaxation factor must be positive. Current value is " + std::to_string(cfg->relaxation_factor));
  if (cfg->relaxation_factor >= 1.0)
    return fail(GB_ERR_BAD_ARG,
                "Relaxation factor must be less than 1.0. Current value is " + std::to_string(cfg->relaxation_factor));
  // scales (ObjectToObjectOptimizerBase::StartOptimization): > epsilon each; all
  // within 0.01 of 1 means identity, and the gradient is then not rescaled
  // a displacement field has 3 local parameters per voxel; its scales are per local
  // parameter and apply to parameter i as scales[i % 3] (ModifyGradientByScalesOverSubRange,
  // Numerics/Optimizersv4/include/itkGradientDescentOptimizerv4.hxx:204-238)
  const int64_t nlocal = m->tkind == GB_TRANSFORM_DISPLACEMENT_FIELD ? 3 : P;
  std::vector<double> inv_s((size_t)P, 1.0);
  if (nscales != 0) {
    if (!scales) return fail(GB_ERR_BAD_ARG, "null scales");
    if (nscales != nlocal)
      return fail(GB_ERR_BAD_ARG, "Size of scales (" + std::to_string(nscales) +
                                      ") must equal number of local parameters (" + std::to_string(nlocal) + ").");
    bool identity = true;
    for (int64_t i = 0; i < nlocal; ++i) {
      if (!(scales[i] > DBL_EPSILON)) return fail(GB_ERR_BAD_ARG, "m_Scales values must be > epsilon.");
      if (std::fabs(1.0 - scales[i]) > 0.01) identity = false;
    }
    if (!identity)
      for (int64_t i = 0; i < P; ++i) inv_s[(size_t)i] = 1.0 / scales[i % nlocal];
  }
  GB_OPT_CUDA(cudaSetDevice(m->ctx->device));
  cudaStream_t st = m->stream;
  GB_OPT_CUDA(m->d_opt.alloc_on(st, sizeof(OptState)));
  GB_OPT_CUDA(m->d_opt_vec.alloc_on(st, (size_t)(4 * P)));
  if (!m->h_opt) GB_OPT_CUDA(cudaMallocHost(&m->h_opt, sizeof(OptState)));
  if (!m->h_halt) GB_OPT_CUDA(cudaMallocHost(&m->h_halt, 2 * sizeof(int)));
  OptState* S = reinterpret_cast<OptState*>(m->d_opt.p);
  double* d_prev = m->d_opt_vec.p;
  double* d_grad = d_prev + P;
  double* d_best = d_grad + P;
  double* d_inv = d_best + P;

  // relaxation 1, iteration 0, zero gradients, best = start
  OptState* h = reinterpret_cast<OptState*>(m->h_opt);
  memset(h, 0, sizeof(OptState));
  h->relaxation = 1.0;
  h->best_value = DBL_MAX;
  h->stop = kRunning;
  h->status = GB_OK;
  double* hp = m->h_params;  // pinned, P doubles
  std::copy(m->tparams.begin(), m->tparams.end(), hp);
  GB_OPT_CUDA(cudaMemcpyAsync(S, h, sizeof(OptState), cudaMemcpyHostToDevice, st));
  GB_OPT_CUDA(cudaMemcpyAsync(m->d_params.p, hp, sizeof(double) * P, cudaMemcpyHostToDevice, st));
  GB_OPT_CUDA(cudaMemcpyAsync(d_best, m->d_params.p, sizeof(double) * P, cudaMemcpyDeviceToDevice, st));
  GB_OPT_CUDA(cudaMemsetAsync(d_prev, 0, sizeof(double) * P, st));
  GB_OPT_CUDA(cudaMemcpyAsync(d_inv, inv_s.data(), sizeof(double) * P, cudaMemcpyHostToDevice, st));
  GB_OPT_CUDA(cudaStreamSynchronize(st));  // inv_s is pageable host memory

  memset(&a, 0, sizeof(a));
  a.out = m->d_out.p;
  a.status = m->d_status.p;
  a.params = m->d_params.p;
  a.prev = d_prev;
  a.grad = d_grad;
  a.best = d_best;
  a.inv_scales = d_inv;
  a.st = S;
  a.P = P;
  a.max_iterations = cfg->number_of_iterations;
  a.learning_rate = cfg->learning_rate;
  a.relaxation_factor = cfg->relaxation_factor;
  a.min_step = cfg->minimum_step_length;
  a.grad_tol = cfg->gradient_magnitude_tolerance;
  a.return_best = cfg->return_best_parameters_and_value ? 1 : 0;
  a.msq = m->kind != GB_METRIC_MATTES ? 1 : 0;  // MeanSquares, Correlation: no valid point is a warning
  return GB_OK;
}

// Enqueues the copies of the final state and parameters into the handle's pinned buffers.
int opt_fetch(gb_metric* m, const StepArgs& a, cudaStream_t st) {
  GB_OPT_CUDA(cudaMemcpyAsync(m->h_opt, a.st, sizeof(OptState), cudaMemcpyDeviceToHost, st));
  GB_OPT_CUDA(cudaMemcpyAsync(m->h_params, a.params, sizeof(double) * a.P, cudaMemcpyDeviceToHost, st));
  GB_OPT_CUDA(cudaMemcpyAsync(m->h_out, a.out, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
  return GB_OK;
}

// After opt_fetch has completed: the handle's parameters, the report and the status.
int opt_collect(gb_metric* m, const StepArgs& a, gb_optimizer_report* report) {
  const OptState* h = reinterpret_cast<const OptState*>(m->h_opt);
  std::copy(m->h_params, m->h_params + a.P, m->tparams.begin());
  if (h->iteration > 0 || h->stop == GB_STOP_COSTFUNCTION_ERROR) m->last_nvalid = (uint64_t)m->h_out[1];
  if (report) {
    report->stop_condition = h->stop;
    report->metric_status = h->status;
    report->iterations = h->iteration;
    report->value = h->value;
    report->current_step_length = h->step_length;
    report->gradient_magnitude = h->grad_mag;
    report->learning_rate_relaxation = h->relaxation;
  }
  if (h->stop == GB_STOP_COSTFUNCTION_ERROR) {
    m->last_status = h->status;
    if (h->status == GB_ERR_NO_VALID_POINTS)
      return fail(h->status,
                  "All samples map outside moving image buffer. The images do not sufficiently overlap. They need to "
                  "be initialized to have more overlap before this metric will work. For instance, you can align the "
                  "image centers by translation.");
    if (h->status == GB_ERR_JOINT_PDF_SUM_ZERO) return fail(h->status, "Joint PDF summed to zero");
    return fail(h->status, "metric evaluation failed during optimization");
  }
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_metric_set_optimizer_graphs(gb_metric* m, int on) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  m->opt_graphs = on != 0;
  return GB_OK;
}

extern "C" int gb_metric_optimize_regular_step(gb_metric* m, const gb_regular_step_settings* cfg,
                                               const double* scales, int64_t nscales, gb_optimizer_report* report) {
  gb::ErrorScope scope_(m, __func__);
  StepArgs a;
  int rc = opt_setup(m, cfg, scales, nscales, a);
  if (rc) return rc;
  cudaStream_t st = m->stream;
  OptState* S = a.st;
  const unsigned blocks = (unsigned)std::min<int64_t>(kStepMaxBlocks, (a.P + kStepBlock - 1) / kStepBlock);

  LoopGuard guard{m, m->profiling};
  m->profiling = false;
  m->eval_halt = &S->halt;
  const int64_t N = cfg->number_of_iterations;

  // one iteration as a CUDA graph (no graph when there is nothing to evaluate:
  // that path stages its result from host memory)
  if (m->opt_graphs && m->nsamples > 0 && N > 0) {
    bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
      const int rc2 = enqueue_iteration(m, a, blocks);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(st, &g);
      ok = rc2 == GB_OK && e == cudaSuccess && g != nullptr;
      if (g) guard.graph = g;
      if (ok) ok = cudaGraphInstantiate(&guard.exec, g, 0) == cudaSuccess;
    }
    if (!ok) {
      (void)cudaGetLastError();  // a failed capture leaves no sticky error; fall back to direct launches
      if (guard.exec) cudaGraphExecDestroy(guard.exec);
      guard.exec = nullptr;
    }
  }

  GB_OPT_CUDA(cudaEventCreateWithFlags(&guard.ev[0], cudaEventDisableTiming));
  GB_OPT_CUDA(cudaEventCreateWithFlags(&guard.ev[1], cudaEventDisableTiming));
  int64_t done = 0;
  int64_t batch = 2;
  int slot = 0;
  bool pending = false;  // a batch whose halt word has not been read yet
  while (done < N) {
    const int64_t k = std::min(batch, N - done);
    for (int64_t i = 0; i < k; ++i) {
      if (guard.exec) {
        GB_OPT_CUDA(cudaGraphLaunch(guard.exec, st));
      } else {
        const int rc2 = enqueue_iteration(m, a, blocks);
        if (rc2) return rc2;
      }
    }
    done += k;
    GB_OPT_CUDA(cudaMemcpyAsync(m->h_halt + slot, &S->halt, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_OPT_CUDA(cudaEventRecord(guard.ev[slot], st));
    if (pending) {  // the previous batch: stop enqueueing once it has halted
      GB_OPT_CUDA(cudaEventSynchronize(guard.ev[slot ^ 1]));
      if (m->h_halt[slot ^ 1]) break;
    }
    pending = true;
    slot ^= 1;
    batch = std::min<int64_t>(batch * 2, kMaxBatch);
  }
  // iterations exhausted without another stop: MAXIMUM_NUMBER_OF_ITERATIONS
  GB_OPT_CUDA(launch_dependent(st, k_opt_finish, 1u, a));
  rc = opt_fetch(m, a, st);
  if (rc) return rc;
  GB_OPT_CUDA(cudaStreamSynchronize(st));
  return opt_collect(m, a, report);
}
