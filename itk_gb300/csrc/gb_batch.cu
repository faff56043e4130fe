// gb_batch.cu -- many affine registrations advancing together.
//
// Every registration keeps its own metric handle (images, samples, caches,
// accumulators) and optimizer state in HBM.  One optimizer iteration of all of
// them is one launch per phase:
//   k_batch_clear    accumulators of every running registration
//   k_batch_prepare  per-evaluation transform constants (22 FP64 entries each)
//   k_batch_msq      MeanSquares value and derivative      } blocks of all
//   k_batch_pass1    Mattes joint histogram, last block's   } registrations in
//                    log(p / pm) table                      } one grid, each
//   k_batch_pass2    Mattes value and derivative            } block one virtual
//   k_batch_step     AdvanceOneStep (one block per registration)   block of one
// captured once as a CUDA graph and relaunched per iteration.     registration
// A registration's blocks are a fixed function of its own sample count and the
// samples-per-block setting (chosen by gb_batch_autotune), so its results are
// the same alone and in any mix: the reduction orders do not depend on the
// other registrations.  Registrations that stop are collected between batches
// of iterations and the tables are rebuilt without them.
//
// Reference semantics: the single-registration loop (gb_optimizer.cu) and the
// metric kernels (gb_kernels.cuh); the stop at NumberOfIterations is checked
// in the step kernel (itkGradientDescentOptimizerv4.hxx:82-89).
#define GB_KERNELS_HELPERS_ONLY
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "gb_internal.h"
#include "gb_kernels.cuh"
#include "gb_step.cuh"

namespace gb {

enum { kGrpMsqImage = 0, kGrpMsqCD = 1, kGrpP1Image = 2, kGrpP1CD = 3, kGrpP2 = 4, kGroups = 5 };
enum { kSpbMsq = 0, kSpbPass1 = 1, kSpbPass2 = 2 };

struct ClearItem {
  unsigned long long* p;
  long long words;
  const int* halt;
};

// The registration's evaluation arguments into shared memory (one copy per block).
__device__ __forceinline__ void load_reg(const EvalArgs* __restrict__ regs, int r, EvalArgs& sa) {
  const unsigned* src = reinterpret_cast<const unsigned*>(regs + r);
  unsigned* dst = reinterpret_cast<unsigned*>(&sa);
  for (int k = threadIdx.x; k < (int)(sizeof(EvalArgs) / 4); k += blockDim.x) dst[k] = __ldg(src + k);
  __syncthreads();
}

__global__ void __launch_bounds__(kBlock) k_batch_clear(const ClearItem* __restrict__ items) {
  griddep_wait();
  const ClearItem it = items[blockIdx.x];
  if (__ldcg(it.halt)) return;
  griddep_launch_dependents();
  for (long long k = threadIdx.x; k < it.words; k += blockDim.x) it.p[k] = 0ull;
}

// One block (one lane) per (registration, constant entry).
__global__ void __launch_bounds__(32) k_batch_prepare(const EvalArgs* __restrict__ regs) {
  griddep_wait();
  const int r = blockIdx.x / kConstEntries, e = blockIdx.x - r * kConstEntries;
  const EvalArgs& a = regs[r];
  if (halted(a)) return;
  griddep_launch_dependents();
  if (threadIdx.x == 0)
    affine_const_entry(e, a.params, a.center, a.m_p2i, a.m_origin, a.dense ? a.v_i2p : nullptr, a.v_origin,
                       *const_cast<EvalConsts*>(a.consts));
}

// work[b] = (registration, virtual block, virtual blocks of that registration, 0)
template <int GRAD>
__global__ void __launch_bounds__(kBlock) k_batch_msq(const EvalArgs* __restrict__ regs, const int4* __restrict__ work) {
  __shared__ EvalArgs sa;
  const int4 w = work[blockIdx.x];
  load_reg(regs, w.x, sa);
  msq_affine_body<GRAD>(sa, VGrid{w.y, w.z});
}

template <int GRAD>
__global__ void __launch_bounds__(kBlock, GRAD == kGradImage ? 5 : 4)
    k_batch_pass1(const EvalArgs* __restrict__ regs, const int4* __restrict__ work) {
  __shared__ EvalArgs sa;
  const int4 w = work[blockIdx.x];
  load_reg(regs, w.x, sa);
  mattes_pass1_affine_body<GRAD>(sa, VGrid{w.y, w.z});
}

__global__ void __launch_bounds__(kBlock, 4) k_batch_pass2(const EvalArgs* __restrict__ regs,
                                                           const int4* __restrict__ work) {
  __shared__ EvalArgs sa;
  const int4 w = work[blockIdx.x];
  load_reg(regs, w.x, sa);
  mattes_pass2_affine_body<false>(sa, VGrid{w.y, w.z});
}

// AdvanceOneStep of one registration per block (step_block), one warp for the
// 12 affine parameters.
__global__ void __launch_bounds__(32) k_batch_step(const StepArgs* __restrict__ steps) {
  griddep_wait();
  const StepArgs s = steps[blockIdx.x];
  griddep_launch_dependents();
  step_block<32>(s);
}

// out[r] = halt word of registration r; out[n] = the number still running.
__global__ void __launch_bounds__(kBlock) k_batch_halts(const StepArgs* __restrict__ steps, int n, int* out) {
  griddep_wait();
  __shared__ int running;
  if (threadIdx.x == 0) running = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int h = __ldcg(&steps[r].st->halt);
    out[r] = h;
    if (!h) atomicAdd(&running, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) out[n] = running;
}

static int cuda_fail(cudaError_t e, const char* where) {
  return fail(GB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GB_B_CUDA(call)                                 \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

template <typename... KArgs, typename... Args>
static cudaError_t launch_dep(cudaStream_t st, void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace gb

using namespace gb;

struct gb_batch {
  struct Reg {
    gb_metric* m = nullptr;
    StepArgs step;
    gb_optimizer_report report;
    int rc = GB_OK;
    bool done = false;
  };
  gb_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  int64_t spb[3] = {8192, 8192, 8192};  // samples per virtual block: MeanSquares, Mattes pass 1, Mattes pass 2
  bool use_graph = true;
  std::vector<Reg> regs;
  // tables of the running registrations
  std::vector<int> active;
  DevBuf<EvalArgs> d_eval;
  DevBuf<StepArgs> d_step;
  DevBuf<ClearItem> d_clear;
  DevBuf<int4> d_work;
  DevBuf<int> d_halts;
  int* h_halts = nullptr;  // pinned, 2 slots of (capacity + 1)
  size_t h_halts_cap = 0;
  int64_t goff[kGroups] = {}, gcnt[kGroups] = {};
  std::vector<int64_t> reg_work;  // work items of each running registration (all passes)
  int64_t total_work = 0;
  int64_t iterations = 0, rebuilds = 0;
  double rebuild_seconds = 0.0;
  size_t smem1 = 0, smem2 = 0;
  bool dirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};

  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

namespace {

int64_t vblocks(int64_t n, int64_t spb) {
  return std::max<int64_t>(1, std::min<int64_t>((n + spb - 1) / spb, kMaxBlocks));
}

// One iteration (or, with step = false, one evaluation of every running registration).
int enqueue_iteration(gb_batch* b, bool step) {
  const unsigned n = (unsigned)b->active.size();
  cudaStream_t st = b->stream;
  GB_B_CUDA(launch_dep(st, k_batch_clear, n, kBlock, 0, (const ClearItem*)b->d_clear.p));
  GB_B_CUDA(launch_dep(st, k_batch_prepare, n * kConstEntries, 32, 0, (const EvalArgs*)b->d_eval.p));
  const EvalArgs* regs = b->d_eval.p;
  const int4* w = b->d_work.p;
  if (b->gcnt[kGrpMsqImage])
    GB_B_CUDA(launch_dep(st, k_batch_msq<kGradImage>, (unsigned)b->gcnt[kGrpMsqImage], kBlock, 0, regs,
                         w + b->goff[kGrpMsqImage]));
  if (b->gcnt[kGrpMsqCD])
    GB_B_CUDA(launch_dep(st, k_batch_msq<kGradCentralDifference>, (unsigned)b->gcnt[kGrpMsqCD], kBlock, 0, regs,
                         w + b->goff[kGrpMsqCD]));
  if (b->gcnt[kGrpP1Image])
    GB_B_CUDA(launch_dep(st, k_batch_pass1<kGradImage>, (unsigned)b->gcnt[kGrpP1Image], kBlock, b->smem1, regs,
                         w + b->goff[kGrpP1Image]));
  if (b->gcnt[kGrpP1CD])
    GB_B_CUDA(launch_dep(st, k_batch_pass1<kGradCentralDifference>, (unsigned)b->gcnt[kGrpP1CD], kBlock, b->smem1,
                         regs, w + b->goff[kGrpP1CD]));
  if (b->gcnt[kGrpP2])
    GB_B_CUDA(launch_dep(st, k_batch_pass2, (unsigned)b->gcnt[kGrpP2], kBlock, b->smem2, regs, w + b->goff[kGrpP2]));
  if (step) GB_B_CUDA(launch_dep(st, k_batch_step, n, 32, 0, (const StepArgs*)b->d_step.p));
  return GB_OK;
}

// Tables of the registrations still running, uploaded; the iteration graph re-captured.
int rebuild_tables(gb_batch* b);

int rebuild(gb_batch* b) {
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = rebuild_tables(b);
  b->rebuild_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  b->rebuilds += 1;
  return rc;
}

int rebuild_tables(gb_batch* b) {
  b->drop_graph();
  b->active.clear();
  for (size_t i = 0; i < b->regs.size(); ++i)
    if (!b->regs[i].done) b->active.push_back((int)i);
  const size_t n = b->active.size();
  b->dirty = false;
  if (n == 0) return GB_OK;
  std::vector<EvalArgs> ev(n);
  std::vector<StepArgs> sa(n);
  std::vector<ClearItem> ci(n);
  std::vector<int4> work[kGroups];
  int maxbins = 0;
  b->reg_work.assign(n, 0);
  b->total_work = 0;
  for (size_t k = 0; k < n; ++k) {
    gb_batch::Reg& R = b->regs[(size_t)b->active[k]];
    gb_metric* m = R.m;
    m->eval_halt = &R.step.st->halt;
    batch_eval_args(m, ev[k]);
    m->eval_halt = nullptr;
    sa[k] = R.step;
    ci[k] = ClearItem{reinterpret_cast<unsigned long long*>(m->d_acc.p), (long long)(m->acc_bytes / 8),
                      &R.step.st->halt};
    const bool cd = m->grad_source == GB_GRADIENT_CENTRAL_DIFFERENCE;
    if (m->kind == GB_METRIC_MEAN_SQUARES) {
      const int64_t nv = vblocks(m->nsamples, b->spb[kSpbMsq]);
      for (int64_t v = 0; v < nv; ++v)
        work[cd ? kGrpMsqCD : kGrpMsqImage].push_back(make_int4((int)k, (int)v, (int)nv, 0));
      b->reg_work[k] = nv;
    } else {
      maxbins = std::max(maxbins, (int)m->bins);
      const int64_t n1 = vblocks(m->nsamples, b->spb[kSpbPass1]);
      for (int64_t v = 0; v < n1; ++v)
        work[cd ? kGrpP1CD : kGrpP1Image].push_back(make_int4((int)k, (int)v, (int)n1, 0));
      const int64_t n2 = vblocks(m->nsamples, b->spb[kSpbPass2]);
      for (int64_t v = 0; v < n2; ++v) work[kGrpP2].push_back(make_int4((int)k, (int)v, (int)n2, 0));
      b->reg_work[k] = n1 + n2;
    }
    b->total_work += b->reg_work[k];
  }
  std::vector<int4> all;
  for (int g = 0; g < kGroups; ++g) {
    b->goff[g] = (int64_t)all.size();
    b->gcnt[g] = (int64_t)work[g].size();
    all.insert(all.end(), work[g].begin(), work[g].end());
  }
  b->smem1 = sizeof(unsigned long long) * (size_t)(maxbins * maxbins + maxbins) + sizeof(unsigned) * (size_t)maxbins;
  b->smem2 = mattes_pass2_smem(maxbins);
  if (maxbins > 0) {
    if (b->smem1 > 200 * 1024) return fail(GB_ERR_UNSUPPORTED, "histogram too large for shared memory (bins > 160)");
    GB_B_CUDA(cudaFuncSetAttribute(k_batch_pass1<kGradImage>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)b->smem1));
    GB_B_CUDA(cudaFuncSetAttribute(k_batch_pass1<kGradCentralDifference>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem1));
    GB_B_CUDA(cudaFuncSetAttribute(k_batch_pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem2));
  }
  GB_B_CUDA(b->d_eval.alloc_on(b->stream, n));
  GB_B_CUDA(b->d_step.alloc_on(b->stream, n));
  GB_B_CUDA(b->d_clear.alloc_on(b->stream, n));
  GB_B_CUDA(b->d_work.alloc_on(b->stream, std::max<size_t>(all.size(), 1)));
  GB_B_CUDA(b->d_halts.alloc_on(b->stream, n + 1));
  if (b->h_halts_cap < n + 1) {
    if (b->h_halts) cudaFreeHost(b->h_halts);
    b->h_halts = nullptr;
    GB_B_CUDA(cudaMallocHost(&b->h_halts, 2 * sizeof(int) * (n + 1)));
    b->h_halts_cap = n + 1;
  }
  cudaStream_t st = b->stream;
  GB_B_CUDA(cudaMemcpyAsync(b->d_eval.p, ev.data(), sizeof(EvalArgs) * n, cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemcpyAsync(b->d_step.p, sa.data(), sizeof(StepArgs) * n, cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemcpyAsync(b->d_clear.p, ci.data(), sizeof(ClearItem) * n, cudaMemcpyHostToDevice, st));
  if (!all.empty())
    GB_B_CUDA(cudaMemcpyAsync(b->d_work.p, all.data(), sizeof(int4) * all.size(), cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaStreamSynchronize(st));  // the host tables are pageable
  if (b->use_graph) {
    bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
      const int rc = enqueue_iteration(b, true);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(st, &g);
      ok = rc == GB_OK && e == cudaSuccess && g != nullptr;
      b->graph = g;
      if (ok) ok = cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess;
    }
    if (!ok) {
      (void)cudaGetLastError();
      b->drop_graph();
    }
  }
  return GB_OK;
}

}  // namespace

extern "C" int gb_batch_create(gb_ctx* ctx, gb_batch** out) {
  if (!ctx || !out) return fail(GB_ERR_BAD_ARG, "null argument");
  GB_B_CUDA(cudaSetDevice(ctx->device));
  gb_batch* b = new gb_batch();
  b->ctx = ctx;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev[1], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "gb_batch_create");
  }
  *out = b;
  return GB_OK;
}

extern "C" int gb_batch_destroy(gb_batch* b) {
  if (!b) return GB_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->stream);
  b->drop_graph();
  b->d_eval.reset();  // stream-ordered frees, before the stream goes
  b->d_step.reset();
  b->d_clear.reset();
  b->d_work.reset();
  b->d_halts.reset();
  cudaStreamSynchronize(b->stream);
  for (cudaEvent_t e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->h_halts) cudaFreeHost(b->h_halts);
  cudaStreamDestroy(b->stream);
  delete b;
  return GB_OK;
}

extern "C" int gb_batch_set_graphs(gb_batch* b, int on) {
  if (!b) return fail(GB_ERR_BAD_ARG, "null batch");
  b->use_graph = on != 0;
  b->dirty = true;
  return GB_OK;
}

extern "C" int gb_batch_set_samples_per_block(gb_batch* b, const int64_t spb[3]) {
  if (!b || !spb) return fail(GB_ERR_BAD_ARG, "null argument");
  for (int i = 0; i < 3; ++i)
    if (spb[i] < kBlock) return fail(GB_ERR_BAD_ARG, "samples per block must be >= 256");
  for (int i = 0; i < 3; ++i) b->spb[i] = spb[i];
  b->dirty = true;
  return GB_OK;
}

extern "C" int gb_batch_get_samples_per_block(gb_batch* b, int64_t spb[3]) {
  if (!b || !spb) return fail(GB_ERR_BAD_ARG, "null argument");
  for (int i = 0; i < 3; ++i) spb[i] = b->spb[i];
  return GB_OK;
}

extern "C" int gb_batch_add(gb_batch* b, gb_metric* m, const gb_regular_step_settings* cfg, const double* scales,
                            int64_t nscales, int64_t* slot) {
  if (!b || !m || !cfg || !slot) return fail(GB_ERR_BAD_ARG, "null argument");
  if (m->ctx->device != b->ctx->device) return fail(GB_ERR_BAD_ARG, "metric and batch on different devices");
  if (m->tkind != GB_TRANSFORM_AFFINE) return fail(GB_ERR_UNSUPPORTED, "the batched engine runs affine registrations");
  if (m->kind == GB_METRIC_CORRELATION || m->kind == GB_METRIC_JOINT_HISTOGRAM_MI)
    return fail(GB_ERR_UNSUPPORTED, "the batched engine runs MeanSquares and Mattes registrations");
  if (m->kind == GB_METRIC_MEAN_SQUARES && m->fp_res > 0.0)
    return fail(GB_ERR_UNSUPPORTED, "the batched engine runs without the floating point correction");
  for (const gb_batch::Reg& R : b->regs)
    if (R.m == m && !R.done) return fail(GB_ERR_BAD_ARG, "metric already running in this batch");
  gb_batch::Reg R;
  R.m = m;
  memset(&R.report, 0, sizeof(R.report));
  int rc = opt_setup(m, cfg, scales, nscales, R.step);
  if (rc) return rc;
  *slot = (int64_t)b->regs.size();
  if (cfg->number_of_iterations == 0 || m->nsamples == 0) {
    // nothing to batch: no iteration at all, or no fixed sample (the evaluation is
    // staged from the host) -- the single-registration loop gives the result now
    R.rc = gb_metric_optimize_regular_step(m, cfg, scales, nscales, &R.report);
    R.done = true;
    b->regs.push_back(R);
    return GB_OK;
  }
  b->regs.push_back(R);
  b->dirty = true;
  return GB_OK;
}

// Collects every registration of the current tables that has stopped (the stream drains first).
static int collect_halted(gb_batch* b, bool& any) {
  cudaStream_t st = b->stream;
  const int n = (int)b->active.size();
  any = false;
  if (n == 0) return GB_OK;
  GB_B_CUDA(cudaStreamSynchronize(st));
  GB_B_CUDA(launch_dep(st, k_batch_halts, 1u, kBlock, 0, (const StepArgs*)b->d_step.p, n, b->d_halts.p));
  GB_B_CUDA(cudaMemcpyAsync(b->h_halts, b->d_halts.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st));
  GB_B_CUDA(cudaStreamSynchronize(st));
  std::vector<int> idx;
  for (int k = 0; k < n; ++k)
    if (b->h_halts[k] && !b->regs[(size_t)b->active[k]].done) idx.push_back(b->active[k]);
  for (int r : idx) {  // the copies of every stopped registration, then one wait
    int rc = opt_fetch(b->regs[(size_t)r].m, b->regs[(size_t)r].step, st);
    if (rc) return rc;
  }
  GB_B_CUDA(cudaStreamSynchronize(st));
  for (int r : idx) {
    gb_batch::Reg& R = b->regs[(size_t)r];
    R.rc = opt_collect(R.m, R.step, &R.report);
    R.done = true;
    any = true;
  }
  return GB_OK;
}

extern "C" int gb_batch_run(gb_batch* b, int64_t max_iterations, int64_t* running) {
  if (!b) return fail(GB_ERR_BAD_ARG, "null batch");
  GB_B_CUDA(cudaSetDevice(b->ctx->device));
  cudaStream_t st = b->stream;
  int64_t done = 0;
  int64_t batch = 2;
  bool collected = false;
  while (max_iterations <= 0 || done < max_iterations) {
    if (b->dirty) {
      const int rc = rebuild(b);
      if (rc) return rc;
    }
    const int n = (int)b->active.size();
    if (n == 0) break;
    // Two batches of iterations in flight: batch j + 1 is enqueued before batch j's
    // halt words are read.  Stopped registrations stay in the tables (their blocks
    // return at once) until they hold half of the work items, then the tables are
    // rebuilt without them.
    int slot = 0;
    bool pending = false, shrink = false;
    while (max_iterations <= 0 || done < max_iterations) {
      const int64_t k = max_iterations <= 0 ? batch : std::min(batch, max_iterations - done);
      for (int64_t i = 0; i < k; ++i) {
        if (b->exec) {
          GB_B_CUDA(cudaGraphLaunch(b->exec, st));
        } else {
          const int rc = enqueue_iteration(b, true);
          if (rc) return rc;
        }
      }
      done += k;
      b->iterations += k;
      batch = std::min<int64_t>(batch * 2, 16);
      int* hh = b->h_halts + slot * (n + 1);
      GB_B_CUDA(launch_dep(st, k_batch_halts, 1u, kBlock, 0, (const StepArgs*)b->d_step.p, n, b->d_halts.p));
      GB_B_CUDA(cudaMemcpyAsync(hh, b->d_halts.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st));
      GB_B_CUDA(cudaEventRecord(b->ev[slot], st));
      if (pending) {
        GB_B_CUDA(cudaEventSynchronize(b->ev[slot ^ 1]));
        const int* ph = b->h_halts + (slot ^ 1) * (n + 1);
        if (ph[n] == 0) {  // all stopped
          shrink = true;
          break;
        }
        if (ph[n] < n) {
          int64_t hw = 0;
          for (int r = 0; r < n; ++r)
            if (ph[r]) hw += b->reg_work[(size_t)r];
          if (2 * hw >= b->total_work) {
            shrink = true;
            break;
          }
        }
      }
      pending = true;
      slot ^= 1;
    }
    bool any = false;
    const int rc = collect_halted(b, any);
    if (rc) return rc;
    collected = collected || any;
    if (!shrink) break;  // iteration budget of this call used up
    b->dirty = true;
  }
  // the caller may re-initialize or destroy the metrics of finished registrations:
  // the next call starts from tables without them
  if (collected) b->dirty = true;
  if (running) {
    int64_t r = 0;
    for (const gb_batch::Reg& R : b->regs) r += R.done ? 0 : 1;
    *running = r;
  }
  return GB_OK;
}

extern "C" int gb_batch_get_stats(gb_batch* b, int64_t* iterations, int64_t* rebuilds, double* rebuild_seconds) {
  if (!b) return fail(GB_ERR_BAD_ARG, "null batch");
  if (iterations) *iterations = b->iterations;
  if (rebuilds) *rebuilds = b->rebuilds;
  if (rebuild_seconds) *rebuild_seconds = b->rebuild_seconds;
  return GB_OK;
}

// Registration `slot`: *finished = 1 and its report once it has stopped (the
// handle then holds the final parameters); returns its status (a metric error
// that stopped it, as gb_metric_optimize_regular_step would).
extern "C" int gb_batch_result(gb_batch* b, int64_t slot, int* finished, gb_optimizer_report* report) {
  if (!b || !finished) return fail(GB_ERR_BAD_ARG, "null argument");
  if (slot < 0 || slot >= (int64_t)b->regs.size()) return fail(GB_ERR_BAD_ARG, "no such slot");
  const gb_batch::Reg& R = b->regs[(size_t)slot];
  *finished = R.done ? 1 : 0;
  if (!R.done) return GB_OK;
  if (report) *report = R.report;
  return R.rc;
}

// Chooses the samples per virtual block of each pass: for every candidate, the
// evaluation of all running registrations (no optimizer step, so no state
// changes) timed over `iterations` launches; the fastest stays set.
extern "C" int gb_batch_autotune(gb_batch* b, int iterations, int64_t spb_out[3]) {
  if (!b) return fail(GB_ERR_BAD_ARG, "null batch");
  if (iterations < 1) iterations = 1;
  GB_B_CUDA(cudaSetDevice(b->ctx->device));
  cudaStream_t st = b->stream;
  const int64_t cand[] = {2048, 4096, 8192, 16384, 32768, 65536};
  cudaEvent_t t0, t1;
  GB_B_CUDA(cudaEventCreate(&t0));
  GB_B_CUDA(cudaEventCreate(&t1));
  const bool graphs = b->use_graph;
  b->use_graph = false;
  int rc = GB_OK;
  for (int pass = 0; pass < 3 && rc == GB_OK; ++pass) {
    float best_ms = 0.f;
    int64_t best = b->spb[pass];
    for (int64_t c : cand) {
      b->spb[pass] = c;
      rc = rebuild(b);
      if (rc) break;
      if (b->active.empty()) break;
      if ((rc = enqueue_iteration(b, false))) break;  // warm-up
      if (cudaEventRecord(t0, st) != cudaSuccess) { rc = cuda_fail(cudaGetLastError(), "autotune"); break; }
      for (int i = 0; i < iterations && rc == GB_OK; ++i) rc = enqueue_iteration(b, false);
      if (rc) break;
      float ms = 0.f;
      if (cudaEventRecord(t1, st) != cudaSuccess || cudaEventSynchronize(t1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "autotune timing");
        break;
      }
      if (best_ms == 0.f || ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    b->spb[pass] = best;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  b->use_graph = graphs;
  b->dirty = true;
  if (rc) return rc;
  if (spb_out)
    for (int i = 0; i < 3; ++i) spb_out[i] = b->spb[i];
  return GB_OK;
}
