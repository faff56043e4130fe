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

// ---------------------------------------------------------------------------
// The persistent form: `iters` iterations of every running registration in ONE
// launch.  The items of one iteration (a table of per_iter entries, the same for
// every iteration) are, in order: the accumulator clears, the 22 constant entries
// of every registration, the MeanSquares / Mattes pass-1 virtual blocks, the
// pass-2 virtual blocks, the steps; the launch's queue is that table repeated
// `iters` times.  Blocks take items in queue order (one atomic counter) and each
// item waits only for its own registration's earlier items, through monotonic
// completion counters:
//   clear / constants of iteration i   after the step of iteration i - 1
//   MeanSquares / pass 1 of i          after the 23 clear and constant items of i
//   pass 2 of i                        after every pass-1 block of i
//   step of i                          after every MeanSquares / pass-2 block of i
// Every item an item waits for comes earlier in the queue and has therefore been
// taken by a block that is running, so the launch always completes, whether or not
// all its blocks are resident.  Waits are bounded (kDepWaitNs of the GPU's global
// timer); one that runs out records GB_ERR_TIMEOUT and the item is skipped.  A
// registration's virtual blocks and bodies are those of the per-phase launches,
// so its results are bitwise the same in both forms.
enum { kItClear = 0, kItPrepare = 1, kItMsqImage = 2, kItMsqCD = 3, kItP1Image = 4, kItP1CD = 5, kItP2 = 6,
       kItStep = 7 };

struct RegSync {  // per running registration; zeroed when the tables are built
  unsigned prep, p1, eval, step;
};

struct LaunchSync {
  unsigned next;      // next queue entry of this launch
  unsigned finished;  // blocks done with this launch
  unsigned base;      // iterations launched since the tables were built
  int error;          // GB_ERR_TIMEOUT once a dependency wait ran out
};

constexpr unsigned long long kDepWaitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Thread 0 waits until *c >= target (bounded); the whole block then proceeds.
__device__ __forceinline__ bool block_wait_at_least(const unsigned* c, unsigned target, int* err) {
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    if (ld_acquire(c) < target) {
      const unsigned long long t0 = global_ns();
      unsigned polls = 0;
      while (ld_acquire(c) < target) {
        __nanosleep(polls < 64 ? 32 : 256);
        if ((++polls & 255u) == 0 && global_ns() - t0 > kDepWaitNs) {
          atomicExch(err, GB_ERR_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  const bool r = ok != 0;
  __syncthreads();
  return r;
}

// The block is done with its item: its writes, then the counter.
__device__ __forceinline__ void block_signal(unsigned* c) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(c, 1u);
  }
}

// The bodies out of line: each gets its own register allocation, and a call costs
// once per work item.
static __device__ __noinline__ void item_msq(const EvalArgs& a, VGrid vg, bool cd) {
  if (cd) msq_affine_body<kGradCentralDifference>(a, vg);
  else msq_affine_body<kGradImage>(a, vg);
}
static __device__ __noinline__ void item_pass1(const EvalArgs& a, VGrid vg, bool cd) {
  if (cd) mattes_pass1_affine_body<kGradCentralDifference>(a, vg);
  else mattes_pass1_affine_body<kGradImage>(a, vg);
}
static __device__ __noinline__ void item_pass2(const EvalArgs& a, VGrid vg) { mattes_pass2_affine_body<false>(a, vg); }
static __device__ __noinline__ void item_step(const StepArgs* steps, int r) {
  const StepArgs sarg = steps[r];
  step_block<32>(sarg);  // every thread: its barrier is the block's
}
static __device__ __noinline__ void item_prepare(const EvalArgs* regs, int r, int e) {
  const EvalArgs& a = regs[r];
  affine_const_entry(e, a.params, a.center, a.m_p2i, a.m_origin, a.dense ? a.v_i2p : nullptr, a.v_origin,
                     *const_cast<EvalConsts*>(a.consts));
}

// meta[r] = (virtual blocks of the MeanSquares pass or of Mattes pass 1, of Mattes pass 2 (0: MeanSquares))
__global__ void __launch_bounds__(kBlock, 3) k_batch_persistent(const EvalArgs* __restrict__ regs,
                                                             const StepArgs* __restrict__ steps,
                                                             const ClearItem* __restrict__ clears,
                                                             const int4* __restrict__ items,
                                                             const int2* __restrict__ meta, unsigned per_iter,
                                                             unsigned iters, LaunchSync* ls, RegSync* rs) {
  __shared__ EvalArgs sa;
  __shared__ unsigned s_q, s_base;
  if (threadIdx.x == 0) s_base = *reinterpret_cast<volatile unsigned*>(&ls->base);
  __syncthreads();
  const unsigned base = s_base;
  const unsigned total = per_iter * iters;
  for (;;) {
    if (threadIdx.x == 0) s_q = atomicAdd(&ls->next, 1u);
    __syncthreads();
    const unsigned q = s_q;
    __syncthreads();
    if (q >= total) break;
    const unsigned it = base + q / per_iter;  // iteration since the tables were built
    const int4 w = __ldg(items + q % per_iter);
    const int r = w.y;
    RegSync* R = rs + r;
    const int2 nv = __ldg(meta + r);
    switch (w.x) {
      case kItClear:
      case kItPrepare: {
        const bool ok = block_wait_at_least(&R->step, it, &ls->error);
        const ClearItem ci = clears[r];
        if (ok && !__ldcg(ci.halt)) {
          if (w.x == kItClear) {
            for (long long k = threadIdx.x; k < ci.words; k += blockDim.x) ci.p[k] = 0ull;
          } else if (threadIdx.x == 0) {
            item_prepare(regs, r, w.z);
          }
        }
        block_signal(&R->prep);
        break;
      }
      case kItMsqImage:
      case kItMsqCD:
      case kItP1Image:
      case kItP1CD: {
        const bool ok = block_wait_at_least(&R->prep, (1u + kConstEntries) * (it + 1u), &ls->error);
        if (ok) {
          load_reg(regs, r, sa);
          const VGrid vg{w.z, w.w};
          if (w.x <= kItMsqCD) item_msq(sa, vg, w.x == kItMsqCD);
          else item_pass1(sa, vg, w.x == kItP1CD);
        }
        block_signal(w.x <= kItMsqCD ? &R->eval : &R->p1);
        break;
      }
      case kItP2: {
        const bool ok = block_wait_at_least(&R->p1, (unsigned)nv.x * (it + 1u), &ls->error);
        if (ok) {
          load_reg(regs, r, sa);
          item_pass2(sa, VGrid{w.z, w.w});
        }
        block_signal(&R->eval);
        break;
      }
      default: {  // kItStep
        const unsigned want = (unsigned)(nv.y > 0 ? nv.y : nv.x) * (it + 1u);
        const bool ok = block_wait_at_least(&R->eval, want, &ls->error);
        if (ok) item_step(steps, r);
        block_signal(&R->step);
        break;
      }
    }
  }
  // the last block to finish readies the counters for the next launch
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ls->finished, 1u) == gridDim.x - 1) {
      ls->next = 0u;
      ls->finished = 0u;
      ls->base = base + iters;
      __threadfence();
    }
  }
}

// out[r] = halt word of registration r; out[n] = the number still running;
// out[n + 1] = the persistent launches' error word (0 without them).
__global__ void __launch_bounds__(kBlock) k_batch_halts(const StepArgs* __restrict__ steps, int n, int* out,
                                                        const LaunchSync* ls) {
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
  if (threadIdx.x == 0) {
    out[n] = running;
    out[n + 1] = ls ? __ldcg(&ls->error) : 0;
  }
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
  bool persistent = false;  // k_batch_persistent: several iterations per launch
  std::vector<Reg> regs;
  // tables of the running registrations
  std::vector<int> active;
  DevBuf<EvalArgs> d_eval;
  DevBuf<StepArgs> d_step;
  DevBuf<ClearItem> d_clear;
  DevBuf<int4> d_work;
  DevBuf<int> d_halts;
  int* h_halts = nullptr;  // pinned, 2 slots of (capacity + 2)
  // the persistent form's tables: one iteration's items, per-registration pass sizes,
  // completion counters, the launch counters
  DevBuf<int4> d_items;
  DevBuf<int2> d_meta;
  DevBuf<RegSync> d_rs;
  DevBuf<LaunchSync> d_ls;
  unsigned per_iter = 0;
  int pgrid = 0;
  size_t psmem = 0;
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

// Kernel arguments of one persistent launch of `iters` iterations.
struct PersistentArgs {
  const EvalArgs* regs;
  const StepArgs* steps;
  const ClearItem* clears;
  const int4* items;
  const int2* meta;
  unsigned per_iter, iters;
  LaunchSync* ls;
  RegSync* rs;
  std::vector<void*> data() {
    return {&regs, &steps, &clears, &items, &meta, &per_iter, &iters, &ls, &rs};
  }
};

PersistentArgs persistent_args_of(gb_batch* b, unsigned iters) {
  return PersistentArgs{b->d_eval.p, b->d_step.p, b->d_clear.p, b->d_items.p, b->d_meta.p, b->per_iter, iters,
                        b->d_ls.p, b->d_rs.p};
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
  // the persistent form's items of one iteration: clears, constants, the first passes
  // (largest registrations first, so the longest chains start earliest), pass 2, steps
  std::vector<int> order(n);
  for (size_t k = 0; k < n; ++k) order[k] = (int)k;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return b->regs[(size_t)b->active[(size_t)x]].m->nsamples > b->regs[(size_t)b->active[(size_t)y]].m->nsamples;
  });
  std::vector<int4> items;
  std::vector<int2> meta(n, make_int2(0, 0));
  for (size_t k = 0; k < n; ++k) items.push_back(make_int4(kItClear, (int)k, 0, 0));
  for (size_t k = 0; k < n; ++k)
    for (int e = 0; e < kConstEntries; ++e) items.push_back(make_int4(kItPrepare, (int)k, e, 0));
  for (int k : order) {
    gb_metric* m = b->regs[(size_t)b->active[(size_t)k]].m;
    const bool cd = m->grad_source == GB_GRADIENT_CENTRAL_DIFFERENCE;
    const bool msq = m->kind == GB_METRIC_MEAN_SQUARES;
    const int64_t nv = vblocks(m->nsamples, b->spb[msq ? kSpbMsq : kSpbPass1]);
    const int kind = msq ? (cd ? kItMsqCD : kItMsqImage) : (cd ? kItP1CD : kItP1Image);
    for (int64_t v = 0; v < nv; ++v) items.push_back(make_int4(kind, k, (int)v, (int)nv));
    meta[(size_t)k].x = (int)nv;
    if (!msq) meta[(size_t)k].y = (int)vblocks(m->nsamples, b->spb[kSpbPass2]);
  }
  for (int k : order)
    for (int v = 0; v < meta[(size_t)k].y; ++v) items.push_back(make_int4(kItP2, k, v, meta[(size_t)k].y));
  for (size_t k = 0; k < n; ++k) items.push_back(make_int4(kItStep, (int)k, 0, 0));
  b->per_iter = (unsigned)items.size();
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
  GB_B_CUDA(b->d_halts.alloc_on(b->stream, n + 2));
  if (b->h_halts_cap < n + 2) {
    if (b->h_halts) cudaFreeHost(b->h_halts);
    b->h_halts = nullptr;
    GB_B_CUDA(cudaMallocHost(&b->h_halts, 2 * sizeof(int) * (n + 2)));
    b->h_halts_cap = n + 2;
  }
  GB_B_CUDA(b->d_items.alloc_on(b->stream, items.size()));
  GB_B_CUDA(b->d_meta.alloc_on(b->stream, n));
  GB_B_CUDA(b->d_rs.alloc_on(b->stream, n));
  GB_B_CUDA(b->d_ls.alloc_on(b->stream, 1));
  if (b->persistent) {
    b->psmem = std::max(b->smem1, b->smem2);
    GB_B_CUDA(cudaFuncSetAttribute(k_batch_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->psmem));
    int per_sm = 0;
    GB_B_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_persistent, kBlock, b->psmem));
    b->pgrid = std::max(1, per_sm) * b->ctx->sm_count;
  }
  cudaStream_t st = b->stream;
  GB_B_CUDA(cudaMemcpyAsync(b->d_eval.p, ev.data(), sizeof(EvalArgs) * n, cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemcpyAsync(b->d_step.p, sa.data(), sizeof(StepArgs) * n, cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemcpyAsync(b->d_clear.p, ci.data(), sizeof(ClearItem) * n, cudaMemcpyHostToDevice, st));
  if (!all.empty())
    GB_B_CUDA(cudaMemcpyAsync(b->d_work.p, all.data(), sizeof(int4) * all.size(), cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemcpyAsync(b->d_items.p, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemcpyAsync(b->d_meta.p, meta.data(), sizeof(int2) * n, cudaMemcpyHostToDevice, st));
  GB_B_CUDA(cudaMemsetAsync(b->d_rs.p, 0, sizeof(RegSync) * n, st));
  GB_B_CUDA(cudaMemsetAsync(b->d_ls.p, 0, sizeof(LaunchSync), st));
  GB_B_CUDA(cudaStreamSynchronize(st));  // the host tables are pageable
  if (b->use_graph && !b->persistent) {
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
  b->d_items.reset();
  b->d_meta.reset();
  b->d_rs.reset();
  b->d_ls.reset();
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

extern "C" int gb_batch_set_persistent(gb_batch* b, int on) {
  if (!b) return fail(GB_ERR_BAD_ARG, "null batch");
  b->persistent = on != 0;
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
  GB_B_CUDA(launch_dep(st, k_batch_halts, 1u, kBlock, 0, (const StepArgs*)b->d_step.p, n, b->d_halts.p,
                       (const LaunchSync*)b->d_ls.p));
  GB_B_CUDA(cudaMemcpyAsync(b->h_halts, b->d_halts.p, sizeof(int) * (n + 2), cudaMemcpyDeviceToHost, st));
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
  NvtxRange range(__func__);
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
      if (b->persistent) {
        // one launch for all k iterations (plain launch: the next must not start early)
        PersistentArgs pa = persistent_args_of(b, (unsigned)k);
        std::vector<void*> av = pa.data();
        GB_B_CUDA(cudaLaunchKernel((const void*)k_batch_persistent, dim3((unsigned)b->pgrid), dim3(kBlock),
                                   av.data(), b->psmem, st));
      } else {
        for (int64_t i = 0; i < k; ++i) {
          if (b->exec) {
            GB_B_CUDA(cudaGraphLaunch(b->exec, st));
          } else {
            const int rc = enqueue_iteration(b, true);
            if (rc) return rc;
          }
        }
      }
      done += k;
      b->iterations += k;
      batch = std::min<int64_t>(batch * 2, 16);
      int* hh = b->h_halts + slot * (n + 2);
      GB_B_CUDA(launch_dep(st, k_batch_halts, 1u, kBlock, 0, (const StepArgs*)b->d_step.p, n, b->d_halts.p,
                           (const LaunchSync*)b->d_ls.p));
      GB_B_CUDA(cudaMemcpyAsync(hh, b->d_halts.p, sizeof(int) * (n + 2), cudaMemcpyDeviceToHost, st));
      GB_B_CUDA(cudaEventRecord(b->ev[slot], st));
      if (pending) {
        GB_B_CUDA(cudaEventSynchronize(b->ev[slot ^ 1]));
        const int* ph = b->h_halts + (slot ^ 1) * (n + 2);
        if (ph[n + 1] != 0)
          return fail(GB_ERR_TIMEOUT, "batched iteration: a dependency wait ran out in the persistent kernel");
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
