// gb_step.cuh -- device state and step arithmetic of RegularStepGradientDescentOptimizerv4,
// shared by the single-registration loop (gb_optimizer.cu) and the batched
// engine (gb_batch.cu).
//
// Reference semantics (paths relative to ITK's Modules/):
//   AdvanceOneStep                    Numerics/Optimizersv4/include/itkRegularStepGradientDescentOptimizerv4.hxx:78-171
//   loop, best value, StopOptimization Numerics/Optimizersv4/include/itkGradientDescentOptimizerv4.hxx:59-169
//   Transform::UpdateTransformParameters  Core/Transform/include/itkTransform.hxx:69-121
//
// ||g||^2 and g . g_prev are compensated FP64 sums over a fixed tree of two-sum
// pairs (the reference runs a sequential Kahan loop; both are exact to about
// one rounding of the result).  Every other operation is the reference's,
// rounding for rounding (FP64, no contraction).
#pragma once

#include <cuda_runtime.h>

#include "../../include/itk_gb300.h"
#include "gb_device.cuh"

namespace gb {

constexpr int kStepBlock = 256;
constexpr int kStepMaxBlocks = 256;  // blocks of the multi-block step (grid-stride beyond 65536 parameters)

enum { kActNone = 0, kActStep = 1, kActRestoreBest = 2 };
enum { kRunning = -1 };

struct OptState {
  double relaxation;   // m_CurrentLearningRateRelaxation
  double value;        // m_CurrentMetricValue
  double best_value;   // m_CurrentBestValue
  double grad_mag;     // ||g|| of the last step
  double step_length;  // relaxation * learning rate of the last step
  double inv_mag;      // 1 / ||g||, the update factor
  long long iteration; // m_CurrentIteration
  int stop;            // GB_STOP_*, kRunning while the loop runs
  int halt;            // nonzero once stopped
  int status;          // metric status of the last evaluation
  int action;          // what the apply phase does this iteration
  int save_best;       // the apply phase copies the new position to the best parameters
  unsigned ticket;
  double part[kStepMaxBlocks][4];  // per block: (hi, lo) of ||g||^2 and of g . g_prev
};

struct StepArgs {
  const double* out;   // metric output [value, nvalid, derivative...]
  const int* status;   // metric status word
  double* params;
  double* prev;        // previous modified gradient (scaled, times relaxation * rate)
  double* grad;        // this iteration's scaled gradient
  double* best;        // best parameters (return-best)
  const double* inv_scales;
  OptState* st;
  long long P;
  long long max_iterations;  // NumberOfIterations (checked in-kernel by the batched step)
  double learning_rate, relaxation_factor, min_step, grad_tol;
  int return_best;
  int msq;  // MeanSquares / Correlation: no valid points is a warning (value max, derivative 0), not an error
};

// Compensated pair: the sum is hi + lo, |lo| <= ulp(hi) / 2.
struct DD {
  double hi, lo;
};

__device__ __forceinline__ DD dd_add(DD a, DD b) {
  const double s = __dadd_rn(a.hi, b.hi);
  const double bb = __dsub_rn(s, a.hi);
  const double e = __dadd_rn(__dsub_rn(a.hi, __dsub_rn(s, bb)), __dsub_rn(b.hi, bb));  // two-sum error
  const double t = __dadd_rn(__dadd_rn(a.lo, b.lo), e);
  const double hi = __dadd_rn(s, t);
  return {hi, __dsub_rn(t, __dsub_rn(hi, s))};
}

__device__ __forceinline__ DD dd_shfl_down(DD v, int off) {
  return {__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off)};
}

// Sum over a block of NT threads (32 or kStepBlock) in a fixed order (lane tree,
// then warp tree); the result is in thread 0.
template <int NT = kStepBlock>
__device__ __forceinline__ void block_dd2(DD& x, DD& y) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const DD ox = dd_shfl_down(x, off), oy = dd_shfl_down(y, off);
    if (lane < off) {
      x = dd_add(x, ox);
      y = dd_add(y, oy);
    }
  }
  if constexpr (NT == 32) return;
  __shared__ DD sx[NT / 32], sy[NT / 32];
  if (lane == 0) {
    sx[w] = x;
    sy[w] = y;
  }
  __syncthreads();
  if (w == 0) {
    constexpr int W = NT / 32;
    x = lane < W ? sx[lane] : DD{0.0, 0.0};
    y = lane < W ? sy[lane] : DD{0.0, 0.0};
#pragma unroll
    for (int off = W / 2; off > 0; off >>= 1) {
      const DD ox = dd_shfl_down(x, off), oy = dd_shfl_down(y, off);
      if (lane < off) {
        x = dd_add(x, ox);
        y = dd_add(y, oy);
      }
    }
  }
}

__device__ __forceinline__ bool metric_error(const StepArgs& s, int status) {
  return status != GB_OK && !(s.msq && status == GB_ERR_NO_VALID_POINTS);
}

// StopOptimization (itkGradientDescentOptimizerv4.hxx:59-68): with return-best,
// the value becomes the best value and the apply phase restores the best parameters.
__device__ __forceinline__ void stop_here(const StepArgs& s, OptState* S, int cond) {
  S->stop = cond;
  S->halt = 1;
  if (s.return_best) {
    S->value = S->best_value;
    S->action = kActRestoreBest;
  } else {
    S->action = kActNone;
  }
}

// The decisions of one iteration (one thread): the metric's status, ||g||^2 = x
// and g . g_prev = y summed over all parameters.
__device__ __forceinline__ void step_decide(const StepArgs& s, OptState* S, int status, DD x, DD y) {
  S->status = status;
  S->save_best = 0;
  const double value = __ldcg(s.out);
  S->value = value;
  if (metric_error(s, status)) {  // the metric threw: COSTFUNCTION_ERROR, no iteration counted
    stop_here(s, S, GB_STOP_COSTFUNCTION_ERROR);
    return;
  }
  const double mag = sqrt(__dadd_rn(x.hi, x.lo));
  S->grad_mag = mag;
  if (mag < s.grad_tol) {
    stop_here(s, S, GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE);
    S->iteration += 1;
    return;
  }
  const double sp = __dadd_rn(y.hi, y.lo);
  double relax = S->relaxation;
  if (sp < 0.0) relax = __dmul_rn(relax, s.relaxation_factor);
  S->relaxation = relax;
  const double step = __dmul_rn(relax, s.learning_rate);
  S->step_length = step;
  if (step < s.min_step) {
    stop_here(s, S, GB_STOP_STEP_TOO_SMALL);
    S->iteration += 1;
    return;
  }
  S->inv_mag = 1.0 / mag;
  S->action = kActStep;
  if (s.return_best && value < S->best_value) {
    S->best_value = value;
    S->save_best = 1;
  }
  S->iteration += 1;
}

// ModifyGradientByScalesOverSubRange for parameter j: g = derivative / scale,
// g_prev / scale; returns the two products of the sums.
__device__ __forceinline__ void step_terms(const StepArgs& s, long long j, double& q, double& r) {
  const double is = __ldg(s.inv_scales + j);
  const double g = __dmul_rn(__ldcg(s.out + 2 + j), is);
  const double gp = __dmul_rn(__ldcg(s.prev + j), is);
  s.grad[j] = g;
  q = __dmul_rn(g, g);
  r = __dmul_rn(g, gp);
}

// ModifyGradientByLearningRateOverSubRange, then UpdateTransformParameters(g, 1/||g||),
// or the return-best restore, for parameter j.
__device__ __forceinline__ void step_apply(const StepArgs& s, const OptState* S, int act, long long j) {
  if (act == kActRestoreBest) {
    s.params[j] = __ldcg(s.best + j);
    return;
  }
  if (act != kActStep) return;
  const double glr = __dmul_rn(__dmul_rn(__ldcg(s.grad + j), __ldcg(&S->relaxation)), s.learning_rate);
  s.prev[j] = glr;
  const double p = __dadd_rn(s.params[j], __dmul_rn(glr, __ldcg(&S->inv_mag)));
  s.params[j] = p;
  if (__ldcg(&S->save_best)) s.best[j] = p;
}

// One registration's whole step in one block of NT threads: the compensated sums,
// the decisions, the update, then the NumberOfIterations stop that the reference
// checks at the top of its next loop pass (itkGradientDescentOptimizerv4.hxx:82-89).
// Called by every thread of the block; threads from NT on take part only in its
// barrier (the batched engine's persistent kernel runs the step in larger blocks).
template <int NT>
__device__ __forceinline__ void step_block(const StepArgs& s) {
  OptState* S = s.st;
  // thread 0 reads the halt word for the block: thread 0 itself may set it below,
  // and every thread must take the same branch (the block's barrier follows)
  __shared__ int halted_s;
  if (threadIdx.x == 0) halted_s = __ldcg(&S->halt);
  __syncthreads();
  if (halted_s) return;
  const int status = __ldcg(s.status);
  const bool err = metric_error(s, status);
  const bool mine = (int)threadIdx.x < NT;
  DD q = {0.0, 0.0}, r = {0.0, 0.0};
  if (!err && mine)
    for (long long j = threadIdx.x; j < s.P; j += NT) {
      double qq, rr;
      step_terms(s, j, qq, rr);
      q = dd_add(q, DD{qq, 0.0});
      r = dd_add(r, DD{rr, 0.0});
    }
  block_dd2<NT>(q, r);
  __shared__ int act, fin_max;
  if (threadIdx.x == 0) {
    step_decide(s, S, status, q, r);
    int fm = 0;
    if (!S->halt && S->iteration >= s.max_iterations) {
      S->stop = GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS;
      S->halt = 1;
      fm = 1;
      if (s.return_best) S->value = S->best_value;
    }
    act = S->action;
    fin_max = fm;
  }
  __syncthreads();
  for (long long j = threadIdx.x; mine && j < s.P; j += NT) {
    step_apply(s, S, act, j);
    if (fin_max && s.return_best) s.params[j] = __ldcg(s.best + j);
  }
}

// Host side (gb_optimizer.cu).  opt_setup: StartOptimization of one registration
// (validation, the handle's optimizer buffers, initial state; synchronizes);
// opt_fetch: enqueue the copies of the final state and parameters; opt_collect:
// after those copies, the handle's parameters, the report and the status.
int opt_setup(gb_metric* m, const gb_regular_step_settings* cfg, const double* scales, int64_t nscales, StepArgs& a);
int opt_fetch(gb_metric* m, const StepArgs& a, cudaStream_t st);
int opt_collect(gb_metric* m, const StepArgs& a, gb_optimizer_report* report);

}  // namespace gb
