// gb_field.cuh -- metric kernels under a displacement-field transform (local support).
//
// DisplacementFieldTransform<double,3> has local support: its Jacobian with
// respect to the parameters is the identity at the point's own field voxel
// (Filtering/DisplacementField/include/itkDisplacementFieldTransform.h:336-351),
// and the metric's derivative is a field over the virtual domain.  Each valid
// point's local derivative is added at 3 * (its virtual voxel) and not divided
// by the number of valid points
// (Registration/Metricsv4/include/itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:128-172,276-327).
//
//   MeanSquares: d[3v + i] += 2 (f - m) g_i
//     (Registration/Metricsv4/include/itkMeanSquaresImageToImageMetricv4GetValueAndDerivativeThreader.hxx:62-82);
//   Mattes: d[3v + i] = -1 / (binsize N) sum_k beta3'(arg_k) log(p / pm)[f][m_k] g_i
//     (LocalDerivativeByParzenBin and PRatioArray,
//      Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:300-351,394-412,
//      Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4.hxx:446-495).
//
// On the dense virtual grid every voxel holds at most one sample, so each
// thread writes its sample's three entries with plain stores; when every voxel
// holds one (field_full), invalid samples store zeros and the derivative needs
// no clearing.  A point set can put several samples in one voxel: their blocks
// are added with FP64 atomics (each sample's Mattes block uses its own joint-PDF
// bins; the reference keeps the last point's bins for the whole voxel, which is
// the same whenever a voxel holds one sample).
#pragma once

#include "gb_kernels.cuh"

namespace gb {

template <int TK>
__device__ __forceinline__ void field_store(const EvalArgs& a, unsigned voxel, bool ok, float c, float3 g) {
  double* d = a.out + 2 + 3ull * voxel;
  if (TK == kMapFieldDense) {
    if (!ok && !a.field_full) return;
    d[0] = ok ? (double)(c * g.x) : 0.0;
    d[1] = ok ? (double)(c * g.y) : 0.0;
    d[2] = ok ? (double)(c * g.z) : 0.0;
  } else {
    if (!ok || voxel == ~0u) return;
    atomicAdd(d, (double)(c * g.x));
    atomicAdd(d + 1, (double)(c * g.y));
    atomicAdd(d + 2, (double)(c * g.z));
  }
}

// MeanSquares under a displacement field: value = sum (f - m)^2 / N (fixed-order
// sums as the affine kernel), derivative blocks stored per sample.
template <int GRAD, int TK>
__global__ void __launch_bounds__(kBlock) k_msq_field(EvalArgs a) {
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][1];
  __shared__ double blk[1], fin[1];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  __syncthreads();
  KahanF acc[1];
  acc[0].zero();
  unsigned nv = 0;
  const bool deriv = a.with_derivative != 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float4 s_next = i < a.n ? __ldcs(a.samples + i) : zero;
  for (; i < a.n; i += stride) {
    // the next record travels while this sample is formed
    const float4 s = s_next;
    s_next = i + stride < a.n ? __ldcs(a.samples + i + stride) : zero;
    unsigned voxel = ~0u;
    const DFPos p = sample_pos<TK>(a, K, s, i, voxel);
    float m = 0.f;
    float3 g = make_float3(0.f, 0.f, 0.f);
    const bool ok = eval_moving<GRAD>(a, p, deriv, m, g);
    const float diff = ok ? s.w - m : 0.f;  // FixedImagePixelType diff
    if (ok) {
      acc[0].add(diff * diff);
      ++nv;
    }
    if (deriv) field_store<TK>(a, voxel, ok, 2.f * diff, field_grad(K, g));
  }
  block_count(nv, a.acc_n);
  block_sums<1>(acc, red, blk);
  if (!grid_sums<1>(blk, a.part, a.grp, a.tickets + kTicketMain, fin)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    if (N == 0) {  // VerifyNumberOfValidPoints: value max, derivative zero (no block was stored)
      a.out[0] = DBL_MAX;
      a.out[1] = 0.0;
      *a.status = GB_ERR_NO_VALID_POINTS;
    } else {
      a.out[0] = fin[0] / (double)N;
      a.out[1] = (double)N;
      *a.status = GB_OK;
    }
  }
}

// Mattes pass 1 under a displacement field: the affine kernel's histogram pass
// with the field's sample positions.
template <int GRAD, int TK>
__global__ void __launch_bounds__(kBlock, 4) k_mattes_pass1_field(EvalArgs a) {
  mattes_pass1_affine_body<GRAD, TK>(a, hw_grid());
}

// Mattes pass 2 under a displacement field, after k_mattes_finalize: each
// sample's block from its cached Parzen term and gradient and the log(p / pm)
// table.  Dynamic shared memory: the bins^2 table.
template <int TK>
__global__ void __launch_bounds__(kBlock) k_mattes_pass2_field(EvalArgs a) {
  extern __shared__ float pr[];
  __shared__ float coef;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  const int B = a.bins;
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) pr[k] = __ldcg(&a.pratio[k]);
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    coef = N > 0 ? (float)(-1.0 / (a.m_bs * (double)N)) : 0.f;  // -nFactor, Mattes...v4.hxx:415
  }
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 cc = __ldcs(a.cache + i);
    const float4 s = __ldcs(a.samples + i);
    const unsigned voxel = TK == kMapFieldDense
                               ? (unsigned)s.x + (unsigned)a.vnx * ((unsigned)s.y + (unsigned)a.vny * (unsigned)s.z)
                               : __ldg(a.voff + i);
    const bool ok = cc.x == cc.x;  // NaN term: rejected sample
    float w = 0.f;
    if (ok) {
      int pdfm;
      float tt, d[4];
      parzen_window(cc.x, B, pdfm, tt);
      parzen_deriv(tt, d);
      const float* row = pr + __float_as_int(s.w) * B + pdfm;
      w = row[0] * d[0] + row[1] * d[1] + row[2] * d[2] + row[3] * d[3];
    }
    field_store<TK>(a, voxel, ok, coef * w, make_float3(cc.y, cc.z, cc.w));
  }
}

}  // namespace gb
