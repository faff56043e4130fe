// gb_corr_bspline.cuh -- CorrelationImageToImageMetricv4 under B-spline and
// [affine, B-spline] composite transforms.
//
// The affine kernels accumulate fdm = sum f1 J^T g and mdm = sum m1 J^T g directly
// (12 entries each).  The B-spline Jacobian has 192 nonzeros per sample, so here
// the derivative 2 fm / (f2 m2) (fdm - fm / m2 mdm)
// (itkCorrelationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:62-130) is
// formed by linearity as sum_s a_s W_s with the per-sample factor
// a_s = 2 fm / (f2 m2) (f1_s - fm / m2 m1_s) M^T g_s, once fm, f2, m2 are known,
// and the B-spline chunk and parameter kernels do the sparse sums:
//   k_corr_mean_bspline    B-spline position, moving value and M^T g cached; sums of
//                          f and m over the valid points; the last block writes the averages;
//   k_corr_sums_bspline    from the cache: fm, f2, m2 with the averages as double-float;
//                          the last block writes value, status and the factor's two scalars;
//   k_corr_factor_bspline  a_s (times N: the parameter kernel divides by the count) into the cache.
#pragma once

#include "gb_bspline.cuh"
#include "gb_kernels.cuh"

namespace gb {

template <int GRAD, bool SMEM>
__global__ void __launch_bounds__(kBlock) k_corr_mean_bspline(EvalArgs a) {
  extern __shared__ float4 nodes_sh[];
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][2];
  __shared__ double blk[2], fin[2];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  const float4* nodes = stage_nodes<SMEM>(a, nodes_sh);
  __syncthreads();
  KahanF acc[2];
  acc[0].zero();
  acc[1].zero();
  unsigned nv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 s = __ldcs(a.samples + i);
    const float4 su = __ldcs(a.sup + i);
    bool has_jac;
    const DFPos p = bspline_position(K, nodes, a, s, su, has_jac);
    float m = 0.f;
    float3 g = make_float3(0.f, 0.f, 0.f);
    const bool ok = eval_moving<GRAD>(a, p, a.with_derivative != 0 && has_jac, m, g);
    if (a.with_derivative) {
      const float3 gm = has_jac ? grad_map(K, g) : make_float3(0.f, 0.f, 0.f);
      __stcg(a.cache + i, ok ? make_float4(m, gm.x, gm.y, gm.z) : make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f));
    }
    if (!ok) continue;
    acc[0].add(s.w);
    acc[1].add(m);
    ++nv;
  }
  block_count(nv, a.acc_n);
  block_sums<2>(acc, red, blk);
  if (!grid_sums<2>(blk, a.part, a.grp, a.tickets + kTicketMain, fin)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    a.marg[2] = N > 0 ? fin[0] / (double)N : 0.0;  // m_AverageFix
    a.marg[3] = N > 0 ? fin[1] / (double)N : 0.0;  // m_AverageMov
  }
}

// The value (and, with the derivative, the cache's moving values) give fm, f2, m2.
// GetValue runs k_corr_mean_bspline without the derivative: then the moving values
// are not cached, so this kernel re-evaluates them (VALUE_ONLY).
template <int GRAD, bool SMEM, bool VALUE_ONLY>
__global__ void __launch_bounds__(kBlock) k_corr_sums_bspline(EvalArgs a) {
  extern __shared__ float4 nodes_sh[];
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][3];
  __shared__ double blk[3], fin[3];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  const float4* nodes = VALUE_ONLY ? stage_nodes<SMEM>(a, nodes_sh) : nullptr;
  float afh, afl, amh, aml;
  split_df(__ldcg(&a.marg[2]), afh, afl);
  split_df(__ldcg(&a.marg[3]), amh, aml);
  __syncthreads();
  KahanF acc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) acc[k].zero();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float f = __ldcs(&a.samples[i].w);
    float m;
    if (VALUE_ONLY) {
      const float4 s = __ldcs(a.samples + i);
      const float4 su = __ldcs(a.sup + i);
      bool has_jac;
      float3 g;
      if (!eval_moving<GRAD>(a, bspline_position(K, nodes, a, s, su, has_jac), false, m, g)) continue;
    } else {
      m = __ldcg(&a.cache[i].x);
      if (!(m == m)) continue;
    }
    const float f1 = __fsub_rn(__fsub_rn(f, afh), afl);
    const float m1 = __fsub_rn(__fsub_rn(m, amh), aml);
    acc[0].add(f1 * m1);
    acc[1].add(f1 * f1);
    acc[2].add(m1 * m1);
  }
  block_sums<3>(acc, red, blk);
  if (!grid_sums<3>(blk, a.part + kPartPass2, a.grp, a.tickets + kTicketPass2, fin)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    a.out[1] = (double)N;
    a.marg[4] = 0.0;
    a.marg[5] = 0.0;
    if (N == 0) {  // VerifyNumberOfValidPoints: a warning, value max, zero derivative
      a.out[0] = DBL_MAX;
      *a.status = GB_ERR_NO_VALID_POINTS;
      return;
    }
    *a.status = GB_OK;
    const double fm = fin[0], f2 = fin[1], m2 = fin[2];
    const double m2f2 = m2 * f2;
    if (m2f2 <= DBL_EPSILON) {
      a.out[0] = 0.0;
      return;
    }
    a.out[0] = -1.0 * fm * fm / m2f2;
    a.marg[4] = 2.0 * fm / (f2 * m2);  // the derivative's scale
    a.marg[5] = fm / m2;               // the weight of mdm
  }
}

__global__ void __launch_bounds__(kBlock) k_corr_factor_bspline(EvalArgs a) {
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  float afh, afl, amh, aml;
  split_df(__ldcg(&a.marg[2]), afh, afl);
  split_df(__ldcg(&a.marg[3]), amh, aml);
  const unsigned long long N = __ldcg(a.acc_n);
  // N sc: the parameter kernel divides the sums by the count N
  const float nsc = (float)((double)N * __ldcg(&a.marg[4]));
  const float r = (float)__ldcg(&a.marg[5]);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 c = __ldcg(a.cache + i);
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (c.x == c.x) {
      const float f = __ldcs(&a.samples[i].w);
      const float f1 = __fsub_rn(__fsub_rn(f, afh), afl);
      const float m1 = __fsub_rn(__fsub_rn(c.x, amh), aml);
      const float w = nsc * fmaf(-r, m1, f1);
      out = make_float4(w * c.y, w * c.z, w * c.w, 1.f);
    }
    __stcg(a.cache + i, out);
  }
}

}  // namespace gb
