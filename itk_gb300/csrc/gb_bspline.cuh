// gb_bspline.cuh -- B-spline (order 3) and [affine, B-spline] composite moving transforms.
//
// Reference semantics (paths relative to ITK's Modules/):
//   BSplineTransform::TransformPoint / Jacobian   Core/Transform/include/itkBSplineTransform.hxx:478-652
//   BSplineInterpolationWeightFunction::Evaluate  Core/Common/include/itkBSplineInterpolationWeightFunction.hxx:43-93
//   CompositeTransform point and chain rule        Core/Transform/include/itkCompositeTransform.hxx:60-70,466-580
//
// Each sample's support (first node, in-cell fractions, valid-region flag) is
// fixed by its virtual point, so Initialize computes it once in FP64 with the
// reference's InsideValidRegion rules.  Per evaluation a sample needs the 64
// tensor weights and the displacement sum over the coefficients (staged in
// shared memory when they fit).  The Jacobian has 192 nonzeros per sample,
//   (J^T g)[n_k + d * nper] = W_k (M^T g)_d,
// M the composite's initial affine (identity for a plain B-spline).  Samples
// are sorted by B-spline cell; a chunk kernel sums W_k a_s over each run of
// same-cell samples (one thread per support node), and a gather kernel adds,
// for every parameter, the chunk sums of the cells whose support holds its
// node -- in a fixed order, with no atomics.
#pragma once

#include "gb_kernels.cuh"

namespace gb {

constexpr int kChunkLen = 256;     // samples per chunk (at most); also the chunk kernel's block size
constexpr int kParamsBlock = 256;  // k_bspline_params: 8 nodes per block (warp form) or 1 (block form)

__device__ __forceinline__ void unpack_support(float w, int& sx, int& sy, int& sz, bool& valid) {
  const unsigned u = __float_as_uint(w);
  sx = (int)(u & 1023u);
  sy = (int)((u >> 10) & 1023u);
  sz = (int)((u >> 20) & 1023u);
  valid = ((u >> 30) & 1u) != 0u;
}

// Weights of the 4 nodes along one axis at in-cell position t in [0, 1]:
// BSplineKernelFunction<3> at t+1, t, t-1, t-2; 1/6 applied as hi + lo parts.
__device__ __forceinline__ void bspline_basis(float t, float* w) {
  constexpr float c_hi = 0.16666667163372039795f;  // nearest float to 1/6
  constexpr float c_lo = -4.96705373e-09f;         // 1/6 - c_hi
  float w6[4];
  parzen6(t, w6);
#pragma unroll
  for (int k = 0; k < 4; ++k) w[k] = fmaf(w6[k], c_hi, w6[k] * c_lo);
}

// One coefficient node (c_x, c_y, c_z, 0) from the FP64 parameters
// (BSplineTransform's parameter layout: all x coefficients, then y, then z).
__device__ __forceinline__ float4 node_from_params(const double* __restrict__ p, int nper, int n) {
  return make_float4((float)__ldg(p + n), (float)__ldg(p + nper + n), (float)__ldg(p + 2 * nper + n), 0.f);
}

#ifndef GB_KERNELS_HELPERS_ONLY
// Float4 node array from device-resident parameters (the host call converts on
// the host and uploads the nodes); one conversion per node per evaluation,
// rather than one per node in every block of the sample pass.
__global__ void k_prepare_bspline(EvalArgs a) {
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  if (a.clear_acc) clear_accumulators(a);
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < a.nper) a.nodes[n] = node_from_params(a.params, a.nper, n);
}
#endif  // GB_KERNELS_HELPERS_ONLY

// The nodes in shared memory (SMEM), else the global array.  A compile-time
// choice, so node reads compile to shared-memory loads rather than generic ones.
template <bool SMEM>
__device__ __forceinline__ const float4* stage_nodes(const EvalArgs& a, float4* sh) {
  if constexpr (SMEM) {
    for (int k = threadIdx.x; k < a.nper; k += blockDim.x) sh[k] = __ldcg(a.nodes + k);
    return sh;
  } else {
    return a.nodes;
  }
}

// Moving continuous index of one sample under the B-spline (+ initial affine):
// cidx = A x + b + P2I M u, A x + b in double-float, the displacement u in FP32.
// has_jac: inside the B-spline valid region (else the transform is the identity
// there and its Jacobian is zero, itkBSplineTransform.hxx:519-523,610-616).
__device__ __forceinline__ DFPos bspline_position(const EvalConsts& K, const float4* nodes, const EvalArgs& a,
                                                  const float4& s, const float4& su, bool& has_jac) {
  DFPos p = map_pos(K.map, s.x, s.y, s.z);
  int sx, sy, sz;
  bool valid;
  unpack_support(su.w, sx, sy, sz, valid);
  has_jac = valid;
  if (!valid) return p;
  float wx[4], wy[4], wz[4];
  bspline_basis(su.x, wx);
  bspline_basis(su.y, wy);
  bspline_basis(su.z, wz);
  float u0 = 0.f, u1 = 0.f, u2 = 0.f;
#pragma unroll
  for (int kz = 0; kz < 4; ++kz)
#pragma unroll
    for (int ky = 0; ky < 4; ++ky) {
      const float4* row = nodes + (sx + a.gx * ((sy + ky) + a.gy * (sz + kz)));
      const float wyz = wy[ky] * wz[kz];
#pragma unroll
      for (int kx = 0; kx < 4; ++kx) {
        const float W = wx[kx] * wyz;
        const float4 c = row[kx];
        u0 = fmaf(W, c.x, u0);
        u1 = fmaf(W, c.y, u1);
        u2 = fmaf(W, c.z, u2);
      }
    }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float corr = fmaf(K.Pm[3 * k], u0, fmaf(K.Pm[3 * k + 1], u1, K.Pm[3 * k + 2] * u2));
    float hs, he;
    two_sum(p.hi[k], corr, hs, he);
    he = __fadd_rn(he, p.lo[k]);
    p.hi[k] = __fadd_rn(hs, he);
    p.lo[k] = __fsub_rn(he, __fsub_rn(p.hi[k], hs));
  }
  return p;
}

__device__ __forceinline__ float3 grad_map(const EvalConsts& K, float3 g) {
  return make_float3(fmaf(K.Mg[0], g.x, fmaf(K.Mg[1], g.y, K.Mg[2] * g.z)),
                     fmaf(K.Mg[3], g.x, fmaf(K.Mg[4], g.y, K.Mg[5] * g.z)),
                     fmaf(K.Mg[6], g.x, fmaf(K.Mg[7], g.y, K.Mg[8] * g.z)));
}

#ifndef GB_KERNELS_HELPERS_ONLY
// MeanSquares, B-spline: value sum and count; per sample a = 2 (f - m) M^T g in the cache.
template <int GRAD, bool SMEM>
__global__ void __launch_bounds__(kBlock) k_msq_bspline(EvalArgs a) {
  extern __shared__ float4 nodes_sh[];
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][1];
  __shared__ double blk[1], fin[1];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  const float4* nodes = stage_nodes<SMEM>(a, nodes_sh);
  __syncthreads();
  KahanF acc[1];
  acc[0].zero();
  unsigned nv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 s = __ldcs(a.samples + i);
    const float4 su = __ldcs(a.sup + i);
    bool has_jac;
    const DFPos p = bspline_position(K, nodes, a, s, su, has_jac);
    float m;
    float3 g;
    float4 cache = make_float4(0.f, 0.f, 0.f, 0.f);
    if (eval_moving<GRAD>(a, p, a.with_derivative != 0 && has_jac, m, g)) {
      const float diff = s.w - m;  // MeanSquares...Threader.hxx:46
      acc[0].add(diff * diff);
      ++nv;
      if (has_jac) {
        const float3 gm = grad_map(K, g);
        const float t = 2.f * diff;
        cache = make_float4(t * gm.x, t * gm.y, t * gm.z, 1.f);
      }
    }
    if (a.with_derivative) __stcs(a.cache + i, cache);
  }
  block_count(nv, a.acc_n);
  block_sums<1>(acc, red, blk);
  if (!grid_sums<1>(blk, a.part, a.grp, a.tickets + kTicketMain, fin)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    a.out[1] = (double)N;
    if (N == 0) {
      a.out[0] = DBL_MAX;
      *a.status = GB_ERR_NO_VALID_POINTS;
    } else {
      a.out[0] = fin[0] / (double)N;
      *a.status = GB_OK;
    }
  }
}

// Dynamic shared memory of the B-spline Mattes pass 1: histogram, column sums,
// fixed counts, then (16-byte aligned) the nodes.
__host__ __device__ inline size_t mattes_bspline_node_offset(int B) {
  return ((size_t)8 * (B * B + B) + 4 * (size_t)B + 15) / 16 * 16;
}

// Mattes pass 1, B-spline: as k_mattes_pass1_affine, caching (term, M^T g).
template <int GRAD, bool SMEM>
__global__ void __launch_bounds__(kBlock, SMEM ? 4 : 3) k_mattes_pass1_bspline(EvalArgs a) {
  extern __shared__ unsigned long long smem_u64[];
  const int B = a.bins;
  unsigned long long* hist = smem_u64;
  unsigned long long* cs = smem_u64 + B * B;
  unsigned* fm = reinterpret_cast<unsigned*>(smem_u64 + B * B + B);
  float4* nodes_sh = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(smem_u64) + mattes_bspline_node_offset(B));
  __shared__ EvalConsts K;
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) hist[k] = 0ull;
  for (int k = threadIdx.x; k < B; k += blockDim.x) {
    fm[k] = 0u;
    cs[k] = 0ull;
  }
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  const float4* nodes = stage_nodes<SMEM>(a, nodes_sh);
  __syncthreads();
  unsigned nv = 0;
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  // the next iteration's record and support travel while this one is evaluated
  float4 s_next = base + lane < a.n ? __ldcs(a.samples + base + lane) : zero;
  float4 su_next = base + lane < a.n ? __ldcs(a.sup + base + lane) : zero;
  for (; base < a.n; base += stride) {
    const int64_t i = base + lane;
    const bool live = i < a.n;
    const float4 s = s_next, su = su_next;
    s_next = i + stride < a.n ? __ldcs(a.samples + i + stride) : zero;
    su_next = i + stride < a.n ? __ldcs(a.sup + i + stride) : zero;
    float m = 0.f;
    float3 g = make_float3(0.f, 0.f, 0.f);
    bool ok = false, has_jac = false;
    if (live) {
      const DFPos p = bspline_position(K, nodes, a, s, su, has_jac);
      ok = eval_moving<GRAD>(a, p, a.with_derivative != 0 && has_jac, m, g);
      ok = ok && !(m < a.mmin) && !(m > a.mmax);  // Mattes...Threader.hxx:238-245
    }
    const float term = fmaf(m - a.mmin, a.m_inv_bs, 2.f);
    if (a.with_derivative && live) {
      const float3 gm = has_jac ? grad_map(K, g) : make_float3(0.f, 0.f, 0.f);
      __stcs(a.cache + i, ok ? make_float4(term, gm.x, gm.y, gm.z)
                             : make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f));
    }
    int pdfm = 0;
    unsigned q[4] = {0u, 0u, 0u, 0u};
    const int fidx = __float_as_int(s.w);
    if (ok) {
      float t, w6[4];
      parzen_window(term, B, pdfm, t);
      parzen6(t, w6);
#pragma unroll
      for (int k = 0; k < 4; ++k) q[k] = (__float2uint_rn(w6[k] * kQScale) + 3u) / 6u;
    }
    hist_add_aggregated(ok, fidx * B + pdfm, fidx, q, hist, fm);
    nv += ok ? 1u : 0u;
  }
  // the derivative's table is formed by k_mattes_table, not by the last block
  mattes_pass1_epilogue(a, nv, hist, cs, fm, hw_grid(), false);
}

// One block per chunk of same-cell samples (at most kChunkLen = blockDim).
// Load phase: thread j stages sample j's 12 axis weights and its 3-vector
// a_s = 2 (f - m) M^T g (MeanSquares) or w(term) M^T g (Mattes,
// w = sum_k log(p/pm)[f][m_k] beta3'(m_k - term)).  Sum phase: thread t owns
// the 4 x-adjacent support nodes of row (ky, kz) = (t & 3, (t >> 2) & 3) over
// the sample slice t >> 4 (16 slices, slice s holding samples s, s + 16, ...): per
// sample one 16-byte load of the x weights, 12 FMAs.  The 16 slice sums of each
// output are then added in slice order.
constexpr int kChunkSlices = 16;
// Grid-stride over the chunks (one full wave of blocks): block b forms chunks b, b + G, ...
// The next chunk's per-sample inputs are loaded into registers while the current
// chunk is summed, and (Mattes) the log(p / pm) table is staged in shared memory
// (dynamic shared memory, bins^2 floats) once per block.
template <bool MATTES>
__global__ void __launch_bounds__(kChunkLen) k_bspline_chunks(EvalArgs a) {
  extern __shared__ float pr_sh[];
  __shared__ __align__(16) float W1[kChunkLen][12];
  __shared__ float4 AV[kChunkLen];
  __shared__ float qs[kChunkSlices][192];
  griddep_wait();
  if (halted(a)) return;
  const int B = a.bins;
  const int t = threadIdx.x;
  if (MATTES) {
    mattes_value_groups<true>(a);  // the value's group partials (blocks b, b + G, ...) and their sum
    for (int k = t; k < B * B; k += blockDim.x) pr_sh[k] = __ldcg(a.pratio + k);
  }
  // this thread's inputs of one chunk: the run, the sample's support, cache and fixed bin
  struct In {
    int4 ch;
    float4 su, c;
    int fbin;
  };
  auto fetch = [&](int cidx) {
    In in;
    in.ch = make_int4(0, 0, 0, 0);
    in.su = in.c = make_float4(0.f, 0.f, 0.f, 0.f);
    in.fbin = 0;
    if (cidx < a.nchunks) {
      in.ch = __ldg(a.chunks + cidx);
      if (t < in.ch.y - in.ch.x) {
        const int64_t i = (int64_t)in.ch.x + t;
        in.su = __ldg(a.sup + i);
        in.c = __ldcg(a.cache + i);
        if (MATTES) in.fbin = __float_as_int(__ldg(&a.samples[i].w));
      }
    }
    return in;
  };
  In cur = fetch(blockIdx.x);
  __syncthreads();  // the staged table
  for (int cidx = blockIdx.x; cidx < a.nchunks; cidx += gridDim.x) {
    const In nxt = fetch(cidx + gridDim.x);  // in flight while this chunk is summed
    const int len = cur.ch.y - cur.ch.x;
    if (t < len) {
      float4 av = make_float4(0.f, 0.f, 0.f, 0.f);
      if (MATTES) {
        const float4 c = cur.c;
        if (c.x == c.x) {
          int pdfm;
          float tt, d[4];
          parzen_window(c.x, B, pdfm, tt);
          parzen_deriv(tt, d);
          const float* row = pr_sh + cur.fbin * B + pdfm;
          const float w = row[0] * d[0] + row[1] * d[1] + row[2] * d[2] + row[3] * d[3];
          av = make_float4(w * c.y, w * c.z, w * c.w, 0.f);
        }
      } else {
        av = make_float4(cur.c.x, cur.c.y, cur.c.z, 0.f);
      }
      bspline_basis(cur.su.x, &W1[t][0]);
      bspline_basis(cur.su.y, &W1[t][4]);
      bspline_basis(cur.su.z, &W1[t][8]);
      AV[t] = av;
    }
    __syncthreads();
    // slice sl sums samples sl, sl + 16, ...: the two half-warps read adjacent rows of
    // W1 and AV, in different shared-memory banks
    const int ky = t & 3, kz = (t >> 2) & 3, sl = t >> 4;
    float acc[4][3];
#pragma unroll
    for (int kx = 0; kx < 4; ++kx) acc[kx][0] = acc[kx][1] = acc[kx][2] = 0.f;
    for (int j = sl; j < len; j += kChunkSlices) {
      const float4 wx = *reinterpret_cast<const float4*>(&W1[j][0]);
      const float wyz = W1[j][4 + ky] * W1[j][8 + kz];
      const float4 v = AV[j];
      const float w[4] = {wx.x * wyz, wx.y * wyz, wx.z * wyz, wx.w * wyz};
#pragma unroll
      for (int kx = 0; kx < 4; ++kx) {
        acc[kx][0] = fmaf(w[kx], v.x, acc[kx][0]);
        acc[kx][1] = fmaf(w[kx], v.y, acc[kx][1]);
        acc[kx][2] = fmaf(w[kx], v.z, acc[kx][2]);
      }
    }
    const int k0 = 4 * ky + 16 * kz;
#pragma unroll
    for (int kx = 0; kx < 4; ++kx) {
      qs[sl][k0 + kx] = acc[kx][0];
      qs[sl][64 + k0 + kx] = acc[kx][1];
      qs[sl][128 + k0 + kx] = acc[kx][2];
    }
    __syncthreads();
    if (t < 192) {
      float sum = qs[0][t];
#pragma unroll
      for (int q = 1; q < kChunkSlices; ++q) sum = __fadd_rn(sum, qs[q][t]);
      a.chunk_part[(size_t)cidx * 192 + t] = sum;
    }
    __syncthreads();  // the next chunk overwrites W1, AV and qs
    cur = nxt;
  }
  griddep_launch_dependents();
}

// For each node n and its three parameters (n + d * nper): the sum of the
// chunk sums of every cell whose 4x4x4 support holds n, listed at Initialize in
// node_entries (chunk * 192 + support position).  Compensated FP32 over the
// list, fixed XOR trees, FP64 only for the metric's scale (1/N for MeanSquares,
// -1/(binsize N) for Mattes, MeanSquares...Threader.hxx:71-79,
// Mattes...Threader.hxx:446-457).  BLOCK = false: one warp per node (lane-strided
// list); BLOCK = true, for coarse grids whose nodes hold thousands of entries:
// one block per node (thread-strided list, warps added in fixed order), so the
// few hundred nodes still spread over every SM.
template <bool MATTES, bool BLOCK>
__global__ void __launch_bounds__(kParamsBlock) k_bspline_params(EvalArgs a) {
  const int n = BLOCK ? (int)blockIdx.x : (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  // MeanSquares: the status of the value pass, scale 1 / N; Mattes: the scale formed by
  // the table kernel (0 unless the status is OK), and block 0 writes the value summed by
  // the chunk kernel's last group warp, the count and the status
  double scale;
  if (MATTES) {
    scale = __ldcg(&a.marg[2]);
  } else {
    __shared__ double scale_s;  // FP64 division: once per block
    if (threadIdx.x == 0) {
      const unsigned long long N = __ldcg(a.acc_n);
      scale_s = (__ldcg(a.status) == GB_OK && N > 0) ? 1.0 / (double)N : 0.0;
    }
    __syncthreads();
    scale = scale_s;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    a.out[1] = (double)N;
    if (MATTES) {
      const int st = mattes_status(a);
      *a.status = st;
      a.out[0] = st == GB_OK ? -1.0 * __ldcg(&a.part[kPartValue]) : 0.0;
    }
  }
  if (n >= a.nper) return;
  const int e0 = __ldg(a.node_first + n), e1 = __ldg(a.node_first + n + 1);
  KahanF s0, s1, s2;
  s0.zero();
  s1.zero();
  s2.zero();
  const int first = BLOCK ? (int)threadIdx.x : lane;
  const int step = BLOCK ? (int)blockDim.x : 32;
#pragma unroll 4
  for (int e = e0 + first; e < e1; e += step) {
    const float* src = a.chunk_part + __ldg(a.node_entries + e);
    s0.add(__ldcg(src));
    s1.add(__ldcg(src + 64));
    s2.add(__ldcg(src + 128));
  }
  float t0 = warp_sum(s0.value()), t1 = warp_sum(s1.value()), t2 = warp_sum(s2.value());
  if (BLOCK) {
    __shared__ float wsum[kParamsBlock / 32][3];
    const int w = threadIdx.x >> 5;
    if (lane == 0) {
      wsum[w][0] = t0;
      wsum[w][1] = t1;
      wsum[w][2] = t2;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    KahanF b0, b1, b2;
    b0.zero();
    b1.zero();
    b2.zero();
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      b0.add(wsum[k][0]);
      b1.add(wsum[k][1]);
      b2.add(wsum[k][2]);
    }
    t0 = b0.value();
    t1 = b1.value();
    t2 = b2.value();
  }
  if (lane == 0) {
    a.out[2 + n] = (double)t0 * scale;
    a.out[2 + a.nper + n] = (double)t1 * scale;
    a.out[2 + 2 * a.nper + n] = (double)t2 * scale;
  }
}
#endif  // GB_KERNELS_HELPERS_ONLY

}  // namespace gb
