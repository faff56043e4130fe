// gb_kernels.cuh -- kernel argument blocks and the kernels of one metric
// evaluation (MeanSquares single pass; Mattes pass 1 / finalize / pass 2).
//
// Reference semantics restated here (paths relative to ITK's Modules/):
//   per-point skeleton   Registration/Metricsv4/include/itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:176-273
//   MeanSquares          Registration/Metricsv4/include/itkMeanSquaresImageToImageMetricv4GetValueAndDerivativeThreader.hxx:31-84
//   Mattes point         Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:220-387
//   Mattes results       Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4.hxx:358-542
//   affine Jacobian      Core/Transform/include/itkMatrixOffsetTransformBase.hxx:566-594
//
// Mattes derivative by linearity: instead of the reference's
// JointPDFDerivatives[f][m][mu] array (P x bins^2 scattered adds per sample),
// pass 2 re-reads each sample's cached Parzen term and gradient and forms
//   w = sum_k log(p/pm)[f][m_k] * beta3'(m_k - term),
//   derivative[mu] = -1/(binsize * N) * sum_samples w * (J^T grad)[mu],
// which is ComputeResults' contraction (Mattes...v4.hxx:446-461) reordered.
#pragma once

#include <cfloat>

#include "../../include/itk_gb300.h"
#include "gb_bulk.cuh"
#include "gb_device.cuh"

namespace gb {

enum { kGradImage = 0, kGradCentralDifference = 1 };

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 2048;          // grid cap of the evaluation kernels
constexpr int kTicketMain = 0;            // grid_sums of the MeanSquares kernel: [0, 128]
constexpr int kTicketFinalize = 160;      // last_block of the Mattes finalize
constexpr int kTicketPass2 = 192;         // grid_sums of Mattes pass 2: [192, 320]
constexpr int kTicketPass1 = 176;         // last_block of Mattes pass 1
constexpr int kTicketValue = 340;         // the Mattes derivative pass's value groups done
constexpr int kTicketCount = 352;
constexpr int kPartPass2 = 4096;          // offset of pass-2 partials (finalize blocks use [0, 4096))
constexpr int kPartValue = kPartPass2 - 1;  // the Mattes derivative pass's value (sum of the groups)
constexpr size_t kGroupOffset = kPartPass2 + (size_t)kMaxBlocks * 16;  // per-group partials: 128 groups x 16
constexpr size_t kMargOffset = kGroupOffset + 2048;     // [T, 1/T, derivative scale]
constexpr size_t kScratchDoubles = kMargOffset + 8;
constexpr int kFinalizeThreads = 32;
constexpr float kQScale = 67108864.f;  // 2^26 fixed point of histogram weights
constexpr double kQInv = 1.0 / 67108864.0;

// Per-evaluation transform constants (computed in FP64 once per evaluation,
// stored as FP32 / double-float).  Sample records hold "domain coordinates":
// the physical point for a sampled point set, the integer grid index for the
// dense virtual domain (so dense points are exact).  `map` takes domain
// coordinates to the moving continuous index; U, joff give the affine
// Jacobian's x - c = U u + joff.
struct EvalConsts {
  AffineDF map;
  float U[9];
  float joff[3];
  float Mg[9];  // B-spline paths: gradient -> (M^T g), M the initial affine of a composite (identity otherwise)
  float Pm[9];  // B-spline paths: physical displacement -> moving index offset, P2I M
  // displacement-field paths (map = the identity transform's map):
  AffineDF umap;  // physical displacement -> moving index offset (the moving image's P2I; b unused)
  AffineDF fmap;  // point set: physical point -> field continuous index
  float fdiag;    // nonzero: map and umap are diagonal (axis-aligned grids), the field
                  // position takes one product per axis (bitwise the same result)
};

__device__ __forceinline__ float3 jac_vec(const EvalConsts& K, float x, float y, float z) {
  return make_float3(fmaf(K.U[0], x, fmaf(K.U[1], y, fmaf(K.U[2], z, K.joff[0]))),
                     fmaf(K.U[3], x, fmaf(K.U[4], y, fmaf(K.U[5], z, K.joff[1]))),
                     fmaf(K.U[6], x, fmaf(K.U[7], y, fmaf(K.U[8], z, K.joff[2]))));
}

// MatrixOffsetTransformBase::ComputeOffset (itkMatrixOffsetTransformBase.hxx:612-631)
// composed with ImageBase::TransformPhysicalPointToContinuousIndex (itkImageBase.h:515-531).
__host__ __device__ inline void split_df(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)dadd(x, -(double)hi);
}

// dom2phys / dom_origin: domain coordinates -> physical point (the virtual
// grid's index-to-physical map for dense sampling; null for a point set).
// One output of the constants: e in [0, 9) the map's matrix entry (r, c) = (e / 3, e % 3),
// e in [9, 12) its offset row e - 9, e == 12 the Jacobian terms and M^T, e in
// [13, 22) the entry e - 13 of P2I M.  Rows of the physical-point -> moving-index
// map: A = P2I M, b = P2I (offset - origin_m), offset = t + c - M c.
constexpr int kConstEntries = 22;
__host__ __device__ inline void affine_const_entry(int e, const double* p, const double center[3],
                                                   const double m_p2i[9], const double m_origin[3],
                                                   const double* dom2phys, const double* dom_origin, EvalConsts& K) {
  const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, Z[3] = {0, 0, 0};
  const double* U = dom2phys ? dom2phys : I;
  const double* u0 = dom2phys ? dom_origin : Z;
  if (e == 12) {
    for (int i = 0; i < 9; ++i) K.U[i] = (float)U[i];
    for (int i = 0; i < 3; ++i) K.joff[i] = (float)(u0[i] - center[i]);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) K.Mg[r * 3 + c] = (float)p[c * 3 + r];  // M^T
    return;
  }
  if (e >= 13) {
    const int r = (e - 13) / 3, c = (e - 13) % 3;
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s = dadd(s, dmul(m_p2i[r * 3 + k], p[k * 3 + c]));
    K.Pm[r * 3 + c] = (float)s;
    return;
  }
  const int r = e < 9 ? e / 3 : e - 9;
  double Ar[3];
  for (int c = 0; c < 3; ++c) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s = dadd(s, dmul(m_p2i[r * 3 + k], p[k * 3 + c]));
    Ar[c] = s;
  }
  if (e < 9) {
    const int c = e % 3;
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s = dadd(s, dmul(Ar[k], U[k * 3 + c]));
    split_df(s, K.map.Ahi[e], K.map.Alo[e]);
    return;
  }
  double br = 0.0;
  for (int k = 0; k < 3; ++k) {
    double o = dadd(p[9 + k], center[k]);
    for (int j = 0; j < 3; ++j) o = dadd(o, -dmul(p[k * 3 + j], center[j]));
    br = dadd(br, dmul(m_p2i[r * 3 + k], dadd(o, -m_origin[k])));
  }
  for (int k = 0; k < 3; ++k) br = dadd(br, dmul(Ar[k], u0[k]));
  split_df(br, K.map.bhi[r], K.map.blo[r]);
}

__host__ __device__ inline void affine_consts(const double* p, const double center[3], const double m_p2i[9],
                                              const double m_origin[3], const double* dom2phys,
                                              const double* dom_origin, EvalConsts& K) {
  for (int e = 0; e < kConstEntries; ++e) affine_const_entry(e, p, center, m_p2i, m_origin, dom2phys, dom_origin, K);
}

struct EvalArgs {
  const float4* __restrict__ samples;
  int64_t n;
  const float4* __restrict__ mov4;  // (value, gx, gy, gz)
  const float* __restrict__ mov1;   // scalar moving image (central difference path)
  int nx, ny, nz;
  double m_p2i[9];
  double m_origin[3];
  float cd_hi[9], cd_lo[9];  // [3*d + k]: index-space offset along k of +0.5 spacing on physical axis d
  float cd_inv_delta[3];     // 1 / spacing[d]
  // transform
  const double* params;   // device parameters (device-resident path: k_prepare reads them)
  const EvalConsts* consts;
  int nparams;
  double center[3];       // affine centre
  int dense;              // sample records hold virtual grid indices
  double v_i2p[9];        // virtual grid index -> physical point (dense)
  double v_origin[3];
  // Mattes
  int bins;
  float mmin, mmax, m_inv_bs;
  double m_bs;
  // accumulators (cleared per evaluation)
  unsigned long long* acc_n;
  unsigned* tickets;            // [kTicketCount]
  unsigned long long* hist;     // bins*bins, 2^26 fixed point
  unsigned long long* fmarg;    // bins
  unsigned long long* colsum;   // bins: moving marginal, 2^26 fixed point
  // scratch (overwritten per evaluation)
  double* part;                 // per-block partials
  double* grp;                  // per-group partials
  double* marg;                 // [fixed-point total T, 1 / T]
  float4* cache;
  float* pratio;
  double* pdf_out;
  double* out;                  // [value, nvalid, derivative...]
  int* status;
  int with_derivative;
  // B-spline / composite transforms
  const float4* __restrict__ sup;    // per sample: (tx, ty, tz, packed support start | valid << 30)
  float4* nodes;                     // coefficient nodes (cx, cy, cz, 0), written by k_prepare_bspline
  int gx, gy, gz, nper;
  int nodes_smem;                    // evaluation kernels stage the nodes in shared memory
  const int4* __restrict__ chunks;   // (first sample, end sample, cell id, 0) of same-cell sample runs
  int nchunks;
  const int* __restrict__ node_first;    // per node: first entry in node_entries (nper + 1 values)
  const int* __restrict__ node_entries;  // chunk * 192 + support position of each (node, chunk) pair
  float* chunk_part;                 // nchunks x 192 per-chunk Jacobian partial sums
  // optimizer loop: nonzero once the optimizer has stopped; every evaluation
  // kernel then returns at once (iterations enqueued ahead become no-ops)
  const int* halt;
  // displacement-field transform (local support)
  const double* __restrict__ field;   // 3 doubles per virtual voxel: the transform's parameters
  int vnx, vny, vnz;                  // the virtual grid, which is the field's
  const unsigned* __restrict__ voff;  // point sets: each sample's nearest virtual voxel (~0u: outside)
  int field_full;                     // dense, one sample per voxel: every derivative entry is written
  // UseFloatingPointCorrection (MeanSquares, affine): each sample's local derivatives
  // truncated to 1 / fp_res and summed in FP64; 0 = off
  double fp_res;
  // fault injection (gb_metric_set_fault_injection): GB_FAULT_STALLED_COPY makes the
  // affine Mattes derivative pass issue none of its record copies
  int inject_stall;
  // the per-evaluation accumulators (acc_n, tickets, histogram, marginals) as 16-byte
  // words; with clear_acc the chain's first kernel zeroes them (no memset node)
  uint4* acc;
  int acc_words;
  int clear_acc;
  // the affine Mattes derivative pass takes the final histogram and marginals (hist,
  // fmarg, colsum: contiguous, 16-byte aligned) into shared memory with one bulk copy
  int hist_bulk;
};

// The optimizer's stop flag (read once per block, after the launch dependency).
__device__ __forceinline__ bool halted(const EvalArgs& a) { return a.halt != nullptr && __ldcg(a.halt) != 0; }

#ifndef GB_KERNELS_HELPERS_ONLY
// Device twin of the host constant computation (parameters already in HBM).
// 13 threads, one output each, so the FP64 dependency chains run side by side.
// One block (one warp, lane 0) per output: the entries take different code
// paths, and one SM's FP64 pipe would serve them one after another.
// Zeroes the accumulators, grid-strided over the launch (after the launch dependency,
// so no kernel of the previous evaluation still reads them).
__device__ __forceinline__ void clear_accumulators(const EvalArgs& a) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.acc_words; k += gridDim.x * blockDim.x)
    a.acc[k] = make_uint4(0u, 0u, 0u, 0u);
}

__global__ void k_prepare_affine(EvalArgs a, EvalConsts* out) {
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  if (a.clear_acc) clear_accumulators(a);
  const int e = blockIdx.x;
  if (threadIdx.x == 0 && e < kConstEntries)
    affine_const_entry(e, a.params, a.center, a.m_p2i, a.m_origin, a.dense ? a.v_i2p : nullptr, a.v_origin, *out);
}

#endif  // GB_KERNELS_HELPERS_ONLY

// The constants through L2 (not the read-only path): the batched engine's
// persistent kernel rewrites them between iterations within one launch.
__device__ __forceinline__ void load_consts(const EvalConsts* g, EvalConsts& s) {
  const float* src = reinterpret_cast<const float*>(g);
  float* dst = reinterpret_cast<float*>(&s);
  for (int k = threadIdx.x; k < (int)(sizeof(EvalConsts) / 4); k += blockDim.x) dst[k] = __ldcg(src + k);
}

// ---------------------------------------------------------------------------
// moving-image evaluation at a mapped continuous index

// CentralDifferenceImageFunction::EvaluateSpecialized (point form, image direction on),
// Core/ImageFunction/include/itkCentralDifferenceImageFunction.hxx:256-316
__device__ __forceinline__ float3 central_difference(const EvalArgs& a, const DFPos& p) {
  float g[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const CIdx n1 = to_cidx(df_offset(p, a.cd_hi + 3 * d, a.cd_lo + 3 * d, -1.f));
    if (!ci_inside(n1, a.nx, a.ny, a.nz)) { g[d] = 0.f; continue; }
    const CIdx n2 = to_cidx(df_offset(p, a.cd_hi + 3 * d, a.cd_lo + 3 * d, 1.f));
    if (!ci_inside(n2, a.nx, a.ny, a.nz)) { g[d] = 0.f; continue; }
    const float v1 = gather1(a.mov1, make_stencil(n1, a.nx, a.ny, a.nz), a.nx, a.ny);
    const float v2 = gather1(a.mov1, make_stencil(n2, a.nx, a.ny, a.nz), a.nx, a.ny);
    g[d] = (v2 - v1) * a.cd_inv_delta[d];
  }
  return make_float3(g[0], g[1], g[2]);
}

// TransformAndEvaluateMovingPoint + ComputeMovingImageGradientAtPoint
// (itkImageToImageMetricv4.hxx:331-425): buffer test, trilinear value, gradient.
template <int GRAD>
__device__ __forceinline__ bool eval_moving(const EvalArgs& a, const DFPos& p, bool need_grad, float& m, float3& g) {
  const CIdx c = to_cidx(p);
  if (!ci_inside(c, a.nx, a.ny, a.nz)) return false;
  const Stencil st = make_stencil(c, a.nx, a.ny, a.nz);
  if (GRAD == kGradImage) {
    const float4 v = gather4(a.mov4, st, a.nx, a.ny);
    m = v.x;
    g = make_float3(v.y, v.z, v.w);
  } else {
    m = gather1(a.mov1, st, a.nx, a.ny);
    g = need_grad ? central_difference(a, p) : make_float3(0.f, 0.f, 0.f);
  }
  return true;
}

// ---------------------------------------------------------------------------
// deterministic reductions
//
// Within a block: per-thread Kahan FP32 sums, XOR-shuffle warp sums, then a
// fixed-order FP64 sum over warps.  Across blocks: each block writes its FP64
// partials; the last block of each group of 16 (atomic ticket) sums its group
// in block order, and the last group sums the groups in group order.  The
// result is bitwise reproducible for a given grid, so GetValue and
// GetValueAndDerivative agree exactly.

constexpr int kGroup = 16;

// The blocks one evaluation of one registration runs on: block b of n.  A plain
// launch uses the hardware grid; a batched launch (several registrations in one
// grid) gives each registration its own range of blocks.
struct VGrid {
  int b, n;
};
__device__ __forceinline__ VGrid hw_grid() { return VGrid{(int)blockIdx.x, (int)gridDim.x}; }

template <int NV>
__device__ __forceinline__ void block_sums(KahanF (&acc)[NV], float (*red)[NV], double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const float v = warp_sum(acc[k].value());
    if (lane == 0) red[warp][k] = v;
  }
  __syncthreads();
  const int nwarps = blockDim.x >> 5;
  for (int k = threadIdx.x; k < NV; k += blockDim.x) {
    KahanF s;
    s.zero();
    for (int w = 0; w < nwarps; ++w) s.add(red[w][k]);
    out[k] = (double)s.value();  // FP32 compensated inside the block, FP64 across blocks
  }
  __syncthreads();
}

// dst[k] = sum_{j < cnt} src[j * NV + k] for k < NV, one warp per k: lane l loads
// entries l, l + 32, ... (independent loads in flight together), then a fixed
// XOR-shuffle tree -- the same order on every call.
template <int NV>
__device__ __forceinline__ void strided_sums(const double* src, int cnt, double* dst) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int k = warp; k < NV; k += nwarps) {
    double s = 0.0;
    for (int j = lane; j < cnt; j += 32) s += __ldcg(&src[j * NV + k]);
    s = warp_sum_d(s);
    if (lane == 0) dst[k] = s;
  }
}

// Returns true in exactly one block, which then holds the grid-wide sums in `fin`.
template <int NV>
__device__ __forceinline__ bool grid_sums(const double* blk, double* part, double* grp, unsigned* tick, double* fin,
                                          VGrid vg = hw_grid()) {
  __shared__ unsigned t;
  const int b = vg.b, g = b / kGroup;
  const int ng = (vg.n + kGroup - 1) / kGroup;
  const int gsize = min(kGroup, vg.n - g * kGroup);
  for (int k = threadIdx.x; k < NV; k += blockDim.x) part[b * NV + k] = blk[k];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(&tick[g], 1u);
  __syncthreads();
  if (t != (unsigned)(gsize - 1)) return false;
  __threadfence();
  strided_sums<NV>(part + g * kGroup * NV, gsize, grp + g * NV);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(&tick[ng], 1u);
  __syncthreads();
  if (t != (unsigned)(ng - 1)) return false;
  __threadfence();
  __shared__ double fin_s[NV];
  strided_sums<NV>(grp, ng, fin_s);
  __syncthreads();
  for (int k = threadIdx.x; k < NV; k += blockDim.x) fin[k] = fin_s[k];
  __syncthreads();
  return true;
}

// Double-float values: hi + lo, two FP32 numbers with |lo| <= ulp(hi) / 2, about 48
// significant bits.  The Mattes derivative pass sums its block partials this way:
// FP32 adds at the FP32 rate, where GB300's FP64 rate (about 1/64 of it) makes an
// FP64 chain over a few hundred partials take microseconds in the one block that
// forms the sums.  Addition: Knuth's two-sum of the high parts, the low parts added
// in, Dekker's fast two-sum to renormalize (the _rn intrinsics are never contracted
// or reassociated).
struct DFloat {
  float hi, lo;
};
__device__ __forceinline__ DFloat df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return DFloat{s, e};
}
__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
  const DFloat s = df_two_sum(a.hi, b.hi);
  const float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  const float hi = __fadd_rn(s.hi, lo);
  return DFloat{hi, __fsub_rn(lo, __fsub_rn(hi, s.hi))};
}
__device__ __forceinline__ double df_to_double(DFloat v) { return (double)v.hi + (double)v.lo; }

// block_sums with the block's compensated FP32 sums kept exactly: s - c as a double-float.
template <int NV>
__device__ __forceinline__ void block_sums_df(KahanF (&acc)[NV], float (*red)[NV], DFloat* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const float v = warp_sum(acc[k].value());
    if (lane == 0) red[warp][k] = v;
  }
  __syncthreads();
  const int nwarps = blockDim.x >> 5;
  for (int k = threadIdx.x; k < NV; k += blockDim.x) {
    KahanF s;
    s.zero();
    for (int w = 0; w < nwarps; ++w) s.add(red[w][k]);
    out[k] = df_two_sum(s.s, -s.c);
  }
  __syncthreads();
}

// strided_sums in double-float: dst[k] = sum_{j < cnt} src[j * NV + k], one warp per k,
// lane l adding entries l, l + 32, ... (loads in flight together), then a fixed XOR tree.
template <int NV>
__device__ __forceinline__ void strided_sums_df(const DFloat* src, int cnt, DFloat* dst) {
  constexpr int kBatch = 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int k = warp; k < NV; k += nwarps) {
    DFloat s{0.f, 0.f};
    for (int j0 = lane; j0 < cnt; j0 += kBatch * 32) {
      float2 v[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int j = j0 + u * 32;
        v[u] = j < cnt ? __ldcg(reinterpret_cast<const float2*>(src + j * NV + k)) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u)
        if (j0 + u * 32 < cnt) s = df_add(s, DFloat{v[u].x, v[u].y});
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      s = df_add(s, DFloat{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
    if (lane == 0) dst[k] = s;
  }
}

// strided_sums_df over partials staged in shared memory, by warps [0, nwarps).
template <int NV>
__device__ __forceinline__ void strided_sums_df_shared(const DFloat* src, int cnt, DFloat* dst, int nwarps) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = warp; k < NV; k += nwarps) {
    DFloat s{0.f, 0.f};
    for (int j = lane; j < cnt; j += 32) s = df_add(s, src[j * NV + k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      s = df_add(s, DFloat{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
    if (lane == 0) dst[k] = s;
  }
}

// grid_sums / grid_sums_flat over double-float partials (part and grp hold DFloat);
// `fin` receives the sums as doubles.
template <int NV>
__device__ __forceinline__ bool grid_sums_df(const DFloat* blk, DFloat* part, DFloat* grp, unsigned* tick,
                                             double* fin, VGrid vg = hw_grid()) {
  __shared__ unsigned t;
  const int b = vg.b, g = b / kGroup;
  const int ng = (vg.n + kGroup - 1) / kGroup;
  const int gsize = min(kGroup, vg.n - g * kGroup);
  for (int k = threadIdx.x; k < NV; k += blockDim.x) part[b * NV + k] = blk[k];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(&tick[g], 1u);
  __syncthreads();
  if (t != (unsigned)(gsize - 1)) return false;
  __threadfence();
  strided_sums_df<NV>(part + g * kGroup * NV, gsize, grp + g * NV);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(&tick[ng], 1u);
  __syncthreads();
  if (t != (unsigned)(ng - 1)) return false;
  __threadfence();
  __shared__ DFloat fin_s[NV];
  strided_sums_df<NV>(grp, ng, fin_s);
  __syncthreads();
  for (int k = threadIdx.x; k < NV; k += blockDim.x) fin[k] = df_to_double(fin_s[k]);
  __syncthreads();
  return true;
}

// One-level form of grid_sums for grids of at most kFlatMaxBlocks blocks: every block
// writes its partials and takes one ticket; the last sums all blocks' partials in
// block order (lane-strided, fixed XOR trees).  One global round trip fewer than
// the grouped form.
constexpr int kFlatMaxBlocks = 1024;
template <int NV>
__device__ __forceinline__ bool grid_sums_flat(const double* blk, double* part, unsigned* tick, double* fin,
                                               VGrid vg = hw_grid()) {
  __shared__ unsigned t;
  for (int k = threadIdx.x; k < NV; k += blockDim.x) part[vg.b * NV + k] = blk[k];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(tick, 1u);
  __syncthreads();
  if (t != (unsigned)(vg.n - 1)) return false;
  __threadfence();
  __shared__ double fin_s[NV];
  strided_sums<NV>(part, vg.n, fin_s);
  __syncthreads();
  for (int k = threadIdx.x; k < NV; k += blockDim.x) fin[k] = fin_s[k];
  __syncthreads();
  return true;
}

// The flat form's first half: this block's partials and its ticket; true in the last block.
template <int NV>
__device__ __forceinline__ bool grid_ticket_flat_df(const DFloat* blk, DFloat* part, unsigned* tick, VGrid vg) {
  __shared__ unsigned t;
  for (int k = threadIdx.x; k < NV; k += blockDim.x) part[vg.b * NV + k] = blk[k];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(tick, 1u);
  __syncthreads();
  if (t != (unsigned)(vg.n - 1)) return false;
  __threadfence();
  return true;
}

// dst[0, n) <- src[0, n) (global, 8-byte entries), every entry requested before the
// first lands: one L2 round trip for a few thousand entries.
__device__ __forceinline__ void stage_u64(const unsigned long long* src, int n, unsigned long long* dst) {
  constexpr int kLoads = 16;
  for (int e0 = threadIdx.x; e0 < n; e0 += kLoads * blockDim.x) {
    unsigned long long v[kLoads];
#pragma unroll
    for (int u = 0; u < kLoads; ++u) {
      const int e = e0 + u * (int)blockDim.x;
      v[u] = e < n ? __ldcg(src + e) : 0ull;
    }
#pragma unroll
    for (int u = 0; u < kLoads; ++u) {
      const int e = e0 + u * (int)blockDim.x;
      if (e < n) dst[e] = v[u];
    }
  }
}

template <int NV>
__device__ __forceinline__ bool grid_sums_flat_df(const DFloat* blk, DFloat* part, unsigned* tick, double* fin,
                                                  VGrid vg = hw_grid()) {
  __shared__ unsigned t;
  for (int k = threadIdx.x; k < NV; k += blockDim.x) part[vg.b * NV + k] = blk[k];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) t = atomicAdd(tick, 1u);
  __syncthreads();
  if (t != (unsigned)(vg.n - 1)) return false;
  __threadfence();
  __shared__ DFloat fin_s[NV];
  strided_sums_df<NV>(part, vg.n, fin_s);
  __syncthreads();
  for (int k = threadIdx.x; k < NV; k += blockDim.x) fin[k] = df_to_double(fin_s[k]);
  __syncthreads();
  return true;
}

__device__ __forceinline__ void block_count(unsigned nv, unsigned long long* gn) {
  __shared__ unsigned sh;
  if (threadIdx.x == 0) sh = 0u;
  __syncthreads();
  const unsigned w = warp_sum_u(nv);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(&sh, w);
  __syncthreads();
  if (threadIdx.x == 0 && sh) atomicAdd(gn, (unsigned long long)sh);
}

// true in exactly one block: the last to finish (threadFenceReduction pattern)
__device__ __forceinline__ bool last_block(unsigned* ticket, VGrid vg = hw_grid()) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = atomicAdd(ticket, 1u) == (unsigned)vg.n - 1u;
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// ---------------------------------------------------------------------------
// MeanSquares, affine: value = sum (f - m)^2 / N, d[p] = sum 2 (f - m) (J^T g)[p] / N

template <int GRAD, bool FPC = false>
__device__ __forceinline__ void msq_affine_body(const EvalArgs& a, VGrid vg) {
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][13];
  __shared__ double redd[FPC ? kBlock / 32 : 1][12];
  __shared__ double blk[13], fin[13];
  double dacc[FPC ? 12 : 1];
#pragma unroll
  for (int k = 0; k < (FPC ? 12 : 1); ++k) dacc[k] = 0.0;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  __syncthreads();
  KahanF acc[13];
#pragma unroll
  for (int k = 0; k < 13; ++k) acc[k].zero();
  unsigned nv = 0;
  const int64_t stride = (int64_t)vg.n * blockDim.x;
  int64_t i = (int64_t)vg.b * blockDim.x + threadIdx.x;
  float4 s_next = i < a.n ? __ldcs(a.samples + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  for (; i < a.n; i += stride) {
    const float4 s = s_next;
    s_next = i + stride < a.n ? __ldcs(a.samples + i + stride) : make_float4(0.f, 0.f, 0.f, 0.f);
    float m;
    float3 g;
    const DFPos p = map_pos(load_map(K.map), s.x, s.y, s.z);
    if (!eval_moving<GRAD>(a, p, a.with_derivative != 0, m, g)) continue;
    const float diff = s.w - m;  // FixedImagePixelType diff, MeanSquares...Threader.hxx:46
    acc[0].add(diff * diff);
    ++nv;
    if (a.with_derivative) {
      const float t = 2.f * diff;
      const float3 v = jac_vec(K, s.x, s.y, s.z);
      const float vx = v.x, vy = v.y, vz = v.z;
      const float t0 = t * g.x, t1 = t * g.y, t2 = t * g.z;
      if (FPC) {
        // StorePointDerivativeResult with UseFloatingPointCorrection
        // (ThreaderBase.hxx:284-294): static_cast<intmax_t>(d * r) / r per parameter
        const float ld[12] = {t0 * vx, t0 * vy, t0 * vz, t1 * vx, t1 * vy, t1 * vz,
                              t2 * vx, t2 * vy, t2 * vz, t0, t1, t2};
#pragma unroll
        for (int k = 0; k < (FPC ? 12 : 1); ++k)
          dacc[k] += (double)(long long)((double)ld[k] * a.fp_res) / a.fp_res;
      } else {
        acc[1].add(t0 * vx); acc[2].add(t0 * vy); acc[3].add(t0 * vz);
        acc[4].add(t1 * vx); acc[5].add(t1 * vy); acc[6].add(t1 * vz);
        acc[7].add(t2 * vx); acc[8].add(t2 * vy); acc[9].add(t2 * vz);
        acc[10].add(t0); acc[11].add(t1); acc[12].add(t2);
      }
    }
  }
  block_count(nv, a.acc_n);
  block_sums<13>(acc, red, blk);
  if (FPC) {
    // the truncated derivatives: FP64 warp trees, warps in order
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < (FPC ? 12 : 1); ++k) {
      const double w = warp_sum_d(dacc[k]);
      if (lane == 0) redd[warp][k] = w;
    }
    __syncthreads();
    if (threadIdx.x < 12) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += redd[w][threadIdx.x];
      blk[1 + threadIdx.x] = s;
    }
    __syncthreads();
  }
  if (!grid_sums<13>(blk, a.part, a.grp, a.tickets + kTicketMain, fin, vg)) return;
  if (threadIdx.x < 32) {
    // AfterThreadedExecution + VerifyNumberOfValidPoints (ThreaderBase.hxx:116-172); lane
    // k divides entry k (the FP64 divisions side by side, not one after another)
    const int lane = threadIdx.x;
    const unsigned long long N = __ldcg(a.acc_n);
    const int P = a.with_derivative ? a.nparams : 0;
    for (int k = lane; k < 1 + P; k += 32) a.out[k == 0 ? 0 : 1 + k] = N == 0 ? (k == 0 ? DBL_MAX : 0.0)
                                                                               : fin[k] / (double)N;
    if (lane == 0) {
      a.out[1] = (double)N;
      *a.status = N == 0 ? GB_ERR_NO_VALID_POINTS : GB_OK;
    }
  }
}

template <int GRAD, bool FPC = false>
__global__ void __launch_bounds__(kBlock) k_msq_affine(EvalArgs a) {
  msq_affine_body<GRAD, FPC>(a, hw_grid());
}

// ---------------------------------------------------------------------------
// Correlation, affine (CorrelationImageToImageMetricv4), two passes:
//   pass A: the sums of the fixed and moving values over the valid points; its
//     last block writes the averages (the helper threader,
//     itkCorrelationImageToImageMetricv4HelperThreader.hxx:58-169);
//   pass B: with f1 = f - avg_f, m1 = m - avg_m (the averages as double-float),
//     fm, f2, m2 and fdm = sum f1 (J^T g), mdm = sum m1 (J^T g); the last block:
//     value = -fm^2 / (f2 m2), derivative = 2 fm / (f2 m2) (fdm - fm / m2 mdm),
//     0 when m2 f2 <= epsilon (...GetValueAndDerivativeThreader.hxx:62-130,270-325).
constexpr int kCorrMaxBlocks = 1024;  // pass B's 27 partials per block fit the scratch

template <int GRAD>
__device__ __forceinline__ void corr_mean_body(const EvalArgs& a, VGrid vg) {
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][2];
  __shared__ double blk[2], fin[2];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  __syncthreads();
  KahanF acc[2];
  acc[0].zero();
  acc[1].zero();
  unsigned nv = 0;
  const int64_t stride = (int64_t)vg.n * blockDim.x;
  for (int64_t i = (int64_t)vg.b * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 s = __ldcs(a.samples + i);
    float m;
    float3 g;
    if (!eval_moving<GRAD>(a, map_pos(K.map, s.x, s.y, s.z), false, m, g)) continue;
    acc[0].add(s.w);
    acc[1].add(m);
    ++nv;
  }
  block_count(nv, a.acc_n);
  block_sums<2>(acc, red, blk);
  if (!grid_sums<2>(blk, a.part, a.grp, a.tickets + kTicketMain, fin, vg)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.acc_n);
    a.marg[2] = N > 0 ? fin[0] / (double)N : 0.0;  // m_AverageFix
    a.marg[3] = N > 0 ? fin[1] / (double)N : 0.0;  // m_AverageMov
  }
}

template <int GRAD>
__device__ __forceinline__ void corr_body(const EvalArgs& a, VGrid vg) {
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][27];
  __shared__ double blk[27], fin[27];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  float afh, afl, amh, aml;
  split_df(__ldcg(&a.marg[2]), afh, afl);
  split_df(__ldcg(&a.marg[3]), amh, aml);
  __syncthreads();
  KahanF acc[3];  // fm, f2, m2
#pragma unroll
  for (int k = 0; k < 3; ++k) acc[k].zero();
  float d[24];  // fdm (12), mdm (12): plain FP32 per thread (a few samples each)
#pragma unroll
  for (int k = 0; k < 24; ++k) d[k] = 0.f;
  const int64_t stride = (int64_t)vg.n * blockDim.x;
  for (int64_t i = (int64_t)vg.b * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 s = __ldcs(a.samples + i);
    float m;
    float3 g;
    if (!eval_moving<GRAD>(a, map_pos(K.map, s.x, s.y, s.z), a.with_derivative != 0, m, g)) continue;
    const float f1 = __fsub_rn(__fsub_rn(s.w, afh), afl);
    const float m1 = __fsub_rn(__fsub_rn(m, amh), aml);
    acc[0].add(f1 * m1);
    acc[1].add(f1 * f1);
    acc[2].add(m1 * m1);
    if (a.with_derivative) {
      const float3 v = jac_vec(K, s.x, s.y, s.z);
      const float gg[3] = {g.x, g.y, g.z}, vv[3] = {v.x, v.y, v.z};
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float tf = f1 * gg[r], tm = m1 * gg[r];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          d[3 * r + c] = fmaf(tf, vv[c], d[3 * r + c]);
          d[12 + 3 * r + c] = fmaf(tm, vv[c], d[12 + 3 * r + c]);
        }
        d[9 + r] += tf;
        d[21 + r] += tm;
      }
    }
  }
  KahanF kacc[27];
#pragma unroll
  for (int k = 0; k < 3; ++k) kacc[k] = acc[k];
#pragma unroll
  for (int k = 0; k < 24; ++k) {
    kacc[3 + k].s = d[k];
    kacc[3 + k].c = 0.f;
  }
  block_sums<27>(kacc, red, blk);
  if (!grid_sums<27>(blk, a.part, a.grp, a.tickets + kTicketPass2, fin, vg)) return;
  if (threadIdx.x < 32) {
    // one derivative entry per lane (every lane forms the same FP64 factors)
    const int lane = threadIdx.x;
    const unsigned long long N = __ldcg(a.acc_n);
    const int P = a.with_derivative ? a.nparams : 0;
    const double fm = fin[0], f2 = fin[1], m2 = fin[2];
    const double m2f2 = m2 * f2;
    // VerifyNumberOfValidPoints (no valid point: a warning, value max, derivative 0); a
    // zero denominator gives value 0 and derivative 0
    const bool live = N != 0 && !(m2f2 <= DBL_EPSILON);
    const double sc = live ? 2.0 * fm / (f2 * m2) : 0.0, r = live ? fm / m2 : 0.0;
    for (int p = lane; p < P; p += 32) a.out[2 + p] = live ? sc * (fin[3 + p] - r * fin[15 + p]) : 0.0;
    if (lane == 0) {
      a.out[1] = (double)N;
      *a.status = N == 0 ? GB_ERR_NO_VALID_POINTS : GB_OK;
      a.out[0] = N == 0 ? DBL_MAX : (live ? -1.0 * fm * fm / m2f2 : 0.0);
    }
  }
}

template <int GRAD>
__global__ void __launch_bounds__(kBlock) k_corr_mean_affine(EvalArgs a) {
  corr_mean_body<GRAD>(a, hw_grid());
}

template <int GRAD>
__global__ void __launch_bounds__(kBlock) k_corr_affine(EvalArgs a) {
  corr_body<GRAD>(a, hw_grid());
}

// ---------------------------------------------------------------------------
// Sample position in the moving image for each transform form:
//   kMapAffine       the per-evaluation affine map of the record's coordinates;
//   kMapFieldDense   the dense virtual grid under a displacement field: the
//                    identity map plus P2I_moving u, u the field value at the
//                    record's own voxel (DisplacementFieldTransform::TransformPoint
//                    at a grid point: the interpolation weight is 1 there);
//   kMapFieldPoints  a point set under a displacement field: u interpolated
//                    trilinearly (VectorLinearInterpolateImageFunction, neighbours
//                    clamped to the buffer), zero outside the field's buffer
//                    (Filtering/DisplacementField/include/itkDisplacementFieldTransform.hxx:67-100).
// `voxel` receives the virtual voxel whose derivative block the sample feeds.
enum { kMapAffine = 0, kMapFieldDense = 1, kMapFieldPoints = 2 };

__device__ __forceinline__ float3 field_interp(const double* __restrict__ f, const Stencil& st, int nx, int ny) {
  const unsigned sy = (unsigned)nx, sz = (unsigned)nx * (unsigned)ny;
  const unsigned zs[2] = {st.z0 * sz, st.z1 * sz}, ys[2] = {st.y0 * sy, st.y1 * sy}, xs[2] = {(unsigned)st.x0,
                                                                                             (unsigned)st.x1};
  float v[8][3];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const double* q = f + 3ull * (zs[c >> 2] + ys[(c >> 1) & 1] + xs[c & 1]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float h, l;
      split_double_bits(__ldg(q + k), h, l);
      v[c][k] = __fadd_rn(h, l);
    }
  }
  float u[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float x00 = lerp(v[0][k], v[1][k], st.dx), x10 = lerp(v[2][k], v[3][k], st.dx);
    const float x01 = lerp(v[4][k], v[5][k], st.dx), x11 = lerp(v[6][k], v[7][k], st.dx);
    u[k] = lerp(lerp(x00, x10, st.dy), lerp(x01, x11, st.dy), st.dz);
  }
  return make_float3(u[0], u[1], u[2]);
}

// map(x) + umap u with diagonal matrices: the general double-float sums with their
// zero terms left out (adding an exact zero changes neither the sum nor its error term).
__device__ __forceinline__ DFPos field_pos_diag(const EvalConsts& K, float x, float y, float z, const float uhi[3],
                                                const float ulo[3]) {
  const float xs[3] = {x, y, z};
  DFPos r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float s = K.map.bhi[k], err = K.map.blo[k];
    const float a = K.map.Ahi[4 * k];
    const float p = __fmul_rn(a, xs[k]);
    const float pe = __fmaf_rn(a, xs[k], -p);
    float t, e;
    two_sum(s, p, t, e);
    s = t;
    err = __fadd_rn(err, __fadd_rn(e, __fmaf_rn(K.map.Alo[4 * k], xs[k], pe)));
    r.hi[k] = __fadd_rn(s, err);
    r.lo[k] = __fsub_rn(err, __fsub_rn(r.hi[k], s));
  }
  DFPos q;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float s = r.hi[k], err = r.lo[k];
    const float a = K.umap.Ahi[4 * k];
    const float p = __fmul_rn(a, uhi[k]);
    const float pe = __fmaf_rn(a, uhi[k], -p);
    float t, e;
    two_sum(s, p, t, e);
    s = t;
    err = __fadd_rn(err, __fadd_rn(e, __fadd_rn(pe, __fmaf_rn(K.umap.Alo[4 * k], uhi[k], __fmul_rn(a, ulo[k])))));
    q.hi[k] = __fadd_rn(s, err);
    q.lo[k] = __fsub_rn(err, __fsub_rn(q.hi[k], s));
  }
  return q;
}

// A displacement field's local Jacobian product: M^T g behind an initial affine
// (identity M: g exactly), K.Mg = M^T.
__device__ __forceinline__ float3 field_grad(const EvalConsts& K, float3 g) {
  return make_float3(fmaf(K.Mg[0], g.x, fmaf(K.Mg[1], g.y, K.Mg[2] * g.z)),
                     fmaf(K.Mg[3], g.x, fmaf(K.Mg[4], g.y, K.Mg[5] * g.z)),
                     fmaf(K.Mg[6], g.x, fmaf(K.Mg[7], g.y, K.Mg[8] * g.z)));
}

template <int TK>
__device__ __forceinline__ DFPos sample_pos(const EvalArgs& a, const EvalConsts& K, const float4& s, int64_t i,
                                            unsigned& voxel) {
  if (TK == kMapFieldDense && K.fdiag != 0.f) {
    voxel = (unsigned)s.x + (unsigned)a.vnx * ((unsigned)s.y + (unsigned)a.vny * (unsigned)s.z);
    const double* q = a.field + 3ull * voxel;
    float uhi[3], ulo[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) split_double_bits(__ldg(q + k), uhi[k], ulo[k]);
    return field_pos_diag(K, s.x, s.y, s.z, uhi, ulo);
  }
  const DFPos p = map_pos(load_map(K.map), s.x, s.y, s.z);
  if (TK == kMapAffine) return p;
  float uhi[3], ulo[3];
  if (TK == kMapFieldDense) {
    voxel = (unsigned)s.x + (unsigned)a.vnx * ((unsigned)s.y + (unsigned)a.vny * (unsigned)s.z);
    const double* q = a.field + 3ull * voxel;
#pragma unroll
    for (int k = 0; k < 3; ++k) split_double_bits(__ldg(q + k), uhi[k], ulo[k]);
  } else {
    voxel = __ldg(a.voff + i);
    const CIdx c = to_cidx(map_pos(K.fmap, s.x, s.y, s.z));
    if (!ci_inside(c, a.vnx, a.vny, a.vnz)) return p;
    const float3 u = field_interp(a.field, make_stencil(c, a.vnx, a.vny, a.vnz), a.vnx, a.vny);
    uhi[0] = u.x;
    uhi[1] = u.y;
    uhi[2] = u.z;
    ulo[0] = ulo[1] = ulo[2] = 0.f;
  }
  return df_add_matvec(p, K.umap, uhi, ulo);
}

// ---------------------------------------------------------------------------
// Mattes pass 1, affine: joint histogram (Parzen: box on fixed, cubic B-spline
// on moving), fixed marginal counts, moving marginal, valid count, per-sample
// cache.  Histogram weights are 2^26 fixed point: integer adds are
// associative, so the histogram does not depend on scheduling.

// Moving Parzen window of one sample: first bin and the position t in [0, 1]
// (Mattes...Threader.hxx:248-264).
__device__ __forceinline__ void parzen_window(float term, int B, int& pdfm, float& t) {
  int midx = (int)term;  // static_cast<OffsetValueType>
  midx = midx < 2 ? 2 : (midx > B - 3 ? B - 3 : midx);
  pdfm = midx - 1;
  t = term - (float)midx;
}

// Adds one sample's four Parzen weights into the block histogram.  Lanes with
// the same (fixed bin, first moving bin) key are summed with one redux per
// weight, and only the group leader issues the shared atomics.
__device__ __forceinline__ void hist_add_aggregated(bool ok, int key, int fidx, const unsigned q[4],
                                                    unsigned long long* hist, unsigned* fm) {
  const unsigned okmask = __ballot_sync(0xffffffffu, ok);
  if (!ok) return;
  const unsigned peers = __match_any_sync(okmask, key);
  const int leader = __ffs(peers) - 1;
  const int lane = threadIdx.x & 31;
  unsigned s[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) s[k] = __reduce_add_sync(peers, q[k]);
  if (lane == leader) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (s[k]) atomicAdd(&hist[key + k], (unsigned long long)s[k]);
    atomicAdd(&fm[fidx], (unsigned)__popc(peers));
  }
}

// Barrier among the kBlock streaming threads of a pass-2 block (barrier 0 is
// __syncthreads, which would also wait for the block's group warp).
__device__ __forceinline__ void stream_barrier() { asm volatile("bar.sync 1, %0;" ::"n"(kBlock) : "memory"); }

// The table's validity thresholds from the fixed-point total T and the valid count N:
// p > eps <=> h > floor(eps T), pf > eps <=> count > floor(eps T / 2^26), and no
// table at all when N = 0 or the joint PDF sums to zero.  FP64 (a handful of
// operations at GB300's FP64 rate): formed by one thread and shared.
struct PratioThresholds {
  unsigned long long hthr, fthr;
  int bad;
};
__device__ __forceinline__ PratioThresholds pratio_thresholds(double T, unsigned long long N) {
  PratioThresholds t;
  t.bad = (N == 0 || !(T * kQInv >= DBL_EPSILON)) ? 1 : 0;
  t.hthr = (unsigned long long)(DBL_EPSILON * T);
  t.fthr = (unsigned long long)(DBL_EPSILON * T * kQInv);
  return t;
}

template <bool STREAMERS>
static __device__ __noinline__ void mattes_pratio_build(const EvalArgs& a, double T, float* dst, float* colf,
                                                        unsigned* fmask);

// u64 count -> float from its two 32-bit halves, FP32 arithmetic only (two roundings,
// relative error below 2^-23)
__device__ __forceinline__ float u64_to_float(unsigned long long v) {
  return fmaf(__uint2float_rn((unsigned)(v >> 32)), 4294967296.f, __uint2float_rn((unsigned)v));
}

// End of Mattes pass 1 (any transform): flush the block histogram, marginals and
// count; the last block forms the fixed-point total T and, with `table`, the
// derivative's log(p / pm) table in global memory (the affine derivative pass
// builds the table itself, in shared memory).
__device__ __forceinline__ void mattes_pass1_epilogue(const EvalArgs& a, unsigned nv, unsigned long long* hist,
                                                      unsigned long long* cs, unsigned* fm, VGrid vg = hw_grid(),
                                                      bool table = true) {
  const int B = a.bins;
  const int BB = B * B;
  __syncthreads();
  // flush the nonzero bins; the block's column sums ride along as shared atomics.  Each
  // block starts at its own bin, so the blocks finishing together do not queue on the
  // same global addresses.
  const int rot = (int)(((long long)vg.b * 97) % BB);
  for (int k0 = threadIdx.x; k0 < BB; k0 += blockDim.x) {
    const int k = k0 + rot < BB ? k0 + rot : k0 + rot - BB;
    const unsigned long long h = hist[k];
    if (h) {
      atomicAdd(&a.hist[k], h);
      atomicAdd(&cs[k % B], h);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < B; k += blockDim.x) {
    const unsigned c = fm[k];
    if (c) atomicAdd(&a.fmarg[k], (unsigned long long)c);
    if (cs[k]) atomicAdd(&a.colsum[k], cs[k]);
  }
  block_count(nv, a.acc_n);
  if (!last_block(a.tickets + kTicketPass1, vg)) return;
  // Last block: the fixed-point total T of the joint histogram (the value's
  // normalization, JointPDFSum).  It is on the critical path, so it does no FP64
  // transcendental work.
  __shared__ unsigned long long tot_sh;
  if (threadIdx.x == 0) tot_sh = 0ull;
  __syncthreads();
  unsigned long long t = 0ull;
  for (int k = threadIdx.x; k < B; k += blockDim.x) t += __ldcg(&a.colsum[k]);
  // one shared atomic per warp: a block's worth of same-address atomics would serialize
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0 && t) atomicAdd(&tot_sh, t);
  __syncthreads();
  const double T = (double)tot_sh;
  if (threadIdx.x == 0) {
    a.marg[0] = T;                         // fixed-point total
    a.marg[1] = T > 0.0 ? 1.0 / T : 0.0;   // normalization factor (of the fixed-point histogram)
  }
  if (table) mattes_pratio_build<false>(a, T, a.pratio, reinterpret_cast<float*>(cs), fm);
}

// The derivative's FP32 table log(p / pm) = log(h / colsum) (pRatio,
// Mattes...v4.hxx:446-457), 0 where p, pm or pf is not above DBL_EPSILON:
// for integer counts p > eps <=> h > floor(eps T) and pf > eps <=> count >
// floor(eps T / 2^26).  Run by a whole block (STREAMERS: by the kBlock streaming
// threads of a pass-2 block, synchronized on their own barrier), into global
// (dst = a.pratio) or shared memory, from the final histogram and marginals;
// colf / fmask are B entries of shared scratch.  Kept out of line so the sample
// loops' code is unaffected; every caller forms the same bits.
template <bool STREAMERS>
static __device__ __noinline__ void mattes_pratio_build(const EvalArgs& a, double T, float* dst, float* colf,
                                                        unsigned* fmask) {
  const int B = a.bins;
  const int nt = STREAMERS ? kBlock : (int)blockDim.x;
  auto sync = [] {
    if (STREAMERS) stream_barrier();
    else __syncthreads();
  };
  __shared__ PratioThresholds th_s;
  if (threadIdx.x == 0) th_s = pratio_thresholds(T, __ldcg(a.acc_n));  // FP64: once per block
  sync();  // the thresholds; colf / fmask may alias scratch the caller has just used
  const bool bad = th_s.bad != 0;
  const unsigned long long hthr = th_s.hthr, fthr = th_s.fthr;
  // marginals into shared memory: column sums as floats (0 where pm is not above
  // eps), fixed-bin validity
  for (int k = threadIdx.x; k < B; k += nt) {
    const unsigned long long c = __ldcg(&a.colsum[k]);
    colf[k] = c > hthr ? u64_to_float(c) : 0.f;
    fmask[k] = __ldcg(&a.fmarg[k]) > fthr ? 1u : 0u;
  }
  sync();
  constexpr int kBatch = 8;  // independent histogram loads in flight per thread
  for (int k0 = threadIdx.x; k0 < B * B; k0 += kBatch * nt) {
    unsigned long long h[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int k = k0 + j * nt;
      h[j] = (!bad && k < B * B) ? __ldcg(&a.hist[k]) : 0ull;
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int k = k0 + j * nt;
      if (k >= B * B) break;
      const int f = k / B, m = k - f * B;
      const float c = colf[m];
      // fast intrinsics: the ratio is in (0, 1], __logf's error there is below 2^-21 absolute
      dst[k] = (h[j] > hthr && c > 0.f && fmask[f]) ? __logf(__fdividef(u64_to_float(h[j]), c)) : 0.f;
    }
  }
  sync();
}

// Mattes status after pass 1 (Mattes...v4.hxx:367-370 and the valid-point check).
__device__ __forceinline__ int mattes_status(const EvalArgs& a) {
  const unsigned long long N = __ldcg(a.acc_n);
  if (N == 0) return GB_ERR_NO_VALID_POINTS;
  return __ldcg(&a.marg[0]) * kQInv >= DBL_EPSILON ? GB_OK : GB_ERR_JOINT_PDF_SUM_ZERO;
}

// One warp, bins [32 g, 32 g + 32) of the joint histogram: the FP64 terms
// p (log(p/pm) - log pf) (ComputeResults, Mattes...v4.hxx:358-499) summed over
// the lanes by a fixed XOR tree, and the normalized PDF written out.  With T
// the fixed-point total, p = h / T, pm = colsum / T and pf = count 2^26 / T, so
// log(p / pm) = log h - log colsum and log pf = log count + 26 ln 2 - log T.
// Every kernel that forms the value uses this and mattes_value_sum, so GetValue
// and GetValueAndDerivative give the same bits.
__device__ __forceinline__ double mattes_group_partial(const EvalArgs& a, int g, int lane) {
  const int B = a.bins;
  const double T = __ldcg(&a.marg[0]);
  const double invT = __ldcg(&a.marg[1]);
  const bool bad = (__ldcg(a.acc_n) == 0) || !(T * kQInv >= DBL_EPSILON);  // JointPDFSum
  const int bin = g * 32 + lane;
  double part = 0.0;
  if (bin < B * B) {
    const int f = bin / B, m = bin - f * B;
    double p = 0.0;
    if (!bad) {
      const double h = (double)__ldcg(&a.hist[bin]);
      const double c = (double)__ldcg(&a.colsum[m]);
      const double n = (double)__ldcg(&a.fmarg[f]);
      p = h * invT;
      const double pm = c * invT;
      const double pf = n * (invT * 67108864.0);
      if (pf > DBL_EPSILON && pm > DBL_EPSILON && p > DBL_EPSILON) {
        // log(p / pm) - log pf = log(h T / (c n 2^26)): the counts and T are integers
        // below 2^53, so each product rounds once; one FP64 log per bin (GB300's FP64
        // rate makes every log call cost microseconds per warp)
        part = p * log((h * T) / ((c * n) * 67108864.0));
      }
    }
    a.pdf_out[bin] = p;
  }
  return warp_sum_d(part);
}

__host__ __device__ inline int mattes_groups(int bins) { return (bins * bins + 31) / 32; }

// Sum of the group partials part[0, ngroups): lane-strided, then a fixed XOR tree.
__device__ __forceinline__ double mattes_value_sum(const double* part, int ngroups, int lane) {
  constexpr int kBatch = 8;  // loads in flight together, added in the same order
  double s = 0.0;
  for (int r0 = lane; r0 < ngroups; r0 += kBatch * 32) {
    double v[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) v[u] = r0 + u * 32 < ngroups ? __ldcg(&part[r0 + u * 32]) : 0.0;
#pragma unroll
    for (int u = 0; u < kBatch; ++u)
      if (r0 + u * 32 < ngroups) s += v[u];
  }
  return warp_sum_d(s);
}

// Group partials computed by the last warp of blocks b, b + gridDim.x, ... (all blocks participate).
// After a warp has written the partial of one group: the warp that completes the last
// group sums all of them into part[kPartValue] (the same order as mattes_value_sum at
// the end of the pass), so the derivative pass's last block only reads the value.
// It writes before its block takes its cross-block ticket, so the last block sees it.
__device__ __forceinline__ void mattes_value_group_done(const EvalArgs& a, int ng) {
  const int lane = threadIdx.x & 31;
  __threadfence();
  unsigned t = 0u;
  if (lane == 0) t = atomicAdd(&a.tickets[kTicketValue], 1u);
  t = __shfl_sync(0xffffffffu, t, 0);
  if (t != (unsigned)(ng - 1)) return;
  __threadfence();
  const double s = mattes_value_sum(a.part, ng, lane);
  if (lane == 0) a.part[kPartValue] = s;
}

// SUM: the derivative pass's form, with the value summed by the warp completing the
// last group (mattes_value_group_done).
template <bool SUM = false>
__device__ __forceinline__ void mattes_value_groups(const EvalArgs& a, VGrid vg = hw_grid()) {
  if ((int)(threadIdx.x >> 5) != (int)(blockDim.x >> 5) - 1) return;
  const int lane = threadIdx.x & 31;
  const int ng = mattes_groups(a.bins);
  for (int g = vg.b; g < ng; g += vg.n) {
    const double s = mattes_group_partial(a, g, lane);
    if (lane == 0) a.part[g] = s;
    if (SUM) mattes_value_group_done(a, ng);
  }
}

// One sample of Mattes pass 1 (affine and displacement-field maps): position, moving
// value and gradient, range reject, cache write, Parzen weights into the block
// histogram `hist` (warp-aggregated), valid count.  Called by all 32 lanes of a warp.
template <int GRAD, int TK>
__device__ __forceinline__ void mattes_pass1_sample(const EvalArgs& a, const EvalConsts& K, const float4& s, int64_t i,
                                                    bool live, unsigned long long* hist, unsigned* fm, unsigned& nv) {
  const int B = a.bins;
  float m = 0.f;
  float3 g = make_float3(0.f, 0.f, 0.f);
  bool ok = false;
  if (live) {
    unsigned voxel;
    const DFPos p = sample_pos<TK>(a, K, s, i, voxel);
    ok = eval_moving<GRAD>(a, p, a.with_derivative != 0, m, g);
    if (TK != kMapAffine) g = field_grad(K, g);
    // reject moving values outside [MovingImageTrueMin, MovingImageTrueMax], Mattes...Threader.hxx:238-245
    ok = ok && !(m < a.mmin) && !(m > a.mmax);
  }
  // m / binsize - normalizedMin == (m - min) / binsize + 2 (padding), Mattes...v4.hxx:309-317
  const float term = fmaf(m - a.mmin, a.m_inv_bs, 2.f);
  if (a.with_derivative && live)
    __stcs(a.cache + i, ok ? make_float4(term, g.x, g.y, g.z) : make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f));
  int pdfm = 0;
  unsigned q[4] = {0u, 0u, 0u, 0u};
  const int fidx = __float_as_int(s.w);
  if (ok) {
    float t, w6[4];
    parzen_window(term, B, pdfm, t);
    parzen6(t, w6);
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = (__float2uint_rn(w6[k] * kQScale) + 3u) / 6u;  // unbiased 1/6
  }
  hist_add_aggregated(ok, fidx * B + pdfm, fidx, q, hist, fm);
  nv += ok ? 1u : 0u;
}

template <int GRAD, int TK = kMapAffine>
__device__ __forceinline__ void mattes_pass1_affine_body(const EvalArgs& a, VGrid vg) {
  extern __shared__ unsigned long long smem_u64[];
  const int B = a.bins;
  unsigned long long* hist = smem_u64;
  unsigned long long* cs = smem_u64 + B * B;
  unsigned* fm = reinterpret_cast<unsigned*>(smem_u64 + B * B + B);
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
  __syncthreads();
  unsigned nv = 0;
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)vg.n * blockDim.x;
  // the affine derivative pass builds the log(p / pm) table itself
  constexpr bool kOwnTable = TK == kMapAffine;
  int64_t base = (int64_t)vg.b * blockDim.x + (threadIdx.x & ~31);
  float4 s_next = base + lane < a.n ? __ldcs(a.samples + base + lane) : make_float4(0.f, 0.f, 0.f, 0.f);
  for (; base < a.n; base += stride) {
    const int64_t i = base + lane;
    const bool live = i < a.n;
    const float4 s = s_next;
    // prefetch the next record so its latency overlaps this iteration's gathers
    s_next = i + stride < a.n ? __ldcs(a.samples + i + stride) : make_float4(0.f, 0.f, 0.f, 0.f);
    mattes_pass1_sample<GRAD, TK>(a, K, s, i, live, hist, fm, nv);
  }
  mattes_pass1_epilogue(a, nv, hist, cs, fm, vg, !kOwnTable);
}

template <int GRAD>
__global__ void __launch_bounds__(kBlock, GRAD == kGradImage ? 5 : 4) k_mattes_pass1_affine(EvalArgs a) {
  mattes_pass1_affine_body<GRAD>(a, hw_grid());
}

#ifndef GB_KERNELS_HELPERS_ONLY
// The derivative's log(p / pm) table in global memory, one entry per thread (the
// same arithmetic as mattes_pratio_build), for the derivative kernels that read it
// from global memory (B-spline chunk sums).  A few blocks launched after pass 1,
// instead of pass 1's last block forming all bins^2 entries alone on one SM.
__global__ void __launch_bounds__(kBlock) k_mattes_table(EvalArgs a) {
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  const int B = a.bins;
  __shared__ PratioThresholds th_s;
  if (threadIdx.x == 0) {
    const double T = __ldcg(&a.marg[0]);
    const unsigned long long N = __ldcg(a.acc_n);
    th_s = pratio_thresholds(T, N);  // FP64: once per block
    // the derivative scale for the parameter gather: nFactor = -1 / (MovingImageBinSize
    // * N), Mattes...Threader.hxx:446-457, 0 when the status is not OK (formed once here)
    if (blockIdx.x == 0) a.marg[2] = th_s.bad ? 0.0 : -1.0 / (a.m_bs * (double)N);
  }
  __syncthreads();
  const bool bad = th_s.bad != 0;
  const unsigned long long hthr = th_s.hthr, fthr = th_s.fthr;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < B * B; k += gridDim.x * blockDim.x) {
    const int f = k / B, m = k - f * B;
    const unsigned long long cs = __ldcg(&a.colsum[m]);
    const float c = cs > hthr ? u64_to_float(cs) : 0.f;
    const bool fok = __ldcg(&a.fmarg[f]) > fthr;
    const unsigned long long h = bad ? 0ull : __ldcg(&a.hist[k]);
    a.pratio[k] = (h > hthr && c > 0.f && fok) ? __logf(__fdividef(u64_to_float(h), c)) : 0.f;
  }
}

// Mattes value without the derivative: one warp per group of 32 joint-histogram
// bins (mattes_group_partial), the last block adds the group partials.  With the
// derivative the same groups are formed by spare warps of the derivative pass
// (k_mattes_pass2_affine, k_bspline_chunks) and summed at its end.
__global__ void __launch_bounds__(kFinalizeThreads) k_mattes_finalize(EvalArgs a) {
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  const int lane = threadIdx.x;
  const double part = mattes_group_partial(a, blockIdx.x, lane);
  if (lane == 0) a.part[blockIdx.x] = part;
  if (!last_block(a.tickets + kTicketFinalize)) return;
  const double s = mattes_value_sum(a.part, (int)gridDim.x, lane);
  if (lane == 0) {
    const int st = mattes_status(a);
    *a.status = st;
    a.out[0] = st == GB_OK ? -1.0 * s : 0.0;  // metrics minimize: value = -MI
    a.out[1] = (double)__ldcg(a.acc_n);
  }
}

#endif  // GB_KERNELS_HELPERS_ONLY

// Streamed record tiles: each block owns a contiguous, tile-aligned range of
// samples; thread 0 keeps kStreamStages tiles of (cache, sample) records in
// flight with bulk asynchronous copies, completed on one mbarrier per stage.
constexpr int kStreamStages = 4;
constexpr int kStreamPer = 2;                     // records per thread and tile
constexpr int kStreamTile = kBlock * kStreamPer;  // records per stage and stream
constexpr size_t kStreamBytes = (size_t)2 * kStreamStages * kStreamTile * sizeof(float4);
// mbarrier polls of a wait under the stalled-copy fault injection (GB_FAULT_STALLED_COPY)
constexpr unsigned kInjectWaitPolls = 256;

// Dynamic shared memory of the Mattes derivative pass: the record stages, the
// bins^2 log(p / pm) table, B column sums and B fixed-bin flags.
__host__ __device__ inline size_t mattes_pass2_smem(int bins) {
  return kStreamBytes + sizeof(float) * (size_t)bins * bins + 8 * (size_t)bins;
}

// With EvalArgs::hist_bulk: the copied histogram and marginals (B^2 + 2B u64, rounded
// up to 16 bytes; the accumulator buffer is padded for the rounding) after the above,
// at a 16-byte boundary.
__host__ __device__ inline size_t mattes_pass2_hist_offset(int bins) { return (mattes_pass2_smem(bins) + 15) / 16 * 16; }
__host__ __device__ inline size_t mattes_pass2_hist_bytes(int bins) {
  return (8 * ((size_t)bins * bins + 2 * (size_t)bins) + 15) / 16 * 16;
}

// The derivative's log(p / pm) table (the same bits as mattes_pratio_build) formed by
// the kBlock streaming threads from the copied histogram hs (then fmarg, colsum).
__device__ __forceinline__ void mattes_pratio_from_copy(const EvalArgs& a, double T, unsigned long long N,
                                                        const unsigned long long* hs, float* dst, float* colf,
                                                        unsigned* fmask) {
  const int B = a.bins;
  const int BB = B * B;
  __shared__ PratioThresholds th_s;
  if (threadIdx.x == 0) th_s = pratio_thresholds(T, N);  // FP64: once per block
  stream_barrier();
  const PratioThresholds th = th_s;
  const unsigned long long* fs = hs + BB;
  const unsigned long long* cs = fs + B;
  for (int k = threadIdx.x; k < B; k += kBlock) {
    colf[k] = cs[k] > th.hthr ? u64_to_float(cs[k]) : 0.f;
    fmask[k] = fs[k] > th.fthr ? 1u : 0u;
  }
  stream_barrier();
  // kBatch independent entries per thread in flight; f = k / B by a multiply-high
  // (exact: k < 2^32 / B)
  constexpr int kBatch = 4;
  const unsigned long long inv = (0x100000000ull + (unsigned)B - 1u) / (unsigned)B;
  for (int k0 = threadIdx.x; k0 < BB; k0 += kBatch * kBlock) {
    unsigned long long h[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int k = k0 + j * kBlock;
      h[j] = (!th.bad && k < BB) ? hs[k] : 0ull;
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int k = k0 + j * kBlock;
      if (k >= BB) break;
      const int f = (int)(((unsigned long long)k * inv) >> 32), m = k - f * B;
      const float c = colf[m];
      dst[k] = (h[j] > th.hthr && c > 0.f && fmask[f]) ? __logf(__fdividef(u64_to_float(h[j]), c)) : 0.f;
    }
  }
  stream_barrier();
}

// Whole tiles spread evenly: block b gets tiles [b T / G, (b + 1) T / G).
__device__ __forceinline__ void block_range(int64_t n, int64_t& b0, int64_t& b1, VGrid vg) {
  const int64_t tiles = (n + kStreamTile - 1) / kStreamTile;
  b0 = min(n, (int64_t)vg.b * tiles / vg.n * kStreamTile);
  b1 = min(n, (int64_t)(vg.b + 1) * tiles / vg.n * kStreamTile);
}

// Threads of a plain pass-2 block: kBlock streaming threads and one group warp.
constexpr int kPass2Threads = kBlock + 32;

// Mattes pass 2, affine: derivative from the cached Parzen terms and gradients.
// Dynamic shared memory: mattes_pass2_smem(bins).
//
// GROUP_WARP (the plain launch, kPass2Threads threads): the block's last warp forms
// the value's FP64 group partial (block b: group b) while the other kBlock threads
// stream the records, so the FP64 chain -- GB300 issues FP64 at a small fraction of
// its FP32 rate -- overlaps the streaming instead of delaying it; the streaming
// threads synchronize per tile on a named barrier of their own.  Without it (the
// batched engine, kBlock threads) the last warp forms the groups before the loop.
template <bool GROUP_WARP>
__device__ __forceinline__ void mattes_pass2_affine_body(const EvalArgs& a, VGrid vg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int kWarps = (GROUP_WARP ? kPass2Threads : kBlock) / 32;
  const int B = a.bins;
  float4* cbuf = reinterpret_cast<float4*>(smem_raw);  // [stage][tile] cache records
  float4* sbuf = cbuf + kStreamStages * kStreamTile;    // [stage][tile] sample records
  float* pr = reinterpret_cast<float*>(smem_raw + kStreamBytes);
  float* colf = pr + B * B;
  unsigned* fmask = reinterpret_cast<unsigned*>(colf + B);
  __shared__ unsigned long long full[kStreamStages];
  __shared__ unsigned long long hbar;  // the histogram copy (hist_bulk)
  __shared__ int failed;
  __shared__ EvalConsts K;
  __shared__ float red[kWarps][12];
  __shared__ DFloat blk[12];
  __shared__ double fin[12];
  int64_t b0, b1;
  block_range(a.n, b0, b1, vg);
  const int ntiles = (int)((b1 - b0 + kStreamTile - 1) / kStreamTile);
  // fault injection: no copy is ever issued, so every wait runs out (after a short limit)
  const bool stall = a.inject_stall != 0;
  const unsigned limit = stall ? kInjectWaitPolls : kWaitLimit;
  const bool streamer = !GROUP_WARP || (int)threadIdx.x < kBlock;
  const bool hb = GROUP_WARP && a.hist_bulk != 0;
  unsigned long long* hsh = reinterpret_cast<unsigned long long*>(smem_raw + mattes_pass2_hist_offset(B));
  int issued = 0;  // thread 0: tiles whose copies are issued
  // tile t -> stage t % kStreamStages; the stage's phase parity is (t / kStreamStages) & 1
  auto issue = [&](int t) {
    const int st = t % kStreamStages;
    const int64_t r0 = b0 + (int64_t)t * kStreamTile;
    const unsigned bytes = (unsigned)(min((int64_t)kStreamTile, b1 - r0) * sizeof(float4));
    const uint64_t pol = l2_policy_evict_first();  // last use of both records in this evaluation
    mbar_arrive_expect_tx(&full[st], 2 * bytes);
    bulk_g2s_hint(cbuf + st * kStreamTile, a.cache + r0, bytes, &full[st], pol);
    bulk_g2s_hint(sbuf + st * kStreamTile, a.samples + r0, bytes, &full[st], pol);
    issued = t + 1;
  };
  if (threadIdx.x == 0) {
    for (int st = 0; st < kStreamStages; ++st) mbar_init(&full[st], 1);
    mbar_init(&hbar, 1);
    mbar_init_fence();
    failed = 0;
  }
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  // this thread's word of the transform constants, the fixed-point total and the valid
  // count are requested before the bulk copies, so that their replies do not queue
  // behind the copies' data
  constexpr int kConstWords = (int)(sizeof(EvalConsts) / 4);
  const int cw = (int)threadIdx.x;
  const float cword = cw < kConstWords ? __ldcg(reinterpret_cast<const float*>(a.consts) + cw) : 0.f;
  const double T = streamer ? __ldcg(&a.marg[0]) : 0.0;
  const unsigned long long N = streamer ? __ldcg(a.acc_n) : 0ull;
  // nFactor = -1 / (MovingImageBinSize * N), Mattes...Threader.hxx:446-457: formed now,
  // off the last block's tail (FP64 division)
  __shared__ double nfac_s;
  // the histogram (first), then the first tiles
  if (threadIdx.x == 0 && !stall) {
    if (hb) {
      const unsigned hbytes = (unsigned)mattes_pass2_hist_bytes(B);
      mbar_arrive_expect_tx(&hbar, hbytes);
      bulk_g2s(hsh, a.hist, hbytes, &hbar);
    }
    for (int t = 0; t < min(kStreamStages, ntiles); ++t) issue(t);
  }
  for (int k = cw; k < kConstWords; k += blockDim.x)
    reinterpret_cast<float*>(&K)[k] = k == cw ? cword : __ldcg(reinterpret_cast<const float*>(a.consts) + k);
  __syncthreads();  // the barriers' initialization and the constants
  float acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = 0.f;
  if (!GROUP_WARP) {
    if (threadIdx.x == 0) nfac_s = -1.0 / (a.m_bs * (double)N);
    mattes_pratio_build<false>(a, T, pr, colf, fmask);
    mattes_value_groups<true>(a, vg);  // the value's FP64 group partials and sum, last warp
    __syncthreads();
  } else if (streamer) {
    if (threadIdx.x == 0) nfac_s = -1.0 / (a.m_bs * (double)N);
    if (hb) {
      if (!mbar_wait(&hbar, 0u, limit)) failed = 1;
      stream_barrier();
      if (!failed) mattes_pratio_from_copy(a, T, N, hsh, pr, colf, fmask);
    } else {
      mattes_pratio_build<true>(a, T, pr, colf, fmask);
    }
  } else {
    // the group warp: its FP64 chain runs while the other warps stream
    const int ng = mattes_groups(B);
    for (int g = vg.b; g < ng; g += vg.n) {
      const double sg = mattes_group_partial(a, g, threadIdx.x & 31);
      if ((threadIdx.x & 31) == 0) a.part[g] = sg;
      mattes_value_group_done(a, ng);
    }
  }
  int t = 0;
  const bool looped = streamer && !failed;  // uniform: `failed` is read after a barrier
  if (looped) {
    // plain FP32 per thread (a thread adds a few dozen samples; the warp tree and the
    // FP64 cross-block sums follow)
    for (; t < ntiles; ++t) {
      const int st = t % kStreamStages;
      const bool landed = mbar_wait(&full[st], (unsigned)(t / kStreamStages) & 1u, limit);
      if (!landed) failed = 1;
      const int64_t r0 = b0 + (int64_t)t * kStreamTile;
      const int cnt = (int)min((int64_t)kStreamTile, b1 - r0);
#pragma unroll
      for (int u = 0; u < kStreamPer; ++u) {
        const int j = threadIdx.x + u * kBlock;
        if (!landed || j >= cnt) continue;
        const float4 cc = cbuf[st * kStreamTile + j];
        const float4 s = sbuf[st * kStreamTile + j];
        if (cc.x != cc.x) continue;  // NaN term: rejected sample
        int pdfm;
        float tt, d[4];
        parzen_window(cc.x, B, pdfm, tt);
        parzen_deriv(tt, d);
        const float* row = pr + __float_as_int(s.w) * B + pdfm;
        const float w = row[0] * d[0] + row[1] * d[1] + row[2] * d[2] + row[3] * d[3];
        const float3 v = jac_vec(K, s.x, s.y, s.z);
        const float t0 = w * cc.y, t1 = w * cc.z, t2 = w * cc.w;
        acc[0] = fmaf(t0, v.x, acc[0]); acc[1] = fmaf(t0, v.y, acc[1]); acc[2] = fmaf(t0, v.z, acc[2]);
        acc[3] = fmaf(t1, v.x, acc[3]); acc[4] = fmaf(t1, v.y, acc[4]); acc[5] = fmaf(t1, v.z, acc[5]);
        acc[6] = fmaf(t2, v.x, acc[6]); acc[7] = fmaf(t2, v.y, acc[7]); acc[8] = fmaf(t2, v.z, acc[8]);
        acc[9] += t0; acc[10] += t1; acc[11] += t2;
      }
      // stage st consumed by every streaming thread; `failed` seen by all of them
      if (GROUP_WARP) stream_barrier();
      else __syncthreads();
      if (failed) break;
      if (threadIdx.x == 0 && t + kStreamStages < ntiles) {
        fence_proxy_async_smem();
        issue(t + kStreamStages);
      }
    }
  }
  if (GROUP_WARP) __syncthreads();  // the group warp joins
  if (failed) {
    // a copy never completed: report, wait (bounded) for the copies still in flight, leave
    if (threadIdx.x == 0) {
      atomicExch(a.status, GB_ERR_TIMEOUT);
      // the tile (or, before the loop, the histogram) whose wait ran out is not waited on again
      for (int u = looped ? t + 1 : 0; u < issued; ++u)
        mbar_wait(&full[u % kStreamStages], (unsigned)(u / kStreamStages) & 1u);
    }
    return;
  }
  KahanF kacc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    kacc[k].s = acc[k];
    kacc[k].c = 0.f;
  }
  block_sums_df<12>(kacc, red, blk);
  DFloat* part = reinterpret_cast<DFloat*>(a.part + kPartPass2);
  // staged form: the last block requests every block partial at once into the (now idle)
  // record stages, then sums them from shared memory
  const bool staged = vg.n <= kFlatMaxBlocks && (size_t)(vg.n * 12) * 8 <= kStreamBytes;
  if (staged) {
    if (!grid_ticket_flat_df<12>(blk, part, a.tickets + kTicketPass2, vg)) return;
    DFloat* sp = reinterpret_cast<DFloat*>(smem_raw);
    stage_u64(reinterpret_cast<const unsigned long long*>(part), vg.n * 12,
              reinterpret_cast<unsigned long long*>(sp));
    __syncthreads();
    __shared__ DFloat fin_s[12];
    strided_sums_df_shared<12>(sp, vg.n, fin_s, kWarps);
    __syncthreads();
    for (int k = threadIdx.x; k < 12; k += blockDim.x) fin[k] = df_to_double(fin_s[k]);
    __syncthreads();
  } else {
    const bool last = vg.n <= kFlatMaxBlocks
                          ? grid_sums_flat_df<12>(blk, part, a.tickets + kTicketPass2, fin, vg)
                          : grid_sums_df<12>(blk, part, reinterpret_cast<DFloat*>(a.grp), a.tickets + kTicketPass2,
                                             fin, vg);
    if (!last) return;
  }
  // last block: the value summed by the warp that completed the last group (written before
  // its block's ticket); warp 0, one derivative entry per lane
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int st = N == 0 ? GB_ERR_NO_VALID_POINTS : T * kQInv >= DBL_EPSILON ? GB_OK : GB_ERR_JOINT_PDF_SUM_ZERO;
    const double s = __ldcg(&a.part[kPartValue]);
    const double nFactor = nfac_s;
    if (lane == 0) {
      *a.status = st;
      a.out[1] = (double)N;
      a.out[0] = st == GB_OK ? -1.0 * s : 0.0;
    }
    for (int p = lane; p < a.nparams; p += 32) a.out[2 + p] = st == GB_OK ? fin[p] * nFactor : 0.0;
  }
}

#ifndef GB_KERNELS_HELPERS_ONLY
__global__ void __launch_bounds__(kPass2Threads, 3) k_mattes_pass2_affine(EvalArgs a) {
  mattes_pass2_affine_body<true>(a, hw_grid());
}
#endif  // GB_KERNELS_HELPERS_ONLY

}  // namespace gb
