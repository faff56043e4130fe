// gb_noalloc.cu -- MeanSquares value and derivative under an affine transform
// for callers that cannot allocate device memory.
//
// The metric handles (gb_metric_*) own their scratch and allocate it in
// Initialize.  Some callers cannot call cudaMalloc at all: code running inside
// another framework's memory pool or arena, real-time loops that forbid
// allocation after start-up, and libraries embedded in hosts that account for
// every device allocation.  This entry point takes all inputs and the output
// in caller-owned device memory and keeps its own scratch -- block partial
// sums and counters -- in one file-scope __device__ array of
// kNoAllocScratchBytes (about 112 KiB), which every GPU that loads this
// library holds until the process exits.
//
// The array's device address belongs to a CUDA context, not to a device: a
// cudaDeviceReset re-creates the primary context (and reloads this module), and
// a caller may make the call under a context of its own.  The address is
// therefore looked up once per context, keyed by the context's unique ID
// (cuCtxGetId, never reused within a process), with that context current.
#define GB_KERNELS_HELPERS_ONLY
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "gb_internal.h"
#include "gb_kernels.cuh"

namespace gb {
namespace {

constexpr int kNoAllocMaxBlocks = 1024;  // grid cap: the partial-sum capacity of the scratch array
constexpr int kNoAllocGroups = kNoAllocMaxBlocks / kGroup;
constexpr int kNoAllocValues = 13;  // value + 12 affine derivative terms
// byte layout: header (counter, tickets; cleared by every call) | block partials | group partials
constexpr size_t kNoAllocHeaderBytes = 1024;
constexpr size_t kNoAllocPartOffset = kNoAllocHeaderBytes;
constexpr size_t kNoAllocGroupOffset = kNoAllocPartOffset + sizeof(double) * kNoAllocMaxBlocks * kNoAllocValues;
constexpr size_t kNoAllocScratchBytes = kNoAllocGroupOffset + sizeof(double) * kNoAllocGroups * kNoAllocValues;
static_assert(8 + 4 * (kNoAllocGroups + 1) <= kNoAllocHeaderBytes, "scratch header too small");
static_assert(kNoAllocScratchBytes == GB_NOALLOC_SCRATCH_BYTES, "header constant out of date");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch and the grid size, per CUDA context.
constexpr int kMaxContexts = 64;
struct ScratchEntry {
  unsigned long long ctx_id;  // 0: unused
  void* ptr;
  int blocks;
};
std::mutex g_setup_mutex;
ScratchEntry g_entries[kMaxContexts] = {};
int g_next_entry = 0;  // round-robin replacement once every entry is used

struct NoAllocArgs {
  EvalConsts K;  // by value: nothing to copy into device memory first
  const float4* __restrict__ samples;
  int64_t n;
  const float4* __restrict__ mov4;
  int nx, ny, nz;
  unsigned char* scratch;
  double* out;
};

// The MeanSquares per-sample body of k_msq_affine<kGradImage>, with the
// constants taken from the kernel parameters and the scratch in g_noalloc_scratch.
__global__ void __launch_bounds__(kBlock) k_msq_affine_noalloc(NoAllocArgs na) {
  __shared__ EvalConsts K;
  __shared__ float red[kBlock / 32][kNoAllocValues];
  __shared__ double blk[kNoAllocValues], fin[kNoAllocValues];
  if (threadIdx.x == 0) K = na.K;
  __syncthreads();
  unsigned long long* acc_n = reinterpret_cast<unsigned long long*>(na.scratch);
  unsigned* tickets = reinterpret_cast<unsigned*>(na.scratch + 8);
  double* part = reinterpret_cast<double*>(na.scratch + kNoAllocPartOffset);
  double* grp = reinterpret_cast<double*>(na.scratch + kNoAllocGroupOffset);
  KahanF acc[kNoAllocValues];
#pragma unroll
  for (int k = 0; k < kNoAllocValues; ++k) acc[k].zero();
  unsigned nv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < na.n; i += stride) {
    const float4 s = __ldcs(na.samples + i);
    const CIdx c = to_cidx(map_pos(K.map, s.x, s.y, s.z));
    if (!ci_inside(c, na.nx, na.ny, na.nz)) continue;
    const float4 v = gather4(na.mov4, make_stencil(c, na.nx, na.ny, na.nz), na.nx, na.ny);
    const float diff = s.w - v.x;
    acc[0].add(diff * diff);
    ++nv;
    const float t = 2.f * diff;
    const float3 q = jac_vec(K, s.x, s.y, s.z);
    const float t0 = t * v.y, t1 = t * v.z, t2 = t * v.w;
    acc[1].add(t0 * q.x); acc[2].add(t0 * q.y); acc[3].add(t0 * q.z);
    acc[4].add(t1 * q.x); acc[5].add(t1 * q.y); acc[6].add(t1 * q.z);
    acc[7].add(t2 * q.x); acc[8].add(t2 * q.y); acc[9].add(t2 * q.z);
    acc[10].add(t0); acc[11].add(t1); acc[12].add(t2);
  }
  block_count(nv, acc_n);
  block_sums<kNoAllocValues>(acc, red, blk);
  if (!grid_sums<kNoAllocValues>(blk, part, grp, tickets, fin)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(acc_n);
    if (N == 0) {
      na.out[0] = DBL_MAX;  // VerifyNumberOfValidPoints, itkObjectToObjectMetric.hxx:512-527
      na.out[1] = 0.0;
      for (int p = 0; p < 12; ++p) na.out[2 + p] = 0.0;
    } else {
      na.out[0] = fin[0] / (double)N;
      na.out[1] = (double)N;
      for (int p = 0; p < 12; ++p) na.out[2 + p] = fin[1 + p] / (double)N;
    }
  }
}

// The unique ID of the calling thread's current context (0 when none is
// current), through the runtime's driver entry points (no libcuda link).
int current_context_id(unsigned long long* id) {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  static cudaError_t load_err = cudaSuccess;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSuccess, q2 = cudaDriverEntryPointSuccess;
    load_err = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&get_current), 4000,
                                                cudaEnableDefault, &q1);
    if (load_err == cudaSuccess)
      load_err = cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&get_id), 12000,
                                                  cudaEnableDefault, &q2);
    if (load_err == cudaSuccess && (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess))
      load_err = cudaErrorSymbolNotFound;
  });
  if (load_err != cudaSuccess || !get_current || !get_id)
    return fail(GB_ERR_CUDA, std::string("driver entry points cuCtxGetCurrent / cuCtxGetId: ") +
                                 cudaGetErrorString(load_err));
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return fail(GB_ERR_CUDA, "cuCtxGetCurrent failed");
  *id = 0;
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return fail(GB_ERR_CUDA, "cuCtxGetId failed");
  return GB_OK;
}

// Once per context, with that context current: the device address of the
// scratch array (the host-side symbol is only a stand-in) and the grid size.
int setup_context(int dev, void** scratch, int* blocks) {
  unsigned long long id = 0;
  int rc = current_context_id(&id);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (id)
    for (const ScratchEntry& en : g_entries)
      if (en.ctx_id == id) {
        *scratch = en.ptr;
        *blocks = en.blocks;
        return GB_OK;
      }
  // the lookup makes the device's primary context current when no context was
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(GB_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
  if (!id) {
    rc = current_context_id(&id);
    if (rc) return rc;
    if (!id) return fail(GB_ERR_CUDA, "no CUDA context is current after the symbol lookup");
  }
  int sms = 0, per_sm = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_msq_affine_noalloc, kBlock, 0);
  if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
  ScratchEntry& en = g_entries[g_next_entry];
  g_next_entry = (g_next_entry + 1) % kMaxContexts;
  en.ctx_id = id;
  en.ptr = p;
  en.blocks = std::max(1, std::min(kNoAllocMaxBlocks, sms * std::max(per_sm, 1)));
  *scratch = en.ptr;
  *blocks = en.blocks;
  return GB_OK;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int gb_msq_affine_noalloc(const void* device_samples, int64_t n, const void* device_moving,
                                     const int64_t moving_size[3], const double moving_spacing[3],
                                     const double moving_origin[3], const double moving_direction[9],
                                     const double params[12], const double center[3], double* device_out,
                                     uint64_t stream) {
  if (!device_samples || !device_moving || !moving_size || !moving_spacing || !moving_origin || !moving_direction ||
      !params || !center || !device_out)
    return fail(GB_ERR_BAD_ARG, "null argument");
  if (n < 1) return fail(GB_ERR_BAD_ARG, "at least one sample is required");
  if (n > GB_NOALLOC_MAX_SAMPLES)
    return fail(GB_ERR_BAD_ARG, "gb_msq_affine_noalloc takes at most 2^31-1 samples per call");
  Geom mg;
  int rc = geom_init(mg, moving_size, moving_spacing, moving_origin, moving_direction);
  if (rc) return rc;
  if (mg.voxels() > GB_NOALLOC_MAX_VOXELS)
    return fail(GB_ERR_BAD_ARG, "gb_msq_affine_noalloc takes moving images of at most 2^31 voxels");
  for (int i = 0; i < 12; ++i)
    if (!std::isfinite(params[i])) return fail(GB_ERR_BAD_ARG, "non-finite transform parameter");
  if (((uintptr_t)device_samples | (uintptr_t)device_moving) & 15)
    return fail(GB_ERR_BAD_ARG, "samples and moving image must be 16-byte aligned (float4 records)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  void* scratch = nullptr;
  int blocks = 0;
  rc = setup_context(dev, &scratch, &blocks);
  if (rc) return rc;

  NoAllocArgs na;
  affine_consts(params, center, mg.p2i, mg.origin, nullptr, nullptr, na.K);
  na.samples = static_cast<const float4*>(device_samples);
  na.n = n;
  na.mov4 = static_cast<const float4*>(device_moving);
  na.nx = (int)mg.size[0];
  na.ny = (int)mg.size[1];
  na.nz = (int)mg.size[2];
  na.scratch = static_cast<unsigned char*>(scratch);
  na.out = device_out;
  const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: clear the counter and tickets
  e = cudaMemsetAsync(scratch, 0, kNoAllocHeaderBytes, st);
  if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  const int64_t want = (n + kBlock - 1) / kBlock;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, blocks));
  k_msq_affine_noalloc<<<grid, kBlock, 0, st>>>(na);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("k_msq_affine_noalloc: ") + cudaGetErrorString(e));
  return GB_OK;
}
