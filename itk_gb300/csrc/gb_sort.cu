// gb_sort.cu -- device key/value sort used at Initialize to put samples in
// spatial (Morton / B-spline cell) order.  Kept in its own translation unit so
// the radix-sort templates compile in parallel with the metric kernels.
#include <cub/device/device_radix_sort.cuh>

#include <cstdint>

#include "gb_internal.h"

namespace gb {

// Sorts (keys, values) ascending by key on `stream`.  Temporary storage is
// allocated and freed here (Initialize-time only).
cudaError_t sort_pairs_u64(const uint64_t* keys_in, uint64_t* keys_out, const uint32_t* vals_in, uint32_t* vals_out,
                           int64_t n, int end_bit, cudaStream_t stream) {
  size_t temp_bytes = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys_in, keys_out, vals_in, vals_out,
                                                  (int64_t)n, 0, end_bit, stream);
  if (e != cudaSuccess) return e;
  void* temp = nullptr;
  e = cudaMallocAsync(&temp, temp_bytes, stream);
  if (e != cudaSuccess) return e;
  e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys_in, keys_out, vals_in, vals_out, (int64_t)n, 0, end_bit,
                                      stream);
  cudaError_t e2 = cudaFreeAsync(temp, stream);
  return e != cudaSuccess ? e : e2;
}

}  // namespace gb
