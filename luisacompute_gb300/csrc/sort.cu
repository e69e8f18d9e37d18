// sort.cu — Morton key/value radix sort for the BVH builds.  A library call
// into CUB (CUDA toolkit), kept in its own translation unit so that the
// template instantiation compiles in parallel with the kernels.
#include <cub/device/device_radix_sort.cuh>

#include "lcx_internal.h"

namespace lcx {

size_t sort_temp_bytes(uint32_t n) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, static_cast<const unsigned long long *>(nullptr),
                                    static_cast<unsigned long long *>(nullptr), static_cast<const uint32_t *>(nullptr),
                                    static_cast<uint32_t *>(nullptr), int(n), 0, 63);
    return bytes;
}

cudaError_t sort_pairs(void *tmp, size_t tmp_bytes, const unsigned long long *kin, unsigned long long *kout,
                       const uint32_t *vin, uint32_t *vout, uint32_t n, uint32_t end_bit, cudaStream_t s) {
    size_t bytes = tmp_bytes;
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, kin, kout, vin, vout, int(n), 0, int(end_bit), s);
}

}  // namespace lcx
