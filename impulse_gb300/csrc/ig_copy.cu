// ig_copy.cu -- byte copies run by the SMs, for host memory the GPU reaches
// through the host's page tables (pageable memory on a GPU with address
// translation services).  A copy engine moving pageable memory waits for the
// host, so the host-memory pipeline's copies would not overlap; these kernels
// are ordinary asynchronous launches on the pipeline's streams.
#include <algorithm>
#include <cstdint>

#include "ig_launch.h"

namespace ig {

// n units of W bytes; four units in flight per thread and iteration
template <class U>
__global__ void __launch_bounds__(256) k_copy_units(const U *__restrict__ src, U *__restrict__ dst, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const U v0 = src[i], v1 = src[i + stride], v2 = src[i + 2 * stride], v3 = src[i + 3 * stride];
        dst[i] = v0;
        dst[i + stride] = v1;
        dst[i + 2 * stride] = v2;
        dst[i + 3 * stride] = v3;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

template <class U> static cudaError_t copy_go(const void *src, void *dst, size_t bytes, int sms, cudaStream_t st)
{
    const size_t n = bytes / sizeof(U);
    const size_t want = (n + 4 * 256 - 1) / (4 * 256);
    const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 8));
    k_copy_units<U><<<grid, 256, 0, st>>>((const U *)src, (U *)dst, n);
    return cudaGetLastError();
}

cudaError_t launch_copy(const void *src, void *dst, size_t bytes, int sms, cudaStream_t st)
{
    if (bytes == 0) return cudaSuccess;
    // widest unit that both addresses and the size are multiples of
    const uintptr_t m = (uintptr_t)src | (uintptr_t)dst | (uintptr_t)bytes;
    if (m % 16 == 0) return copy_go<uint4>(src, dst, bytes, sms, st);
    if (m % 8 == 0) return copy_go<uint2>(src, dst, bytes, sms, st);
    if (m % 4 == 0) return copy_go<uint32_t>(src, dst, bytes, sms, st);
    return copy_go<uint8_t>(src, dst, bytes, sms, st);
}

}  // namespace ig
