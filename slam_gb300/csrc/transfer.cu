// Small host <-> device transfers of the tracking calls (argument blocks,
// tracking states, proposals) as a copy kernel over pinned host memory,
// which the device addresses directly (unified addressing), instead of the
// copy engines.  A caller that streams its frames in with large
// asynchronous copies keeps the copy engines busy for tens of milliseconds;
// a small cudaMemcpyAsync of the tracker queued behind them would hold the
// tracking call until they drain.  The kernel reads or writes host memory
// over the host link directly and does not wait for them.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/slam_gb300.h"
#include "odo_internal.h"

namespace slamgb {
namespace {

__global__ void k_host_copy16(uint4 *__restrict__ dst, const uint4 *__restrict__ src, size_t n16) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
__global__ void k_host_copy1(uint8_t *__restrict__ dst, const uint8_t *__restrict__ src, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

}  // namespace

cudaError_t launch_host_copy(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    if (bytes == 0) return cudaSuccess;
    const bool aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | bytes) & 15) == 0;
    const size_t units = aligned ? bytes / 16 : bytes;
    size_t blocks = (units + 255) / 256;
    if (blocks > 1216) blocks = 1216;  // 8 blocks per SM of a 152-SM GPU: enough requests in flight on the link
    if (aligned)
        k_host_copy16<<<(unsigned)blocks, 256, 0, s>>>(static_cast<uint4 *>(dst), static_cast<const uint4 *>(src),
                                                        units);
    else
        k_host_copy1<<<(unsigned)blocks, 256, 0, s>>>(static_cast<uint8_t *>(dst), static_cast<const uint8_t *>(src),
                                                       units);
    return cudaGetLastError();
}

}  // namespace slamgb

extern "C" int odo_host_copy(void *dst, const void *src, size_t bytes, void *stream) {
    if (!dst || !src) return ODO_ERR_ARG;
    return slamgb::launch_host_copy(dst, src, bytes, (cudaStream_t)stream) == cudaSuccess ? ODO_OK : ODO_ERR_CUDA;
}
