// Host-to-device staging by a kernel that reads pinned host memory directly.
//
// On a GB300 node the GPU reaches the Grace host memory coherently over
// NVLink-C2C, so a kernel can load page-locked host buffers through their
// unified address.  A few CTAs of 16-byte loads stream a buffer into device
// memory without the copy engines; used by the host feed of the fused step
// (jerald_gb300.ldl.HostFeed) to bring each step's positions and target in.

#include "common.cuh"

namespace jld {

// dst[i] = src[i] for n16 16-byte words, then the tail bytes.
__global__ void __launch_bounds__(512)
host_stream_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, int64_t n16,
                   const unsigned char* __restrict__ src_tail, unsigned char* __restrict__ dst_tail, int tail) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // four independent loads in flight per thread
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
  if (blockIdx.x == 0 && threadIdx.x < tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

}  // namespace jld

using namespace jld;

extern "C" {

JLD_API int jld_copy_from_host(jld_stream_t stream, void* dst, const void* src_host, size_t bytes, int32_t ctas) {
  clear_error();
  if (bytes == 0) return JLD_OK;
  if (!dst || !src_host) return set_error(JLD_ERR_ARG, "jld_copy_from_host: NULL pointer");
  if (((uintptr_t)dst | (uintptr_t)src_host) & 15u)
    return set_error(JLD_ERR_ARG, "jld_copy_from_host: both buffers must be 16-byte aligned");
  cudaPointerAttributes at;
  JLD_CUDA_TRY(cudaPointerGetAttributes(&at, src_host));
  if (at.type != cudaMemoryTypeHost)
    return set_error(JLD_ERR_ARG, "jld_copy_from_host: source is not page-locked host memory");
  const int64_t n16 = (int64_t)(bytes / 16);
  const int tail = (int)(bytes - (size_t)n16 * 16);
  const unsigned grid = (unsigned)std::max(1, std::min(ctas > 0 ? ctas : 2 * sm_count(), 4 * sm_count()));
  host_stream_kernel<<<grid, 512, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const uint4*>(at.devicePointer ? at.devicePointer : src_host), reinterpret_cast<uint4*>(dst),
      n16, reinterpret_cast<const unsigned char*>(at.devicePointer ? at.devicePointer : src_host) + n16 * 16,
      reinterpret_cast<unsigned char*>(dst) + n16 * 16, tail);
  JLD_LAUNCH_CHECK("host_stream_kernel");
  return JLD_OK;
}

}  // extern "C"
