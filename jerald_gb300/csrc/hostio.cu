// Host-to-device staging by a kernel that reads pinned host memory directly.
//
// On a GB300 node the GPU reaches the Grace host memory coherently over
// NVLink-C2C, so a kernel can load page-locked host buffers through their
// unified address.  A few CTAs of 16-byte loads stream a buffer into device
// memory without the copy engines; used by the host feed of the fused step
// (jerald_gb300.ldl.HostFeed) to bring each step's positions and target in.

#include "common.cuh"

namespace jld {

// dst[i] = src[i] for n16 16-byte words, then the tail bytes.  CTAs of 1024
// threads with 8 loads of 16 bytes in flight each (128 KB per CTA): a copy
// running under the fused step holds a few whole SMs, and the step's
// persistent kernels (which hand out their tiles and particle batches
// dynamically) run on the others.  Many small CTAs instead would hold a
// slot on many SMs, and the step's kernels that fill an SM's register file
// could not use those SMs at all.
constexpr int kHostCopyThreads = 1024;
__global__ void __launch_bounds__(kHostCopyThreads, 1)
host_stream_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, int64_t n16,
                   const unsigned char* __restrict__ src_tail, unsigned char* __restrict__ dst_tail, int tail) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // eight independent loads in flight per thread
  for (; i + 7 * stride < n16; i += 8 * stride) {
    uint4 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = src[i + k * stride];
#pragma unroll
    for (int k = 0; k < 8; ++k) dst[i + k * stride] = v[k];
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
  const unsigned grid = (unsigned)std::max(1, std::min(ctas > 0 ? ctas : 4, 2 * sm_count()));
  host_stream_kernel<<<grid, kHostCopyThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const uint4*>(at.devicePointer ? at.devicePointer : src_host), reinterpret_cast<uint4*>(dst),
      n16, reinterpret_cast<const unsigned char*>(at.devicePointer ? at.devicePointer : src_host) + n16 * 16,
      reinterpret_cast<unsigned char*>(dst) + n16 * 16, tail);
  JLD_LAUNCH_CHECK("host_stream_kernel");
  return JLD_OK;
}

}  // extern "C"
