// Status strings, the thread-local error message and the stateless layout
// entry points (initLayout / clean of lib/cpu.cc:29-49).

#include <vector>

#include "common.cuh"

#include <string.h>

#include <map>
#include <mutex>
#include <utility>

namespace jld {

static thread_local char g_msg[512] = "";

int set_error(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  return status;
}

void clear_error() { g_msg[0] = '\0'; }

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (dev >= 0 && dev < 64 && cached[dev]) return cached[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    n = 148;
  if (dev >= 0 && dev < 64) cached[dev] = n;
  return n;
}

int resident_blocks_ptr(const void* func, int block, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<std::pair<const void*, int>, std::pair<int, size_t>>, int> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(std::make_pair(func, dev), std::make_pair(block, smem));
  auto it = done.find(key);
  if (it != done.end()) return it->second;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, block, smem) != cudaSuccess || per_sm < 1) {
    (void)cudaGetLastError();
    per_sm = 1;
  }
  done[key] = per_sm;
  return per_sm;
}

int ensure_smem_ptr(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  JLD_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_pair(func, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return JLD_OK;
  // The limit is per kernel (the opt-in maximum minus the kernel's static
  // shared memory), so raise it exactly to what this launch needs.
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(JLD_ERR_UNSUPPORTED, "kernel cannot get %zu bytes of dynamic shared memory: %s", bytes,
                     cudaGetErrorString(e));
  }
  done[key] = bytes;
  return JLD_OK;
}

}  // namespace jld

extern "C" {

const char* jld_version(void) { return "jerald-gb300 0.1 (sm_103a)"; }

const char* jld_status_string(int status) {
  switch (status) {
    case JLD_OK: return "ok";
    case JLD_ERR_ARG: return "invalid argument";
    case JLD_ERR_UNSUPPORTED: return "unsupported size";
    case JLD_ERR_WORKSPACE: return "workspace too small";
    case JLD_ERR_CUDA: return "CUDA error";
    case JLD_ERR_TIMEOUT: return "device wait timed out";
    case JLD_ERR_NOPLAN: return "FFT plan missing during stream capture";
    default: return "unknown status";
  }
}

const char* jld_last_error(void) { return jld::g_msg; }

// The reference keeps up to five decomposition layouts indexed by lyidx
// (lib/cpu.cc:15, jaxpops_bind.py:157).  This library keeps none; the entry
// points only validate their arguments so callers get the same errors.
int jld_init_layout(int32_t commsize, int32_t lyidx) {
  jld::clear_error();
  if (commsize != 1)
    return jld::set_error(JLD_ERR_UNSUPPORTED, "initLayout: world size %d (only 1 is supported)",
                          commsize);
  if (lyidx < 0 || lyidx > 4)
    return jld::set_error(JLD_ERR_ARG, "initLayout: lyidx needs to be between 0 and 4");
  return JLD_OK;
}

// Kernel nodes of a captured CUDA graph (the launches one replay issues).
int jld_graph_kernel_nodes(void* graph, int64_t* kernels) {
  jld::clear_error();
  if (!graph || !kernels) return jld::set_error(JLD_ERR_ARG, "jld_graph_kernel_nodes: NULL argument");
  size_t n = 0;
  JLD_CUDA_TRY(cudaGraphGetNodes((cudaGraph_t)graph, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  if (n) JLD_CUDA_TRY(cudaGraphGetNodes((cudaGraph_t)graph, nodes.data(), &n));
  int64_t k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    JLD_CUDA_TRY(cudaGraphNodeGetType(nodes[i], &t));
    if (t == cudaGraphNodeTypeKernel) ++k;
  }
  *kernels = k;
  return JLD_OK;
}

int jld_clean(int32_t lyidx) {
  jld::clear_error();
  if (lyidx < 0 || lyidx > 4)
    return jld::set_error(JLD_ERR_ARG, "clean: lyidx needs to be between 0 and 4");
  return JLD_OK;
}

}  // extern "C"
