// NVTX ranges around the phases of the fused step, for timeline tools
// (Nsight Systems; `ncu --nvtx --nvtx-include "jld_ldl_step/"` to capture one
// step's kernels).  Host-side markers only: they launch nothing and are
// legal inside stream capture; without an attached tool a push or pop is
// one check of a function pointer.  Where the CUDA toolkit ships no nvtx3
// headers the ranges compile to nothing.
#pragma once

#include <cstdio>

#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define JLD_HAVE_NVTX 1
#endif
#endif

namespace jld {

// Pushes a range on construction and pops it on destruction, so every
// return path of the enclosing scope closes it.
class ScopedRange {
 public:
  explicit ScopedRange(const char* name) { push(name); }
  // name with one integer, e.g. ("jld adjoint layer %d", l)
  ScopedRange(const char* fmt, int i) {
    char buf[64];
    std::snprintf(buf, sizeof buf, fmt, i);
    push(buf);
  }
  ~ScopedRange() {
#ifdef JLD_HAVE_NVTX
    nvtxRangePop();
#endif
  }
  ScopedRange(const ScopedRange&) = delete;
  ScopedRange& operator=(const ScopedRange&) = delete;

 private:
  static void push(const char* name) {
#ifdef JLD_HAVE_NVTX
    nvtxRangePushA(name);
#else
    (void)name;
#endif
  }
};

}  // namespace jld
