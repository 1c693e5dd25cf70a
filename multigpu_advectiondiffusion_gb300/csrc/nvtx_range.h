// nvtx_range.h -- an NVTX range around one C-ABI call (host side only, not installed).
//
// Each public entry point that launches work opens a range named after itself, so a profiler can
// attribute and filter the kernels (and graph launches) one call issued, e.g.
//   ncu --nvtx --nvtx-include "adv_heat_run/" ...
// NVTX 3 is header-only: with no tool attached (NVTX_INJECTION64_PATH unset) the first call
// finds no injection library and every later push and pop returns at once. A toolkit installed
// without its NVTX headers builds the ranges as no-ops.
#pragma once

#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define ADV_HAVE_NVTX 1
#endif
#endif

namespace adv {

class NvtxRange {
 public:
#ifdef ADV_HAVE_NVTX
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
#else
  explicit NvtxRange(const char*) {}
#endif
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace adv

#define ADV_NVTX_RANGE(name) ::adv::NvtxRange adv_nvtx_range_(name)
