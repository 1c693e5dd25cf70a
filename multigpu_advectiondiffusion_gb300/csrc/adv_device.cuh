// adv_device.cuh -- sm_103a device helpers: mbarrier, TMA (cp.async.bulk.tensor), cp.async,
// bounded waits. Every wait has a wall-clock limit; on expiry the kernel records
// ADV_ERR_TIMEOUT in the device status word and the caller returns early, so no launch can
// spin forever.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace adv {

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Records the first error code in the device status word (0 = OK).
__device__ __forceinline__ void raise_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// Bounds checking, compiled into the checked build of the library only (-DADV_BOUNDS_CHECK,
// libadvdiff_checked.so): ADV_IN_RANGE(i, n, status) is true when 0 <= i < n; otherwise it records
// ADV_ERR_BOUNDS in the device status word and is false, and the caller skips the access (no trap,
// no fault). In the normal build it is the constant true and the checks vanish.
#ifdef ADV_BOUNDS_CHECK
__device__ __forceinline__ bool adv_in_range(long long i, long long n, int* status) {
  if (i >= 0 && i < n) return true;
  raise_status(status, 8 /* ADV_ERR_BOUNDS */);
  return false;
}
#define ADV_IN_RANGE(i, n, status) ::adv::adv_in_range((long long)(i), (long long)(n), (status))
#else
#define ADV_IN_RANGE(i, n, status) true
#endif

// ------------------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: returns false (and raises ADV_ERR_TIMEOUT) if the phase did not complete within
// limit_ns of the first failed poll.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int* status,
                                                  unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer_ns() - t0 > limit_ns) {
      raise_status(status, 3 /* ADV_ERR_TIMEOUT */);
      return false;
    }
  }
  return true;
}

// Warp-convergent bounded wait: lane 0 polls, the other lanes wait at the shuffle instead of
// spinning (no divergent spin loops eating issue slots), then every lane performs its own
// (immediately successful) try_wait so it acquires the completed phase itself.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, unsigned parity, int* status, int lane) {
  int ok = 1;
  if (lane == 0) ok = mbar_wait_bounded(bar, parity, status) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  if (ok) (void)mbar_try_wait(bar, parity);
  return ok != 0;
}

// ----------------------------------------------------------------------------- TMA
// 3D tiled load of one box into shared memory, completion signalled on `bar` (complete_tx).
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* tmap, int x, int y,
                                            int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

// ------------------------------------------------------------------------ cp.async
// 4- or 8-byte asynchronous copy global -> shared; src_bytes == 0 zero-fills the destination.
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* smem_dst, const void* gsrc, bool valid) {
  const int sz = valid ? BYTES : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(smem_u32(smem_dst)), "l"(gsrc),
               "n"(BYTES), "r"(sz)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// ----------------------------------------------------------------- max|u| reduction
// |v| as an order-preserving unsigned key (NaN sorts above +inf, so it propagates).
__device__ __forceinline__ unsigned abs_key(float v) { return __float_as_uint(v) & 0x7fffffffu; }
__device__ __forceinline__ unsigned long long abs_key(double v) {
  return static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned warp_max(unsigned v) {
  return __reduce_max_sync(0xffffffffu, v);
}
__device__ __forceinline__ unsigned long long warp_max(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ float key_to_value(unsigned k) { return __uint_as_float(k); }
__device__ __forceinline__ double key_to_value(unsigned long long k) {
  return __longlong_as_double(static_cast<long long>(k));
}

template <class T> struct KeyOf;
template <> struct KeyOf<float> { using type = unsigned; };
template <> struct KeyOf<double> { using type = unsigned long long; };

}  // namespace adv
