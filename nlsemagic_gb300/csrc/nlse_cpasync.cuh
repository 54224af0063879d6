// Asynchronous global -> shared copies (cp.async, sm_80 and later) for tile
// staging: every copy of a thread is in flight at once and no register holds
// the data on the way.  A copy whose source lies outside the grid fills its
// shared-memory cell with zeros (source size 0; the source address given is
// then a valid one that is not read).
#pragma once

namespace nlse {

template <int BYTES>
__device__ __forceinline__ void cp_async(void* sdst, const void* gsrc, bool valid) {
  static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  const int n = valid ? BYTES : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gsrc),
               "n"(BYTES), "r"(n)
               : "memory");
}

// Hint: fetch the line holding p into L2 (no register receives it).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}

// Wait for all of this thread's copies; a block barrier after it makes every
// thread's copies visible to the block.
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

}  // namespace nlse
