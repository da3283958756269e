/*
 * device_common.cuh -- device helpers shared by the persistent traversal
 * kernels (single-source, frontier-matrix batch, multi-instance, Brandes).
 */
#ifndef TBFS_DEVICE_COMMON_CUH
#define TBFS_DEVICE_COMMON_CUH

#include <cuda_runtime.h>

#include "tbfs.h"
#include "tbfs_internal.h"

namespace tbfs {
namespace dev {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile(const int *p) {
  return *reinterpret_cast<const volatile int *>(p);
}

/* a + b in uint64; flags sums that reach 2^63 or wrap */
__device__ __forceinline__ unsigned long long add_chk(unsigned long long a,
                                                      unsigned long long b, bool &ovf) {
  const unsigned long long s = a + b;
  if (s < a || (s >> 63)) ovf = true;
  return s;
}

/* *acc += x for a 64-bit accumulator in shared memory kept as two words in
 * separate arrays (*lo, *hi), with two native 32-bit atomics: the low word's
 * returned old value yields the carry, which is folded into the high word's
 * add; the high word's returned old value detects sums reaching 2^63.
 * Exact modulo 2^64 under any interleaving. */
__device__ __forceinline__ void smem_add_split(unsigned *lo, unsigned *hi, unsigned long long x,
                                               bool &ovf) {
  const unsigned xl = (unsigned)x, xh = (unsigned)(x >> 32);
  const unsigned old_l = atomicAdd(lo, xl);
  const unsigned carry = (old_l + xl) < old_l ? 1u : 0u;
  const unsigned add_h = xh + carry;
  const unsigned old_h = atomicAdd(hi, add_h);
  const unsigned new_h = old_h + add_h;
  if (new_h < old_h || (new_h >> 31) || add_h < xh) ovf = true;
}

/* Grid-wide barrier over a control block with fields bar (GridBarrier),
 * status and timeout_level.  Thread 0 of every CTA arrives with one atomic
 * on a single counter and waits for the counter's top bit to flip: CTA 0
 * adds 2^31 - (gridDim.x - 1) and every other CTA adds 1, so the barrier's
 * arrivals add exactly 2^31 and the top bit changes only with the last one
 * (the idea of the cooperative-groups grid barrier).  The counter needs no
 * reset and no generation word, and a wait costs one fence, one atomic and
 * the round trip of the poll that sees the flip -- a third of the chain of
 * a counter that the last CTA resets before bumping a generation word.  A
 * fence before the arrival releases the CTA's writes (made CTA-visible by
 * the __syncthreads); the acquiring poll makes every CTA's writes visible
 * after it.  The counter starts at 0 (control blocks are zeroed) and is
 * back at 0 or 2^31 after every complete barrier.  Every wait is bounded
 * by timeout_ns of wall time (globaltimer): on expiry the CTA records
 * TBFS_ERR_TIMEOUT and returns false, and so does every CTA that sees the
 * error word set, so the kernel always terminates (a CTA that left makes
 * the others' next wait expire).  `level` is recorded (+2) in
 * timeout_level. */
template <class Ctl>
__device__ bool grid_barrier(Ctl *ctl, long long timeout_ns, int level) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(&ctl->bar.arrive, inc);
    const unsigned want = (old & 0x80000000u) ^ 0x80000000u;
    if (((old + inc) & 0x80000000u) != want) {
      const unsigned long long t0 = global_ns();
      unsigned spins = 0;
      while ((ld_acquire_u32(&ctl->bar.arrive) & 0x80000000u) != want) {
        if ((++spins & 31u) == 0) {
          if (ld_volatile(&ctl->status) != 0) {
            ok = 0;
            break;
          }
          if ((long long)(global_ns() - t0) > timeout_ns) {
            atomicCAS(&ctl->status, 0, (int)TBFS_ERR_TIMEOUT);
            atomicCAS(&ctl->timeout_level, 0, level + 2);
            ok = 0;
            break;
          }
        }
      }
    } else {
      /* the last arrival: its atomic read every other arrival; the fence
       * orders the CTA's next reads after them */
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

/* Largest i in [0, qn) with e[i] <= target (e nondecreasing, e[0] = 0).
 * 32-ary search: each step narrows the range 32x with one load per lane.
 * Must be called by all 32 lanes with the same arguments. */
__device__ __forceinline__ unsigned warp_find_owner(const int *e, unsigned qn, unsigned target) {
  const int lane = threadIdx.x & 31;
  unsigned lo = 0, hi = qn;
  while (hi - lo > 32) {
    const unsigned step = (hi - lo + 31) / 32;
    const unsigned pidx = lo + lane * step;
    const bool pred = pidx < hi && (unsigned)__ldcg(e + pidx) <= target;
    const unsigned m = __ballot_sync(FULL, pred);
    const unsigned last = 31 - __clz(m);
    lo = lo + last * step;
    const unsigned nhi = lo + step;
    hi = nhi < hi ? nhi : hi;
  }
  const unsigned pidx = lo + lane;
  const bool pred = pidx < hi && (unsigned)__ldcg(e + pidx) <= target;
  const unsigned m = __ballot_sync(FULL, pred);
  return lo + (31 - __clz(m));
}

}  // namespace dev
}  // namespace tbfs

#endif
