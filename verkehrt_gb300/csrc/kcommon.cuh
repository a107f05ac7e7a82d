// Device helpers shared by the kernel families.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vkc_internal.h"

namespace vkc {

constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------------ float order keys
//
// GB300 runs FP64 at about 0.5 T ops/s (a sixteenth of its integer rate), so comparisons,
// extremes and predicates on f64 are done on integer keys. key(x) is the IEEE bits with the
// magnitude bits flipped for negative values: signed comparison of keys is the IEEE order,
// with -0 ranked below +0 (the order of Ordered::less, src/kernels/scalar/reduce.rs:186-197),
// and NaNs outside [key(-inf), key(+inf)].
__device__ __forceinline__ long long f64_key(unsigned long long b) {
    return static_cast<long long>(b ^ (static_cast<unsigned long long>(static_cast<long long>(b) >> 63) >> 1));
}
__host__ __device__ constexpr long long key_of_bits(unsigned long long b) {
    return static_cast<long long>((b >> 63) ? (b ^ 0x7fffffffffffffffull) : b);
}
__host__ __device__ constexpr unsigned long long bits_of_key(long long k) {
    return k < 0 ? (static_cast<unsigned long long>(k) ^ 0x7fffffffffffffffull)
                 : static_cast<unsigned long long>(k);
}
constexpr long long KEY_POS_INF = 0x7ff0000000000000ll;
constexpr long long KEY_NEG_INF = static_cast<long long>(0xfff0000000000000ull ^ 0x7fffffffffffffffull);

// A comparison x <cmp> c against a constant, as a key range [lo, hi] (inclusive) plus a flag
// for the `ne` comparison, which is the complement of an `eq` range and true on NaN. Built on
// the host by cmp_range (k_reduce.cu); the IEEE rules (NaN compares false, -0 == +0) are in
// the range.
struct CmpRange {
    long long lo, hi;
    int negate;
};

__device__ __forceinline__ bool in_range(const CmpRange &r, unsigned long long bits) {
    long long k = f64_key(bits);
    bool in = k >= r.lo && k <= r.hi;
    return in != static_cast<bool>(r.negate);
}

// in_range for a non-empty, non-negated range of non-negative keys (pos_range): there a key is
// the value's bits, and a negative value's bits, read unsigned, lie above every such range, so
// one unsigned comparison decides.
__host__ __device__ __forceinline__ bool pos_range(const CmpRange &r) { return r.lo >= 0 && r.lo <= r.hi && !r.negate; }
__device__ __forceinline__ bool in_pos_range(const CmpRange &r, unsigned long long bits) {
    return bits - static_cast<unsigned long long>(r.lo) <= static_cast<unsigned long long>(r.hi - r.lo);
}
template <bool POS> __device__ __forceinline__ bool in_range_t(const CmpRange &r, unsigned long long bits) {
    return POS ? in_pos_range(r, bits) : in_range(r, bits);
}

// ------------------------------------------------------------------ lookback flags

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Spin budget of every device-side wait: after this many polls (with backoff, on the order
// of a second) the waiter records a timeout in the status word and gives up, so no kernel
// of this library can hang the GPU.
constexpr unsigned SPIN_LIMIT = 1u << 22;

// The poll budget of a wait on another block: the context's test override when set (the low 31
// bits of a status word's spin_limit), else SPIN_LIMIT. Waits for a block's own copies always
// use SPIN_LIMIT. Bit 31 is a second test hook (lookback_never_ready): lookbacks then poll for
// records of an epoch no block writes, so every wait on another tile runs out.
constexpr unsigned NEVER_READY = 1u << 31;
__device__ __forceinline__ unsigned wait_limit(const DevStatus *st) {
    const unsigned v = *reinterpret_cast<const volatile unsigned *>(&st->spin_limit) & ~NEVER_READY;
    return v ? v : SPIN_LIMIT;
}
__device__ __forceinline__ bool never_ready(const DevStatus *st) {
    return (*reinterpret_cast<const volatile unsigned *>(&st->spin_limit) & NEVER_READY) != 0;
}

__device__ __forceinline__ void backoff(unsigned it) {
    if (it > 64) __nanosleep(it > 4096 ? 256 : 32);
}

__device__ __forceinline__ void set_timeout(DevStatus *st) { atomicExch(&st->timeout, 1u); }

// ------------------------------------------------------------------ reductions

template <class T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// Last-block-done: returns true in every thread of the one block that arrives last. The
// counter is reset by that block, so the next launch starts from zero.
__device__ __forceinline__ bool last_block(unsigned *counter) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        last = prev == gridDim.x - 1;
        if (last) *counter = 0;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

}  // namespace vkc
