// Device-side helpers shared by the kernels.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>
#include "hgpu_internal.cuh"

namespace hg {

constexpr double H_EPSILON = 1e-13;  // src/horseir/v3/backend/h_system.cc:9

__device__ __forceinline__ void flag_error(unsigned* derr, unsigned bit) { atomicOr(derr, bit); }

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- acquire/release accesses for decoupled look-back status words
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---- warp reductions / scans
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned warp_incl_scan(unsigned v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= (unsigned)o) v += t;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= (unsigned)o) v += t;
    }
    return v;
}

// ---- decoupled look-back (Merrill & Garland, "Single-pass Parallel Prefix
// Scan with Decoupled Look-back", 2016).  Status word per tile:
//   bits 63..62 = 0 not ready, 1 aggregate ready, 2 inclusive prefix ready
//   bits 61..0  = value.
// Tiles are numbered in launch order by an atomic ticket so every
// predecessor has started; waits are bounded by SPIN_LIMIT.
constexpr unsigned long long LB_AGG = 1ull << 62, LB_INC = 2ull << 62, LB_MASK = (1ull << 62) - 1;

// Called by one full warp (warp 0) of the tile.  Publishes `agg` and returns
// the exclusive prefix of tile `t` (valid in all lanes).
__device__ __forceinline__ unsigned long long lookback_exclusive(unsigned long long* status, long long t,
                                                                 unsigned long long agg, unsigned* derr,
                                                                 long long limit = SPIN_LIMIT) {
    const unsigned lane = lane_id();
    if (t == 0) {
        if (lane == 0) st_release(&status[0], LB_INC | agg);
        return 0;
    }
    if (lane == 0) st_release(&status[t], LB_AGG | agg);
    unsigned long long excl = 0;
    long long base = t - 1;  // look at tiles base, base-1, ..., base-31 in one round
    long long spins = 0;
    for (;;) {
        long long j = base - (long long)lane;
        unsigned long long s = (j >= 0) ? ld_acquire(&status[j]) : LB_INC;  // before tile 0: prefix 0
        unsigned flag = (unsigned)(s >> 62);
        // lowest lane holding an inclusive prefix closes the window
        unsigned inc = __ballot_sync(0xffffffffu, flag == 2);
        unsigned notready = __ballot_sync(0xffffffffu, flag == 0);
        int stop = inc ? __ffs(inc) - 1 : 31;
        unsigned upto = stop == 31 ? 0xffffffffu : ((1u << (stop + 1)) - 1u);
        if (notready & upto) {
            if (++spins > limit) {
                if (lane == 0) flag_error(derr, DERR_TIMEOUT);
                break;
            }
            continue;  // a predecessor has not published yet: reread the window
        }
        unsigned long long v = ((int)lane <= stop) ? (s & LB_MASK) : 0;
        excl += warp_sum(v);
        if (inc) break;
        base -= 32;
    }
    if (lane == 0) st_release(&status[t], LB_INC | (excl + agg));
    return excl;
}

// lookback_exclusive restricted to the tiles [first, t) (a segmented scan
// restarts at `first`)
__device__ __forceinline__ unsigned long long lookback_seg(unsigned long long* status, long long t, long long first,
                                                           unsigned long long agg, unsigned* derr) {
    const unsigned lane = lane_id();
    if (t == first) {
        if (lane == 0) st_release(&status[t], LB_INC | agg);
        return 0;
    }
    if (lane == 0) st_release(&status[t], LB_AGG | agg);
    unsigned long long excl = 0;
    long long base = t - 1, spins = 0;
    for (;;) {
        long long j = base - (long long)lane;
        unsigned long long s = (j >= first) ? ld_acquire(&status[j]) : LB_INC;
        unsigned flag = (unsigned)(s >> 62);
        unsigned inc = __ballot_sync(0xffffffffu, flag == 2);
        unsigned notready = __ballot_sync(0xffffffffu, flag == 0);
        int stop = inc ? __ffs(inc) - 1 : 31;
        unsigned upto = stop == 31 ? 0xffffffffu : ((1u << (stop + 1)) - 1u);
        if (notready & upto) {
            if (++spins > SPIN_LIMIT) {
                if (lane == 0) flag_error(derr, DERR_TIMEOUT);
                break;
            }
            continue;
        }
        unsigned long long v = ((int)lane <= stop && j >= first) ? (s & LB_MASK) : 0;
        excl += warp_sum(v);
        if (inc) break;
        base -= 32;
    }
    if (lane == 0) st_release(&status[t], LB_INC | (excl + agg));
    return excl;
}

// Look-back along one chain of status words (status[j * stride] for tiles j
// in [first, t)), one thread per chain: the per-digit prefixes of the radix
// passes.
__device__ __forceinline__ unsigned long long chain_lookback(unsigned long long* status, size_t stride, long long t,
                                                             long long first, unsigned long long c, unsigned* derr,
                                                             long long limit = SPIN_LIMIT) {
    unsigned long long* st = status + (size_t)t * stride;
    if (t == first) {
        st_release(st, LB_INC | c);
        return 0;
    }
    st_release(st, LB_AGG | c);
    unsigned long long excl = 0;
    long long j = t - 1, spins = 0;
    while (j >= first) {
        unsigned long long sv = ld_acquire(status + (size_t)j * stride);
        unsigned long long f = sv >> 62;
        if (f == 0) {
            if (++spins > limit) { flag_error(derr, DERR_TIMEOUT); break; }
            continue;
        }
        excl += sv & LB_MASK;
        if (f == 2) break;
        j--;
    }
    st_release(st, LB_INC | (excl + c));
    return excl;
}

// ---- compareFloat (h_primitive.cc:1061) against a fixed double s without
// FP64 arithmetic.  With s fixed, compareFloat(v, s) is a non-decreasing step
// function of v (-1, then 0, then 1) and compareFloat(s, v) a non-increasing
// one, so both reduce to two thresholds on an integer image of v that keeps
// the IEEE order: c = ord(v) < ta ? ca : (ord(v) < tb ? cb : cc).  The host
// finds the thresholds by bisection, evaluating compareFloat itself in
// double arithmetic; NaN compares as 1 either way round.
struct F64Cmp {
    long long ta, tb;
    int ca, cb, cc;
};
__host__ __device__ __forceinline__ long long f64_ord(unsigned long long b) {
    return (b >> 63) ? -(long long)(b & 0x7fffffffffffffffull) : (long long)b;  // -0.0 and +0.0 both map to 0
}
__host__ __device__ __forceinline__ bool f64_nan_bits(unsigned long long b) {
    return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ int f64_cmp_fixed(double v, const F64Cmp& t) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if (f64_nan_bits(b)) return 1;
    const long long o = f64_ord(b);
    return o < t.ta ? t.ca : (o < t.tb ? t.cb : t.cc);
}
F64Cmp f64_cmp_thresholds(double s, bool scalar_first);  // host (k_elementwise.cu)

// ---- fixed-order deterministic tile sum (used by @sum/@avg and every
// segmented sum).  A chunk of up to TILE_SUM = 4096 elements is summed as:
//   lane t (0..255) accumulates e[t], e[t+256], ..., e[t+3840] in order
//   (missing elements contribute +0.0), then each 32-lane warp folds with a
//   xor butterfly (offsets 16,8,4,2,1), then the 8 warp sums combine as
//   ((w0+w1)+(w2+w3))+((w4+w5)+(w6+w7)).
// A vector (or segment) longer than one chunk is reduced chunk by chunk and
// the chunk partials are reduced again by the same procedure, until one
// value is left.  The accumulator starts at +0.0 and can never become -0.0,
// so the +0.0 of a missing element is an exact no-op: kernels may skip
// missing elements, lanes and warps.  The oracle restates exactly this
// order, so results are bit-exact.
constexpr int TILE_SUM = 4096;

template <typename T>
__device__ __forceinline__ T combine8(const T* w) {
    return ((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7]));
}

}  // namespace hg
