// Reductions: @sum, @avg, @min, @max, @len.
//
// Reference (src/horseir/v3/backend/h_primitive.cc):
//   pfnSum :764-786   ints accumulate in i64, f32 in f32, f64 in f64 with an
//                     OpenMP reduction(+) (order depends on the thread count)
//   pfnAvg :788-800   sum / len (ints -> f64)
//   pfnReduce :802-839 serial MIN/MAX fold from x[0]; empty input gives
//                     LLONG_MAX/LLONG_MIN (as i64), FLT_MAX/FLT_MIN, DBL_MAX/DBL_MIN
//
// GB300: reductions work on 4096-element tiles, then on the tile partials,
// until one value is left.  f64 sums add in 128-bit fixed point on the
// integer pipe (GB300's FP64 rate would bound a DADD sum below HBM speed);
// f32 and integer sums and integer min/max run the fixed-order tile tree of
// dev_common.cuh; f64/f32 min/max reproduce the reference's serial fold,
// NaN and signed zeros included, on integer keys.  Float sums are
// bit-identical from run to run and equal to the oracle's restatements; they
// differ from the reference's thread-count-dependent order by rounding only
// (tested at 1e-12 relative for f64).
#include <cfloat>
#include <climits>

#include "dev_common.cuh"

namespace hg {

enum { RED_SUM = 0, RED_MIN = 1, RED_MAX = 2 };

template <typename A, int OP>
__device__ __forceinline__ A red_op(A a, A b) {
    if constexpr (OP == RED_SUM) {
        if constexpr (std::is_same<A, double>::value) return __dadd_rn(a, b);
        else if constexpr (std::is_same<A, float>::value) return __fadd_rn(a, b);
        else if constexpr (std::is_same<A, long long>::value) return (long long)((unsigned long long)a + (unsigned long long)b);
        else return a + b;
    } else if constexpr (OP == RED_MIN) {
        return (a < b) ? a : b;
    } else {
        return (a > b) ? a : b;
    }
}

template <typename A, int OP>
__device__ __forceinline__ A warp_red(A v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = red_op<A, OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block = 256 threads, one 4096-element tile per block.
template <typename T, typename A, int OP>
__global__ void __launch_bounds__(256) k_tile_reduce(const T* __restrict__ x, long long n, A* __restrict__ out, A ident) {
    __shared__ A ws[8];
    const long long base = (long long)blockIdx.x * TILE_SUM;
    A acc = ident;
    T v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        long long i = base + k * 256 + threadIdx.x;
        v[k] = i < n ? x[i] : T(0);
    }
#pragma unroll
    for (int k = 0; k < 16; k++) {
        long long i = base + k * 256 + threadIdx.x;
        acc = red_op<A, OP>(acc, i < n ? (A)v[k] : ident);
    }
    acc = warp_red<A, OP>(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        A w01 = red_op<A, OP>(ws[0], ws[1]), w23 = red_op<A, OP>(ws[2], ws[3]);
        A w45 = red_op<A, OP>(ws[4], ws[5]), w67 = red_op<A, OP>(ws[6], ws[7]);
        out[blockIdx.x] = red_op<A, OP>(red_op<A, OP>(w01, w23), red_op<A, OP>(w45, w67));
    }
}

// ---- f64 @sum / @avg on the integer pipe.
// GB300 runs FP64 arithmetic at a small fraction of its integer rate, so a
// sum that adds with DADD is bound by the FP64 units, not by HBM.  Each tile
// of 4096 elements is instead summed exactly in a 128-bit fixed-point
// accumulator and rounded once:
//   E    the largest biased exponent among the tile's finite elements (>= 1),
//   F    min(62, E - 1); one unit is 2^(E - 1075 - F),
//   an element m * 2^(e - 1075) (m the 53-bit significand; a subnormal has
//        e = 1 and no implicit bit) is m * 2^(e - E + F) units, truncated
//        toward zero when e - E + F < 0 (only elements more than 2^62 times
//        below the tile's largest binade lose bits),
//   the total (|total| < 4096 * 2^115 < 2^127) is rounded to nearest-even.
// A NaN in the tile, or +inf with -inf, gives the quiet NaN 0x7ff8...; an
// infinity otherwise gives itself.  Longer vectors sum their tile partials
// the same way until one value is left.  Within a tile the result does not
// depend on the order of the elements; the oracle restates it bit for bit.
struct Fx128 {
    unsigned long long lo, hi;
};

__device__ __forceinline__ void fx_add(Fx128& a, unsigned long long lo, unsigned long long hi) {
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(a.lo), "+l"(a.hi) : "l"(lo), "l"(hi));
}

// The element with bits b in units of 2^(E - 1075 - F), signed, added to a.
__device__ __forceinline__ void fx_accumulate(Fx128& a, unsigned long long b, int E, int F) {
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = (b & 0xfffffffffffffull) | ((unsigned long long)(e != 0) << 52);
    const int k = F - E + (e > 1 ? e : 1);
    unsigned long long lo, hi;
    if (k >= 0) {
        lo = m << k;
        hi = k ? m >> (64 - k) : 0ull;
    } else {
        lo = k > -64 ? m >> (-k) : 0ull;
        hi = 0;
    }
    const unsigned long long s = (unsigned long long)((long long)b >> 63);  // all ones when negative
    fx_add(a, lo ^ s, hi ^ s);
    fx_add(a, s & 1ull, 0ull);
}

// Round a (signed, |a| < 2^127) times 2^sexp to the nearest double (ties to
// even).  sexp >= -1074, so a result below 2^-1022 is exact.
__device__ __forceinline__ unsigned long long fx_round(Fx128 a, int sexp) {
    const unsigned long long sign = a.hi >> 63;
    unsigned long long lo = a.lo, hi = a.hi;
    if (sign) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0 ? 1ull : 0ull);
    }
    if (!hi && !lo) return 0ull;
    const int p = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    int biased = p + sexp + 1023;
    if (biased <= 0) return (sign << 63) | (lo << (sexp + 1074));  // subnormal: p <= 51, exact
    const int sh = p - 52;
    unsigned long long M;
    bool up;
    if (sh <= 0) {
        M = lo << (-sh);
        up = false;
    } else if (sh < 64) {
        M = (lo >> sh) | (hi << (64 - sh));
        const unsigned long long rem = lo & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        up = rem > half || (rem == half && (M & 1ull));
    } else {
        const int r = sh - 64;
        M = hi >> r;
        if (r == 0) {
            up = lo > (1ull << 63) || (lo == (1ull << 63) && (M & 1ull));
        } else {
            const unsigned long long remhi = hi & ((1ull << r) - 1ull), halfhi = 1ull << (r - 1);
            up = remhi > halfhi || (remhi == halfhi && (lo != 0 || (M & 1ull)));
        }
    }
    if (up && ++M == (1ull << 53)) {
        M >>= 1;
        biased++;
    }
    if (biased >= 2047) return (sign << 63) | 0x7ff0000000000000ull;
    return (sign << 63) | ((unsigned long long)biased << 52) | (M & 0xfffffffffffffull);
}

// Block = 256 threads, one 4096-element tile per block.
__global__ void __launch_bounds__(256) k_tile_sum_fx(const unsigned long long* __restrict__ x, long long n,
                                                     double* __restrict__ out) {
    __shared__ unsigned s_e[8], s_f[8];
    __shared__ Fx128 s_acc[8];
    const long long base = (long long)blockIdx.x * TILE_SUM;
    unsigned long long v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const long long i = base + k * 256 + threadIdx.x;
        v[k] = i < n ? x[i] : 0ull;
    }
    unsigned emax = 1, flags = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const unsigned e = (unsigned)(v[k] >> 52) & 0x7ffu;
        if (e == 0x7ffu) flags |= (v[k] & 0xfffffffffffffull) ? 1u : ((v[k] >> 63) ? 4u : 2u);
        else emax = max(emax, e);
    }
    const unsigned w = threadIdx.x >> 5;
    emax = __reduce_max_sync(0xffffffffu, emax);
    flags = __reduce_or_sync(0xffffffffu, flags);
    if (lane_id() == 0) {
        s_e[w] = emax;
        s_f[w] = flags;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 8; j++) {
        emax = max(emax, s_e[j]);
        flags |= s_f[j];
    }
    if (flags) {  // NaN / infinity: uniform over the block
        if (threadIdx.x == 0) {
            const unsigned long long r = ((flags & 1u) || (flags & 6u) == 6u) ? 0x7ff8000000000000ull
                                         : (flags & 2u)                       ? 0x7ff0000000000000ull
                                                                              : 0xfff0000000000000ull;
            out[blockIdx.x] = __longlong_as_double((long long)r);
        }
        return;
    }
    const int E = (int)emax, F = min(62, E - 1);
    Fx128 acc = {0ull, 0ull};
#pragma unroll
    for (int k = 0; k < 16; k++) fx_accumulate(acc, v[k], E, F);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, acc.lo, o);
        const unsigned long long h2 = __shfl_xor_sync(0xffffffffu, acc.hi, o);
        fx_add(acc, l2, h2);
    }
    if (lane_id() == 0) s_acc[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        Fx128 t = s_acc[0];
#pragma unroll
        for (int j = 1; j < 8; j++) fx_add(t, s_acc[j].lo, s_acc[j].hi);
        out[blockIdx.x] = __longlong_as_double((long long)fx_round(t, E - 1075 - F));
    }
}

// f64 sum of n >= 1 elements at x into *result by fixed-point tiles, level
// after level.  With `fixed` null the levels come from the scratch arena and
// launches go through HG_LAUNCH on the library stream; otherwise `fixed`
// holds two level buffers (fixed[0] >= ceil(n/4096) doubles, fixed[1] >=
// ceil(n/4096^2)) and the kernels go on stream s untracked.
static void fx_launch(unsigned grid, const void* in, long long n, double* out, cudaStream_t s, bool tracked) {
    if (tracked) HG_LAUNCH("tile_sum_fx", grid, 256, 0, k_tile_sum_fx, (const unsigned long long*)in, n, out);
    else k_tile_sum_fx<<<grid, 256, 0, s>>>((const unsigned long long*)in, n, out);
}

static I fx_sum_f64(const double* x, long long n, double* result, cudaStream_t s, double* const* fixed) {
    const bool tracked = fixed == nullptr;
    long long tiles = (n + TILE_SUM - 1) / TILE_SUM;
    double* part = tracked ? (double*)salloc((size_t)tiles * sizeof(double)) : fixed[0];
    if (!part) return E_DEVICE_OOM;
    fx_launch((unsigned)tiles, x, n, tiles == 1 ? result : part, s, tracked);
    HG_CHECK(last_launch_error());
    long long m = tiles;
    double* cur = part;
    while (m > 1) {
        long long t2 = (m + TILE_SUM - 1) / TILE_SUM;
        double* nxt = tracked ? (double*)salloc((size_t)t2 * sizeof(double)) : (cur == fixed[0] ? fixed[1] : fixed[0]);
        if (!nxt) return E_DEVICE_OOM;
        fx_launch((unsigned)t2, cur, m, t2 == 1 ? result : nxt, s, tracked);
        HG_CHECK(last_launch_error());
        cur = nxt;
        m = t2;
    }
    return 0;
}

// ---- f64 / f32 @min / @max: the reference's serial fold
//   t = x[0]; for each v: t = (t > v) ? t : v      (min: t < v)
// without FP64 compares.  A NaN never wins a compare, so the fold restarts
// after the last NaN: the result is x[n-1] when that is NaN, else the
// maximum of the elements after the last NaN, equal values (+0.0 and -0.0)
// going to the later one.  Each tile (and each block of tile summaries)
// finds its last NaN position J first, then the largest (key, position)
// among its elements after J, the key being an integer image of the value
// that keeps the IEEE order with -0.0 == +0.0.  A summary is (J, key,
// position); combining summaries in any grouping keeps this meaning, and the
// last step reads the answer's bits from x.
template <typename T>
__device__ __forceinline__ long long fkey(T v) {
    if constexpr (sizeof(T) == 8) return f64_ord((unsigned long long)__double_as_longlong(v));
    else {
        const unsigned b = __float_as_uint(v);
        return (b >> 31) ? -(long long)(b & 0x7fffffffu) : (long long)b;
    }
}
template <typename T>
__device__ __forceinline__ bool fnan(T v) {
    if constexpr (sizeof(T) == 8) return f64_nan_bits((unsigned long long)__double_as_longlong(v));
    else return (__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u;
}

// Is (k2, p2) the better candidate than (k1, p1)?  p < 0 marks "none".
template <int OP>
__device__ __forceinline__ bool mm_better(long long k2, long long p2, long long k1, long long p1) {
    if (p2 < 0) return false;
    if (p1 < 0) return true;
    if (k2 != k1) return OP == RED_MAX ? k2 > k1 : k2 < k1;
    return p2 > p1;
}

template <int OP>
__device__ __forceinline__ void mm_block_finish(long long J, long long bk, long long bp, long long* onan, long long* okey,
                                                long long* opos) {
    __shared__ long long s_k[8], s_p[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long k2 = __shfl_xor_sync(0xffffffffu, bk, o), p2 = __shfl_xor_sync(0xffffffffu, bp, o);
        if (mm_better<OP>(k2, p2, bk, bp)) {
            bk = k2;
            bp = p2;
        }
    }
    if (lane_id() == 0) {
        s_k[threadIdx.x >> 5] = bk;
        s_p[threadIdx.x >> 5] = bp;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        bk = s_k[0];
        bp = s_p[0];
        for (int j = 1; j < 8; j++)
            if (mm_better<OP>(s_k[j], s_p[j], bk, bp)) {
                bk = s_k[j];
                bp = s_p[j];
            }
        onan[blockIdx.x] = J;
        okey[blockIdx.x] = bk;
        opos[blockIdx.x] = bp;
    }
}

__device__ __forceinline__ long long block_max_i64(long long v) {
    __shared__ long long s_m[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, (long long)__shfl_xor_sync(0xffffffffu, v, o));
    if (lane_id() == 0) s_m[threadIdx.x >> 5] = v;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 8; j++) v = max(v, s_m[j]);
    return v;
}

// Tile summaries of x: one 4096-element tile per 256-thread block.
template <typename T, int OP>
__global__ void __launch_bounds__(256) k_tile_minmax_f(const T* __restrict__ x, long long n, long long* __restrict__ onan,
                                                       long long* __restrict__ okey, long long* __restrict__ opos) {
    const long long base = (long long)blockIdx.x * TILE_SUM;
    const int lim = (int)min((long long)TILE_SUM, n - base);
    T v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int off = k * 256 + (int)threadIdx.x;
        v[k] = off < lim ? x[base + off] : T(0);
    }
    int lastnan = -1;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int off = k * 256 + (int)threadIdx.x;
        if (off < lim && fnan(v[k])) lastnan = off;
    }
    lastnan = __reduce_max_sync(0xffffffffu, lastnan);
    const long long J = block_max_i64(lastnan);
    long long bk = 0, bp = -1;
    if (J < 0 && lim == TILE_SUM) {
        // a full tile without NaN (the common case): the best key in 32-bit
        // halves, first the signed high words, then among the elements that
        // share the best high word the low words, the later element winning
        // ties as in the fold below
        int hi[16];
        unsigned lo[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const long long key = fkey(v[k]);
            hi[k] = (int)(key >> 32);
            lo[k] = (unsigned)key;
        }
        int hb = hi[0];
#pragma unroll
        for (int k = 1; k < 16; k++) hb = OP == RED_MAX ? max(hb, hi[k]) : min(hb, hi[k]);
        unsigned lb = 0;
        int kb = -1;
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (hi[k] == hb && (kb < 0 || (OP == RED_MAX ? lo[k] >= lb : lo[k] <= lb))) {
                lb = lo[k];
                kb = k;
            }
        bk = (long long)(((unsigned long long)(unsigned)hb << 32) | lb);
        bp = kb * 256 + (int)threadIdx.x;
    } else {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const int off = k * 256 + (int)threadIdx.x;
            if (off < lim && off > J) {
                const long long key = fkey(v[k]);
                if (bp < 0 || (OP == RED_MAX ? key >= bk : key <= bk)) {
                    bk = key;
                    bp = off;
                }
            }
        }
    }
    mm_block_finish<OP>(J >= 0 ? base + J : -1, bk, bp >= 0 ? base + bp : -1, onan, okey, opos);
}

// Summaries of m consecutive summaries, 4096 per block.
template <int OP>
__global__ void __launch_bounds__(256) k_minmax_combine(const long long* __restrict__ inan, const long long* __restrict__ ikey,
                                                        const long long* __restrict__ ipos, long long m,
                                                        long long* __restrict__ onan, long long* __restrict__ okey,
                                                        long long* __restrict__ opos) {
    const long long base = (long long)blockIdx.x * TILE_SUM;
    long long J = -1;
    for (int k = 0; k < 16; k++) {
        const long long i = base + k * 256 + threadIdx.x;
        if (i < m) J = max(J, inan[i]);
    }
    J = block_max_i64(J);
    long long bk = 0, bp = -1;
    for (int k = 0; k < 16; k++) {
        const long long i = base + k * 256 + threadIdx.x;
        if (i < m && ipos[i] > J && mm_better<OP>(ikey[i], ipos[i], bk, bp)) {
            bk = ikey[i];
            bp = ipos[i];
        }
    }
    mm_block_finish<OP>(J, bk, bp, onan, okey, opos);
}

template <typename T>
__global__ void k_minmax_pick(const T* __restrict__ x, const long long* nan, const long long* pos, T* out) {
    *out = x[*pos >= 0 ? *pos : *nan];
}

template <typename T, int OP>
static I run_minmax_float(V x, void* dres) {
    const void* p;
    HG_CHECK(in_ptr(x, &p));
    const long long n = x->len;
    long long m = (n + TILE_SUM - 1) / TILE_SUM;
    long long* a = (long long*)salloc((size_t)m * 3 * sizeof(long long));
    if (!a) return E_DEVICE_OOM;
    HG_LAUNCH("tile_minmax", (unsigned)m, 256, 0, (k_tile_minmax_f<T, OP>), (const T*)p, n, a, a + m, a + 2 * m);
    HG_CHECK(last_launch_error());
    while (m > 1) {
        const long long m2 = (m + TILE_SUM - 1) / TILE_SUM;
        long long* b = (long long*)salloc((size_t)m2 * 3 * sizeof(long long));
        if (!b) return E_DEVICE_OOM;
        HG_LAUNCH("tile_minmax", (unsigned)m2, 256, 0, k_minmax_combine<OP>, a, a + m, a + 2 * m, m, b, b + m2, b + 2 * m2);
        HG_CHECK(last_launch_error());
        a = b;
        m = m2;
    }
    HG_LAUNCH("minmax_pick", 1, 1, 0, k_minmax_pick<T>, (const T*)p, a, a + 2, (T*)dres);
    return last_launch_error();
}

// Reduces n elements of x to one value at *result (device); levels of tile
// partials live in scratch.
template <typename T, typename A, int OP>
static I tree_reduce(const T* x, long long n, A ident, A* result) {
    long long tiles = (n + TILE_SUM - 1) / TILE_SUM;
    A* part = (A*)salloc((size_t)(tiles > 0 ? tiles : 1) * sizeof(A));
    if (!part) return E_DEVICE_OOM;
    HG_LAUNCH("tile_reduce", (unsigned)tiles, 256, 0, (k_tile_reduce<T, A, OP>), x, n, tiles == 1 ? result : part, ident);
    HG_CHECK(last_launch_error());
    long long m = tiles;
    A* cur = part;
    while (m > 1) {
        long long t2 = (m + TILE_SUM - 1) / TILE_SUM;
        A* nxt = (A*)salloc((size_t)t2 * sizeof(A));
        if (!nxt) return E_DEVICE_OOM;
        HG_LAUNCH("tile_reduce", (unsigned)t2, 256, 0, (k_tile_reduce<A, A, OP>), cur, m, t2 == 1 ? result : nxt, ident);
        HG_CHECK(last_launch_error());
        cur = nxt;
        m = t2;
    }
    return 0;
}

// avg = sum / len (pfnAvg, h_primitive.cc:792-797)
template <typename A>
__global__ void k_avg_final(const A* s, long long n, void* out) {
    if constexpr (std::is_same<A, long long>::value) *(double*)out = __ddiv_rn((double)*s * 1.0, (double)n);
    else if constexpr (std::is_same<A, float>::value) *(float*)out = __fdiv_rn(*s, (float)n);
    else *(double*)out = __ddiv_rn(*s, (double)n);
}

template <typename T, typename A>
static I run_sum(V x, A* dres) {
    const void* p;
    HG_CHECK(in_ptr(x, &p));
    if (x->len == 0) {
        HG_CU(cudaMemsetAsync(dres, 0, sizeof(A), g_stream));
        return 0;
    }
    return tree_reduce<T, A, RED_SUM>((const T*)p, x->len, (A)0, dres);
}

static I sum_into(V x, I* typZ, void** dres) {
    *typZ = x->typ == H_F ? H_F : x->typ == H_E ? H_E : H_L;
    *dres = salloc(16);
    if (!*dres) return E_DEVICE_OOM;
    switch (x->typ) {
    case H_B: return run_sum<bool, long long>(x, (long long*)*dres);
    case H_J: return run_sum<int8_t, long long>(x, (long long*)*dres);
    case H_H: return run_sum<int16_t, long long>(x, (long long*)*dres);
    case H_I: return run_sum<int32_t, long long>(x, (long long*)*dres);
    case H_L: return run_sum<long long, long long>(x, (long long*)*dres);
    case H_F: return run_sum<float, float>(x, (float*)*dres);
    default: {
        const void* p;
        HG_CHECK(in_ptr(x, &p));
        if (x->len == 0) {
            HG_CU(cudaMemsetAsync(*dres, 0, sizeof(double), g_stream));
            return 0;
        }
        return fx_sum_f64((const double*)p, x->len, (double*)*dres, g_stream, nullptr);
    }
    }
}

template <typename T, int OP>
static I run_minmax(V x, void* dres, T ident) {
    const void* p;
    HG_CHECK(in_ptr(x, &p));
    return tree_reduce<T, T, OP>((const T*)p, x->len, ident, (T*)dres);
}

// Reduction of n accumulator values (type typ; op 0 sum, 1 min, 2 max) to
// one value at result, by the same fixed-order tile tree.
I tree_reduce_any(int typ, int op, const void* part, long long n, void* result) {
#define TRA(T, ID0, IDMIN, IDMAX)                                                                  \
    if (op == 0) return tree_reduce<T, T, RED_SUM>((const T*)part, n, (T)(ID0), (T*)result);     \
    if (op == 1) return tree_reduce<T, T, RED_MIN>((const T*)part, n, (T)(IDMIN), (T*)result);   \
    return tree_reduce<T, T, RED_MAX>((const T*)part, n, (T)(IDMAX), (T*)result);
    switch (typ) {
    case H_E: { TRA(double, 0.0, __builtin_huge_val(), -__builtin_huge_val()) }
    case H_F: { TRA(float, 0.0f, __builtin_huge_valf(), -__builtin_huge_valf()) }
    case H_L: { TRA(long long, 0, LLONG_MAX, LLONG_MIN) }
    case H_I: { TRA(int32_t, 0, INT32_MAX, INT32_MIN) }
    case H_H: { TRA(int16_t, 0, INT16_MAX, INT16_MIN) }
    case H_J: { TRA(int8_t, 0, INT8_MAX, INT8_MIN) }
    default: { TRA(bool, 0, true, false) }
    }
#undef TRA
}

}  // namespace hg

using namespace hg;

extern "C" {

I pfnSum(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!is_real(x->typ)) return E_DOMAIN;
    I typZ;
    void* d;
    HG_CHECK(sum_into(x, &typZ, &d));
    z->typ = typZ;
    z->len = 1;
    return finish_out(z, d);
}

I pfnAvg(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!is_real(x->typ)) return E_DOMAIN;
    I typS;
    void* s;
    HG_CHECK(sum_into(x, &typS, &s));
    void* d = salloc(16);
    if (!d) return E_DEVICE_OOM;
    long long n = x->len;
    switch (typS) {
    case H_L: HG_LAUNCH("avg", 1, 1, 0, k_avg_final<long long>, (const long long*)s, n, d); break;
    case H_F: HG_LAUNCH("avg", 1, 1, 0, k_avg_final<float>, (const float*)s, n, d); break;
    default: HG_LAUNCH("avg", 1, 1, 0, k_avg_final<double>, (const double*)s, n, d); break;
    }
    HG_CHECK(last_launch_error());
    z->typ = typS == H_F ? H_F : H_E;
    z->len = 1;
    return finish_out(z, d);
}

I pfnReduce(V z, V x, I op) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!is_real(x->typ)) return E_DOMAIN;
    if (x->len < 1) {  // sentinels of h_primitive.cc:803-806,810-819
        I typZ = is_int(x->typ) ? H_L : x->typ;
        z->typ = typZ;
        z->len = 1;
        z->g = (G)&z->b;
        switch (typZ) {
        case H_L: z->i64 = 0 == op ? LLONG_MAX : LLONG_MIN; break;
        case H_F: z->f32 = 0 == op ? FLT_MAX : FLT_MIN; break;
        default: z->f64 = 0 == op ? DBL_MAX : DBL_MIN; break;
        }
        return apply_residency(z);
    }
    void* d = salloc(16);
    if (!d) return E_DEVICE_OOM;
    bool mn = op == 0;
    switch (x->typ) {
    case H_B: HG_CHECK(mn ? run_minmax<bool, RED_MIN>(x, d, true) : run_minmax<bool, RED_MAX>(x, d, false)); break;
    case H_J: HG_CHECK(mn ? run_minmax<int8_t, RED_MIN>(x, d, INT8_MAX) : run_minmax<int8_t, RED_MAX>(x, d, INT8_MIN)); break;
    case H_H: HG_CHECK(mn ? run_minmax<int16_t, RED_MIN>(x, d, INT16_MAX) : run_minmax<int16_t, RED_MAX>(x, d, INT16_MIN)); break;
    case H_I: HG_CHECK(mn ? run_minmax<int32_t, RED_MIN>(x, d, INT32_MAX) : run_minmax<int32_t, RED_MAX>(x, d, INT32_MIN)); break;
    case H_L: HG_CHECK(mn ? run_minmax<long long, RED_MIN>(x, d, LLONG_MAX) : run_minmax<long long, RED_MAX>(x, d, LLONG_MIN)); break;
    case H_F: HG_CHECK(mn ? run_minmax_float<float, RED_MIN>(x, d) : run_minmax_float<float, RED_MAX>(x, d)); break;
    default: HG_CHECK(mn ? run_minmax_float<double, RED_MIN>(x, d) : run_minmax_float<double, RED_MAX>(x, d)); break;
    }
    z->typ = x->typ;
    z->len = 1;
    return finish_out(z, d);
}
I pfnMin(V z, V x) { return pfnReduce(z, x, 0); }
I pfnMax(V z, V x) { return pfnReduce(z, x, 1); }

// pfnLen: h_primitive.cc:656-662 (metadata only)
I pfnLen(V z, V x) {
    L n = x->len;
    z->typ = H_L;
    z->len = 1;
    z->g = (G)&z->b;
    z->i64 = n;
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free f64 sum.
//
// Some callers cannot allocate device memory at the point where they need a
// sum: a query engine that reserved a fixed device-memory budget up front and
// must not grow it, and latency-critical paths that cannot afford the
// device-wide synchronisation an allocation (or an arena's first chunk) may
// cause.  hgpuSumF64Static serves them: it computes the same
// fixed-point tile sum as pfnSum on f64 data, but keeps the tile
// partials in the file-scope array below instead of the scratch arena, and
// touches no arena, no cudaMalloc/cudaFree and no allocating library call.
//
// Limits and sharing:
//   * n <= HGPU_STATIC_SUM_MAX_ROWS (65,536 tiles of 4,096 = 268,435,456);
//     larger n is rejected with E_LENGTH.
//   * The array (about 512 KiB) is held by every GPU that loads the library
//     until the process exits.
//   * Every call shares the array.  Each call overwrites every partial it
//     reads, so nothing needs clearing, but calls whose kernels overlap on the
//     GPU (different streams, or different host threads) race on it: issue
//     them on one stream or serialise them.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (the host-side name is only a stand-in).  The
//     address is kept for the life of the process: after cudaDeviceReset on
//     that device it would be stale, so a device reset is not supported (the library's
//     arenas and stream do not survive one either).
// ---------------------------------------------------------------------------
#define HGPU_STATIC_SUM_MAX_TILES 65536LL
#define HGPU_STATIC_SUM_MAX_ROWS (HGPU_STATIC_SUM_MAX_TILES * 4096LL)
static __device__ __align__(256) double g_static_sum_partials[HGPU_STATIC_SUM_MAX_TILES + 64];

namespace hg {
static void* g_static_sum_ptr[64];  // device address of the array, per device
}

extern "C" I hgpuSumF64Static(const double* x, L n, double* result, void* stream) {
    using namespace hg;
    if (n < 0 || n > HGPU_STATIC_SUM_MAX_ROWS)
        return set_error(E_LENGTH, "hgpuSumF64Static: n = %lld is outside [0, %lld]", n, HGPU_STATIC_SUM_MAX_ROWS);
    int dev = 0;
    HG_CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(E_DEVICE, "hgpuSumF64Static: device %d out of range", dev);
    if (!g_static_sum_ptr[dev]) HG_CU(cudaGetSymbolAddress(&g_static_sum_ptr[dev], g_static_sum_partials));
    cudaStream_t s = (cudaStream_t)stream;
    if (n == 0) {
        HG_CU(cudaMemsetAsync(result, 0, sizeof(double), s));
        return 0;
    }
    double* level0 = (double*)g_static_sum_ptr[dev];                  // up to 65,536 tile partials
    double* const levels[2] = {level0, level0 + HGPU_STATIC_SUM_MAX_TILES};  // then up to 16 partials of those
    return fx_sum_f64(x, n, result, s, levels);  // checks each launch
}
