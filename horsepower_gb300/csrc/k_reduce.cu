// Reductions: @sum, @avg, @min, @max, @len.
//
// Reference (src/horseir/v3/backend/h_primitive.cc):
//   pfnSum :764-786   ints accumulate in i64, f32 in f32, f64 in f64 with an
//                     OpenMP reduction(+) (order depends on the thread count)
//   pfnAvg :788-800   sum / len (ints -> f64)
//   pfnReduce :802-839 serial MIN/MAX fold from x[0]; empty input gives
//                     LLONG_MAX/LLONG_MIN (as i64), FLT_MAX/FLT_MIN, DBL_MAX/DBL_MIN
//
// GB300: every reduction runs the fixed-order tile tree of dev_common.cuh
// (tiles of 4096, 256 lanes x 16 strided elements, xor butterfly, pairwise
// warp combine), recursively over the tile partials until one value is
// left.  Float sums are therefore bit-identical from run to run and equal to
// the oracle's restatement of the same order; they differ from the
// reference's thread-count-dependent order by rounding only (tested at 1e-12
// relative for f64).
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
    default: return run_sum<double, double>(x, (double*)*dres);
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
    case H_F: HG_CHECK(mn ? run_minmax<float, RED_MIN>(x, d, __builtin_huge_valf()) : run_minmax<float, RED_MAX>(x, d, -__builtin_huge_valf())); break;
    default: HG_CHECK(mn ? run_minmax<double, RED_MIN>(x, d, __builtin_huge_val()) : run_minmax<double, RED_MAX>(x, d, -__builtin_huge_val())); break;
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
// sum: code running while a CUDA graph is being captured (cudaMalloc is not
// allowed there), callers with a fixed, pre-reserved memory budget, and
// latency-critical paths that cannot afford the device-wide synchronisation
// an allocation may cause.  hgpuSumF64Static serves them: it computes the same
// fixed-order tile-tree sum as pfnSum on f64 data, but keeps the tile
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
//     cudaGetSymbolAddress (the host-side name is only a stand-in).  Make
//     that first call before any stream capture begins.
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
    double* level1 = level0 + HGPU_STATIC_SUM_MAX_TILES;              // up to 16 partials of those
    long long tiles = (n + TILE_SUM - 1) / TILE_SUM;
    k_tile_reduce<double, double, RED_SUM><<<(unsigned)tiles, 256, 0, s>>>(x, n, tiles == 1 ? result : level0, 0.0);
    long long m = tiles;
    double* cur = level0;
    while (m > 1) {
        long long t2 = (m + TILE_SUM - 1) / TILE_SUM;
        double* nxt = (cur == level0) ? level1 : level0;
        k_tile_reduce<double, double, RED_SUM><<<(unsigned)t2, 256, 0, s>>>(cur, m, t2 == 1 ? result : nxt, 0.0);
        cur = nxt;
        m = t2;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "hgpuSumF64Static launch", __FILE__, __LINE__);
    return 0;
}
