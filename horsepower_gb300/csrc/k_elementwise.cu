// Elementwise builtins: compare, arithmetic, logic, not.
//
// Semantics (src/horseir/v3/backend/h_primitive.cc):
//   pfnCompare :1073-1170  operands promoted to MAX(type codes); f32/f64 use
//                          compareFloat (:1061) with absolute eps 1e-13, so
//                          NaN compares "greater"; ints compare exactly.
//   pfnArith   :1227-1289  result type = MAX(type codes); ints wrap; bool
//                          results are (value != 0); @div checks the divisor
//                          for zeros first (checkZero, h_system.cc:254-267).
//   pfnLogic   :1315-1332  bool only; nand/nor compute ~(x&y)/~(x|y) as bool,
//                          i.e. true for every input (h_system.cc:902-912).
//
// GB300 layout: each thread owns 16 consecutive elements, so a bool result
// is one 16-byte store and inputs are read with 16-byte vector loads when the
// chunk is aligned and complete.  Operands of different types are first
// converted to the common type (the reference's promoteValue), then the
// same-type kernel runs.
#include <climits>
#include <cstring>

#include "dev_common.cuh"

namespace hg {

enum { MODE_VV = 0, MODE_SV = 1, MODE_VS = 2 };  // scalar on the left / right

template <typename T>
__device__ __forceinline__ void load16(const T* __restrict__ p, long long i0, long long n, T (&v)[16]) {
    if (i0 + 16 <= n && ((reinterpret_cast<uintptr_t>(p + i0) & 15) == 0)) {
        const uint4* q = reinterpret_cast<const uint4*>(p + i0);
        constexpr int NV = (16 * sizeof(T)) / 16;
        uint4 tmp[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) tmp[k] = __ldcs(q + k);
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = reinterpret_cast<const T*>(tmp)[k];
    } else {
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = (i0 + k < n) ? p[i0 + k] : T(0);
    }
}

template <typename T>
__device__ __forceinline__ void store16(T* __restrict__ p, long long i0, long long n, const T (&v)[16]) {
    if (i0 + 16 <= n && ((reinterpret_cast<uintptr_t>(p + i0) & 15) == 0)) {
        uint4* q = reinterpret_cast<uint4*>(p + i0);
        constexpr int NV = (16 * sizeof(T)) / 16;
#pragma unroll
        for (int k = 0; k < NV; k++) q[k] = reinterpret_cast<const uint4*>(v)[k];
    } else {
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (i0 + k < n) p[i0 + k] = v[k];
    }
}

// compareFloat(x,y) (h_primitive.cc:1061) and the op switch of COMPFN (:1067-1071)
template <typename T>
__device__ __forceinline__ bool cmp_op(int op, T a, T b) {
    if constexpr (std::is_floating_point<T>::value) {
        int c = a < b ? ((double)(b - a) < H_EPSILON ? 0 : -1) : ((double)(a - b) < H_EPSILON ? 0 : 1);
        switch (op) {
        case 0: return c < 0;
        case 1: return c <= 0;
        case 2: return c > 0;
        case 3: return c >= 0;
        case 4: return c == 0;
        default: return c != 0;
        }
    } else {
        switch (op) {
        case 0: return a < b;
        case 1: return a <= b;
        case 2: return a > b;
        case 3: return a >= b;
        case 4: return a == b;
        default: return a != b;
        }
    }
}

// ARITH2 (h_primitive.cc:1225) in the promoted type.
template <typename T>
__device__ __forceinline__ T arith_op(int op, T a, T b, bool& divzero) {
    if constexpr (std::is_same<T, double>::value) {
        switch (op) {
        case 0: return __dadd_rn(a, b);
        case 1: return __dsub_rn(a, b);
        case 2: return __dmul_rn(a, b);
        default: if (b == 0.0) divzero = true; return __ddiv_rn(a, b);
        }
    } else if constexpr (std::is_same<T, float>::value) {
        switch (op) {
        case 0: return __fadd_rn(a, b);
        case 1: return __fsub_rn(a, b);
        case 2: return __fmul_rn(a, b);
        default: if (b == 0.0f) divzero = true; return __fdiv_rn(a, b);
        }
    } else if constexpr (std::is_same<T, bool>::value) {
        int x = a, y = b, r;
        switch (op) {
        case 0: r = x + y; break;
        case 1: r = x - y; break;
        case 2: r = x * y; break;
        default: if (y == 0) { divzero = true; r = 0; } else r = x / y; break;
        }
        return r != 0;
    } else if constexpr (sizeof(T) <= 2) {  // i8 / i16: computed in int, stored truncated
        int x = a, y = b, r;
        switch (op) {
        case 0: r = x + y; break;
        case 1: r = x - y; break;
        case 2: r = x * y; break;
        default: if (y == 0) { divzero = true; r = 0; } else r = x / y; break;
        }
        return (T)r;
    } else {  // i32 / i64 wrap; MIN / -1 is the wrapped negation
        using UT = typename std::make_unsigned<T>::type;
        switch (op) {
        case 0: return (T)((UT)a + (UT)b);
        case 1: return (T)((UT)a - (UT)b);
        case 2: return (T)((UT)a * (UT)b);
        default:
            if (b == 0) { divzero = true; return 0; }
            if (b == (T)-1) return (T)((UT)0 - (UT)a);
            return a / b;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_compare(const T* __restrict__ x, const T* __restrict__ y,
                                                 bool* __restrict__ z, long long n, int op, int mode, T sx, T sy) {
    long long nchunks = (n + 15) / 16;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nchunks;
         c += (long long)gridDim.x * blockDim.x) {
        long long i0 = c * 16;
        T a[16], b[16];
        if (mode == MODE_SV) {
#pragma unroll
            for (int k = 0; k < 16; k++) a[k] = sx;
        } else load16(x, i0, n, a);
        if (mode == MODE_VS) {
#pragma unroll
            for (int k = 0; k < 16; k++) b[k] = sy;
        } else load16(y, i0, n, b);
        bool r[16];
#pragma unroll
        for (int k = 0; k < 16; k++) r[k] = cmp_op<T>(op, a[k], b[k]);
        store16(z, i0, n, r);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_arith(const T* __restrict__ x, const T* __restrict__ y,
                                               T* __restrict__ z, long long n, int op, int mode, T sx, T sy,
                                               unsigned* derr) {
    long long nchunks = (n + 15) / 16;
    bool dz = false;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nchunks;
         c += (long long)gridDim.x * blockDim.x) {
        long long i0 = c * 16;
        T a[16], b[16], r[16];
        if (mode == MODE_SV) {
#pragma unroll
            for (int k = 0; k < 16; k++) a[k] = sx;
        } else load16(x, i0, n, a);
        if (mode == MODE_VS) {
#pragma unroll
            for (int k = 0; k < 16; k++) b[k] = sy;
        } else load16(y, i0, n, b);
#pragma unroll
        for (int k = 0; k < 16; k++) {
            bool d = false;
            r[k] = arith_op<T>(op, a[k], b[k], d);
            if (d && i0 + k < n) dz = true;
        }
        store16(z, i0, n, r);
    }
    if (dz) flag_error(derr, DERR_DIVZERO);
}

// bool logic over 16-byte words: and/or/xor act bytewise on 0/1 bytes
__global__ void __launch_bounds__(256) k_logic(const uint8_t* __restrict__ x, const uint8_t* __restrict__ y,
                                               uint8_t* __restrict__ z, long long n, int op, int mode,
                                               uint8_t sx, uint8_t sy) {
    long long nchunks = (n + 15) / 16;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nchunks;
         c += (long long)gridDim.x * blockDim.x) {
        long long i0 = c * 16;
        uint8_t a[16], b[16], r[16];
        if (mode == MODE_SV) {
#pragma unroll
            for (int k = 0; k < 16; k++) a[k] = sx;
        } else load16(x, i0, n, a);
        if (mode == MODE_VS) {
#pragma unroll
            for (int k = 0; k < 16; k++) b[k] = sy;
        } else load16(y, i0, n, b);
#pragma unroll
        for (int k = 0; k < 16; k++) {
            switch (op) {
            case 0: r[k] = a[k] & b[k]; break;
            case 2: r[k] = a[k] | b[k]; break;
            case 4: r[k] = a[k] ^ b[k]; break;
            case 5: r[k] = a[k] ^ 1u; break;  // not
            default: r[k] = 1; break;         // nand / nor: ~(.) as bool is always true
            }
        }
        store16(z, i0, n, r);
    }
}

// promotion of a vector of type `st` to T (promoteValueWithIndex, h_system.cc:168-252)
template <typename T>
__global__ void k_convert(const void* __restrict__ src, int st, T* __restrict__ dst, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        T v;
        switch (st) {
        case H_B: v = (T)((const bool*)src)[i]; break;
        case H_J: v = (T)((const int8_t*)src)[i]; break;
        case H_H: v = (T)((const int16_t*)src)[i]; break;
        case H_I: v = (T)((const int32_t*)src)[i]; break;
        case H_L: v = (T)((const long long*)src)[i]; break;
        case H_F: v = (T)((const float*)src)[i]; break;
        default: v = (T)((const double*)src)[i]; break;
        }
        dst[i] = v;
    }
}

static unsigned ew_grid(long long n) {
    long long chunks = (n + 15) / 16;
    long long b = (chunks + 255) / 256;
    long long cap = (long long)g_sms * 8;
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// Host value of element 0 of x converted to T (scalar operands are passed by value).
template <typename T>
static I scalar_as(V x, T* out) {
    uint64_t bits;
    HG_CHECK(read_elem0(x, &bits));
    switch (x->typ) {
    case H_B: *out = (T)(*(bool*)&bits); break;
    case H_J: case H_C: *out = (T)(*(int8_t*)&bits); break;
    case H_H: *out = (T)(*(int16_t*)&bits); break;
    case H_I: case H_M: case H_D: case H_U: case H_W: case H_T: *out = (T)(*(int32_t*)&bits); break;
    case H_L: case H_Z: *out = (T)(*(long long*)&bits); break;
    case H_F: *out = (T)(*(float*)&bits); break;
    case H_E: *out = (T)(*(double*)&bits); break;
    default: return E_NOT_IMPL;
    }
    return 0;
}

// Device vector of x in type T (converted into scratch when x has another type)
template <typename T>
static I vector_as(V x, I xt, const T** out) {
    const void* p;
    HG_CHECK(in_ptr(x, &p));
    if (x->typ == xt) { *out = (const T*)p; return 0; }
    T* d = (T*)salloc((size_t)x->len * sizeof(T));
    if (!d) return E_DEVICE_OOM;
    HG_LAUNCH("convert", ew_grid(x->len * 16 / 16), 256, 0, k_convert<T>, p, (int)x->typ, d, (long long)x->len);
    *out = d;
    return 0;
}

static int compare_float_host(double a, double b) {
    return a < b ? ((b - a) < H_EPSILON ? 0 : -1) : ((a - b) < H_EPSILON ? 0 : 1);
}
static double from_ord(long long o) {
    unsigned long long b = o >= 0 ? (unsigned long long)o : (0x8000000000000000ull | (unsigned long long)(-o));
    double d;
    memcpy(&d, &b, 8);
    return d;
}

F64Cmp f64_cmp_thresholds(double s, bool scalar_first) {
    F64Cmp t;
    if (s != s) {  // a NaN operand compares as 1 everywhere
        t.ta = t.tb = LLONG_MAX;
        t.ca = t.cb = t.cc = 1;
        return t;
    }
    const long long lo = f64_ord(0xfff0000000000000ull), hi = f64_ord(0x7ff0000000000000ull) + 1;  // -inf .. +inf + 1
    auto c = [&](long long o) { return scalar_first ? compare_float_host(s, from_ord(o)) : compare_float_host(from_ord(o), s); };
    // smallest o in [lo, hi] with pred(o); o = hi stands for "no such value"
    auto first = [&](auto pred) {
        long long a = lo, b = hi;
        while (a < b) {
            long long m = a + (long long)(((unsigned long long)b - (unsigned long long)a) / 2);  // b - a can exceed 2^63
            if (pred(m)) b = m; else a = m + 1;
        }
        return a;
    };
    if (!scalar_first) {  // compareFloat(v, s): -1, 0, 1 as v grows
        t.ta = first([&](long long o) { return c(o) >= 0; });
        t.tb = first([&](long long o) { return c(o) >= 1; });
        t.ca = -1; t.cb = 0; t.cc = 1;
    } else {  // compareFloat(s, v): 1, 0, -1 as v grows
        t.ta = first([&](long long o) { return c(o) <= 0; });
        t.tb = first([&](long long o) { return c(o) <= -1; });
        t.ca = 1; t.cb = 0; t.cc = -1;
    }
    return t;
}

// a double vector against a fixed double, by the integer thresholds
__global__ void __launch_bounds__(256) k_compare_f64_fixed(const double* __restrict__ x, bool* __restrict__ z,
                                                           long long n, int op, F64Cmp t) {
    long long nchunks = (n + 15) / 16;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nchunks;
         c += (long long)gridDim.x * blockDim.x) {
        long long i0 = c * 16;
        double a[16];
        load16(x, i0, n, a);
        bool r[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            int cv = f64_cmp_fixed(a[k], t);
            r[k] = op == 0 ? cv < 0 : op == 1 ? cv <= 0 : op == 2 ? cv > 0 : op == 3 ? cv >= 0 : op == 4 ? cv == 0 : cv != 0;
        }
        store16(z, i0, n, r);
    }
}

template <typename T>
static I run_compare(V z, V x, V y, I typX, int op) {
    bool ox = x->len == 1, oy = y->len == 1;
    L n = ox ? y->len : x->len;
    int mode = ox ? MODE_SV : (oy ? MODE_VS : MODE_VV);
    T sx = 0, sy = 0;
    const T *px = nullptr, *py = nullptr;
    if (mode == MODE_SV) HG_CHECK(scalar_as<T>(x, &sx)); else HG_CHECK(vector_as<T>(x, typX, &px));
    if (mode == MODE_VS) HG_CHECK(scalar_as<T>(y, &sy)); else HG_CHECK(vector_as<T>(y, typX, &py));
    void* dz;
    HG_CHECK(alloc_out(z, H_B, n, &dz));
    if constexpr (std::is_same<T, double>::value) {
        if (mode != MODE_VV && n > 0) {  // one side fixed: integer thresholds instead of FP64 subtractions
            const F64Cmp t = f64_cmp_thresholds(mode == MODE_SV ? sx : sy, mode == MODE_SV);
            HG_LAUNCH("compare", ew_grid(n), 256, 0, k_compare_f64_fixed, mode == MODE_SV ? py : px, (bool*)dz,
                      (long long)n, op, t);
            HG_CHECK(last_launch_error());
            return finish_out(z, dz);
        }
    }
    if (n > 0) HG_LAUNCH("compare", ew_grid(n), 256, 0, k_compare<T>, px, py, (bool*)dz, (long long)n, op, mode, sx, sy);
    HG_CHECK(last_launch_error());
    return finish_out(z, dz);
}

template <typename T>
static I run_arith(V z, V x, V y, I typ, int op) {
    bool ox = x->len == 1, oy = y->len == 1;
    L n = ox ? y->len : x->len;
    int mode = ox ? MODE_SV : (oy ? MODE_VS : MODE_VV);
    T sx = 0, sy = 0;
    const T *px = nullptr, *py = nullptr;
    if (mode == MODE_SV) HG_CHECK(scalar_as<T>(x, &sx)); else HG_CHECK(vector_as<T>(x, typ, &px));
    if (mode == MODE_VS) HG_CHECK(scalar_as<T>(y, &sy)); else HG_CHECK(vector_as<T>(y, typ, &py));
    long long mark = out_mark();
    void* dz;
    HG_CHECK(alloc_out(z, typ, n, &dz));
    if (n > 0)
        HG_LAUNCH("arith", ew_grid(n), 256, 0, k_arith<T>, px, py, (T*)dz, (long long)n, op, mode, sx, sy, g_derr);
    HG_CHECK(last_launch_error());
    if (op == 3) {  // checkZero (h_system.cc:254-267) runs before the division in the reference
        I e = check_device_errors();
        if (e) { out_rewind(mark); return e; }
    }
    return finish_out(z, dz);
}

// Device vector of x converted to basic type `typ` (promoteValue semantics).
I promote_to(V x, I typ, const void** out) {
    switch (typ) {
    case H_B: return vector_as<bool>(x, typ, (const bool**)out);
    case H_J: return vector_as<int8_t>(x, typ, (const int8_t**)out);
    case H_H: return vector_as<int16_t>(x, typ, (const int16_t**)out);
    case H_I: return vector_as<int32_t>(x, typ, (const int32_t**)out);
    case H_L: return vector_as<long long>(x, typ, (const long long**)out);
    case H_F: return vector_as<float>(x, typ, (const float**)out);
    case H_E: return vector_as<double>(x, typ, (const double**)out);
    default: return E_NOT_IMPL;
    }
}

}  // namespace hg

using namespace hg;

extern "C" {

I pfnCompare(V z, V x, V y, I op) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!(is_comparable(x->typ) && is_comparable(y->typ))) return E_DOMAIN;
    if (!(x->len == 1 || y->len == 1 || x->len == y->len)) return E_LENGTH;
    if (is_real(x->typ) && is_real(y->typ)) {
        I t = x->typ > y->typ ? x->typ : y->typ;
        switch (t) {
        case H_B: return run_compare<bool>(z, x, y, t, op);
        case H_J: return run_compare<int8_t>(z, x, y, t, op);
        case H_H: return run_compare<int16_t>(z, x, y, t, op);
        case H_I: return run_compare<int32_t>(z, x, y, t, op);
        case H_L: return run_compare<long long>(z, x, y, t, op);
        case H_F: return run_compare<float>(z, x, y, t, op);
        default: return run_compare<double>(z, x, y, t, op);
        }
    }
    if (x->typ == y->typ) {
        switch (x->typ) {
        case H_C: return run_compare<int8_t>(z, x, y, H_C, op);  // signed char, as the reference's x86 build
        case H_M: case H_D: case H_U: case H_T: return run_compare<int32_t>(z, x, y, x->typ, op);
        case H_Z: return run_compare<long long>(z, x, y, H_Z, op);
        case H_Q: return compare_symbols(z, x, y, op);
        default: return set_error(E_NOT_IMPL, "compare of type %d (no case in the reference)", x->typ);
        }
    }
    return E_TYPE;
}
I pfnLt(V z, V x, V y) { return pfnCompare(z, x, y, 0); }
I pfnLeq(V z, V x, V y) { return pfnCompare(z, x, y, 1); }
I pfnGt(V z, V x, V y) { return pfnCompare(z, x, y, 2); }
I pfnGeq(V z, V x, V y) { return pfnCompare(z, x, y, 3); }
I pfnEq(V z, V x, V y) { return pfnCompare(z, x, y, 4); }
I pfnNeq(V z, V x, V y) { return pfnCompare(z, x, y, 5); }

I pfnArith(V z, V x, V y, I op) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (is_real(x->typ) && is_real(y->typ)) {
        if (!(x->len == 1 || y->len == 1 || x->len == y->len)) return E_LENGTH;
        I t = x->typ > y->typ ? x->typ : y->typ;
        if (op == 3 && y->len == 1) {  // scalar divisor: checkZero on the host value
            double d;
            HG_CHECK(scalar_as<double>(y, &d));
            if (d == 0.0) return E_DIV_ZERO;
        }
        switch (t) {
        case H_B: return run_arith<bool>(z, x, y, t, op);
        case H_J: return run_arith<int8_t>(z, x, y, t, op);
        case H_H: return run_arith<int16_t>(z, x, y, t, op);
        case H_I: return run_arith<int32_t>(z, x, y, t, op);
        case H_L: return run_arith<long long>(z, x, y, t, op);
        case H_F: return run_arith<float>(z, x, y, t, op);
        default: return run_arith<double>(z, x, y, t, op);
        }
    }
    if (is_dtime(x->typ) && is_dtime(y->typ)) return E_NOT_IMPL;
    return E_DOMAIN;
}
I pfnPlus(V z, V x, V y) { return pfnArith(z, x, y, 0); }
I pfnMinus(V z, V x, V y) { return pfnArith(z, x, y, 1); }
I pfnMul(V z, V x, V y) { return pfnArith(z, x, y, 2); }
I pfnDiv(V z, V x, V y) { return pfnArith(z, x, y, 3); }

static I logic(V z, V x, V y, int op) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!(x->typ == H_B && y->typ == H_B)) return E_DOMAIN;
    if (!(x->len == 1 || y->len == 1 || x->len == y->len)) return E_LENGTH;
    bool ox = x->len == 1, oy = y->len == 1;
    L n = ox ? y->len : x->len;
    int mode = ox ? MODE_SV : (oy ? MODE_VS : MODE_VV);
    uint64_t bx = 0, by = 0;
    const void *px = nullptr, *py = nullptr;
    if (mode == MODE_SV) HG_CHECK(read_elem0(x, &bx)); else HG_CHECK(in_ptr(x, &px));
    if (mode == MODE_VS) HG_CHECK(read_elem0(y, &by)); else HG_CHECK(in_ptr(y, &py));
    void* dz;
    HG_CHECK(alloc_out(z, H_B, n, &dz));
    if (n > 0)
        HG_LAUNCH("logic", ew_grid(n), 256, 0, k_logic, (const uint8_t*)px, (const uint8_t*)py, (uint8_t*)dz,
                  (long long)n, op, mode, (uint8_t)(bx & 1), (uint8_t)(by & 1));
    HG_CHECK(last_launch_error());
    return finish_out(z, dz);
}
I pfnAnd(V z, V x, V y) { return logic(z, x, y, 0); }
I pfnNand(V z, V x, V y) { return logic(z, x, y, 1); }
I pfnOr(V z, V x, V y) { return logic(z, x, y, 2); }
I pfnNor(V z, V x, V y) { return logic(z, x, y, 3); }
I pfnXor(V z, V x, V y) { return logic(z, x, y, 4); }

// pfnNot: h_primitive.cc:606-615
I pfnNot(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (x->typ != H_B) return E_DOMAIN;
    const void* px;
    HG_CHECK(in_ptr(x, &px));
    void* dz;
    HG_CHECK(alloc_out(z, H_B, x->len, &dz));
    if (x->len > 0)
        HG_LAUNCH("not", ew_grid(x->len), 256, 0, k_logic, (const uint8_t*)px, (const uint8_t*)px, (uint8_t*)dz,
                  (long long)x->len, 5, MODE_VV, (uint8_t)0, (uint8_t)0);
    HG_CHECK(last_launch_error());
    return finish_out(z, dz);
}

}  // extern "C"
