// @index (gather) and the list plumbing used around it.
//
// pfnIndex (h_primitive.cc:43-94): z[i] = x[y[i]] with y promoted to i64 and
// checked against len(x) (E_INDEX).  The reference does not check negative
// indices (it reads before the buffer); here they are E_INDEX as well, since
// a device read out of bounds is never issued.  For a non-i64 index vector
// the reference reads the narrow buffer at 8-byte stride (:60); here the
// promoted value is used.
#include <vector>

#include "dev_common.cuh"

namespace hg {

template <typename IT>
__device__ __forceinline__ long long load_idx(const void* y, long long i) {
    return (long long)((const IT*)y)[i];
}

template <typename ET, typename IT>
__global__ void __launch_bounds__(256) k_gather(const ET* __restrict__ x, long long nx, const void* __restrict__ y,
                                                ET* __restrict__ z, long long n, unsigned* derr, int vec) {
    bool bad = false;
    long long stride = (long long)gridDim.x * blockDim.x * 4;
    for (long long i0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4; i0 < n; i0 += stride) {
        long long ix[4];
        if constexpr (sizeof(IT) == 8) {
            if (vec && i0 + 4 <= n) {  // the thread's 4 indices: two 16-byte loads (i0 is a multiple of 4)
                const longlong2* q = reinterpret_cast<const longlong2*>((const long long*)y + i0);
                longlong2 a = __ldcs(q), b = __ldcs(q + 1);
                ix[0] = a.x; ix[1] = a.y; ix[2] = b.x; ix[3] = b.y;
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++) ix[k] = (i0 + k < n) ? load_idx<IT>(y, i0 + k) : 0;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) ix[k] = (i0 + k < n) ? load_idx<IT>(y, i0 + k) : 0;
        }
        ET v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            bool ok = ix[k] >= 0 && ix[k] < nx;
            if (!ok && i0 + k < n) bad = true;
            v[k] = (ok && i0 + k < n) ? __ldg(x + ix[k]) : ET(0);
        }
        if constexpr (sizeof(ET) == 8) {
            if (vec && i0 + 4 <= n) {
                ulonglong2* q = reinterpret_cast<ulonglong2*>(z + i0);
                q[0] = make_ulonglong2((unsigned long long)v[0], (unsigned long long)v[1]);
                q[1] = make_ulonglong2((unsigned long long)v[2], (unsigned long long)v[3]);
                continue;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (i0 + k < n) z[i0 + k] = v[k];
    }
    if (bad) flag_error(derr, DERR_INDEX);
}

template <typename ET>
static void launch_gather(const void* x, long long nx, const void* y, I ytyp, void* z, long long n) {
    unsigned grid = grid_for((n + 3) / 4, 256);
    unsigned cap = (unsigned)g_sms * 16;
    if (grid > cap) grid = cap;
    // 16-byte index loads and value stores need both vectors 16-byte aligned
    const int vec = (((uintptr_t)y | (uintptr_t)z) & 15) == 0;
    switch (ytyp) {
    case H_B: HG_LAUNCH("gather", grid, 256, 0, (k_gather<ET, bool>), (const ET*)x, nx, y, (ET*)z, n, g_derr, vec); break;
    case H_J: HG_LAUNCH("gather", grid, 256, 0, (k_gather<ET, int8_t>), (const ET*)x, nx, y, (ET*)z, n, g_derr, vec); break;
    case H_H: HG_LAUNCH("gather", grid, 256, 0, (k_gather<ET, int16_t>), (const ET*)x, nx, y, (ET*)z, n, g_derr, vec); break;
    case H_I: HG_LAUNCH("gather", grid, 256, 0, (k_gather<ET, int32_t>), (const ET*)x, nx, y, (ET*)z, n, g_derr, vec); break;
    default: HG_LAUNCH("gather", grid, 256, 0, (k_gather<ET, long long>), (const ET*)x, nx, y, (ET*)z, n, g_derr, vec); break;
    }
}

I gather_into(const void* x, long long nx, int es, const void* y, I ytyp, void* z, long long n) {
    if (n <= 0) return 0;
    switch (es) {
    case 1: launch_gather<uint8_t>(x, nx, y, ytyp, z, n); break;
    case 2: launch_gather<uint16_t>(x, nx, y, ytyp, z, n); break;
    case 4: launch_gather<uint32_t>(x, nx, y, ytyp, z, n); break;
    default: launch_gather<unsigned long long>(x, nx, y, ytyp, z, n); break;
    }
    return last_launch_error();
}

// ---- several columns gathered by one index (pattern.cc:558-672, the
// "common index" pattern: every use of an index vector is an @index with it
// as the second argument).  Each thread reads its four indices once and
// issues the loads of every column, so the index vector is read once and
// the columns' loads overlap.
constexpr int GM_MAXCOL = 8;
struct GatherCols {
    const void* src[GM_MAXCOL];
    void* dst[GM_MAXCOL];
    long long nx[GM_MAXCOL];
    int es[GM_MAXCOL];
    int ncol;
};

template <int ES>
struct UintOf;
template <> struct UintOf<1> { using T = uint8_t; };
template <> struct UintOf<2> { using T = uint16_t; };
template <> struct UintOf<4> { using T = uint32_t; };
template <> struct UintOf<8> { using T = unsigned long long; };

template <int ES>
__device__ __forceinline__ void gm_column(const void* src, long long nx, void* dst, const long long (&ix)[4],
                                          long long i0, long long n, bool full, bool& bad) {
    using ET = typename UintOf<ES>::T;
    ET v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const bool in = i0 + k < n, ok = ix[k] >= 0 && ix[k] < nx;
        if (in && !ok) bad = true;
        v[k] = (in && ok) ? __ldg((const ET*)src + ix[k]) : ET(0);
    }
    ET* z = (ET*)dst + i0;
    if (full) {  // i0 is a multiple of 4 and dst is 16-byte aligned
        if constexpr (ES == 1) {
            *(uint32_t*)z = (uint32_t)v[0] | ((uint32_t)v[1] << 8) | ((uint32_t)v[2] << 16) | ((uint32_t)v[3] << 24);
        } else if constexpr (ES == 2) {
            *(uint2*)z = make_uint2((uint32_t)v[0] | ((uint32_t)v[1] << 16), (uint32_t)v[2] | ((uint32_t)v[3] << 16));
        } else if constexpr (ES == 4) {
            *(uint4*)z = make_uint4(v[0], v[1], v[2], v[3]);
        } else {
            ((ulonglong2*)z)[0] = make_ulonglong2(v[0], v[1]);
            ((ulonglong2*)z)[1] = make_ulonglong2(v[2], v[3]);
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (i0 + k < n) z[k] = v[k];
}

template <typename IT>
__global__ void __launch_bounds__(256) k_gather_many(GatherCols c, const void* __restrict__ y, long long n, unsigned* derr,
                                                     int vec) {
    bool bad = false;
    const long long stride = (long long)gridDim.x * blockDim.x * 4;
    for (long long i0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4; i0 < n; i0 += stride) {
        const bool full = vec && i0 + 4 <= n;
        long long ix[4];
        if (full && sizeof(IT) == 8) {
            const longlong2* q = reinterpret_cast<const longlong2*>((const long long*)y + i0);
            const longlong2 a = __ldcs(q), b = __ldcs(q + 1);
            ix[0] = a.x; ix[1] = a.y; ix[2] = b.x; ix[3] = b.y;
        } else if (full && sizeof(IT) == 4) {
            const int4 a = __ldcs(reinterpret_cast<const int4*>((const int32_t*)y + i0));
            ix[0] = a.x; ix[1] = a.y; ix[2] = a.z; ix[3] = a.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) ix[k] = (i0 + k < n) ? (long long)((const IT*)y)[i0 + k] : 0;
        }
        for (int j = 0; j < c.ncol; j++) {
            switch (c.es[j]) {
            case 1: gm_column<1>(c.src[j], c.nx[j], c.dst[j], ix, i0, n, full, bad); break;
            case 2: gm_column<2>(c.src[j], c.nx[j], c.dst[j], ix, i0, n, full, bad); break;
            case 4: gm_column<4>(c.src[j], c.nx[j], c.dst[j], ix, i0, n, full, bad); break;
            default: gm_column<8>(c.src[j], c.nx[j], c.dst[j], ix, i0, n, full, bad); break;
            }
        }
    }
    if (bad) flag_error(derr, DERR_INDEX);
}

static I gather_many(const GatherCols& c, const void* y, I ytyp, long long n) {
    if (n <= 0) return 0;
    unsigned grid = grid_for((n + 3) / 4, 256);
    const unsigned cap = (unsigned)g_sms * 16;
    if (grid > cap) grid = cap;
    uintptr_t al = (uintptr_t)y;
    for (int j = 0; j < c.ncol; j++) al |= (uintptr_t)c.dst[j];
    const int vec = (al & 15) == 0;
    switch (ytyp) {
    case H_B: HG_LAUNCH("gather_many", grid, 256, 0, k_gather_many<bool>, c, y, n, g_derr, 0); break;
    case H_J: HG_LAUNCH("gather_many", grid, 256, 0, k_gather_many<int8_t>, c, y, n, g_derr, 0); break;
    case H_H: HG_LAUNCH("gather_many", grid, 256, 0, k_gather_many<int16_t>, c, y, n, g_derr, 0); break;
    case H_I: HG_LAUNCH("gather_many", grid, 256, 0, k_gather_many<int32_t>, c, y, n, g_derr, vec); break;
    default: HG_LAUNCH("gather_many", grid, 256, 0, k_gather_many<long long>, c, y, n, g_derr, vec); break;
    }
    return last_launch_error();
}

}  // namespace hg

using namespace hg;

extern "C" {

// z[k] = x[k][y] for k < n, as n pfnIndex calls on basic-typed columns, in
// one pass over y.  Any index outside any column gives E_INDEX and no output.
I hgpuIndexMany(V* z, V* x, V y, L n) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!is_int(y->typ)) return E_DOMAIN;
    if (n < 1) return 0;
    for (L k = 0; k < n; k++)
        if (!is_basic(x[k]->typ)) return E_NOT_IMPL;
    const void* py;
    HG_CHECK(in_ptr(y, &py));
    const long long m = y->len, mark = out_mark();
    std::vector<void*> dz((size_t)n);
    bool in_range = y->typ == H_L;
    for (L k0 = 0; k0 < n; k0 += GM_MAXCOL) {
        GatherCols c{};
        c.ncol = (int)((n - k0) < GM_MAXCOL ? (n - k0) : GM_MAXCOL);
        for (int j = 0; j < c.ncol; j++) {
            V xk = x[k0 + j];
            HG_CHECK(in_ptr(xk, &c.src[j]));
            c.nx[j] = xk->len;
            c.es[j] = esize(xk->typ);
            I rc = alloc_out(z[k0 + j], xk->typ, m, &dz[(size_t)(k0 + j)]);
            if (rc) { out_rewind(mark); return rc; }
            c.dst[j] = dz[(size_t)(k0 + j)];
            in_range = in_range && known_in_range(y->g, m, xk->len);
        }
        I rc = gather_many(c, py, y->typ, m);
        if (rc) { out_rewind(mark); return rc; }
    }
    if (!in_range) {
        I e = check_device_errors();
        if (e) { out_rewind(mark); return e; }
    }
    for (L k = 0; k < n; k++) HG_CHECK(finish_out(z[k], dz[(size_t)k]));
    return 0;
}

I pfnIndex(V z, V x, V y) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!is_int(y->typ)) return E_DOMAIN;
    if (is_basic(x->typ)) {
        const void *px, *py;
        HG_CHECK(in_ptr(x, &px));
        HG_CHECK(in_ptr(y, &py));
        long long mark = out_mark();
        void* dz;
        HG_CHECK(alloc_out(z, x->typ, y->len, &dz));
        HG_CHECK(gather_into(px, x->len, esize(x->typ), py, y->typ, dz, y->len));
        if (!(y->typ == H_L && known_in_range(y->g, y->len, x->len))) {
            I e = check_device_errors();
            if (e) { out_rewind(mark); return e; }
        }
        return finish_out(z, dz);
    }
    if (x->typ == H_G) {  // list indexed by one integer: alias the element (h_primitive.cc:74-88)
        if (y->len != 1) return E_NOT_IMPL;
        uint64_t bits;
        HG_CHECK(read_elem0(y, &bits));
        long long k;
        switch (y->typ) {
        case H_B: k = *(bool*)&bits; break;
        case H_J: k = *(int8_t*)&bits; break;
        case H_H: k = *(int16_t*)&bits; break;
        case H_I: k = *(int32_t*)&bits; break;
        default: k = *(long long*)&bits; break;
        }
        if (k < 0 || k >= x->len) return E_INDEX;
        V0* e = host_nodes(x) + k;
        *z = *e;
        if (is_inline(e)) z->g = (G)&z->b;
        return 0;
    }
    return E_NOT_IMPL;
}

// pfnList: h_primitive.cc:32-36 (node copies, payloads aliased)
I pfnList(V z, L n, V x[]) {
    HG_CHECK(ensure_init());
    HG_CHECK(init_list(z, H_G, n));
    V0* d = host_nodes(z);
    for (L i = 0; i < n; i++) {
        d[i] = *x[i];
        if (is_inline(x[i])) d[i].g = (G)&d[i].b;
    }
    return 0;
}

// pfnKeys / pfnValues on dicts, tables and enums (h_primitive.cc:191-217, h_system.cc:501-515)
I pfnKeys(V z, V x) {
    if (x->typ == H_Y) {  // the enum's key node (copyV)
        if (!x->y || !x->y->ek) return E_DOMAIN;
        V ek = (V)x->y->ek;
        *z = *ek;
        if (is_inline(ek)) z->g = (G)&z->b;
        return 0;
    }
    if (x->typ != H_N && x->typ != H_A) return E_DOMAIN;
    V0* e = host_nodes(x);
    *z = e[0];
    if (is_inline(&e[0])) z->g = (G)&z->b;
    return 0;
}
I pfnValues(V z, V x) {
    if (x->typ == H_Y) {  // copyEnumIndex (h_system.cc:501-506): the i64 index itself
        z->typ = H_L;
        z->len = x->len;
        if (x->len > 1) { z->g = x->g; return 0; }
        z->g = (G)&z->b;
        z->i64 = 0;
        if (x->len == 1) {
            HG_CHECK(ensure_init());
            V0 t = *x;
            t.typ = H_L;
            uint64_t bits;
            HG_CHECK(read_elem0(&t, &bits));
            z->i64 = (L)bits;
        }
        return 0;
    }
    if (x->typ != H_N && x->typ != H_A) return E_DOMAIN;
    V0* e = host_nodes(x) + 1;
    *z = *e;
    if (is_inline(e)) z->g = (G)&z->b;
    return 0;
}

}  // extern "C"
