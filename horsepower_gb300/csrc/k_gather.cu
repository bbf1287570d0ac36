// @index (gather) and the list plumbing used around it.
//
// pfnIndex (h_primitive.cc:43-94): z[i] = x[y[i]] with y promoted to i64 and
// checked against len(x) (E_INDEX).  The reference does not check negative
// indices (it reads before the buffer); here they are E_INDEX as well, since
// a device read out of bounds is never issued.  For a non-i64 index vector
// the reference reads the narrow buffer at 8-byte stride (:60); here the
// promoted value is used.
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

}  // namespace hg

using namespace hg;

extern "C" {

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
