// Stream compaction: @compress, @where and the multi-column compress that
// the pattern pass emits.
//
// Reference: pfnCompress (h_primitive.cc:1479-1521) counts the selected rows
// per OpenMP thread (getNumOfNonZero, h_system.cc:304-310), scans the counts
// and scatters in a second pass; the result is stable, and when every row is
// selected the output aliases the input (copyV, :1513-1515).  pfnWhere
// (:728-762) does the same writing i64 row numbers.
//
// GB300 kernel: one pass.  A tile is 4096 rows handled by 8 warps; each lane
// reads its 16 mask bytes with one 128-bit load and counts them with popc;
// the tile's offset comes from a decoupled look-back over tile status words;
// each warp then walks its 512 rows in rounds of 32, and selected lanes write
// to consecutive positions found with ballot/popc.  Values are only read for
// selected rows, so a sparse mask reads a fraction of the value column.
#include "dev_common.cuh"

namespace hg {

constexpr int CT_THREADS = 256, CT_ITEMS = 16, CT_TILE = CT_THREADS * CT_ITEMS;  // 4096 rows
constexpr int CT_MAXCOL = 8;

struct CompactCols {
    const void* src[CT_MAXCOL];
    void* dst[CT_MAXCOL];
    int es[CT_MAXCOL];  // element bytes; 0 = write the row number as i64 (@where)
    int ncol;
};

__device__ __forceinline__ void copy_elem(const void* src, void* dst, long long i, long long o, int es) {
    switch (es) {
    case 1: ((uint8_t*)dst)[o] = ((const uint8_t*)src)[i]; break;
    case 2: ((uint16_t*)dst)[o] = ((const uint16_t*)src)[i]; break;
    case 4: ((uint32_t*)dst)[o] = ((const uint32_t*)src)[i]; break;
    case 8: ((uint64_t*)dst)[o] = ((const uint64_t*)src)[i]; break;
    default: ((long long*)dst)[o] = i; break;
    }
}

__global__ void __launch_bounds__(CT_THREADS) k_compact(const uint8_t* __restrict__ mask, long long n, CompactCols cols,
                                                        unsigned long long* status, unsigned* ticket,
                                                        unsigned long long* total, unsigned* derr) {
    __shared__ __align__(16) uint8_t smask[CT_TILE];
    __shared__ unsigned warp_tot[8];
    __shared__ unsigned long long tile_off;
    __shared__ long long tile_id;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) tile_id = atomicAdd(ticket, 1u);
    __syncthreads();
    const long long t = tile_id;
    const long long base = t * CT_TILE;
    // ---- phase 1: count (blocked: lane owns 16 consecutive mask bytes)
    const int lofs = (int)warp * 512 + (int)lane * 16;
    uint4 m4 = make_uint4(0, 0, 0, 0);
    if (base + lofs + 16 <= n) {
        m4 = __ldcs(reinterpret_cast<const uint4*>(mask + base + lofs));
    } else {
        uint8_t b[16];
#pragma unroll
        for (int k = 0; k < 16; k++) b[k] = (base + lofs + k < n) ? (mask[base + lofs + k] != 0) : 0;
        m4 = *reinterpret_cast<uint4*>(b);
    }
    *reinterpret_cast<uint4*>(smask + lofs) = m4;
    unsigned cnt = __popc(m4.x) + __popc(m4.y) + __popc(m4.z) + __popc(m4.w);
    unsigned wsum = warp_sum(cnt);
    if (lane == 0) warp_tot[warp] = wsum;
    __syncthreads();
    if (warp == 0) {
        unsigned v = lane < 8 ? warp_tot[lane] : 0;
        unsigned agg = warp_sum(v);
        unsigned long long excl = lookback_exclusive(status, t, agg, derr);
        if (lane == 0) {
            tile_off = excl;
            if (base + CT_TILE >= n) *total = excl + agg;  // last tile
        }
    }
    __syncthreads();
    // ---- phase 2: scatter (warp-striped rounds of 32 rows)
    unsigned long long off = tile_off;
    for (unsigned w = 0; w < warp; w++) off += warp_tot[w];
    const int wbase = (int)warp * 512;
#pragma unroll 4
    for (int k = 0; k < 16; k++) {
        const int li = wbase + k * 32 + (int)lane;
        const bool sel = smask[li] != 0;
        const unsigned bal = __ballot_sync(0xffffffffu, sel);
        if (sel) {
            const long long o = (long long)off + __popc(bal & lanemask_lt());
            const long long i = base + li;
            for (int c = 0; c < cols.ncol; c++) copy_elem(cols.src[c], cols.dst[c], i, o, cols.es[c]);
        }
        off += __popc(bal);
    }
}

// Runs the single-pass compaction; *count receives the number of selected rows.
static I compact(const uint8_t* mask, long long n, CompactCols& cols, long long* count) {
    long long ntiles = (n + CT_TILE - 1) / CT_TILE;
    if (ntiles == 0) { *count = 0; return 0; }
    char* s = (char*)salloc(ntiles * 8 + 64);
    if (!s) return E_DEVICE_OOM;
    unsigned long long* status = (unsigned long long*)s;
    unsigned* ticket = (unsigned*)(s + ntiles * 8);
    unsigned long long* total = (unsigned long long*)(s + ntiles * 8 + 8);
    HG_CU(cudaMemsetAsync(s, 0, ntiles * 8 + 64, g_stream));
    HG_LAUNCH("compact", (unsigned)ntiles, CT_THREADS, 0, k_compact, mask, n, cols, status, ticket, total, g_derr);
    HG_CHECK(last_launch_error());
    unsigned long long h = 0;
    HG_CU(cudaMemcpyAsync(&h, total, 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());  // synchronises
    *count = (long long)h;
    return 0;
}

static bool compress_type_ok(I t) {
    // types pfnCompress handles (h_primitive.cc:1497-1510)
    return t == H_B || t == H_J || t == H_H || t == H_I || t == H_L || t == H_F || t == H_E || t == H_Q ||
           t == H_C || t == H_S || t == H_D;
}

// One compress into z.  The output is allocated at full length, written in
// one pass and shrunk to the selected count.
static I compress_one(V z, V x, V y) {
    if (x->typ != H_B) return E_DOMAIN;
    if (x->len != y->len) return E_LENGTH;
    if (!compress_type_ok(y->typ)) return set_error(E_NOT_IMPL, "compress: type %d", y->typ);
    long long n = x->len;
    const void *pm, *pv;
    HG_CHECK(in_ptr(x, &pm));
    HG_CHECK(in_ptr(y, &pv));
    int es = esize(y->typ);
    long long mark = out_mark();
    void* d = n > 1 ? dalloc((size_t)n * es) : salloc(16);
    if (!d) return E_DEVICE_OOM;
    CompactCols cols{};
    cols.src[0] = pv; cols.dst[0] = d; cols.es[0] = es; cols.ncol = 1;
    long long cnt = 0;
    I e = compact((const uint8_t*)pm, n, cols, &cnt);
    if (e) { out_rewind(mark); return e; }
    if (cnt == n && n > 0) {  // every row selected: alias the input (copyV)
        out_rewind(mark);
        *z = *y;
        if (is_inline(y)) z->g = (G)&z->b;
        return 0;
    }
    z->typ = y->typ;
    z->len = cnt;
    if (cnt <= 1) {
        void* tmp = d;
        z->g = (G)&z->b;
        z->i64 = 0;
        if (cnt == 1) HG_CU(cudaMemcpyAsync(&z->b, tmp, es, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaStreamSynchronize(g_stream));
        out_rewind(mark);
        return apply_residency(z);
    }
    dshrink(d, (size_t)cnt * es);
    z->g = (G)d;
    return apply_residency(z);
}

// Row numbers of the set bytes of mask, written to out (device), count to *count.
I compact_rows(const uint8_t* mask, long long n, long long* out, long long* count) {
    CompactCols cols{};
    cols.src[0] = nullptr; cols.dst[0] = out; cols.es[0] = 0; cols.ncol = 1;
    return compact(mask, n, cols, count);
}

}  // namespace hg

using namespace hg;

extern "C" {

I pfnCompress(V z, V x, V y) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    return compress_one(z, x, y);
}

I pfnWhere(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (x->typ != H_B) return x->typ == H_G ? set_error(E_NOT_IMPL, "where on a list of bools is outside the path") : E_DOMAIN;
    long long n = x->len;
    const void* pm;
    HG_CHECK(in_ptr(x, &pm));
    long long mark = out_mark();
    void* d = n > 1 ? dalloc((size_t)n * 8) : salloc(16);
    if (!d) return E_DEVICE_OOM;
    CompactCols cols{};
    cols.src[0] = nullptr; cols.dst[0] = d; cols.es[0] = 0; cols.ncol = 1;
    long long cnt = 0;
    I e = compact((const uint8_t*)pm, n, cols, &cnt);
    if (e) { out_rewind(mark); return e; }
    z->typ = H_L;
    z->len = cnt;
    if (cnt <= 1) {
        z->g = (G)&z->b;
        z->i64 = 0;
        if (cnt == 1) HG_CU(cudaMemcpyAsync(&z->b, d, 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaStreamSynchronize(g_stream));
        out_rewind(mark);
        return apply_residency(z);
    }
    dshrink(d, (size_t)cnt * 8);
    z->g = (G)d;
    register_bound(d, cnt, n);
    return apply_residency(z);
}

// Multi-column compress sharing one mask (pattern.cc:452-520, genPatternCompress):
// one pass over the mask writes every output column.
I hgpuCompressMany(V* z, V x, V* y, L n) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (x->typ != H_B) return E_DOMAIN;
    if (n < 1) return 0;
    for (L k = 0; k < n; k++) {
        if (y[k]->len != x->len) return E_LENGTH;
        if (!compress_type_ok(y[k]->typ)) return E_NOT_IMPL;
    }
    for (L k0 = 0; k0 < n; k0 += CT_MAXCOL) {
        L kn = (n - k0) < CT_MAXCOL ? (n - k0) : CT_MAXCOL;
        long long rows = x->len;
        const void* pm;
        HG_CHECK(in_ptr(x, &pm));
        CompactCols cols{};
        cols.ncol = (int)kn;
        for (L k = 0; k < kn; k++) {
            const void* pv;
            HG_CHECK(in_ptr(y[k0 + k], &pv));
            cols.src[k] = pv;
            cols.es[k] = esize(y[k0 + k]->typ);
            cols.dst[k] = salloc((size_t)(rows > 0 ? rows : 1) * cols.es[k]);
            if (!cols.dst[k]) return E_DEVICE_OOM;
        }
        long long cnt = 0;
        HG_CHECK(compact((const uint8_t*)pm, rows, cols, &cnt));
        for (L k = 0; k < kn; k++) {
            V zk = z[k0 + k], yk = y[k0 + k];
            if (cnt == rows && rows > 0) { *zk = *yk; if (is_inline(yk)) zk->g = (G)&zk->b; continue; }
            void* dz;
            HG_CHECK(alloc_out(zk, yk->typ, cnt, &dz));
            if (cnt > 0) HG_CU(cudaMemcpyAsync(dz, cols.dst[k], (size_t)cnt * cols.es[k], cudaMemcpyDeviceToDevice, g_stream));
            HG_CHECK(finish_out(zk, dz));
        }
    }
    return 0;
}

}  // extern "C"
