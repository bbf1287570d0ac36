// Stream compaction: @compress, @where and the multi-column compress that
// the pattern pass emits.
//
// Reference: pfnCompress (h_primitive.cc:1479-1521) counts the selected rows
// per OpenMP thread (getNumOfNonZero, h_system.cc:304-310), scans the counts
// and scatters in a second pass; the result is stable, and when every row is
// selected the output aliases the input (copyV, :1513-1515).  pfnWhere
// (:728-762) does the same writing i64 row numbers.
//
// GB300 kernels: a tile is 4096 rows handled by 8 warps; each lane reads its
// 16 mask bytes with one 128-bit load and counts them with popc.  A count
// pass writes the tiles' counts, one block scans them, and a scatter pass
// re-reads the mask (1 byte a row) and writes each tile's selected rows from
// its offset: each warp walks its 512 rows in rounds of 32, and selected
// lanes write to consecutive positions found with ballot/popc.  Values are
// only read for selected rows, so a sparse mask reads a fraction of the
// value column.
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

// A lane's 16 mask bytes (rows base+lofs .. +15), as 0/1 bytes
__device__ __forceinline__ uint4 load_mask16(const uint8_t* __restrict__ mask, long long n, long long base, int lofs) {
    if (base + lofs + 16 <= n && ((reinterpret_cast<uintptr_t>(mask + base + lofs) & 15) == 0))
        return __ldcs(reinterpret_cast<const uint4*>(mask + base + lofs));
    uint8_t b[16];
#pragma unroll
    for (int k = 0; k < 16; k++) b[k] = (base + lofs + k < n) ? (mask[base + lofs + k] != 0) : 0;
    return *reinterpret_cast<uint4*>(b);
}

// pass 1: selected rows per 4096-row tile
__global__ void __launch_bounds__(CT_THREADS) k_compact_count(const uint8_t* __restrict__ mask, long long n,
                                                              unsigned* __restrict__ counts) {
    __shared__ unsigned warp_tot[8];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * CT_TILE;
    const uint4 m4 = load_mask16(mask, n, base, (int)threadIdx.x * 16);
    unsigned c = warp_sum(__popc(m4.x) + __popc(m4.y) + __popc(m4.z) + __popc(m4.w));
    if (lane == 0) warp_tot[warp] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < 8; w++) t += warp_tot[w];
        counts[blockIdx.x] = t;
    }
}

// exclusive scan of the tile counts in one block (tiles are 4096 rows, so
// even 2^31 rows make only 2^19 counts); out[ntiles] = total
__global__ void __launch_bounds__(1024) k_scan_counts(const unsigned* __restrict__ in, long long n,
                                                      unsigned long long* __restrict__ out) {
    // Rounds of 8192 counts, element k * 1024 + t of a round held by thread
    // t, so that every load and store of a warp covers 32 consecutive
    // counts.  The round's order is k-major: the exclusive prefix of element
    // (k, warp, lane) = the totals of all (k', warp') before it + the warp's
    // own inclusive scan.
    constexpr int PER = 8;
    __shared__ unsigned long long part[PER * 32];  // total of each (k, warp), then its exclusive prefix
    __shared__ unsigned long long wtot[PER];
    __shared__ unsigned long long carry;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long c0 = 0; c0 < n; c0 += 1024 * PER) {
        unsigned long long v[PER], incl[PER];
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const long long i = c0 + (long long)k * 1024 + threadIdx.x;
            v[k] = i < n ? in[i] : 0u;
        }
#pragma unroll
        for (int k = 0; k < PER; k++) {
            incl[k] = warp_incl_scan64(v[k]);
            if (lane == 31) part[k * 32 + warp] = incl[k];
        }
        __syncthreads();
        // scan of the 256 (k, warp) totals in k-major order by the first 8 warps
        unsigned long long x = 0, xi = 0;
        if (threadIdx.x < PER * 32) {
            x = part[threadIdx.x];
            xi = warp_incl_scan64(x);
            if (lane == 31) wtot[warp] = xi;
        }
        __syncthreads();
        if (threadIdx.x < PER * 32) {
            unsigned long long before = 0;
            for (unsigned w = 0; w < warp; w++) before += wtot[w];
            part[threadIdx.x] = before + xi - x;
        }
        __syncthreads();
        const unsigned long long base = carry;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const long long i = c0 + (long long)k * 1024 + threadIdx.x;
            if (i < n) out[i] = base + part[k * 32 + warp] + incl[k] - v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int w = 0; w < PER; w++) t += wtot[w];
            carry = base + t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

// offs[0..n) = exclusive prefix of counts[0..n), offs[n] = total (device)
I scan_counts(const unsigned* counts, long long n, unsigned long long* offs) {
    HG_LAUNCH("counts_scan", 1, 1024, 0, k_scan_counts, counts, n, offs);
    return last_launch_error();
}

// pass 2: each tile writes its selected rows from its known offset; each warp
// walks its 512 rows in rounds of 32 and selected lanes write to consecutive
// positions found with ballot/popc
// One column of a warp's 512 rows: the values of the lane's selected rows in
// all 16 rounds are loaded before the first store (the stores could alias
// the source as far as the compiler knows, so loads and stores interleaved
// round by round would wait one memory latency per round).
template <typename E>
__device__ __forceinline__ void scatter_col(const void* __restrict__ src, void* __restrict__ dst, unsigned selbits,
                                            long long rowbase, unsigned long long off) {
    const unsigned lane = lane_id();
    E v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const long long i = rowbase + k * 32 + lane;
        if constexpr (sizeof(E) == 8 && std::is_signed<E>::value) v[k] = (E)i;  // @where: the row number
        else v[k] = ((selbits >> k) & 1u) ? reinterpret_cast<const E*>(src)[i] : E(0);
    }
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const bool sel = (selbits >> k) & 1u;
        const unsigned bal = __ballot_sync(0xffffffffu, sel);
        if (sel) reinterpret_cast<E*>(dst)[off + __popc(bal & lanemask_lt())] = v[k];
        off += __popc(bal);
    }
}

__global__ void __launch_bounds__(CT_THREADS) k_compact_scatter(const uint8_t* __restrict__ mask, long long n,
                                                                CompactCols cols,
                                                                const unsigned long long* __restrict__ offs) {
    __shared__ __align__(16) uint8_t smask[CT_TILE];
    __shared__ unsigned warp_tot[8];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * CT_TILE;
    const int lofs = (int)threadIdx.x * 16;
    const uint4 m4 = load_mask16(mask, n, base, lofs);
    *reinterpret_cast<uint4*>(smask + lofs) = m4;
    unsigned c = warp_sum(__popc(m4.x) + __popc(m4.y) + __popc(m4.z) + __popc(m4.w));
    if (lane == 0) warp_tot[warp] = c;
    __syncthreads();
    unsigned long long off = offs[blockIdx.x];
    for (unsigned w = 0; w < warp; w++) off += warp_tot[w];
    const int wbase = (int)warp * 512;
    unsigned selbits = 0;  // bit k: row wbase + 32 k + lane is selected
#pragma unroll
    for (int k = 0; k < 16; k++) selbits |= (smask[wbase + k * 32 + (int)lane] != 0 ? 1u : 0u) << k;
    const long long rowbase = base + wbase;
    for (int c2 = 0; c2 < cols.ncol; c2++) {
        switch (cols.es[c2]) {
        case 1: scatter_col<uint8_t>(cols.src[c2], cols.dst[c2], selbits, rowbase, off); break;
        case 2: scatter_col<uint16_t>(cols.src[c2], cols.dst[c2], selbits, rowbase, off); break;
        case 4: scatter_col<uint32_t>(cols.src[c2], cols.dst[c2], selbits, rowbase, off); break;
        case 8: scatter_col<unsigned long long>(cols.src[c2], cols.dst[c2], selbits, rowbase, off); break;
        default: scatter_col<long long>(cols.src[c2], cols.dst[c2], selbits, rowbase, off); break;
        }
    }
}

// Single-column scatter with the element size fixed at compile time (ES = 0:
// the row number as i64, for @where; the only instance launched).  The
// tile's kept values are staged in shared memory in output order, then
// written out by consecutive threads to consecutive addresses, so every
// output line is written whole.
template <int ES>
__global__ void __launch_bounds__(CT_THREADS) k_compact_scatter1(const uint8_t* __restrict__ mask, long long n,
                                                                 const void* __restrict__ src, void* __restrict__ dst,
                                                                 const unsigned long long* __restrict__ offs) {
    using E = typename std::conditional<ES == 1, uint8_t,
              typename std::conditional<ES == 2, uint16_t,
              typename std::conditional<ES == 4, uint32_t, unsigned long long>::type>::type>::type;
    __shared__ __align__(16) uint8_t smask[CT_TILE];
    __shared__ __align__(16) E sbuf[CT_TILE];
    __shared__ unsigned warp_tot[8];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * CT_TILE;
    const int lofs = (int)threadIdx.x * 16;
    const uint4 m4 = load_mask16(mask, n, base, lofs);
    *reinterpret_cast<uint4*>(smask + lofs) = m4;
    unsigned c = warp_sum(__popc(m4.x) + __popc(m4.y) + __popc(m4.z) + __popc(m4.w));
    if (lane == 0) warp_tot[warp] = c;
    __syncthreads();
    unsigned loc = 0, total = 0;
    for (unsigned w = 0; w < 8; w++) {
        if (w < warp) loc += warp_tot[w];
        total += warp_tot[w];
    }
    const int wbase = (int)warp * 512;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int li = wbase + k * 32 + (int)lane;
        const bool sel = smask[li] != 0;
        const unsigned bal = __ballot_sync(0xffffffffu, sel);
        if (sel) {
            const unsigned o = loc + __popc(bal & lanemask_lt());
            if constexpr (ES == 0) sbuf[o] = (unsigned long long)(base + li);
            else sbuf[o] = reinterpret_cast<const E*>(src)[base + li];
        }
        loc += __popc(bal);
    }
    __syncthreads();
    E* out = reinterpret_cast<E*>(dst) + offs[blockIdx.x];
    for (unsigned k = threadIdx.x; k < total; k += CT_THREADS) out[k] = sbuf[k];
}

// Compaction in two passes with no dependence between tiles: count per
// tile, scan the counts, scatter.  (A single pass with a decoupled look-back
// across tiles measured several times slower here: the tiles waited on the
// look-back chain rather than on memory.)  *count receives the number of
// selected rows.
static I compact(const uint8_t* mask, long long n, CompactCols& cols, long long* count) {
    long long ntiles = (n + CT_TILE - 1) / CT_TILE;
    if (ntiles == 0) { *count = 0; return 0; }
    unsigned* counts = (unsigned*)salloc(ntiles * 4);
    unsigned long long* offs = (unsigned long long*)salloc((ntiles + 1) * 8);
    if (!counts || !offs) return E_DEVICE_OOM;
    HG_LAUNCH("compact_count", (unsigned)ntiles, CT_THREADS, 0, k_compact_count, mask, n, counts);
    HG_LAUNCH("compact_scan", 1, 1024, 0, k_scan_counts, counts, ntiles, offs);
    if (cols.ncol == 1 && cols.es[0] == 0) {  // @where: staged row numbers (measured 0.094 -> 0.074 ms at 60M)
        HG_LAUNCH("compact", (unsigned)ntiles, CT_THREADS, 0, k_compact_scatter1<0>, mask, n, cols.src[0], cols.dst[0], offs);
    } else {  // value columns: direct stores measured faster than staging for 8-byte values
        HG_LAUNCH("compact", (unsigned)ntiles, CT_THREADS, 0, k_compact_scatter, mask, n, cols, offs);
    }
    HG_CHECK(last_launch_error());
    unsigned long long h = 0;
    HG_CHECK(rb_queue(&h, offs + ntiles, 8));
    HG_CHECK(check_device_errors());  // synchronises
    *count = (long long)h;
    return 0;
}

// i64 columns compacted by one mask (the multi-column join's pair filter);
// dst[c] must hold n rows, *count receives the rows kept
I compact_i64_cols(const uint8_t* mask, long long n, const long long* const* src, long long** dst, int ncol,
                   long long* count) {
    CompactCols cols{};
    cols.ncol = ncol;
    for (int c = 0; c < ncol; c++) { cols.src[c] = src[c]; cols.dst[c] = dst[c]; cols.es[c] = 8; }
    return compact(mask, n, cols, count);
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
    // the reference stops the process on an enum here (TODO at h_primitive.cc:1492-1494)
    if (y->typ == H_Y) return set_error(E_NOT_IMPL, "compress of an enum");
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
        if (cnt == 1) HG_CHECK(rb_queue(&z->b, tmp, es));
        HG_CU(stream_sync());
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
        if (cnt == 1) HG_CHECK(rb_queue(&z->b, d, 8));
        HG_CU(stream_sync());
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
