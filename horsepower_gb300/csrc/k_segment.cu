// Segmented aggregation: the interpreter chain
//     raze(each(@sum|@avg|@min|@max|@len, each_right(@index, x, groups)))
// (h_primitive.cc:1818-1904 each/each_right, :935-955 raze, per-group
// pfnIndex :43-94 and pfnSum/pfnAvg/pfnReduce/pfnLen :656-847) and its fused
// form, the peephole functions of the pattern pass (optimizer/pattern.cc:
// 63-105 FP1/2/5/6/7, emitter :180-219), exported as hgpuGroupSum & co.
//
// Per-group semantics follow the interpreter (ints sum in i64, avg in f64,
// min/max keep the type, empty groups give the pfnReduce sentinels).  Every
// group is reduced with the fixed-order tile tree of dev_common.cuh, so the
// chain and the fused entry points are bit-identical to each other and to a
// plain @sum of the gathered vector.
//
// GB300 layout: the rows of all groups are one device array with group
// starts (the @group output), so a group is a contiguous segment.  Groups of
// up to 4096 rows are reduced by one warp each; longer groups are split into
// 4096-row chunks reduced by one CTA each, and their chunk partials are
// reduced again the same way.
#include <limits>
#include <vector>

#include "dev_common.cuh"

namespace hg {

I scan_exclusive(const unsigned* in, long long n, unsigned long long* out, unsigned long long* total_h);
I compact_rows(const uint8_t* mask, long long n, long long* out, long long* count);

enum { AG_SUM = 0, AG_AVG = 1, AG_MIN = 2, AG_MAX = 3, AG_LEN = 4 };
enum { OP_SUM = 0, OP_MIN = 1, OP_MAX = 2 };

template <typename A, int OP>
__device__ __forceinline__ A sop(A a, A b) {
    if constexpr (OP == OP_SUM) {
        if constexpr (std::is_same<A, double>::value) return __dadd_rn(a, b);
        else if constexpr (std::is_same<A, float>::value) return __fadd_rn(a, b);
        else return (A)((unsigned long long)a + (unsigned long long)b);
    } else if constexpr (OP == OP_MIN) return (a < b) ? a : b;
    else return (a > b) ? a : b;
}
template <typename A, int OP>
__device__ __forceinline__ A swarp(A v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = sop<A, OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// element j of segment [s, e): x[rows[s+j]] (gather) or vals[s+j]
template <typename T, bool GATHER>
__device__ __forceinline__ T seg_elem(const T* __restrict__ src, const long long* __restrict__ rows, long long nx,
                                      long long k, bool& bad) {
    if constexpr (GATHER) {
        long long r = rows[k];
        if (r < 0 || r >= nx) { bad = true; return T(0); }
        return src[r];
    } else {
        return src[k];
    }
}

// The 16 elements k * 256 + (first - k * 256 ...) of one lane of a 256-lane
// tile: positions first + k * 256, k = 0..15, those below `end` loaded (row
// numbers first, then the values, so all 16 gathers are in flight together).
template <typename T, bool GATHER>
__device__ __forceinline__ void seg_load16(const T* __restrict__ src, const long long* __restrict__ rows, long long nx,
                                           long long first, long long end, T v[16], bool& bad) {
    if constexpr (GATHER) {
        long long r[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const long long j = first + (long long)k * 256;
            r[k] = j < end ? rows[j] : 0;
        }
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const bool in = first + (long long)k * 256 < end;
            const bool ok = r[k] >= 0 && r[k] < nx;
            bad |= in && !ok;
            v[k] = (in && ok) ? src[r[k]] : T(0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const long long j = first + (long long)k * 256;
            v[k] = j < end ? src[j] : T(0);
        }
    }
}

// Segments by size class, so that each is reduced by the narrowest unit that
// reproduces the tile tree exactly: sizes 0-1, 2, 3-4, 5-8, 9-16, 17-32
// (classes 0-5), 33-4096 (6) and longer (7).
constexpr int SEG_CLASSES = 8;
static_assert(SEG_PLAN_HDR_BYTES == (SEG_CLASSES + 2) * 8, "plan header layout");
__device__ __forceinline__ int seg_class(long long m) {
    if (m <= 1) return 0;
    if (m > TILE_SUM) return 7;
    if (m > 32) return 6;
    return 32 - __clz((int)(m - 1));  // ceil(log2 m): 2 -> 1, 3-4 -> 2, ..., 17-32 -> 5
}
// pass 1: segments per class (cnt[c])
__global__ void k_seg_class_count(const long long* __restrict__ starts, long long ng, long long total,
                                  unsigned* __restrict__ cnt) {
    __shared__ unsigned sc[SEG_CLASSES];
    if (threadIdx.x < SEG_CLASSES) sc[threadIdx.x] = 0;
    __syncthreads();
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g < ng) atomicAdd(&sc[seg_class(((g + 1 < ng) ? starts[g + 1] : total) - starts[g])], 1u);
    __syncthreads();
    if (threadIdx.x < SEG_CLASSES && sc[threadIdx.x]) atomicAdd(&cnt[threadIdx.x], sc[threadIdx.x]);
}
// pass 2: the segment ids of class c at ids[off_c ...] (off_c = segments of
// lower classes; order inside a class is immaterial); cur[c] counts the
// places taken
__global__ void k_seg_class_ids(const long long* __restrict__ starts, long long ng, long long total,
                                const unsigned* __restrict__ cnt, unsigned* __restrict__ cur,
                                unsigned* __restrict__ ids) {
    __shared__ unsigned sc[SEG_CLASSES], sbase[SEG_CLASSES];
    if (threadIdx.x < SEG_CLASSES) sc[threadIdx.x] = 0;
    __syncthreads();
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int c = 0;
    unsigned local = 0;
    if (g < ng) {
        c = seg_class(((g + 1 < ng) ? starts[g + 1] : total) - starts[g]);
        local = atomicAdd(&sc[c], 1u);
    }
    __syncthreads();
    if (threadIdx.x < SEG_CLASSES) {
        unsigned off = 0;
        for (int k = 0; k < (int)threadIdx.x; k++) off += cnt[k];
        sbase[threadIdx.x] = sc[threadIdx.x] ? off + atomicAdd(&cur[threadIdx.x], sc[threadIdx.x]) : 0;
    }
    __syncthreads();
    if (g < ng) ids[sbase[c] + local] = (unsigned)g;
}

// Segments of classes 0-5 in one launch.  Class c (at most P = 2^c
// elements): the segment's elements sit in lanes 0..m-1 of warp 0 of the
// 256-lane tile and every other lane and warp holds the identity, so the
// tile tree reduces to the xor butterfly over the first P lanes; a warp
// reduces 32 / P such segments in sub-warps of P lanes.
template <typename T, typename A, int OP, bool GATHER>
__global__ void __launch_bounds__(256) k_seg_warps(const T* __restrict__ src, const long long* __restrict__ rows,
                                                   long long nx, const long long* __restrict__ starts, long long ng,
                                                   long long total, const unsigned* __restrict__ ids,
                                                   const unsigned* __restrict__ cnt, A ident, A* __restrict__ out,
                                                   unsigned* derr) {
    __shared__ long long wfirst[7];  // first warp of each class 0-5; wfirst[6] = warps in all
    __shared__ unsigned cfirst[6];   // first id of each class
    if (threadIdx.x == 0) {
        long long w = 0;
        unsigned o = 0;
        for (int c = 0; c < 6; c++) {
            wfirst[c] = w;
            cfirst[c] = o;
            const long long per = 32 >> c;  // segments per warp
            w += ((long long)cnt[c] + per - 1) / per;
            o += cnt[c];
        }
        wfirst[6] = w;
    }
    __syncthreads();
    const unsigned lane = lane_id();
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    bool bad = false;
    for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < wfirst[6]; w += warps) {
        int c = 0;
        while (c < 5 && w >= wfirst[c + 1]) c++;
        const int P = 1 << c;
        const unsigned q = lane >> c, j = lane & (P - 1);
        const long long k = (w - wfirst[c]) * (32 >> c) + q;
        A acc = ident;
        long long g = -1;
        if (k < (long long)cnt[c]) {
            g = ids[cfirst[c] + k];
            const long long s = starts[g], e = (g + 1 < ng) ? starts[g + 1] : total;
            if ((long long)j < e - s) acc = sop<A, OP>(ident, (A)seg_elem<T, GATHER>(src, rows, nx, s + j, bad));
        }
        for (int o = P >> 1; o > 0; o >>= 1) acc = sop<A, OP>(acc, __shfl_xor_sync(0xffffffffu, acc, o));
        if (j == 0 && g >= 0) out[g] = acc;
    }
    if (bad) flag_error(derr, DERR_INDEX);
}

// Class 6 (33 to 4096 elements): one warp per segment walks the tile's 8
// virtual warps, each lane's 16 elements loaded before they are added in order.
template <typename T, typename A, int OP, bool GATHER>
__global__ void __launch_bounds__(256) k_seg_mid(const T* __restrict__ src, const long long* __restrict__ rows,
                                                 long long nx, const long long* __restrict__ starts, long long ng,
                                                 long long total, const unsigned* __restrict__ ids,
                                                 const unsigned* __restrict__ cnt, A ident, A* __restrict__ out,
                                                 unsigned* derr) {
    __shared__ unsigned first;
    if (threadIdx.x == 0) {
        unsigned o = 0;
        for (int c = 0; c < 6; c++) o += cnt[c];
        first = o;
    }
    __syncthreads();
    const long long n6 = cnt[6];
    const unsigned lane = lane_id();
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    bool bad = false;
    for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n6; w += warps) {
        const long long g = ids[first + w];
        const long long s = starts[g], e = (g + 1 < ng) ? starts[g + 1] : total, m = e - s;
        A ws[8];
#pragma unroll
        for (int v = 0; v < 8; v++) ws[v] = ident;
        for (int v = 0; v < 8 && v * 32 < m; v++) {  // virtual warp v of the 256-lane tile
            T x[16];
            seg_load16<T, GATHER>(src, rows, nx, s + v * 32 + lane, e, x, bad);
            A acc = ident;
#pragma unroll
            for (int k = 0; k < 16; k++)
                if ((long long)k * 256 + v * 32 + lane < m) acc = sop<A, OP>(acc, (A)x[k]);
            ws[v] = swarp<A, OP>(acc);
        }
        if (lane == 0) {
            A w01 = sop<A, OP>(ws[0], ws[1]), w23 = sop<A, OP>(ws[2], ws[3]);
            A w45 = sop<A, OP>(ws[4], ws[5]), w67 = sop<A, OP>(ws[6], ws[7]);
            out[g] = sop<A, OP>(sop<A, OP>(w01, w23), sop<A, OP>(w45, w67));
        }
    }
    if (bad) flag_error(derr, DERR_INDEX);
}

// The chunk partials of the long segments, one CTA per segment of at most
// 4096 partials (the caller checks): thread t holds partials t, t + 256, ...
// exactly as the tile tree places them (the order k_seg_mid's virtual warps
// follow, whatever size class would have scheduled the segment); the result
// goes straight to the segment's slot of out.
template <typename A, int OP>
__global__ void __launch_bounds__(256) k_seg_partials(const A* __restrict__ part, const long long* __restrict__ pstarts,
                                                      const long long* __restrict__ big, long long nbig,
                                                      long long nchunks, A ident, A* __restrict__ out) {
    __shared__ A ws[8];
    const long long g = blockIdx.x;
    const long long s = pstarts[g], e = (g + 1 < nbig) ? pstarts[g + 1] : nchunks;
    bool bad = false;
    A v[16];
    seg_load16<A, false>(part, nullptr, 0, s + threadIdx.x, e, v, bad);
    A acc = ident;
#pragma unroll
    for (int k = 0; k < 16; k++)
        if (s + k * 256 + threadIdx.x < e) acc = sop<A, OP>(acc, v[k]);
    acc = swarp<A, OP>(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        A w01 = sop<A, OP>(ws[0], ws[1]), w23 = sop<A, OP>(ws[2], ws[3]);
        A w45 = sop<A, OP>(ws[4], ws[5]), w67 = sop<A, OP>(ws[6], ws[7]);
        out[big[g]] = sop<A, OP>(sop<A, OP>(w01, w23), sop<A, OP>(w45, w67));
    }
}

// The chunk a reduction CTA takes: from its descriptor (one 16-byte load)
// when the chunks run in a planned order, else chunk blockIdx.x, found
// among the long segments by a binary search over their first chunks.
// base = its first element, e = one past its last (at most base + 4096).
__device__ __forceinline__ void chunk_of_block(const ChunkDesc* __restrict__ order, const long long* __restrict__ starts,
                                               long long ng, long long total, const long long* __restrict__ big,
                                               const unsigned long long* __restrict__ chunk0, long long nbig,
                                               long long& c, long long& base, long long& e) {
    if (order) {
        const ChunkDesc d = order[blockIdx.x];
        c = d.chunk;
        base = d.first;
        e = d.first + d.len;
        return;
    }
    c = blockIdx.x;
    long long lo = 0, hi = nbig - 1;  // the long segment owning chunk c
    while (lo < hi) {
        long long mid = (lo + hi + 1) >> 1;
        if ((long long)chunk0[mid] <= c) lo = mid; else hi = mid - 1;
    }
    const long long g = big[lo];
    const long long s = starts[g];
    const long long se = (g + 1 < ng) ? starts[g + 1] : total;
    base = s + (c - (long long)chunk0[lo]) * TILE_SUM;
    e = se < base + TILE_SUM ? se : base + TILE_SUM;
}

// one CTA per 4096-element chunk of the long segments
template <typename T, typename A, int OP, bool GATHER>
__global__ void __launch_bounds__(256) k_seg_chunk(const T* __restrict__ src, const long long* __restrict__ rows,
                                                   long long nx, const long long* __restrict__ starts, long long ng,
                                                   long long total, const long long* __restrict__ big,
                                                   const unsigned long long* __restrict__ chunk0, long long nbig,
                                                   const ChunkDesc* __restrict__ order, A ident, A* __restrict__ part,
                                                   unsigned* derr) {
    __shared__ A ws[8];
    long long c, base, e;
    chunk_of_block(order, starts, ng, total, big, chunk0, nbig, c, base, e);
    bool bad = false;
    T v[16];
    seg_load16<T, GATHER>(src, rows, nx, base + threadIdx.x, e, v, bad);
    A acc = ident;
#pragma unroll
    for (int k = 0; k < 16; k++)
        if (base + k * 256 + threadIdx.x < e) acc = sop<A, OP>(acc, (A)v[k]);
    acc = swarp<A, OP>(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        A w01 = sop<A, OP>(ws[0], ws[1]), w23 = sop<A, OP>(ws[2], ws[3]);
        A w45 = sop<A, OP>(ws[4], ws[5]), w67 = sop<A, OP>(ws[6], ws[7]);
        part[c] = sop<A, OP>(sop<A, OP>(w01, w23), sop<A, OP>(w45, w67));
    }
    if (bad) flag_error(derr, DERR_INDEX);
}

__global__ void k_big_flags(const long long* __restrict__ starts, long long ng, long long total, uint8_t* __restrict__ f,
                            unsigned* __restrict__ nch) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        long long m = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
        f[g] = m > TILE_SUM;
        if (nch) nch[g] = 0;
    }
}
__global__ void k_big_chunks(const long long* __restrict__ starts, long long ng, long long total,
                             const long long* __restrict__ big, long long nbig, unsigned* __restrict__ nch) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nbig; k += (long long)gridDim.x * blockDim.x) {
        long long g = big[k];
        long long m = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
        nch[k] = (unsigned)((m + TILE_SUM - 1) / TILE_SUM);
    }
}
template <typename A>
__global__ void k_scatter_big(const A* __restrict__ r, const long long* __restrict__ big, long long nbig, A* __restrict__ out) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nbig; k += (long long)gridDim.x * blockDim.x)
        out[big[k]] = r[k];
}
// The chunk starts as i64 and, for a few long segments, the order in which
// the chunk CTAs run.  A segment's rows are spread over the whole source
// column, so running one segment's chunks after another's would sweep the
// column once per segment.  Instead chunk (k, c) of long segment k (n_k
// chunks) runs at the rank of its relative position (2c + 1) / (2 n_k), ties
// to the lower k: the CTAs resident together then cover the same region of
// the column in every segment, and a sector fetched for one segment is
// still in L2 when the others reach it.  Only the schedule changes; each
// chunk's partial lands at its own index as before.
// Chunk orders are built for 2..CHUNK_ORDER_MAX_SEGS long segments (each
// chunk's rank costs one step per long segment), by one CTA from shared
// memory for the lists @group plans (at most CHUNK_ORDER_SMALL_SEGS).
constexpr long long CHUNK_ORDER_MAX_SEGS = 2048;
constexpr long long CHUNK_ORDER_SMALL_SEGS = 64;
// below this many elements the values of a list fit in L2 whatever the
// order, and the general plan builds none (it costs a launch's worth of work)
constexpr long long CHUNK_ORDER_MIN_TOTAL = 4ll << 20;
// order[rank of chunk t] = chunk t's descriptor, for chunk t of nchunks (c0:
// the long segments' first chunks; seg_first/seg_end(k): long segment k's
// element range)
template <typename SegRange>
__device__ __forceinline__ void chunk_rank(const unsigned long long* c0, long long nbig, unsigned long long nchunks,
                                           long long t, ChunkDesc* __restrict__ order, SegRange range) {
    long long lo = 0, hi = nbig - 1;  // the long segment owning chunk t
    while (lo < hi) {
        long long mid = (lo + hi + 1) >> 1;
        if ((long long)c0[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const long long k = lo, c = t - (long long)c0[k];
    const long long nk = (long long)((k + 1 < nbig ? c0[k + 1] : nchunks) - c0[k]);
    long long rank = c;
    for (long long k2 = 0; k2 < nbig; k2++) {
        if (k2 == k) continue;
        const long long n2 = (long long)((k2 + 1 < nbig ? c0[k2 + 1] : nchunks) - c0[k2]);
        // chunks c2 of segment k2 placed before (k, c): (2 c2 + 1) n_k < (2c + 1) n2, or equal and k2 < k
        const long long x = (2 * c + 1) * n2 + (k2 < k ? 1 : 0);
        const long long q = x <= 0xffffffffll ? (long long)((unsigned)(x - 1) / (unsigned)nk) : (x - 1) / nk;
        const long long cnt = (q + 1) / 2;
        rank += cnt < n2 ? cnt : n2;
    }
    long long sf, se;
    range(k, sf, se);
    const long long first = sf + c * TILE_SUM;
    const long long len = se - first < TILE_SUM ? se - first : TILE_SUM;
    order[rank] = ChunkDesc{first, (unsigned)len, (unsigned)t};
}
// The general plan: ps = the first chunks as i64 and, with `order`, the
// chunk order of up to CHUNK_ORDER_MAX_SEGS long segments, one warp per chunk
// (the lanes share the walk over the other segments).
__global__ void k_chunk_plan(const unsigned long long* __restrict__ c0, long long nbig, unsigned long long nchunks,
                             const long long* __restrict__ starts, long long ng, long long total,
                             const long long* __restrict__ big, long long* __restrict__ ps,
                             ChunkDesc* __restrict__ order) {
    extern __shared__ unsigned long long sc0[];  // the first chunks, when there is an order to build
    const long long nth = (long long)gridDim.x * blockDim.x;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nbig; t += nth) ps[t] = (long long)c0[t];
    if (!order) return;
    for (long long k = threadIdx.x; k < nbig; k += blockDim.x) sc0[k] = c0[k];
    __syncthreads();
    const unsigned lane = lane_id();
    const long long nwarps = nth >> 5;
    for (long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; t < (long long)nchunks; t += nwarps) {
        long long lo = 0, hi = nbig - 1;  // the long segment owning chunk t
        while (lo < hi) {
            const long long mid = (lo + hi + 1) >> 1;
            if ((long long)sc0[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const long long k = lo, c = t - (long long)sc0[k];
        const long long nk = (long long)((k + 1 < nbig ? sc0[k + 1] : nchunks) - sc0[k]);
        long long part = 0;
        for (long long k2 = lane; k2 < nbig; k2 += 32) {
            if (k2 == k) continue;
            const long long n2 = (long long)((k2 + 1 < nbig ? sc0[k2 + 1] : nchunks) - sc0[k2]);
            // chunks c2 of segment k2 placed before (k, c): (2 c2 + 1) n_k < (2c + 1) n2, or equal and k2 < k
            const long long x = (2 * c + 1) * n2 + (k2 < k ? 1 : 0);
            const long long q = x <= 0xffffffffll ? (long long)((unsigned)(x - 1) / (unsigned)nk) : (x - 1) / nk;
            const long long cnt = (q + 1) / 2;
            part += cnt < n2 ? cnt : n2;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) {
            const long long g = big[k];
            const long long sf = starts[g], se = (g + 1 < ng) ? starts[g + 1] : total;
            const long long first = sf + c * TILE_SUM;
            const long long len = se - first < TILE_SUM ? se - first : TILE_SUM;
            order[c + part] = ChunkDesc{first, (unsigned)len, (unsigned)t};
        }
    }
}

// The whole plan of a list of at most SEG_PLAN_SMALL segments in one CTA of
// 1024 threads (four consecutive segments each): the class counts and ids
// of seg_classes, then the long segments in ascending order with their
// first chunks (an exclusive scan over the threads) and the chunk order.
// hdr = {the 8 class counts, nbig, nchunks}.
__global__ void __launch_bounds__(1024) k_seg_plan_small(const long long* __restrict__ starts, long long ng,
                                                         long long total, unsigned* __restrict__ cc,
                                                         unsigned* __restrict__ ids, long long* __restrict__ big,
                                                         unsigned long long* __restrict__ c0, long long* __restrict__ ps,
                                                         ChunkDesc* __restrict__ order, unsigned long long* __restrict__ hdr) {
    __shared__ unsigned sc[SEG_CLASSES], soff[SEG_CLASSES], scur[SEG_CLASSES];
    __shared__ unsigned wb[32];
    __shared__ unsigned long long wc[32];
    __shared__ unsigned long long s_nbig, s_nch;
    __shared__ unsigned long long sc0[CHUNK_ORDER_SMALL_SEGS];
    __shared__ long long sfirst[CHUNK_ORDER_SMALL_SEGS], send[CHUNK_ORDER_SMALL_SEGS];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t < SEG_CLASSES) { sc[t] = 0; scur[t] = 0; }
    __syncthreads();
    int cls[4];
    long long len[4];
    unsigned nb = 0;
    unsigned long long nc = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const long long g = (long long)t * 4 + k;
        cls[k] = -1;
        len[k] = 0;
        if (g < ng) {
            len[k] = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
            cls[k] = seg_class(len[k]);
            atomicAdd(&sc[cls[k]], 1u);
            if (len[k] > TILE_SUM) { nb++; nc += (unsigned long long)((len[k] + TILE_SUM - 1) / TILE_SUM); }
        }
    }
    // exclusive scan of (nb, nc) over the threads
    unsigned ib = nb;
    unsigned long long ic = nc;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned ob = __shfl_up_sync(0xffffffffu, ib, d);
        const unsigned long long oc = __shfl_up_sync(0xffffffffu, ic, d);
        if (lane >= d) { ib += ob; ic += oc; }
    }
    if (lane == 31) { wb[w] = ib; wc[w] = ic; }
    __syncthreads();
    if (t == 0) {
        unsigned ab = 0;
        unsigned long long ac = 0;
        for (int k = 0; k < 32; k++) {
            const unsigned b = wb[k];
            const unsigned long long c = wc[k];
            wb[k] = ab; wc[k] = ac;
            ab += b; ac += c;
        }
        s_nbig = ab;
        s_nch = ac;
        unsigned off = 0;
        for (int c = 0; c < SEG_CLASSES; c++) {
            soff[c] = off;
            off += sc[c];
            cc[c] = sc[c];
            cc[SEG_CLASSES + c] = sc[c];
            hdr[c] = sc[c];
        }
    }
    __syncthreads();
    unsigned pb = wb[w] + ib - nb;
    unsigned long long pc = wc[w] + ic - nc;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (cls[k] < 0) continue;
        const long long g = (long long)t * 4 + k;
        ids[soff[cls[k]] + atomicAdd(&scur[cls[k]], 1u)] = (unsigned)g;
        if (len[k] > TILE_SUM) {
            big[pb] = g;
            c0[pb] = pc;
            ps[pb] = (long long)pc;
            if (pb < CHUNK_ORDER_SMALL_SEGS) {
                sc0[pb] = pc;
                sfirst[pb] = starts[g];
                send[pb] = starts[g] + len[k];
            }
            pb++;
            pc += (unsigned long long)((len[k] + TILE_SUM - 1) / TILE_SUM);
        }
    }
    __syncthreads();
    const long long nbig = (long long)s_nbig;
    const unsigned long long nchunks = s_nch;
    if (t == 0) { hdr[SEG_CLASSES] = nbig; hdr[SEG_CLASSES + 1] = nchunks; }
    auto range = [&](long long k, long long& f, long long& e) {
        f = sfirst[k];
        e = send[k];
    };
    if (order && nbig > 1 && nbig <= CHUNK_ORDER_SMALL_SEGS)  // the long segments from shared memory
        for (long long q = t; q < (long long)nchunks; q += 1024) chunk_rank(sc0, nbig, nchunks, q, order, range);
}

static unsigned gcap(long long n, int per = 256) {
    unsigned g = grid_for(n, per);
    return g > (unsigned)g_sms * 32 ? (unsigned)g_sms * 32 : g;
}

// Segment ids by size class (kept with the list when there is one, with a
// host copy of the class counts so that empty classes launch nothing).
static I seg_classes(const long long* starts, long long ng, long long total, ListInfo* li, const unsigned** ids,
                     const unsigned** ccnt) {
    if (li && li->cls_ids) {
        *ids = li->cls_ids;
        *ccnt = li->cls_cnt;
        return 0;
    }
    unsigned* cc = (unsigned*)(li ? dalloc(2 * SEG_CLASSES * 4) : salloc(2 * SEG_CLASSES * 4));
    unsigned* id = (unsigned*)(li ? dalloc((size_t)ng * 4) : salloc((size_t)ng * 4));
    if (!cc || !id) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(cc, 0, 2 * SEG_CLASSES * 4, g_stream));
    const unsigned gb = (unsigned)((ng + 255) / 256);
    HG_LAUNCH("seg_class", gb, 256, 0, k_seg_class_count, starts, ng, total, cc);
    HG_LAUNCH("seg_class_ids", gb, 256, 0, k_seg_class_ids, starts, ng, total, (const unsigned*)cc,
              cc + SEG_CLASSES, id);
    *ids = id;
    *ccnt = cc;
    if (li) {
        li->cls_ids = id;
        li->cls_cnt = cc;
        // a list's segments are reduced several times (one aggregate per
        // column): read the class counts once, so empty classes are skipped
        HG_CHECK(rb_queue(li->cls_host, cc, sizeof(li->cls_host)));
        HG_CU(stream_sync());
        li->cls_known = 1;
    }
    return last_launch_error();
}

// The split of the segments longer than one tile into 4096-element chunks:
// big[k] = the k-th long segment, chunk0[k] its first chunk, pstarts[k] the
// same as i64, nchunks in all (kept with the list when there is one).
struct LongPlan {
    long long nbig = 0;
    unsigned long long nchunks = 0;
    const long long* big = nullptr;
    const unsigned long long* c0 = nullptr;
    const long long* pstarts = nullptr;
    const ChunkDesc* order = nullptr;
};
static I seg_plan_long(const long long* starts, long long ng, long long total, ListInfo* li, LongPlan* pl) {
    if (li && li->planned) {
        pl->nbig = li->nbig; pl->nchunks = li->nchunks; pl->big = li->big; pl->c0 = li->chunk0; pl->pstarts = li->pstarts;
        pl->order = li->corder;
        return 0;
    }
    uint8_t* f = (uint8_t*)salloc((size_t)ng);
    long long* bigs = (long long*)(li ? dalloc((size_t)ng * 8) : salloc((size_t)ng * 8));
    if (!f || !bigs) return E_DEVICE_OOM;
    HG_LAUNCH("seg_flags", gcap(ng), 256, 0, k_big_flags, starts, ng, total, f, (unsigned*)nullptr);
    long long nbig = 0;
    unsigned long long nchunks = 0;
    HG_CHECK(compact_rows(f, ng, bigs, &nbig));
    unsigned* nch = (unsigned*)salloc((size_t)(nbig > 0 ? nbig : 1) * 4);
    unsigned long long* c0s = (unsigned long long*)(li ? dalloc((size_t)(nbig > 0 ? nbig : 1) * 8) : salloc((size_t)(nbig > 0 ? nbig : 1) * 8));
    long long* ps = (long long*)(li ? dalloc((size_t)(nbig > 0 ? nbig : 1) * 8) : salloc((size_t)(nbig > 0 ? nbig : 1) * 8));
    if (!nch || !c0s || !ps) return E_DEVICE_OOM;
    ChunkDesc* order = nullptr;
    if (nbig > 0) {
        HG_LAUNCH("seg_chunks", gcap(nbig), 256, 0, k_big_chunks, starts, ng, total, bigs, nbig, nch);
        HG_CHECK(scan_exclusive(nch, nbig, c0s, &nchunks));
        if (nbig > 1 && nbig <= CHUNK_ORDER_MAX_SEGS && total >= CHUNK_ORDER_MIN_TOTAL) {
            const size_t ob = (size_t)nchunks * sizeof(ChunkDesc);
            order = (ChunkDesc*)(li ? dalloc(ob) : salloc(ob));
            if (!order) return E_DEVICE_OOM;
        }
        const long long nt = nbig > (long long)nchunks ? nbig : (long long)nchunks;
        const size_t csm = order ? (size_t)nbig * 8 : 0;  // at most 16 KB
        const long long nthreads = order ? (long long)nchunks * 32 : nt;  // a warp per chunk for the order
        HG_LAUNCH("chunk_plan", gcap(nthreads), 256, csm, k_chunk_plan, c0s, nbig, nchunks, starts, ng, total, bigs, ps,
                  order);
    }
    pl->nbig = nbig; pl->nchunks = nchunks; pl->big = bigs; pl->c0 = c0s; pl->pstarts = ps; pl->order = order;
    if (li) {
        li->planned = 1; li->nbig = nbig; li->nchunks = nchunks; li->big = bigs; li->chunk0 = c0s; li->pstarts = ps;
        li->corder = order;
    }
    return last_launch_error();
}

I seg_plan_small(const long long* starts, long long ng, long long total, SmallPlan* p) {
    *p = SmallPlan{};
    if (ng <= 0 || ng > SEG_PLAN_SMALL) return 0;
    const size_t maxch = (size_t)(total / TILE_SUM) + (size_t)ng + 1;
    p->cc = (unsigned*)dalloc(2 * SEG_CLASSES * 4);
    p->ids = (unsigned*)dalloc((size_t)ng * 4);
    p->big = (long long*)dalloc((size_t)ng * 8);
    p->c0 = (unsigned long long*)dalloc((size_t)ng * 8);
    p->ps = (long long*)dalloc((size_t)ng * 8);
    p->order = ng > 1 ? (ChunkDesc*)dalloc(maxch * sizeof(ChunkDesc)) : nullptr;
    unsigned long long* hd = (unsigned long long*)salloc(16 * 8);
    p->hdr = (unsigned long long*)halloc(16 * 8);
    if (p->hdr) memset(p->hdr, 0, 16 * 8);
    if (!p->cc || !p->ids || !p->big || !p->c0 || !p->ps || (ng > 1 && !p->order) || !hd || !p->hdr) {
        *p = SmallPlan{};
        return E_DEVICE_OOM;
    }
    HG_LAUNCH("seg_plan_small", 1, 1024, 0, k_seg_plan_small, starts, ng, total, p->cc, p->ids, p->big, p->c0, p->ps,
              p->order, hd);
    p->hdr_dev = hd;
    return last_launch_error();
}

void seg_plan_adopt(ListInfo& li, const SmallPlan& p) {
    if (!p.hdr) return;
    li.cls_ids = p.ids;
    li.cls_cnt = p.cc;
    for (int c = 0; c < SEG_CLASSES; c++) li.cls_host[c] = (unsigned)p.hdr[c];
    li.cls_known = 1;
    li.planned = 1;
    li.nbig = (long long)p.hdr[SEG_CLASSES];
    li.nchunks = p.hdr[SEG_CLASSES + 1];
    li.big = p.big;
    li.chunk0 = p.c0;
    li.pstarts = p.ps;
    li.corder = (li.nbig > 1 && li.nbig <= CHUNK_ORDER_SMALL_SEGS) ? p.order : nullptr;
}

// Reduces every segment of (src via rows | src) into out[ng] (device).  When
// `li` is given, the split of the long segments is computed once per list
// and kept with it.
template <typename T, typename A, int OP, bool GATHER>
static I seg_reduce(const T* src, const long long* rows, long long nx, const long long* starts, long long ng,
                    long long total, A ident, A* out, ListInfo* li = nullptr) {
    if (ng == 0) return 0;
    const unsigned *ids, *ccnt;
    HG_CHECK(seg_classes(starts, ng, total, li, &ids, &ccnt));
    const bool known = li && li->cls_known;
    bool small = true, mid = true;
    if (known) {
        small = false;
        for (int c = 0; c < 6; c++) small = small || li->cls_host[c] != 0;
        mid = li->cls_host[6] != 0;
    }
    if (small)
        HG_LAUNCH("seg_warps", gcap(ng * 4), 256, 0, (k_seg_warps<T, A, OP, GATHER>), src, rows, nx, starts, ng, total,
                  ids, ccnt, ident, out, g_derr);
    if (mid)
        HG_LAUNCH("seg_mid", gcap(ng), 256, 0, (k_seg_mid<T, A, OP, GATHER>), src, rows, nx, starts, ng, total, ids,
                  ccnt, ident, out, g_derr);
    if (known && li->cls_host[7] == 0) return last_launch_error();
    LongPlan pl;
    HG_CHECK(seg_plan_long(starts, ng, total, li, &pl));
    const long long nbig = pl.nbig;
    const unsigned long long nchunks = pl.nchunks;
    if (nbig == 0) return last_launch_error();
    A* part = (A*)salloc((size_t)nchunks * sizeof(A));
    A* res = (A*)salloc((size_t)nbig * sizeof(A));
    if (!part || !res) return E_DEVICE_OOM;
    HG_LAUNCH("seg_chunk", (unsigned)nchunks, 256, 0, (k_seg_chunk<T, A, OP, GATHER>), src, rows, nx, starts, ng,
              total, pl.big, pl.c0, nbig, pl.order, ident, part, g_derr);
    // partials of each long segment are reduced by the same procedure: at
    // most 4096 of them per segment (certain when there are at most 4096 in
    // all) in one launch straight into out, else as segments of their own
    if (nchunks <= (unsigned long long)TILE_SUM) {
        HG_LAUNCH("seg_partials", (unsigned)nbig, 256, 0, (k_seg_partials<A, OP>), part, pl.pstarts, pl.big, nbig,
                  (long long)nchunks, ident, out);
        return last_launch_error();
    }
    HG_CHECK((seg_reduce<A, A, OP, false>(part, nullptr, 0, pl.pstarts, nbig, (long long)nchunks, ident, res)));
    HG_LAUNCH("scatter_big", gcap(nbig), 256, 0, k_scatter_big<A>, res, pl.big, nbig, out);
    return last_launch_error();
}

// ---- several f64 sums over the long segments of one grouping at once.
// One CTA per 4096-element chunk, as k_seg_chunk, but the chunk's row ids
// are read once and each of the ncol columns is gathered through them (all
// 16 x ncol gathers of a lane issued before the first add); each column's
// chunk partial follows the tile tree, so part[col * nchunks + c] is
// bit-identical to k_seg_chunk's for that column.
constexpr int SEG_MANY = 4;
struct SegCols { const double* src[SEG_MANY]; };
template <int NCOL>
__global__ void __launch_bounds__(256) k_seg_chunk_many(SegCols cols, int ncol, const long long* __restrict__ rows,
                                                        long long nx, const long long* __restrict__ starts, long long ng,
                                                        long long total, const long long* __restrict__ big,
                                                        const unsigned long long* __restrict__ chunk0, long long nbig,
                                                        unsigned long long nchunks, const ChunkDesc* __restrict__ order,
                                                        double* __restrict__ part, unsigned* derr) {
    __shared__ double ws[SEG_MANY][8];
    long long c, base, e;
    chunk_of_block(order, starts, ng, total, big, chunk0, nbig, c, base, e);
    const long long first = base + threadIdx.x;
    long long r[16];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const long long j = first + (long long)k * 256;
        r[k] = j < e ? rows[j] : -1;
        bad |= j < e && (r[k] < 0 || r[k] >= nx);
    }
#pragma unroll 1
    for (int q = 0; q < NCOL; q++) {  // one column at a time: 16 gathers in flight, few registers
        double v[16];
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = (r[k] >= 0 && r[k] < nx) ? cols.src[q][r[k]] : 0.0;
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (first + (long long)k * 256 < e) acc = __dadd_rn(acc, v[k]);
        acc = swarp<double, OP_SUM>(acc);
        if ((threadIdx.x & 31) == 0) ws[q][threadIdx.x >> 5] = acc;
    }
    __syncthreads();
    if (threadIdx.x < (unsigned)NCOL) {
        const double* w = ws[threadIdx.x];
        const double w01 = __dadd_rn(w[0], w[1]), w23 = __dadd_rn(w[2], w[3]);
        const double w45 = __dadd_rn(w[4], w[5]), w67 = __dadd_rn(w[6], w[7]);
        part[(unsigned long long)threadIdx.x * nchunks + c] = __dadd_rn(__dadd_rn(w01, w23), __dadd_rn(w45, w67));
    }
    if (bad) flag_error(derr, DERR_INDEX);
}

// the chunk partials of column blockIdx.y, as k_seg_partials does for one
struct SegOut { double* dst[SEG_MANY]; };
__global__ void __launch_bounds__(256) k_seg_partials_many(const double* __restrict__ part,
                                                           const long long* __restrict__ pstarts,
                                                           const long long* __restrict__ big, long long nbig,
                                                           long long nchunks, SegOut so) {
    __shared__ double ws[8];
    const long long g = blockIdx.x;
    const double* p = part + (size_t)blockIdx.y * (size_t)nchunks;
    const long long s = pstarts[g], e = (g + 1 < nbig) ? pstarts[g + 1] : nchunks;
    bool bad = false;
    double v[16];
    seg_load16<double, false>(p, nullptr, 0, s + threadIdx.x, e, v, bad);
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 16; k++)
        if (s + k * 256 + threadIdx.x < e) acc = __dadd_rn(acc, v[k]);
    acc = swarp<double, OP_SUM>(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        const double w01 = __dadd_rn(ws[0], ws[1]), w23 = __dadd_rn(ws[2], ws[3]);
        const double w45 = __dadd_rn(ws[4], ws[5]), w67 = __dadd_rn(ws[6], ws[7]);
        so.dst[blockIdx.y][big[g]] = __dadd_rn(__dadd_rn(w01, w23), __dadd_rn(w45, w67));
    }
}

// f64 sums of several columns over the segments of one grouping whose
// segments are all longer than one tile, with at most 4096 chunks in all;
// sums[q] receives column q's ng sums.  Returns 1 (nothing done) when the
// grouping is of another shape.
I seg_sum_f64_many(const double* const* srcs, int ncol, const long long* rows, long long nx, const long long* starts,
                   long long ng, long long total, ListInfo* li, double* const* sums) {
    if (ncol < 1 || ncol > SEG_MANY || ng == 0 || !li) return 1;
    const unsigned *ids, *ccnt;
    HG_CHECK(seg_classes(starts, ng, total, li, &ids, &ccnt));
    if (!li->cls_known) return 1;
    for (int c = 0; c < 7; c++)
        if (li->cls_host[c]) return 1;
    LongPlan pl;
    HG_CHECK(seg_plan_long(starts, ng, total, li, &pl));
    if (pl.nbig == 0 || pl.nchunks > (unsigned long long)TILE_SUM) return 1;
    double* part = (double*)salloc((size_t)pl.nchunks * ncol * sizeof(double));
    if (!part) return E_DEVICE_OOM;
    SegCols sc{};
    for (int q = 0; q < ncol; q++) sc.src[q] = srcs[q];
#define SEG_MANY_LAUNCH(NC)                                                                                          \
    HG_LAUNCH("seg_chunk_many", (unsigned)pl.nchunks, 256, 0, k_seg_chunk_many<NC>, sc, ncol, rows, nx, starts, ng, total, \
              pl.big, pl.c0, pl.nbig, pl.nchunks, pl.order, part, g_derr)
    if (ncol == 1) SEG_MANY_LAUNCH(1);
    else if (ncol == 2) SEG_MANY_LAUNCH(2);
    else if (ncol == 3) SEG_MANY_LAUNCH(3);
    else SEG_MANY_LAUNCH(4);
#undef SEG_MANY_LAUNCH
    SegOut so{};
    for (int q = 0; q < ncol; q++) so.dst[q] = sums[q];
    HG_LAUNCH("seg_partials", dim3((unsigned)pl.nbig, (unsigned)ncol), 256, 0, k_seg_partials_many, part, pl.pstarts,
              pl.big, pl.nbig, (long long)pl.nchunks, so);
    return last_launch_error();
}

// f64 sums of segments gathered through row ids, for the batched plans: the
// same kernels and order as hgpuGroupSum.
I seg_sum_f64(const double* src, const long long* rows, long long nx, const long long* starts, long long ng,
              long long total, double* out) {
    return seg_reduce<double, double, OP_SUM, true>(src, rows, nx, starts, ng, total, 0.0, out);
}

// f64 sums of contiguous segments (no row indirection), same order
I seg_sum_f64_direct(const double* src, const long long* starts, long long ng, long long total, double* out) {
    return seg_reduce<double, double, OP_SUM, false>(src, nullptr, 0, starts, ng, total, 0.0, out);
}

// ---------------------------------------------------------- finishing steps
template <typename A>
__global__ void k_avg_seg(const A* __restrict__ s, const long long* __restrict__ starts, long long ng, long long total,
                          void* __restrict__ out) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        long long m = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
        if constexpr (std::is_same<A, long long>::value) ((double*)out)[g] = __ddiv_rn((double)s[g] * 1.0, (double)m);
        else if constexpr (std::is_same<A, float>::value) ((float*)out)[g] = __fdiv_rn(s[g], (float)m);
        else ((double*)out)[g] = __ddiv_rn(s[g], (double)m);
    }
}
__global__ void k_len_seg(const long long* __restrict__ starts, long long ng, long long total, long long* __restrict__ out) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x)
        out[g] = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
}
// empty groups in min/max: the pfnReduce sentinel (ints become i64)
template <typename T>
__global__ void k_minmax_fix(const T* __restrict__ r, const long long* __restrict__ starts, long long ng, long long total,
                             int op, int to_long, void* __restrict__ out) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        long long m = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
        if (to_long) ((long long*)out)[g] = m ? (long long)r[g] : (op == AG_MIN ? LLONG_MAX : LLONG_MIN);
        else if constexpr (std::is_same<T, float>::value) ((float*)out)[g] = m ? r[g] : (op == AG_MIN ? 3.402823466e+38f : 1.175494351e-38f);
        else if constexpr (std::is_same<T, double>::value) ((double*)out)[g] = m ? r[g] : (op == AG_MIN ? 1.7976931348623157e308 : 2.2250738585072014e-308);
        else ((T*)out)[g] = r[g];
    }
}
__global__ void k_any_empty(const long long* __restrict__ starts, long long ng, long long total, unsigned* flag) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x)
        if (((g + 1 < ng) ? starts[g + 1] : total) == starts[g]) atomicOr(flag, 1u);
}

// Aggregates segments of x: result vector (device) of ng values, type in *typ.
template <typename T, bool GATHER>
static I agg_typed(int ag, I xt, const T* src, const long long* rows, long long nx, const long long* starts, long long ng,
                   long long total, void** out, I* typ, ListInfo* li) {
    constexpr bool isF = std::is_same<T, float>::value, isE = std::is_same<T, double>::value;
    using SA = typename std::conditional<isF, float, typename std::conditional<isE, double, long long>::type>::type;
    if (ag == AG_LEN) {
        *typ = H_L;
        *out = salloc((size_t)(ng > 0 ? ng : 1) * 8);
        if (!*out) return E_DEVICE_OOM;
        if (ng > 0) HG_LAUNCH("len_seg", gcap(ng), 256, 0, k_len_seg, starts, ng, total, (long long*)*out);
        return last_launch_error();
    }
    if (ag == AG_SUM || ag == AG_AVG) {
        SA* s = (SA*)salloc((size_t)(ng > 0 ? ng : 1) * sizeof(SA));
        if (!s) return E_DEVICE_OOM;
        HG_CHECK((seg_reduce<T, SA, OP_SUM, GATHER>(src, rows, nx, starts, ng, total, (SA)0, s, li)));
        if (ag == AG_SUM) {
            *typ = isF ? H_F : (isE ? H_E : H_L);
            *out = s;
            return 0;
        }
        *typ = isF ? H_F : H_E;
        *out = salloc((size_t)(ng > 0 ? ng : 1) * 8);
        if (!*out) return E_DEVICE_OOM;
        if (ng > 0) HG_LAUNCH("avg_seg", gcap(ng), 256, 0, k_avg_seg<SA>, s, starts, ng, total, *out);
        return last_launch_error();
    }
    // min / max
    T* r = (T*)salloc((size_t)(ng > 0 ? ng : 1) * sizeof(T));
    if (!r) return E_DEVICE_OOM;
    T identity;
    if (ag == AG_MIN) identity = std::numeric_limits<T>::has_infinity ? std::numeric_limits<T>::infinity() : std::numeric_limits<T>::max();
    else identity = std::numeric_limits<T>::has_infinity ? -std::numeric_limits<T>::infinity() : std::numeric_limits<T>::lowest();
    if (ag == AG_MIN) HG_CHECK((seg_reduce<T, T, OP_MIN, GATHER>(src, rows, nx, starts, ng, total, identity, r, li)));
    else HG_CHECK((seg_reduce<T, T, OP_MAX, GATHER>(src, rows, nx, starts, ng, total, identity, r, li)));
    unsigned h = 0;
    if (!(li && li->group_rows)) {  // @group never yields an empty group
        unsigned* fl = (unsigned*)salloc(16);
        if (!fl) return E_DEVICE_OOM;
        HG_CU(cudaMemsetAsync(fl, 0, 4, g_stream));
        if (ng > 0) HG_LAUNCH("any_empty", gcap(ng), 256, 0, k_any_empty, starts, ng, total, fl);
        HG_CHECK(rb_queue(&h, fl, 4));
        HG_CU(stream_sync());
    }
    bool to_long = h && is_int(xt);
    *typ = to_long ? H_L : xt;
    *out = salloc((size_t)(ng > 0 ? ng : 1) * (to_long ? 8 : sizeof(T)));
    if (!*out) return E_DEVICE_OOM;
    if (ng > 0) HG_LAUNCH("minmax_fix", gcap(ng), 256, 0, k_minmax_fix<T>, r, starts, ng, total, ag, to_long ? 1 : 0, *out);
    return last_launch_error();
}

template <bool GATHER>
static I agg_dispatch(int ag, I xt, const void* src, const long long* rows, long long nx, const long long* starts,
                      long long ng, long long total, void** out, I* typ, ListInfo* li) {
    switch (xt) {
    case H_B: return agg_typed<bool, GATHER>(ag, xt, (const bool*)src, rows, nx, starts, ng, total, out, typ, li);
    case H_J: return agg_typed<int8_t, GATHER>(ag, xt, (const int8_t*)src, rows, nx, starts, ng, total, out, typ, li);
    case H_H: return agg_typed<int16_t, GATHER>(ag, xt, (const int16_t*)src, rows, nx, starts, ng, total, out, typ, li);
    case H_I: return agg_typed<int32_t, GATHER>(ag, xt, (const int32_t*)src, rows, nx, starts, ng, total, out, typ, li);
    case H_L: return agg_typed<long long, GATHER>(ag, xt, (const long long*)src, rows, nx, starts, ng, total, out, typ, li);
    case H_F: return agg_typed<float, GATHER>(ag, xt, (const float*)src, rows, nx, starts, ng, total, out, typ, li);
    case H_E: return agg_typed<double, GATHER>(ag, xt, (const double*)src, rows, nx, starts, ng, total, out, typ, li);
    default: return E_DOMAIN;
    }
}

// ------------------------------------------------ lists -> contiguous segments
__global__ void k_node_lens(const V0* __restrict__ nodes, long long ng, unsigned* __restrict__ lens) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x)
        lens[g] = (unsigned)nodes[g].len;
}
// copies each element's payload to data + off[g] * es, one warp per element
// and one item per lane; `nodes` is a device copy of the host node array at
// host_base, so an inline element (its g points into its own host node)
// reads its item from the copy
template <typename T>
__global__ void k_node_copy(const V0* __restrict__ nodes, long long ng, unsigned long long host_base,
                            const unsigned long long* __restrict__ off, T* __restrict__ data) {
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ng; g += warps) {
        const V0 v = nodes[g];
        const unsigned long long own = host_base + (unsigned long long)g * sizeof(V0) + offsetof(V0, b);
        const T* src = ((unsigned long long)v.g == own) ? reinterpret_cast<const T*>(&nodes[g].b) : (const T*)v.g;
        for (long long b = lane_id(); b < v.len; b += 32) data[off[g] + b] = src[b];
    }
}
__global__ void k_offsets_i64(const unsigned long long* __restrict__ a, long long n, long long* __restrict__ b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (long long)a[i];
}

// Segments of a list whose elements all have type `typ`.  Lists built by this
// library are found in the registry; any other list is read through a device
// copy of its nodes.  Payloads must be device-readable.
static I list_segments(V y, I typ, const long long** starts, long long* total, const void** data,
                       ListInfo** info = nullptr) {
    long long ng = y->len;
    ListInfo* li = find_list(host_nodes(y), ng);
    if (info) *info = nullptr;
    if (li && li->kind == LIST_SEGMENTS && li->typ == typ) {
        *starts = li->starts;
        *total = li->total;
        *data = li->data;
        if (info) *info = li;
        return 0;
    }
    const V0* nodes = host_nodes(y);
    int es = esize(typ);
    for (long long g = 0; g < ng; g++) {
        if (nodes[g].typ != typ) return set_error(E_TYPE, "list element %lld has type %d, expected %d", g, nodes[g].typ, typ);
        const bool inl = nodes[g].g == (G)&nodes[g].b;
        if (nodes[g].len > 0 && !inl && !is_device_ptr(nodes[g].g))
            return set_error(E_NOT_IMPL, "list element %lld lives in pageable host memory; stage it with hgpuToDevice", g);
        if (inl && nodes[g].len > 1) return set_error(E_DOMAIN, "list element %lld: inline node with %lld items", g, nodes[g].len);
    }
    // the kernels read a device copy of the node array (one bulk copy, not
    // one host access per node)
    const unsigned long long host_base = (unsigned long long)(uintptr_t)nodes;
    V0* dn = (V0*)salloc((size_t)(ng > 0 ? ng : 1) * sizeof(V0));
    if (!dn) return E_DEVICE_OOM;
    if (ng > 0) HG_CU(cudaMemcpyAsync(dn, nodes, (size_t)ng * sizeof(V0), cudaMemcpyDefault, g_stream));
    if (!is_device_ptr(nodes)) HG_CU(stream_sync());  // pageable source: finish before returning
    nodes = dn;
    unsigned* lens = (unsigned*)salloc((size_t)(ng > 0 ? ng : 1) * 4);
    unsigned long long* off = (unsigned long long*)salloc((size_t)(ng > 0 ? ng : 1) * 8);
    long long* st = (long long*)salloc((size_t)(ng > 0 ? ng : 1) * 8);
    if (!lens || !off || !st) return E_DEVICE_OOM;
    unsigned long long tot = 0;
    if (ng > 0) {
        HG_LAUNCH("node_lens", gcap(ng), 256, 0, k_node_lens, nodes, ng, lens);
        HG_CHECK(scan_exclusive(lens, ng, off, &tot));
    }
    char* d = (char*)salloc((size_t)(tot > 0 ? tot : 1) * es);
    if (!d) return E_DEVICE_OOM;
    if (ng > 0) {
        const unsigned gr = gcap(ng * 32);
        switch (es) {
        case 1: HG_LAUNCH("node_copy", gr, 256, 0, k_node_copy<uint8_t>, nodes, ng, host_base, off, (uint8_t*)d); break;
        case 2: HG_LAUNCH("node_copy", gr, 256, 0, k_node_copy<uint16_t>, nodes, ng, host_base, off, (uint16_t*)d); break;
        case 4: HG_LAUNCH("node_copy", gr, 256, 0, k_node_copy<uint32_t>, nodes, ng, host_base, off, (uint32_t*)d); break;
        default: HG_LAUNCH("node_copy", gr, 256, 0, k_node_copy<unsigned long long>, nodes, ng, host_base, off,
                           (unsigned long long*)d); break;
        }
        HG_LAUNCH("offsets", gcap(ng), 256, 0, k_offsets_i64, off, ng, st);
    }
    *starts = st;
    *total = (long long)tot;
    *data = d;
    return last_launch_error();
}

// writes ng one-element nodes holding vals[g] (es bytes) into a device
// staging copy of the host node array at host_base (node g inline: its g
// points at its own host node)
__global__ void k_scalar_nodes(const char* __restrict__ vals, long long ng, int es, I typ, V0* __restrict__ out,
                               unsigned long long host_base) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        V0 v;
        v.len = 1;
        v.typ = typ;
        v.i64 = 0;
        for (int b = 0; b < es; b++) ((char*)&v.b)[b] = vals[g * es + b];
        v.g = (G)(host_base + (unsigned long long)g * sizeof(V0) + offsetof(V0, b));
        out[g] = v;
    }
}
// segment nodes over a contiguous payload (inline when one element)
__global__ void k_segment_nodes(const char* __restrict__ data, const long long* __restrict__ starts, long long ng,
                                long long total, int es, I typ, V0* __restrict__ out, unsigned long long host_base) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        long long s = starts[g], e = (g + 1 < ng) ? starts[g + 1] : total;
        V0 v;
        v.len = e - s;
        v.typ = typ;
        v.i64 = 0;
        if (e - s == 1) {
            for (int b = 0; b < es; b++) ((char*)&v.b)[b] = data[s * es + b];
            v.g = (G)(host_base + (unsigned long long)g * sizeof(V0) + offsetof(V0, b));
        } else {
            v.g = (G)(data + s * es);
        }
        out[g] = v;
    }
}

static I group_agg(V z, V x, V y, int ag) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (y->typ != H_G) return E_DOMAIN;
    if (!is_real(x->typ)) return E_DOMAIN;
    const long long* starts;
    long long total;
    const void* rows;
    ListInfo* li;
    HG_CHECK(list_segments(y, H_L, &starts, &total, &rows, &li));
    const void* px;
    HG_CHECK(in_ptr(x, &px));
    void* res;
    I typ;
    HG_CHECK(agg_dispatch<true>(ag, x->typ, px, (const long long*)rows, x->len, starts, y->len, total, &res, &typ, li));
    if (!(li && li->group_rows && x->len >= total)) HG_CHECK(check_device_errors());  // rows of @group are in range
    void* dz;
    HG_CHECK(alloc_out(z, typ, y->len, &dz));
    if (y->len > 0) HG_CU(cudaMemcpyAsync(dz, res, (size_t)y->len * esize(typ), cudaMemcpyDeviceToDevice, g_stream));
    return finish_out(z, dz);
}

}  // namespace hg

using namespace hg;

extern "C" {

I hgpuGroupSum(V z, V x, V y) { return group_agg(z, x, y, AG_SUM); }
I hgpuGroupAvg(V z, V x, V y) { return group_agg(z, x, y, AG_AVG); }
I hgpuGroupMin(V z, V x, V y) { return group_agg(z, x, y, AG_MIN); }
I hgpuGroupMax(V z, V x, V y) { return group_agg(z, x, y, AG_MAX); }
I hgpuGroupLen(V z, V x, V y) { return group_agg(z, x, y, AG_LEN); }

// z[k] = the aggregate aggs[k] (0 sum, 1 avg, 2 min, 3 max, 4 len) of x[k]
// over the grouping y, each bit for bit what hgpuGroupSum/Avg/Min/Max/Len
// returns.  The f64 sums and averages over a @group whose groups are all
// longer than one 4096-row tile share one pass that reads each group's row
// ids once (the common-index pattern applied to the segmented reductions).
I hgpuGroupAggMany(V* z, V* x, V y, const I* aggs, L n) {
    HG_CHECK(ensure_init());
    if (n < 0) return E_LENGTH;
    if (y->typ != H_G) return E_DOMAIN;
    int fused[SEG_MANY];
    int nf = 0;
    for (L k = 0; k < n; k++) {
        if (aggs[k] < AG_SUM || aggs[k] > AG_LEN || !is_real(x[k]->typ)) return E_DOMAIN;
        if ((aggs[k] == AG_SUM || aggs[k] == AG_AVG) && x[k]->typ == H_E && nf < SEG_MANY) fused[nf++] = (int)k;
    }
    bool done[64] = {false};
    if (nf >= 2 && n <= 64) {
        ScratchScope ss;
        const long long* starts;
        long long total;
        const void* rows;
        ListInfo* li;
        HG_CHECK(list_segments(y, H_L, &starts, &total, &rows, &li));
        const long long ng = y->len;
        const double* srcs[SEG_MANY];
        double* sums[SEG_MANY];
        bool in_range = li && li->group_rows;
        long long nx = -1;
        for (int q = 0; q < nf; q++) {
            const void* px;
            HG_CHECK(in_ptr(x[fused[q]], &px));
            srcs[q] = (const double*)px;
            sums[q] = (double*)salloc((size_t)(ng > 0 ? ng : 1) * 8);
            if (!sums[q]) return E_DEVICE_OOM;
            nx = nx < 0 ? x[fused[q]]->len : (x[fused[q]]->len < nx ? x[fused[q]]->len : nx);
        }
        in_range = in_range && nx >= total;
        I rc = seg_sum_f64_many(srcs, nf, (const long long*)rows, nx, starts, ng, total, li, sums);
        if (rc > 1) return rc;
        if (rc == 0) {
            if (!in_range) HG_CHECK(check_device_errors());
            for (int q = 0; q < nf; q++) {
                const int k = fused[q];
                void* dz;
                HG_CHECK(alloc_out(z[k], H_E, ng, &dz));
                if (aggs[k] == AG_AVG) {
                    if (ng > 0) HG_LAUNCH("avg_seg", gcap(ng), 256, 0, k_avg_seg<double>, sums[q], starts, ng, total, dz);
                    HG_CHECK(last_launch_error());
                } else if (ng > 0) {
                    HG_CU(cudaMemcpyAsync(dz, sums[q], (size_t)ng * 8, cudaMemcpyDeviceToDevice, g_stream));
                }
                HG_CHECK(finish_out(z[k], dz));
                done[k] = true;
            }
        }
    }
    for (L k = 0; k < n; k++)
        if (!(k < 64 && done[k])) HG_CHECK(group_agg(z[k], x[k], y, aggs[k]));
    return 0;
}

// pfnEachRight: h_primitive.cc:1882-1904.  With @index over a list of i64 row
// vectors all groups are gathered in one kernel into one contiguous payload.
I pfnEachRight(V z, V x, V y, I (*foo)(V, V, V)) {
    HG_CHECK(ensure_init());
    if (y->typ != H_G) return foo(z, x, y);
    long long ng = y->len;
    if (foo == pfnIndex && is_basic(x->typ) && ng > 0) {
        bool all_long = true;
        const V0* nodes = host_nodes(y);
        const ListInfo* li = find_list(nodes, ng);
        if (!li) for (long long g = 0; g < ng && all_long; g++) all_long = nodes[g].typ == H_L;
        if (all_long) {
            ScratchScope ss;
            const long long* starts;
            long long total;
            const void* rows;
            HG_CHECK(list_segments(y, H_L, &starts, &total, &rows));
            const void* px;
            HG_CHECK(in_ptr(x, &px));
            int es = esize(x->typ);
            char* data = (char*)dalloc((size_t)(total > 0 ? total : 1) * es);
            long long* keep = (long long*)dalloc((size_t)ng * 8);
            if (!data || !keep) return E_DEVICE_OOM;
            HG_CHECK(gather_into(px, x->len, es, rows, H_L, data, total));
            HG_CHECK(check_device_errors());
            HG_CU(cudaMemcpyAsync(keep, starts, (size_t)ng * 8, cudaMemcpyDeviceToDevice, g_stream));
            HG_CHECK(init_list(z, H_G, ng));
            V0* stage = (V0*)salloc((size_t)ng * sizeof(V0));
            if (!stage) return E_DEVICE_OOM;
            HG_LAUNCH("segment_nodes", gcap(ng), 256, 0, k_segment_nodes, data, keep, ng, total, es, x->typ, stage,
                      (unsigned long long)(uintptr_t)host_nodes(z));
            HG_CU(cudaMemcpyAsync(host_nodes(z), stage, (size_t)ng * sizeof(V0), cudaMemcpyDeviceToHost, g_stream));
            HG_CHECK(last_launch_error());
            HG_CHECK(sync());
            register_list({host_nodes(z), ng, LIST_SEGMENTS, x->typ, keep, total, data, 0, 0, 0, 0, nullptr, nullptr, nullptr});
            return apply_residency(z);
        }
    }
    HG_CHECK(init_list(z, H_G, ng));
    for (long long i = 0; i < ng; i++) HG_CHECK(foo(host_nodes(z) + i, x, host_nodes(y) + i));
    return 0;
}

// pfnEach: h_primitive.cc:1818-1832.  @sum/@avg/@min/@max/@len over a list of
// vectors run as one segmented reduction; other functions are applied per element.
I pfnEach(V z, V x, I (*foo)(V, V)) {
    HG_CHECK(ensure_init());
    if (x->typ != H_G) return E_DOMAIN;
    long long ng = x->len;
    int ag = foo == pfnSum ? AG_SUM : foo == pfnAvg ? AG_AVG : foo == pfnMin ? AG_MIN : foo == pfnMax ? AG_MAX
           : foo == pfnLen ? AG_LEN : -1;
    if (ag >= 0 && ng > 0) {
        const V0* nodes = host_nodes(x);
        I t = nodes[0].typ;
        bool same = is_real(t);
        const ListInfo* li = find_list(nodes, ng);
        if (!li) for (long long g = 1; g < ng && same; g++) same = nodes[g].typ == t;
        else same = same && li->typ == t && li->kind == LIST_SEGMENTS;
        if (same) {
            ScratchScope ss;
            const long long* starts;
            long long total;
            const void* vals;
            HG_CHECK(list_segments(x, t, &starts, &total, &vals));
            void* res;
            I typ;
            ListInfo* lk = find_list(host_nodes(x), ng);
            HG_CHECK(agg_dispatch<false>(ag, t, vals, nullptr, 0, starts, ng, total, &res, &typ, lk));
            int es = esize(typ);
            char* keep = (char*)dalloc((size_t)ng * es);
            if (!keep) return E_DEVICE_OOM;
            HG_CU(cudaMemcpyAsync(keep, res, (size_t)ng * es, cudaMemcpyDeviceToDevice, g_stream));
            HG_CHECK(init_list(z, H_G, ng));
            V0* stage = (V0*)salloc((size_t)ng * sizeof(V0));
            if (!stage) return E_DEVICE_OOM;
            HG_LAUNCH("scalar_nodes", gcap(ng), 256, 0, k_scalar_nodes, keep, ng, es, typ, stage,
                      (unsigned long long)(uintptr_t)host_nodes(z));
            HG_CU(cudaMemcpyAsync(host_nodes(z), stage, (size_t)ng * sizeof(V0), cudaMemcpyDeviceToHost, g_stream));
            HG_CHECK(last_launch_error());
            HG_CHECK(sync());
            register_list({host_nodes(z), ng, LIST_SCALARS, typ, nullptr, ng, keep, 0, 0, 0, 0, nullptr, nullptr, nullptr});
            return apply_residency(z);
        }
    }
    HG_CHECK(init_list(z, H_G, ng));
    for (long long i = 0; i < ng; i++) HG_CHECK(foo(host_nodes(z) + i, host_nodes(x) + i));
    return 0;
}

// pfnRaze: h_primitive.cc:935-955 — the elements' common type, concatenated.
I pfnRaze(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (x->typ != H_G) {
        if (is_basic(x->typ)) { *z = *x; if (is_inline(x)) z->g = (G)&z->b; return 0; }
        return E_DOMAIN;
    }
    long long ng = x->len;
    if (ng == 0) return set_error(E_RAZE_LIST, "an empty list cannot be razed");
    const V0* nodes = host_nodes(x);
    const ListInfo* li = find_list(nodes, ng);
    if (li && li->kind == LIST_SCALARS) {  // one value per element, already contiguous on the device
        void* dz;
        HG_CHECK(alloc_out(z, li->typ, ng, &dz));
        HG_CU(cudaMemcpyAsync(dz, li->data, (size_t)ng * esize(li->typ), cudaMemcpyDeviceToDevice, g_stream));
        return finish_out(z, dz);
    }
    I typ = -1;
    for (long long g = 0; g < ng; g++) {
        I t = nodes[g].typ;
        if (!is_basic(t)) return set_error(E_NOT_IMPL, "raze of nested lists");
        if (typ == -1) typ = t;
        else if (typ != t) {
            if (is_real(typ) && is_real(t)) typ = t > typ ? t : typ;
            else return E_RAZE_LIST;
        }
    }
    for (long long g = 0; g < ng; g++)
        if (nodes[g].typ != typ) return set_error(E_NOT_IMPL, "raze with type promotion across elements");
    const long long* starts;
    long long total;
    const void* data;
    HG_CHECK(list_segments(x, typ, &starts, &total, &data));
    void* dz;
    HG_CHECK(alloc_out(z, typ, total, &dz));
    if (total > 0) HG_CU(cudaMemcpyAsync(dz, data, (size_t)total * esize(typ), cudaMemcpyDeviceToDevice, g_stream));
    return finish_out(z, dz);
}

}  // extern "C"
