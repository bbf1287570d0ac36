// The reference's comparison sorts reproduced on the device: @order and
// @group keys of the types its radix and merge sorts do not take (bool, i8,
// i16, f32, f64, the date and time types) and lists of columns holding them.
//
//   lib_partition / lib_quicksort_other  src/horseir/v3/backend/h_libs.cc:409-442
//   lib_quicksort_char                   h_libs.cc:386-407
//   lib_order_by_sorted                  h_libs.cc:604-617
//   lib_quicksort_list                   h_libs.cc:637-697
//   lib_order_by_vector                  h_libs.cc:730-736
//
// The quicksort is unstable but deterministic, and the order it leaves equal
// keys in is the reference's result, so it is reproduced step for step.  One
// partition of a range [lo, hi) with the first element as pivot P computes:
//   * c = the number of elements of (lo, hi) comparing <= P; j = lo + c;
//   * the elements > P inside (lo, j] and the elements <= P inside (j, hi)
//     are equally many, and the k-th of the first (counted from the left)
//     trades places with the k-th of the second (counted from the right):
//     these are exactly the pairs the reference's two scans meet;
//   * then x[lo] and x[j] trade places, unless every element compares equal
//     to P (leftSame), in which case nothing moves and the range is done;
//   * the recursion continues on [lo, j) and [j+1, hi).
// Ranges are independent, so every range of one recursion depth is
// partitioned at once: a flag pair per element (<= P, < P), one scan over
// all ranges, the trade partners from the scan's ranks, and the next depth's
// ranges.  Depths repeat until no range of two or more elements is left.
// A NaN key makes the reference's comparator non-reflexive and its scans
// leave the range (undefined behaviour), so NaN keys return E_NOT_IMPL.
#include "dev_common.cuh"

namespace hg {

template <typename K>
I radix_sort(const K* keys, long long n, const K** kres, const unsigned** vres, const unsigned* init_vals);
I compact_rows(const uint8_t* mask, long long n, long long* out, long long* count);

constexpr unsigned QS_DONE = 0xffffffffu;
constexpr int QS_THREADS = 256, QS_ITEMS = 8, QS_TILE = QS_THREADS * QS_ITEMS;
constexpr int QS_SPLIT_LEVELS = 8;  // recursion depths issued between two reads of the active count
// A recursion deeper than max(8192, 2^36 / n) levels (first-element pivots
// on nearly ordered keys, where the reference's own sort is quadratic) is
// refused, which bounds a call to about 2^36 element visits.
static long long qs_max_levels(long long n) {
    const long long m = (1LL << 36) / (n > 0 ? n : 1);
    return m > 8192 ? m : 8192;
}

__device__ __forceinline__ long long qs_ival(const void* p, int typ, long long i) {
    switch (typ) {
    case H_B: return ((const uint8_t*)p)[i];
    case H_J: case H_C: return ((const int8_t*)p)[i];
    case H_H: return ((const int16_t*)p)[i];
    case H_I: case H_M: case H_D: case H_U: case H_W: case H_T: return ((const int32_t*)p)[i];
    default: return ((const long long*)p)[i];
    }
}

// An unsigned image of element i that orders as lib_quicksort_cmp_item
// (h_libs.cc:455-488) compares: integers (chars signed) by value, floats by
// value with -0.0 == +0.0.  Descending keys are complemented, so one
// ascending comparison of images serves both directions.
__device__ __forceinline__ unsigned long long qs_image(const void* p, int typ, long long i, unsigned* nanflag) {
    if (typ == H_F || typ == H_E) {
        double f = typ == H_F ? (double)((const float*)p)[i] : ((const double*)p)[i];
        if (f != f) { *nanflag = 1u; return 0; }
        if (f == 0.0) f = 0.0;
        const unsigned long long b = (unsigned long long)__double_as_longlong(f);
        return (b >> 63) ? ~b : (b | (1ull << 63));
    }
    return (unsigned long long)qs_ival(p, typ, i) ^ (1ull << 63);
}

__device__ __forceinline__ int qs_cmp(unsigned long long a, unsigned long long b) { return a < b ? -1 : (a > b ? 1 : 0); }

// img[p] = image of col[perm[p]] (perm null: row p)
__global__ void k_qs_image(const void* __restrict__ col, int typ, const unsigned* __restrict__ perm, long long n,
                           unsigned long long flip, unsigned long long* __restrict__ img, unsigned* nanflag) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        img[p] = qs_image(col, typ, perm ? (long long)perm[p] : p, nanflag) ^ flip;
}

__global__ void k_qs_iota(unsigned* __restrict__ v, long long n) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        v[p] = (unsigned)p;
}

// ---- one recursion depth over all ranges
// flag pair of position p: (x[p] <= P) + ((x[p] < P) << 32), 0 for the pivot
// itself and for finished positions.  Counts stay below 2^32, so the two
// halves of a packed prefix never carry into each other.
__device__ __forceinline__ unsigned long long qs_flag(const unsigned* __restrict__ lo, const unsigned long long* __restrict__ K,
                                                      long long p) {
    const unsigned l = lo[p];
    if (l == QS_DONE || (long long)l == p) return 0;
    const int c = qs_cmp(K[p], K[l]);
    return (unsigned long long)(c <= 0) | ((unsigned long long)(c < 0) << 32);
}

__global__ void __launch_bounds__(QS_THREADS) k_qs_count(const unsigned* __restrict__ lo, const unsigned long long* __restrict__ K,
                                                         long long n, unsigned long long* __restrict__ tile_sum) {
    __shared__ unsigned long long ws[QS_THREADS / 32];
    const long long base = (long long)blockIdx.x * QS_TILE + (long long)threadIdx.x * QS_ITEMS;
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < QS_ITEMS; k++)
        if (base + k < n) s += qs_flag(lo, K, base + k);
    s = warp_sum(s);
    if (lane_id() == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < QS_THREADS / 32; w++) t += ws[w];
        tile_sum[blockIdx.x] = t;
    }
}

// exclusive scan of the nt tile sums in place (one block); tile_sum[nt] = total
__global__ void __launch_bounds__(1024) k_qs_scan_sums(unsigned long long* __restrict__ ts, long long nt) {
    __shared__ unsigned long long wsum[32];
    const long long per = (nt + 1023) / 1024;
    const long long a = (long long)threadIdx.x * per, b = a + per < nt ? a + per : nt;
    unsigned long long s = 0;
    for (long long i = a; i < b; i++) s += ts[i];
    const unsigned long long incl = warp_incl_scan64(s);
    if (lane_id() == 31) wsum[threadIdx.x >> 5] = incl;
    __syncthreads();
    if (threadIdx.x < 32) {
        const unsigned long long w = wsum[threadIdx.x];
        const unsigned long long wi = warp_incl_scan64(w);
        wsum[threadIdx.x] = wi - w;
    }
    __syncthreads();
    unsigned long long off = wsum[threadIdx.x >> 5] + incl - s;
    for (long long i = a; i < b; i++) { const unsigned long long v = ts[i]; ts[i] = off; off += v; }
    if (threadIdx.x == 1023) ts[nt] = off;
}

// S[p] = exclusive prefix of the flag pairs; S[n] = total
__global__ void __launch_bounds__(QS_THREADS) k_qs_prefix(const unsigned* __restrict__ lo, const unsigned long long* __restrict__ K,
                                                          long long n, const unsigned long long* __restrict__ tile_sum,
                                                          long long nt, unsigned long long* __restrict__ S) {
    __shared__ unsigned long long ws[QS_THREADS / 32];
    const long long base = (long long)blockIdx.x * QS_TILE + (long long)threadIdx.x * QS_ITEMS;
    unsigned long long v[QS_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < QS_ITEMS; k++) {
        v[k] = base + k < n ? qs_flag(lo, K, base + k) : 0;
        s += v[k];
    }
    const unsigned long long incl = warp_incl_scan64(s);
    if (lane_id() == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    unsigned long long off = tile_sum[blockIdx.x] + incl - s;
    for (unsigned w = 0; w < (threadIdx.x >> 5); w++) off += ws[w];
#pragma unroll
    for (int k = 0; k < QS_ITEMS; k++) {
        if (base + k < n) S[base + k] = off;
        off += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) S[n] = tile_sum[nt];
}

__device__ __forceinline__ unsigned qs_le(unsigned long long s) { return (unsigned)s; }
__device__ __forceinline__ unsigned qs_lt(unsigned long long s) { return (unsigned)(s >> 32); }

// Lpos[lo + k] = the k-th element > P inside (lo, j] from the left;
// Rpos[lo + k] = the k-th element <= P inside (j, hi) from the right
// (Every slot index lies in [lo, hi) by the counting above; a slot outside
// it would mean inconsistent ranges and is recorded, not written.)
__global__ void k_qs_pos(const unsigned* __restrict__ lo, const unsigned* __restrict__ hi,
                         const unsigned long long* __restrict__ K, const unsigned long long* __restrict__ S, long long n,
                         unsigned* __restrict__ Lpos, unsigned* __restrict__ Rpos, unsigned* derr) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const unsigned l = lo[p];
        if (l == QS_DONE || (long long)l == p) continue;
        const unsigned h = hi[p];
        const unsigned le_lo = qs_le(S[l]), le_hi = qs_le(S[h]), le_p = qs_le(S[p]);
        const long long j = (long long)l + (le_hi - le_lo);
        const int c = qs_cmp(K[p], K[l]);
        long long slot = -1;
        unsigned* dst = nullptr;
        if (p <= j && c > 0) { slot = (long long)l + (long long)(p - l - 1) - (long long)(le_p - le_lo); dst = Lpos; }
        else if (p > j && c <= 0) { slot = (long long)l + (long long)le_hi - (long long)le_p - 1; dst = Rpos; }
        if (!dst) continue;
        if (slot >= (long long)l && slot < (long long)h) dst[slot] = (unsigned)p;
        else flag_error(derr, DERR_INDEX);
    }
}

// Moves every element of the partitioned ranges to its place, records the
// next depth's range of every element (or its final place) and counts the
// elements still in a range of two or more.
__global__ void k_qs_move(unsigned* __restrict__ lo, unsigned* __restrict__ hi, const unsigned long long* __restrict__ K,
                          const unsigned* __restrict__ P, const unsigned long long* __restrict__ S, long long n,
                          const unsigned* __restrict__ Lpos, const unsigned* __restrict__ Rpos,
                          unsigned long long* __restrict__ K2, unsigned* __restrict__ P2, unsigned* __restrict__ fin,
                          unsigned* __restrict__ active, unsigned* derr) {
    unsigned still = 0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const unsigned l = lo[p];
        if (l == QS_DONE) continue;
        const unsigned h = hi[p];
        const unsigned long long sl = S[l], sh = S[h];
        const unsigned cle = qs_le(sh) - qs_le(sl);
        const long long j = (long long)l + cle;
        if (cle == h - l - 1 && qs_lt(sh) == qs_lt(sl)) {  // leftSame: every element equals the pivot
            fin[p] = P[p];
            lo[p] = QS_DONE;
            continue;
        }
        const unsigned long long kp = K[l];
        // slot of the k-th element > P in (l, j] counted from the left, or of
        // the k-th element <= P in (j, h) counted from the right
        auto left_slot = [&](long long x) { return (long long)l + (x - l - 1) - (long long)(qs_le(S[x]) - qs_le(sl)); };
        auto right_slot = [&](long long x) { return (long long)l + (long long)qs_le(sh) - (long long)qs_le(S[x]) - 1; };
        long long q = p, slot = -1;
        const unsigned* from = nullptr;
        if (p == (long long)l) {
            q = j;
            if (j > (long long)l && qs_cmp(K[j], kp) > 0) { slot = left_slot(j); from = Rpos; }
        } else if (p == j) {
            q = l;
        } else {
            const int c = qs_cmp(K[p], kp);
            if (p < j && c > 0) { slot = left_slot(p); from = Rpos; }
            else if (p > j && c <= 0) { slot = right_slot(p); from = Lpos; }
        }
        if (from) {
            if (slot >= (long long)l && slot < (long long)h) q = from[slot];
            else { flag_error(derr, DERR_INDEX); q = p; }
        }
        if (q < (long long)l || q >= (long long)h) { flag_error(derr, DERR_INDEX); q = p; }
        long long nl, nh;
        if (p < j) { nl = l; nh = j; } else { nl = j + 1; nh = h; }
        if (p == j || nh - nl < 2) {
            fin[p] = P[q];
            lo[p] = QS_DONE;
        } else {
            P2[p] = P[q];
            K2[p] = K[q];
            lo[p] = (unsigned)nl;
            hi[p] = (unsigned)nh;
            still++;
        }
    }
    still = warp_sum(still);
    if (lane_id() == 0 && still) atomicAdd(active, still);
}

// ---- ranges (segments) of a list sort
// seg[p] = index of the segment holding position p (starts ascending)
__global__ void k_qs_segid(const long long* __restrict__ starts, long long ns, long long n, unsigned* __restrict__ seg) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        long long a = 0, b = ns - 1;  // last start <= p
        while (a < b) {
            const long long m = (a + b + 1) >> 1;
            if (starts[m] <= p) a = m; else b = m - 1;
        }
        seg[p] = (unsigned)a;
    }
}
// lib_order_by_sorted per segment: up[s] / down[s] = some neighbour pair rises / falls
__global__ void k_qs_updown(const unsigned long long* __restrict__ img, const unsigned* __restrict__ seg, long long n,
                            uint8_t* __restrict__ up, uint8_t* __restrict__ down) {
    for (long long p = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const unsigned s = seg[p];
        if (s != seg[p - 1]) continue;
        const unsigned long long a = img[p - 1], b = img[p];
        if (a < b && !up[s]) up[s] = 1;
        if (a > b && !down[s]) down[s] = 1;
    }
}
enum : uint8_t { QS_SORT = 0, QS_KEEP = 1, QS_REVERSE = 2 };
// mode of each segment: an ascending-ordered segment (rises, never falls)
// is kept; for a descending key (images complemented) a segment whose values
// ascend (images fall, never rise) is reversed; every other one is sorted
__global__ void k_qs_mode(const uint8_t* __restrict__ up, const uint8_t* __restrict__ down, long long ns, int desc,
                          uint8_t* __restrict__ mode, unsigned* __restrict__ nrev) {
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ns; s += (long long)gridDim.x * blockDim.x) {
        uint8_t m = QS_SORT;
        if (!desc && up[s] && !down[s]) m = QS_KEEP;
        if (desc && down[s] && !up[s]) { m = QS_REVERSE; atomicAdd(nrev, 1u); }
        mode[s] = m;
    }
}
__global__ void k_qs_reverse(const unsigned* __restrict__ perm, const unsigned* __restrict__ seg,
                             const long long* __restrict__ starts, long long ns, long long n, const uint8_t* __restrict__ mode,
                             unsigned* __restrict__ out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const unsigned s = seg[p];
        long long q = p;
        if (mode[s] == QS_REVERSE) {
            const long long a = starts[s], b = s + 1 < ns ? starts[s + 1] : n;
            q = a + b - 1 - p;
        }
        out[p] = perm[q];
    }
}
// range of each position for the quicksort: its segment when that is sorted
// and holds two or more elements; finished positions keep their row
__global__ void k_qs_ranges(const unsigned* __restrict__ seg, const long long* __restrict__ starts, long long ns, long long n,
                            const uint8_t* __restrict__ mode, const unsigned* __restrict__ perm,
                            unsigned* __restrict__ lo, unsigned* __restrict__ hi, unsigned* __restrict__ fin) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const unsigned s = seg ? seg[p] : 0;
        const long long a = seg ? starts[s] : 0, b = seg ? (s + 1 < ns ? starts[s + 1] : n) : n;
        if ((mode && mode[s] != QS_SORT) || b - a < 2) {
            lo[p] = QS_DONE;
            fin[p] = perm[p];
        } else {
            lo[p] = (unsigned)a;
            hi[p] = (unsigned)b;
        }
    }
}
// stable sort of the segments in (segment, image) order: the key of a
// position that must not move (a kept, reversed or small char segment) is 0
__global__ void k_qs_skey(const unsigned long long* __restrict__ img, const unsigned* __restrict__ seg,
                          const long long* __restrict__ starts, long long ns, long long n, const uint8_t* __restrict__ mode,
                          int min_len, unsigned long long* __restrict__ key) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const unsigned s = seg[p];
        const long long a = starts[s], b = s + 1 < ns ? starts[s + 1] : n;
        key[p] = (mode[s] == QS_SORT && b - a >= min_len) ? img[p] : 0;
    }
}
__global__ void k_qs_gather_seg(const unsigned* __restrict__ seg, const unsigned* __restrict__ pos, long long n,
                                unsigned* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = seg[pos[i]];
}
__global__ void k_qs_permute(const unsigned* __restrict__ perm, const unsigned* __restrict__ pos, long long n,
                             unsigned* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = perm[pos[i]];
}
// lib_quicksort_char below ten elements (h_libs.cc:388-390): the all-pairs
// exchange on a[rtn[i]] > a[rtn[j]], one thread per sorted segment
__global__ void k_qs_char_small(const int8_t* __restrict__ a, const long long* __restrict__ starts, long long ns, long long n,
                                const uint8_t* __restrict__ mode, unsigned* __restrict__ perm) {
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ns; s += (long long)gridDim.x * blockDim.x) {
        const long long lo = starts[s], hi = s + 1 < ns ? starts[s + 1] : n;
        if (mode[s] != QS_SORT || hi - lo >= 10 || hi - lo < 2) continue;
        unsigned r[10];
        const int m = (int)(hi - lo);
        for (int i = 0; i < m; i++) r[i] = perm[lo + i];
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++)
                if (a[r[i]] > a[r[j]]) { const unsigned t = r[i]; r[i] = r[j]; r[j] = t; }
        for (int i = 0; i < m; i++) perm[lo + i] = r[i];
    }
}
// run heads of the next column: a new segment or a new image value
__global__ void k_qs_heads(const unsigned long long* __restrict__ img, const unsigned* __restrict__ seg, long long n,
                           uint8_t* __restrict__ head) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        head[p] = p == 0 || seg[p] != seg[p - 1] || img[p] != img[p - 1];
}

static unsigned qs_grid(long long n) {
    unsigned g = grid_for(n, 256);
    return g > (unsigned)g_sms * 16 ? (unsigned)g_sms * 16 : g;
}

// The quicksort of every range at once.  perm/img: the elements in their
// current order (consumed); lo/hi: each position's range (QS_DONE: not in
// one, fin already holds its row).  On return fin holds every position's row.
static I qs_run(long long n, unsigned* perm, unsigned long long* img, unsigned* lo, unsigned* hi, unsigned* fin) {
    const long long nt = (n + QS_TILE - 1) / QS_TILE;
    unsigned* P2 = (unsigned*)salloc((size_t)n * 4);
    unsigned long long* K2 = (unsigned long long*)salloc((size_t)n * 8);
    unsigned long long* S = (unsigned long long*)salloc((size_t)(n + 1) * 8);
    unsigned long long* ts = (unsigned long long*)salloc((size_t)(nt + 1) * 8);
    unsigned* Lpos = (unsigned*)salloc((size_t)n * 4);
    unsigned* Rpos = (unsigned*)salloc((size_t)n * 4);
    unsigned* act = (unsigned*)salloc(QS_SPLIT_LEVELS * 4);
    if (!P2 || !K2 || !S || !ts || !Lpos || !Rpos || !act) return E_DEVICE_OOM;
    unsigned* Pc = perm;
    unsigned long long* Kc = img;
    const unsigned g = qs_grid(n);
    const long long max_levels = qs_max_levels(n);
    for (long long level = 0;; level += QS_SPLIT_LEVELS) {
        if (level >= max_levels)
            return set_error(E_NOT_IMPL, "the reference's quicksort recursion is deeper than %lld levels here "
                             "(first-element pivots on nearly ordered keys)", max_levels);
        HG_CU(cudaMemsetAsync(act, 0, QS_SPLIT_LEVELS * 4, g_stream));
        for (int d = 0; d < QS_SPLIT_LEVELS; d++) {
            HG_LAUNCH("qs_count", (unsigned)nt, QS_THREADS, 0, k_qs_count, lo, Kc, n, ts);
            HG_LAUNCH("qs_scan_sums", 1, 1024, 0, k_qs_scan_sums, ts, nt);
            HG_LAUNCH("qs_prefix", (unsigned)nt, QS_THREADS, 0, k_qs_prefix, lo, Kc, n, ts, nt, S);
            HG_LAUNCH("qs_pos", g, 256, 0, k_qs_pos, lo, hi, Kc, S, n, Lpos, Rpos, g_derr);
            unsigned* Pn = Pc == perm ? P2 : perm;
            unsigned long long* Kn = Kc == img ? K2 : img;
            HG_LAUNCH("qs_move", g, 256, 0, k_qs_move, lo, hi, Kc, Pc, S, n, Lpos, Rpos, Kn, Pn, fin, act + d, g_derr);
            Pc = Pn;
            Kc = Kn;
        }
        HG_CHECK(last_launch_error());
        unsigned h = 0;
        HG_CHECK(rb_queue(&h, act + QS_SPLIT_LEVELS - 1, 4));
        HG_CU(stream_sync());
        if (h == 0) break;
    }
    return check_device_errors();
}

static I qs_image_of(const void* col, I typ, const unsigned* perm, long long n, bool desc, unsigned long long* img,
                     unsigned* nanflag) {
    if (n > 0)
        HG_LAUNCH("qs_image", qs_grid(n), 256, 0, k_qs_image, col, (int)typ, perm, n, desc ? ~0ull : 0ull, img, nanflag);
    return last_launch_error();
}

static I qs_nan_check(unsigned* nanflag) {
    unsigned h = 0;
    HG_CHECK(rb_queue(&h, nanflag, 4));
    HG_CU(stream_sync());
    if (h) return set_error(E_NOT_IMPL, "NaN sort key: the reference's quicksort compares NaN as greater than "
                            "itself and scans outside the range");
    return 0;
}

// lib_order_by_vector (h_libs.cc:730-736) on a key its quicksort sorts:
// rows 0..n-1 in order, then lib_quicksort_other over [0, n).
I qs_sort_vector(const void* col, I typ, long long n, bool asc, const unsigned** perm_out) {
    if (n >= (1LL << 31)) return set_error(E_NOT_IMPL, "quicksort order of 2^31 or more rows");
    unsigned* perm = (unsigned*)salloc((size_t)(n > 0 ? n : 1) * 4);
    unsigned* fin = (unsigned*)salloc((size_t)(n > 0 ? n : 1) * 4);
    unsigned long long* img = (unsigned long long*)salloc((size_t)(n > 0 ? n : 1) * 8);
    unsigned* lo = (unsigned*)salloc((size_t)(n > 0 ? n : 1) * 4);
    unsigned* hi = (unsigned*)salloc((size_t)(n > 0 ? n : 1) * 4);
    unsigned* nanflag = (unsigned*)salloc(16);
    if (!perm || !fin || !img || !lo || !hi || !nanflag) return E_DEVICE_OOM;
    *perm_out = fin;
    if (n == 0) return 0;
    HG_CU(cudaMemsetAsync(nanflag, 0, 4, g_stream));
    HG_LAUNCH("qs_iota", qs_grid(n), 256, 0, k_qs_iota, perm, n);
    HG_CHECK(qs_image_of(col, typ, nullptr, n, !asc, img, nanflag));
    HG_CHECK(qs_nan_check(nanflag));
    HG_LAUNCH("qs_ranges", qs_grid(n), 256, 0, k_qs_ranges, (const unsigned*)nullptr, (const long long*)nullptr, 0LL, n,
              (const uint8_t*)nullptr, perm, lo, hi, fin);
    return qs_run(n, perm, img, lo, hi, fin);
}

// lib_quicksort_list (h_libs.cc:637-697) over nc columns: for each column in
// turn, every run of rows equal on the columns before it is checked by
// lib_order_by_sorted (kept, or reversed for a descending column whose values
// ascend) and otherwise sorted -- i32/i64 columns by the stable merge sort,
// char columns by lib_quicksort_char, the rest by the quicksort -- and its
// runs of equal values form the next column's ranges.
I qs_sort_list(int nc, const void* const* cols, const I* typs, const B* asc, long long n, const unsigned** perm_out) {
    if (n >= (1LL << 31)) return set_error(E_NOT_IMPL, "quicksort order of 2^31 or more rows");
    const size_t nn = (size_t)(n > 0 ? n : 1);
    unsigned* perm = (unsigned*)salloc(nn * 4);
    unsigned* tmp = (unsigned*)salloc(nn * 4);
    unsigned* seg = (unsigned*)salloc(nn * 4);
    unsigned long long* img = (unsigned long long*)salloc(nn * 8);
    long long* starts = (long long*)salloc(nn * 8);
    uint8_t* flags = (uint8_t*)salloc(nn * 3);
    unsigned* aux = (unsigned*)salloc(64);
    if (!perm || !tmp || !seg || !img || !starts || !flags || !aux) return E_DEVICE_OOM;
    *perm_out = perm;
    if (n == 0) return 0;
    uint8_t* up = flags;
    uint8_t* down = flags + nn;
    uint8_t* mode = flags + 2 * nn;
    unsigned* nanflag = aux;
    unsigned* nrev = aux + 1;
    HG_CU(cudaMemsetAsync(nanflag, 0, 4, g_stream));
    const unsigned g = qs_grid(n);
    HG_LAUNCH("qs_iota", g, 256, 0, k_qs_iota, perm, n);
    long long ns = 1;  // segments: runs of rows equal on the columns sorted so far
    HG_CU(cudaMemsetAsync(starts, 0, 8, g_stream));
    HG_CU(cudaMemsetAsync(seg, 0, nn * 4, g_stream));
    for (int c = 0; c < nc; c++) {
        const I typ = typs[c];
        const bool desc = asc && !asc[c];
        if (typ == H_C && desc)
            return set_error(E_NOT_IMPL, "descending char column in a list order (the reference indexes past the range)");
        HG_CHECK(qs_image_of(cols[c], typ, perm, n, desc, img, nanflag));
        // lib_order_by_sorted
        HG_CU(cudaMemsetAsync(flags, 0, 2 * nn, g_stream));
        HG_CU(cudaMemsetAsync(nrev, 0, 4, g_stream));
        HG_LAUNCH("qs_updown", g, 256, 0, k_qs_updown, img, seg, n, up, down);
        HG_LAUNCH("qs_mode", qs_grid(ns), 256, 0, k_qs_mode, up, down, ns, desc ? 1 : 0, mode, nrev);
        unsigned hrev = 0;
        HG_CHECK(rb_queue(&hrev, nrev, 4));
        HG_CU(stream_sync());
        HG_CHECK(qs_nan_check(nanflag));
        if (hrev) {
            HG_LAUNCH("qs_reverse", g, 256, 0, k_qs_reverse, perm, seg, starts, ns, n, mode, tmp);
            unsigned* t = perm; perm = tmp; tmp = t;
            HG_CHECK(qs_image_of(cols[c], typ, perm, n, desc, img, nanflag));
        }
        if (typ == H_I || typ == H_L || typ == H_C) {
            // stable by (segment, image): radix sort on the image, then on
            // the segment index; kept, reversed and small char segments have
            // key 0 and do not move
            unsigned long long* key = (unsigned long long*)salloc(nn * 8);
            unsigned* sk = (unsigned*)salloc(nn * 4);
            if (!key || !sk) return E_DEVICE_OOM;
            HG_LAUNCH("qs_skey", g, 256, 0, k_qs_skey, img, seg, starts, ns, n, mode, typ == H_C ? 10 : 2, key);
            const unsigned long long* k1;
            const unsigned* pos1;
            HG_CHECK(radix_sort<unsigned long long>(key, n, &k1, &pos1, nullptr));
            HG_LAUNCH("qs_gather_seg", g, 256, 0, k_qs_gather_seg, seg, pos1, n, sk);
            const unsigned* k2;
            const unsigned* pos2;
            HG_CHECK(radix_sort<unsigned>(sk, n, &k2, &pos2, pos1));
            HG_LAUNCH("qs_permute", g, 256, 0, k_qs_permute, perm, pos2, n, tmp);
            unsigned* t = perm; perm = tmp; tmp = t;
            if (typ == H_C)
                HG_LAUNCH("qs_char_small", qs_grid(ns), 256, 0, k_qs_char_small, (const int8_t*)cols[c], starts, ns, n,
                          mode, perm);
        } else {
            unsigned* lo = (unsigned*)salloc(nn * 4);
            unsigned* hi = (unsigned*)salloc(nn * 4);
            if (!lo || !hi) return E_DEVICE_OOM;
            HG_LAUNCH("qs_ranges", g, 256, 0, k_qs_ranges, seg, starts, ns, n, mode, perm, lo, hi, tmp);
            HG_CHECK(qs_run(n, perm, img, lo, hi, tmp));
            unsigned* t = perm; perm = tmp; tmp = t;
        }
        if (c + 1 < nc) {  // the runs of equal values become the next column's segments
            HG_CHECK(qs_image_of(cols[c], typ, perm, n, desc, img, nanflag));
            HG_LAUNCH("qs_heads", g, 256, 0, k_qs_heads, img, seg, n, up);
            HG_CHECK(compact_rows(up, n, starts, &ns));
            HG_LAUNCH("qs_segid", g, 256, 0, k_qs_segid, starts, ns, n, seg);
        }
    }
    HG_CHECK(last_launch_error());
    *perm_out = perm;
    return 0;
}

}  // namespace hg
