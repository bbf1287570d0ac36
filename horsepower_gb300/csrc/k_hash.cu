// Hash-based builtins: @index_of, @member, @join_index.
//
// Reference (src/horseir/v3/backend):
//   pfnIndexOf  h_primitive.cc:1523-1579 — first row of x holding y[i], else
//               len(x).  A monotone (or constant) i32/i64 x takes the
//               recursive binary search of searchOrdered (h_system.cc:715-745),
//               which returns whatever matching row the recursion lands on
//               and misses on descending x; that recursion is reproduced.
//               Bool uses lib_index_of_B (h_libs.cc:309-314), whose flag
//               table maps `true` to row 0 always.
//   pfnMember   h_primitive.cc:2287-2336 (z, probe, set) — sets of <= 2
//               elements compare directly, larger sets hash.
//   pfnJoinIndex h_primitive.cc:2122-2155 + lib_join_radix_hash_v3
//               (h_hash_v3.cc:230-260): the shorter side is built; for each
//               probe row in order every matching build row in order is
//               emitted; builds of < 10 rows use the linear join, which keeps
//               only the first match (h_libs.cc:1542-1575).
//
// GB300 design: open-addressing tables in HBM (linear probing, murmur3
// finaliser, capacity = next power of two >= n / load factor).  Slots hold
// the key and the minimum row (atomicMin), plus a count for joins.  The join
// probe is one pass over the probe side: a tile of 4096 probe rows looks up
// its keys, takes its output offset from a decoupled look-back and writes the
// (build row, probe row) pairs with ballot/popc compaction.  Keys with
// duplicate build rows use a count / scan / write path over a CSR of build
// rows sorted per slot.
#include <climits>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "dev_common.cuh"

namespace hg {

I scan_exclusive(const unsigned* in, long long n, unsigned long long* out, unsigned long long* total_h);

static double g_load_factor = 0.5;  // hash-table load factor, 0.5 - 0.8 (autotuner knob)
void set_hash_load_factor(double f) { g_load_factor = f < 0.5 ? 0.5 : (f > 0.8 ? 0.8 : f); }
double get_hash_load_factor() { return g_load_factor; }

__device__ __forceinline__ unsigned long long fmix64(unsigned long long k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdULL; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ULL; k ^= k >> 33;
    return k;
}
__device__ __forceinline__ unsigned fmix32(unsigned h) {
    h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
    return h;
}
template <typename K>
__device__ __forceinline__ unsigned long long hash_key(K k) {
    if constexpr (sizeof(K) == 4) return fmix32((unsigned)k);
    else return fmix64((unsigned long long)k);
}

// key bits of element i of a vector already promoted to `typ`; false for NaN
template <typename K>
__device__ __forceinline__ bool key_at(const void* p, int typ, long long i, K* k) {
    switch (typ) {
    case H_J: *k = (K)(long long)((const int8_t*)p)[i]; return true;
    case H_H: *k = (K)(long long)((const int16_t*)p)[i]; return true;
    case H_I: *k = (K)(long long)((const int32_t*)p)[i]; return true;
    case H_L: *k = (K)((const long long*)p)[i]; return true;
    case H_F: { float f = ((const float*)p)[i]; if (f != f) return false; *k = (K)__float_as_uint(f); return true; }
    case H_E: { double f = ((const double*)p)[i]; if (f != f) return false; *k = (K)__double_as_longlong(f); return true; }
    default: *k = (K)((const bool*)p)[i]; return true;
    }
}

// Slots.  32-bit keys: one u64 per slot = (key << 32) | row, so a probe is a
// single 8-byte read and an insert a CAS followed, for a repeated key, by an
// atomicMin on the packed word (same key bits: the minimum is the minimum row).
// EMPTY (all ones) cannot collide with a real entry because rows are < 2^32-1.
// 64-bit keys: 16-byte slots {key, row} read with one vector load; the key
// equal to EMPTY lives in a side slot.
template <typename K>
struct Table {
    void* slots;
    unsigned* cnt;      // rows per slot (duplicate-key joins only), may be null
    unsigned* special;  // 64-bit keys: [0] min row, [1] count of the key equal to EMPTY
    unsigned* flags;    // [0] = a key was inserted twice
    unsigned long long cap;  // slots; the home slot is (hash32 * cap) >> 32
    // presence filter read before any slot: a miss costs one small,
    // cache-resident bitmap read instead of a walk along the probe sequence
    unsigned* filter;
    unsigned long long fmask;  // hash mode: filter bits - 1
    // direct mode (integer keys whose range is at most a few times n):
    // slots is a u32 row array indexed by key - kmin, filter bit = key - kmin
    int direct;
    long long kmin, kmax;
};

template <typename K>
__device__ __forceinline__ long long key_signed(K k) {
    if constexpr (sizeof(K) == 4) return (long long)(int)k;
    else return (long long)k;
}
// filter bit of a key, or -1 when the key cannot be present (outside the direct range)
template <typename K>
__device__ __forceinline__ long long filter_bit(const Table<K>& t, K k) {
    if (t.direct) {
        long long v = key_signed<K>(k);
        return (v < t.kmin || v > t.kmax) ? -1 : v - t.kmin;
    }
    unsigned long long h = hash_key<K>(k);
    return (long long)(((h >> 17) ^ (h << 7)) & t.fmask);
}

template <typename K>
__device__ __forceinline__ unsigned long long home_slot(K k, unsigned long long cap) {
    unsigned long long h = hash_key<K>(k);
    unsigned h32 = sizeof(K) == 4 ? (unsigned)h : (unsigned)(h >> 32);
    return ((unsigned long long)h32 * cap) >> 32;
}
__device__ __forceinline__ unsigned long long next_slot(unsigned long long h, unsigned long long cap) {
    return (h + 1 == cap) ? 0 : h + 1;
}

template <typename K>
__device__ __forceinline__ void table_insert(Table<K> t, K k, unsigned r, unsigned* derr) {
    {
        long long fb = filter_bit<K>(t, k);
        if (fb < 0) { flag_error(derr, DERR_CAPACITY); return; }
        if (t.filter) atomicOr(&t.filter[fb >> 5], 1u << (fb & 31));
        if (t.direct) {  // the minimum row wins; a second insert flags a repeated key
            unsigned* row = (unsigned*)t.slots;
            if (atomicMin(&row[fb], r) != 0xffffffffu) atomicOr(t.flags, 1u);
            return;
        }
    }
    unsigned long long h = home_slot<K>(k, t.cap);
    if constexpr (sizeof(K) == 4) {
        unsigned long long* sl = (unsigned long long*)t.slots;
        const unsigned long long mine = ((unsigned long long)k << 32) | r;
        for (unsigned long long p = 0; p < t.cap; p++) {
            unsigned long long cur = sl[h];
            if (cur == ~0ull) {
                cur = atomicCAS(&sl[h], ~0ull, mine);
                if (cur == ~0ull) return;
            }
            if ((unsigned)(cur >> 32) == (unsigned)k) {
                atomicMin(&sl[h], mine);
                atomicOr(t.flags, 1u);
                return;
            }
            h = next_slot(h, t.cap);
        }
    } else {
        if (k == ~0ull) {
            if (atomicAdd(&t.special[1], 1u)) atomicOr(t.flags, 1u);
            atomicMin(&t.special[0], r);
            return;
        }
        ulonglong2* sl = (ulonglong2*)t.slots;
        for (unsigned long long p = 0; p < t.cap; p++) {
            unsigned long long cur = sl[h].x;
            if (cur == ~0ull) {
                cur = atomicCAS(&sl[h].x, ~0ull, (unsigned long long)k);
                if (cur == ~0ull) { atomicMin(&sl[h].y, (unsigned long long)r); return; }
            }
            if (cur == (unsigned long long)k) {
                atomicMin(&sl[h].y, (unsigned long long)r);
                atomicOr(t.flags, 1u);
                return;
            }
            h = next_slot(h, t.cap);
        }
    }
    flag_error(derr, DERR_CAPACITY);
}

// Looks up N keys at once: all first-slot reads are issued before any is
// examined, so a lane keeps N table reads in flight.  slot[j] = slot index
// (-2 for the 64-bit side slot, -1 if absent), row[j] = minimum row
// (0xffffffff if absent).
template <typename K, int N>
__device__ __forceinline__ void table_find_n(const Table<K>& t, const K* key, const bool* valid, long long* slot,
                                             unsigned* row) {
    // 1. presence filter: N independent reads of a small bitmap
    long long fb[N];
    unsigned fw[N];
    bool cand[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        fb[j] = valid[j] ? filter_bit<K>(t, key[j]) : -1;
        fw[j] = fb[j] >= 0 ? __ldg(t.filter + (fb[j] >> 5)) : 0u;
    }
#pragma unroll
    for (int j = 0; j < N; j++) {
        cand[j] = fb[j] >= 0 && ((fw[j] >> (fb[j] & 31)) & 1u);
        slot[j] = -1;
        row[j] = 0xffffffffu;
    }
    if (t.direct) {  // 2a. one row read per candidate
        const unsigned* rs = (const unsigned*)t.slots;
        unsigned rr[N];
#pragma unroll
        for (int j = 0; j < N; j++) rr[j] = cand[j] ? __ldg(rs + fb[j]) : 0xffffffffu;
#pragma unroll
        for (int j = 0; j < N; j++)
            if (cand[j] && rr[j] != 0xffffffffu) { slot[j] = fb[j]; row[j] = rr[j]; }
        return;
    }
    // 2b. hash slots of the candidates, first reads issued together
    unsigned long long h[N];
    if constexpr (sizeof(K) == 4) {
        const unsigned long long* sl = (const unsigned long long*)t.slots;
        unsigned long long sv[N];
#pragma unroll
        for (int j = 0; j < N; j++) { h[j] = home_slot<K>(key[j], t.cap); sv[j] = cand[j] ? __ldg(sl + h[j]) : ~0ull; }
#pragma unroll
        for (int j = 0; j < N; j++) {
            if (!cand[j]) continue;
            for (unsigned long long p = 0; p < t.cap; p++) {
                if (sv[j] == ~0ull) break;
                if ((unsigned)(sv[j] >> 32) == (unsigned)key[j]) { slot[j] = (long long)h[j]; row[j] = (unsigned)sv[j]; break; }
                h[j] = next_slot(h[j], t.cap);
                sv[j] = __ldg(sl + h[j]);
            }
        }
    } else {
        const ulonglong2* sl = (const ulonglong2*)t.slots;
        ulonglong2 sv[N];
#pragma unroll
        for (int j = 0; j < N; j++) {
            h[j] = home_slot<K>(key[j], t.cap);
            sv[j] = (cand[j] && key[j] != ~0ull) ? __ldg(sl + h[j]) : make_ulonglong2(~0ull, ~0ull);
        }
#pragma unroll
        for (int j = 0; j < N; j++) {
            if (!cand[j]) continue;
            if (key[j] == ~0ull) {
                if (t.special[1]) { slot[j] = -2; row[j] = t.special[0]; }
                continue;
            }
            for (unsigned long long p = 0; p < t.cap; p++) {
                if (sv[j].x == ~0ull) break;
                if (sv[j].x == (unsigned long long)key[j]) { slot[j] = (long long)h[j]; row[j] = (unsigned)sv[j].y; break; }
                h[j] = next_slot(h[j], t.cap);
                sv[j] = __ldg(sl + h[j]);
            }
        }
    }
}

template <typename K>
__device__ __forceinline__ long long table_find(const Table<K>& t, K k, long long* row) {
    bool v = true;
    long long s;
    unsigned r;
    table_find_n<K, 1>(t, &k, &v, &s, &r);
    *row = (long long)r;
    return s;
}

template <typename K>
__global__ void k_build(Table<K> t, const void* __restrict__ x, int typ, long long n, unsigned* derr) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        if (key_at<K>(x, typ, i, &k)) table_insert<K>(t, k, (unsigned)i, derr);
    }
}

__global__ void k_key_minmax(const void* __restrict__ x, int typ, long long n, long long* mm) {
    long long a = LLONG_MAX, b = LLONG_MIN;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v;
        switch (typ) {
        case H_J: v = ((const int8_t*)x)[i]; break;
        case H_H: v = ((const int16_t*)x)[i]; break;
        case H_I: v = ((const int32_t*)x)[i]; break;
        default: v = ((const long long*)x)[i]; break;
        }
        a = v < a ? v : a;
        b = v > b ? v : b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long q = __shfl_xor_sync(0xffffffffu, a, o); a = q < a ? q : a;
        long long r = __shfl_xor_sync(0xffffffffu, b, o); b = r > b ? r : b;
    }
    // one pair of atomics per block, not per warp (they serialise on two words)
    __shared__ long long sa[32], sb[32];
    const unsigned nw = (blockDim.x + 31) >> 5;
    if (lane_id() == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 1; w < nw; w++) { a = sa[w] < a ? sa[w] : a; b = sb[w] > b ? sb[w] : b; }
        atomicMin(mm, a);
        atomicMax(mm + 1, b);
    }
}

template <typename K>
static I table_create(Table<K>* t, long long n, bool with_count, int direct, long long kmin, long long kmax,
                      bool filter = true) {
    const size_t ss = sizeof(K) == 4 ? 8 : 16;
    t->direct = direct;
    t->kmin = kmin;
    t->kmax = kmax;
    unsigned long long fbits;
    if (direct) {
        t->cap = (unsigned long long)(kmax - kmin + 1);
        fbits = t->cap;
        t->slots = salloc(t->cap * 4);
    } else {
        unsigned long long cap = (unsigned long long)((double)n / g_load_factor) + 16;
        if (cap > 0xffffffffull) cap = 0xffffffffull;
        t->cap = cap;
        fbits = 4096;
        while (fbits < 16ull * (unsigned long long)n) fbits <<= 1;
        t->slots = salloc(cap * ss);
    }
    if (!direct) filter = true;  // hash probes always read the filter first
    t->fmask = fbits - 1;
    size_t fwords = (size_t)((fbits + 31) / 32);
    t->filter = filter ? (unsigned*)salloc(fwords * 4) : nullptr;
    t->cnt = with_count ? (unsigned*)salloc(t->cap * 4) : nullptr;
    t->special = (unsigned*)salloc(32);
    if (!t->slots || (filter && !t->filter) || (with_count && !t->cnt) || !t->special) return E_DEVICE_OOM;
    t->flags = t->special + 2;
    HG_CU(cudaMemsetAsync(t->slots, 0xff, t->cap * (direct ? 4 : ss), g_stream));
    if (filter) HG_CU(cudaMemsetAsync(t->filter, 0, fwords * 4, g_stream));
    if (with_count) HG_CU(cudaMemsetAsync(t->cnt, 0, t->cap * 4, g_stream));
    HG_CU(cudaMemsetAsync(t->special, 0xff, 4, g_stream));
    HG_CU(cudaMemsetAsync(t->special + 1, 0, 12, g_stream));
    return 0;
}

// Builds the table of x's keys.  Integer keys whose range is at most 8n
// (and below 2^31) use direct addressing; others hash.
template <typename K>
// `dense_unfiltered`: a direct table whose keys fill at least half of their
// range gets no presence filter (index_of then reads the row word alone).
static I table_build(Table<K>* t, const void* x, int typ, long long n, bool with_count, bool dense_unfiltered = false) {
    int direct = 0;
    long long kmin = 0, kmax = -1;
    if (n > 0 && (typ == H_J || typ == H_H || typ == H_I || typ == H_L)) {
        long long* mm = (long long*)salloc(16);
        if (!mm) return E_DEVICE_OOM;
        long long init[2] = {LLONG_MAX, LLONG_MIN};
        HG_CU(cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, g_stream));
        unsigned g = grid_for(n, 256);
        if (g > (unsigned)g_sms * 8) g = g_sms * 8;
        HG_LAUNCH("key_minmax", g, 256, 0, k_key_minmax, x, typ, n, mm);
        long long h[2];
        HG_CHECK(rb_queue(h, mm, 16));
        HG_CU(stream_sync());
        unsigned long long range = (unsigned long long)h[1] - (unsigned long long)h[0] + 1ull;
        unsigned long long lim = 8ull * (unsigned long long)n;
        if (lim < (1ull << 16)) lim = 1ull << 16;
        if (range <= lim && range < (1ull << 31)) { direct = 1; kmin = h[0]; kmax = h[1]; }
    }
    const bool filter = !(dense_unfiltered && direct && 2 * n >= kmax - kmin + 1);
    HG_CHECK(table_create<K>(t, n, with_count, direct, kmin, kmax, filter));
    if (n > 0) {
        unsigned grid = grid_for(n, 256);
        if (grid > (unsigned)g_sms * 16) grid = g_sms * 16;
        HG_LAUNCH("hash_build", grid, 256, 0, k_build<K>, *t, x, typ, n, g_derr);
        HG_CHECK(last_launch_error());
    }
    return 0;
}

static bool key64(I typ) { return typ == H_L || typ == H_E; }

// ------------------------------------------------------------------ index_of
// Optional miss flag: set when some probe found no equal key (its index is
// len(x)).  pfnEnum turns that into E_ENUM_INDEX (h_primitive.cc:2204).
// Every lane of a warp reaches the call (the grid-stride loops exit
// uniformly), so one ballot per warp suffices.
__device__ __forceinline__ void note_miss(unsigned* miss, bool missed) {
    if (miss && __any_sync(0xffffffffu, missed) && lane_id() == 0) atomicOr(miss, 1u);
}
template <typename K>
__global__ void k_index_of(Table<K> t, const void* __restrict__ y, int typ, long long n, long long lenX,
                           long long* __restrict__ z, unsigned* miss) {
    bool missed = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        long long r = lenX;
        if (key_at<K>(y, typ, i, &k)) {
            long long row;
            if (table_find<K>(t, k, &row) != -1) r = row;
        }
        z[i] = r;
        missed |= r >= lenX;
    }
    note_miss(miss, missed);
}

// has_up / has_down over adjacent pairs (isOrdered, h_system.cc:678-698),
// plus bit 4 when some adjacent pair is equal (a strictly increasing x has
// flags == 1)
template <typename T>
__global__ void k_order_flags(const T* __restrict__ x, long long n, unsigned* flags) {
    bool up = false, down = false, eq = false;
    for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        T a = x[i - 1], b = x[i];
        up |= b > a;
        down |= b < a;
        eq |= b == a;
    }
    if (__any_sync(0xffffffffu, up) && lane_id() == 0) atomicOr(flags, 1u);
    if (__any_sync(0xffffffffu, down) && lane_id() == 0) atomicOr(flags, 2u);
    if (__any_sync(0xffffffffu, eq) && lane_id() == 0) atomicOr(flags, 4u);
}

// Strictly increasing x: a key has one index, so any exact search returns
// what the reference's binary search returns.  Instead of ~log2(n)
// dependent loads per probe, a bucket table over the key range narrows each
// search to a few keys: bucket b = (key - x0) >> s holds x[bst[b] .. bst[b+1]),
// with about four keys per bucket, so a probe reads two adjacent table words
// and usually one line of x.
__device__ __forceinline__ unsigned long long bucket_of(long long v, long long x0, int s) {
    return ((unsigned long long)v - (unsigned long long)x0) >> s;
}
// bst[b] = first index of bucket b, for every non-empty bucket (rest stay ~0u)
template <typename T>
__global__ void k_bucket_firsts(const T* __restrict__ x, long long n, long long x0, int s, unsigned* __restrict__ bst,
                                unsigned long long nb) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long b = bucket_of((long long)x[i], x0, s);
        if (i == 0 || bucket_of((long long)x[i - 1], x0, s) != b) bst[b] = (unsigned)i;
        if (i == n - 1) bst[nb] = (unsigned)n;
    }
}
// empty bucket b: the first index whose key is >= the bucket's first value
template <typename T>
__global__ void k_bucket_fill(const T* __restrict__ x, long long n, long long x0, int s, unsigned* __restrict__ bst,
                              unsigned long long nb) {
    for (unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; b < nb;
         b += (unsigned long long)gridDim.x * blockDim.x) {
        if (bst[b] != ~0u) continue;
        const long long start = (long long)((unsigned long long)x0 + (b << s));
        long long lo = 0, hi = n;
        while (lo < hi) {
            long long mid = (lo + hi) >> 1;
            if ((long long)x[mid] < start) lo = mid + 1; else hi = mid;
        }
        bst[b] = (unsigned)lo;
    }
}
template <typename T>
__global__ void k_search_bucketed(const T* __restrict__ x, long long lenX, long long x0, long long xl, int s,
                                  const unsigned* __restrict__ bst, const void* __restrict__ y, int ytyp, long long n,
                                  long long* __restrict__ z, unsigned* miss) {
    bool missed = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v;
        switch (ytyp) {
        case H_B: v = ((const bool*)y)[i]; break;
        case H_J: v = ((const int8_t*)y)[i]; break;
        case H_H: v = ((const int16_t*)y)[i]; break;
        case H_I: v = ((const int32_t*)y)[i]; break;
        default: v = ((const long long*)y)[i]; break;
        }
        long long r = lenX;
        if (v >= x0 && v <= xl) {
            const unsigned long long b = bucket_of(v, x0, s);
            unsigned lo = __ldg(bst + b), hi = __ldg(bst + b + 1);
            while (lo < hi) {
                unsigned mid = (lo + hi) >> 1;
                if ((long long)x[mid] < v) lo = mid + 1; else hi = mid;
            }
            if (lo < (unsigned long long)lenX && (long long)x[lo] == v) r = lo;
        }
        z[i] = r;
        missed |= r >= lenX;
    }
    note_miss(miss, missed);
}

__device__ __forceinline__ long long probe_val(const void* __restrict__ y, int ytyp, long long i) {
    switch (ytyp) {
    case H_B: return ((const bool*)y)[i];
    case H_J: return ((const int8_t*)y)[i];
    case H_H: return ((const int16_t*)y)[i];
    case H_I: return ((const int32_t*)y)[i];
    default: return ((const long long*)y)[i];
    }
}

// Strictly increasing keys over a range of at most 8 per key: a rank table.
// Word w covers keys x0 + 64w .. x0 + 64w + 63 and holds {bit set of the
// keys present, index of the first of them}, so the index of key v is
// first + popcount(bits below v's bit): one 16-byte read per probe from a
// table of at most 2 bytes per key (L2 resident for tens of millions of keys).
template <typename T>
__global__ void k_rank_bits(const T* __restrict__ x, long long x0, const unsigned* __restrict__ bst, unsigned long long nw,
                            ulonglong2* __restrict__ ent) {
    for (unsigned long long w = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; w < nw;
         w += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned lo = bst[w], hi = bst[w + 1];
        unsigned long long bits = 0;
        for (unsigned i = lo; i < hi; i++) bits |= 1ull << (((unsigned long long)(long long)x[i] - (unsigned long long)x0) & 63u);
        ent[w] = make_ulonglong2(bits, (unsigned long long)lo);
    }
}
__global__ void k_search_rank(long long x0, long long xl, const ulonglong2* __restrict__ ent, const void* __restrict__ y,
                              int ytyp, long long n, long long lenX, long long* __restrict__ z, unsigned* miss) {
    bool missed = false;
#pragma unroll 1
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long v = probe_val(y, ytyp, i);
        long long r = lenX;
        if (v >= x0 && v <= xl) {
            const unsigned long long d = (unsigned long long)v - (unsigned long long)x0;
            const ulonglong2 e = __ldg(ent + (d >> 6));
            const unsigned bit = (unsigned)(d & 63u);
            if ((e.x >> bit) & 1ull) r = (long long)e.y + __popcll(e.x & ((1ull << bit) - 1ull));
        }
        z[i] = r;
        missed |= r >= lenX;
    }
    note_miss(miss, missed);
}

// index_of on a direct-addressed table.  Dense keys (FILTER false): the row
// word alone says present or absent (~0u), one read per probe.  Sparse keys,
// where most probes miss: the presence filter first, a row only for hits.
template <typename K, bool FILTER>
__global__ void k_index_of_direct(const unsigned* __restrict__ rows, const unsigned* __restrict__ filter, long long kmin,
                                  long long kmax, const void* __restrict__ y, int typ, long long n, long long lenX,
                                  long long* __restrict__ z, unsigned* miss) {
    bool missed = false;
#pragma unroll 1
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        long long r = lenX;
        if (key_at<K>(y, typ, i, &k)) {
            const long long v = key_signed<K>(k);
            if (v >= kmin && v <= kmax) {
                const long long off = v - kmin;
                bool cand = true;
                if constexpr (FILTER) cand = (__ldg(filter + (off >> 5)) >> (off & 31)) & 1u;
                if (cand) {
                    const unsigned rr = __ldg(rows + off);
                    if (rr != 0xffffffffu) r = rr;
                }
            }
        }
        z[i] = r;
        missed |= r >= lenX;
    }
    note_miss(miss, missed);
}

// binarySearch_I/L (h_system.cc:715-729) and searchOrdered (:731-745); y is
// read as words of `ytyp` (x's type, as the reference reads it)
template <typename T>
__global__ void k_search_ordered(const T* __restrict__ x, long long lenX, const void* __restrict__ y, int ytyp,
                                 long long n, long long* __restrict__ z, unsigned* miss) {
    bool missed = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v;
        switch (ytyp) {
        case H_B: v = ((const bool*)y)[i]; break;
        case H_J: v = ((const int8_t*)y)[i]; break;
        case H_H: v = ((const int16_t*)y)[i]; break;
        case H_I: v = ((const int32_t*)y)[i]; break;
        default: v = ((const long long*)y)[i]; break;
        }
        long long r = lenX;
        if (lenX > 0) {
            long long lo = 0, hi = lenX;
            for (;;) {
                long long mid = (lo + hi) >> 1;
                long long xm = (long long)x[mid];
                if (xm == v) { r = mid; break; }
                if (lo == mid) break;
                if (xm > v) hi = mid; else lo = mid;
            }
        }
        z[i] = r;
        missed |= r >= lenX;
    }
    note_miss(miss, missed);
}

__global__ void k_first_false(const bool* __restrict__ x, long long n, unsigned long long* first) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!x[i]) atomicMin(first, (unsigned long long)i);
}
__global__ void k_index_of_bool(const bool* __restrict__ y, long long n, const unsigned long long* first,
                                long long lenX, long long* __restrict__ z, unsigned* miss) {
    long long f = (*first == ~0ull) ? lenX : (long long)*first;
    bool missed = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long r = y[i] ? 0 : f;
        z[i] = r;
        missed |= r >= lenX;
    }
    note_miss(miss, missed);
}

static unsigned grid_cap(long long n) {
    unsigned g = grid_for(n, 256);
    return g > (unsigned)g_sms * 16 ? (unsigned)g_sms * 16 : g;
}

// ------------------------------------------------------------------ member
template <typename K>
__global__ void k_member(Table<K> t, const void* __restrict__ y, int typ, long long n, bool* __restrict__ z) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        bool r = false;
        long long row;
        if (key_at<K>(y, typ, i, &k)) r = table_find<K>(t, k, &row) != -1;
        z[i] = r;
    }
}

// sets of one or two elements: direct == compares (lib_member_fast1/2, h_libs.cc:900-945)
template <typename T>
__global__ void k_member_small(const T* __restrict__ y, long long n, T a, T b, int m, bool* __restrict__ z) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        T v = y[i];
        z[i] = (m >= 1 && v == a) || (m >= 2 && v == b);
    }
}
__global__ void k_member_bool(const bool* __restrict__ x, long long nx, const bool* __restrict__ y, long long n,
                              unsigned* seen, bool* __restrict__ z, int phase) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (phase ? n : nx); i += (long long)gridDim.x * blockDim.x) {
        if (phase == 0) atomicOr(seen, x[i] ? 2u : 1u);
        else z[i] = (*seen & (y[i] ? 2u : 1u)) != 0;
    }
}

// ------------------------------------------------------------------ join
constexpr int JT_THREADS = 256;

// mode 0: hash table with unique build keys; mode 1: linear scan of a build
// side of < 10 rows keeping the first match (eq = op 4, neq = op 5)
struct LinearBuild {
    long long k[10];
    int n;
    int eq;
};

template <typename K>
__device__ __forceinline__ bool key_stream(const void* p, int typ, long long i, K* k) {
    switch (typ) {  // streaming loads: the probe column is read once, keep the table in L2
    case H_I: *k = (K)(long long)__ldcs((const int*)p + i); return true;
    case H_L: *k = (K)__ldcs((const long long*)p + i); return true;
    default: return key_at<K>(p, typ, i, k);
    }
}

// One pass per tile of 256 x R probe rows.  Each warp owns 32 x R
// consecutive rows (lane l: rows l, l+32, ...) and looks them up 8 at a time
// with all their reads in flight together (streamed key, presence-filter
// bit, then the build row of the candidates), keeping the build rows in
// registers.  Each warp then takes its output offset from its own decoupled
// look-back over the warp sub-tiles (no block barrier: while one warp waits
// for its prefix the others keep loading) and writes the (build row, probe
// row) pairs with ballot/popc.  R (8, 16 or 32) is the autotuner's tile knob.
template <typename K, int R>
__global__ void __launch_bounds__(JT_THREADS, (R > 16 ? 2 : 4)) k_join_probe(
    Table<K> t, LinearBuild lin, int mode, const void* __restrict__ y, int ytyp, long long n,
    long long* __restrict__ zb, long long* __restrict__ zp, unsigned long long* status, unsigned* ticket,
    unsigned long long* total, unsigned* derr) {
    constexpr long long SUB = 32LL * R;  // rows per warp sub-tile
    __shared__ long long tile_id;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) tile_id = atomicAdd(ticket, 1u);
    __syncthreads();
    const long long sub = tile_id * (JT_THREADS / 32) + warp, base = sub * SUB;
    unsigned hit[R];  // build row of each of the lane's R probe rows, 0xffffffff if none
    unsigned cnt = 0;
#pragma unroll
    for (int h8 = 0; h8 < R; h8 += 8) {
        K key[8];
        bool valid[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            long long i = base + (h8 + k) * 32 + lane;
            valid[k] = i < n && key_stream<K>(y, ytyp, i, &key[k]);
        }
        if (mode == 0) {
            long long slot[8];
            unsigned r8[8];
            table_find_n<K, 8>(t, key, valid, slot, r8);
#pragma unroll
            for (int k = 0; k < 8; k++) hit[h8 + k] = r8[k];
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                unsigned r = 0xffffffffu;
#pragma unroll
                for (int j = 9; j >= 0; j--) {  // first match wins: scan backwards, keep the last hit
                    bool m = lin.eq ? ((K)lin.k[j] == key[k]) : ((K)lin.k[j] != key[k]);
                    if (valid[k] && j < lin.n && m) r = (unsigned)j;
                }
                hit[h8 + k] = r;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < R; k++) cnt += __popc(__ballot_sync(0xffffffffu, hit[k] != 0xffffffffu));
    const unsigned long long excl = lookback_exclusive(status, sub, cnt, derr);
    if (lane == 0 && base < n && base + SUB >= n) *total = excl + cnt;  // the sub-tile holding row n-1
    unsigned long long off = excl;
#pragma unroll
    for (int k = 0; k < R; k++) {
        bool sel = hit[k] != 0xffffffffu;
        unsigned bal = __ballot_sync(0xffffffffu, sel);
        if (sel) {
            long long o = (long long)off + __popc(bal & lanemask_lt());
            __stcs(zb + o, (long long)hit[k]);
            __stcs(zp + o, base + k * 32 + lane);
        }
        off += __popc(bal);
    }
}

// duplicate build keys: CSR of build rows per slot, filled then sorted per slot
template <typename K>
__global__ void k_csr_fill(Table<K> t, const void* __restrict__ x, int typ, long long n,
                           const unsigned long long* __restrict__ start, unsigned* fillc, unsigned* rows) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        if (!key_at<K>(x, typ, i, &k)) continue;
        long long row;
        long long s = table_find<K>(t, k, &row);
        long long slot = s >= 0 ? s : (long long)t.cap;  // special slot stored last
        unsigned p = atomicAdd(&fillc[slot], 1u);
        rows[start[slot] + p] = (unsigned)i;
    }
}
template <typename K>
__global__ void k_slot_counts(Table<K> t, const void* __restrict__ x, int typ, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        if (!key_at<K>(x, typ, i, &k)) continue;
        long long row;
        long long s = table_find<K>(t, k, &row);
        if (s >= 0) atomicAdd(&t.cnt[s], 1u);
    }
}
__global__ void k_csr_sort(const unsigned long long* __restrict__ start, const unsigned* __restrict__ cnt,
                           long long nslots, unsigned* rows) {
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nslots; s += (long long)gridDim.x * blockDim.x) {
        unsigned c = cnt[s];
        if (c < 2) continue;
        unsigned* r = rows + start[s];
        for (unsigned a = 1; a < c; a++) {  // insertion sort: per-slot lists are short
            unsigned v = r[a];
            long long b = (long long)a - 1;
            while (b >= 0 && r[b] > v) { r[b + 1] = r[b]; b--; }
            r[b + 1] = v;
        }
    }
}
template <typename K>
__global__ void k_join_count(Table<K> t, const void* __restrict__ y, int ytyp, long long n,
                             unsigned* __restrict__ c, unsigned* __restrict__ slot) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        K k;
        unsigned cc = 0, ss = 0;
        if (key_at<K>(y, ytyp, i, &k)) {
            long long row;
            long long s = table_find<K>(t, k, &row);
            if (s >= 0) { cc = t.cnt[s]; ss = (unsigned)s; }
            else if (s == -2) { cc = t.special[1]; ss = (unsigned)t.cap; }
        }
        c[i] = cc;
        slot[i] = ss;
    }
}
__global__ void k_join_write(const unsigned* __restrict__ c, const unsigned* __restrict__ slot,
                             const unsigned long long* __restrict__ off, long long n,
                             const unsigned long long* __restrict__ start, const unsigned* __restrict__ rows,
                             long long* __restrict__ zb, long long* __restrict__ zp) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned cc = c[i];
        unsigned long long o = off[i], s0 = start[slot[i]];
        for (unsigned q = 0; q < cc; q++) { zb[o + q] = rows[s0 + q]; zp[o + q] = i; }
    }
}

// Writes the two i64 index vectors of a join into z (a 2-element list).
static I join_outputs(V z, long long m, long long** zb, long long** zp) {
    HG_CHECK(init_list(z, H_G, 2));
    V0* e = host_nodes(z);
    void *b, *p;
    HG_CHECK(alloc_out(&e[0], H_L, m, &b));
    HG_CHECK(alloc_out(&e[1], H_L, m, &p));
    *zb = (long long*)b;
    *zp = (long long*)p;
    return 0;
}

// Asynchronous copies global -> shared (cp.async, 4 bytes): a load that holds
// no register while in flight, so a thread can keep all of its lookups
// outstanding at once.  Each thread reads back only the slots it filled.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Probe of a direct-addressed table with i32 keys (the common shape: a
// dimension's dense integer key), in two passes with no dependence between
// tiles.  A tile is 256 x R probe rows; warp w owns rows [32 R w, 32 R (w+1))
// of it, lane l row 32 k + l of its k-th round.
I scan_counts(const unsigned* counts, long long n, unsigned long long* offs);

// Pass 1 reads the probe keys, one word of the presence filter per key (L2)
// and the build row of each match (a row-array word), and writes the warp's
// (build row, probe row - warp base) pairs as two u32 words, compacted in
// probe order, into the warp's own region of a staging buffer (32 R pairs),
// with the warp's count, its offset within the tile and the tile's count.
// Pass 2, after the scan of the tile counts, copies each warp's pairs to its
// offset as i64 pairs.  (An earlier pass 2 re-read the probe keys of the
// matching rows and the row array from a bit per row: 0.066 ms against
// 0.172 ms for this copy at 60M probes, 8.67M matches.)
template <int R>
__global__ void __launch_bounds__(JT_THREADS) k_jp_stage(Table<unsigned> t, const int* __restrict__ y, long long n,
                                                         uint2* __restrict__ stage, unsigned* __restrict__ wcounts,
                                                         unsigned* __restrict__ wpre, unsigned* __restrict__ tcounts) {
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long wid = (long long)blockIdx.x * (JT_THREADS / 32) + warp;
    const long long base = wid * (32 * R);
    const unsigned long long range = (unsigned long long)(t.kmax - t.kmin);  // < 2^31 in direct mode
    unsigned off[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        long long i = base + k * 32 + lane;
        long long v = i < n ? (long long)__ldcs(y + i) - t.kmin : -1;
        off[k] = (unsigned long long)v <= range ? (unsigned)v : 0xffffffffu;
    }
    unsigned word[R];
#pragma unroll
    for (int k = 0; k < R; k++) word[k] = off[k] != 0xffffffffu ? __ldg(t.filter + (off[k] >> 5)) : 0u;
    const unsigned* rows = (const unsigned*)t.slots;
    unsigned r[R];
    bool hit[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        hit[k] = off[k] != 0xffffffffu && ((word[k] >> (off[k] & 31)) & 1u);
        r[k] = hit[k] ? __ldg(rows + off[k]) : 0u;
    }
    uint2* out = stage + base;
    unsigned pos = 0;
#pragma unroll
    for (int k = 0; k < R; k++) {
        const unsigned bal = __ballot_sync(0xffffffffu, hit[k]);
        if (hit[k]) out[pos + __popc(bal & lanemask_lt())] = make_uint2(r[k], (unsigned)(k * 32 + lane));
        pos += __popc(bal);
    }
    // the warp's count, its offset within the tile, and the tile's count
    __shared__ unsigned wc[JT_THREADS / 32];
    if (lane == 0) wc[warp] = pos;
    __syncthreads();
    if (threadIdx.x < JT_THREADS / 32) {
        unsigned before = 0, tot = 0;
        for (int v = 0; v < JT_THREADS / 32; v++) {
            before += v < (int)threadIdx.x ? wc[v] : 0u;
            tot += wc[v];
        }
        const long long w2 = (long long)blockIdx.x * (JT_THREADS / 32) + threadIdx.x;
        wcounts[w2] = wc[threadIdx.x];
        wpre[w2] = before;
        if (threadIdx.x == 0) tcounts[blockIdx.x] = tot;
    }
}

// The same pass 1 with the presence bitmap held in the shared memory of a
// thread-block cluster: CTA r of a cluster of QC keeps bitmap words
// [r * per, (r + 1) * per), and a probe reads its key's word from the owning
// CTA's shared memory (distributed shared memory) instead of L1/L2.  The
// grid is persistent (tiles strided by gridDim.x); every CTA waits at the
// cluster barrier before it exits, so no CTA's shared memory goes away while
// another may still read it.  Outputs are those of k_jp_stage, tile for tile.
constexpr int QC = 16;
template <int R>
__global__ void __launch_bounds__(JT_THREADS) k_jp_stage_dsmem(Table<unsigned> t, const int* __restrict__ y, long long n,
                                                               long long ntiles, unsigned nwords, int shift,
                                                               uint2* __restrict__ stage, unsigned* __restrict__ wcounts,
                                                               unsigned* __restrict__ wpre, unsigned* __restrict__ tcounts) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) unsigned qs_bits[];
    __shared__ const unsigned* peer[QC];
    __shared__ unsigned wc[JT_THREADS / 32];
    cg::cluster_group cl = cg::this_cluster();
    const unsigned rank = cl.block_rank();
    const unsigned per = 1u << shift;
    {  // this CTA's slice of the bitmap
        const unsigned w0 = rank * per;
        for (unsigned i = threadIdx.x; i < per; i += JT_THREADS) qs_bits[i] = w0 + i < nwords ? t.filter[w0 + i] : 0u;
        if (threadIdx.x < QC) peer[threadIdx.x] = cl.map_shared_rank(qs_bits, threadIdx.x);
    }
    cl.sync();
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const unsigned long long range = (unsigned long long)(t.kmax - t.kmin);
    const unsigned* rows = (const unsigned*)t.slots;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long wid = tile * (JT_THREADS / 32) + warp;
        const long long base = wid * (32 * R);
        unsigned off[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            long long i = base + k * 32 + lane;
            long long v = i < n ? (long long)__ldcs(y + i) - t.kmin : -1;
            off[k] = (unsigned long long)v <= range ? (unsigned)v : 0xffffffffu;
        }
        unsigned word[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            const unsigned wi = off[k] >> 5;
            word[k] = off[k] != 0xffffffffu ? peer[wi >> shift][wi & (per - 1)] : 0u;
        }
        unsigned r[R];
        bool hit[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            hit[k] = off[k] != 0xffffffffu && ((word[k] >> (off[k] & 31)) & 1u);
            r[k] = hit[k] ? __ldg(rows + off[k]) : 0u;
        }
        uint2* out = stage + base;
        unsigned pos = 0;
#pragma unroll
        for (int k = 0; k < R; k++) {
            const unsigned bal = __ballot_sync(0xffffffffu, hit[k]);
            if (hit[k]) out[pos + __popc(bal & lanemask_lt())] = make_uint2(r[k], (unsigned)(k * 32 + lane));
            pos += __popc(bal);
        }
        if (lane == 0) wc[warp] = pos;
        __syncthreads();
        if (threadIdx.x < JT_THREADS / 32) {
            unsigned before = 0, tot = 0;
            for (int v = 0; v < JT_THREADS / 32; v++) {
                before += v < (int)threadIdx.x ? wc[v] : 0u;
                tot += wc[v];
            }
            const long long w2 = tile * (JT_THREADS / 32) + threadIdx.x;
            wcounts[w2] = wc[threadIdx.x];
            wpre[w2] = before;
            if (threadIdx.x == 0) tcounts[tile] = tot;
        }
        __syncthreads();
    }
    cl.sync();
}

int g_join_filter = 0;  // 0: presence bitmap read through L2; 1: held in a cluster's shared memory

// Launches k_jp_stage_dsmem when the bitmap fits the shared memory of a
// cluster of QC CTAs and such clusters can be resident; *ok = false otherwise.
template <int R>
static I launch_stage_dsmem(const Table<unsigned>& t, const int* y, long long ny, long long ntiles, uint2* stage,
                            unsigned* wcounts, unsigned* wpre, unsigned* tcounts, bool* ok) {
    *ok = false;
    const unsigned long long range = (unsigned long long)(t.kmax - t.kmin) + 1;
    const unsigned long long nwords = (range + 31) / 32;
    int shift = 0;  // words per CTA: the power of two covering a QC-th of the bitmap
    while ((unsigned long long)QC << shift < nwords) shift++;
    const size_t smem = (size_t)4 << shift;
    if (smem > 128 * 1024) return 0;
    auto kern = k_jp_stage_dsmem<R>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = QC;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(JT_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = g_stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(QC * 256);
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, (void*)kern, &cfg) != cudaSuccess || nclusters < 1) {
        cudaGetLastError();
        return 0;
    }
    cfg.gridDim = dim3((unsigned)(QC * nclusters));
    {
        LaunchScope ls("join_probe");
        if (cudaLaunchKernelEx(&cfg, kern, t, y, ny, ntiles, (unsigned)nwords, shift, stage, wcounts, wpre, tcounts) !=
            cudaSuccess) {
            cudaGetLastError();  // not launched: the caller takes the L2 kernel
            return 0;
        }
    }
    *ok = true;
    return 0;
}

// Pass 2: one warp per four staged warps.  Lanes 0-3 read the four counts
// and offsets; the first 32 pairs of all four regions are loaded before any
// is stored (a region rarely holds more), so four loads are in flight per lane.
constexpr int JU_GROUP = 4;
__global__ void __launch_bounds__(256) k_jp_unstage(const uint2* __restrict__ stage, const unsigned* __restrict__ wcounts,
                                                    const unsigned* __restrict__ wpre,
                                                    const unsigned long long* __restrict__ toffs, long long nwarps, int per,
                                                    long long* __restrict__ zb, long long* __restrict__ zp) {
    const unsigned lane = lane_id();
    const long long w0 = ((long long)blockIdx.x * 8 + (threadIdx.x >> 5)) * JU_GROUP;
    if (w0 >= nwarps) return;
    unsigned myc = 0;
    unsigned long long myo = 0;
    if (lane < JU_GROUP && w0 + lane < nwarps) {
        myc = wcounts[w0 + lane];
        myo = toffs[(w0 + lane) / (JT_THREADS / 32)] + wpre[w0 + lane];
    }
    unsigned c[JU_GROUP];
    unsigned long long o[JU_GROUP];
    uint2 p[JU_GROUP];
#pragma unroll
    for (int q = 0; q < JU_GROUP; q++) {
        c[q] = __shfl_sync(0xffffffffu, myc, q);
        o[q] = __shfl_sync(0xffffffffu, myo, q);
        p[q] = lane < c[q] ? __ldcs(stage + (w0 + q) * per + lane) : make_uint2(0u, 0u);
    }
#pragma unroll
    for (int q = 0; q < JU_GROUP; q++) {
        const long long base = (w0 + q) * per;
        if (lane < c[q]) {
            __stcs(zb + o[q] + lane, (long long)p[q].x);
            __stcs(zp + o[q] + lane, base + (long long)p[q].y);
        }
        for (unsigned i = lane + 32; i < c[q]; i += 32) {
            const uint2 t = __ldcs(stage + base + i);
            __stcs(zb + o[q] + i, (long long)t.x);
            __stcs(zp + o[q] + i, base + (long long)t.y);
        }
    }
}

template <int R>
static I probe_direct_staged(const Table<unsigned>& t, const int* y, long long ny, long long ntiles, long long* zb,
                             long long* zp, unsigned long long* m) {
    const long long nwarps = ntiles * (JT_THREADS / 32);
    uint2* stage = (uint2*)salloc((size_t)nwarps * 32 * R * sizeof(uint2));
    unsigned* wcounts = (unsigned*)salloc((size_t)nwarps * 4);
    unsigned* wpre = (unsigned*)salloc((size_t)nwarps * 4);
    unsigned* tcounts = (unsigned*)salloc((size_t)ntiles * 4);
    unsigned long long* toffs = (unsigned long long*)salloc((size_t)(ntiles + 1) * 8);
    if (!stage || !wcounts || !wpre || !tcounts || !toffs) return E_DEVICE_OOM;
    bool done = false;
    if (g_join_filter == 1) HG_CHECK(launch_stage_dsmem<R>(t, y, ny, ntiles, stage, wcounts, wpre, tcounts, &done));
    if (!done) HG_LAUNCH("join_probe", (unsigned)ntiles, JT_THREADS, 0, k_jp_stage<R>, t, y, ny, stage, wcounts, wpre, tcounts);
    HG_CHECK(scan_counts(tcounts, ntiles, toffs));
    HG_LAUNCH("join_emit", (unsigned)((nwarps + 8 * JU_GROUP - 1) / (8 * JU_GROUP)), 256, 0, k_jp_unstage, (const uint2*)stage,
              (const unsigned*)wcounts, (const unsigned*)wpre, (const unsigned long long*)toffs, nwarps, 32 * R, zb, zp);
    HG_CHECK(last_launch_error());
    return rb_queue(m, toffs + ntiles, 8);  // read by the caller's check_device_errors
}

// s: one status word per warp sub-tile, then the tile ticket and the total
template <typename K, int R>
static I launch_probe(const Table<K>& t, const LinearBuild& lin, int mode, const void* py, I ytyp, long long ny,
                      long long* zb, long long* zp, char* s, long long ntiles) {
    const long long nsub = ntiles * (JT_THREADS / 32);
    unsigned long long* total = (unsigned long long*)(s + nsub * 8 + 8);
    HG_LAUNCH("join_probe", (unsigned)ntiles, JT_THREADS, 0, (k_join_probe<K, R>), t, lin, mode, py, (int)ytyp, ny, zb,
              zp, (unsigned long long*)s, (unsigned*)(s + nsub * 8), total, g_derr);
    return last_launch_error();
}

// Probe in one pass with compaction, writing straight into the two output
// vectors: both are allocated for ny rows, the second (the last allocation)
// shrinks to the m matches afterwards, the first keeps its unused tail until
// the arena is rewound.  No copy of the pairs is made.
// With `repeat_flag` (the build's repeated-key word) the probe runs before
// the build is known to be unique and the flag comes back with the match
// count: when it is set, *repeated is set and nothing is returned in z.
template <typename K>
static I join_probe_unique(V z, const Table<K>& t, const LinearBuild& lin, int mode, const void* py, I ytyp,
                           long long ny, long long nbuild, const unsigned* repeat_flag = nullptr,
                           bool* repeated = nullptr) {
    const int R = g_tile_rows;
    const long long tile = (long long)JT_THREADS * R;
    long long ntiles = (ny + tile - 1) / tile;
    const long long mark = out_mark();
    unsigned rep = 0;
    const size_t cap = (size_t)(ny > 1 ? ny : 2) * 8;
    long long* zb = (long long*)dalloc(cap);
    long long* zp = (long long*)dalloc(cap);
    const long long sbytes = ntiles * (JT_THREADS / 32) * 8 + 64;
    char* s = (char*)salloc(sbytes);
    if (!zb || !zp || !s) return E_DEVICE_OOM;
    unsigned long long m = 0;
    bool direct = false;
    if constexpr (sizeof(K) == 4) direct = mode == 0 && t.direct && ytyp == H_I;
    if (ntiles > 0 && direct) {
        if constexpr (sizeof(K) == 4) {
            const int* y = (const int*)py;
            if (R == 8) HG_CHECK(probe_direct_staged<8>(t, y, ny, ntiles, zb, zp, &m));
            else if (R == 32) HG_CHECK(probe_direct_staged<32>(t, y, ny, ntiles, zb, zp, &m));
            else HG_CHECK(probe_direct_staged<16>(t, y, ny, ntiles, zb, zp, &m));
        }
        if (repeat_flag) HG_CHECK(rb_queue(&rep, repeat_flag, 4));
        HG_CHECK(check_device_errors());
    } else if (ntiles > 0) {
        HG_CU(cudaMemsetAsync(s, 0, sbytes, g_stream));
        if (R == 8) HG_CHECK((launch_probe<K, 8>(t, lin, mode, py, ytyp, ny, zb, zp, s, ntiles)));
        else if (R == 32) HG_CHECK((launch_probe<K, 32>(t, lin, mode, py, ytyp, ny, zb, zp, s, ntiles)));
        else HG_CHECK((launch_probe<K, 16>(t, lin, mode, py, ytyp, ny, zb, zp, s, ntiles)));
        HG_CHECK(rb_queue(&m, s + sbytes - 56, 8));
        if (repeat_flag) HG_CHECK(rb_queue(&rep, repeat_flag, 4));
        HG_CHECK(check_device_errors());
    } else if (repeat_flag) {
        HG_CHECK(rb_queue(&rep, repeat_flag, 4));
        HG_CHECK(check_device_errors());
    }
    if (rep) {  // repeated build keys: the caller takes the other path
        *repeated = true;
        out_rewind(mark);
        return 0;
    }
    HG_CHECK(init_list(z, H_G, 2));
    V0* e = host_nodes(z);
    dshrink(zp, (size_t)(m > 1 ? m : 1) * 8);
    long long* outs[2] = {zb, zp};
    for (int i = 0; i < 2; i++) {
        e[i].typ = H_L;
        e[i].len = (L)m;
        e[i].g = m > 1 ? (G)outs[i] : (G)&e[i].b;
        e[i].i64 = 0;
        HG_CHECK(finish_out(&e[i], outs[i]));
    }
    register_bound(e[0].g, e[0].len, nbuild);
    register_bound(e[1].g, e[1].len, ny);
    return 0;
}

template <typename K>
static I join_hash(V z, const void* px, I typ, long long nx, const void* py, long long ny) {
    Table<K> t;
    // the per-slot row counts serve only repeated build keys: they are
    // allocated and zeroed once a repeat has been seen (a direct table of a
    // 15M-key range would otherwise clear 60 MB per join for nothing)
    HG_CHECK(table_build<K>(&t, px, typ, nx, false));
    unsigned long long nslots = t.cap + 1;  // + the side slot of 64-bit keys
    if (t.direct) {
        // a direct table: probe as if the build keys were unique and read
        // the repeated-key flag with the match count, in one round trip
        LinearBuild lin{};
        bool repeated = false;
        HG_CHECK(join_probe_unique<K>(z, t, lin, 0, py, typ, ny, nx, t.flags, &repeated));
        if (!repeated) return 0;
    } else {
        unsigned dup = 0;
        HG_CHECK(rb_queue(&dup, t.flags, 4));
        HG_CHECK(check_device_errors());
        if (!dup) {
            LinearBuild lin{};
            return join_probe_unique<K>(z, t, lin, 0, py, typ, ny, nx);
        }
    }
    t.cnt = (unsigned*)salloc(t.cap * 4);
    if (!t.cnt) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(t.cnt, 0, t.cap * 4, g_stream));
    if (nx > 0) HG_LAUNCH("slot_counts", grid_cap(nx), 256, 0, k_slot_counts<K>, t, px, (int)typ, nx);
    // duplicate build keys: CSR of build rows per slot (special slot last)
    unsigned* cnt_all = (unsigned*)salloc(nslots * 4);
    unsigned long long* start = (unsigned long long*)salloc(nslots * 8);
    unsigned* fillc = (unsigned*)salloc(nslots * 4);
    unsigned* rows = (unsigned*)salloc((size_t)(nx > 0 ? nx : 1) * 4);
    if (!cnt_all || !start || !fillc || !rows) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(cnt_all, t.cnt, t.cap * 4, cudaMemcpyDeviceToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(cnt_all + t.cap, t.special + 1, 4, cudaMemcpyDeviceToDevice, g_stream));
    HG_CU(cudaMemsetAsync(fillc, 0, nslots * 4, g_stream));
    unsigned long long tot = 0;
    HG_CHECK(scan_exclusive(cnt_all, (long long)nslots, start, &tot));
    HG_LAUNCH("csr_fill", grid_cap(nx), 256, 0, k_csr_fill<K>, t, px, (int)typ, nx, start, fillc, rows);
    HG_LAUNCH("csr_sort", grid_cap((long long)nslots), 256, 0, k_csr_sort, start, cnt_all, (long long)nslots, rows);
    unsigned* c = (unsigned*)salloc((size_t)(ny > 0 ? ny : 1) * 4);
    unsigned* slot = (unsigned*)salloc((size_t)(ny > 0 ? ny : 1) * 4);
    unsigned long long* off = (unsigned long long*)salloc((size_t)(ny > 0 ? ny : 1) * 8);
    if (!c || !slot || !off) return E_DEVICE_OOM;
    HG_LAUNCH("join_count", grid_cap(ny), 256, 0, k_join_count<K>, t, py, (int)typ, ny, c, slot);
    unsigned long long m = 0;
    HG_CHECK(scan_exclusive(c, ny, off, &m));
    long long *zb, *zp;
    HG_CHECK(join_outputs(z, (long long)m, &zb, &zp));
    V0* e = host_nodes(z);
    long long *wb = zb, *wp = zp;
    if (m <= 1) {  // one-element outputs are inline: write to scratch first
        wb = (long long*)salloc(16);
        wp = (long long*)salloc(16);
    }
    if (m > 0) HG_LAUNCH("join_write", grid_cap(ny), 256, 0, k_join_write, c, slot, off, ny, start, rows, wb, wp);
    HG_CHECK(last_launch_error());
    HG_CHECK(finish_out(&e[0], wb));
    HG_CHECK(finish_out(&e[1], wp));
    register_bound(e[0].g, e[0].len, nx);
    register_bound(e[1].g, e[1].len, ny);
    return check_device_errors();
}

static void swap2(V z) {
    V0* e = host_nodes(z);
    V0 a = e[0], b = e[1];
    e[0] = b;
    e[1] = a;
    if (is_inline(&a)) e[1].g = (G)&e[1].b;
    if (is_inline(&b)) e[0].g = (G)&e[0].b;
}

// pfnJoinIndexSingle (h_primitive.cc:1944-2040) for eq/neq over real types
static I join_single(V z, V x, V y, V f) {
    const char* name = getSymbolStr(f->q);
    int op = !strcmp(name, "lt") ? 0 : !strcmp(name, "leq") ? 1 : !strcmp(name, "gt") ? 2 : !strcmp(name, "geq") ? 3
           : !strcmp(name, "eq") ? 4 : !strcmp(name, "neq") ? 5 : -1;
    if (op < 0) return E_DOMAIN;
    if (!(is_real(x->typ) && is_real(y->typ)))
        return x->typ == y->typ ? set_error(E_NOT_IMPL, "join on this type is outside the path") : E_TYPE;
    if (op != 4 && op != 5) return set_error(E_NOT_IMPL, "non-equi single-column join is outside the path");
    I typ = x->typ > y->typ ? x->typ : y->typ;
    if (typ != H_H && typ != H_I && typ != H_L && typ != H_F && typ != H_E) return E_NOT_IMPL;
    const void *px, *py;
    long long nx = x->len, ny = y->len;
    if (nx >= 10) {  // NUM_JOIN_LINEAR (common.h:152)
        if (op != 4) return set_error(E_NOT_IMPL, "hash join supports @eq only (as the reference)");
        if (typ != H_I && typ != H_L) return set_error(E_NOT_IMPL, "hash join keys must be i32 or i64");
        HG_CHECK(promote_to(x, typ, &px));
        HG_CHECK(promote_to(y, typ, &py));
        if (typ == H_I) return join_hash<unsigned>(z, px, typ, nx, py, ny);
        return join_hash<unsigned long long>(z, px, typ, nx, py, ny);
    }
    if (typ != H_I && typ != H_L && typ != H_E) return set_error(E_NOT_IMPL, "linear join supports i32/i64/f64 keys");
    HG_CHECK(promote_to(y, typ, &py));
    // build side (< 10 rows) read on the host and passed by value
    LinearBuild lin{};
    lin.n = (int)nx;
    lin.eq = op == 4;
    if (nx > 0) {
        const void* pxd;
        HG_CHECK(promote_to(x, typ, &pxd));
        HG_CU(cudaMemcpyAsync(lin.k, pxd, nx * 8 / (typ == H_I ? 2 : 1), cudaMemcpyDefault, g_stream));
        HG_CU(stream_sync());
        if (typ == H_I) {
            int tmp[10];
            memcpy(tmp, lin.k, nx * 4);
            for (int i = 0; i < nx; i++) lin.k[i] = tmp[i];
        }
    }
    Table<unsigned long long> none{};
    if (typ == H_I) {
        Table<unsigned> n32{};
        for (int i = 0; i < lin.n; i++) lin.k[i] = (long long)(unsigned)(int)lin.k[i];
        return join_probe_unique<unsigned>(z, n32, lin, 1, py, typ, ny, nx);
    }
    return join_probe_unique<unsigned long long>(z, none, lin, 1, py, typ, ny, nx);
}

// Strictly increasing i32/i64 x of n >= 2 keys: bucket table in scratch, then the probe.
template <typename T>
static I search_bucketed_t(const T* x, long long lenX, const void* py, I ytyp, long long n, long long* z, unsigned* miss) {
    T ends[2];
    HG_CHECK(rb_queue(&ends[0], x, sizeof(T)));
    HG_CHECK(rb_queue(&ends[1], x + lenX - 1, sizeof(T)));
    HG_CU(stream_sync());
    const long long x0 = (long long)ends[0], xl = (long long)ends[1];
    const unsigned long long range = (unsigned long long)xl - (unsigned long long)x0;
    const bool rank = range < 8ull * (unsigned long long)lenX;  // rank table of <= 2 bytes per key
    int s = 6;
    if (!rank) {
        const unsigned long long target = (unsigned long long)(lenX / 4);
        s = 0;
        while ((range >> s) + 1 > target) s++;
    }
    const unsigned long long nb = (range >> s) + 1;
    unsigned* bst = (unsigned*)salloc((size_t)(nb + 1) * 4);
    if (!bst) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(bst, 0xff, (size_t)(nb + 1) * 4, g_stream));
    HG_LAUNCH("bucket_firsts", grid_cap(lenX), 256, 0, k_bucket_firsts<T>, x, lenX, x0, s, bst, nb);
    HG_LAUNCH("bucket_fill", grid_cap((long long)nb), 256, 0, k_bucket_fill<T>, x, lenX, x0, s, bst, nb);
    if (rank) {
        ulonglong2* ent = (ulonglong2*)salloc((size_t)nb * sizeof(ulonglong2));
        if (!ent) return E_DEVICE_OOM;
        HG_LAUNCH("rank_bits", grid_cap((long long)nb), 256, 0, k_rank_bits<T>, x, x0, bst, nb, ent);
        HG_LAUNCH("search_rank", grid_cap(n), 256, 0, k_search_rank, x0, xl, ent, py, (int)ytyp, n, lenX, z, miss);
    } else {
        HG_LAUNCH("search_bucketed", grid_cap(n), 256, 0, k_search_bucketed<T>, x, lenX, x0, xl, s, bst, py, (int)ytyp, n, z, miss);
    }
    return last_launch_error();
}
static I search_bucketed(const void* px, I xtyp, long long lenX, const void* py, I ytyp, long long n, long long* z,
                         unsigned* miss) {
    if (xtyp == H_I) return search_bucketed_t<int32_t>((const int32_t*)px, lenX, py, ytyp, n, z, miss);
    return search_bucketed_t<long long>((const long long*)px, lenX, py, ytyp, n, z, miss);
}

// pfnIndexOf (h_primitive.cc:1523-1579).  Real x and y: a monotone int x is
// binary searched (searchOrdered, h_system.cc:731-745), anything else is
// hashed on the promoted type (lib_index_of_*, h_libs.cc:299-373).  Dates,
// times and symbols of one type hash as the integers of their width
// (h_libs.h:25-31 maps lib_index_of_M/D/U/W/T to _I and Q/Z to _L), with no
// ordered search.  `miss` (optional, device) is set when some y has no equal x.
static I index_of(V z, V x, V y, unsigned* miss, bool force_hash = false) {
    V0 xa, ya;
    bool hash_only = force_hash;
    if (x->typ == y->typ && (is_dtime(x->typ) || x->typ == H_Q)) {
        xa = *x; ya = *y;
        xa.typ = ya.typ = esize(x->typ) == 4 ? H_I : H_L;
        if (is_inline(x)) xa.g = (G)&xa.b;
        if (is_inline(y)) ya.g = (G)&ya.b;
        x = &xa; y = &ya;
        hash_only = true;
    }
    if (!(is_real(x->typ) && is_real(y->typ)))
        return x->typ == y->typ ? set_error(E_NOT_IMPL, "index_of on this type is outside the path") : E_TYPE;
    long long lenX = x->len, n = y->len;
    void* dz;
    if (!hash_only && (x->typ == H_I || x->typ == H_L)) {
        const void* px;
        HG_CHECK(in_ptr(x, &px));
        unsigned* flags = (unsigned*)salloc(16);
        if (!flags) return E_DEVICE_OOM;
        HG_CU(cudaMemsetAsync(flags, 0, 4, g_stream));
        if (lenX > 1) {
            if (x->typ == H_I) HG_LAUNCH("order_flags", grid_cap(lenX), 256, 0, k_order_flags<int32_t>, (const int32_t*)px, lenX, flags);
            else HG_LAUNCH("order_flags", grid_cap(lenX), 256, 0, k_order_flags<long long>, (const long long*)px, lenX, flags);
        }
        unsigned fl = 0;
        HG_CHECK(rb_queue(&fl, flags, 4));
        HG_CU(stream_sync());
        if ((fl & 3) != 3) {  // monotone or constant: searchOrdered
            // The reference reads y through x's element type (vI(y,i) / vL(y,i),
            // h_system.cc:735-742): a y at least as wide is read as its first
            // len(y) words of x's width; a narrower y would be read past its end.
            if (esize(y->typ) < esize(x->typ))
                return set_error(E_TYPE, "index_of: ordered %d-byte keys probed with %d-byte values", esize(x->typ), esize(y->typ));
            const I ywords = x->typ;
            const void* py;
            HG_CHECK(in_ptr(y, &py));
            HG_CHECK(alloc_out(z, H_L, n, &dz));
            if (n > 0 && fl == 1 && lenX >= 64) {
                HG_CHECK(search_bucketed(px, x->typ, lenX, py, ywords, n, (long long*)dz, miss));
            } else if (n > 0) {
                if (x->typ == H_I) HG_LAUNCH("search_ordered", grid_cap(n), 256, 0, k_search_ordered<int32_t>, (const int32_t*)px, lenX, py, (int)ywords, n, (long long*)dz, miss);
                else HG_LAUNCH("search_ordered", grid_cap(n), 256, 0, k_search_ordered<long long>, (const long long*)px, lenX, py, (int)ywords, n, (long long*)dz, miss);
            }
            HG_CHECK(last_launch_error());
            return finish_out(z, dz);
        }
    }
    I typ = x->typ > y->typ ? x->typ : y->typ;
    const void *px, *py;
    HG_CHECK(promote_to(x, typ, &px));
    HG_CHECK(promote_to(y, typ, &py));
    HG_CHECK(alloc_out(z, H_L, n, &dz));
    if (typ == H_B) {
        unsigned long long* first = (unsigned long long*)salloc(16);
        if (!first) return E_DEVICE_OOM;
        HG_CU(cudaMemsetAsync(first, 0xff, 8, g_stream));
        if (lenX > 0) HG_LAUNCH("first_false", grid_cap(lenX), 256, 0, k_first_false, (const bool*)px, lenX, first);
        if (n > 0) HG_LAUNCH("index_of_bool", grid_cap(n), 256, 0, k_index_of_bool, (const bool*)py, n, first, lenX, (long long*)dz, miss);
        HG_CHECK(last_launch_error());
        return finish_out(z, dz);
    }
    if (key64(typ)) {
        Table<unsigned long long> t;
        HG_CHECK(table_build<unsigned long long>(&t, px, typ, lenX, false, true));
        if (n > 0 && t.direct && t.filter)
            HG_LAUNCH("index_of_direct", grid_cap(n), 256, 0, (k_index_of_direct<unsigned long long, true>),
                      (const unsigned*)t.slots, t.filter, t.kmin, t.kmax, py, (int)typ, n, lenX, (long long*)dz, miss);
        else if (n > 0 && t.direct)
            HG_LAUNCH("index_of_direct", grid_cap(n), 256, 0, (k_index_of_direct<unsigned long long, false>),
                      (const unsigned*)t.slots, t.filter, t.kmin, t.kmax, py, (int)typ, n, lenX, (long long*)dz, miss);
        else if (n > 0) HG_LAUNCH("index_of", grid_cap(n), 256, 0, k_index_of<unsigned long long>, t, py, (int)typ, n, lenX, (long long*)dz, miss);
    } else {
        Table<unsigned> t;
        HG_CHECK(table_build<unsigned>(&t, px, typ, lenX, false, true));
        if (n > 0 && t.direct && t.filter)
            HG_LAUNCH("index_of_direct", grid_cap(n), 256, 0, (k_index_of_direct<unsigned, true>),
                      (const unsigned*)t.slots, t.filter, t.kmin, t.kmax, py, (int)typ, n, lenX, (long long*)dz, miss);
        else if (n > 0 && t.direct)
            HG_LAUNCH("index_of_direct", grid_cap(n), 256, 0, (k_index_of_direct<unsigned, false>),
                      (const unsigned*)t.slots, t.filter, t.kmin, t.kmax, py, (int)typ, n, lenX, (long long*)dz, miss);
        else if (n > 0) HG_LAUNCH("index_of", grid_cap(n), 256, 0, k_index_of<unsigned>, t, py, (int)typ, n, lenX, (long long*)dz, miss);
    }
    HG_CHECK(last_launch_error());
    HG_CHECK(check_device_errors());
    return finish_out(z, dz);
}

// ---- @index_of on two lists of columns (lib_index_of_G, h_libs.cc:370-373;
// compareTuple h_system.cc:567-589): the first row of x whose every column
// equals the y row's, or len(x).  Integer columns (i8/i16/i32/i64) of the
// same type on both sides are packed into one 64-bit code per row (each
// column's offset from x's minimum, at the width of x's range), so equal
// tuples are equal codes; a y value outside x's range cannot match and gets
// a code no x row has.  The codes go through the hash path (first occurrence).
struct PackSpec {
    const void* col[8];
    int typ[8];
    long long mn[8], mx[8];
    int shift[8];
    int nc;
};
__global__ void k_pack_rows(PackSpec s, long long n, unsigned long long* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long key = 0;
        bool ok = true;
        for (int c = 0; c < s.nc; c++) {
            long long v;
            switch (s.typ[c]) {
            case H_J: v = ((const int8_t*)s.col[c])[i]; break;
            case H_H: v = ((const int16_t*)s.col[c])[i]; break;
            case H_I: v = ((const int32_t*)s.col[c])[i]; break;
            default: v = ((const long long*)s.col[c])[i]; break;
            }
            ok = ok && v >= s.mn[c] && v <= s.mx[c];
            key |= ((unsigned long long)v - (unsigned long long)s.mn[c]) << s.shift[c];
        }
        out[i] = ok ? key : ~0ull;
    }
}
__global__ void k_fill_i64(long long* __restrict__ z, long long n, long long v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) z[i] = v;
}

static I index_of_list(V z, V x, V y, unsigned* miss) {
    if (x->len != y->len) return E_DOMAIN;  // isListIndexOf, h_system.cc:591-603
    const int nc = (int)x->len;
    V0 *xc = host_nodes(x), *yc = host_nodes(y);
    const long long lenX = nc > 0 ? xc[0].len : 0, lenY = nc > 0 ? yc[0].len : 0;
    for (int c = 0; c < nc; c++)
        if (xc[c].len != lenX || yc[c].len != lenY) return E_LENGTH;
    if (nc > 8) return set_error(E_NOT_IMPL, "index_of on more than 8 columns");
    bool same_types = true;
    for (int c = 0; c < nc; c++) {
        const I tx = xc[c].typ, ty = yc[c].typ;
        if (!(tx == H_J || tx == H_H || tx == H_I || tx == H_L) || !(ty == H_J || ty == H_H || ty == H_I || ty == H_L))
            return set_error(E_NOT_IMPL, "index_of on lists holding columns of type %d/%d", tx, ty);
        same_types = same_types && tx == ty;
    }
    void* dz;
    HG_CHECK(alloc_out(z, H_L, lenY, &dz));
    if (lenY == 0) return finish_out(z, dz);
    if (!same_types || lenX == 0) {  // compareTupleItem: columns of different types never compare equal
        HG_LAUNCH("fill", grid_cap(lenY), 256, 0, k_fill_i64, (long long*)dz, lenY, lenX);
        if (miss) HG_CU(cudaMemsetAsync(miss, 0xff, 4, g_stream));
        HG_CHECK(last_launch_error());
        return finish_out(z, dz);
    }
    PackSpec xs{}, ys{};
    xs.nc = ys.nc = nc;
    long long* mm = (long long*)salloc(16);
    if (!mm) return E_DEVICE_OOM;
    int shift = 0;
    for (int c = nc - 1; c >= 0; c--) {
        const void *px, *py;
        HG_CHECK(in_ptr(&xc[c], &px));
        HG_CHECK(in_ptr(&yc[c], &py));
        long long init[2] = {LLONG_MAX, LLONG_MIN}, h[2];
        HG_CU(cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, g_stream));
        HG_LAUNCH("key_minmax", grid_cap(lenX), 256, 0, k_key_minmax, px, (int)xc[c].typ, lenX, mm);
        HG_CHECK(rb_queue(h, mm, 16));
        HG_CU(stream_sync());
        const unsigned long long span = (unsigned long long)h[1] - (unsigned long long)h[0];
        const int bits = span == 0 ? 0 : 64 - __builtin_clzll(span);
        xs.col[c] = px; ys.col[c] = py;
        xs.typ[c] = ys.typ[c] = xc[c].typ;
        xs.mn[c] = ys.mn[c] = h[0];
        xs.mx[c] = ys.mx[c] = h[1];
        xs.shift[c] = ys.shift[c] = shift;
        shift += bits;
        if (shift > 63) return set_error(E_NOT_IMPL, "index_of on lists whose columns span more than 63 bits together");
    }
    unsigned long long* kx = (unsigned long long*)salloc((size_t)(lenX > 1 ? lenX : 2) * 8);
    unsigned long long* ky = (unsigned long long*)salloc((size_t)(lenY > 1 ? lenY : 2) * 8);
    if (!kx || !ky) return E_DEVICE_OOM;
    HG_LAUNCH("pack_rows", grid_cap(lenX), 256, 0, k_pack_rows, xs, lenX, kx);
    HG_LAUNCH("pack_rows", grid_cap(lenY), 256, 0, k_pack_rows, ys, lenY, ky);
    HG_CHECK(last_launch_error());
    V0 vx{}, vy{};
    vx.typ = vy.typ = H_L;
    vx.len = lenX; vx.g = (G)kx;
    vy.len = lenY; vy.g = (G)ky;
    if (lenX == 1) { HG_CU(cudaMemcpy(&vx.b, kx, 8, cudaMemcpyDeviceToHost)); vx.g = (G)&vx.b; }
    if (lenY == 1) { HG_CU(cudaMemcpy(&vy.b, ky, 8, cudaMemcpyDeviceToHost)); vy.g = (G)&vy.b; }
    return index_of(z, &vx, &vy, miss, true);
}

}  // namespace hg

using namespace hg;

extern "C" {

I pfnIndexOf(V z, V x, V y) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (x->typ == H_G && y->typ == H_G) return index_of_list(z, x, y, nullptr);
    return index_of(z, x, y, nullptr);
}

// pfnEnum (h_primitive.cc:2198-2222): the enum of the foreign-key column y
// over the key column x.  The index is index_of(x, y) with the miss flag
// folded into the probe kernels, so the range check of :2204
// (E_ENUM_INDEX when some y has no equal key) costs no second pass.  The
// node is H_Y with len(y) and the i64 index (device, never inline) in g; its
// header {source -1, ek x, ev y} points at the caller's x and y, which must
// outlive it, as in the reference.  The index is registered as lying in
// [0, len(x)), so @index(column of x, @values(enum)) skips its bounds check.
// Two lists of the same number of columns (multi-column keys, :2210-2219)
// take the multi-column index_of.
I pfnEnum(V z, V x, V y) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    const bool lists = x->typ == H_G && y->typ == H_G;
    if (lists && x->len != y->len) return E_DOMAIN;
    if (!lists && !is_basic(x->typ)) return E_DOMAIN;
    long long mark = out_mark();
    unsigned* miss = (unsigned*)salloc(16);
    if (!miss) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(miss, 0, 4, g_stream));
    V0 ind;
    I e = lists ? index_of_list(&ind, x, y, miss) : index_of(&ind, x, y, miss);
    if (e) { out_rewind(mark); return e; }
    unsigned h = 0;
    HG_CHECK(rb_queue(&h, miss, 4));
    HG_CU(stream_sync());
    if (h) { out_rewind(mark); return E_ENUM_INDEX; }
    Y hdr = (Y)halloc(sizeof(Y0));
    if (!hdr) { out_rewind(mark); return E_DEVICE_OOM; }
    hdr->source = -1;
    hdr->ek = (G)x;
    hdr->ev = (G)y;
    G payload = ind.g;
    if (is_inline(&ind)) {
        void* d = dalloc(16);
        if (!d) { out_rewind(mark); return E_DEVICE_OOM; }
        HG_CU(cudaMemcpyAsync(d, &ind.b, 8, cudaMemcpyHostToDevice, g_stream));
        HG_CU(stream_sync());
        payload = (G)d;
    }
    z->typ = H_Y;
    z->len = ind.len;
    z->g = payload;
    z->y = hdr;
    register_bound(payload, z->len, lists ? (x->len > 0 ? host_nodes(x)[0].len : 0) : x->len);
    return apply_residency(z);
}

// pfnFetch (h_primitive.cc:219-225): copyV of the enum's value node.
I pfnFetch(V z, V x) {
    if (x->typ != H_Y || !x->y || !x->y->ev) return E_DOMAIN;
    V ev = (V)x->y->ev;
    *z = *ev;
    if (is_inline(ev)) z->g = (G)&z->b;
    return 0;
}

I pfnMember(V z, V y, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    long long n = y->len, nx = x->len;
    void* dz;
    if (is_real(x->typ) && is_real(y->typ)) {
        I typ = x->typ > y->typ ? x->typ : y->typ;
        if (typ == H_J) return set_error(E_NOT_IMPL, "member on i8 (the reference has no i8 case)");
        const void *px, *py;
        HG_CHECK(promote_to(x, typ, &px));
        HG_CHECK(promote_to(y, typ, &py));
        HG_CHECK(alloc_out(z, H_B, n, &dz));
        if (typ == H_B) {
            unsigned* seen = (unsigned*)salloc(16);
            if (!seen) return E_DEVICE_OOM;
            HG_CU(cudaMemsetAsync(seen, 0, 4, g_stream));
            if (nx > 0) HG_LAUNCH("member_bool", grid_cap(nx), 256, 0, k_member_bool, (const bool*)px, nx, (const bool*)py, n, seen, (bool*)dz, 0);
            if (n > 0) HG_LAUNCH("member_bool", grid_cap(n), 256, 0, k_member_bool, (const bool*)px, nx, (const bool*)py, n, seen, (bool*)dz, 1);
        } else if (nx <= 2) {
            uint64_t a = 0, b = 0;
            if (nx >= 1) HG_CU(cudaMemcpyAsync(&a, px, esize(typ), cudaMemcpyDefault, g_stream));
            if (nx >= 2) HG_CU(cudaMemcpyAsync(&b, (const char*)px + esize(typ), esize(typ), cudaMemcpyDefault, g_stream));
            HG_CU(stream_sync());
            int m = (int)nx;
            if (n > 0) switch (typ) {
            case H_H: HG_LAUNCH("member_small", grid_cap(n), 256, 0, k_member_small<int16_t>, (const int16_t*)py, n, *(int16_t*)&a, *(int16_t*)&b, m, (bool*)dz); break;
            case H_I: HG_LAUNCH("member_small", grid_cap(n), 256, 0, k_member_small<int32_t>, (const int32_t*)py, n, *(int32_t*)&a, *(int32_t*)&b, m, (bool*)dz); break;
            case H_L: HG_LAUNCH("member_small", grid_cap(n), 256, 0, k_member_small<long long>, (const long long*)py, n, *(long long*)&a, *(long long*)&b, m, (bool*)dz); break;
            case H_F: HG_LAUNCH("member_small", grid_cap(n), 256, 0, k_member_small<float>, (const float*)py, n, *(float*)&a, *(float*)&b, m, (bool*)dz); break;
            default: HG_LAUNCH("member_small", grid_cap(n), 256, 0, k_member_small<double>, (const double*)py, n, *(double*)&a, *(double*)&b, m, (bool*)dz); break;
            }
        } else if (key64(typ)) {
            Table<unsigned long long> t;
            HG_CHECK(table_build<unsigned long long>(&t, px, typ, nx, false));
            if (n > 0) HG_LAUNCH("member", grid_cap(n), 256, 0, k_member<unsigned long long>, t, py, (int)typ, n, (bool*)dz);
        } else {
            Table<unsigned> t;
            HG_CHECK(table_build<unsigned>(&t, px, typ, nx, false));
            if (n > 0) HG_LAUNCH("member", grid_cap(n), 256, 0, k_member<unsigned>, t, py, (int)typ, n, (bool*)dz);
        }
        HG_CHECK(last_launch_error());
        HG_CHECK(check_device_errors());
        return finish_out(z, dz);
    }
    if (x->typ == y->typ && x->typ == H_C) {  // lib_member_C (h_libs.cc:989-995): bytes as a 256-entry set
        const void *px, *py;
        HG_CHECK(in_ptr(x, &px));
        HG_CHECK(in_ptr(y, &py));
        HG_CHECK(alloc_out(z, H_B, n, &dz));
        Table<unsigned> t;
        HG_CHECK(table_build<unsigned>(&t, px, H_J, nx, false));
        if (n > 0) HG_LAUNCH("member", grid_cap(n), 256, 0, k_member<unsigned>, t, py, (int)H_J, n, (bool*)dz);
        HG_CHECK(last_launch_error());
        HG_CHECK(check_device_errors());
        return finish_out(z, dz);
    }
    if (x->typ == y->typ) return set_error(E_NOT_IMPL, "member on this type is outside the path");
    return E_DOMAIN;
}

}  // extern "C"

namespace hg {

I compact_i64_cols(const uint8_t* mask, long long n, const long long* const* src, long long** dst, int ncol,
                   long long* count);

// element i of a real column, converted to T as promoteValue converts it
template <typename T>
__device__ __forceinline__ T elem_as(const void* p, int typ, long long i) {
    switch (typ) {
    case H_B: return (T)((const bool*)p)[i];
    case H_J: case H_C: return (T)((const int8_t*)p)[i];
    case H_H: return (T)((const int16_t*)p)[i];
    case H_I: case H_M: case H_D: case H_U: case H_W: case H_T: return (T)((const int32_t*)p)[i];
    case H_F: return (T)((const float*)p)[i];
    case H_E: return (T)((const double*)p)[i];
    default: return (T)((const long long*)p)[i];
    }
}

// keep[k] = COMP(op, x[a[k]], y[b[k]]) in type T: the exact compares of
// compareOneColumn (h_system.cc:818-838, COMP h_primitive.cc:1063-1066)
template <typename T>
__global__ void k_pair_keep(const void* __restrict__ x, int xt, const void* __restrict__ y, int yt,
                            const long long* __restrict__ a, const long long* __restrict__ b, long long m, int op,
                            uint8_t* __restrict__ keep) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
        const T u = elem_as<T>(x, xt, a[k]), v = elem_as<T>(y, yt, b[k]);
        bool r;
        switch (op) {
        case 0: r = u < v; break;
        case 1: r = u <= v; break;
        case 2: r = u > v; break;
        case 3: r = u >= v; break;
        case 4: r = u == v; break;
        case 5: r = u != v; break;
        default: r = false; break;
        }
        keep[k] = r;
    }
}

static int op_of_symbol(L q) {
    const char* n = getSymbolStr(q);
    if (!n) return -1;
    return !strcmp(n, "lt") ? 0 : !strcmp(n, "leq") ? 1 : !strcmp(n, "gt") ? 2 : !strcmp(n, "geq") ? 3
         : !strcmp(n, "eq") ? 4 : !strcmp(n, "neq") ? 5 : -1;
}

// pfnJoinIndexMultiple (h_primitive.cc:2094-2110): join on the first @eq
// column (else the first @neq, else column 0) without the shorter-side swap
// (joinOneColumn, h_system.cc:856-880), then keep the pairs whose other
// columns compare true, column by column in order (joinOtherColumns,
// :846-853).  The first column's join must be an equi-join on i32/i64 keys
// (the reference's hash path; its nested-loop and non-equi joins are
// quadratic and are not reproduced).
static I join_multi(V z, V x, V y, V f) {
    if (x->typ != H_G || y->typ != H_G) return E_DOMAIN;
    const long long nc = f->len;
    if (x->len != nc || y->len != nc) return E_LENGTH;
    std::vector<L> sym((size_t)nc);
    if (is_device_ptr(f->g) && !is_inline(f))
        HG_CU(cudaMemcpy(sym.data(), f->g, (size_t)nc * 8, cudaMemcpyDeviceToHost));
    else
        memcpy(sym.data(), f->g, (size_t)nc * 8);
    std::vector<int> ops((size_t)nc);
    long long fx = -1;
    for (long long i = 0; i < nc && fx < 0; i++) if ((ops[i] = op_of_symbol(sym[i])) == 4) fx = i;
    for (long long i = 0; i < nc; i++) ops[i] = op_of_symbol(sym[i]);
    for (long long i = 0; i < nc && fx < 0; i++) if (ops[i] == 5) fx = i;
    if (fx < 0) fx = 0;
    for (long long i = 0; i < nc; i++) if (ops[i] < 0) return E_DOMAIN;
    if (ops[fx] != 4) return set_error(E_NOT_IMPL, "multi-column join without an @eq column is outside the path");
    V0* xc = host_nodes(x);
    V0* yc = host_nodes(y);
    const long long nx = xc[0].len, ny = yc[0].len;
    for (long long i = 0; i < nc; i++) {
        if (xc[i].len != nx || yc[i].len != ny) return E_LENGTH;
        if (!is_real(xc[i].typ) || !is_real(yc[i].typ)) return E_TYPE;
    }
    const I typ = xc[fx].typ > yc[fx].typ ? xc[fx].typ : yc[fx].typ;
    if (typ != H_I && typ != H_L) return set_error(E_NOT_IMPL, "hash join keys must be i32 or i64");
    const void *px, *py;
    HG_CHECK(promote_to(&xc[fx], typ, &px));
    HG_CHECK(promote_to(&yc[fx], typ, &py));
    const long long mark = out_mark();
    V0 j;
    if (typ == H_I) HG_CHECK(join_hash<unsigned>(&j, px, typ, nx, py, ny));
    else HG_CHECK(join_hash<unsigned long long>(&j, px, typ, nx, py, ny));
    V0* jn = host_nodes(&j);
    long long m = jn[0].len;
    // the pairs as device vectors (a length-1 result is inline in its node)
    long long* cur[2];
    for (int c = 0; c < 2; c++) {
        cur[c] = (long long*)salloc((size_t)(m > 0 ? m : 1) * 8);
        if (!cur[c]) return E_DEVICE_OOM;
        if (m > 0) HG_CU(cudaMemcpyAsync(cur[c], jn[c].g, (size_t)m * 8, cudaMemcpyDefault, g_stream));
    }
    uint8_t* keep = (uint8_t*)salloc((size_t)(m > 0 ? m : 1));
    long long* nxt[2] = {(long long*)salloc((size_t)(m > 0 ? m : 1) * 8), (long long*)salloc((size_t)(m > 0 ? m : 1) * 8)};
    if (!keep || !nxt[0] || !nxt[1]) return E_DEVICE_OOM;
    for (long long i = 0; i < nc && m > 0; i++) {
        if (i == fx) continue;
        const void *ax, *ay;
        HG_CHECK(in_ptr(&xc[i], &ax));
        HG_CHECK(in_ptr(&yc[i], &ay));
        const I tm = xc[i].typ > yc[i].typ ? xc[i].typ : yc[i].typ;
        const unsigned g = grid_cap(m);
        switch (tm) {
        case H_F: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<float>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        case H_E: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<double>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        case H_L: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<long long>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        case H_I: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<int>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        case H_H: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<short>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        case H_J: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<signed char>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        default: HG_LAUNCH("pair_keep", g, 256, 0, k_pair_keep<bool>, ax, (int)xc[i].typ, ay, (int)yc[i].typ, cur[0], cur[1], m, ops[i], keep); break;
        }
        long long kept = 0;
        HG_CHECK(compact_i64_cols(keep, m, (const long long* const*)cur, nxt, 2, &kept));
        std::swap(cur[0], nxt[0]);
        std::swap(cur[1], nxt[1]);
        m = kept;
    }
    out_rewind(mark);  // the single-column join's outputs
    HG_CHECK(init_list(z, H_G, 2));
    V0* e = host_nodes(z);
    for (int c = 0; c < 2; c++) {
        void* d;
        HG_CHECK(alloc_out(&e[c], H_L, m, &d));
        if (m > 0) HG_CU(cudaMemcpyAsync(d, cur[c], (size_t)m * 8, cudaMemcpyDeviceToDevice, g_stream));
        HG_CHECK(finish_out(&e[c], d));
    }
    register_bound(e[0].g, e[0].len, nx);
    register_bound(e[1].g, e[1].len, ny);
    return 0;
}

}  // namespace hg

extern "C" {

I pfnJoinIndex(V z, V x, V y, V f) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (f->len == 1) {
        if (x->len > y->len) {
            HG_CHECK(join_single(z, y, x, f));
            swap2(z);
            return 0;
        }
        return join_single(z, x, y, f);
    }
    if (f->len > 1) return join_multi(z, x, y, f);
    return E_DOMAIN;
}

}  // extern "C"
