// Stable LSD radix sort, @group and @order.
//
// Reference orderings reproduced (src/horseir/v3/backend/h_libs.cc):
//   lib_radixsort_core_int  :1184-1207  4 stable passes over the unsigned
//                           bytes of the 32-bit pattern (negatives after positives)
//   lib_radixsort_core_long :1243-1274  32 bits unless some key has
//                           (key >> 32) > 0, then 64
//   lib_radixsort_int/long  :1215-1293  descending = ascending reversed
//   checkOrderCase1         :1912-1940  two i32 columns, one direction: pack
//                           ((i64)x0 << 32) | (i64)x1 (x1 sign-extended)
//   lib_quicksort_list      :637-697    lists of i32/i64 columns: stable merge
//                           sort per column, recursing on runs of equal values
//                           = stable lexicographic order
//   lib_group_by_normal_*   :1295-1403  groups = runs of equal adjacent values
//                           in radix order; key = first row of the run
//   pfnGroupTrie            h_primitive.cc:2656-2681  counting on (c0<<8)+c1
//
// Any stable sort by the same key yields the same permutation, so the GPU
// sorts only the key bits that vary (found with one OR/AND reduction, or
// known from the value range) and packs multi-column integer keys into one
// u64 after range compression.
//
// Radix kernel: onesweep-style LSD (Adinets & Merrill 2022).  One histogram
// pass gives every digit's global bucket base for all passes; each pass
// then ranks a 4096-key tile with warp-level __match_any_sync (warps own
// contiguous sub-ranges, so ranks are stable), resolves per-digit tile
// offsets with a decoupled look-back (one thread per digit, bounded spin) or
// from counts taken by a separate pass and one scan, and scatters keys and
// row ids.
#include <cstring>
#include <vector>

#include "dev_common.cuh"

namespace hg {

I compact_rows(const uint8_t* mask, long long n, long long* out, long long* count);
I scan_exclusive(const unsigned* in, long long n, unsigned long long* out, unsigned long long* total_h);

constexpr int RS_THREADS = 256, RS_ITEMS = 16, RS_TILE = RS_THREADS * RS_ITEMS;
static int g_digit_bits = 8;  // LSD digit width, 4 - 8 bits (autotuner knob)
void set_radix_digit_bits(int b) { g_digit_bits = b < 4 ? 4 : (b > 8 ? 8 : b); }
int get_radix_digit_bits() { return g_digit_bits; }
// how a pass finds each tile's offset per digit (autotuner knob): 0 a
// decoupled look-back over the preceding tiles, 1 a counting pass over the
// keys and one scan of the (digit, tile) counts before the scatter, 2 (the
// default) the counting pass for 32-bit keys and the look-back for 64-bit
// ones.  150M rows: the scatter runs 17-23% faster without the look-back;
// the counting pass reads the keys once more, which leaves @group's 32-bit
// keys 3% ahead (6.14 -> 5.96 ms) and @order's 64-bit keys even.
static int g_radix_pass = 2;
void set_radix_pass_mode(int m) { g_radix_pass = m < 0 ? 0 : (m > 2 ? 2 : m); }
int get_radix_pass_mode() { return g_radix_pass; }

template <typename K>
__global__ void k_key_bits(const K* __restrict__ k, long long n, unsigned long long* orv, unsigned long long* andv) {
    unsigned long long o = 0, a = ~0ull;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        o |= (unsigned long long)k[i];
        a &= (unsigned long long)k[i];
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        o |= __shfl_xor_sync(0xffffffffu, o, s);
        a &= __shfl_xor_sync(0xffffffffu, a, s);
    }
    if (lane_id() == 0) { atomicOr(orv, o); atomicAnd(andv, a); }
}

template <typename K>
__global__ void k_radix_hist(const K* __restrict__ k, long long n, int lo, int bits, int npass,
                             unsigned long long* __restrict__ hist) {
    __shared__ unsigned sh[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const unsigned dmask = (1u << bits) - 1;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long v = (unsigned long long)k[i];
        for (int p = 0; p < npass; p++) atomicAdd(&sh[p][(unsigned)(v >> (lo + p * bits)) & dmask], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * 256; i += blockDim.x)
        if ((&sh[0][0])[i]) atomicAdd(&hist[i], (unsigned long long)(&sh[0][0])[i]);
}

// exclusive scan of each pass's 256 bins (one block per pass)
__global__ void k_bucket_base(const unsigned long long* __restrict__ hist, unsigned long long* __restrict__ base) {
    __shared__ unsigned long long s[256];
    const int p = blockIdx.x, d = threadIdx.x;
    s[d] = hist[p * 256 + d];
    __syncthreads();
    if (d == 0) {
        unsigned long long acc = 0;
        for (int i = 0; i < 256; i++) { unsigned long long v = s[i]; s[i] = acc; acc += v; }
    }
    __syncthreads();
    base[p * 256 + d] = s[d];
}

// One LSD pass per launch: each tile ranks its keys by digit (warp
// match_any, per-warp histograms), takes each digit's global offset from a
// decoupled look-back over the per-digit counts of the preceding tiles,
// stages the tile in shared memory in digit order and writes each digit's
// run contiguously.
//
// OUT selects what a pass writes: RS_OUT_KV the keys and u32 row ids (every
// pass but the last), RS_OUT_KV64 the keys and the row ids as the i64
// result (the last pass of a @group, whose boundaries are read from the
// keys), RS_OUT_V64 the i64 row ids alone (the last pass of an @order), at
// position n - 1 - pos when `reverse`.
//
// PRE: the offsets are counted beforehand (k_rs_count, one scan): `bucket`
// then holds every (digit, tile)'s first position, digit-major, tile t =
// blockIdx.x, and there is no look-back.
enum { RS_OUT_KV = 0, RS_OUT_KV64 = 1, RS_OUT_V64 = 2 };
template <typename K, bool FIRST, int OUT, bool PRE>
__global__ void __launch_bounds__(RS_THREADS, (sizeof(K) == 4 ? 4 : 3)) k_onesweep(const K* __restrict__ kin, const unsigned* __restrict__ vin,
                                                         K* __restrict__ kout, unsigned* __restrict__ vout,
                                                         long long* __restrict__ vout64, int reverse, long long n,
                                                         int shift, int bits, const unsigned long long* __restrict__ bucket,
                                                         unsigned long long* status, unsigned* ticket, unsigned* derr) {
    // dynamic shared memory: the tile's keys and row ids in digit order
    extern __shared__ __align__(16) unsigned char os_smem[];
    K* skey = reinterpret_cast<K*>(os_smem);
    unsigned* sval = reinterpret_cast<unsigned*>(os_smem + RS_TILE * sizeof(K));
    __shared__ unsigned whist[8][256];
    __shared__ unsigned dstart[256];
    __shared__ unsigned long long dbase[256];
    __shared__ unsigned wscan[8];
    __shared__ long long tile_id;
    for (int i = threadIdx.x; i < 8 * 256; i += RS_THREADS) (&whist[0][0])[i] = 0;
    if (threadIdx.x == 0) tile_id = PRE ? (long long)blockIdx.x : (long long)atomicAdd(ticket, 1u);
    __syncthreads();
    const long long t = tile_id;
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;
    const long long wbase = t * RS_TILE + (long long)w * (32 * RS_ITEMS);
    const unsigned dmask = (1u << bits) - 1;
    K key[RS_ITEMS];
    unsigned val[RS_ITEMS], rd[RS_ITEMS];  // rd = digit << 16 | rank within the warp's items
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        long long i = wbase + k * 32 + lane;
        bool valid = i < n;
        key[k] = valid ? kin[i] : K(0);
        val[k] = FIRST ? (unsigned)i : (valid ? vin[i] : 0u);
    }
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        long long i = wbase + k * 32 + lane;
        bool valid = i < n;
        unsigned d = valid ? ((unsigned)((unsigned long long)key[k] >> shift) & dmask) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        unsigned pre = 0;
        if ((int)lane == leader && valid) {
            pre = whist[w][d];
            whist[w][d] = pre + __popc(peers);
        }
        pre = __shfl_sync(0xffffffffu, pre, leader);
        rd[k] = ((d & 0xffffu) << 16) | (pre + __popc(peers & lanemask_lt()));
        __syncwarp();
    }
    __syncthreads();
    {
        const int d = threadIdx.x;  // one thread per digit
        unsigned c = 0;
        for (int ww = 0; ww < 8; ww++) { unsigned h = whist[ww][d]; whist[ww][d] = c; c += h; }
        // tile-local start of digit d: exclusive scan of the 256 digit counts
        unsigned inc = warp_incl_scan(c);
        if (lane == 31) wscan[w] = inc;
        __syncthreads();
        unsigned before = 0;
        for (unsigned ww = 0; ww < w; ww++) before += wscan[ww];
        dstart[d] = before + inc - c;
        if constexpr (PRE) {
            dbase[d] = d <= (int)dmask ? bucket[(size_t)d * gridDim.x + (size_t)t] : 0ull;
        } else {
            unsigned long long excl = 0;
            if (d <= (int)dmask) excl = chain_lookback(status + d, 256, t, 0, c, derr);
            dbase[d] = bucket[d] + excl;
        }
    }
    __syncthreads();
    // place the tile in digit order in shared memory ...
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        long long i = wbase + k * 32 + lane;
        if (i < n) {
            unsigned d = rd[k] >> 16;
            unsigned local = dstart[d] + whist[w][d] + (rd[k] & 0xffffu);
            skey[local] = key[k];
            sval[local] = val[k];
        }
    }
    __syncthreads();
    // ... and write each digit's run contiguously (consecutive threads, consecutive addresses)
    const long long tn = (n - t * RS_TILE) < RS_TILE ? (n - t * RS_TILE) : RS_TILE;
    for (int i = threadIdx.x; i < tn; i += RS_THREADS) {
        K kk = skey[i];
        unsigned d = (unsigned)((unsigned long long)kk >> shift) & dmask;
        unsigned long long pos = dbase[d] + (unsigned long long)(i - (int)dstart[d]);
        if constexpr (PRE) {  // counted offsets: a position outside the output is an error, not a store
            if (pos >= (unsigned long long)n) {
                flag_error(derr, DERR_INDEX);
                continue;
            }
        }
        if constexpr (OUT != RS_OUT_V64) kout[pos] = kk;
        if constexpr (OUT == RS_OUT_KV) vout[pos] = sval[i];
        else vout64[reverse ? (unsigned long long)(n - 1) - pos : pos] = (long long)sval[i];
    }
}

// The digit counts of every 4096-key tile of one pass, digit-major:
// counts[d * ntiles + t] (per-warp histograms in shared memory)
template <typename K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_count(const K* __restrict__ kin, long long n, int shift, int bits,
                                                         unsigned* __restrict__ counts) {
    __shared__ unsigned wh[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += RS_THREADS) (&wh[0][0])[i] = 0;
    __syncthreads();
    const unsigned dmask = (1u << bits) - 1, w = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * RS_TILE + threadIdx.x;
    K key[RS_ITEMS];
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++) {
        const long long i = base + (long long)k * RS_THREADS;
        key[k] = i < n ? kin[i] : K(0);
    }
#pragma unroll
    for (int k = 0; k < RS_ITEMS; k++)
        if (base + (long long)k * RS_THREADS < n)
            atomicAdd(&wh[w][(unsigned)((unsigned long long)key[k] >> shift) & dmask], 1u);
    __syncthreads();
    const unsigned d = threadIdx.x;
    if (d <= dmask) {
        unsigned c = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) c += wh[q][d];
        counts[(size_t)d * gridDim.x + blockIdx.x] = c;
    }
}

// keeps only the bits set in `mask`, packed to the bottom in order
template <typename K>
__global__ void k_squeeze(const K* __restrict__ k, long long n, unsigned long long mask, K* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long v = (unsigned long long)k[i], r = 0, m = mask;
        int o = 0;
        while (m) {
            int b = __ffsll((long long)m) - 1;
            r |= ((v >> b) & 1ull) << o++;
            m &= m - 1;
        }
        out[i] = (K)r;
    }
}

__global__ void k_iota(unsigned* v, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = (unsigned)i;
}

__global__ void k_widen(const unsigned* __restrict__ v, long long n, long long* __restrict__ out, int reverse);

// The digit plan of a sort over the key bits `vary`: passes of `bits`
// bits from bit lo up to bit hi.
struct RadixPlan {
    int lo, hi, bits, npass;
};
static RadixPlan radix_plan(unsigned long long vary) {
    RadixPlan p;
    p.lo = __builtin_ctzll(vary);
    p.hi = 64 - __builtin_clzll(vary);
    p.bits = g_digit_bits;
    p.npass = (p.hi - p.lo + p.bits - 1) / p.bits;
    if (p.npass > 8) { p.bits = 8; p.npass = (p.hi - p.lo + 7) / 8; }
    return p;
}

// Where the last pass puts the permutation: as i64 row ids in perm64 (at
// n - 1 - pos when `reverse`), with the sorted keys too when `keys`.
struct RadixOut {
    long long* perm64 = nullptr;
    bool reverse = false;
    bool keys = true;
};

// Stable sort of keys[0..n) (row ids travel along).  On return *kres/*vres
// point to the sorted keys and row ids (scratch).  When no key bit varies
// the result is the identity permutation.
//   vary_hint: a superset of the key bits that vary, from bit 0, known to
//              the caller (0: found with one OR/AND reduction);
//   hist:      the digit histograms of the plan of vary_hint, already counted
//              (k_make_keys_hist), or null;
//   out:       the last pass writes the i64 permutation there instead of
//              u32 row ids (*vres is then null; *kres too unless out->keys).
template <typename K>
I radix_sort_ex(const K* keys, long long n, const K** kres, const unsigned** vres, const unsigned* init_vals,
                unsigned long long vary_hint, unsigned long long* hist_ready, const RadixOut* out) {
    unsigned grid = grid_for(n, 256);
    if (grid > (unsigned)g_sms * 8) grid = g_sms * 8;
    unsigned long long vary = vary_hint;
    if (!vary_hint && n > 1) {
        unsigned long long* red = (unsigned long long*)salloc(16);
        if (!red) return E_DEVICE_OOM;
        unsigned long long init[2] = {0, ~0ull};
        HG_CU(cudaMemcpyAsync(red, init, 16, cudaMemcpyHostToDevice, g_stream));
        HG_LAUNCH("key_bits", grid, 256, 0, k_key_bits<K>, keys, n, red, red + 1);
        unsigned long long hb[2];
        HG_CHECK(rb_queue(hb, red, 16));
        HG_CU(stream_sync());
        vary = hb[0] ^ hb[1];
    }
    unsigned* vid = (unsigned*)salloc((size_t)(n > 0 ? n : 1) * 4);
    if (!vid) return E_DEVICE_OOM;
    if (vary == 0 || n <= 1) {
        // all keys equal: identity order
        K* kcopy = (K*)salloc((size_t)(n > 0 ? n : 1) * sizeof(K));
        if (!kcopy) return E_DEVICE_OOM;
        if (n > 0) HG_CU(cudaMemcpyAsync(kcopy, keys, n * sizeof(K), cudaMemcpyDeviceToDevice, g_stream));
        if (n > 0) {
            if (init_vals) HG_CU(cudaMemcpyAsync(vid, init_vals, n * 4, cudaMemcpyDeviceToDevice, g_stream));
            else HG_LAUNCH("iota", grid, 256, 0, k_iota, vid, n);
            if (out && out->perm64)
                HG_LAUNCH("widen", grid, 256, 0, k_widen, vid, n, out->perm64, out->reverse ? 1 : 0);
        }
        *kres = kcopy;
        *vres = vid;
        return last_launch_error();
    }
    RadixPlan pl = radix_plan(vary);
    int nvar = __builtin_popcountll(vary);
    if (!hist_ready && (nvar + pl.bits - 1) / pl.bits < pl.npass) {
        // bits that never change inside the range: squeeze them out (order
        // preserving, injective) and sort the shorter keys
        K* sq = (K*)salloc((size_t)n * sizeof(K));
        if (!sq) return E_DEVICE_OOM;
        HG_LAUNCH("squeeze_keys", grid, 256, 0, k_squeeze<K>, keys, n, vary, sq);
        keys = sq;
        pl = radix_plan(nvar >= 64 ? ~0ull : (1ull << nvar) - 1);
    }
    const int lo = pl.lo, bits = pl.bits, npass = pl.npass;
    unsigned long long* hist = hist_ready;
    if (!hist) {
        hist = (unsigned long long*)salloc((size_t)npass * 256 * 8 * 2);
        if (!hist) return E_DEVICE_OOM;
        HG_CU(cudaMemsetAsync(hist, 0, (size_t)npass * 256 * 8, g_stream));
        HG_LAUNCH("radix_hist", grid, 256, 0, k_radix_hist<K>, keys, n, lo, bits, npass, hist);
    }
    unsigned long long* bucket = hist + npass * 256;
    HG_LAUNCH("bucket_base", npass, 256, 0, k_bucket_base, hist, bucket);
    long long ntiles = (n + RS_TILE - 1) / RS_TILE;
    K* kb[2] = {(K*)salloc(n * sizeof(K)), (K*)salloc(n * sizeof(K))};
    unsigned* vb[2] = {vid, (unsigned*)salloc(n * 4)};
    char* st = (char*)salloc((size_t)ntiles * 256 * 8 + 64);
    if (!kb[0] || !kb[1] || !vb[1] || !st) return E_DEVICE_OOM;
    const K* kin = keys;
    const unsigned* vin = init_vals;
    const int dsm = (int)((size_t)RS_TILE * (sizeof(K) + 4));
    const bool counted = g_radix_pass == 1 || (g_radix_pass == 2 && sizeof(K) == 4);
    unsigned* cnts = nullptr;
    unsigned long long* offs = nullptr;
    if (counted) {
        cnts = (unsigned*)salloc((size_t)ntiles * 256 * 4);
        offs = (unsigned long long*)salloc(((size_t)ntiles * 256 + 1) * 8);
        if (!cnts || !offs) return E_DEVICE_OOM;
    }
    for (int p = 0; p < npass; p++) {
        if (counted) {  // the (digit, tile) offsets of this pass, from the keys it reads
            HG_LAUNCH("radix_count", (unsigned)ntiles, RS_THREADS, 0, k_rs_count<K>, kin, n, lo + p * bits, bits, cnts);
            HG_CHECK(scan_exclusive(cnts, (long long)ntiles << bits, offs, nullptr));
        } else {
            HG_CU(cudaMemsetAsync(st, 0, (size_t)ntiles * 256 * 8 + 64, g_stream));
        }
        K* ko = kb[p & 1];
        unsigned* vo = vb[p & 1];
        unsigned* ticket = (unsigned*)(st + (size_t)ntiles * 256 * 8);
        const bool first = p == 0 && !init_vals;
        const int mode = (p == npass - 1 && out && out->perm64) ? (out->keys ? RS_OUT_KV64 : RS_OUT_V64) : RS_OUT_KV;
        long long* v64 = mode == RS_OUT_KV ? nullptr : out->perm64;
        const int rev = (mode != RS_OUT_KV && out->reverse) ? 1 : 0;
#define RS_PASS1(F, M, PR, BASE)                                                                                     \
    do {                                                                                                             \
        /* the attribute belongs to the current device's context: set it on every call (a host-side write) */      \
        HG_CU(cudaFuncSetAttribute(k_onesweep<K, F, M, PR>, cudaFuncAttributeMaxDynamicSharedMemorySize, dsm));      \
        HG_LAUNCH("onesweep", (unsigned)ntiles, RS_THREADS, (size_t)dsm, (k_onesweep<K, F, M, PR>), kin, vin, ko, vo, \
                  v64, rev, n, lo + p * bits, bits, BASE, (unsigned long long*)st, ticket, g_derr);                  \
    } while (0)
#define RS_PASS(F, M)                                            \
    do {                                                         \
        if (counted) RS_PASS1(F, M, true, offs);                 \
        else RS_PASS1(F, M, false, bucket + p * 256);            \
    } while (0)
        if (first) {
            if (mode == RS_OUT_KV) RS_PASS(true, RS_OUT_KV);
            else if (mode == RS_OUT_KV64) RS_PASS(true, RS_OUT_KV64);
            else RS_PASS(true, RS_OUT_V64);
        } else {
            if (mode == RS_OUT_KV) RS_PASS(false, RS_OUT_KV);
            else if (mode == RS_OUT_KV64) RS_PASS(false, RS_OUT_KV64);
            else RS_PASS(false, RS_OUT_V64);
        }
#undef RS_PASS
#undef RS_PASS1
        kin = ko;
        vin = vo;
        if (mode == RS_OUT_V64) kin = nullptr;
        if (mode != RS_OUT_KV) vin = nullptr;
    }
    HG_CHECK(last_launch_error());
    *kres = kin;
    *vres = vin;
    return 0;
}

template <typename K>
I radix_sort(const K* keys, long long n, const K** kres, const unsigned** vres, const unsigned* init_vals = nullptr) {
    return radix_sort_ex<K>(keys, n, kres, vres, init_vals, 0, nullptr, nullptr);
}

template I radix_sort<unsigned>(const unsigned*, long long, const unsigned**, const unsigned**, const unsigned*);
template I radix_sort<unsigned long long>(const unsigned long long*, long long, const unsigned long long**,
                                          const unsigned**, const unsigned*);

// the reference's comparison sorts (k_qsort.cu)
I qs_sort_vector(const void* col, I typ, long long n, bool asc, const unsigned** perm_out);
I qs_sort_list(int nc, const void* const* cols, const I* typs, const B* asc, long long n, const unsigned** perm_out);

// ---------------------------------------------------------------- sort keys
enum KeyXf : int {
    XF_RAW32 = 0,   // (u32)(i32)v: the reference's 32-bit pattern
    XF_LOW32 = 1,   // low 32 bits of an i64
    XF_RAW64 = 2,   // (u64)v
    XF_UBYTE = 3,   // (u8)v
    XF_RANGE = 4,   // (u64)(v - lo), or (u64)(hi - v) when descending
    XF_FLOAT = 5,   // order-preserving float bits (-0.0 taken as +0.0), complemented when descending
    XF_CASE1 = 6,   // ((i64)x0 << 32) | (i64)x1 over columns 0 and 1
};
constexpr int KMAXC = 4;
struct KeySpec {
    const void* col[KMAXC];
    int typ[KMAXC];
    int xf[KMAXC];
    int shift[KMAXC];
    long long lo[KMAXC], hi[KMAXC];
    int desc[KMAXC];
    int ncol;
};

__device__ __forceinline__ long long ival(const void* p, int typ, long long i) {
    switch (typ) {
    case H_B: return ((const bool*)p)[i];
    case H_J: case H_C: return ((const int8_t*)p)[i];
    case H_H: return ((const int16_t*)p)[i];
    case H_I: case H_M: case H_D: case H_U: case H_W: case H_T: return ((const int32_t*)p)[i];
    default: return ((const long long*)p)[i];
    }
}
__device__ __forceinline__ double fval(const void* p, int typ, long long i) {
    return typ == H_F ? (double)((const float*)p)[i] : ((const double*)p)[i];
}

__device__ __forceinline__ unsigned long long spec_key(const KeySpec& s, long long i);
template <typename K>
__global__ void k_make_keys(KeySpec s, long long n, K* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (K)spec_key(s, i);
}
// k_make_keys and k_radix_hist in one pass over the columns: the keys are
// written and the digit histograms of all npass passes counted as they are
// made (when the varying key bits are known before the keys exist)
template <typename K>
__global__ void k_make_keys_hist(KeySpec s, long long n, K* __restrict__ out, int lo, int bits, int npass,
                                 unsigned long long* __restrict__ hist) {
    __shared__ unsigned sh[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const unsigned dmask = (1u << bits) - 1;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const K k = (K)spec_key(s, i);
        out[i] = k;
        const unsigned long long v = (unsigned long long)k;
        for (int p = 0; p < npass; p++) atomicAdd(&sh[p][(unsigned)(v >> (lo + p * bits)) & dmask], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * 256; i += blockDim.x)
        if ((&sh[0][0])[i]) atomicAdd(&hist[i], (unsigned long long)(&sh[0][0])[i]);
}
__device__ __forceinline__ unsigned long long spec_key(const KeySpec& s, long long i) {
    {
        unsigned long long key = 0;
        for (int c = 0; c < s.ncol; c++) {
            unsigned long long u;
            switch (s.xf[c]) {
            case XF_RAW32: u = (unsigned)(int)ival(s.col[c], s.typ[c], i); break;
            case XF_LOW32: u = (unsigned)(unsigned long long)ival(s.col[c], s.typ[c], i); break;
            case XF_RAW64: u = (unsigned long long)ival(s.col[c], s.typ[c], i); break;
            case XF_UBYTE: u = (uint8_t)ival(s.col[c], s.typ[c], i); break;
            case XF_RANGE: {
                long long v = ival(s.col[c], s.typ[c], i);
                u = s.desc[c] ? (unsigned long long)(s.hi[c] - v) : (unsigned long long)(v - s.lo[c]);
            } break;
            case XF_FLOAT: {
                double f = fval(s.col[c], s.typ[c], i);
                if (f == 0.0) f = 0.0;
                unsigned long long b = (unsigned long long)__double_as_longlong(f);
                b = (b >> 63) ? ~b : (b | (1ull << 63));
                u = s.desc[c] ? ~b : b;
            } break;
            default: {  // XF_CASE1
                long long a = ival(s.col[0], s.typ[0], i), b = ival(s.col[1], s.typ[1], i);
                u = ((unsigned long long)a << 32) | (unsigned long long)b;
                c = s.ncol;
            } break;
            }
            key |= u << s.shift[c < KMAXC ? c : 0];
        }
        return key;
    }
}

__global__ void k_minmax_i64(const void* p, int typ, long long n, long long* mn, long long* mx) {
    long long a = LLONG_MAX, b = LLONG_MIN;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v = ival(p, typ, i);
        a = v < a ? v : a;
        b = v > b ? v : b;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        long long o = __shfl_xor_sync(0xffffffffu, a, s); a = o < a ? o : a;
        long long q = __shfl_xor_sync(0xffffffffu, b, s); b = q > b ? q : b;
    }
    if (lane_id() == 0) { atomicMin(mn, a); atomicMax(mx, b); }
}

// ------------------------------------------------------------- permutations
__global__ void k_widen(const unsigned* __restrict__ v, long long n, long long* __restrict__ out, int reverse) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = reverse ? (long long)v[n - 1 - i] : (long long)v[i];
}

// group boundary flags: row i starts a group when its key differs from row i-1
template <typename K>
__global__ void k_bound_keys(const K* __restrict__ k, long long n, uint8_t* __restrict__ f) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        f[i] = (i == 0) || (k[i] != k[i - 1]);
}
// ... or when any column value differs between the rows perm[i-1] and perm[i]
// (equality as the reference's comparator: == on values)
struct ColSet {
    const void* col[KMAXC];
    int typ[KMAXC];
    int ncol;
};
__global__ void k_bound_cols(ColSet c, const unsigned* __restrict__ perm, long long n, uint8_t* __restrict__ f) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        bool b = i == 0;
        if (!b) {
            long long a = perm[i - 1], q = perm[i];
            for (int j = 0; j < c.ncol && !b; j++) {
                if (c.typ[j] == H_F || c.typ[j] == H_E) b = fval(c.col[j], c.typ[j], a) != fval(c.col[j], c.typ[j], q);
                else b = ival(c.col[j], c.typ[j], a) != ival(c.col[j], c.typ[j], q);
            }
        }
        f[i] = b;
    }
}

// keys[g] = perm[start[g]]; node g = group g's rows (inline when one row),
// written to a device staging copy of the host node array at host_base
__global__ void k_group_nodes(const long long* __restrict__ starts, long long ng, long long n,
                              const long long* __restrict__ perm, long long* __restrict__ keys, V0* __restrict__ nodes,
                              unsigned long long host_base) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        long long s = starts[g], e = (g + 1 < ng) ? starts[g + 1] : n;
        long long first = perm[s];
        if (keys) keys[g] = first;
        V0 v;
        v.len = e - s;
        v.typ = H_L;
        if (e - s == 1) {
            v.i64 = first;
            v.g = (G)(host_base + (unsigned long long)g * sizeof(V0) + offsetof(V0, b));
        } else {
            v.i64 = 0;
            v.g = (G)(perm + s);
        }
        nodes[g] = v;
    }
}

// the reference's char sort of fewer than ten rows (h_libs.cc:388-390):
// all-pairs exchange on a[rtn[i]] > a[rtn[j]], which leaves them descending
__global__ void k_char_small(const int8_t* __restrict__ a, long long n, unsigned* __restrict__ perm) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned r[10];
    for (long long i = 0; i < n; i++) r[i] = (unsigned)i;
    for (long long i = 0; i < n; i++)
        for (long long j = 0; j < n; j++)
            if (a[r[i]] > a[r[j]]) { unsigned t = r[i]; r[i] = r[j]; r[j] = t; }
    for (long long i = 0; i < n; i++) perm[i] = r[i];
}

static unsigned gcap(long long n) {
    unsigned g = grid_for(n, 256);
    return g > (unsigned)g_sms * 16 ? (unsigned)g_sms * 16 : g;
}

// ----------------------------------------------- descending list orders
// lib_quicksort_list (h_libs.cc:637-697) first asks lib_order_by_sorted
// (:604-617) whether the range is already in order; for a descending column
// a range that is ascending (non-decreasing with one strict step) is
// reversed instead of sorted, which reverses its ties.  Within every run the
// rows are therefore in ascending or descending row order; one bit per row
// (dirbit) tracks which, and the final order is the lexicographic key order
// with fully tied rows in their run's row order.
__global__ void k_updown(const void* __restrict__ col, int typ, const unsigned* __restrict__ perm,
                         const unsigned* __restrict__ rid, long long n, unsigned* __restrict__ flags) {
    for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned r0 = rid ? rid[i - 1] : 0, r1 = rid ? rid[i] : 0;
        if (r0 != r1) continue;
        long long a = ival(col, typ, perm ? perm[i - 1] : i - 1), b = ival(col, typ, perm ? perm[i] : i);
        if (b > a) atomicOr(&flags[r1], 1u);
        if (b < a) atomicOr(&flags[r1], 2u);
    }
}
// a run whose values are non-decreasing (with a strict step) in its current
// order is reversed: flip the direction bit of its rows
__global__ void k_flip(const unsigned* __restrict__ perm, const unsigned* __restrict__ rid, long long n,
                       const unsigned* __restrict__ flags, uint8_t* __restrict__ dirbit) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned r = perm ? perm[i] : (unsigned)i;
        unsigned f = flags[rid ? rid[i] : 0];
        bool up = f & 1u, down = f & 2u;
        bool rev = dirbit[r] ? (!up && down) : (!down && up);
        if (rev) dirbit[r] ^= 1;
    }
}
__global__ void k_run_ids(const uint8_t* __restrict__ bflag, long long n, unsigned* __restrict__ one) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        one[i] = (i > 0 && bflag[i]) ? 1u : 0u;
}
__global__ void k_add_u32(unsigned* __restrict__ a, const unsigned* __restrict__ b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] += b[i];
}
__global__ void k_u64_to_u32(const unsigned long long* __restrict__ a, long long n, unsigned* __restrict__ b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (unsigned)a[i];
}
__global__ void k_tiebreak(const uint8_t* __restrict__ dirbit, long long n, unsigned* __restrict__ tb, unsigned* any) {
    bool f = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        tb[i] = dirbit[i] ? (unsigned)(n - 1 - i) : (unsigned)i;
        f |= dirbit[i] != 0;
    }
    if (__any_sync(0xffffffffu, f) && lane_id() == 0) atomicOr(any, 1u);
}
template <typename K>
__global__ void k_gather_keys(const K* __restrict__ k, const unsigned* __restrict__ perm, long long n, K* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = k[perm[i]];
}

// ------------------------------------------------------------- sort drivers
struct SortResult {
    const unsigned* perm;   // row ids in sorted order (scratch)
    const void* keys;       // sorted keys (scratch), null for the small-char path
    int key64;
    bool key_injective;     // equal keys <=> equal rows (boundary test on keys)
    const long long* perm64;  // the permutation as i64, written by the last pass (RadixOut), else null
};

template <typename K>
static I sort_keys_spec(const KeySpec& s, long long n, unsigned long long vary_hint, const RadixOut* ro,
                        SortResult* r) {
    K* k = (K*)salloc((size_t)(n > 0 ? n : 1) * sizeof(K));
    if (!k) return E_DEVICE_OOM;
    unsigned long long* hist = nullptr;
    if (n > 1 && vary_hint) {  // the digit plan is known: count the histograms while making the keys
        const RadixPlan pl = radix_plan(vary_hint);
        hist = (unsigned long long*)salloc((size_t)pl.npass * 256 * 8 * 2);
        if (!hist) return E_DEVICE_OOM;
        HG_CU(cudaMemsetAsync(hist, 0, (size_t)pl.npass * 256 * 8, g_stream));
        unsigned grid = grid_for(n, 256);
        if (grid > (unsigned)g_sms * 8) grid = g_sms * 8;
        HG_LAUNCH("make_keys", grid, 256, 0, k_make_keys_hist<K>, s, n, k, pl.lo, pl.bits, pl.npass, hist);
    } else if (n > 0) {
        HG_LAUNCH("make_keys", gcap(n), 256, 0, k_make_keys<K>, s, n, k);
    }
    const K* ks;
    HG_CHECK(radix_sort_ex<K>(k, n, &ks, &r->perm, nullptr, n > 1 ? vary_hint : 0, hist, ro));
    r->keys = ks;
    r->perm64 = ro ? ro->perm64 : nullptr;
    return last_launch_error();
}

// vary_hint: the key bits that can vary, when the caller knows them (0: found
// by the sort); ro: where the permutation goes as i64 (null: u32 in r->perm)
static I sort_by_spec(const KeySpec& s, long long n, int total_bits, SortResult* r, unsigned long long vary_hint = 0,
                      const RadixOut* ro = nullptr) {
    r->key64 = total_bits > 32;
    r->perm64 = nullptr;
    if (r->key64) return sort_keys_spec<unsigned long long>(s, n, vary_hint, ro, r);
    return sort_keys_spec<unsigned>(s, n, vary_hint, ro, r);
}

static int bits_for(unsigned long long range) { return range == 0 ? 1 : 64 - __builtin_clzll(range); }

static I col_minmax(const void* p, I typ, long long n, long long* mn, long long* mx) {
    long long* d = (long long*)salloc(16);
    if (!d) return E_DEVICE_OOM;
    long long init[2] = {LLONG_MAX, LLONG_MIN};
    HG_CU(cudaMemcpyAsync(d, init, 16, cudaMemcpyHostToDevice, g_stream));
    if (n > 0) HG_LAUNCH("minmax", gcap(n), 256, 0, k_minmax_i64, p, (int)typ, n, d, d + 1);
    long long h[2];
    HG_CHECK(rb_queue(h, d, 16));
    HG_CU(stream_sync());
    *mn = h[0];
    *mx = h[1];
    return 0;
}

// Single-column keys following the reference's radix rules (i32 / i64).
// With `ro` the permutation is written as i64 there (for a @group only when
// the keys are injective, since the boundaries are then read from them).
static I sort_int_column(V x, const void* p, long long n, SortResult* r, const long long* known_mm = nullptr,
                         const RadixOut* ro = nullptr) {
    KeySpec s{};
    s.ncol = 1;
    s.col[0] = p;
    s.typ[0] = x->typ;
    s.shift[0] = 0;
    if (x->typ == H_I) {
        s.xf[0] = XF_RAW32;
        r->key_injective = true;
        return sort_by_spec(s, n, 32, r, 0, ro);
    }
    // some value has (x >> 32) > 0 exactly when the maximum is >= 2^32; the
    // low 32 bits are injective when every value lies in one 2^32-wide range
    long long mn = 0, mx = 0;
    if (known_mm) { mn = known_mm[0]; mx = known_mm[1]; }
    else if (n > 0) HG_CHECK(col_minmax(p, H_L, n, &mn, &mx));
    const bool f = n > 0 && mx >= (1LL << 32);
    s.xf[0] = f ? XF_RAW64 : XF_LOW32;
    r->key_injective = f || n == 0 || ((unsigned long long)mx - (unsigned long long)mn) < (1ull << 32);
    if (ro && ro->keys && !r->key_injective) ro = nullptr;
    // non-negative values in [mn, mx] agree on every bit above the highest
    // one in which mn and mx differ: only the bits below it can vary
    unsigned long long hint = 0;
    if (n > 1 && mn >= 0 && mx > mn) hint = (1ull << bits_for((unsigned long long)(mn ^ mx))) - 1;
    return sort_by_spec(s, n, f ? 64 : 32, r, hint, ro);
}

// Key spec for the stable lexicographic order of integer / float columns
// (ascending unless desc[c]); integer columns are range-compressed and all
// columns packed into one key of *bits bits.
static I column_spec(int ncol, V* cols, const void** ptrs, const B* asc, long long n, KeySpec* s, int* bits) {
    if (ncol > KMAXC) return set_error(E_NOT_IMPL, "ordering by more than %d columns", KMAXC);
    memset(s, 0, sizeof *s);
    s->ncol = ncol;
    int shift = 0;
    for (int c = ncol - 1; c >= 0; c--) {
        int width;
        s->col[c] = ptrs[c];
        s->typ[c] = cols[c]->typ;
        s->desc[c] = asc ? !asc[c] : 0;
        if (cols[c]->typ == H_F || cols[c]->typ == H_E) {
            s->xf[c] = XF_FLOAT;
            width = 64;
        } else {
            long long mn, mx;
            HG_CHECK(col_minmax(ptrs[c], cols[c]->typ, n, &mn, &mx));
            s->xf[c] = XF_RANGE;
            s->lo[c] = mn;
            s->hi[c] = mx;
            width = n > 0 ? bits_for((unsigned long long)mx - (unsigned long long)mn) : 1;
        }
        s->shift[c] = shift;
        shift += width;
    }
    if (shift > 64) return set_error(E_NOT_IMPL, "packed order key wider than 64 bits");
    *bits = shift;
    return 0;
}

static I sort_columns(int ncol, V* cols, const void** ptrs, const B* asc, long long n, SortResult* r,
                      const RadixOut* ro = nullptr) {
    KeySpec s;
    int bits;
    HG_CHECK(column_spec(ncol, cols, ptrs, asc, n, &s, &bits));
    r->key_injective = true;
    // range-compressed integer columns: the packed key's top bit is the top
    // column's (hi - lo), so bits 0 .. bits-1 are the ones that can vary
    bool ranged = true;
    for (int c = 0; c < ncol; c++) ranged = ranged && s.xf[c] == XF_RANGE;
    const unsigned long long hint = (ranged && n > 1) ? (bits >= 64 ? ~0ull : (1ull << bits) - 1) : 0;
    return sort_by_spec(s, n, bits, r, hint, ro);
}

// Multi-column @order with descending columns, as lib_quicksort_list does it
// (see k_updown above).
template <typename K>
static I final_order(const KeySpec& s, long long n, const uint8_t* dirbit, SortResult* r) {
    K* k = (K*)salloc((size_t)n * sizeof(K));
    unsigned* tb = (unsigned*)salloc((size_t)n * 4);
    unsigned* any = (unsigned*)salloc(16);
    if (!k || !tb || !any) return E_DEVICE_OOM;
    HG_LAUNCH("make_keys", gcap(n), 256, 0, k_make_keys<K>, s, n, k);
    HG_CU(cudaMemsetAsync(any, 0, 4, g_stream));
    HG_LAUNCH("tiebreak", gcap(n), 256, 0, k_tiebreak, dirbit, n, tb, any);
    unsigned h = 0;
    HG_CHECK(rb_queue(&h, any, 4));
    HG_CU(stream_sync());
    const K* ks;
    if (!h) {  // no range was reversed: ties stay in row order
        HG_CHECK(radix_sort<K>(k, n, &ks, &r->perm));
    } else {  // ties of reversed runs in descending row order: sort by tiebreak first
        const unsigned* tk;
        const unsigned* pt;
        HG_CHECK(radix_sort<unsigned>(tb, n, &tk, &pt));
        K* kg = (K*)salloc((size_t)n * sizeof(K));
        if (!kg) return E_DEVICE_OOM;
        HG_LAUNCH("gather_keys", gcap(n), 256, 0, k_gather_keys<K>, k, pt, n, kg);
        HG_CHECK(radix_sort<K>(kg, n, &ks, &r->perm, pt));
    }
    r->keys = ks;
    r->key64 = sizeof(K) == 8;
    r->key_injective = true;
    return last_launch_error();
}

static I order_columns_exact(int nc, V* cols, const void** ptrs, const B* asc, long long n, SortResult* r) {
    uint8_t* dirbit = (uint8_t*)salloc((size_t)(n > 0 ? n : 1));
    unsigned* flags = (unsigned*)salloc((size_t)(n > 0 ? n : 1) * 4 + 16);
    if (!dirbit || !flags) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(dirbit, 0, (size_t)(n > 0 ? n : 1), g_stream));
    if (n > 1 && !asc[0]) {  // level 0: the whole range in row order
        HG_CU(cudaMemsetAsync(flags, 0, 4, g_stream));
        HG_LAUNCH("updown", gcap(n), 256, 0, k_updown, ptrs[0], (int)cols[0]->typ, (const unsigned*)nullptr,
                  (const unsigned*)nullptr, n, flags);
        HG_LAUNCH("flip", gcap(n), 256, 0, k_flip, (const unsigned*)nullptr, (const unsigned*)nullptr, n, flags, dirbit);
    }
    for (int c = 1; c < nc && n > 1; c++) {
        if (asc[c]) continue;
        // runs of equal columns 0..c-1, rows in ascending row order within each run
        SortResult pr{};
        HG_CHECK(sort_columns(c, cols, ptrs, nullptr, n, &pr));
        uint8_t* bf = (uint8_t*)salloc((size_t)n);
        unsigned* one = (unsigned*)salloc((size_t)n * 4);
        unsigned long long* ex = (unsigned long long*)salloc((size_t)n * 8);
        unsigned* rid = (unsigned*)salloc((size_t)n * 4);
        if (!bf || !one || !ex || !rid) return E_DEVICE_OOM;
        if (pr.key64) HG_LAUNCH("bound_keys", gcap(n), 256, 0, k_bound_keys<unsigned long long>, (const unsigned long long*)pr.keys, n, bf);
        else HG_LAUNCH("bound_keys", gcap(n), 256, 0, k_bound_keys<unsigned>, (const unsigned*)pr.keys, n, bf);
        HG_LAUNCH("run_ids", gcap(n), 256, 0, k_run_ids, bf, n, one);
        unsigned long long nb = 0;
        HG_CHECK(scan_exclusive(one, n, ex, &nb));
        HG_LAUNCH("run_ids", gcap(n), 256, 0, k_u64_to_u32, ex, n, rid);
        HG_LAUNCH("run_ids", gcap(n), 256, 0, k_add_u32, rid, one, n);
        HG_CU(cudaMemsetAsync(flags, 0, (size_t)(nb + 1) * 4, g_stream));
        HG_LAUNCH("updown", gcap(n), 256, 0, k_updown, ptrs[c], (int)cols[c]->typ, pr.perm, rid, n, flags);
        HG_LAUNCH("flip", gcap(n), 256, 0, k_flip, pr.perm, rid, n, flags, dirbit);
    }
    KeySpec s;
    int bits;
    HG_CHECK(column_spec(nc, cols, ptrs, asc, n, &s, &bits));
    if (n == 0) { r->perm = nullptr; r->keys = nullptr; return 0; }
    if (bits > 32) return final_order<unsigned long long>(s, n, dirbit, r);
    return final_order<unsigned>(s, n, dirbit, r);
}

// Builds the @group dict from a sorted permutation.
static I group_finish(V z, long long* starts, long long G, long long* perm, long long n);

// perm_pre: the output-arena buffer for the i64 permutation, allocated by
// the caller before the sort (r.perm64 is set when the sort wrote it)
static I group_dict(V z, const SortResult& r, long long n, const ColSet* cols, long long* perm_pre = nullptr) {
    uint8_t* flags = (uint8_t*)salloc((size_t)(n > 0 ? n : 1));
    long long* starts = (long long*)salloc((size_t)(n > 0 ? n : 1) * 8);
    if (!flags || !starts) return E_DEVICE_OOM;
    if (n > 0) {
        if (cols) HG_LAUNCH("bound_cols", gcap(n), 256, 0, k_bound_cols, *cols, r.perm, n, flags);
        else if (r.key64) HG_LAUNCH("bound_keys", gcap(n), 256, 0, k_bound_keys<unsigned long long>, (const unsigned long long*)r.keys, n, flags);
        else HG_LAUNCH("bound_keys", gcap(n), 256, 0, k_bound_keys<unsigned>, (const unsigned*)r.keys, n, flags);
    }
    long long G = 0;
    HG_CHECK(compact_rows(flags, n, starts, &G));
    {  // group starts stay in the output arena: aggregations over this dict reuse them
        long long* keep = (long long*)dalloc((size_t)(G > 0 ? G : 1) * 8);
        if (!keep) return E_DEVICE_OOM;
        if (G > 0) HG_CU(cudaMemcpyAsync(keep, starts, (size_t)G * 8, cudaMemcpyDeviceToDevice, g_stream));
        starts = keep;
    }
    // permutation as i64 (the rows of every group, concatenated)
    long long* perm = r.perm64 ? (long long*)r.perm64 : perm_pre;
    if (n > 0 && !r.perm64) {
        if (!perm) perm = (long long*)dalloc((size_t)n * 8);
        if (!perm) return E_DEVICE_OOM;
        HG_LAUNCH("widen", gcap(n), 256, 0, k_widen, r.perm, n, perm, 0);
    }
    return group_finish(z, starts, G, perm, n);
}

// The dict of a grouping from its G group starts and its permutation (both
// i64, output arena): keys = each group's first row, values = the row lists.
static I group_finish(V z, long long* starts, long long G, long long* perm, long long n) {
    HG_CHECK(init_list(z, H_N, 2));
    V0* kv = host_nodes(z);
    void* dkeys;
    HG_CHECK(alloc_out(&kv[0], H_L, G, &dkeys));
    HG_CHECK(init_list(&kv[1], H_G, G));
    if (G > 0) {
        // the node array lives in mapped pinned host memory: a few nodes are
        // written there by the kernel directly (no copy operation); many go
        // through a device staging copy, since kernel stores to host memory
        // are slow in bulk (GB300: 8.6M nodes, 276 MB, 5.0 ms against 1.1 ms
        // for the staged kernel and the copy)
        V0* hn = host_nodes(&kv[1]);
        V0* dn = nullptr;
        if (G <= SEG_PLAN_SMALL && cudaHostGetDevicePointer((void**)&dn, hn, 0) != cudaSuccess) {
            cudaGetLastError();  // clears the failed look-up's own error
            dn = nullptr;
        }
        V0* stage = dn ? dn : (V0*)salloc((size_t)G * sizeof(V0));
        if (!stage) return E_DEVICE_OOM;
        HG_LAUNCH("group_nodes", gcap(G), 256, 0, k_group_nodes, starts, G, n, perm, (long long*)dkeys, stage,
                  (unsigned long long)(uintptr_t)hn);
        if (!dn) HG_CU(cudaMemcpyAsync(hn, stage, (size_t)G * sizeof(V0), cudaMemcpyDeviceToHost, g_stream));
    }
    // few groups: plan the aggregations over them now, inside this call's own round trip
    SmallPlan plan;
    HG_CHECK(seg_plan_small(starts, G, n, &plan));
    HG_CHECK(last_launch_error());
    if (plan.hdr) HG_CHECK(rb_queue(plan.hdr, plan.hdr_dev, SEG_PLAN_HDR_BYTES));
    HG_CHECK(check_device_errors());  // synchronises: the node array is written by the kernel
    HG_CHECK(finish_out(&kv[0], dkeys));
    register_bound(kv[0].g, kv[0].len, n);
    if (G > 0) {
        ListInfo li{host_nodes(&kv[1]), G, LIST_SEGMENTS, H_L, starts, n, perm, 1, 0, 0, 0, nullptr, nullptr, nullptr};
        seg_plan_adopt(li, plan);
        register_list(li);
    }
    return apply_residency(z);
}

// The @order result allocated before the sort, so that the last radix pass
// writes it (outputs of one row stay on the ordinary path).
static I order_prealloc(V z, long long n, bool reverse, RadixOut* ro, void** d) {
    *d = nullptr;
    if (n <= 1) return 0;
    HG_CHECK(alloc_out(z, H_L, n, d));
    ro->perm64 = (long long*)*d;
    ro->reverse = reverse;
    ro->keys = false;
    return 0;
}

static I order_output(V z, const SortResult& r, long long n, bool reverse, void* d_pre = nullptr) {
    void* d = d_pre;
    if (!d) HG_CHECK(alloc_out(z, H_L, n, &d));
    if (n > 0 && !r.perm64) HG_LAUNCH("widen", gcap(n), 256, 0, k_widen, r.perm, n, (long long*)d, reverse ? 1 : 0);
    HG_CHECK(last_launch_error());
    // a radix pass whose look-back gave up leaves a wrong permutation: read
    // the device error word before the result is marked as in range
    HG_CHECK(check_device_errors());
    register_bound(d, n, n);
    return finish_out(z, d);
}

static bool list_of_basic(V x) {
    if (x->typ != H_G) return false;
    for (L i = 0; i < x->len; i++)
        if (!is_basic(host_nodes(x)[i].typ)) return false;
    return true;
}

// sort of one char column as lib_quicksort_char (h_libs.cc:386-407)
static I sort_char(const void* p, long long n, SortResult* r) {
    if (n < 10) {
        unsigned* perm = (unsigned*)salloc(64);
        if (!perm) return E_DEVICE_OOM;
        if (n > 0) HG_LAUNCH("char_small", 1, 32, 0, k_char_small, (const int8_t*)p, n, perm);
        r->perm = perm;
        r->keys = nullptr;
        r->key64 = 0;
        r->key_injective = false;
        return last_launch_error();
    }
    KeySpec s{};
    s.ncol = 1; s.col[0] = p; s.typ[0] = H_C; s.xf[0] = XF_UBYTE;
    r->key_injective = true;
    return sort_by_spec(s, n, 8, r);
}

// ---- groupings with few distinct keys of a 16-bit code: a counting sort.
// The code of a row keeps the key order the radix path sorts by: c0 << 8 |
// c1 for two char columns (unsigned bytes), v - min for a non-negative
// integer column spanning fewer than 65536 values.  A code's bucket is its
// rank among the codes present.  Per 4096-row tile: bucket counts (pass 1),
// one scan over (bucket, tile), then each row's stable position (pass 2),
// written straight as an i64 row list.
constexpr int TS_TILE = 4096, TS_MAXG = 256;
struct CodeChars {
    const uint8_t* c0;
    const uint8_t* c1;
    __device__ __forceinline__ unsigned operator()(long long i) const { return ((unsigned)c0[i] << 8) | c1[i]; }
};
template <typename T>
struct CodeInt {
    const T* p;
    long long mn;
    __device__ __forceinline__ unsigned operator()(long long i) const { return (unsigned)((long long)p[i] - mn); }
};
template <typename Code>
__global__ void k_trie_present(Code code_of, long long n, unsigned* __restrict__ bitmap) {
    __shared__ unsigned sb[2048];
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) sb[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned code = code_of(i);
        atomicOr(&sb[code >> 5], 1u << (code & 31));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2048; i += blockDim.x)
        if (sb[i]) atomicOr(&bitmap[i], sb[i]);
}
struct TrieRank { unsigned bits[2048]; unsigned short wpre[2048]; };
__device__ __forceinline__ unsigned trie_bucket(const TrieRank& t, unsigned code) {
    const unsigned w = code >> 5;
    return t.wpre[w] + __popc(t.bits[w] & ((1u << (code & 31)) - 1u));
}
__device__ void load_rank(TrieRank& s, const TrieRank* g) {
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) { s.bits[i] = g->bits[i]; s.wpre[i] = g->wpre[i]; }
}
// pass 1: counts[b * T + tile]
template <typename Code>
__global__ void __launch_bounds__(256) k_trie_count(Code code_of, long long n, const TrieRank* __restrict__ rk, int G,
                                                    long long T, unsigned* __restrict__ counts) {
    __shared__ TrieRank r;
    __shared__ unsigned cnt[TS_MAXG];
    load_rank(r, rk);
    for (int i = threadIdx.x; i < G; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * TS_TILE;
    for (int k = threadIdx.x; k < TS_TILE; k += blockDim.x) {
        const long long i = base + k;
        const bool in = i < n;
        const unsigned b = in ? trie_bucket(r, code_of(i)) : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, b);
        if (in && (int)lane_id() == __ffs(peers) - 1) atomicAdd(&cnt[b], __popc(peers));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < G; b += blockDim.x) counts[(long long)b * T + blockIdx.x] = cnt[b];
}
// pass 2: perm[offs[b * T + tile] + rank of the row among the tile's rows of bucket b] = row
template <typename Code>
__global__ void __launch_bounds__(256) k_trie_scatter(Code code_of, long long n, const TrieRank* __restrict__ rk, int G,
                                                      long long T, const unsigned long long* __restrict__ offs,
                                                      long long* __restrict__ perm) {
    __shared__ TrieRank r;
    __shared__ unsigned wcnt[8][TS_MAXG];  // per warp: rows of each bucket, then the warp's base
    __shared__ unsigned long long toff[TS_MAXG];  // the tile's first position in each bucket
    load_rank(r, rk);  // once per block: each block walks several tiles
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;
    for (long long t = blockIdx.x; t < T; t += gridDim.x) {
    for (int b = lane; b < G; b += 32) wcnt[w][b] = 0;
    for (int b = threadIdx.x; b < G; b += blockDim.x) toff[b] = offs[(long long)b * T + t];
    __syncthreads();
    const long long base = t * TS_TILE + (long long)w * (TS_TILE / 8);
    unsigned bk[16], pr[16];  // bucket, and the lanes sharing it in that round
#pragma unroll
    for (int k = 0; k < 16; k++) {  // warp w owns rows base .. base + 511, in order
        const long long i = base + k * 32 + lane;
        const bool in = i < n;
        bk[k] = in ? trie_bucket(r, code_of(i)) : 0xffffffffu;
        pr[k] = __match_any_sync(0xffffffffu, bk[k]);
        if (in && (int)lane == __ffs(pr[k]) - 1) wcnt[w][bk[k]] += __popc(pr[k]);
        __syncwarp();
    }
    __syncthreads();
    for (int b = threadIdx.x; b < G; b += blockDim.x) {  // warps' exclusive bases per bucket
        unsigned c = 0;
        for (int ww = 0; ww < 8; ww++) { const unsigned h = wcnt[ww][b]; wcnt[ww][b] = c; c += h; }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const long long i = base + k * 32 + lane;
        const bool in = i < n;
        const int leader = __ffs(pr[k]) - 1;
        unsigned pre = 0;
        if (in && (int)lane == leader) { pre = wcnt[w][bk[k]]; wcnt[w][bk[k]] = pre + __popc(pr[k]); }
        pre = __shfl_sync(0xffffffffu, pre, leader);
        if (in) perm[toff[bk[k]] + pre + __popc(pr[k] & lanemask_lt())] = i;
        __syncwarp();
    }
    __syncthreads();
    }
}
__global__ void k_trie_starts(const unsigned long long* __restrict__ offs, int G, long long T, long long* __restrict__ starts) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < G) starts[b] = (long long)offs[(long long)b * T];
}

// *done = 1 with the dict in z; 0 when too many codes are present for the counting path
template <typename Code>
static I small_group(V z, Code code_of, long long n, int* done) {
    *done = 0;
    unsigned* bitmap = (unsigned*)salloc(2048 * 4);
    if (!bitmap) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(bitmap, 0, 2048 * 4, g_stream));
    unsigned grid = grid_for(n, 256);
    if (grid > (unsigned)g_sms * 4) grid = g_sms * 4;
    HG_LAUNCH("trie_present", grid, 256, 0, k_trie_present<Code>, code_of, n, bitmap);
    TrieRank hr;
    HG_CHECK(rb_queue(hr.bits, bitmap, 2048 * 4));
    HG_CU(stream_sync());
    unsigned G = 0;
    for (int i = 0; i < 2048; i++) { hr.wpre[i] = (unsigned short)G; G += (unsigned)__builtin_popcount(hr.bits[i]); }
    if (G == 0 || G > (unsigned)TS_MAXG) return 0;
    TrieRank* drk = (TrieRank*)salloc(sizeof(TrieRank));
    const long long T = (n + TS_TILE - 1) / TS_TILE;
    unsigned* counts = (unsigned*)salloc((size_t)G * (size_t)T * 4);
    unsigned long long* offs = (unsigned long long*)salloc(((size_t)G * (size_t)T + 1) * 8);
    long long* perm = (long long*)dalloc((size_t)n * 8);
    long long* starts = (long long*)dalloc((size_t)G * 8);
    if (!drk || !counts || !offs || !perm || !starts) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(drk, &hr, sizeof(TrieRank), cudaMemcpyHostToDevice, g_stream));
    const unsigned tg = (unsigned)(T < (long long)g_sms * 4 ? T : (long long)g_sms * 4);
    HG_LAUNCH("trie_count", (unsigned)T, 256, 0, k_trie_count<Code>, code_of, n, drk, (int)G, T, counts);
    HG_CHECK(scan_exclusive(counts, (long long)G * T, offs, nullptr));
    HG_LAUNCH("trie_scatter", tg, 256, 0, k_trie_scatter<Code>, code_of, n, drk, (int)G, T, offs, perm);
    HG_LAUNCH("trie_starts", 1, 256, 0, k_trie_starts, offs, (int)G, T, starts);
    HG_CHECK(last_launch_error());
    *done = 1;
    return group_finish(z, starts, (long long)G, perm, n);
}

}  // namespace hg

using namespace hg;

extern "C" {

I pfnGroupTrie(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    V0* c = host_nodes(x);
    long long n = c[0].len;
    const void *p0, *p1;
    HG_CHECK(in_ptr(&c[0], &p0));
    HG_CHECK(in_ptr(&c[1], &p1));
    if (n >= TS_TILE) {
        int done = 0;
        HG_CHECK(small_group(z, CodeChars{(const uint8_t*)p0, (const uint8_t*)p1}, n, &done));
        if (done) return 0;
    }
    KeySpec s{};
    s.ncol = 2;
    s.col[0] = p0; s.typ[0] = H_C; s.xf[0] = XF_UBYTE; s.shift[0] = 8;
    s.col[1] = p1; s.typ[1] = H_C; s.xf[1] = XF_UBYTE; s.shift[1] = 0;
    SortResult r{};
    r.key_injective = true;
    HG_CHECK(sort_by_spec(s, n, 16, &r));
    return group_dict(z, r, n, nullptr);
}

I pfnGroupBasic(V z, V x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    SortResult r{};
    if (x->typ == H_I || x->typ == H_L) {
        const void* p;
        HG_CHECK(in_ptr(x, &p));
        long long mm[2] = {0, 0};
        bool have_mm = false;
        if (x->len >= TS_TILE) {  // few non-negative values in a narrow range: the counting path
            HG_CHECK(col_minmax(p, x->typ, x->len, &mm[0], &mm[1]));
            have_mm = true;
            if (mm[0] >= 0 && mm[1] - mm[0] < 65536) {
                int done = 0;
                if (x->typ == H_I) HG_CHECK(small_group(z, CodeInt<int32_t>{(const int32_t*)p, mm[0]}, x->len, &done));
                else HG_CHECK(small_group(z, CodeInt<long long>{(const long long*)p, mm[0]}, x->len, &done));
                if (done) return 0;
            }
        }
        // the permutation is allocated first, so that the last radix pass writes it
        long long* pre = x->len > 1 ? (long long*)dalloc((size_t)x->len * 8) : nullptr;
        if (x->len > 1 && !pre) return E_DEVICE_OOM;
        RadixOut ro;
        ro.perm64 = pre;
        HG_CHECK(sort_int_column(x, p, x->len, &r, have_mm && x->typ == H_L ? mm : nullptr, pre ? &ro : nullptr));
        if (r.key_injective) return group_dict(z, r, x->len, nullptr, pre);
        ColSet cs{};
        cs.ncol = 1; cs.col[0] = p; cs.typ[0] = x->typ;
        return group_dict(z, r, x->len, &cs, pre);
    }
    if (x->typ == H_G) {
        if (!list_of_basic(x)) return E_DOMAIN;
        int nc = (int)x->len;
        if (nc == 0) return group_dict(z, r, 0, nullptr);
        if (nc > KMAXC) return set_error(E_NOT_IMPL, "group by more than %d columns", KMAXC);
        V0* c = host_nodes(x);
        // one column: pfnOrderBy -> lib_order_basic sorts it as a vector (h_primitive.cc:1776-1778)
        if (nc == 1) return pfnGroupBasic(z, &c[0]);
        long long n = c[0].len;
        V cols[KMAXC];
        const void* ptrs[KMAXC];
        ColSet cs{};
        cs.ncol = nc;
        for (int i = 0; i < nc; i++) {
            if (c[i].len != n) return set_error(E_LENGTH, "group: columns of different lengths");
            cols[i] = &c[i];
            HG_CHECK(in_ptr(&c[i], &ptrs[i]));
            cs.col[i] = ptrs[i];
            cs.typ[i] = c[i].typ;
            if (!(is_real(c[i].typ) || c[i].typ == H_C || is_dtime(c[i].typ)))
                return set_error(E_NOT_IMPL, "group on symbol/string columns is outside the path");
        }
        if (nc == 2 && c[0].typ == H_I && c[1].typ == H_I) {  // pfnOrderBy -> checkOrderCase1
            KeySpec s{};
            s.ncol = 2;
            s.col[0] = ptrs[0]; s.typ[0] = H_I; s.xf[0] = XF_CASE1;
            s.col[1] = ptrs[1]; s.typ[1] = H_I;
            // 32 or 64 bits as lib_radixsort_long decides on the packed keys
            unsigned long long* k = (unsigned long long*)salloc((size_t)(n > 0 ? n : 1) * 8);
            if (!k) return E_DEVICE_OOM;
            if (n > 0) HG_LAUNCH("make_keys", gcap(n), 256, 0, k_make_keys<unsigned long long>, s, n, k);
            V0 tmp{};
            tmp.typ = H_L; tmp.len = n; tmp.g = (G)k;
            HG_CHECK(sort_int_column(&tmp, k, n, &r));
            return group_dict(z, r, n, &cs);
        }
        bool all_int = true;  // i32/i64 columns only: lib_quicksort_list merge sorts each = stable lexicographic
        for (int i = 0; i < nc; i++) all_int = all_int && (c[i].typ == H_I || c[i].typ == H_L);
        if (all_int) HG_CHECK(sort_columns(nc, cols, ptrs, nullptr, n, &r));
        else {
            I typs[KMAXC];
            B up[KMAXC];
            for (int i = 0; i < nc; i++) { typs[i] = c[i].typ; up[i] = 1; }
            HG_CHECK(qs_sort_list(nc, ptrs, typs, up, n, &r.perm));
            r.keys = nullptr;
            r.key64 = 0;
            r.key_injective = false;
        }
        return group_dict(z, r, n, &cs);
    }
    if (x->typ == H_C) {
        const void* p;
        HG_CHECK(in_ptr(x, &p));
        HG_CHECK(sort_char(p, x->len, &r));
        ColSet cs{};
        cs.ncol = 1; cs.col[0] = p; cs.typ[0] = H_C;
        return group_dict(z, r, x->len, &cs);
    }
    if (is_real(x->typ) || is_dtime(x->typ)) {  // pfnOrderBy -> lib_order_by_vector: the reference's quicksort
        const void* p;
        HG_CHECK(in_ptr(x, &p));
        HG_CHECK(qs_sort_vector(p, x->typ, x->len, true, &r.perm));
        r.keys = nullptr;
        r.key64 = 0;
        r.key_injective = false;
        ColSet cs{};
        cs.ncol = 1; cs.col[0] = p; cs.typ[0] = x->typ;
        return group_dict(z, r, x->len, &cs);
    }
    return set_error(E_NOT_IMPL, "group on this type is outside the path");
}

I pfnGroup(V z, V x) {
    if (x->typ == H_G && x->len == 2) {
        V0* c = host_nodes(x);
        if (c[0].typ == H_C && c[1].typ == H_C && c[0].len == c[1].len) return pfnGroupTrie(z, x);
    }
    return pfnGroupBasic(z, x);
}

static I order_basic(V z, V x, V y) {
    if (!(is_basic(x->typ) && y->typ == H_B && y->len == 1)) return 1;  // lib_order_basic returns 1
    uint64_t b;
    HG_CHECK(read_elem0(y, &b));
    bool asc = (b & 1) != 0;
    long long n = x->len;
    const void* p;
    HG_CHECK(in_ptr(x, &p));
    SortResult r{};
    if (x->typ == H_I || x->typ == H_L) {
        RadixOut ro;
        void* d;
        HG_CHECK(order_prealloc(z, n, !asc, &ro, &d));
        HG_CHECK(sort_int_column(x, p, n, &r, nullptr, d ? &ro : nullptr));
        return order_output(z, r, n, !asc, d);
    }
    if (x->typ == H_C) {
        if (!asc) return set_error(E_NOT_IMPL, "descending char order (the reference indexes past the range)");
        HG_CHECK(sort_char(p, n, &r));
        return order_output(z, r, n, false);
    }
    if (is_real(x->typ) || is_dtime(x->typ)) {  // lib_order_by_vector: the reference's quicksort
        HG_CHECK(qs_sort_vector(p, x->typ, n, asc, &r.perm));
        return order_output(z, r, n, false);
    }
    return set_error(E_NOT_IMPL, "order on this type is outside the path");
}

I pfnOrderBy(V z, V x, V y) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (x->typ == H_G && y->typ == H_B && x->len == y->len) {
        if (!list_of_basic(x)) return E_DOMAIN;
        int nc = (int)x->len;
        V0* c = host_nodes(x);
        const void* pb;
        HG_CHECK(in_ptr(y, &pb));
        B dir[KMAXC + 1];
        if (nc > KMAXC) return set_error(E_NOT_IMPL, "order by more than %d columns", KMAXC);
        if (nc > 0) {
            HG_CU(cudaMemcpyAsync(dir, pb, nc, cudaMemcpyDefault, g_stream));
            HG_CU(stream_sync());
        }
        long long n = nc ? c[0].len : 0;
        SortResult r{};
        if (nc == 2 && c[0].typ == H_I && c[1].typ == H_I && dir[0] == dir[1]) {  // checkOrderCase1
            const void *p0, *p1;
            HG_CHECK(in_ptr(&c[0], &p0));
            HG_CHECK(in_ptr(&c[1], &p1));
            KeySpec s{};
            s.ncol = 2;
            s.col[0] = p0; s.typ[0] = H_I; s.xf[0] = XF_CASE1;
            s.col[1] = p1; s.typ[1] = H_I;
            unsigned long long* k = (unsigned long long*)salloc((size_t)(n > 0 ? n : 1) * 8);
            if (!k) return E_DEVICE_OOM;
            if (n > 0) HG_LAUNCH("make_keys", gcap(n), 256, 0, k_make_keys<unsigned long long>, s, n, k);
            V0 tmp{};
            tmp.typ = H_L; tmp.len = n; tmp.g = (G)k;
            RadixOut ro;
            void* d;
            HG_CHECK(order_prealloc(z, n, !dir[0], &ro, &d));
            HG_CHECK(sort_int_column(&tmp, k, n, &r, nullptr, d ? &ro : nullptr));
            return order_output(z, r, n, !dir[0], d);
        }
        if (nc == 1) return order_basic(z, &c[0], y);
        V cols[KMAXC];
        const void* ptrs[KMAXC];
        bool all_int = true;
        for (int i = 0; i < nc; i++) {
            if (c[i].len != n) return E_LENGTH;
            if (!(is_real(c[i].typ) || is_dtime(c[i].typ) || c[i].typ == H_C))
                return set_error(E_NOT_IMPL, "order on symbol or string columns is outside the path");
            cols[i] = &c[i];
            HG_CHECK(in_ptr(&c[i], &ptrs[i]));
            all_int = all_int && (c[i].typ == H_I || c[i].typ == H_L);
        }
        if (!all_int) {  // lib_quicksort_list with the quicksort or the char sort on some column
            I typs[KMAXC];
            for (int i = 0; i < nc; i++) typs[i] = c[i].typ;
            HG_CHECK(qs_sort_list(nc, ptrs, typs, dir, n, &r.perm));
            return order_output(z, r, n, false);
        }
        bool all_asc = true;
        for (int i = 0; i < nc; i++) all_asc = all_asc && dir[i];
        if (all_asc) {
            RadixOut ro;
            void* d;
            HG_CHECK(order_prealloc(z, n, false, &ro, &d));
            HG_CHECK(sort_columns(nc, cols, ptrs, dir, n, &r, d ? &ro : nullptr));
            return order_output(z, r, n, false, d);
        }
        HG_CHECK(order_columns_exact(nc, cols, ptrs, dir, n, &r));
        return order_output(z, r, n, false);
    }
    I rc = order_basic(z, x, y);
    return rc;
}

}  // extern "C"
