// Batched filter-join-aggregate plans (many independent queries, one set of
// launches).
//
// Each plan is the join + group-by query the interpreter runs as
//   d = (dim.date >= lo) & (dim.date < hi); pk2 = compress(d, dim.pk)
//   j = join_index(eq, pk2, fact.fk); fi = j[1]
//   flag' status' qty' price' disc' = index(fact.col, fi)
//   g = group(list(flag', status'))                      (pfnGroupTrie)
//   sum(qty'), avg(price'), sum(disc'), count per group  (hgpuGroup*)
// and hgpuBatchJoinGroup runs every stage for all plans in one launch:
// tiles never straddle two plans, and each plan's look-back stops at its
// first tile, so every plan sees exactly the computation the plain builtins
// perform on it alone: the matched fact rows in row order, the groups'
// stable order by (flag<<8 | status), and per group the same fixed-order
// tile-tree sums (the same seg_sum kernels).  Results are therefore
// bit-identical to running the plans one at a time through the builtins.
//
// The batched kernels cover plans with unique dimension keys whose range is
// at most 64x the dimension (direct presence bitmaps), a compressed key
// column no longer than the fact table, and at most 256 groups.  Any other
// plan of the batch runs through the builtins one call at a time
// (plan_through_builtins), so every result is still the builtins' own.
#include <algorithm>
#include <climits>
#include <cstring>
#include <map>
#include <vector>

#include "dev_common.cuh"

namespace hg {

I scan_exclusive(const unsigned* in, long long n, unsigned long long* out, unsigned long long* total_h);
I scan_counts(const unsigned* counts, long long n, unsigned long long* offs);
I seg_sum_f64(const double* src, const long long* rows, long long nx, const long long* starts, long long ng,
              long long total, double* out);

constexpr int BT = 4096;  // rows per tile

struct DPlan {
    const int* pk;
    const int* date;
    long long nd;
    const int* fk;
    const int8_t* flag;
    const int8_t* status;
    const double* qty;
    const double* price;
    const double* disc;
    long long nf;
    int lo, hi;
    long long kmin, kmax;      // pk range
    unsigned* bitmap;          // pk presence, bit (pk - kmin)
    long long fact_off;        // fact-row offset of the plan's region in the fi buffer
    unsigned* codebits;        // 65536-bit presence of group codes
    unsigned short* dense;     // code -> dense group id (65536 entries)
};

// plan of a tile: tile_first[p] = first tile of plan p, tile_first[np] = total tiles
__device__ __forceinline__ int plan_of_tile(const long long* tile_first, int np, long long t) {
    int lo = 0, hi = np - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tile_first[mid] <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// cp.async global -> shared, 4 bytes (holds no register while in flight)
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// ---------------------------------------------------------------- stage 0/1
__global__ void k_b_minmax(const DPlan* __restrict__ P, const long long* __restrict__ tile_first, int np,
                           long long* __restrict__ mm) {
    const long long t = blockIdx.x;
    const int p = plan_of_tile(tile_first, np, t);
    const long long r0 = (t - tile_first[p]) * BT;
    long long a = LLONG_MAX, b = LLONG_MIN;
    for (long long i = r0 + threadIdx.x; i < r0 + BT && i < P[p].nd; i += blockDim.x) {
        long long v = P[p].pk[i];
        a = v < a ? v : a;
        b = v > b ? v : b;
    }
    for (int o = 16; o > 0; o >>= 1) {
        long long q = __shfl_xor_sync(0xffffffffu, a, o); a = q < a ? q : a;
        long long r = __shfl_xor_sync(0xffffffffu, b, o); b = r > b ? r : b;
    }
    // one atomic pair per block: per-warp atomics on a plan's two words serialise
    __shared__ long long wa[8], wb[8];
    if (lane_id() == 0) { wa[threadIdx.x >> 5] = a; wb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { a = wa[w] < a ? wa[w] : a; b = wb[w] > b ? wb[w] : b; }
        atomicMin(&mm[2 * p], a);
        atomicMax(&mm[2 * p + 1], b);
    }
}

// dimension rows inside the date window set their key's presence bit; nsel
// counts them (the length of the compressed key column)
__global__ void k_b_build(const DPlan* __restrict__ P, const long long* __restrict__ tile_first, int np,
                          unsigned* __restrict__ dup, unsigned long long* __restrict__ nsel) {
    const long long t = blockIdx.x;
    const int p = plan_of_tile(tile_first, np, t);
    const DPlan& q = P[p];
    const long long r0 = (t - tile_first[p]) * BT;
    unsigned cnt = 0;
    for (long long i = r0 + threadIdx.x; i < r0 + BT && i < q.nd; i += blockDim.x) {
        int d = q.date[i];
        long long b = (long long)q.pk[i] - q.kmin;
        if (d >= q.lo && d < q.hi && b >= 0 && b <= q.kmax - q.kmin) {
            unsigned bit = 1u << (b & 31);
            unsigned old = atomicOr(&q.bitmap[b >> 5], bit);
            if (old & bit) atomicOr(&dup[p], 1u);
            cnt++;
        }
    }
    __shared__ unsigned wc[8];
    cnt = warp_sum(cnt);
    if (lane_id() == 0) wc[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned c = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) c += wc[w];
        if (c) atomicAdd(&nsel[p], (unsigned long long)c);
    }
}

// ---------------------------------------------------------------- stage 2
// probe, pass 1: one bit per fact row of each plan (its key is in the
// plan's presence bitmap) and the tile's count.  A tile is 256 x R rows (R,
// 8 to 32, is the autotuner's tile knob): warp w owns words [w R, w R + R) of
// the tile's 8 R bit words, lane l row 32 k + l of word k.  The keys and then
// their presence words come by cp.async into the thread's own shared-memory
// column, all R of a group in flight together.
template <int R>
__global__ void __launch_bounds__(256) k_b_probe(const DPlan* __restrict__ P, const long long* __restrict__ tile_first,
                                                 int np, unsigned* __restrict__ bits, unsigned* __restrict__ counts) {
    extern __shared__ unsigned bp_smem[];
    unsigned(*koff)[256] = reinterpret_cast<unsigned(*)[256]>(bp_smem);            // key - kmin, NONE when out of range
    unsigned(*word)[256] = reinterpret_cast<unsigned(*)[256]>(bp_smem + R * 256);  // presence word of the key
    __shared__ unsigned wc[8];
    constexpr unsigned NONE = 0xffffffffu;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5, me = threadIdx.x;
    const long long t = blockIdx.x;
    const int p = plan_of_tile(tile_first, np, t);
    const DPlan& q = P[p];
    const long long base = (t - tile_first[p]) * (256LL * R) + (long long)warp * (32 * R);  // plan-relative row
    const long long nf = q.nf;
#pragma unroll
    for (int k = 0; k < R; k++) {
        long long i = base + k * 32 + lane;
        if (i < nf) cp_async4(&koff[k][me], q.fk + i);
    }
    cp_async_wait_all();
    const unsigned long long range = (unsigned long long)(q.kmax - q.kmin);  // < 2^31 (host check)
#pragma unroll
    for (int k = 0; k < R; k++) {
        long long i = base + k * 32 + lane;
        long long v = i < nf ? (long long)(int)koff[k][me] - q.kmin : -1;
        unsigned o = (q.kmax >= q.kmin && (unsigned long long)v <= range) ? (unsigned)v : NONE;
        koff[k][me] = o;
        if (o != NONE) cp_async4(&word[k][me], q.bitmap + (o >> 5));
    }
    cp_async_wait_all();
    unsigned cnt = 0;
    unsigned* wout = bits + t * (8LL * R) + (long long)warp * R;
#pragma unroll
    for (int k = 0; k < R; k++) {
        unsigned o = koff[k][me];
        bool m = o != NONE && ((word[k][me] >> (o & 31)) & 1u);
        unsigned bal = __ballot_sync(0xffffffffu, m);
        if (lane == 0) wout[k] = bal;
        cnt += __popc(bal);
    }
    if (lane == 0) wc[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned c = 0;
        for (int w = 0; w < 8; w++) c += wc[w];
        counts[t] = c;
    }
}

// where each tile map's plan writes its rows: its region of the matched-row
// buffer and its slot in mcount
struct EmitPlan {
    long long fact_off;
    int p;
};

// pass 2 (probe and shared selection): each tile writes the plan-relative
// row numbers of its set bits from its offset within the plan (the scan of
// the tile counts, less the scan at the plan's first tile); warp w walks its
// R words, and a word is already the ballot of its 32 rows.  The plan's last
// tile stores the plan's match count.
template <int R>
__global__ void __launch_bounds__(256) k_b_emit(const EmitPlan* __restrict__ E, const long long* __restrict__ tile_first,
                                                int np, const unsigned* __restrict__ bits,
                                                const unsigned long long* __restrict__ offs, unsigned* __restrict__ fi,
                                                unsigned long long* __restrict__ mcount) {
    __shared__ unsigned wc[8];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long t = blockIdx.x;
    const int c = plan_of_tile(tile_first, np, t);
    const long long first = tile_first[c];
    const unsigned* w = bits + t * (8LL * R) + (long long)warp * R;
    unsigned wd[R];
    unsigned cnt = 0;
#pragma unroll
    for (int k = 0; k < R; k++) {
        wd[k] = w[k];
        cnt += __popc(wd[k]);
    }
    if (lane == 0) wc[warp] = cnt;
    __syncthreads();
    unsigned long long off = offs[t] - offs[first];
    for (unsigned v = 0; v < warp; v++) off += wc[v];
    const long long base = (t - first) * (256LL * R) + (long long)warp * (32 * R);
    unsigned* out = fi + E[c].fact_off;
#pragma unroll
    for (int k = 0; k < R; k++) {
        if ((wd[k] >> lane) & 1u) out[off + __popc(wd[k] & lanemask_lt())] = (unsigned)(base + k * 32 + lane);
        off += __popc(wd[k]);
    }
    if (threadIdx.x == 0 && t + 1 == tile_first[c + 1]) mcount[E[c].p] = offs[t + 1] - offs[first];
}

// ---------------------------------------------------------------- shared tables
// Plans over the same dimension and fact columns (a served stream's join
// requests) share one probe: the dimension's dates are stored by key once,
// every fact row looks up the date of its dimension row once, and each plan
// then only selects the rows whose date lies in its window.  With unique
// keys the selected rows are exactly the rows the plan's own probe matches,
// in the same (fact-row) order.
constexpr unsigned short NO_DATE = 0xffffu;

__global__ void k_sh_minmax(const int* __restrict__ a, const int* __restrict__ b, long long n, long long* mm) {
    long long amin = LLONG_MAX, amax = LLONG_MIN, bmin = LLONG_MAX, bmax = LLONG_MIN;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long x = a[i], y = b[i];
        amin = x < amin ? x : amin; amax = x > amax ? x : amax;
        bmin = y < bmin ? y : bmin; bmax = y > bmax ? y : bmax;
    }
    for (int o = 16; o > 0; o >>= 1) {
        long long q;
        q = __shfl_xor_sync(0xffffffffu, amin, o); amin = q < amin ? q : amin;
        q = __shfl_xor_sync(0xffffffffu, amax, o); amax = q > amax ? q : amax;
        q = __shfl_xor_sync(0xffffffffu, bmin, o); bmin = q < bmin ? q : bmin;
        q = __shfl_xor_sync(0xffffffffu, bmax, o); bmax = q > bmax ? q : bmax;
    }
    if (lane_id() == 0) {
        atomicMin(&mm[0], amin); atomicMax(&mm[1], amax);
        atomicMin(&mm[2], bmin); atomicMax(&mm[3], bmax);
    }
}

// date offset by key (NO_DATE where no dimension row has the key), a
// repeated-key flag, and the histogram of the dimension's date offsets
__global__ void k_sh_build(const int* __restrict__ pk, const int* __restrict__ date, long long nd, long long kmin,
                           int dmin, int drange, unsigned short* __restrict__ dt, unsigned* __restrict__ dimhist,
                           unsigned* dup) {
    extern __shared__ unsigned sh_hist[];
    const bool local = drange <= 8192;
    if (local) for (int i = threadIdx.x; i < drange; i += blockDim.x) sh_hist[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
        long long k = (long long)pk[i] - kmin;
        unsigned short dv = (unsigned short)(date[i] - dmin);
        unsigned short old = atomicCAS(dt + k, NO_DATE, dv);
        if (old != NO_DATE) atomicOr(dup, 1u);
        if (local) atomicAdd(&sh_hist[dv], 1u);
        else atomicAdd(&dimhist[dv], 1u);
    }
    __syncthreads();
    if (local)
        for (int i = threadIdx.x; i < drange; i += blockDim.x)
            if (sh_hist[i]) atomicAdd(&dimhist[i], sh_hist[i]);
}

// date offset of every fact row's dimension row, and their histogram
__global__ void k_sh_probe(const int* __restrict__ fk, long long nf, long long kmin, unsigned long long kspan,
                           const unsigned short* __restrict__ dt, int drange, unsigned short* __restrict__ dd,
                           unsigned* __restrict__ facthist) {
    extern __shared__ unsigned sh_hist[];
    const bool local = drange <= 8192;
    if (local) for (int i = threadIdx.x; i < drange; i += blockDim.x) sh_hist[i] = 0;
    __syncthreads();
    for (long long i0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) * 4; i0 < nf;
         i0 += (long long)gridDim.x * blockDim.x * 4) {
        unsigned short d[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            long long i = i0 + u;
            d[u] = NO_DATE;
            if (i < nf) {
                unsigned long long v = (unsigned long long)((long long)__ldcs(fk + i) - kmin);
                if (v < kspan) d[u] = __ldg(dt + v);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (i0 + u < nf) {
                dd[i0 + u] = d[u];
                if (d[u] != NO_DATE) {
                    if (local) atomicAdd(&sh_hist[d[u]], 1u);
                    else atomicAdd(&facthist[d[u]], 1u);
                }
            }
        }
    }
    __syncthreads();
    if (local)
        for (int i = threadIdx.x; i < drange; i += blockDim.x)
            if (sh_hist[i]) atomicAdd(&facthist[i], sh_hist[i]);
}

// ---------------------------------------------------------------- shared tables, grouped
// When every row's (flag, status) code falls in at most SG_MAXG distinct
// values, the plans over one table set skip the per-plan gather and sort:
// one pass counts, per tile, the rows of each (plan, group), a scan turns the
// counts into positions, and a second pass reads each fact tile once and
// writes every plan's matching values straight into that plan's group-ordered
// arrays (rows of a group in fact-row order, as the builtins' @group lists
// them), which the fixed-order segmented sums then reduce in place.
constexpr int SG_MAXG = 8, SG_MAXP = 32, SG_R = 8;
constexpr long long SG_TILE = 256LL * SG_R;

// presence bits of the codes (flag << 8 | status) over the fact table
__global__ void k_sg_codes(const int8_t* __restrict__ flag, const int8_t* __restrict__ status, long long n,
                           unsigned* __restrict__ bits) {
    __shared__ unsigned sb[2048];
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) sb[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned c = ((unsigned)(uint8_t)flag[i] << 8) | (unsigned)(uint8_t)status[i];
        unsigned bit = 1u << (c & 31);
        if (!(sb[c >> 5] & bit)) atomicOr(&sb[c >> 5], bit);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2048; i += blockDim.x)
        if (sb[i]) atomicOr(&bits[i], sb[i]);
}

// The tile preamble shared by both passes: each lane's SG_R date offsets,
// and in lane c (c < G) the ballot of "row has group c" for each round k
// (mygb[k]), so that a (plan, group c) count is a popc in lane c.
__device__ __forceinline__ void sg_tile(const unsigned short* __restrict__ dd, const int8_t* __restrict__ flag,
                                        const int8_t* __restrict__ status, const unsigned char* __restrict__ dense,
                                        long long nf, long long base, int G, unsigned short (&d)[SG_R],
                                        unsigned (&mygb)[SG_R], unsigned char (&g)[SG_R]) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int k = 0; k < SG_R; k++) {
        long long i = base + k * 32 + lane;
        d[k] = 0xffffu;
        g[k] = 0xff;
        if (i < nf) {
            d[k] = __ldcs(dd + i);
            g[k] = __ldg(dense + (((unsigned)(uint8_t)flag[i] << 8) | (unsigned)(uint8_t)status[i]));
        }
        mygb[k] = 0;
    }
#pragma unroll
    for (int k = 0; k < SG_R; k++)
        for (int c = 0; c < G; c++) {
            const unsigned b = __ballot_sync(0xffffffffu, g[k] == c);
            if ((int)lane == c) mygb[k] = b;
        }
}

// this warp's rows of every (plan, group): wc[w][pl * G + c]
__device__ __forceinline__ void sg_warp_counts(const unsigned short (&d)[SG_R], const unsigned (&mygb)[SG_R],
                                               const int* __restrict__ wins, int npl, int G, unsigned* wcw) {
    const unsigned lane = lane_id();
    for (int pl = 0; pl < npl; pl++) {
        const int lo = wins[2 * pl], hi = wins[2 * pl + 1];
        unsigned n = 0;
#pragma unroll
        for (int k = 0; k < SG_R; k++) n += __popc(__ballot_sync(0xffffffffu, (int)d[k] >= lo && (int)d[k] < hi) & mygb[k]);
        if ((int)lane < G) wcw[pl * G + lane] = n;
    }
}

// pass 1: counts[(pl * G + g) * ntiles + t] = rows of plan pl and group g in tile t
__global__ void __launch_bounds__(256) k_sg_count(const unsigned short* __restrict__ dd, const int8_t* __restrict__ flag,
                                                  const int8_t* __restrict__ status,
                                                  const unsigned char* __restrict__ dense, long long nf,
                                                  const int* __restrict__ wins, int npl, int G,
                                                  unsigned* __restrict__ counts, long long ntiles) {
    __shared__ unsigned wc[8][SG_MAXP * SG_MAXG];
    const unsigned w = threadIdx.x >> 5;
    const long long t = blockIdx.x, base = t * SG_TILE + (long long)w * (32 * SG_R);
    unsigned short d[SG_R];
    unsigned mygb[SG_R];
    unsigned char g[SG_R];
    sg_tile(dd, flag, status, dense, nf, base, G, d, mygb, g);
    sg_warp_counts(d, mygb, wins, npl, G, wc[w]);
    __syncthreads();
    for (int j = threadIdx.x; j < npl * G; j += blockDim.x) {
        unsigned n = 0;
        for (int v = 0; v < 8; v++) n += wc[v][j];
        counts[(long long)j * ntiles + t] = n;
    }
}

// one block per (plan, group): exclusive scan of its tile counts into offs,
// total into totals[j]
__global__ void __launch_bounds__(1024) k_sg_scan(const unsigned* __restrict__ counts, long long ntiles,
                                                  unsigned long long* __restrict__ offs,
                                                  unsigned long long* __restrict__ totals) {
    __shared__ unsigned long long wsum[32];
    __shared__ unsigned long long carry;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long j = blockIdx.x;
    const unsigned* in = counts + j * ntiles;
    unsigned long long* out = offs + j * ntiles;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long c0 = 0; c0 < ntiles; c0 += 1024 * 8) {
        const long long b = c0 + (long long)threadIdx.x * 8;
        unsigned v[8];
        unsigned long long sum = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            v[k] = b + k < ntiles ? in[b + k] : 0u;
            sum += v[k];
        }
        unsigned long long incl = warp_incl_scan64(sum);
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            unsigned long long x = wsum[lane];
            wsum[lane] = warp_incl_scan64(x) - x;
        }
        __syncthreads();
        unsigned long long off = carry + wsum[warp] + (incl - sum);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (b + k < ntiles) out[b + k] = off;
            off += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry = off;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[j] = carry;
}

// pass 2: every plan's matching rows of the tile, values written to
// base[j] + offs[j * ntiles + t] + (rows of the same (plan, group) earlier in
// the tile).  Lane c keeps the next position of group c; a matching row takes
// its group's position (shuffled from lane g) plus the matching rows of its
// group in lower lanes of the round.
__global__ void __launch_bounds__(256) k_sg_scatter(const unsigned short* __restrict__ dd, const int8_t* __restrict__ flag,
                                                    const int8_t* __restrict__ status,
                                                    const unsigned char* __restrict__ dense, const double* __restrict__ qty,
                                                    const double* __restrict__ price, const double* __restrict__ disc,
                                                    long long nf, const int* __restrict__ wins, int npl, int G,
                                                    const unsigned long long* __restrict__ offs,
                                                    const unsigned long long* __restrict__ base, long long ntiles,
                                                    double* __restrict__ vq, double* __restrict__ vp,
                                                    double* __restrict__ vd) {
    __shared__ unsigned wc[8][SG_MAXP * SG_MAXG];
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;
    const long long t = blockIdx.x, rbase = t * SG_TILE + (long long)w * (32 * SG_R);
    unsigned short d[SG_R];
    unsigned mygb[SG_R];
    unsigned char g[SG_R];
    sg_tile(dd, flag, status, dense, nf, rbase, G, d, mygb, g);
    double q[SG_R], pr[SG_R], ds[SG_R];
#pragma unroll
    for (int k = 0; k < SG_R; k++) {
        long long i = rbase + k * 32 + lane;
        const bool ok = i < nf;
        q[k] = ok ? __ldcs(qty + i) : 0.0;
        pr[k] = ok ? __ldcs(price + i) : 0.0;
        ds[k] = ok ? __ldcs(disc + i) : 0.0;
    }
    sg_warp_counts(d, mygb, wins, npl, G, wc[w]);
    __syncthreads();
    for (int j = threadIdx.x; j < npl * G; j += blockDim.x) {
        unsigned acc = 0;
        for (int v = 0; v < 8; v++) { unsigned n = wc[v][j]; wc[v][j] = acc; acc += n; }
    }
    __syncthreads();
    for (int pl = 0; pl < npl; pl++) {
        const int lo = wins[2 * pl], hi = wins[2 * pl + 1];
        unsigned long long pos = 0;  // lane c < G: next position of group c
        if ((int)lane < G) {
            const int j = pl * G + (int)lane;
            pos = base[j] + offs[(long long)j * ntiles + t] + wc[w][j];
        }
#pragma unroll
        for (int k = 0; k < SG_R; k++) {
            const bool m = (int)d[k] >= lo && (int)d[k] < hi;
            const unsigned mb = __ballot_sync(0xffffffffu, m);
            const int src = g[k] & 7;  // a non-matching lane's group is immaterial
            const unsigned same = __shfl_sync(0xffffffffu, mygb[k], src);
            const unsigned long long at = __shfl_sync(0xffffffffu, pos, src);
            if (m) {
                const unsigned long long o = at + __popc(mb & same & lanemask_lt());
                vq[o] = q[k];
                vp[o] = pr[k];
                vd[o] = ds[k];
            }
            pos += __popc(mb & mygb[k]);
        }
    }
}

struct CPlan {
    const unsigned short* dd;
    long long nf;
    int dlo, dhi;        // selected date offsets [dlo, dhi)
    long long fact_off;  // the plan's region of the matched-row buffer
    int p;               // index in the batch
};

// shared selection, pass 1: one bit per fact row of each plan (its date
// offset lies in the plan's window) and the tile's count; the k_b_probe
// layout
template <int R>
__global__ void __launch_bounds__(256) k_sh_select(const CPlan* __restrict__ P, const long long* __restrict__ tile_first,
                                                   int np, unsigned* __restrict__ bits, unsigned* __restrict__ counts) {
    __shared__ unsigned wc[8];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const long long t = blockIdx.x;
    const int c = plan_of_tile(tile_first, np, t);
    const CPlan& q = P[c];
    const long long base = (t - tile_first[c]) * (256LL * R) + (long long)warp * (32 * R);
    unsigned short d[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
        long long i = base + k * 32 + lane;
        d[k] = i < q.nf ? __ldcs(q.dd + i) : NO_DATE;
    }
    unsigned cnt = 0;
    unsigned* wout = bits + t * (8LL * R) + (long long)warp * R;
#pragma unroll
    for (int k = 0; k < R; k++) {
        bool m = (int)d[k] >= q.dlo && (int)d[k] < q.dhi;  // NO_DATE is above every window
        unsigned bal = __ballot_sync(0xffffffffu, m);
        if (lane == 0) wout[k] = bal;
        cnt += __popc(bal);
    }
    if (lane == 0) wc[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned s = 0;
        for (int w = 0; w < 8; w++) s += wc[w];
        counts[t] = s;
    }
}

// exclusive prefix of the per-plan match counts (one block)
__global__ void k_b_offsets(const unsigned long long* __restrict__ mcount, int np, long long* __restrict__ moff) {
    if (threadIdx.x == 0) {
        long long acc = 0;
        for (int p = 0; p < np; p++) { moff[p] = acc; acc += (long long)mcount[p]; }
        moff[np] = acc;
    }
}

// ---------------------------------------------------------------- stage 3
// gather the matched rows' columns into contiguous per-plan vectors, and
// record which group codes occur
__global__ void k_b_gather(const DPlan* __restrict__ P, const long long* __restrict__ tile_first, int np,
                           const unsigned* __restrict__ fi, const unsigned long long* __restrict__ mcount,
                           const long long* __restrict__ moff, unsigned* __restrict__ code, double* __restrict__ qty,
                           double* __restrict__ price, double* __restrict__ disc) {
    // codes seen by this block, merged into the plan's presence bits once
    // at the end (a few atomics per block instead of a few per warp)
    __shared__ unsigned seen[2048];
    for (int k = threadIdx.x; k < 2048; k += blockDim.x) seen[k] = 0;
    __syncthreads();
    const long long t = blockIdx.x;
    const int p = plan_of_tile(tile_first, np, t);
    const DPlan& q = P[p];
    const long long r0 = (t - tile_first[p]) * BT;
    const long long m = (long long)mcount[p], o = moff[p];
    const long long end = (r0 + BT < m) ? r0 + BT : m;
    const unsigned* __restrict__ rows = fi + q.fact_off;
    const int8_t* __restrict__ fl = q.flag;
    const int8_t* __restrict__ stt = q.status;
    const double* __restrict__ cq = q.qty;
    const double* __restrict__ cp = q.price;
    const double* __restrict__ cd = q.disc;
    // 4 rows per thread per round, all 24 loads issued before any store
    for (long long i0 = r0 + threadIdx.x; i0 < end; i0 += 4 * (long long)blockDim.x) {
        unsigned r[4];
        bool v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            v[u] = i0 + u * (long long)blockDim.x < end;
            r[u] = v[u] ? rows[i0 + u * blockDim.x] : 0u;
        }
        unsigned c[4];
        double a[4], b[4], d[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (v[u]) {
                c[u] = ((unsigned)(uint8_t)fl[r[u]] << 8) | (unsigned)(uint8_t)stt[r[u]];
                a[u] = cq[r[u]];
                b[u] = cp[r[u]];
                d[u] = cd[r[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (v[u]) {
                long long i = o + i0 + u * (long long)blockDim.x;
                code[i] = c[u];
                qty[i] = a[u];
                price[i] = b[u];
                disc[i] = d[u];
                unsigned bit = 1u << (c[u] & 31);
                if (!(seen[c[u] >> 5] & bit)) atomicOr(&seen[c[u] >> 5], bit);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2048; k += blockDim.x)
        if (seen[k]) atomicOr(&q.codebits[k], seen[k]);
}

// code -> dense group id (ascending codes), one block per plan
__global__ void k_b_dense(const DPlan* __restrict__ P, unsigned* __restrict__ ngroups, unsigned* __restrict__ codes) {
    const int p = blockIdx.x;
    const DPlan& q = P[p];
    __shared__ unsigned wsum[8];
    // 2048 words, 8 per thread
    unsigned c[8], tot = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) { c[k] = __popc(q.codebits[threadIdx.x * 8 + k]); tot += c[k]; }
    unsigned inc = warp_incl_scan(tot);
    if (lane_id() == 31) wsum[threadIdx.x >> 5] = inc;
    __syncthreads();
    unsigned before = 0;
    for (unsigned w = 0; w < (threadIdx.x >> 5); w++) before += wsum[w];
    unsigned id = before + inc - tot;
    for (int k = 0; k < 8; k++) {
        unsigned word = q.codebits[threadIdx.x * 8 + k];
        for (int b = 0; b < 32; b++) {
            unsigned cd = (threadIdx.x * 8 + k) * 32 + b;
            if ((word >> b) & 1u) {
                if (id < 256) codes[p * 256 + id] = cd;
                q.dense[cd] = (unsigned short)id++;
            }
        }
    }
    if (threadIdx.x == 255) ngroups[p] = id;
}

// ---------------------------------------------------------------- stage 4
// per-plan histograms of the dense group ids
__global__ void k_b_hist(const DPlan* __restrict__ P, const long long* __restrict__ tile_first, int np,
                         const unsigned long long* __restrict__ mcount, const long long* __restrict__ moff,
                         const unsigned* __restrict__ code, unsigned* __restrict__ hist) {
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long t = blockIdx.x;
    const int p = plan_of_tile(tile_first, np, t);
    const long long r0 = (t - tile_first[p]) * BT, m = (long long)mcount[p], o = moff[p];
    for (long long i = r0 + threadIdx.x; i < r0 + BT && i < m; i += blockDim.x)
        atomicAdd(&h[P[p].dense[code[o + i]] & 255], 1u);
    __syncthreads();
    if (h[threadIdx.x]) atomicAdd(&hist[p * 256 + threadIdx.x], h[threadIdx.x]);
}

__global__ void k_b_bucket(const unsigned* __restrict__ hist, unsigned* __restrict__ bucket) {
    __shared__ unsigned s[256];
    const int p = blockIdx.x, d = threadIdx.x;
    s[d] = hist[p * 256 + d];
    __syncthreads();
    if (d == 0) {
        unsigned acc = 0;
        for (int i = 0; i < 256; i++) { unsigned v = s[i]; s[i] = acc; acc += v; }
    }
    __syncthreads();
    bucket[p * 256 + d] = s[d];
}

// one stable counting pass over the dense ids of each plan (the onesweep rank
// and per-digit look-back, restricted to the plan's tiles); writes, in group
// order, the global positions of the matched rows
__global__ void __launch_bounds__(256) k_b_sort(const DPlan* __restrict__ P, const long long* __restrict__ tile_first,
                                                int np, const unsigned long long* __restrict__ mcount,
                                                const long long* __restrict__ moff, const unsigned* __restrict__ code,
                                                const unsigned* __restrict__ bucket, long long* __restrict__ rows,
                                                unsigned long long* status, unsigned* ticket, unsigned* derr) {
    __shared__ unsigned whist[8][256];
    __shared__ unsigned long long dbase[256];
    __shared__ long long tile_id;
    for (int i = threadIdx.x; i < 8 * 256; i += 256) (&whist[0][0])[i] = 0;
    if (threadIdx.x == 0) tile_id = atomicAdd(ticket, 1u);
    __syncthreads();
    const long long t = tile_id;
    const int p = plan_of_tile(tile_first, np, t);
    const long long first = tile_first[p], m = (long long)mcount[p], o = moff[p];
    const unsigned lane = lane_id(), w = threadIdx.x >> 5;
    const long long wbase = (t - first) * BT + (long long)w * 512;
    unsigned rd[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        long long i = wbase + k * 32 + lane;
        bool valid = i < m;
        unsigned d = valid ? (P[p].dense[code[o + i]] & 255u) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        unsigned pre = 0;
        if ((int)lane == leader && valid) { pre = whist[w][d]; whist[w][d] = pre + __popc(peers); }
        pre = __shfl_sync(0xffffffffu, pre, leader);
        rd[k] = ((d & 0xffffu) << 16) | (pre + __popc(peers & lanemask_lt()));
        __syncwarp();
    }
    __syncthreads();
    {
        const int d = threadIdx.x;
        unsigned c = 0;
        for (int ww = 0; ww < 8; ww++) { unsigned h = whist[ww][d]; whist[ww][d] = c; c += h; }
        const unsigned long long excl = chain_lookback(status + d, 256, t, first, c, derr);
        dbase[d] = (unsigned long long)o + bucket[p * 256 + d] + excl;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; k++) {
        long long i = wbase + k * 32 + lane;
        if (i < m) {
            unsigned d = rd[k] >> 16;
            rows[dbase[d] + whist[w][d] + (rd[k] & 0xffffu)] = o + i;
        }
    }
}

// group starts of every plan, concatenated
__global__ void k_b_starts(const long long* __restrict__ moff, const unsigned* __restrict__ bucket,
                           const unsigned* __restrict__ ngroups, const long long* __restrict__ segoff, int np,
                           long long* __restrict__ starts) {
    const int p = blockIdx.x, g = threadIdx.x;
    if (g < (int)ngroups[p]) starts[segoff[p] + g] = moff[p] + bucket[p * 256 + g];
}

// avg = sum / count per group (k_avg_seg's division)
__global__ void k_b_avg(const double* __restrict__ s, const long long* __restrict__ starts, long long ng, long long total,
                        double* __restrict__ avg) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < ng; g += (long long)gridDim.x * blockDim.x) {
        long long m = ((g + 1 < ng) ? starts[g + 1] : total) - starts[g];
        avg[g] = __ddiv_rn(s[g], (double)m);
    }
}

static unsigned cap_grid(long long n) {
    unsigned g = grid_for(n, 256);
    return g > (unsigned)g_sms * 16 ? (unsigned)g_sms * 16 : g;
}

static V0 dev_col(const void* p, I typ, L n) {
    V0 v;
    memset(&v, 0, sizeof v);
    v.len = n;
    v.typ = typ;
    v.g = (G)p;
    return v;
}

static V0 int_scalar(I x) {
    V0 v;
    memset(&v, 0, sizeof v);
    v.len = 1;
    v.typ = H_I;
    v.i32 = x;
    v.g = (G)&v.b;
    return v;
}

// One plan through the builtins, call by call, exactly as the interpreter
// runs it.  Plans the batched kernels do not cover take this path, so every
// plan of a batch gets the builtins' own result.
I plan_through_builtins(const hgpuJoinGroupPlan& q, hgpuJoinGroupResult* r) {
    const L mark = getHeapOffset();
    I rc = 0;
    V0 pk = dev_col(q.dim_pk, H_I, q.ndim), date = dev_col(q.dim_date, H_I, q.ndim);
    V0 fk = dev_col(q.fk, H_I, q.nfact), flag = dev_col(q.flag, H_C, q.nfact), status = dev_col(q.status, H_C, q.nfact);
    V0 qty = dev_col(q.qty, H_E, q.nfact), price = dev_col(q.price, H_E, q.nfact), disc = dev_col(q.disc, H_E, q.nfact);
    V0 lo = int_scalar(q.lo), hi = int_scalar(q.hi), one;
    memset(&one, 0, sizeof one);
    one.len = 1; one.typ = H_L; one.i64 = 1; one.g = (G)&one.b;
    V0 eq;
    memset(&eq, 0, sizeof eq);
    eq.len = 1; eq.typ = H_Q; eq.q = getSymbol((S) "eq"); eq.g = (G)&eq.b;
    V0 d1, d2, d3, pk2, j, fi, gf, gs, gq, gp, gd, lst, g, keys, vals, of, os, sq, ap, sd, cnt;
    V0* ln;
#define STEP(call) do { if ((rc = (call)) != 0) goto done; } while (0)
    STEP(pfnGeq(&d1, &date, &lo));
    STEP(pfnLt(&d2, &date, &hi));
    STEP(pfnAnd(&d3, &d1, &d2));
    STEP(pfnCompress(&pk2, &d3, &pk));
    STEP(pfnJoinIndex(&j, &pk2, &fk, &eq));
    STEP(pfnIndex(&fi, &j, &one));
    STEP(pfnIndex(&gf, &flag, &fi));
    STEP(pfnIndex(&gs, &status, &fi));
    STEP(pfnIndex(&gq, &qty, &fi));
    STEP(pfnIndex(&gp, &price, &fi));
    STEP(pfnIndex(&gd, &disc, &fi));
    STEP(init_list(&lst, H_G, 2));
    ln = host_nodes(&lst);
    ln[0] = gf; ln[1] = gs;
    if (gf.len == 1) ln[0].g = (G)&ln[0].b;
    if (gs.len == 1) ln[1].g = (G)&ln[1].b;
    STEP(pfnGroup(&g, &lst));
    STEP(pfnKeys(&keys, &g));
    STEP(pfnValues(&vals, &g));
    if (keys.len > HGPU_PLAN_MAX_GROUPS) { rc = set_error(E_NOT_IMPL, "more than 256 groups"); goto done; }
    STEP(pfnIndex(&of, &gf, &keys));
    STEP(pfnIndex(&os, &gs, &keys));
    STEP(hgpuGroupSum(&sq, &gq, &vals));
    STEP(hgpuGroupAvg(&ap, &gp, &vals));
    STEP(hgpuGroupSum(&sd, &gd, &vals));
    STEP(hgpuGroupLen(&cnt, &gq, &vals));
    {
        const L n = keys.len;
        r->ngroups = n;
        V0* src[6] = {&of, &os, &sq, &ap, &sd, &cnt};
        void* dst[6] = {r->flag, r->st, r->sum_qty, r->avg_price, r->sum_disc, r->count};
        const size_t es[6] = {1, 1, 8, 8, 8, 8};
        for (int k = 0; k < 6 && n > 0; k++) {
            if (n == 1 || !is_device_ptr(src[k]->g)) memcpy(dst[k], src[k]->g, es[k] * n);
            else if (cudaMemcpyAsync(dst[k], src[k]->g, es[k] * n, cudaMemcpyDeviceToHost, g_stream) != cudaSuccess) {
                rc = set_error(E_DEVICE, "copying a plan result");
                goto done;
            }
        }
        if (stream_sync() != cudaSuccess) rc = set_error(E_DEVICE, "copying a plan result");
    }
#undef STEP
done:
    setHeapOffset(mark);
    return rc;
}

I seg_sum_f64_direct(const double* src, const long long* starts, long long ng, long long total, double* out);

// The grouped path for the plans `ps` over one table set (date offsets dd
// already computed).  Returns 1 when it ran (results in out[p], done[p] set),
// 0 when the table set has more than SG_MAXG codes.
static I shared_grouped(const hgpuJoinGroupPlan* plans, const std::vector<int>& ps, const std::vector<int>& plo,
                        const std::vector<int>& phi, const unsigned short* dd, hgpuJoinGroupResult* out,
                        std::vector<char>* done, int* ran) {
    *ran = 0;
    const hgpuJoinGroupPlan& q0 = plans[ps[0]];
    const long long nf = q0.nfact;
    unsigned* bits = (unsigned*)salloc(2048 * 4);
    unsigned char* dense = (unsigned char*)salloc(65536);
    if (!bits || !dense) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(bits, 0, 2048 * 4, g_stream));
    unsigned gr = grid_for(nf, 256);
    if (gr > (unsigned)g_sms * 4) gr = g_sms * 4;
    HG_LAUNCH("sg_codes", gr, 256, 0, k_sg_codes, (const int8_t*)q0.flag, (const int8_t*)q0.status, nf, bits);
    std::vector<unsigned> hb(2048);
    HG_CU(cudaMemcpyAsync(hb.data(), bits, 2048 * 4, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());
    std::vector<unsigned char> hd(65536, 0xff);
    std::vector<unsigned> code_of;
    for (unsigned c = 0; c < 65536; c++)
        if ((hb[c >> 5] >> (c & 31)) & 1u) {
            if (code_of.size() >= (size_t)SG_MAXG) return 0;  // too many codes: the general path
            hd[c] = (unsigned char)code_of.size();
            code_of.push_back(c);
        }
    const int G = (int)code_of.size();
    if (G == 0) return 0;
    HG_CU(cudaMemcpyAsync(dense, hd.data(), 65536, cudaMemcpyHostToDevice, g_stream));
    const long long ntiles = (nf + SG_TILE - 1) / SG_TILE;
    for (size_t c0 = 0; c0 < ps.size(); c0 += SG_MAXP) {
        ScratchScope inner;
        const int npl = (int)std::min<size_t>(SG_MAXP, ps.size() - c0);
        const int nj = npl * G;
        std::vector<int> hw(2 * npl);
        for (int k = 0; k < npl; k++) { hw[2 * k] = plo[c0 + k]; hw[2 * k + 1] = phi[c0 + k]; }
        int* wins = (int*)salloc(8 * npl);
        unsigned* counts = (unsigned*)salloc((size_t)nj * ntiles * 4);
        unsigned long long* offs = (unsigned long long*)salloc((size_t)nj * ntiles * 8);
        unsigned long long* totals = (unsigned long long*)salloc((size_t)nj * 8);
        unsigned long long* base = (unsigned long long*)salloc((size_t)nj * 8);
        if (!wins || !counts || !offs || !totals || !base) return E_DEVICE_OOM;
        HG_CU(cudaMemcpyAsync(wins, hw.data(), 8 * npl, cudaMemcpyHostToDevice, g_stream));
        HG_LAUNCH("sg_count", (unsigned)ntiles, 256, 0, k_sg_count, dd, (const int8_t*)q0.flag,
                  (const int8_t*)q0.status, (const unsigned char*)dense, nf, (const int*)wins, npl, G, counts, ntiles);
        HG_LAUNCH("sg_scan", (unsigned)nj, 1024, 0, k_sg_scan, (const unsigned*)counts, ntiles, offs, totals);
        std::vector<unsigned long long> ht(nj), hbase(nj);
        HG_CU(cudaMemcpyAsync(ht.data(), totals, (size_t)nj * 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CHECK(check_device_errors());
        // each plan's groups in ascending code order, plans one after another
        unsigned long long tot = 0;
        std::vector<long long> seg_start;
        std::vector<int> seg_j;
        for (int j = 0; j < nj; j++) {
            hbase[j] = tot;
            if (ht[j]) { seg_start.push_back((long long)tot); seg_j.push_back(j); }
            tot += ht[j];
        }
        const long long nseg = (long long)seg_start.size();
        double* vq = (double*)salloc((size_t)(tot ? tot : 1) * 8);
        double* vp = (double*)salloc((size_t)(tot ? tot : 1) * 8);
        double* vd = (double*)salloc((size_t)(tot ? tot : 1) * 8);
        long long* st = (long long*)salloc((size_t)(nseg ? nseg : 1) * 8);
        double* res = (double*)salloc((size_t)(nseg ? nseg : 1) * 3 * 8);
        if (!vq || !vp || !vd || !st || !res) return E_DEVICE_OOM;
        HG_CU(cudaMemcpyAsync(base, hbase.data(), (size_t)nj * 8, cudaMemcpyHostToDevice, g_stream));
        if (tot > 0) {
            HG_LAUNCH("sg_scatter", (unsigned)ntiles, 256, 0, k_sg_scatter, dd, (const int8_t*)q0.flag,
                      (const int8_t*)q0.status, (const unsigned char*)dense, q0.qty, q0.price, q0.disc, nf,
                      (const int*)wins, npl, G, (const unsigned long long*)offs, (const unsigned long long*)base,
                      ntiles, vq, vp, vd);
            HG_CU(cudaMemcpyAsync(st, seg_start.data(), (size_t)nseg * 8, cudaMemcpyHostToDevice, g_stream));
            HG_CHECK(seg_sum_f64_direct(vq, st, nseg, (long long)tot, res));
            HG_CHECK(seg_sum_f64_direct(vp, st, nseg, (long long)tot, res + nseg));
            HG_CHECK(seg_sum_f64_direct(vd, st, nseg, (long long)tot, res + 2 * nseg));
            HG_LAUNCH("b_avg", (unsigned)((nseg + 255) / 256), 256, 0, k_b_avg, (const double*)(res + nseg),
                      (const long long*)st, nseg, (long long)tot, res + nseg);
        }
        std::vector<double> hr((size_t)(nseg ? nseg : 1) * 3);
        if (nseg > 0) HG_CU(cudaMemcpyAsync(hr.data(), res, (size_t)nseg * 3 * 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CHECK(check_device_errors());
        for (int k = 0; k < npl; k++) {
            hgpuJoinGroupResult& r = out[ps[c0 + k]];
            r.status = 0;
            r.ngroups = 0;
        }
        for (long long e = 0; e < nseg; e++) {
            const int j = seg_j[e], k = j / G, c = j % G;
            hgpuJoinGroupResult& r = out[ps[c0 + k]];
            const long long g = r.ngroups++;
            r.flag[g] = (C)(code_of[c] >> 8);
            r.st[g] = (C)(code_of[c] & 255);
            r.count[g] = (L)ht[j];
            r.sum_qty[g] = hr[e];
            r.avg_price[g] = hr[nseg + e];
            r.sum_disc[g] = hr[2 * nseg + e];
        }
        for (int k = 0; k < npl; k++) (*done)[ps[c0 + k]] = 1;
    }
    *ran = 1;
    return 0;
}

// Finds the plans that share all their tables with another plan of the
// batch, runs one probe per distinct table set, and describes each such
// plan's window selection (cplans).  Marks plans for the builtin path where
// the shared result could differ from the plan's own builtins: a repeated
// dimension key, or a compressed key column longer than the fact table.
// Table sets whose key range is too wide for a direct date table, or whose
// dates span more than 65,534 days, are left to the per-plan path.
static I shared_probe(const hgpuJoinGroupPlan* plans, int np, std::vector<char>* shared, std::vector<char>* plain,
                      std::vector<unsigned long long>* sel, std::vector<unsigned long long>* mexp,
                      std::vector<CPlan>* cplans, hgpuJoinGroupResult* out, std::vector<char>* done) {
    std::map<std::vector<const void*>, std::vector<int>> sets;
    for (int p = 0; p < np; p++) {
        const hgpuJoinGroupPlan& q = plans[p];
        std::vector<const void*> k = {q.dim_pk, q.dim_date, q.fk, q.flag, q.status, q.qty, q.price, q.disc,
                                      (const void*)(intptr_t)q.ndim, (const void*)(intptr_t)q.nfact};
        sets[k].push_back(p);
    }
    std::vector<std::vector<int>> groups;
    for (auto& kv : sets)
        if (kv.second.size() >= 2 && plans[kv.second[0]].ndim > 0 && plans[kv.second[0]].nfact > 0)
            groups.push_back(kv.second);
    if (groups.empty()) return 0;
    const int ng = (int)groups.size();
    long long* mm = (long long*)salloc((size_t)ng * 32);
    if (!mm) return E_DEVICE_OOM;
    std::vector<long long> init(4 * ng);
    for (int g = 0; g < ng; g++) { init[4 * g] = init[4 * g + 2] = LLONG_MAX; init[4 * g + 1] = init[4 * g + 3] = LLONG_MIN; }
    HG_CU(cudaMemcpyAsync(mm, init.data(), (size_t)ng * 32, cudaMemcpyHostToDevice, g_stream));
    for (int g = 0; g < ng; g++) {
        const hgpuJoinGroupPlan& q = plans[groups[g][0]];
        unsigned gr = grid_for(q.ndim, 256);
        if (gr > (unsigned)g_sms * 8) gr = g_sms * 8;
        HG_LAUNCH("sh_minmax", gr, 256, 0, k_sh_minmax, q.dim_pk, q.dim_date, q.ndim, mm + 4 * g);
    }
    std::vector<long long> hmm(4 * ng);
    HG_CU(cudaMemcpyAsync(hmm.data(), mm, (size_t)ng * 32, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(stream_sync());
    struct Built { int g; long long kmin; unsigned long long kspan; int dmin, drange; unsigned* dimhist; unsigned* facthist;
                   unsigned* dup; unsigned short* dd; };
    std::vector<Built> built;
    for (int g = 0; g < ng; g++) {
        const hgpuJoinGroupPlan& q = plans[groups[g][0]];
        long long kmin = hmm[4 * g], kmax = hmm[4 * g + 1], dmin = hmm[4 * g + 2], dmax = hmm[4 * g + 3];
        unsigned long long kspan = (unsigned long long)(kmax - kmin) + 1, drange = (unsigned long long)(dmax - dmin) + 1;
        if (kspan > 64ull * (unsigned long long)(q.ndim > 1024 ? q.ndim : 1024) || kspan >= (1ull << 31) ||
            drange > 65535ull)
            continue;
        unsigned short* dt = (unsigned short*)salloc(kspan * 2);
        unsigned* hists = (unsigned*)salloc(drange * 8 + 16);
        unsigned short* dd = (unsigned short*)salloc((size_t)q.nfact * 2);
        if (!dt || !hists || !dd) return E_DEVICE_OOM;
        HG_CU(cudaMemsetAsync(dt, 0xff, kspan * 2, g_stream));
        HG_CU(cudaMemsetAsync(hists, 0, drange * 8 + 16, g_stream));
        Built b{g, kmin, kspan, (int)dmin, (int)drange, hists, hists + drange, hists + 2 * drange, dd};
        const size_t smem = drange <= 8192 ? drange * 4 : 0;
        unsigned gr = grid_for(q.ndim, 256);
        if (gr > (unsigned)g_sms * 8) gr = g_sms * 8;
        HG_LAUNCH("sh_build", gr, 256, smem, k_sh_build, q.dim_pk, q.dim_date, q.ndim, kmin, b.dmin, b.drange, dt,
                  b.dimhist, b.dup);
        gr = grid_for((q.nfact + 3) / 4, 256);
        if (gr > (unsigned)g_sms * 8) gr = g_sms * 8;
        HG_LAUNCH("sh_probe", gr, 256, smem, k_sh_probe, q.fk, q.nfact, kmin, kspan, (const unsigned short*)dt,
                  b.drange, dd, b.facthist);
        built.push_back(b);
    }
    if (built.empty()) return 0;
    for (Built& b : built) {
        std::vector<unsigned> h((size_t)b.drange * 2 + 1);
        HG_CU(cudaMemcpyAsync(h.data(), b.dimhist, ((size_t)b.drange * 2 + 1) * 4, cudaMemcpyDeviceToHost, g_stream));
        HG_CHECK(check_device_errors());
        std::vector<unsigned long long> cd(b.drange + 1, 0), cf(b.drange + 1, 0);
        for (int i = 0; i < b.drange; i++) {
            cd[i + 1] = cd[i] + h[i];
            cf[i + 1] = cf[i] + h[b.drange + i];
        }
        const bool dup = h[2 * (size_t)b.drange] != 0;
        std::vector<int> ps, plo, phi;
        for (int p : groups[b.g]) {
            const hgpuJoinGroupPlan& q = plans[p];
            if (dup) { (*plain)[p] = 1; continue; }
            long long lo = (long long)q.lo - b.dmin, hi = (long long)q.hi - b.dmin;
            lo = lo < 0 ? 0 : (lo > b.drange ? b.drange : lo);
            hi = hi < 0 ? 0 : (hi > b.drange ? b.drange : hi);
            if (hi < lo) hi = lo;
            (*sel)[p] = cd[hi] - cd[lo];
            if ((*sel)[p] > (unsigned long long)q.nfact) { (*plain)[p] = 1; continue; }
            (*mexp)[p] = cf[hi] - cf[lo];
            ps.push_back(p);
            plo.push_back((int)lo);
            phi.push_back((int)hi);
        }
        if (ps.empty()) continue;
        int ran = 0;
        HG_CHECK(shared_grouped(plans, ps, plo, phi, b.dd, out, done, &ran));
        if (ran) continue;
        for (size_t k = 0; k < ps.size(); k++) {
            (*shared)[ps[k]] = 1;
            cplans->push_back(CPlan{b.dd, plans[ps[k]].nfact, plo[k], phi[k], 0, ps[k]});
        }
    }
    return 0;
}

}  // namespace hg

using namespace hg;

extern "C" I hgpuBatchJoinGroup(const hgpuJoinGroupPlan* plans, L nplans, hgpuJoinGroupResult* out) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    const int np = (int)nplans;
    if (np <= 0) return 0;
    std::vector<DPlan> hp(np);
    const int R = g_tile_rows;
    const long long ptile = 256LL * R;  // fact rows per probe tile
    std::vector<long long> dtiles(np + 1), ftiles(np + 1);
    dtiles[0] = ftiles[0] = 0;
    long long fact_total = 0;
    for (int p = 0; p < np; p++) {
        const hgpuJoinGroupPlan& q = plans[p];
        const void* ptrs[] = {q.dim_pk, q.dim_date, q.fk, q.flag, q.status, q.qty, q.price, q.disc};
        for (const void* v : ptrs)
            if (!is_device_ptr(v)) return set_error(E_DOMAIN, "batched plan %d: columns must be device or pinned memory", p);
        DPlan& d = hp[p];
        memset(&d, 0, sizeof d);
        d.pk = q.dim_pk; d.date = q.dim_date; d.nd = q.ndim;
        d.fk = q.fk; d.flag = (const int8_t*)q.flag; d.status = (const int8_t*)q.status;
        d.qty = q.qty; d.price = q.price; d.disc = q.disc; d.nf = q.nfact;
        d.lo = q.lo; d.hi = q.hi;
        out[p].status = 0;
        out[p].ngroups = 0;
    }
    std::vector<char> plain(np, 0);
    // plans over the same tables: one shared probe, then a window selection each
    std::vector<CPlan> cplans;
    std::vector<long long> ctiles(1, 0);
    std::vector<char> shared(np, 0);
    std::vector<unsigned long long> sh_sel(np, 0), sh_m(np, 0);
    std::vector<char> done(np, 0);  // results already written by the grouped shared path
    HG_CHECK(shared_probe(plans, np, &shared, &plain, &sh_sel, &sh_m, &cplans, out, &done));
    for (int p = 0; p < np; p++) {
        const hgpuJoinGroupPlan& q = plans[p];
        DPlan& d = hp[p];
        if (shared[p] || plain[p] || done[p]) { d.nd = 0; d.nf = 0; }  // no per-plan build or probe
        d.fact_off = fact_total;
        fact_total += shared[p] ? (long long)sh_m[p] : ((plain[p] || done[p]) ? 0 : q.nfact);
        dtiles[p + 1] = dtiles[p] + (d.nd + BT - 1) / BT;
        ftiles[p + 1] = ftiles[p] + (d.nf + ptile - 1) / ptile;
    }
    for (CPlan& c : cplans) {
        c.fact_off = hp[c.p].fact_off;
        ctiles.push_back(ctiles.back() + (c.nf + ptile - 1) / ptile);
    }
    // device copies of the plan table and tile maps
    DPlan* dP = (DPlan*)salloc(np * sizeof(DPlan));
    long long* dT = (long long*)salloc((np + 1) * 8);
    long long* fT = (long long*)salloc((np + 1) * 8);
    long long* mm = (long long*)salloc(np * 16);
    unsigned* dup = (unsigned*)salloc(np * 4 + 16);
    if (!dP || !dT || !fT || !mm || !dup) return E_DEVICE_OOM;
    std::vector<long long> mminit(2 * np);
    for (int p = 0; p < np; p++) { mminit[2 * p] = LLONG_MAX; mminit[2 * p + 1] = LLONG_MIN; }
    HG_CU(cudaMemcpyAsync(dT, dtiles.data(), (np + 1) * 8, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(fT, ftiles.data(), (np + 1) * 8, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(mm, mminit.data(), np * 16, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(dP, hp.data(), np * sizeof(DPlan), cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemsetAsync(dup, 0, np * 4, g_stream));
    if (dtiles[np] > 0) HG_LAUNCH("b_minmax", (unsigned)dtiles[np], 256, 0, k_b_minmax, dP, dT, np, mm);
    std::vector<long long> hmm(2 * np);
    HG_CU(cudaMemcpyAsync(hmm.data(), mm, np * 16, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(stream_sync());
    // presence bitmaps and code tables
    long long bm_words = 0;
    for (int p = 0; p < np; p++) {
        long long lo = hmm[2 * p], hi = hmm[2 * p + 1];
        if (hp[p].nd == 0) { lo = 0; hi = -1; }
        unsigned long long range = hi >= lo ? (unsigned long long)(hi - lo) + 1 : 0;
        if (!shared[p] && !plain[p] && !done[p] &&
            (range > 64ull * (unsigned long long)(hp[p].nd > 1024 ? hp[p].nd : 1024) || range >= (1ull << 31))) {
            plain[p] = 1;  // too wide for a presence bitmap: no row is built or matched here
            lo = 0; hi = -1; range = 0;
            hp[p].nd = 0;
        }
        hp[p].kmin = lo;
        hp[p].kmax = hi;
        bm_words += (long long)((range + 31) / 32) + 1;
    }
    unsigned* bm = (unsigned*)salloc((size_t)bm_words * 4);
    unsigned* cb = (unsigned*)salloc((size_t)np * 2048 * 4);
    unsigned short* dn = (unsigned short*)salloc((size_t)np * 65536 * 2);
    if (!bm || !cb || !dn) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(bm, 0, (size_t)bm_words * 4, g_stream));
    HG_CU(cudaMemsetAsync(cb, 0, (size_t)np * 2048 * 4, g_stream));
    {
        long long w = 0;
        for (int p = 0; p < np; p++) {
            hp[p].bitmap = bm + w;
            unsigned long long range = hp[p].kmax >= hp[p].kmin ? (unsigned long long)(hp[p].kmax - hp[p].kmin) + 1 : 0;
            w += (long long)((range + 31) / 32) + 1;
            hp[p].codebits = cb + (size_t)p * 2048;
            hp[p].dense = dn + (size_t)p * 65536;
        }
    }
    HG_CU(cudaMemcpyAsync(dP, hp.data(), np * sizeof(DPlan), cudaMemcpyHostToDevice, g_stream));
    unsigned long long* nsel = (unsigned long long*)salloc(np * 8 + 16);
    if (!nsel) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(nsel, 0, np * 8, g_stream));
    if (dtiles[np] > 0) HG_LAUNCH("b_build", (unsigned)dtiles[np], 256, 0, k_b_build, dP, dT, np, dup, nsel);
    // probe: match bits and tile counts (per-plan probes, then the shared
    // selections, as one tile map), a scan of the counts, and the emit pass
    unsigned* fi = (unsigned*)salloc((size_t)(fact_total > 0 ? fact_total : 1) * 4);
    unsigned long long* mcount = (unsigned long long*)salloc(np * 8 + 16);
    long long* moff = (long long*)salloc((np + 1) * 8);
    const long long nt_probe = ftiles[np], nt_all = nt_probe + ctiles.back();
    unsigned* mbits = (unsigned*)salloc((size_t)(nt_all > 0 ? nt_all : 1) * 8 * R * 4);
    unsigned* tcount = (unsigned*)salloc((size_t)(nt_all > 0 ? nt_all : 1) * 4);
    unsigned long long* toffs = (unsigned long long*)salloc((size_t)(nt_all + 1) * 8);
    if (!fi || !mcount || !moff || !mbits || !tcount || !toffs) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(mcount, 0, np * 8, g_stream));
    // the combined tile map: every plan with probe tiles, then every shared selection
    std::vector<EmitPlan> emit;
    std::vector<long long> etiles(1, 0);
    for (int p = 0; p < np; p++) {
        emit.push_back(EmitPlan{hp[p].fact_off, p});
        etiles.push_back(ftiles[p + 1]);
    }
    for (const CPlan& c : cplans) {
        emit.push_back(EmitPlan{c.fact_off, c.p});
        etiles.push_back(etiles.back() + ((c.nf + ptile - 1) / ptile));
    }
    if (nt_probe > 0) {
        const unsigned nt = (unsigned)nt_probe;
        const size_t sm = (size_t)2 * R * 256 * 4;
        // per context: set on every call (a host-side write)
        HG_CU(cudaFuncSetAttribute(k_b_probe<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 32 * 256 * 4));
        if (R == 8) HG_LAUNCH("b_probe", nt, 256, sm, k_b_probe<8>, dP, fT, np, mbits, tcount);
        else if (R == 32) HG_LAUNCH("b_probe", nt, 256, sm, k_b_probe<32>, dP, fT, np, mbits, tcount);
        else HG_LAUNCH("b_probe", nt, 256, sm, k_b_probe<16>, dP, fT, np, mbits, tcount);
    }
    if (ctiles.back() > 0) {
        const int nc = (int)cplans.size();
        CPlan* dC = (CPlan*)salloc(nc * sizeof(CPlan));
        long long* cT = (long long*)salloc((nc + 1) * 8);
        if (!dC || !cT) return E_DEVICE_OOM;
        HG_CU(cudaMemcpyAsync(dC, cplans.data(), nc * sizeof(CPlan), cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaMemcpyAsync(cT, ctiles.data(), (nc + 1) * 8, cudaMemcpyHostToDevice, g_stream));
        const unsigned nt = (unsigned)ctiles.back();
        unsigned* cb2 = mbits + (size_t)nt_probe * 8 * R;
        unsigned* cc2 = tcount + nt_probe;
        if (R == 8) HG_LAUNCH("sh_select", nt, 256, 0, k_sh_select<8>, dC, cT, nc, cb2, cc2);
        else if (R == 32) HG_LAUNCH("sh_select", nt, 256, 0, k_sh_select<32>, dC, cT, nc, cb2, cc2);
        else HG_LAUNCH("sh_select", nt, 256, 0, k_sh_select<16>, dC, cT, nc, cb2, cc2);
    }
    if (nt_all > 0) {
        const int ne = (int)emit.size();
        EmitPlan* dE = (EmitPlan*)salloc(ne * sizeof(EmitPlan));
        long long* eT = (long long*)salloc((ne + 1) * 8);
        if (!dE || !eT) return E_DEVICE_OOM;
        HG_CU(cudaMemcpyAsync(dE, emit.data(), ne * sizeof(EmitPlan), cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaMemcpyAsync(eT, etiles.data(), (ne + 1) * 8, cudaMemcpyHostToDevice, g_stream));
        HG_CHECK(scan_counts(tcount, nt_all, toffs));
        const unsigned nt = (unsigned)nt_all;
        if (R == 8) HG_LAUNCH("b_emit", nt, 256, 0, k_b_emit<8>, dE, eT, ne, mbits, toffs, fi, mcount);
        else if (R == 32) HG_LAUNCH("b_emit", nt, 256, 0, k_b_emit<32>, dE, eT, ne, mbits, toffs, fi, mcount);
        else HG_LAUNCH("b_emit", nt, 256, 0, k_b_emit<16>, dE, eT, ne, mbits, toffs, fi, mcount);
    }
    HG_LAUNCH("b_offsets", 1, 32, 0, k_b_offsets, mcount, np, moff);
    // gather (over the fact tile map: a plan has at most as many matches as rows)
    std::vector<unsigned long long> hm(np);
    HG_CU(cudaMemcpyAsync(hm.data(), mcount, np * 8, cudaMemcpyDeviceToHost, g_stream));
    std::vector<unsigned> hdup(np);
    std::vector<unsigned long long> hsel(np);
    HG_CU(cudaMemcpyAsync(hdup.data(), dup, np * 4, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(cudaMemcpyAsync(hsel.data(), nsel, np * 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());
    // A repeated dimension key emits several rows per fact row, and a
    // compressed key column longer than the fact table makes @join_index
    // build on the fact side and emit rows in key-row order: both plans run
    // through the builtins instead.
    for (int p = 0; p < np; p++) {
        if (shared[p] || done[p]) continue;  // checked by shared_probe
        if (hdup[p] || hsel[p] > (unsigned long long)hp[p].nf) plain[p] = 1;
    }
    long long mtot = 0;
    std::vector<long long> mtiles(np + 1), hmoff(np + 1);
    mtiles[0] = 0;
    for (int p = 0; p < np; p++) {
        hmoff[p] = mtot;
        mtot += (long long)hm[p];
        mtiles[p + 1] = mtiles[p] + ((long long)hm[p] + BT - 1) / BT;
    }
    hmoff[np] = mtot;
    long long* mT = (long long*)salloc((np + 1) * 8);
    unsigned* code = (unsigned*)salloc((size_t)(mtot > 0 ? mtot : 1) * 4);
    double* vq = (double*)salloc((size_t)(mtot > 0 ? mtot : 1) * 8);
    double* vp = (double*)salloc((size_t)(mtot > 0 ? mtot : 1) * 8);
    double* vd = (double*)salloc((size_t)(mtot > 0 ? mtot : 1) * 8);
    long long* rows = (long long*)salloc((size_t)(mtot > 0 ? mtot : 1) * 8);
    unsigned* ngroups = (unsigned*)salloc(np * 4 + 16);
    unsigned* codes = (unsigned*)salloc((size_t)np * 256 * 4);
    unsigned* hist = (unsigned*)salloc((size_t)np * 256 * 4);
    unsigned* bucket = (unsigned*)salloc((size_t)np * 256 * 4);
    char* st2 = (char*)salloc((size_t)mtiles[np] * 256 * 8 + 64);
    if (!mT || !code || !vq || !vp || !vd || !rows || !ngroups || !codes || !hist || !bucket || !st2) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(mT, mtiles.data(), (np + 1) * 8, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemsetAsync(hist, 0, (size_t)np * 256 * 4, g_stream));
    HG_CU(cudaMemsetAsync(st2, 0, (size_t)mtiles[np] * 256 * 8 + 64, g_stream));
    if (mtiles[np] > 0) {
        HG_LAUNCH("b_gather", (unsigned)mtiles[np], 256, 0, k_b_gather, dP, mT, np, fi, mcount, moff, code, vq, vp, vd);
        HG_LAUNCH("b_dense", np, 256, 0, k_b_dense, dP, ngroups, codes);
        HG_LAUNCH("b_hist", (unsigned)mtiles[np], 256, 0, k_b_hist, dP, mT, np, mcount, moff, code, hist);
        HG_LAUNCH("b_bucket", np, 256, 0, k_b_bucket, hist, bucket);
        HG_LAUNCH("b_sort", (unsigned)mtiles[np], 256, 0, k_b_sort, dP, mT, np, mcount, moff, code, bucket, rows,
                  (unsigned long long*)st2, (unsigned*)(st2 + (size_t)mtiles[np] * 256 * 8), g_derr);
    }
    std::vector<unsigned> hg(np);
    HG_CU(cudaMemcpyAsync(hg.data(), ngroups, np * 4, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());
    std::vector<long long> segoff(np + 1);
    segoff[0] = 0;
    for (int p = 0; p < np; p++) {
        if (hm[p] == 0) hg[p] = 0;
        if (hg[p] > 256) {  // the result holds 256 groups
            plain[p] = 1;
            hg[p] = 0;
        }
        segoff[p + 1] = segoff[p] + hg[p];
    }
    const long long nseg = segoff[np];
    long long* dseg = (long long*)salloc((np + 1) * 8);
    long long* starts = (long long*)salloc((size_t)(nseg > 0 ? nseg : 1) * 8);
    double* sq = (double*)salloc((size_t)(nseg > 0 ? nseg : 1) * 8);
    double* sp = (double*)salloc((size_t)(nseg > 0 ? nseg : 1) * 8);
    double* sd = (double*)salloc((size_t)(nseg > 0 ? nseg : 1) * 8);
    if (!dseg || !starts || !sq || !sp || !sd) return E_DEVICE_OOM;
    unsigned* ng_dev = ngroups;
    if (nseg > 0) {
        HG_CU(cudaMemcpyAsync(dseg, segoff.data(), (np + 1) * 8, cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaMemcpyAsync(ng_dev, hg.data(), np * 4, cudaMemcpyHostToDevice, g_stream));
        HG_LAUNCH("b_starts", np, 256, 0, k_b_starts, moff, bucket, ng_dev, dseg, np, starts);
        HG_CHECK(seg_sum_f64(vq, rows, mtot, starts, nseg, mtot, sq));
        HG_CHECK(seg_sum_f64(vp, rows, mtot, starts, nseg, mtot, sp));
        HG_CHECK(seg_sum_f64(vd, rows, mtot, starts, nseg, mtot, sd));
        HG_LAUNCH("b_avg", cap_grid(nseg), 256, 0, k_b_avg, sp, starts, nseg, mtot, sp);
    }
    std::vector<long long> hst(nseg > 0 ? nseg : 1);
    std::vector<double> hq(nseg > 0 ? nseg : 1), hpv(nseg > 0 ? nseg : 1), hd(nseg > 0 ? nseg : 1);
    std::vector<unsigned> hcodes((size_t)np * 256);
    if (nseg > 0) {
        HG_CU(cudaMemcpyAsync(hst.data(), starts, nseg * 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaMemcpyAsync(hq.data(), sq, nseg * 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaMemcpyAsync(hpv.data(), sp, nseg * 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaMemcpyAsync(hd.data(), sd, nseg * 8, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaMemcpyAsync(hcodes.data(), codes, (size_t)np * 256 * 4, cudaMemcpyDeviceToHost, g_stream));
    }
    HG_CHECK(check_device_errors());
    for (int p = 0; p < np; p++) {
        hgpuJoinGroupResult& r = out[p];
        if (plain[p] || done[p]) continue;
        r.ngroups = hg[p];
        for (unsigned g = 0; g < hg[p]; g++) {
            long long k = segoff[p] + g;
            long long e = (g + 1 < hg[p]) ? hst[k + 1] : hmoff[p + 1];
            long long cnt = e - hst[k];
            unsigned c = hcodes[(size_t)p * 256 + g];
            r.flag[g] = (C)(c >> 8);
            r.st[g] = (C)(c & 255);
            r.count[g] = cnt;
            r.sum_qty[g] = hq[k];
            r.sum_disc[g] = hd[k];
            r.avg_price[g] = hpv[k];
        }
    }
    for (int p = 0; p < np; p++)
        if (plain[p]) out[p].status = plan_through_builtins(plans[p], &out[p]);
    return 0;
}
