// Served form: a request loop over tables resident in HBM, with continuous
// batching and admission by HBM footprint.
//
// The loop (hgpuServerRun) keeps a FIFO of requests that have arrived.  Each
// step admits waiting requests in arrival order while the sum of their
// footprint estimates fits the budget (a request larger than the whole
// budget is refused with E_ADMISSION), runs them together, and stamps their
// completion; requests that arrive while a step runs wait for the next one.
// A step runs
//   * every filter-aggregate in one shared scan of the lineitem table
//     (k_s_q6: each 4096-row tile is read once and reduced once per request
//     window, in the fixed tile-tree order of @sum),
//   * every join + group-by through hgpuBatchJoinGroup, and
//   * the top-k orders one after another through the builtins.
// Each request's arithmetic depends only on its own parameters, never on the
// other requests of its step, so a result is bit-identical alone and in any
// mix.  The plain mode runs each request alone through the interpreter's
// builtin sequence, one request at a time: the baseline the served form is
// measured against.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "dev_common.cuh"

namespace hg {

I plan_through_builtins(const hgpuJoinGroupPlan& q, hgpuJoinGroupResult* r);

constexpr int SQ_MAXW = 256;  // request windows per shared-scan launch

// One block per 4096-row tile of the lineitem table.  Each thread evaluates
// the request-independent part of q6 (qty < 24, 0.05 <= disc <= 0.07, the
// value price*disc) for its 16 rows once, then for every request window sums
// its rows in the tile-tree order (lane t: rows t, t+256, ..., t+3840; xor
// butterfly; pairwise warp combine).  Rows outside a window add nothing,
// exactly as in the fused chain's full-range reduction.
__global__ void __launch_bounds__(256) k_s_q6(const int* __restrict__ ship, const int* __restrict__ qty,
                                              const double* __restrict__ disc, const double* __restrict__ price,
                                              long long n, const int* __restrict__ lohi, int nw,
                                              double* __restrict__ part, long long ntiles, F64Cmp d_lo, F64Cmp d_hi) {
    __shared__ int s_lo[SQ_MAXW], s_hi[SQ_MAXW];
    __shared__ double ws[SQ_MAXW][8];
    for (int w = threadIdx.x; w < nw; w += 256) {
        s_lo[w] = lohi[2 * w];
        s_hi[w] = lohi[2 * w + 1];
    }
    const long long base = (long long)blockIdx.x * TILE_SUM, last = n > 0 ? n - 1 : 0;
    int d[16], q[16];
    double v[16], dc[16];
    unsigned live = 0;  // bit k: row k exists and passes the request-independent predicate
#pragma unroll
    for (int k = 0; k < 16; k++) {  // unconditional loads (past the end: the last row), all issued up front
        const long long i = base + k * 256 + threadIdx.x, j = i < n ? i : last;
        dc[k] = disc[j];
        q[k] = qty[j];
        d[k] = ship[j];
        v[k] = price[j];
    }
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const long long i = base + k * 256 + threadIdx.x;
        const bool c = i < n && q[k] < 24 && f64_cmp_fixed(dc[k], d_lo) >= 0 && f64_cmp_fixed(dc[k], d_hi) <= 0;
        v[k] = c ? __dmul_rn(v[k], dc[k]) : 0.0;
        live |= (unsigned)c << k;
    }
    __syncthreads();
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    for (int w = 0; w < nw; w++) {
        const int lo = s_lo[w], hi = s_hi[w];
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (((live >> k) & 1u) && d[k] >= lo && d[k] < hi) acc = __dadd_rn(acc, v[k]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
        if (lane == 0) ws[w][warp] = acc;
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nw; w += 256) part[(long long)w * ntiles + blockIdx.x] = combine8(ws[w]);
}

// One level of the tile tree over every request's row of partials:
// in[w][0..m) -> out[w][0..m2), block (tile, w).
__global__ void __launch_bounds__(256) k_s_rows(const double* __restrict__ in, long long m, double* __restrict__ out,
                                                long long m2) {
    __shared__ double ws[8];
    const long long w = blockIdx.y, base = (long long)blockIdx.x * TILE_SUM;
    const double* x = in + w * m;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        long long i = base + k * 256 + threadIdx.x;
        if (i < m) acc = __dadd_rn(acc, x[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) out[w * m2 + blockIdx.x] = combine8(ws);
}

// Histogram of an integer column over [kmin, kmin + range): bins below 4096
// are counted in shared memory first (the hot bins of skewed keys).
__global__ void k_s_hist(const void* __restrict__ col, int is64, long long n, long long kmin, long long range,
                         unsigned* __restrict__ hist) {
    __shared__ unsigned sh[4096];
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v = (is64 ? ((const long long*)col)[i] : (long long)((const int*)col)[i]) - kmin;
        if (v < 0 || v >= range) continue;
        if (v < 4096) atomicAdd(&sh[v], 1u);
        else atomicAdd(&hist[v], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4096 && i < range; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

__global__ void k_s_minmax(const void* __restrict__ col, int is64, long long n, long long* mm) {
    long long a = LLONG_MAX, b = LLONG_MIN;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long v = is64 ? ((const long long*)col)[i] : (long long)((const int*)col)[i];
        a = v < a ? v : a;
        b = v > b ? v : b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long q = __shfl_xor_sync(0xffffffffu, a, o); a = q < a ? q : a;
        long long r = __shfl_xor_sync(0xffffffffu, b, o); b = r > b ? r : b;
    }
    __shared__ long long wa[32], wb[32];
    if (lane_id() == 0) { wa[threadIdx.x >> 5] = a; wb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { a = wa[w] < a ? wa[w] : a; b = wb[w] > b ? wb[w] : b; }
        atomicMin(&mm[0], a);
        atomicMax(&mm[1], b);
    }
}

// The rows of every top-k request of a step in one pass over the key column:
// a row whose key lies in request r's (narrowed) range [a_r, b_r) is
// appended to r's region of `rows`, warp-aggregated, in no particular order
// (the order step sorts them on (key, sec, row)).
constexpr int TK_MAXR = 64;
__global__ void __launch_bounds__(256) k_s_topk_collect(const long long* __restrict__ key, long long n,
                                                        const long long* __restrict__ rng, int nr,
                                                        const long long* __restrict__ base,
                                                        const long long* __restrict__ cap, long long* __restrict__ rows,
                                                        unsigned long long* __restrict__ cnt, unsigned* derr) {
    __shared__ long long s_a[TK_MAXR], s_b[TK_MAXR];
    for (int r = threadIdx.x; r < nr; r += blockDim.x) { s_a[r] = rng[2 * r]; s_b[r] = rng[2 * r + 1]; }
    __syncthreads();
    const unsigned lane = lane_id();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31u); i0 < n; i0 += stride) {
        const long long i = i0 + lane;
        const bool valid = i < n;
        const long long k = valid ? __ldcs(key + i) : 0;
        for (int r = 0; r < nr; r++) {
            bool m = valid && k >= s_a[r] && k < s_b[r];
            unsigned bal = __ballot_sync(0xffffffffu, m);
            if (!bal) continue;
            const int leader = __ffs(bal) - 1;
            unsigned long long b = 0;
            if ((int)lane == leader) b = atomicAdd(&cnt[r], (unsigned long long)__popc(bal));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (m) {
                unsigned long long pos = b + __popc(bal & lanemask_lt());
                if (pos < (unsigned long long)cap[r]) rows[base[r] + pos] = i;
                else flag_error(derr, DERR_CAPACITY);
            }
        }
    }
}

// ------------------------------------------------------------------ host
struct CumCount {  // rows per value of an integer column, cumulative (empty when not built)
    long long kmin = 0;
    std::vector<long long> cum;  // cum[i] = rows with value < kmin + i
    long long count(long long lo, long long hi, long long n) const {  // rows with value in [lo, hi)
        if (cum.empty()) return n;
        long long R = (long long)cum.size() - 1;
        auto at = [&](long long v) { long long i = v - kmin; i = i < 0 ? 0 : (i > R ? R : i); return cum[(size_t)i]; };
        return hi > lo ? at(hi) - at(lo) : 0;
    }
};

static I build_cum(const void* col, int is64, long long n, long long max_range, CumCount* out) {
    out->cum.clear();
    if (n <= 0) return 0;
    long long* mm = (long long*)salloc(16);
    if (!mm) return E_DEVICE_OOM;
    long long init[2] = {LLONG_MAX, LLONG_MIN}, h[2];
    HG_CU(cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, g_stream));
    unsigned g = grid_for(n, 256);
    if (g > (unsigned)g_sms * 8) g = g_sms * 8;
    HG_LAUNCH("serve_minmax", g, 256, 0, k_s_minmax, col, is64, n, mm);
    HG_CHECK(rb_queue(h, mm, 16));
    HG_CU(stream_sync());
    const unsigned long long range = (unsigned long long)(h[1] - h[0]) + 1;
    if (range > (unsigned long long)max_range) return 0;  // too wide: admission uses the upper bound
    unsigned* hist = (unsigned*)salloc(range * 4);
    if (!hist) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(hist, 0, range * 4, g_stream));
    HG_LAUNCH("serve_hist", g, 256, 0, k_s_hist, col, is64, n, h[0], (long long)range, hist);
    std::vector<unsigned> hh(range);
    HG_CU(cudaMemcpyAsync(hh.data(), hist, range * 4, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());
    out->kmin = h[0];
    out->cum.resize(range + 1);
    out->cum[0] = 0;
    for (size_t i = 0; i < range; i++) out->cum[i + 1] = out->cum[i] + hh[i];
    return 0;
}

}  // namespace hg

using namespace hg;

struct hgpu_server_s {
    hgpuServeTables t;
    L budget, max_step;
    CumCount dim_dates;  // dimension rows per date
    CumCount keys;       // order-table rows per key
};

namespace hg {

static V0 dev_vec(const void* p, I typ, L n) {
    V0 v;
    memset(&v, 0, sizeof v);
    v.len = n;
    v.typ = typ;
    v.g = (G)p;
    return v;
}

static V0 scalar_node(I typ, long long x, double f) {
    V0 v;
    memset(&v, 0, sizeof v);
    v.len = 1;
    v.typ = typ;
    if (typ == H_E) v.f64 = f;
    else if (typ == H_L) v.i64 = x;
    else v.i32 = (I)x;
    v.g = (G)&v.b;
    return v;
}

// a host copy of a node's first k i64 values (inline or device payload)
static I read_i64(const V0& v, L k, L* dst) {
    if (k <= 0) return 0;
    if (v.len == 1 || !is_device_ptr(v.g)) {
        memcpy(dst, v.g, (size_t)k * 8);
        return 0;
    }
    HG_CU(cudaMemcpyAsync(dst, v.g, (size_t)k * 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(stream_sync());
    return 0;
}

#define STEP(call) do { if ((rc = (call)) != 0) goto done; } while (0)

// Top-k of the stable ascending @order on (key, sec) among rows with key in
// [klo, khi), through the builtins: where, two gathers, order, index.
static I topk_request(const hgpu_server_s* s, const hgpuRequest& q, hgpuResponse* r) {
    const L mark = getHeapOffset();
    I rc = 0;
    V0 key = dev_vec(s->t.o_key, H_L, s->t.norder), sec = dev_vec(s->t.o_sec, H_I, s->t.norder);
    V0 a = scalar_node(H_L, q.klo, 0), b = scalar_node(H_L, q.khi, 0);
    V0 m1, m2, m, w, k2, s2, lst, o, view, rows;
    V0* ln;
    B dirs_h[2] = {1, 1};
    V0 dirs = dev_vec(dirs_h, H_B, 2);
    L k = 0;
    STEP(pfnGeq(&m1, &key, &a));
    STEP(pfnLt(&m2, &key, &b));
    STEP(pfnAnd(&m, &m1, &m2));
    STEP(pfnWhere(&w, &m));
    STEP(pfnIndex(&k2, &key, &w));
    STEP(pfnIndex(&s2, &sec, &w));
    STEP(init_list(&lst, H_G, 2));
    ln = host_nodes(&lst);
    ln[0] = k2;
    ln[1] = s2;
    if (k2.len == 1) ln[0].g = (G)&ln[0].b;
    if (s2.len == 1) ln[1].g = (G)&ln[1].b;
    STEP(pfnOrderBy(&o, &lst, &dirs));
    k = o.len < HGPU_TOPK ? o.len : HGPU_TOPK;
    view = o;
    view.len = k;
    if (o.len <= 1) view.g = (G)&view.b;
    STEP(pfnIndex(&rows, &w, &view));
    r->nrows = k;
    if (r->rows) STEP(read_i64(rows, k, r->rows));
done:
    setHeapOffset(mark);
    return rc;
}

// The end of a top-k request whose candidate rows are known: sort them on
// (key, sec, row) -- the stable (key, sec) order of the builtin path, whose
// selection is in row order -- and keep the first HGPU_TOPK.
static I topk_finish(const hgpu_server_s* s, const long long* cand, long long m, hgpuResponse* r) {
    const L mark = getHeapOffset();
    I rc = 0;
    V0 key = dev_vec(s->t.o_key, H_L, s->t.norder), sec = dev_vec(s->t.o_sec, H_I, s->t.norder);
    V0 rowsv = dev_vec(cand, H_L, m);
    V0 k2, s2, lst, o, view, top;
    V0* ln;
    B dirs_h[3] = {1, 1, 1};
    V0 dirs = dev_vec(dirs_h, H_B, 3);
    L k = 0;
    r->nrows = 0;
    if (m == 0) goto done;
    STEP(pfnIndex(&k2, &key, &rowsv));
    STEP(pfnIndex(&s2, &sec, &rowsv));
    STEP(init_list(&lst, H_G, 3));
    ln = host_nodes(&lst);
    ln[0] = k2;
    ln[1] = s2;
    ln[2] = rowsv;
    if (k2.len == 1) ln[0].g = (G)&ln[0].b;
    if (s2.len == 1) ln[1].g = (G)&ln[1].b;
    STEP(pfnOrderBy(&o, &lst, &dirs));
    k = o.len < HGPU_TOPK ? o.len : HGPU_TOPK;
    view = o;
    view.len = k;
    if (o.len <= 1) view.g = (G)&view.b;
    STEP(pfnIndex(&top, &rowsv, &view));
    r->nrows = k;
    if (r->rows) STEP(read_i64(top, k, r->rows));
done:
    setHeapOffset(mark);
    return rc;
}

// [klo, hi) narrowed to the keys that can reach the first HGPU_TOPK rows:
// the smallest hi whose rows in [klo, hi) number at least HGPU_TOPK (every
// row with a smaller key precedes every row with a larger one)
static void topk_range(const hgpu_server_s* s, const hgpuRequest& q, long long* a, long long* b, long long* m) {
    const CumCount& c = s->keys;
    *a = q.klo;
    *b = q.khi;
    *m = c.count(q.klo, q.khi, s->t.norder);
    if (*m <= HGPU_TOPK || c.cum.empty()) return;
    long long lo = q.klo + 1, hi = q.khi;  // smallest x in [lo, hi] with count(klo, x) >= TOPK
    while (lo < hi) {
        long long mid = lo + (hi - lo) / 2;
        if (c.count(q.klo, mid, s->t.norder) >= HGPU_TOPK) hi = mid; else lo = mid + 1;
    }
    *b = lo;
    *m = c.count(q.klo, lo, s->t.norder);
}

// every top-k request of a step: one shared pass collects the candidate
// rows of all of them, then each sorts its own few
static I topk_batch(const hgpu_server_s* s, const hgpuRequest* req, const std::vector<size_t>& ids,
                    hgpuResponse* out) {
    if (ids.empty()) return 0;
    if (s->keys.cum.empty()) {  // no key histogram: the builtin path
        for (size_t r : ids) out[r].status = topk_request(s, req[r], &out[r]);
        return 0;
    }
    ScratchScope ss;
    const long long nr = (long long)ids.size();
    std::vector<long long> rng(2 * nr), base(nr + 1), cap(nr);
    base[0] = 0;
    for (long long k = 0; k < nr; k++) {
        topk_range(s, req[ids[k]], &rng[2 * k], &rng[2 * k + 1], &cap[k]);
        base[k + 1] = base[k] + cap[k];
    }
    long long* d_rng = (long long*)salloc(16 * nr);
    long long* d_base = (long long*)salloc(8 * (nr + 1));
    long long* d_cap = (long long*)salloc(8 * nr);
    unsigned long long* d_cnt = (unsigned long long*)salloc(8 * nr);
    long long* rows = (long long*)salloc(8 * (base[nr] > 0 ? base[nr] : 1));
    if (!d_rng || !d_base || !d_cap || !d_cnt || !rows) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(d_rng, rng.data(), 16 * nr, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(d_base, base.data(), 8 * (nr + 1), cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(d_cap, cap.data(), 8 * nr, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemsetAsync(d_cnt, 0, 8 * nr, g_stream));
    if (s->t.norder > 0) {
        unsigned g = grid_for(s->t.norder, 256);
        if (g > (unsigned)g_sms * 8) g = g_sms * 8;
        for (long long c0 = 0; c0 < nr; c0 += TK_MAXR) {
            int cn = (int)std::min<long long>(TK_MAXR, nr - c0);
            HG_LAUNCH("serve_topk_collect", g, 256, 0, k_s_topk_collect, s->t.o_key, s->t.norder, d_rng + 2 * c0, cn,
                      d_base + c0, d_cap + c0, rows, d_cnt + c0, g_derr);
        }
    }
    std::vector<unsigned long long> cnt(nr);
    HG_CU(cudaMemcpyAsync(cnt.data(), d_cnt, 8 * nr, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());
    for (long long k = 0; k < nr; k++) {
        if ((long long)cnt[k] != cap[k]) return set_error(E_GENERAL, "top-k candidate count %llu, expected %lld", cnt[k], cap[k]);
        out[ids[k]].status = topk_finish(s, rows + base[k], cap[k], &out[ids[k]]);
    }
    return 0;
}

// q6 through the builtins, one call per @builtin (plain mode)
static I q6_builtins(const hgpu_server_s* s, const hgpuRequest& q, double* out) {
    const L mark = getHeapOffset();
    I rc = 0;
    const hgpuServeTables& t = s->t;
    V0 ship = dev_vec(t.l_shipdate, H_I, t.nline), qty = dev_vec(t.l_qty, H_I, t.nline);
    V0 disc = dev_vec(t.l_disc, H_E, t.nline), price = dev_vec(t.l_price, H_E, t.nline);
    V0 lo = scalar_node(H_I, q.lo, 0), hi = scalar_node(H_I, q.hi, 0), c24 = scalar_node(H_I, 24, 0);
    V0 d5 = scalar_node(H_E, 0, 0.05), d7 = scalar_node(H_E, 0, 0.07);
    V0 t18, t19, t20, t21, t22, t23, t24, t25, t26, t32, t33, t43, z;
    STEP(pfnGeq(&t18, &ship, &lo));
    STEP(pfnLt(&t19, &ship, &hi));
    STEP(pfnAnd(&t20, &t18, &t19));
    STEP(pfnLt(&t21, &qty, &c24));
    STEP(pfnGeq(&t22, &disc, &d5));
    STEP(pfnLeq(&t23, &disc, &d7));
    STEP(pfnAnd(&t24, &t22, &t23));
    STEP(pfnAnd(&t25, &t20, &t21));
    STEP(pfnAnd(&t26, &t25, &t24));
    STEP(pfnCompress(&t32, &t26, &price));
    STEP(pfnCompress(&t33, &t26, &disc));
    STEP(pfnMul(&t43, &t32, &t33));
    STEP(pfnSum(&z, &t43));
    *out = z.f64;
done:
    setHeapOffset(mark);
    return rc;
}
#undef STEP

// every filter-aggregate of a step in one shared scan
static I filter_aggs(const hgpu_server_s* s, const hgpuRequest* req, const std::vector<size_t>& ids,
                     hgpuResponse* out) {
    const hgpuServeTables& t = s->t;
    const long long nw = (long long)ids.size();
    if (nw == 0) return 0;
    if (t.nline <= 0) {
        for (size_t r : ids) out[r].value = 0.0;
        return 0;
    }
    ScratchScope ss;
    const long long ntiles = (t.nline + TILE_SUM - 1) / TILE_SUM;
    std::vector<int> lohi(2 * nw);
    for (long long w = 0; w < nw; w++) {
        lohi[2 * w] = req[ids[w]].lo;
        lohi[2 * w + 1] = req[ids[w]].hi;
    }
    int* dl = (int*)salloc(8 * nw);
    double* part = (double*)salloc((size_t)nw * ntiles * 8);
    if (!dl || !part) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(dl, lohi.data(), 8 * nw, cudaMemcpyHostToDevice, g_stream));
    const F64Cmp d_lo = f64_cmp_thresholds(0.05, false), d_hi = f64_cmp_thresholds(0.07, false);
    for (long long c0 = 0; c0 < nw; c0 += SQ_MAXW) {
        int cw = (int)std::min<long long>(SQ_MAXW, nw - c0);
        HG_LAUNCH("serve_q6", (unsigned)ntiles, 256, 0, k_s_q6, t.l_shipdate, t.l_qty, t.l_disc, t.l_price, t.nline,
                  dl + 2 * c0, cw, part + c0 * ntiles, ntiles, d_lo, d_hi);
    }
    double* cur = part;
    long long m = ntiles;
    while (m > 1) {
        long long m2 = (m + TILE_SUM - 1) / TILE_SUM;
        double* nxt = (double*)salloc((size_t)nw * m2 * 8);
        if (!nxt) return E_DEVICE_OOM;
        for (long long c0 = 0; c0 < nw; c0 += 65535) {
            unsigned cw = (unsigned)std::min<long long>(65535, nw - c0);
            HG_LAUNCH("serve_q6_tree", dim3((unsigned)m2, cw), 256, 0, k_s_rows, cur + c0 * m, m, nxt + c0 * m2, m2);
        }
        cur = nxt;
        m = m2;
    }
    std::vector<double> res(nw);
    HG_CU(cudaMemcpyAsync(res.data(), cur, nw * 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CHECK(check_device_errors());
    for (long long w = 0; w < nw; w++) out[ids[w]].value = res[w];
    return 0;
}

static hgpuJoinGroupPlan plan_of(const hgpuServeTables& t, const hgpuRequest& q) {
    hgpuJoinGroupPlan p;
    p.dim_pk = t.dim_pk; p.dim_date = t.dim_date; p.ndim = t.ndim;
    p.fk = t.fk; p.flag = t.flag; p.status = t.status; p.qty = t.qty; p.price = t.price; p.disc = t.disc;
    p.nfact = t.nfact; p.lo = q.lo; p.hi = q.hi;
    return p;
}

static I join_groups(const hgpu_server_s* s, const hgpuRequest* req, const std::vector<size_t>& ids,
                     hgpuResponse* out) {
    if (ids.empty()) return 0;
    std::vector<hgpuJoinGroupPlan> plans;
    std::vector<hgpuJoinGroupResult> res(ids.size());
    for (size_t r : ids) plans.push_back(plan_of(s->t, req[r]));
    I rc = hgpuBatchJoinGroup(plans.data(), (L)plans.size(), res.data());
    for (size_t k = 0; k < ids.size(); k++) {
        hgpuResponse& o = out[ids[k]];
        o.status = rc ? rc : res[k].status;
        if (o.group) *o.group = res[k];
    }
    return 0;
}

static long long request_footprint(const hgpu_server_s* s, const hgpuRequest& q, int mode) {
    const hgpuServeTables& t = s->t;
    switch (q.kind) {
    case HGPU_REQ_FILTER_AGG: {
        long long tiles = (t.nline + TILE_SUM - 1) / TILE_SUM;
        return 16 * tiles + 4096;
    }
    case HGPU_REQ_JOIN_GROUP: {
        // the batched executor's scratch for one plan of a shared-table
        // step: the matched-row list, the gathered code/qty/price/disc and
        // group rows of the expected matches, per-plan code tables and
        // look-back words (the step's shared probe is step_footprint)
        long long dsel = s->dim_dates.count(q.lo, q.hi, t.ndim);
        double frac = t.ndim > 0 ? (double)dsel / (double)t.ndim : 0.0;
        long long m = (long long)std::ceil(frac * (double)t.nfact * 1.05) + 4096;
        return 40 * m + t.nfact / 64 + (1 << 20);
    }
    default: {
        if (mode == HGPU_SERVE_BATCHED && !s->keys.cum.empty()) {
            // the narrowed candidates: row ids, gathered key and sec, the
            // sort's keys, values and buffers
            long long a, b, m;
            topk_range(s, q, &a, &b, &m);
            return 96 * m + (1 << 20);
        }
        // three boolean vectors over the table, then for the selection:
        // row ids, gathered key and sec, the sort's keys, values and buffers
        long long sel = s->keys.count(q.klo, q.khi, t.norder);
        return 3 * t.norder + 72 * sel + (1 << 20);
    }
    }
}

// scratch a step holds once for all its requests of one kind: the shared
// probe of the join requests (date by key, date of every fact row)
static long long step_footprint(const hgpu_server_s* s, int kind) {
    const hgpuServeTables& t = s->t;
    if (kind == HGPU_REQ_JOIN_GROUP) return 2 * t.nfact + 2 * 64 * (t.ndim > 1024 ? t.ndim : 1024) / 8 + (1 << 20);
    return 0;
}

static double secs_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

static I run_step(hgpu_server_s* s, const hgpuRequest* req, const std::vector<size_t>& batch, hgpuResponse* out,
                  int mode) {
    const L mark = getHeapOffset();
    std::vector<size_t> fa, jg, tk;
    for (size_t r : batch) {
        int k = req[r].kind;
        (k == HGPU_REQ_FILTER_AGG ? fa : k == HGPU_REQ_JOIN_GROUP ? jg : tk).push_back(r);
    }
    I rc = 0;
    if (mode == HGPU_SERVE_BATCHED) {
        rc = filter_aggs(s, req, fa, out);
        for (size_t r : fa) out[r].status = rc;
        join_groups(s, req, jg, out);
    } else {
        for (size_t r : fa) out[r].status = q6_builtins(s, req[r], &out[r].value);
        for (size_t r : jg) {
            hgpuJoinGroupResult tmp;
            hgpuJoinGroupPlan p = plan_of(s->t, req[r]);
            out[r].status = plan_through_builtins(p, out[r].group ? out[r].group : &tmp);
            if (out[r].group) out[r].group->status = out[r].status;
        }
    }
    if (mode == HGPU_SERVE_BATCHED) {
        I e = topk_batch(s, req, tk, out);
        if (e)
            for (size_t r : tk) out[r].status = e;
    } else {
        for (size_t r : tk) out[r].status = topk_request(s, req[r], &out[r]);
    }
    setHeapOffset(mark);
    return rc;
}

}  // namespace hg

extern "C" {

I hgpuServerCreate(hgpuServer* out, const hgpuServeTables* tables, L hbm_budget_bytes, L max_step_requests) {
    HG_CHECK(ensure_init());
    if (!out || !tables) return E_DOMAIN;
    ScratchScope ss;
    hgpu_server_s* s = new hgpu_server_s();
    s->t = *tables;
    s->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (L)32 << 30;
    s->max_step = max_step_requests;
    // the budget is the scratch the admitted requests of a step may hold:
    // reserve it now, so that no step waits on a device allocation.  The
    // output arena (step results) and the pinned host arena (list nodes,
    // copied-out rows) get chunks up front too: pinning a fresh host chunk
    // mid-run took tens of milliseconds and set a step's latency.
    I rc = scratch_reserve((size_t)s->budget);
    if (!rc) rc = out_reserve((size_t)s->budget / 4);
    if (!rc) rc = host_reserve((size_t)1 << 30);
    if (!rc && s->t.ndim > 0 && s->t.dim_date) rc = build_cum(s->t.dim_date, 0, s->t.ndim, 1 << 20, &s->dim_dates);
    if (!rc && s->t.norder > 0 && s->t.o_key) rc = build_cum(s->t.o_key, 1, s->t.norder, 1 << 26, &s->keys);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return 0;
}

L hgpuServerFootprint(hgpuServer s, const hgpuRequest* r) {
    return (s && r) ? request_footprint(s, *r, HGPU_SERVE_BATCHED) : -1;
}

I hgpuServerRun(hgpuServer s, const hgpuRequest* req, L n, hgpuResponse* out, I mode, hgpuServeStats* stats) {
    HG_CHECK(ensure_init());
    if (!s || (n > 0 && (!req || !out))) return E_DOMAIN;
    if (mode != HGPU_SERVE_BATCHED && mode != HGPU_SERVE_PLAIN) return E_DOMAIN;
    for (L i = 1; i < n; i++)
        if (req[i].arrival_s < req[i - 1].arrival_s) return set_error(E_DOMAIN, "requests must be sorted by arrival");
    for (L i = 0; i < n; i++) {
        out[i].status = 0;
        out[i].value = 0.0;
        out[i].nrows = 0;
        out[i].step = -1;
        out[i].footprint = request_footprint(s, req[i], mode);
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::deque<size_t> pending;
    size_t next = 0;
    L done = 0, steps = 0, rejected = 0, max_req = 0, max_bytes = 0;
    I rc = 0;
    while (done < n) {
        double now = secs_since(t0);
        while (next < (size_t)n && req[next].arrival_s <= now) pending.push_back(next++);
        if (pending.empty()) {  // idle until the next arrival
            double wait = req[next].arrival_s - now;
            if (wait > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(wait - 1e-4));
            else std::this_thread::yield();
            continue;
        }
        std::vector<size_t> batch;
        L bytes = 0;
        bool kind_in[3] = {false, false, false};
        while (!pending.empty()) {
            size_t r = pending.front();
            const int kind = req[r].kind;
            L fp = out[r].footprint;
            const L once = (mode == HGPU_SERVE_BATCHED && !kind_in[kind]) ? step_footprint(s, kind) : 0;
            if (fp + step_footprint(s, kind) > s->budget) {  // can never fit: refuse it
                out[r].status = set_error(E_ADMISSION, "request %zu needs %lld bytes, budget %lld", r, (long long)fp,
                                          (long long)s->budget);
                out[r].admit_s = out[r].done_s = now;
                pending.pop_front();
                rejected++;
                done++;
                continue;
            }
            if (!batch.empty() && (bytes + fp + once > s->budget || mode == HGPU_SERVE_PLAIN ||
                                   (s->max_step > 0 && (L)batch.size() >= s->max_step)))
                break;
            bytes += fp + once;
            kind_in[kind] = true;
            batch.push_back(r);
            pending.pop_front();
        }
        if (batch.empty()) continue;
        for (size_t r : batch) out[r].admit_s = now;
        I e = run_step(s, req, batch, out, mode);
        if (e && !rc) rc = e;
        const double t = secs_since(t0);
        for (size_t r : batch) {
            out[r].done_s = t;
            out[r].step = steps;
        }
        done += (L)batch.size();
        steps++;
        max_req = std::max<L>(max_req, (L)batch.size());
        max_bytes = std::max(max_bytes, bytes);
    }
    if (stats) {
        std::vector<double> lat;
        double last = 0.0;
        for (L i = 0; i < n; i++) {
            if (out[i].status == E_ADMISSION) continue;
            lat.push_back(1e3 * (out[i].done_s - req[i].arrival_s));
            last = std::max(last, out[i].done_s);
        }
        std::sort(lat.begin(), lat.end());
        memset(stats, 0, sizeof *stats);
        stats->steps = steps;
        stats->rejected = rejected;
        stats->max_step_requests = max_req;
        stats->max_step_bytes = max_bytes;
        stats->wall_s = secs_since(t0);
        if (!lat.empty()) {
            auto pct = [&](double p) {
                size_t i = (size_t)std::ceil(p * (double)lat.size());
                return lat[i > 0 ? i - 1 : 0];
            };
            double sum = 0.0;
            for (double v : lat) sum += v;
            stats->p50_ms = pct(0.50);
            stats->p99_ms = pct(0.99);
            stats->mean_ms = sum / (double)lat.size();
            stats->max_ms = lat.back();
            stats->qps = last > 0 ? (double)lat.size() / last : 0.0;
        }
    }
    return rc;
}

I hgpuServerDestroy(hgpuServer s) {
    delete s;
    return 0;
}

}  // extern "C"
