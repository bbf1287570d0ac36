// Generic single-pass exclusive scan (decoupled look-back) over u32 counts,
// producing u64 offsets and the total.  Used by the duplicate-key join,
// group boundaries and the batched plans.
#include "dev_common.cuh"

namespace hg {

constexpr int SC_THREADS = 256, SC_ITEMS = 16, SC_TILE = SC_THREADS * SC_ITEMS;

__global__ void __launch_bounds__(SC_THREADS) k_scan_u32(const unsigned* __restrict__ in, long long n,
                                                         unsigned long long* __restrict__ out,
                                                         unsigned long long* status, unsigned* ticket,
                                                         unsigned long long* total, unsigned* derr) {
    __shared__ unsigned long long warp_tot[8];
    __shared__ unsigned long long tile_off;
    __shared__ long long tile_id;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) tile_id = atomicAdd(ticket, 1u);
    __syncthreads();
    const long long t = tile_id, base = t * SC_TILE + (long long)threadIdx.x * SC_ITEMS;
    unsigned v[SC_ITEMS];
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < SC_ITEMS; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    unsigned long long incl = warp_incl_scan64(s);
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < 8 ? warp_tot[lane] : 0;
        unsigned long long agg = warp_sum(w);
        unsigned long long excl = lookback_exclusive(status, t, agg, derr);
        if (lane == 0) {
            tile_off = excl;
            if ((t + 1) * SC_TILE >= n) *total = excl + agg;
        }
    }
    __syncthreads();
    unsigned long long off = tile_off + (incl - s);
    for (unsigned w = 0; w < warp; w++) off += warp_tot[w];
#pragma unroll
    for (int k = 0; k < SC_ITEMS; k++) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
}

// out[i] = sum(in[0..i)), *total_h = sum(in) (synchronous read of the total).
I scan_exclusive(const unsigned* in, long long n, unsigned long long* out, unsigned long long* total_h) {
    long long ntiles = (n + SC_TILE - 1) / SC_TILE;
    if (ntiles == 0) { if (total_h) *total_h = 0; return 0; }
    char* s = (char*)salloc(ntiles * 8 + 64);
    if (!s) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(s, 0, ntiles * 8 + 64, g_stream));
    unsigned long long* total = (unsigned long long*)(s + ntiles * 8 + 8);
    HG_LAUNCH("scan", (unsigned)ntiles, SC_THREADS, 0, k_scan_u32, in, n, out, (unsigned long long*)s,
              (unsigned*)(s + ntiles * 8), total, g_derr);
    HG_CHECK(last_launch_error());
    if (total_h) {
        HG_CHECK(rb_queue(total_h, total, 8));
        HG_CHECK(check_device_errors());
    }
    return 0;
}

// Self-test of the bounded device waits: a look-back over four tiles in
// which tile 0 never publishes its status (a flag nothing sets).  The waits
// of the later tiles give up after `limit` polls each, record DERR_TIMEOUT
// and return, so the kernel ends and the context stays usable.  mode 0: the
// block-wide look-back of the scans and compactions; mode 1: the per-digit
// chain look-back of the radix passes.
__global__ void k_selftest_wait(unsigned long long* status, unsigned* ticket, int mode, long long limit, unsigned* derr) {
    __shared__ long long tile;
    if (threadIdx.x == 0) tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const long long t = tile;
    if (t == 0) return;  // withholds its status
    if (mode == 0) lookback_exclusive(status, t, 1, derr, limit);  // one full warp per tile
    else if (threadIdx.x == 0) chain_lookback(status, 1, t, 0, 1, derr, limit);
}

}  // namespace hg

using namespace hg;

extern "C" I hgpuSelfTestWait(I mode, L limit) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (mode < 0 || mode > 1) return set_error(E_DOMAIN, "hgpuSelfTestWait: mode %d is not 0 or 1", mode);
    if (limit < 1 || limit > (1LL << 20)) return set_error(E_DOMAIN, "hgpuSelfTestWait: limit %lld outside [1, 2^20]", limit);
    char* s = (char*)salloc(256);
    if (!s) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(s, 0, 256, g_stream));
    HG_LAUNCH("selftest_wait", 4, 32, 0, k_selftest_wait, (unsigned long long*)s, (unsigned*)(s + 128), (int)mode,
              (long long)limit, g_derr);
    HG_CHECK(last_launch_error());
    return check_device_errors();
}
