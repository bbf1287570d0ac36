// Seeded synthetic tables generated on the device, for the batched and
// served benchmarks (hundreds of millions of rows would take minutes to
// generate on the host).  Every value is a pure function of (seed, column,
// row) through SplitMix64 (Steele, Lea & Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014), so a table is reproducible
// and any slice can be regenerated independently.
//
// Distributions follow the join + group-by configuration:
//   dim.pk   permutation of 0..ndim-1 (4-round Feistel network on the next
//            power of two, cycle-walking back into range)
//   dim.date 8035 + U{0..2525}          fact.fk   U{0..ndim-1}
//   fact.flag U{0,1,2}   fact.status U{0,1}   fact.qty U{1..50} (as f64)
//   fact.price round(qty * U(900,105000) / 100, 2)   fact.disc U{0..10}/100
#include <cmath>
#include <vector>

#include "dev_common.cuh"

namespace hg {

__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ unsigned long long rnd(unsigned long long seed, unsigned col, long long row) {
    return splitmix(splitmix(seed * 0x100000001b3ull + col) ^ (unsigned long long)row);
}

// bijection on [0, 2^(2h)) by a 4-round Feistel network
__device__ __forceinline__ unsigned long long feistel(unsigned long long x, int h, unsigned long long seed) {
    const unsigned long long m = (1ull << h) - 1;
    unsigned long long l = x >> h, r = x & m;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        unsigned long long f = splitmix(r ^ (seed + k * 0x51ed27ull)) & m;
        unsigned long long nl = r;
        r = l ^ f;
        l = nl;
    }
    return (l << h) | r;
}

__global__ void k_synth_dim(unsigned long long seed, long long nd, int h, int* __restrict__ pk, int* __restrict__ date,
                            unsigned* derr) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long x = (unsigned long long)i;
        int guard = 0;
        do {  // cycle-walking: a bijection's cycle returns to [0, nd)
            x = feistel(x, h, seed);
        } while (x >= (unsigned long long)nd && ++guard < (1 << 20));
        if (x >= (unsigned long long)nd) flag_error(derr, DERR_TIMEOUT);
        pk[i] = (int)x;
        date[i] = 8035 + (int)(rnd(seed, 1, i) % 2526ull);
    }
}

__global__ void k_synth_fact(unsigned long long seed, long long nf, long long nd, int* __restrict__ fk,
                             int8_t* __restrict__ flag, int8_t* __restrict__ status, double* __restrict__ qty,
                             double* __restrict__ price, double* __restrict__ disc) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nf; i += (long long)gridDim.x * blockDim.x) {
        fk[i] = (int)(rnd(seed, 2, i) % (unsigned long long)nd);
        flag[i] = (int8_t)(rnd(seed, 3, i) % 3ull);
        status[i] = (int8_t)(rnd(seed, 4, i) % 2ull);
        double q = (double)(1 + rnd(seed, 5, i) % 50ull);
        double u = 900.0 + (double)(rnd(seed, 6, i) >> 11) * (1.0 / 9007199254740992.0) * (105000.0 - 900.0);
        qty[i] = q;
        price[i] = __ddiv_rn(rint(__dmul_rn(q, u)), 100.0);
        disc[i] = __ddiv_rn((double)(rnd(seed, 7, i) % 11ull), 100.0);
    }
}

// Zipf keys by inverse CDF: key = 1 + (number of CDF entries <= u), u uniform
// in [0, 1); sec uniform over [0, 2^20].
__global__ void k_synth_order(unsigned long long seed, long long n, const double* __restrict__ cdf, long long nr,
                              long long* __restrict__ key, int* __restrict__ sec) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double u = (double)(rnd(seed, 8, i) >> 11) * (1.0 / 9007199254740992.0);
        long long lo = 0, hi = nr;  // first index with cdf > u
        while (lo < hi) {
            long long mid = (lo + hi) >> 1;
            if (cdf[mid] <= u) lo = mid + 1; else hi = mid;
        }
        key[i] = lo + 1;
        sec[i] = (int)(rnd(seed, 9, i) % ((1ull << 20) + 1));
    }
}

}  // namespace hg

using namespace hg;

// Fills dim (a list of 2 nodes: pk, date) and fact (a list of 6 nodes: fk,
// flag, status, qty, price, disc) with device-resident columns.
extern "C" I hgpuSynthJoinTables(unsigned long long seed, L nfact, L ndim, V dim, V fact) {
    HG_CHECK(ensure_init());
    if (ndim < 1 || nfact < 0 || ndim >= (1LL << 31)) return E_DOMAIN;
    HG_CHECK(init_list(dim, H_G, 2));
    HG_CHECK(init_list(fact, H_G, 6));
    V0* d = host_nodes(dim);
    V0* f = host_nodes(fact);
    void *pk, *date, *fk, *flag, *status, *qty, *price, *disc;
    HG_CHECK(alloc_out(&d[0], H_I, ndim, &pk));
    HG_CHECK(alloc_out(&d[1], H_I, ndim, &date));
    HG_CHECK(alloc_out(&f[0], H_I, nfact, &fk));
    HG_CHECK(alloc_out(&f[1], H_C, nfact, &flag));
    HG_CHECK(alloc_out(&f[2], H_C, nfact, &status));
    HG_CHECK(alloc_out(&f[3], H_E, nfact, &qty));
    HG_CHECK(alloc_out(&f[4], H_E, nfact, &price));
    HG_CHECK(alloc_out(&f[5], H_E, nfact, &disc));
    int bits = 1;
    while ((1LL << bits) < ndim) bits++;
    int h = (bits + 1) / 2;
    unsigned g = grid_for(ndim, 256);
    if (g > (unsigned)g_sms * 32) g = g_sms * 32;
    HG_LAUNCH("synth_dim", g, 256, 0, k_synth_dim, seed, ndim, h, (int*)pk, (int*)date, g_derr);
    if (nfact > 0) {
        g = grid_for(nfact, 256);
        if (g > (unsigned)g_sms * 32) g = g_sms * 32;
        HG_LAUNCH("synth_fact", g, 256, 0, k_synth_fact, seed, nfact, ndim, (int*)fk, (int8_t*)flag, (int8_t*)status,
                  (double*)qty, (double*)price, (double*)disc);
    }
    HG_CHECK(last_launch_error());
    HG_CHECK(check_device_errors());
    void* dp[2] = {pk, date};
    void* fp[6] = {fk, flag, status, qty, price, disc};
    for (int i = 0; i < 2; i++) HG_CHECK(finish_out(&d[i], dp[i]));
    for (int i = 0; i < 6; i++) HG_CHECK(finish_out(&f[i], fp[i]));
    return 0;
}

// Fills order (a list of 2 nodes: key i64, sec i32) with device-resident
// columns: key Zipf over 1..nranks with exponent s (cdf computed here, in
// double precision), sec uniform over [0, 2^20].
extern "C" I hgpuSynthOrderTable(unsigned long long seed, L n, L nranks, E s, V order) {
    HG_CHECK(ensure_init());
    if (n < 0 || nranks < 1 || nranks > (1LL << 30)) return E_DOMAIN;
    ScratchScope ss;
    HG_CHECK(init_list(order, H_G, 2));
    V0* o = host_nodes(order);
    void *key, *sec;
    HG_CHECK(alloc_out(&o[0], H_L, n, &key));
    HG_CHECK(alloc_out(&o[1], H_I, n, &sec));
    std::vector<double> cdf((size_t)nranks);
    double acc = 0.0;
    for (L r = 0; r < nranks; r++) cdf[(size_t)r] = (acc += pow((double)(r + 1), -s));
    for (L r = 0; r < nranks; r++) cdf[(size_t)r] /= acc;
    double* dc = (double*)salloc((size_t)nranks * 8);
    if (!dc) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(dc, cdf.data(), (size_t)nranks * 8, cudaMemcpyHostToDevice, g_stream));
    if (n > 0) {
        unsigned g = grid_for(n, 256);
        if (g > (unsigned)g_sms * 32) g = g_sms * 32;
        HG_LAUNCH("synth_order", g, 256, 0, k_synth_order, seed, n, (const double*)dc, nranks, (long long*)key,
                  (int*)sec);
    }
    HG_CHECK(last_launch_error());
    HG_CHECK(check_device_errors());
    HG_CHECK(finish_out(&o[0], key));
    HG_CHECK(finish_out(&o[1], sec));
    return 0;
}
