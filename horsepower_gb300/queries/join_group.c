/*
 * The join + group-by benchmark query compiled to C, the way HorseIR's code
 * generator turns a query into C: one builtin call per statement over the
 * library's C ABI (include/hgpu.h), with the optimizer's rewrites applied:
 * the dimension filter's elementwise statements fused into one kernel
 * (autofusion), the common-index pattern (optimizer/pattern.cc:558-672) on
 * the five gathers by the join's fact rows and on the four aggregates over
 * the groups.  Otherwise statement for statement plans.join_group in
 * horsepower_gb300/plans.py, whose results it reproduces bit for bit.  This
 * is a caller of libhgpu, built into its own libhgpu_queries.so, not part of
 * the library.
 */
#include <stdio.h>
#include <string.h>

#include "hgpu.h"

static void scalar_i64(V0 *v, L x) {
    memset(v, 0, sizeof *v);
    v->typ = H_L;
    v->len = 1;
    v->g = (G)&v->b;
    v->i64 = x;
}

static void symbol(V0 *v, const char *name) {
    memset(v, 0, sizeof *v);
    v->typ = H_Q;
    v->len = 1;
    v->g = (G)&v->b;
    v->i64 = getSymbol((S)name);
}

#define CK(call)                   \
    do {                           \
        I rc_ = (call);            \
        if (rc_) return rc_;       \
    } while (0)

/* The dimension filter's three elementwise statements (geq, lt, and) as
 * HorseIR's optimizer fuses them (optimizer/autofusion.cc:770-935): one
 * kernel, compiled once per window with the window's bounds as literals. */
static hgpuChain g_filter;
static I g_filter_lo, g_filter_hi;

static I filter_chain(I lo, I hi, hgpuChain *out) {
    if (!g_filter || lo != g_filter_lo || hi != g_filter_hi) {
        char prog[128];
        if (g_filter) hgpuChainDestroy(g_filter);
        g_filter = 0;
        snprintf(prog, sizeof prog, "(map (and (geq x0 %d:i32) (lt x0 %d:i32)))", (int)lo, (int)hi);
        CK(hgpuChainCreate(&g_filter, prog));
        g_filter_lo = lo;
        g_filter_hi = hi;
    }
    *out = g_filter;
    return 0;
}

/* in[0..7]: dim date, dim pk, fact fk, flag, status, qty, price, disc;
 * lo <= date < hi selects the dimension rows.
 * out[0..5]: per group flag, status, sum(qty), avg(price), sum(disc), count. */
I hgpuQueryJoinGroup(V *in, I lo, I hi, V *out) {
    V0 one, eq, d3, pk2, j, fi, flag, status, lst, g, keys, vals, qty, price, disc;
    hgpuChain filter;
    scalar_i64(&one, 1);
    symbol(&eq, "eq");
    CK(filter_chain(lo, hi, &filter));
    {
        V x[1] = {in[0]};
        CK(hgpuChainRun(filter, &d3, x));  /* d3 = (date >= lo) & (date < hi) */
    }
    CK(pfnCompress(&pk2, &d3, in[1]));
    CK(pfnJoinIndex(&j, &pk2, in[2], &eq));
    CK(pfnIndex(&fi, &j, &one));
    {
        V z[2] = {&flag, &status}, x[2] = {in[3], in[4]};
        CK(hgpuIndexMany(z, x, &fi, 2));
    }
    {
        V items[2] = {&flag, &status};
        CK(pfnList(&lst, 2, items));
    }
    CK(pfnGroup(&g, &lst));
    CK(pfnKeys(&keys, &g));
    CK(pfnValues(&vals, &g));
    {
        V z[3] = {&qty, &price, &disc}, x[3] = {in[5], in[6], in[7]};
        CK(hgpuIndexMany(z, x, &fi, 3));
    }
    CK(pfnIndex(out[0], &flag, &keys));
    CK(pfnIndex(out[1], &status, &keys));
    {  /* the four aggregates over the same groups in one call */
        V z[4] = {out[2], out[3], out[4], out[5]}, x[4] = {&qty, &price, &disc, &qty};
        const I aggs[4] = {HGPU_AGG_SUM, HGPU_AGG_AVG, HGPU_AGG_SUM, HGPU_AGG_LEN};
        CK(hgpuGroupAggMany(z, x, &vals, aggs, 4));
    }
    return 0;
}
