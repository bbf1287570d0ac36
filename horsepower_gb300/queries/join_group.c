/*
 * The join + group-by benchmark query compiled to C, the way HorseIR's code
 * generator turns a query into C: one builtin call per statement over the
 * library's C ABI (include/hgpu.h), with the common-index pattern
 * (optimizer/pattern.cc:558-672) applied to the five gathers by the join's
 * fact rows and to the four aggregates over the groups.  Statement for statement the same as plans.join_group in
 * horsepower_gb300/plans.py.  This is a caller of libhgpu, built into its own
 * libhgpu_queries.so, not part of the library.
 */
#include <string.h>

#include "hgpu.h"

static void scalar_i32(V0 *v, I x) {
    memset(v, 0, sizeof *v);
    v->typ = H_I;
    v->len = 1;
    v->g = (G)&v->b;
    v->i32 = x;
}

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

/* in[0..7]: dim date, dim pk, fact fk, flag, status, qty, price, disc;
 * lo <= date < hi selects the dimension rows.
 * out[0..5]: per group flag, status, sum(qty), avg(price), sum(disc), count. */
I hgpuQueryJoinGroup(V *in, I lo, I hi, V *out) {
    V0 slo, shi, one, eq, d1, d2, d3, pk2, j, fi, flag, status, lst, g, keys, vals, qty, price, disc;
    scalar_i32(&slo, lo);
    scalar_i32(&shi, hi);
    scalar_i64(&one, 1);
    symbol(&eq, "eq");
    CK(pfnGeq(&d1, in[0], &slo));
    CK(pfnLt(&d2, in[0], &shi));
    CK(pfnAnd(&d3, &d1, &d2));
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
