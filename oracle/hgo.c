/*
 * hgo.c — CPU oracle: arena, symbols, elementwise, reductions, compaction,
 * gather, hash search and hash join.
 *
 * THIS IS TEST INFRASTRUCTURE, NOT THE PRODUCT (see hgo.h).  Every builtin is
 * a restatement of the reference algorithm at the cited file:line, with
 * OpenMP where the reference parallelises (its DOP/DOT macros,
 * src/horseir/v3/backend/common.h:93-103) and serial code where it does not.
 */
#include "hgo.h"

L hgo_cores = 1;
const E H_EPSILON = 1e-13;

/* ------------------------------------------------------------------ arena */
/* Bump arena in 1 GiB chunks, never freed per op (h_memory.cc:93-112).
 * Heap offsets encode (chunk << 40) | cursor so setHeapOffset can rewind. */
#define HGO_CHUNK (1LL << 30)
typedef struct { G base; L cap, cur; } Chunk;
static Chunk hgo_chunks[4096];
static int hgo_nchunks = 0, hgo_curchunk = 0;

G hgo_alloc(L bytes) {
    if (bytes & 0xF) bytes = ((bytes >> 4) + 1) << 4;
    if (bytes == 0) bytes = 16;
    for (;;) {
        if (hgo_curchunk < hgo_nchunks) {
            Chunk *c = &hgo_chunks[hgo_curchunk];
            if (c->cur + bytes <= c->cap) { G g = c->base + c->cur; c->cur += bytes; R g; }
            if (hgo_curchunk + 1 < hgo_nchunks) { hgo_curchunk++; hgo_chunks[hgo_curchunk].cur = 0; continue; }
        }
        L cap = bytes > HGO_CHUNK ? bytes : HGO_CHUNK;
        G base = (G)malloc((size_t)cap);
        if (!base || hgo_nchunks >= 4096) { fprintf(stderr, "oracle: arena exhausted (%lld)\n", bytes); abort(); }
        hgo_chunks[hgo_nchunks].base = base; hgo_chunks[hgo_nchunks].cap = cap; hgo_chunks[hgo_nchunks].cur = 0;
        hgo_curchunk = hgo_nchunks++;
    }
}

L getHeapOffset(void) {
    if (hgo_nchunks == 0) R 0;
    R ((L)hgo_curchunk << 40) | hgo_chunks[hgo_curchunk].cur;
}

L setHeapOffset(L cur) {
    int c = (int)(cur >> 40);
    if (c < hgo_nchunks) { hgo_curchunk = c; hgo_chunks[c].cur = cur & ((1LL << 40) - 1); }
    R cur;
}

/* getTypeSize: h_memory.cc:124-153 */
L getTypeSize(I typ, L len) {
    L r = -1, k = 0;
    switch (typ) {
    case H_B: r = sizeof(B); break;
    case H_J: r = sizeof(J); break;
    case H_C: r = sizeof(C); k = 1; break;
    case H_H: r = sizeof(H); break;
    case H_I: case H_M: case H_D: case H_U: case H_W: case H_T: r = 4; break;
    case H_L: case H_Q: case H_Z: case H_Y: r = 8; break;
    case H_F: r = sizeof(F); break;
    case H_E: r = sizeof(E); break;
    case H_X: r = sizeof(X); break;
    case H_S: r = sizeof(S); break;
    case H_G: case H_N: case H_A: case H_K: case H_V: r = sizeof(V0); break;
    default: r = 8; break;
    }
    R r * len + k;
}

V allocNode(void) { V x = (V)hgo_alloc(sizeof(V0)); memset(x, 0, sizeof(V0)); R x; }

/* initV: h_memory.cc:182-196 — basic vectors of length <= 1 are stored inline */
V initV(V x, I typ, L len) {
    x->typ = typ; x->len = len;
    if (hgo_is_basic(typ)) x->g = (len > 1) ? hgo_alloc(getTypeSize(typ, len)) : (G)&x->b;
    else {
        x->g = hgo_alloc(getTypeSize(typ, len));
        if (typ == H_G || typ == H_N) memset(x->g, 0, (size_t)getTypeSize(typ, len));
        if (typ == H_Y) { x->y = (Y)hgo_alloc(sizeof(Y0)); memset(x->y, 0, sizeof(Y0)); }
    }
    R x;
}

/* ---------------------------------------------------------------- symbols */
/* Interning table standing in for h_symbol.cc:146-241: ids are assigned in
 * order of first appearance; an open-addressed hash of the texts finds them. */
static char **hgo_syms = NULL;
static L hgo_nsyms = 0, hgo_symcap = 0;
static L *hgo_symtab = NULL, hgo_symtab_n = 0;  /* slots hold id + 1, 0 = empty */
static uint64_t sym_hash(const char *s) { uint64_t h = 1469598103934665603ULL; while (*s) h = (h ^ (unsigned char)*s++) * 1099511628211ULL; R h; }
static void sym_rehash(L n) {
    free(hgo_symtab);
    hgo_symtab_n = n;
    hgo_symtab = (L *)calloc((size_t)n, sizeof(L));
    for (L i = 0; i < hgo_nsyms; i++) {
        L k = (L)(sym_hash(hgo_syms[i]) & (uint64_t)(n - 1));
        while (hgo_symtab[k]) k = (k + 1) & (n - 1);
        hgo_symtab[k] = i + 1;
    }
}
L getSymbol(S name) {
    if (2 * (hgo_nsyms + 1) > hgo_symtab_n) sym_rehash(hgo_symtab_n ? 2 * hgo_symtab_n : 1024);
    L k = (L)(sym_hash(name) & (uint64_t)(hgo_symtab_n - 1));
    while (hgo_symtab[k]) {
        if (!strcmp(hgo_syms[hgo_symtab[k] - 1], name)) R hgo_symtab[k] - 1;
        k = (k + 1) & (hgo_symtab_n - 1);
    }
    if (hgo_nsyms == hgo_symcap) {
        hgo_symcap = hgo_symcap ? 2 * hgo_symcap : 1024;
        hgo_syms = (char **)realloc(hgo_syms, (size_t)hgo_symcap * sizeof(char *));
    }
    hgo_syms[hgo_nsyms] = strdup(name);
    hgo_symtab[k] = hgo_nsyms + 1;
    R hgo_nsyms++;
}
S getSymbolStr(L x) { R (x >= 0 && x < hgo_nsyms) ? hgo_syms[x] : (S) ""; }

/* initBackend: global.cc:26-35 (arena, symbols, H_CORE from h_system.cc:14-24) */
void initBackend(void) {
    hgo_cores = omp_get_max_threads();
    if (hgo_nchunks == 0) { G g = hgo_alloc(16); (void)g; setHeapOffset(0); }
}

/* ------------------------------------------------------------- type groups */
B hgo_is_int(I t) { R t == H_B || t == H_J || t == H_H || t == H_I || t == H_L; }
B hgo_is_float(I t) { R t == H_F || t == H_E; }
B hgo_is_real(I t) { R hgo_is_int(t) || hgo_is_float(t); }
static B is_date(I t) { R t == H_M || t == H_D || t == H_Z; }
static B is_time(I t) { R t == H_U || t == H_W || t == H_T; }
static B is_string(I t) { R t == H_C || t == H_Q || t == H_S; }
static B is_dtime(I t) { R is_date(t) || is_time(t); }
B hgo_is_basic(I t) { R hgo_is_real(t) || is_string(t) || t == H_X || is_dtime(t); }
/* isTypeGroupComparable: h_system.cc:963-965 */
static B is_comparable(I t) { R hgo_is_real(t) || t == H_C || t == H_Q || is_dtime(t); }

I hgo_copyV(V z, V x) { *z = *x; if (vn(x) <= 1 && hgo_is_basic(vp(x)) && vg(x) == (G)&x->b) z->g = (G)&z->b; R 0; }

/* swap2: h_system.cc:47-56 */
void hgo_swap2(V z) {
    V0 t0 = *vV(z, 0), t1 = *vV(z, 1);
    initV(z, H_G, 2);
    *vV(z, 0) = t1; *vV(z, 1) = t0;
}

/* promoteValueWithIndex(z, x, typMax, NULL): h_system.cc:168-252 */
I hgo_promote(V z, V x, I typMax) {
    L n = vn(x);
    if (vp(x) == typMax) R hgo_copyV(z, x);
    initV(z, typMax, n);
#define PROM(TZ, sz, CAST)                                                         \
    switch (vp(x)) {                                                              \
    case H_B: _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) sz(z)[i] = (CAST)sB(x)[i]; break; \
    case H_J: _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) sz(z)[i] = (CAST)sJ(x)[i]; break; \
    case H_H: _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) sz(z)[i] = (CAST)sH(x)[i]; break; \
    case H_I: _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) sz(z)[i] = (CAST)sI(x)[i]; break; \
    case H_L: _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) sz(z)[i] = (CAST)sL(x)[i]; break; \
    case H_F: _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) sz(z)[i] = (CAST)sF(x)[i]; break; \
    default: R E_NOT_IMPL;                                                        \
    }
    switch (typMax) {
    case H_J: PROM(J, sJ, J) break;
    case H_H: PROM(H, sH, H) break;
    case H_I: PROM(I, sI, I) break;
    case H_L: PROM(L, sL, L) break;
    case H_F: PROM(F, sF, F) break;
    case H_E: PROM(E, sE, E) break;
    default: R E_NOT_IMPL;
    }
#undef PROM
    R 0;
}

/* checkZero: h_system.cc:254-267 */
static B check_zero(V x) {
    L n = vn(x);
    switch (vp(x)) {
    case H_B: for (L i = 0; i < n; i++) if (0 == sB(x)[i]) R 1; break;
    case H_J: for (L i = 0; i < n; i++) if (0 == sJ(x)[i]) R 1; break;
    case H_H: for (L i = 0; i < n; i++) if (0 == sH(x)[i]) R 1; break;
    case H_I: for (L i = 0; i < n; i++) if (0 == sI(x)[i]) R 1; break;
    case H_L: for (L i = 0; i < n; i++) if (0 == sL(x)[i]) R 1; break;
    case H_F: for (L i = 0; i < n; i++) if (0 == sF(x)[i]) R 1; break;
    case H_E: for (L i = 0; i < n; i++) if (0 == sE(x)[i]) R 1; break;
    }
    R 0;
}

/* isOrdered: h_system.cc:678-698 (ints and longs only) */
B hgo_is_ordered(V x) {
#define ORDERED(sX)                                                                  \
    {                                                                                \
        I order = -2; L n = vn(x);                                                   \
        for (L i = 1; i < n; i++) {                                                  \
            I v = sX(x)[i] > sX(x)[i - 1] ? 1 : sX(x)[i] < sX(x)[i - 1] ? -1 : 0;  \
            if (order == -2 && v != 0) { order = v; break; }                         \
        }                                                                            \
        if (order == -2) R 1;                                                        \
        for (L i = 1; i < n; i++) {                                                  \
            I v = sX(x)[i] > sX(x)[i - 1] ? 1 : sX(x)[i] < sX(x)[i - 1] ? -1 : 0;  \
            if (v != 0 && order != v) R 0;                                           \
        }                                                                            \
        R 1;                                                                         \
    }
    if (vp(x) == H_I) ORDERED(sI)
    if (vp(x) == H_L) ORDERED(sL)
#undef ORDERED
    R 0;
}

/* ----------------------------------------------------------- compaction */
/* getNumOfNonZero (h_system.cc:304-310) with DOT static chunks
 * (common.h:97-103); the offsets and scatter of pfnCompress
 * (h_primitive.cc:1479-1521) and pfnWhere (:728-762). */
static void count_per_thread(B *m, L n, L *par) {
    L nc = hgo_cores, seg = n / nc;
#pragma omp parallel num_threads(nc)
    {
        L tid = omp_get_thread_num();
        L c = 0;
        for (L i = tid * seg, i2 = (tid != nc - 1 ? (i + seg) : n); i < i2; i++) c += m[i];
        par[tid] = c;
    }
}

I pfnCompress(V z, V x, V y) {
    if (vp(x) != H_B) R E_DOMAIN;
    if (vn(x) != vn(y)) R E_LENGTH;
    L lenX = vn(x), nc = hgo_cores, lenZ = 0;
    I typZ = vp(y);
    L *par = calloc(nc, sizeof(L)), *off = calloc(nc, sizeof(L));
    count_per_thread(sB(x), lenX, par);
    for (L i = 0; i < nc; i++) lenZ += par[i];
    for (L i = 1; i < nc; i++) off[i] = par[i - 1] + off[i - 1];
    switch (typZ) {  /* types handled at h_primitive.cc:1497-1510; an enum exits at :1492-1494 */
    case H_B: case H_J: case H_C: case H_H: case H_I: case H_L: case H_F: case H_E: case H_Q: case H_S: case H_D: break;
    default: free(par); free(off); R E_NOT_IMPL;
    }
    initV(z, typZ, lenZ);
    if (lenX != lenZ) {
        L es = getTypeSize(typZ, 1) - (typZ == H_C ? 1 : 0);
        L seg = lenX / nc;
        B *m = sB(x);
        G src = vg(y), dst = vg(z);
#pragma omp parallel num_threads(nc)
        {
            L tid = omp_get_thread_num(), o = off[tid];
            for (L i = tid * seg, i2 = (tid != nc - 1 ? (i + seg) : lenX); i < i2; i++)
                if (m[i]) { memcpy(dst + o * es, src + i * es, (size_t)es); o++; }
        }
    } else if (lenZ > 0) {
        hgo_copyV(z, y);  /* all selected: alias the input (h_primitive.cc:1513-1515) */
    }
    free(par); free(off);
    R 0;
}

I pfnWhere(V z, V x) {
    if (vp(x) != H_B) R E_DOMAIN;  /* list-of-bool form (h_primitive.cc:750-760) is outside the path */
    L lenX = vn(x), lenZ = 0;
    if (lenX < 10000) {
        L c = 0;
        for (L i = 0; i < lenX; i++) lenZ += sB(x)[i];
        initV(z, H_L, lenZ);
        for (L i = 0; i < lenX; i++) if (sB(x)[i]) sL(z)[c++] = i;
    } else {
        L nc = hgo_cores, seg = lenX / nc;
        L *par = calloc(nc, sizeof(L)), *off = calloc(nc, sizeof(L));
        count_per_thread(sB(x), lenX, par);
        for (L i = 0; i < nc; i++) lenZ += par[i];
        for (L i = 1; i < nc; i++) off[i] = par[i - 1] + off[i - 1];
        initV(z, H_L, lenZ);
        L *d = sL(z);
        B *m = sB(x);
#pragma omp parallel num_threads(nc)
        {
            L tid = omp_get_thread_num(), o = off[tid];
            for (L i = tid * seg, i2 = (tid != nc - 1 ? (i + seg) : lenX); i < i2; i++) if (m[i]) d[o++] = i;
        }
        free(par); free(off);
    }
    R 0;
}

/* ------------------------------------------------------------ elementwise */
/* compareFloat and COMP/COMPFN: h_primitive.cc:1061-1071 */
#define CMPF(x, y) ((x) < (y) ? (((y) - (x)) < H_EPSILON ? 0 : -1) : (((x) - (y)) < H_EPSILON ? 0 : 1))
#define COMP(op, x, y) (0 == op ? (x) < (y) : 1 == op ? (x) <= (y) : 2 == op ? (x) > (y) : 3 == op ? (x) >= (y) : 4 == op ? (x) == (y) : 5 == op ? (x) != (y) : 0)
#define COMPF(op, c) (0 == op ? (c) < 0 : 1 == op ? (c) <= 0 : 2 == op ? (c) > 0 : 3 == op ? (c) >= 0 : 4 == op ? (c) == 0 : 5 == op ? (c) != 0 : 0)

#define BCAST_LOOP(n, EXPR)                                                          \
    if (ox) { _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) { L ix = 0, iy = i; (void)ix; (void)iy; EXPR; } } \
    else if (oy) { _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) { L ix = i, iy = 0; (void)ix; (void)iy; EXPR; } } \
    else { _Pragma("omp parallel for simd") for (L i = 0; i < n; i++) { L ix = i, iy = i; (void)ix; (void)iy; EXPR; } }

/* pfnCompare: h_primitive.cc:1073-1170 */
/* compareSymbol (h_symbol.cc:241-243) under COMPFN's operator (h_primitive.cc:1068-1071) */
static B sym_op(I op, L u, L v) {
    int c = u == v ? 0 : strcmp(getSymbolStr(u), getSymbolStr(v));
    R op == 0 ? c < 0 : op == 1 ? c <= 0 : op == 2 ? c > 0 : op == 3 ? c >= 0 : op == 4 ? c == 0 : c != 0;
}

I pfnCompare(V z, V x, V y, I op) {
    if (!(is_comparable(vp(x)) && is_comparable(vp(y)))) R E_DOMAIN;
    B ox = vn(x) == 1, oy = vn(y) == 1;
    if (!(ox || oy || vn(x) == vn(y))) R E_LENGTH;
    L lenZ = ox ? vn(y) : vn(x);
    if (hgo_is_real(vp(x)) && hgo_is_real(vp(y))) {
        I typMax = MAX(vp(x), vp(y));
        V0 tx, ty;
        CHECKE(hgo_promote(&tx, x, typMax));
        CHECKE(hgo_promote(&ty, y, typMax));
        initV(z, H_B, lenZ);
        B *r = sB(z);
        switch (typMax) {
        case H_B: { B *a = sB(&tx), *b = sB(&ty); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_J: { J *a = sJ(&tx), *b = sJ(&ty); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_H: { H *a = sH(&tx), *b = sH(&ty); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_I: { I *a = sI(&tx), *b = sI(&ty); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_L: { L *a = sL(&tx), *b = sL(&ty); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_F: { F *a = sF(&tx), *b = sF(&ty); BCAST_LOOP(lenZ, r[i] = COMPF(op, CMPF(a[ix], b[iy]))) } break;
        case H_E: { E *a = sE(&tx), *b = sE(&ty); BCAST_LOOP(lenZ, r[i] = COMPF(op, CMPF(a[ix], b[iy]))) } break;
        default: R E_NOT_IMPL;
        }
        R 0;
    } else if (vp(x) == vp(y)) {
        initV(z, H_B, lenZ);
        B *r = sB(z);
        switch (vp(x)) {
        case H_C: { int8_t *a = (int8_t *)vg(x), *b = (int8_t *)vg(y);  /* char is signed in the reference's x86 build */
                    BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_M: case H_D: case H_U: case H_T: { I *a = sI(x), *b = sI(y); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_Z: { L *a = sL(x), *b = sL(y); BCAST_LOOP(lenZ, r[i] = COMP(op, a[ix], b[iy])) } break;
        case H_Q: { L *a = sL(x), *b = sL(y); BCAST_LOOP(lenZ, r[i] = sym_op(op, a[ix], b[iy])) } break;
        default: R E_NOT_IMPL;  /* H_W has no case in the reference (EP) */
        }
        R 0;
    }
    R E_TYPE;
}
I pfnLt (V z, V x, V y) { R pfnCompare(z, x, y, 0); }
I pfnLeq(V z, V x, V y) { R pfnCompare(z, x, y, 1); }
I pfnGt (V z, V x, V y) { R pfnCompare(z, x, y, 2); }
I pfnGeq(V z, V x, V y) { R pfnCompare(z, x, y, 3); }
I pfnEq (V z, V x, V y) { R pfnCompare(z, x, y, 4); }
I pfnNeq(V z, V x, V y) { R pfnCompare(z, x, y, 5); }

/* pfnArith: h_primitive.cc:1227-1289, ARITH2 at :1225.  Integer types compute in
 * int (C promotion) and store truncated; bool stores x!=0. */
#define ARITH2(op, a, b) (0 == op ? (a) + (b) : 1 == op ? (a) - (b) : 2 == op ? (a) * (b) : 3 == op ? (a) / (b) : 0)
I pfnArith(V z, V x, V y, I op) {
    if (hgo_is_real(vp(x)) && hgo_is_real(vp(y))) {
        B ox = vn(x) == 1, oy = vn(y) == 1;
        if (!(ox || oy || vn(x) == vn(y))) R E_LENGTH;
        if (3 == op && check_zero(y)) R E_DIV_ZERO;
        L lenZ = ox ? vn(y) : vn(x);
        I typMax = MAX(vp(x), vp(y));
        V0 tx, ty;
        CHECKE(hgo_promote(&tx, x, typMax));
        CHECKE(hgo_promote(&ty, y, typMax));
        initV(z, typMax, lenZ);
        switch (typMax) {
        case H_B: { B *a = sB(&tx), *b = sB(&ty), *r = sB(z); BCAST_LOOP(lenZ, r[i] = (B)(ARITH2(op, (int)a[ix], (int)b[iy]) != 0)) } break;
        case H_J: { J *a = sJ(&tx), *b = sJ(&ty), *r = sJ(z); BCAST_LOOP(lenZ, r[i] = (J)ARITH2(op, (int)a[ix], (int)b[iy])) } break;
        case H_H: { H *a = sH(&tx), *b = sH(&ty), *r = sH(z); BCAST_LOOP(lenZ, r[i] = (H)ARITH2(op, (int)a[ix], (int)b[iy])) } break;
        /* i32/i64 overflow wraps; MIN/-1 (a trap on x86) is taken as the wrapped negation */
        case H_I: { I *a = sI(&tx), *b = sI(&ty), *r = sI(z);
                    BCAST_LOOP(lenZ, r[i] = (op == 3) ? (b[iy] == -1 ? (I)(0u - (uint32_t)a[ix]) : (I)(a[ix] / b[iy])) : (I)(uint32_t)ARITH2(op, (uint32_t)a[ix], (uint32_t)b[iy])) } break;
        case H_L: { L *a = sL(&tx), *b = sL(&ty), *r = sL(z);
                    BCAST_LOOP(lenZ, r[i] = (op == 3) ? (b[iy] == -1 ? (L)(0ull - (uint64_t)a[ix]) : (a[ix] / b[iy])) : (L)(uint64_t)ARITH2(op, (uint64_t)a[ix], (uint64_t)b[iy])) } break;
        case H_F: { F *a = sF(&tx), *b = sF(&ty), *r = sF(z); BCAST_LOOP(lenZ, r[i] = ARITH2(op, a[ix], b[iy])) } break;
        case H_E: { E *a = sE(&tx), *b = sE(&ty), *r = sE(z); BCAST_LOOP(lenZ, r[i] = ARITH2(op, a[ix], b[iy])) } break;
        default: R E_NOT_IMPL;
        }
        R 0;
    }
    if (is_dtime(vp(x)) && is_dtime(vp(y))) R E_NOT_IMPL;
    R E_DOMAIN;
}
I pfnPlus (V z, V x, V y) { R pfnArith(z, x, y, 0); }
I pfnMinus(V z, V x, V y) { R pfnArith(z, x, y, 1); }
I pfnMul  (V z, V x, V y) { R pfnArith(z, x, y, 2); }
I pfnDiv  (V z, V x, V y) { R pfnArith(z, x, y, 3); }

/* pfnLogic: h_primitive.cc:1315-1332 with logicAnd..logicXor (h_system.cc:898-916).
 * logicNand/logicNor return ~(x&y)/~(x|y) converted to bool, which is true for
 * every input; that is what the reference computes and what is restated. */
static I logic(V z, V x, V y, int op) {
    if (!(vp(x) == H_B && vp(y) == H_B)) R E_DOMAIN;
    B ox = vn(x) == 1, oy = vn(y) == 1;
    if (!(ox || oy || vn(x) == vn(y))) R E_LENGTH;
    L lenZ = ox ? vn(y) : vn(x);
    initV(z, H_B, lenZ);
    B *a = sB(x), *b = sB(y), *r = sB(z);
    switch (op) {
    case 0: BCAST_LOOP(lenZ, r[i] = (B)(a[ix] & b[iy])) break;
    case 1: BCAST_LOOP(lenZ, r[i] = (B)(~(a[ix] & b[iy]))) break;
    case 2: BCAST_LOOP(lenZ, r[i] = (B)(a[ix] | b[iy])) break;
    case 3: BCAST_LOOP(lenZ, r[i] = (B)(~(a[ix] | b[iy]))) break;
    case 4: BCAST_LOOP(lenZ, r[i] = (B)(a[ix] ^ b[iy])) break;
    }
    R 0;
}
I pfnAnd (V z, V x, V y) { R logic(z, x, y, 0); }
I pfnNand(V z, V x, V y) { R logic(z, x, y, 1); }
I pfnOr  (V z, V x, V y) { R logic(z, x, y, 2); }
I pfnNor (V z, V x, V y) { R logic(z, x, y, 3); }
I pfnXor (V z, V x, V y) { R logic(z, x, y, 4); }

/* pfnNot: h_primitive.cc:606-615, NOT(x) = (!x) at :352 */
I pfnNot(V z, V x) {
    if (vp(x) != H_B) R E_DOMAIN;
    L n = vn(x);
    initV(z, H_B, n);
#pragma omp parallel for simd
    for (L i = 0; i < n; i++) sB(z)[i] = !sB(x)[i];
    R 0;
}

/* ------------------------------------------------------------- reductions */
/* pfnSum: h_primitive.cc:764-786 — ints accumulate in i64, f32 in f32, f64 in
 * f64, each with an OpenMP reduction(+) whose order depends on the thread count. */
I pfnSum(V z, V x) {
    if (!hgo_is_real(vp(x))) R E_DOMAIN;
    I typZ = vp(x) == H_F ? H_F : vp(x) == H_E ? H_E : H_L;
    L n = vn(x);
    initV(z, typZ, 1);
#define SUMI(sX) { L t = 0; _Pragma("omp parallel for simd reduction(+:t)") for (L i = 0; i < n; i++) t += sX(x)[i]; z->i64 = t; }
    switch (vp(x)) {
    case H_B: SUMI(sB) break;
    case H_J: SUMI(sJ) break;
    case H_H: SUMI(sH) break;
    case H_I: SUMI(sI) break;
    case H_L: { uint64_t t = 0; uint64_t *p = (uint64_t *)vg(x);
#pragma omp parallel for simd reduction(+:t)
                for (L i = 0; i < n; i++) t += p[i];
                z->i64 = (L)t; } break;
    case H_F: { F t = 0;
#pragma omp parallel for simd reduction(+:t)
                for (L i = 0; i < n; i++) t += sF(x)[i];
                z->f32 = t; } break;
    case H_E: { E t = 0;
#pragma omp parallel for simd reduction(+:t)
                for (L i = 0; i < n; i++) t += sE(x)[i];
                z->f64 = t; } break;
    }
#undef SUMI
    R 0;
}

/* pfnAvg: h_primitive.cc:788-800 */
I pfnAvg(V z, V x) {
    V0 t;
    CHECKE(pfnSum(&t, x));
    I typZ = vp(&t) == H_F ? H_F : H_E;
    initV(z, typZ, 1);
    switch (vp(&t)) {
    case H_L: z->f64 = t.i64 * 1.0 / vn(x); break;
    case H_F: z->f32 = t.f32 / vn(x); break;
    case H_E: z->f64 = t.f64 / vn(x); break;
    }
    R 0;
}

/* pfnReduce: h_primitive.cc:802-839 — serial fold from x[0]; empty input
 * returns LLONG_MAX/LLONG_MIN, FLT_MAX/FLT_MIN, DBL_MAX/DBL_MIN sentinels. */
I pfnReduce(V z, V x, I op) {
    if (!hgo_is_real(vp(x))) R E_DOMAIN;
    L n = vn(x);
    if (n < 1) {
        I typZ = hgo_is_int(vp(x)) ? H_L : vp(x);
        initV(z, typZ, 1);
        switch (typZ) {
        case H_L: z->i64 = 0 == op ? LLONG_MAX : LLONG_MIN; break;
        case H_F: z->f32 = 0 == op ? FLT_MAX : FLT_MIN; break;
        case H_E: z->f64 = 0 == op ? DBL_MAX : DBL_MIN; break;
        default: R E_NOT_IMPL;
        }
        R 0;
    }
    initV(z, vp(x), 1);
#define FOLD(TY, sX, fld) { TY t = sX(x)[0]; for (L i = 0; i < n; i++) { TY v = sX(x)[i]; t = 0 == op ? ((t < v) ? t : v) : ((t > v) ? t : v); } z->fld = t; }
    switch (vp(x)) {
    case H_B: FOLD(B, sB, b) break;
    case H_J: FOLD(J, sJ, j) break;
    case H_H: FOLD(H, sH, h) break;
    case H_I: FOLD(I, sI, i32) break;
    case H_L: FOLD(L, sL, i64) break;
    case H_F: FOLD(F, sF, f32) break;
    case H_E: FOLD(E, sE, f64) break;
    default: R E_NOT_IMPL;
    }
#undef FOLD
    R 0;
}
I pfnMin(V z, V x) { R pfnReduce(z, x, 0); }
I pfnMax(V z, V x) { R pfnReduce(z, x, 1); }

/* pfnLen: h_primitive.cc:656-662 */
I pfnLen(V z, V x) { L n = vn(x); initV(z, H_L, 1); z->i64 = n; R 0; }

/* ----------------------------------------------------------------- gather */
/* pfnIndex: h_primitive.cc:43-94.  The index vector is promoted to i64 and
 * checked against len(x) (E_INDEX).  Two reference behaviours are undefined
 * and replaced here: a negative index (read before the buffer) also yields
 * E_INDEX, and a non-i64 index vector is read through its promoted copy
 * (the reference reads the narrow buffer at 8-byte stride, :60). */
I pfnIndex(V z, V x, V y) {
    if (!hgo_is_int(vp(y))) R E_DOMAIN;
    I typZ = vp(x);
    L lenZ = vn(y), lenX = vn(x);
    V0 ty;
    CHECKE(hgo_promote(&ty, y, H_L));
    L *iy = sL(&ty);
    for (L i = 0; i < lenZ; i++) if (lenX <= iy[i] || iy[i] < 0) R E_INDEX;
    if (hgo_is_basic(vp(x))) {
        initV(z, typZ, lenZ);
        L es = getTypeSize(typZ, 1) - (typZ == H_C ? 1 : 0);
        G src = vg(x), dst = vg(z);
        switch (es) {
        case 1: { int8_t *s = (int8_t *)src, *d = (int8_t *)dst;
#pragma omp parallel for simd
                  for (L i = 0; i < lenZ; i++) d[i] = s[iy[i]]; } break;
        case 2: { int16_t *s = (int16_t *)src, *d = (int16_t *)dst;
#pragma omp parallel for simd
                  for (L i = 0; i < lenZ; i++) d[i] = s[iy[i]]; } break;
        case 4: { int32_t *s = (int32_t *)src, *d = (int32_t *)dst;
#pragma omp parallel for simd
                  for (L i = 0; i < lenZ; i++) d[i] = s[iy[i]]; } break;
        case 8: { int64_t *s = (int64_t *)src, *d = (int64_t *)dst;
#pragma omp parallel for simd
                  for (L i = 0; i < lenZ; i++) d[i] = s[iy[i]]; } break;
        default: R E_NOT_IMPL;
        }
        R 0;
    } else if (vp(x) == H_G) {
        if (lenZ == 1 && hgo_is_int(vp(y))) R hgo_copyV(z, vV(x, iy[0]));
        R E_NOT_IMPL;
    }
    R E_NOT_IMPL;
}

/* ------------------------------------------------------------ hash search */
/* Open-addressing table mapping a key's bit pattern to the first row that
 * holds it.  It restates the observable behaviour of the chained tables of
 * insert_hash/find_hash (h_libs.cc:160-206, unique insert: first row wins)
 * with equality on the value (so NaN never matches). */
typedef struct { uint64_t *key; L *row; L mask; } HT;
static uint64_t mix64(uint64_t k) { k ^= k >> 33; k *= 0xff51afd7ed558ccdULL; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ULL; k ^= k >> 33; R k; }
static void ht_init(HT *t, L n) {
    L cap = 16; while (cap < 2 * n) cap <<= 1;
    t->mask = cap - 1;
    t->key = malloc(sizeof(uint64_t) * cap);
    t->row = malloc(sizeof(L) * cap);
    for (L i = 0; i < cap; i++) t->row[i] = -1;
}
static void ht_free(HT *t) { free(t->key); free(t->row); }
/* insert: returns the row already stored for the key, or stores r */
static L ht_insert(HT *t, uint64_t k, L r) {
    L h = (L)(mix64(k) & (uint64_t)t->mask);
    while (t->row[h] >= 0) { if (t->key[h] == k) R t->row[h]; h = (h + 1) & t->mask; }
    t->key[h] = k; t->row[h] = r; R r;
}
static L ht_find(HT *t, uint64_t k) {
    L h = (L)(mix64(k) & (uint64_t)t->mask);
    while (t->row[h] >= 0) { if (t->key[h] == k) R t->row[h]; h = (h + 1) & t->mask; }
    R -1;
}
/* Key bits of element i of a promoted vector; returns 0 for NaN (never equal). */
static B key_bits(V x, L i, uint64_t *k) {
    switch (vp(x)) {
    case H_B: *k = (uint64_t)sB(x)[i]; R 1;
    case H_J: *k = (uint64_t)(int64_t)sJ(x)[i]; R 1;
    case H_H: *k = (uint64_t)(int64_t)sH(x)[i]; R 1;
    case H_I: *k = (uint64_t)(int64_t)sI(x)[i]; R 1;
    case H_L: *k = (uint64_t)sL(x)[i]; R 1;
    case H_F: { F f = sF(x)[i]; if (f != f) R 0; uint32_t u; memcpy(&u, &f, 4); *k = u; R 1; }
    case H_E: { E f = sE(x)[i]; if (f != f) R 0; uint64_t u; memcpy(&u, &f, 8); *k = u; R 1; }
    }
    R 0;
}

/* binarySearch_I/L and searchOrdered: h_system.cc:715-745 — returns the index
 * the recursion lands on, or len(x).  An empty x (which the reference reads
 * at x[0]) yields len(x)=0. */
static L bsearch_L(const L *x, L low, L high, L val) {
    for (;;) {
        L mid = (low + high) >> 1;
        if (x[mid] == val) R mid;
        if (low == mid) R -1;
        if (x[mid] > val) high = mid; else low = mid;
    }
}
static L bsearch_I(const I *x, L low, L high, I val) {
    for (;;) {
        L mid = (low + high) >> 1;
        if (x[mid] == val) R mid;
        if (low == mid) R -1;
        if (x[mid] > val) high = mid; else low = mid;
    }
}

static L elem_l(V x, L i);

/* pfnIndexOf on two lists (lib_index_of_G, h_libs.cc:370-373; isListIndexOf
 * h_system.cc:591-603): for each y row, the first x row whose columns all
 * equal it (compareTuple, h_system.cc:567-589: columns of different types
 * never compare equal), else len(x).  Integer columns only here (float,
 * string and complex columns: E_NOT_IMPL; the reference exits on the others). */
static I index_of_list(V z, V x, V y) {
    if (vn(x) != vn(y)) R E_DOMAIN;
    L nc = vn(x), lenX = nc ? vn(vV(x, 0)) : 0, lenY = nc ? vn(vV(y, 0)) : 0;
    for (L c = 0; c < nc; c++) if (vn(vV(x, c)) != lenX || vn(vV(y, c)) != lenY) R E_LENGTH;
    if (nc > 8) R E_NOT_IMPL;
    B same = 1;
    for (L c = 0; c < nc; c++) {
        I tx = vp(vV(x, c)), ty = vp(vV(y, c));
        if (!(tx == H_J || tx == H_H || tx == H_I || tx == H_L) || !(ty == H_J || ty == H_H || ty == H_I || ty == H_L)) R E_NOT_IMPL;
        same = same && tx == ty;
    }
    initV(z, H_L, lenY);
    if (!same || lenX == 0) { for (L i = 0; i < lenY; i++) sL(z)[i] = lenX; R 0; }
    L cap = 16; while (cap < 2 * lenX) cap <<= 1;
    L *slot = (L *)malloc(sizeof(L) * (size_t)cap);
    for (L k = 0; k < cap; k++) slot[k] = -1;
#define ROW_HASH(V_, r_) ({ uint64_t h_ = 1469598103934665603ULL; for (L c_ = 0; c_ < nc; c_++) h_ = mix64(h_ ^ (uint64_t)elem_l(vV(V_, c_), r_)); h_; })
#define ROW_EQ(A_, a_, B_, b_) ({ B e_ = 1; for (L c_ = 0; c_ < nc && e_; c_++) e_ = elem_l(vV(A_, c_), a_) == elem_l(vV(B_, c_), b_); e_; })
    for (L r = 0; r < lenX; r++) {  /* first occurrence of each tuple */
        L k = (L)(ROW_HASH(x, r) & (uint64_t)(cap - 1));
        while (slot[k] >= 0 && !ROW_EQ(x, slot[k], x, r)) k = (k + 1) & (cap - 1);
        if (slot[k] < 0) slot[k] = r;
    }
    for (L i = 0; i < lenY; i++) {
        L k = (L)(ROW_HASH(y, i) & (uint64_t)(cap - 1)), found = lenX;
        while (slot[k] >= 0) {
            if (ROW_EQ(x, slot[k], y, i)) { found = slot[k]; break; }
            k = (k + 1) & (cap - 1);
        }
        sL(z)[i] = found;
    }
#undef ROW_HASH
#undef ROW_EQ
    free(slot);
    R 0;
}

/* pfnIndexOf: h_primitive.cc:1523-1579, lib_index_of_*: h_libs.cc:299-373 */
I pfnIndexOf(V z, V x, V y) {
    if (vp(x) == H_G && vp(y) == H_G) R index_of_list(z, x, y);
    if (hgo_is_real(vp(x)) && hgo_is_real(vp(y))) {
        L lenX = vn(x), lenZ = vn(y);
        if (hgo_is_ordered(x)) {
            /* searchOrdered (h_system.cc:731-745) reads y through x's element
             * type, vI(y,i) / vL(y,i), whatever y's type: a y at least as wide
             * as x is read as its first len(y) words of x's width; a narrower y
             * would be read past its end (undefined): E_TYPE here. */
            if (getTypeSize(vp(y), 1) < getTypeSize(vp(x), 1)) R E_TYPE;
            initV(z, H_L, lenZ);
            if (lenX == 0) { for (L i = 0; i < lenZ; i++) sL(z)[i] = 0; R 0; }
            if (vp(x) == H_I) {
                const I *yw = (const I *)vg(y);
#pragma omp parallel for
                for (L i = 0; i < lenZ; i++) { L k = bsearch_I(sI(x), 0, lenX, yw[i]); sL(z)[i] = k < 0 ? lenX : k; }
            } else {
                const L *yw = (const L *)vg(y);
#pragma omp parallel for
                for (L i = 0; i < lenZ; i++) { L k = bsearch_L(sL(x), 0, lenX, yw[i]); sL(z)[i] = k < 0 ? lenX : k; }
            }
            R 0;
        }
        I typMax = MAX(vp(x), vp(y));
        V0 tx, ty;
        CHECKE(hgo_promote(&tx, x, typMax));
        CHECKE(hgo_promote(&ty, y, typMax));
        initV(z, H_L, lenZ);
        if (typMax == H_B) {
            /* lib_index_of_B (h_libs.cc:309-314): flag[2]={-1} leaves flag[1]=0, so
             * `true` always maps to 0 and `false` to its first row (or len). */
            L flag[2] = {-1, 0};
            for (L i = 0; i < lenX; i++) if (!sB(&tx)[i] && flag[0] == -1) { flag[0] = i; break; }
            for (L i = 0; i < lenZ; i++) { L t = flag[sB(&ty)[i] ? 1 : 0]; sL(z)[i] = t < 0 ? lenX : t; }
            R 0;
        }
        HT t;
        ht_init(&t, lenX);
        for (L i = 0; i < lenX; i++) { uint64_t k; if (key_bits(&tx, i, &k)) ht_insert(&t, k, i); }
        for (L i = 0; i < lenZ; i++) {
            uint64_t k; L r = -1;
            if (key_bits(&ty, i, &k)) r = ht_find(&t, k);
            sL(z)[i] = r < 0 ? lenX : r;
        }
        ht_free(&t);
        R 0;
    }
    if (vp(x) == vp(y) && (is_dtime(vp(x)) || vp(x) == H_Q)) {
        /* INDEXOF(M/D/Z/U/W/T/Q) = lib_index_of_I/L (h_libs.h:25-31): hashed,
         * never binary searched */
        V0 tx = *x, ty = *y;
        tx.typ = ty.typ = getTypeSize(vp(x), 1) == 4 ? H_I : H_L;
        if (vg(x) == (G)&x->b) tx.g = (G)&tx.b;
        if (vg(y) == (G)&y->b) ty.g = (G)&ty.b;
        L lenX = vn(x), lenZ = vn(y);
        initV(z, H_L, lenZ);
        HT t;
        ht_init(&t, lenX);
        for (L i = 0; i < lenX; i++) { uint64_t k; if (key_bits(&tx, i, &k)) ht_insert(&t, k, i); }
        for (L i = 0; i < lenZ; i++) {
            uint64_t k; L r = -1;
            if (key_bits(&ty, i, &k)) r = ht_find(&t, k);
            sL(z)[i] = r < 0 ? lenX : r;
        }
        ht_free(&t);
        R 0;
    }
    if (vp(x) == vp(y)) R E_NOT_IMPL;  /* strings, lists: outside the path */
    R E_TYPE;
}

/* pfnEnum: h_primitive.cc:2198-2222.  The enum's index is index_of(x, y);
 * an index >= the key rows is E_ENUM_INDEX (:2204, :2216).  Header
 * {source -1, ek x, ev y} (initEnum, h_primitive.h:12-16).  x and y may be
 * two lists of the same number of columns (multi-column keys). */
I pfnEnum(V z, V x, V y) {
    B lists = vp(x) == H_G && vp(y) == H_G;
    if (lists && vn(x) != vn(y)) R E_DOMAIN;
    if (!lists && !hgo_is_basic(vp(x))) R E_DOMAIN;
    V0 ind;
    CHECKE(pfnIndexOf(&ind, x, y));
    L lenZ = vn(&ind), lenX = lists ? (vn(x) ? vn(vV(x, 0)) : 0) : vn(x);
    for (L i = 0; i < lenZ; i++) if (sL(&ind)[i] >= lenX) R E_ENUM_INDEX;
    initV(z, H_Y, lenZ);
    z->y->source = -1; z->y->ek = (G)x; z->y->ev = (G)y;
    memcpy(vg(z), sL(&ind), (size_t)lenZ * 8);
    R 0;
}

/* pfnFetch: h_primitive.cc:219-225 */
I pfnFetch(V z, V x) { if (vp(x) == H_Y) R hgo_copyV(z, (V)x->y->ev); R E_DOMAIN; }

/* pfnMember(z, y, x): h_primitive.cc:2287-2336, lib_member_*: h_libs.cc:897-1018.
 * z[i] = y[i] in x.  Sets of <= 2 elements use direct compares (== on the
 * promoted value, lib_member_fast1/2); larger sets hash.  An empty x (read at
 * x[0] by the reference) yields false. */
I pfnMember(V z, V y, V x) {
    if (hgo_is_real(vp(x)) && hgo_is_real(vp(y))) {
        I typMax = MAX(vp(x), vp(y));
        if (typMax == H_J) R E_NOT_IMPL;  /* the reference has no i8 case (EP) */
        V0 tx, ty;
        CHECKE(hgo_promote(&tx, x, typMax));
        CHECKE(hgo_promote(&ty, y, typMax));
        L sLen = vn(x), vLen = vn(y);
        initV(z, H_B, vLen);
        B *r = sB(z);
        if (typMax == H_B) {  /* lib_member_B: h_libs.cc:969-974 */
            B flag[2] = {0, 0};
            for (L i = 0; i < sLen; i++) flag[sB(&tx)[i] ? 1 : 0] = 1;
            for (L i = 0; i < vLen; i++) r[i] = flag[sB(&ty)[i] ? 1 : 0];
            R 0;
        }
#define EQV(a, ia, b, ib) (typMax == H_F ? sF(a)[ia] == sF(b)[ib] : typMax == H_E ? sE(a)[ia] == sE(b)[ib] : \
                           typMax == H_H ? sH(a)[ia] == sH(b)[ib] : typMax == H_I ? sI(a)[ia] == sI(b)[ib] : sL(a)[ia] == sL(b)[ib])
        if (sLen == 0) { for (L i = 0; i < vLen; i++) r[i] = 0; R 0; }
        if (sLen <= 2) {
#pragma omp parallel for
            for (L i = 0; i < vLen; i++) r[i] = EQV(&ty, i, &tx, 0) || (sLen == 2 && EQV(&ty, i, &tx, 1));
            R 0;
        }
#undef EQV
        HT t;
        ht_init(&t, sLen);
        for (L i = 0; i < sLen; i++) { uint64_t k; if (key_bits(&tx, i, &k)) ht_insert(&t, k, i); }
#pragma omp parallel for
        for (L i = 0; i < vLen; i++) { uint64_t k; r[i] = key_bits(&ty, i, &k) && ht_find(&t, k) >= 0; }
        ht_free(&t);
        R 0;
    }
    if (vp(x) == vp(y) && vp(x) == H_C) {  /* lib_member_C: h_libs.cc:989-995 (bytes as unsigned) */
        B buff[256] = {0};
        L vLen = vn(y);
        for (L i = 0; i < vn(x); i++) buff[((unsigned char *)vg(x))[i]] = 1;
        initV(z, H_B, vLen);
        for (L i = 0; i < vLen; i++) sB(z)[i] = buff[((unsigned char *)vg(y))[i]];
        R 0;
    }
    if (vp(x) == vp(y)) R E_NOT_IMPL;
    R E_DOMAIN;
}

/* ------------------------------------------------------------- hash join */
/* lib_join_radix_hash_v3 (h_hash_v3.cc:230-260): build on x (the shorter
 * side), probe y in row order, and for each probe row j emit every build row
 * holding y[j], in build-row order.  The reference only accepts i32 keys on
 * this path (else EP); i64 keys are accepted here with the same ordering
 * contract (extension).  Duplicate build keys are unlimited (the reference
 * caps them at 1024, :9,27). */
static I join_hash(V z0, V z1, V x, V y) {
    L nx = vn(x), ny = vn(y);
    HT t;
    ht_init(&t, nx);
    L *cnt = calloc(nx > 0 ? nx : 1, sizeof(L)), *first = malloc(sizeof(L) * (nx > 0 ? nx : 1));
    L *slot_of = malloc(sizeof(L) * (nx > 0 ? nx : 1));
    for (L i = 0; i < nx; i++) {  /* distinct keys numbered in first-seen order */
        uint64_t k = vp(x) == H_I ? (uint64_t)(int64_t)sI(x)[i] : (uint64_t)sL(x)[i];
        L r = ht_insert(&t, k, i);
        slot_of[i] = r;
        cnt[r]++;
    }
    /* per first-row, the list of rows with that key, ascending */
    L *start = malloc(sizeof(L) * (nx + 1)), *rows = malloc(sizeof(L) * (nx > 0 ? nx : 1));
    L acc = 0;
    for (L i = 0; i < nx; i++) { start[i] = acc; acc += cnt[i]; }
    start[nx] = acc;
    memset(first, 0, sizeof(L) * (nx > 0 ? nx : 1));
    for (L i = 0; i < nx; i++) { L r = slot_of[i]; rows[start[r] + first[r]++] = i; }
    L *hit = malloc(sizeof(L) * (ny > 0 ? ny : 1));
    L c = 0;
    for (L j = 0; j < ny; j++) {
        uint64_t k = vp(y) == H_I ? (uint64_t)(int64_t)sI(y)[j] : (uint64_t)sL(y)[j];
        L r = ht_find(&t, k);
        hit[j] = r;
        if (r >= 0) c += cnt[r];
    }
    initV(z0, H_L, c);
    initV(z1, H_L, c);
    c = 0;
    for (L j = 0; j < ny; j++) {
        L r = hit[j];
        if (r < 0) continue;
        for (L q = 0; q < cnt[r]; q++) { sL(z0)[c] = rows[start[r] + q]; sL(z1)[c] = j; c++; }
    }
    free(hit); free(rows); free(start); free(slot_of); free(first); free(cnt);
    ht_free(&t);
    R 0;
}

/* lib_join_index_linear: h_libs.cc:1542-1575 — for each y row, the FIRST x row
 * that compares (== or !=); i32, i64 and f64 keys. */
static I join_linear(V z0, V z1, V x, V y, B isEq) {
    L nx = vn(x), ny = vn(y), size = 0;
#define JL_MATCH(j, i) (vp(x) == H_I ? (isEq ? sI(y)[i] == sI(x)[j] : sI(y)[i] != sI(x)[j]) : \
                        vp(x) == H_L ? (isEq ? sL(y)[i] == sL(x)[j] : sL(y)[i] != sL(x)[j]) : \
                                       (isEq ? sE(y)[i] == sE(x)[j] : sE(y)[i] != sE(x)[j]))
    if (vp(x) != H_I && vp(x) != H_L && vp(x) != H_E) R E_NOT_IMPL;
    for (L i = 0; i < ny; i++) for (L j = 0; j < nx; j++) if (JL_MATCH(j, i)) { size++; break; }
    initV(z0, H_L, size);
    initV(z1, H_L, size);
    size = 0;
    for (L i = 0; i < ny; i++) for (L j = 0; j < nx; j++) if (JL_MATCH(j, i)) { sL(z0)[size] = j; sL(z1)[size++] = i; break; }
#undef JL_MATCH
    R 0;
}

/* pfnJoinIndexSingle: h_primitive.cc:1944-2040 (eq/neq over real types) */
static I join_single(V z, V x, V y, V f) {
    S name = getSymbolStr(f->q);
    I op = !strcmp(name, "lt") ? 0 : !strcmp(name, "leq") ? 1 : !strcmp(name, "gt") ? 2 : !strcmp(name, "geq") ? 3
         : !strcmp(name, "eq") ? 4 : !strcmp(name, "neq") ? 5 : -1;
    if (op < 0) R E_DOMAIN;
    if (!(hgo_is_real(vp(x)) && hgo_is_real(vp(y)))) R vp(x) == vp(y) ? E_NOT_IMPL : E_TYPE;
    if (op != 4 && op != 5) R E_NOT_IMPL;  /* brute-force path waits on getchar() (:2012) */
    I typMax = MAX(vp(x), vp(y));
    V0 tx, ty;
    CHECKE(hgo_promote(&tx, x, typMax));
    CHECKE(hgo_promote(&ty, y, typMax));
    initV(z, H_G, 2);
    switch (typMax) {
    case H_H: case H_I: case H_L: case H_F: case H_E:
        if (vn(x) >= 10) {  /* NUM_JOIN_LINEAR, common.h:152 */
            if (op != 4) R E_NOT_IMPL;
            if (typMax != H_I && typMax != H_L) R E_NOT_IMPL;
            R join_hash(vV(z, 0), vV(z, 1), &tx, &ty);
        }
        R join_linear(vV(z, 0), vV(z, 1), &tx, &ty, op == 4);
    default: R E_NOT_IMPL;
    }
}

static I op_of_sym(L q) {
    S n = getSymbolStr(q);
    if (!n) R -1;
    R !strcmp(n, "lt") ? 0 : !strcmp(n, "leq") ? 1 : !strcmp(n, "gt") ? 2 : !strcmp(n, "geq") ? 3
    : !strcmp(n, "eq") ? 4 : !strcmp(n, "neq") ? 5 : -1;
}
/* element i of a real column as a double / an i64 (promoteValue's C casts);
 * COMP on the promoted type (h_primitive.cc:1063-1066) */
static E elem_e(V x, L i) {
    switch (vp(x)) {
    case H_B: R (E)sB(x)[i]; case H_J: case H_C: R (E)((signed char *)vg(x))[i]; case H_H: R (E)sH(x)[i];
    case H_I: R (E)sI(x)[i]; case H_F: R (E)sF(x)[i]; case H_E: R sE(x)[i]; default: R (E)sL(x)[i];
    }
}
static L elem_l(V x, L i) {
    switch (vp(x)) {
    case H_B: R sB(x)[i]; case H_J: case H_C: R ((signed char *)vg(x))[i]; case H_H: R sH(x)[i];
    case H_I: R sI(x)[i]; default: R sL(x)[i];
    }
}
static B comp_pair(V x, V y, L a, L b, I op) {
    I t = MAX(vp(x), vp(y));
    if (t == H_F) {
        F u = vp(x) == H_F ? sF(x)[a] : (F)elem_l(x, a), v = vp(y) == H_F ? sF(y)[b] : (F)elem_l(y, b);
        R op == 0 ? u < v : op == 1 ? u <= v : op == 2 ? u > v : op == 3 ? u >= v : op == 4 ? u == v : u != v;
    }
    if (t == H_E) {
        E u = elem_e(x, a), v = elem_e(y, b);
        R op == 0 ? u < v : op == 1 ? u <= v : op == 2 ? u > v : op == 3 ? u >= v : op == 4 ? u == v : u != v;
    }
    L u = elem_l(x, a), v = elem_l(y, b);
    switch (t) {  /* narrower integer types wrap as the promoted C type would */
    case H_B: u = (B)u; v = (B)v; break;
    case H_J: u = (signed char)u; v = (signed char)v; break;
    case H_H: u = (short)u; v = (short)v; break;
    case H_I: u = (int)u; v = (int)v; break;
    default: break;
    }
    R op == 0 ? u < v : op == 1 ? u <= v : op == 2 ? u > v : op == 3 ? u >= v : op == 4 ? u == v : u != v;
}
/* pfnJoinIndexMultiple: h_primitive.cc:2094-2110 — join on the first @eq
 * column (getFirstEqual :2088-2092; else @neq, else column 0) with no
 * shorter-side swap and no linear path (joinOneColumn, h_system.cc:856-880),
 * then keep the pairs whose other columns compare true, column by column
 * (joinOtherColumns :846-853, compareOneColumn :818-838).  Equi-joins on
 * i32/i64 keys only (the reference's hash path; i64 is an extension). */
static I join_multi(V z, V x, V y, V f) {
    if (vp(x) != H_G || vp(y) != H_G) R E_DOMAIN;
    L nc = vn(f);
    if (vn(x) != nc || vn(y) != nc) R E_LENGTH;
    L fx = -1;
    for (L i = 0; i < nc && fx < 0; i++) if (op_of_sym(sL(f)[i]) == 4) fx = i;
    for (L i = 0; i < nc && fx < 0; i++) if (op_of_sym(sL(f)[i]) == 5) fx = i;
    if (fx < 0) fx = 0;
    for (L i = 0; i < nc; i++) if (op_of_sym(sL(f)[i]) < 0) R E_DOMAIN;
    if (op_of_sym(sL(f)[fx]) != 4) R E_NOT_IMPL;
    V x0 = vV(x, fx), y0 = vV(y, fx);
    L nx = vn(x0), ny = vn(y0);
    for (L i = 0; i < nc; i++) {
        if (vn(vV(x, i)) != nx || vn(vV(y, i)) != ny) R E_LENGTH;
        if (!hgo_is_real(vp(vV(x, i))) || !hgo_is_real(vp(vV(y, i)))) R E_TYPE;
    }
    I typMax = MAX(vp(x0), vp(y0));
    if (typMax != H_I && typMax != H_L) R E_NOT_IMPL;
    V0 tx, ty, j0, j1;
    CHECKE(hgo_promote(&tx, x0, typMax));
    CHECKE(hgo_promote(&ty, y0, typMax));
    CHECKE(join_hash(&j0, &j1, &tx, &ty));
    L m = vn(&j0);
    L *a = malloc(sizeof(L) * (m > 0 ? m : 1)), *b = malloc(sizeof(L) * (m > 0 ? m : 1));
    memcpy(a, sL(&j0), sizeof(L) * m);
    memcpy(b, sL(&j1), sizeof(L) * m);
    for (L i = 0; i < nc; i++) {
        if (i == fx) continue;
        I op = op_of_sym(sL(f)[i]);
        L k = 0;
        for (L q = 0; q < m; q++) if (comp_pair(vV(x, i), vV(y, i), a[q], b[q], op)) { a[k] = a[q]; b[k] = b[q]; k++; }
        m = k;
    }
    initV(z, H_G, 2);
    initV(vV(z, 0), H_L, m);
    initV(vV(z, 1), H_L, m);
    memcpy(sL(vV(z, 0)), a, sizeof(L) * m);
    memcpy(sL(vV(z, 1)), b, sizeof(L) * m);
    free(a); free(b);
    R 0;
}

/* pfnJoinIndex: h_primitive.cc:2122-2155 — the shorter side is built; when x
 * is strictly longer the call is mirrored and the two outputs swapped. */
I pfnJoinIndex(V z, V x, V y, V f) {
    if (vn(f) == 1) {
        if (vn(x) > vn(y)) { CHECKE(join_single(z, y, x, f)); hgo_swap2(z); R 0; }
        R join_single(z, x, y, f);
    }
    if (vn(f) > 1) R join_multi(z, x, y, f);
    R E_DOMAIN;
}

/* ----------------------------------------------------------------- lists */
/* pfnList: h_primitive.cc:32-36 */
I pfnList(V z, L n, V x[]) {
    initV(z, H_G, n);
    for (L i = 0; i < n; i++) { *vV(z, i) = *x[i]; if (vn(x[i]) <= 1 && hgo_is_basic(vp(x[i])) && vg(x[i]) == (G)&x[i]->b) vV(z, i)->g = (G)&vV(z, i)->b; }
    R 0;
}
/* pfnKeys / pfnValues on a dict: h_primitive.cc:191-217, getDictValue h_system.cc:508-515 */
I pfnKeys(V z, V x) {
    if (vp(x) == H_Y) R hgo_copyV(z, (V)x->y->ek);
    if (vp(x) == H_N || vp(x) == H_A) R hgo_copyV(z, vV(x, 0));
    R E_DOMAIN;
}
/* enum: copyEnumIndex (h_system.cc:501-506), the index as an i64 vector */
I pfnValues(V z, V x) {
    if (vp(x) == H_Y) { z->typ = H_L; z->len = vn(x); z->g = vg(x); R 0; }
    if (vp(x) == H_N || vp(x) == H_A) R hgo_copyV(z, vV(x, 1));
    R E_DOMAIN;
}

/* pfnEach: h_primitive.cc:1818-1832 (plain lists) */
I pfnEach(V z, V x, I (*foo)(V, V)) {
    if (vp(x) != H_G) R E_DOMAIN;
    L n = vn(x);
    initV(z, H_G, n);
    for (L i = 0; i < n; i++) CHECKE(foo(vV(z, i), vV(x, i)));
    R 0;
}
/* pfnEachRight: h_primitive.cc:1882-1904 (plain lists) */
I pfnEachRight(V z, V x, V y, I (*foo)(V, V, V)) {
    if (vp(y) == H_G) {
        L n = vn(y);
        initV(z, H_G, n);
        for (L i = 0; i < n; i++) CHECKE(foo(vV(z, i), x, vV(y, i)));
        R 0;
    }
    R foo(z, x, y);
}

/* pfnRaze: h_primitive.cc:935-955 with getCommonType/fillRaze
 * (h_system.cc:358-420): the items' common (max real) type, concatenated. */
static I raze_type(V x, I *typ, L *len) {
    if (vp(x) == H_G) { for (L i = 0; i < vn(x); i++) CHECKE(raze_type(vV(x, i), typ, len)); R 0; }
    if (*typ == -1) *typ = vp(x);
    else if (*typ != vp(x)) {
        if (hgo_is_real(*typ) && hgo_is_real(vp(x))) *typ = MAX(*typ, vp(x));
        else R E_RAZE_LIST;
    }
    *len += vn(x);
    R 0;
}
static void raze_fill(V z, L *n, V x) {
    if (vp(x) == H_G) { for (L i = 0; i < vn(x); i++) raze_fill(z, n, vV(x, i)); R; }
    for (L i = 0; i < vn(x); i++) {
        E v = 0; L iv = 0; B isf = vp(x) == H_F || vp(x) == H_E;
        switch (vp(x)) {
        case H_B: iv = sB(x)[i]; break; case H_J: iv = sJ(x)[i]; break; case H_H: iv = sH(x)[i]; break;
        case H_I: iv = sI(x)[i]; break; case H_L: iv = sL(x)[i]; break;
        case H_F: v = sF(x)[i]; break; case H_E: v = sE(x)[i]; break;
        default: memcpy(vg(z) + (*n) * getTypeSize(vp(z), 1), vg(x) + i * getTypeSize(vp(x), 1), (size_t)getTypeSize(vp(x), 1)); (*n)++; continue;
        }
        switch (vp(z)) {
        case H_B: sB(z)[*n] = (B)iv; break; case H_J: sJ(z)[*n] = (J)iv; break; case H_H: sH(z)[*n] = (H)iv; break;
        case H_I: sI(z)[*n] = (I)iv; break; case H_L: sL(z)[*n] = iv; break;
        case H_F: sF(z)[*n] = isf ? (F)v : (F)iv; break; case H_E: sE(z)[*n] = isf ? v : (E)iv; break;
        }
        (*n)++;
    }
}
I pfnRaze(V z, V x) {
    if (vp(x) == H_G) {
        if (vn(x) == 0) R E_RAZE_LIST;  /* the reference exits (EP, :938) */
        I typ = -1; L len = 0, n = 0;
        CHECKE(raze_type(x, &typ, &len));
        initV(z, typ, len);
        raze_fill(z, &n, x);
        R n == len ? 0 : E_UNKNOWN;
    }
    if (hgo_is_basic(vp(x))) R hgo_copyV(z, x);
    R E_DOMAIN;
}

/* Fused segmented reductions: the interpreter's
 * raze(each(@agg, each_right(@index, x, groups))) evaluated group by group
 * (pattern.cc:63-105 describes the chain; the per-group semantics are pfnIndex
 * followed by pfnSum/pfnAvg/pfnReduce/pfnLen). */
static I group_agg(V z, V x, V y, int kind) {
    if (vp(y) != H_G) R E_DOMAIN;
    L ng = vn(y);
    V0 each;
    initV(&each, H_G, ng);
    for (L g = 0; g < ng; g++) {
        V0 t;
        CHECKE(pfnIndex(&t, x, vV(y, g)));
        switch (kind) {
        case 0: CHECKE(pfnSum(vV(&each, g), &t)); break;
        case 1: CHECKE(pfnAvg(vV(&each, g), &t)); break;
        case 2: CHECKE(pfnReduce(vV(&each, g), &t, 0)); break;
        case 3: CHECKE(pfnReduce(vV(&each, g), &t, 1)); break;
        case 4: CHECKE(pfnLen(vV(&each, g), &t)); break;
        }
        V e = vV(&each, g);
        if (vn(e) <= 1 && hgo_is_basic(vp(e))) e->g = (G)&e->b;
    }
    if (ng == 0) {
        I typ = kind == 4 ? H_L : kind == 1 ? (vp(x) == H_F ? H_F : H_E)
              : kind == 0 ? (vp(x) == H_F ? H_F : vp(x) == H_E ? H_E : H_L) : vp(x);
        initV(z, typ, 0);
        R 0;
    }
    R pfnRaze(z, &each);
}
I hgpuGroupSum(V z, V x, V y) { R group_agg(z, x, y, 0); }
I hgpuGroupAvg(V z, V x, V y) { R group_agg(z, x, y, 1); }
I hgpuGroupMin(V z, V x, V y) { R group_agg(z, x, y, 2); }
I hgpuGroupMax(V z, V x, V y) { R group_agg(z, x, y, 3); }
I hgpuGroupLen(V z, V x, V y) { R group_agg(z, x, y, 4); }

/* Multi-column compress sharing one mask (pattern.cc:482-520): each y[k]
 * compressed by x, exactly as n separate pfnCompress calls. */
I hgpuCompressMany(V *z, V x, V *y, L n) {
    for (L k = 0; k < n; k++) CHECKE(pfnCompress(z[k], x, y[k]));
    R 0;
}

/* Several columns gathered by one index (pattern.cc:558-672, the generated
 * qN_patternindex_K): exactly n separate pfnIndex calls. */
I hgpuIndexMany(V *z, V *x, V y, L n) {
    for (L k = 0; k < n; k++) CHECKE(pfnIndex(z[k], x[k], y));
    R 0;
}

/* ------------------------------------------------ fixed-order tile tree sum */
/* Restatement of libhgpu's deterministic summation order for segmented
 * (per-group) sums, for bit-exact checks (the reference's own order depends on the
 * OpenMP thread count, so against it sums agree within a tolerance only):
 * chunks of 4096 elements; lane t (0..255) adds e[t], e[t+256], ... from
 * +0.0; each 32-lane group folds by a xor butterfly (offsets 16,8,4,2,1);
 * the 8 group sums combine as ((w0+w1)+(w2+w3))+((w4+w5)+(w6+w7)); chunk
 * partials are reduced again the same way until one value is left. */
static E tile_tree_f64(const E *x, L n) {
    E lanes[256], ws[8];
    for (int t = 0; t < 256; t++) {
        E acc = 0.0;
        for (int k = 0; k < 16; k++) { L j = (L)k * 256 + t; if (j < n) acc = acc + x[j]; }
        lanes[t] = acc;
    }
    for (int w = 0; w < 8; w++) {
        E v[32];
        for (int l = 0; l < 32; l++) v[l] = lanes[w * 32 + l];
        for (int o = 16; o > 0; o >>= 1) {
            E nv[32];
            for (int l = 0; l < 32; l++) nv[l] = v[l] + v[l ^ o];
            memcpy(v, nv, sizeof v);
        }
        ws[w] = v[0];
    }
    return ((ws[0] + ws[1]) + (ws[2] + ws[3])) + ((ws[4] + ws[5]) + (ws[6] + ws[7]));
}
/* libhgpu's f64 @sum/@avg: each 4096-element tile summed exactly in fixed
 * point and rounded once, tile partials summed the same way until one value
 * is left.  Restated from the definition: E = the largest biased exponent of
 * the tile's finite elements (at least 1), F = min(62, E - 1), unit
 * 2^(E - 1075 - F); each element's magnitude m * 2^(e - 1075) (subnormals at
 * e = 1) is floor(m * 2^(e - E + F)) units with its sign; the signed total is
 * rounded to nearest, ties to even.  NaN, or +inf with -inf, gives the quiet
 * NaN 0x7ff8...; one kind of infinity gives itself. */
static E u64_as_f64(unsigned long long b) { E d; memcpy(&d, &b, 8); return d; }
static unsigned long long f64_bits(E d) { unsigned long long b; memcpy(&b, &d, 8); return b; }

static E fixed_round(__int128 total, int unit_exp) {
    int neg = total < 0;
    unsigned __int128 mag = neg ? (unsigned __int128)(-total) : (unsigned __int128)total;
    if (mag == 0) return 0.0;
    int p = 127;
    while (!((mag >> p) & 1)) p--;
    /* value = mag * 2^unit_exp; normal iff p + unit_exp >= -1022 */
    unsigned long long bits;
    if (p + unit_exp < -1022) {
        bits = (unsigned long long)(mag << (unit_exp + 1074)); /* exact: a multiple of 2^-1074 */
    } else {
        int drop = p - 52, ex = p + unit_exp;
        unsigned __int128 sig = drop > 0 ? mag >> drop : mag << -drop;
        if (drop > 0) {
            unsigned __int128 rem = mag - (sig << drop), half = (unsigned __int128)1 << (drop - 1);
            if (rem > half || (rem == half && (sig & 1))) sig++;
            if (sig >> 53) { sig >>= 1; ex++; }
        }
        if (ex > 1023) bits = 0x7ff0000000000000ull;
        else bits = ((unsigned long long)(ex + 1023) << 52) | ((unsigned long long)sig & 0xfffffffffffffull);
    }
    return u64_as_f64(bits | ((unsigned long long)neg << 63));
}

static E tile_fixed_f64(const E *x, L n) {
    int E_ = 1, nan = 0, pinf = 0, ninf = 0;
    for (L i = 0; i < n; i++) {
        unsigned long long b = f64_bits(x[i]);
        int e = (int)((b >> 52) & 0x7ff);
        if (e == 0x7ff) { if (b & 0xfffffffffffffull) nan = 1; else if (b >> 63) ninf = 1; else pinf = 1; }
        else if (e > E_) E_ = e;
    }
    if (nan || (pinf && ninf)) return u64_as_f64(0x7ff8000000000000ull);
    if (pinf) return u64_as_f64(0x7ff0000000000000ull);
    if (ninf) return u64_as_f64(0xfff0000000000000ull);
    int F = E_ - 1 < 62 ? E_ - 1 : 62;
    __int128 total = 0;
    for (L i = 0; i < n; i++) {
        unsigned long long b = f64_bits(x[i]);
        int e = (int)((b >> 52) & 0x7ff);
        unsigned __int128 m = (b & 0xfffffffffffffull) | (e ? 1ull << 52 : 0);
        int k = F - E_ + (e > 1 ? e : 1);
        unsigned __int128 units = k >= 0 ? m << k : (k > -128 ? m >> -k : 0);
        total += (b >> 63) ? -(__int128)units : (__int128)units;
    }
    return fixed_round(total, E_ - 1075 - F);
}

E hgoFixedSumF64(const E *x, L n) {
    if (n <= 4096) return n ? tile_fixed_f64(x, n) : 0.0;
    L m = (n + 4095) / 4096;
    E *p = malloc(sizeof(E) * m);
    for (L c = 0; c < m; c++) p[c] = tile_fixed_f64(x + c * 4096, (n - c * 4096) < 4096 ? (n - c * 4096) : 4096);
    E r = hgoFixedSumF64(p, m);
    free(p);
    return r;
}

E hgoTreeSumF64(const E *x, L n) {
    if (n <= 4096) return tile_tree_f64(x, n);
    L m = (n + 4095) / 4096;
    E *p = malloc(sizeof(E) * m);
    for (L c = 0; c < m; c++) p[c] = tile_tree_f64(x + c * 4096, (n - c * 4096) < 4096 ? (n - c * 4096) : 4096);
    E r = hgoTreeSumF64(p, m);
    free(p);
    return r;
}

/* hgoTreeSumF64 per group: out[g] = the fixed-order tile-tree sum of
 * x[perm[starts[g]]], ..., x[perm[starts[g+1] - 1]] (starts[ng] = n), the
 * order every segmented sum of the GPU library follows.  Groups are
 * independent, so they run as OpenMP iterations. */
void hgoSegTreeSumF64(const E *x, const L *perm, const L *starts, L ng, L n, E *out) {
#pragma omp parallel
    {
        L cap = 4096;
        E *buf = malloc(sizeof(E) * cap);
#pragma omp for schedule(dynamic, 1024)
        for (L g = 0; g < ng; g++) {
            L a = starts[g], b = g + 1 < ng ? starts[g + 1] : n;
            if (b - a > cap) { cap = b - a; buf = realloc(buf, sizeof(E) * cap); }
            for (L k = a; k < b; k++) buf[k - a] = x[perm[k]];
            out[g] = hgoTreeSumF64(buf, b - a);
        }
        free(buf);
    }
}
