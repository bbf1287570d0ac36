/*
 * hgo_sort.c — CPU oracle: radix sorts, merge sort, the reference quicksort,
 * @group and @order.
 *
 * THIS IS TEST INFRASTRUCTURE, NOT THE PRODUCT (see hgo.h).  These
 * restatements reproduce the reference's exact output permutations,
 * including its unstable quicksort (h_libs.cc:409-442) and the char sort of
 * fewer than ten rows (h_libs.cc:388-390, which orders them descending), so
 * the GPU library's bit-exact and partition-equivalent claims can both be
 * checked against them.
 */
#include "hgo.h"

static I hgo_sort_err = 0;  /* set by void helpers on undefined reference behaviour */

/* ------------------------------------------------------------ comparators */
/* lib_quicksort_cmp_item: h_libs.cc:455-488 (SORT_MERGE undefined: ties -> 0) */
L hgo_cmp_item(V t, L a, L b, B *isUp) {
    B f = isUp ? *isUp : 1;
#define CMP_T(sX) if (sX(t)[a] != sX(t)[b]) R sX(t)[a] < sX(t)[b] ? (f ? -1 : 1) : (f ? 1 : -1); break
    switch (vp(t)) {
    case H_B: CMP_T(sB);
    case H_J: CMP_T(sJ);
    case H_H: CMP_T(sH);
    case H_I: case H_M: case H_D: case H_U: case H_W: case H_T: CMP_T(sI);
    case H_L: case H_Z: CMP_T(sL);
    case H_F: CMP_T(sF);
    case H_E: CMP_T(sE);
    case H_C: { int8_t *s = (int8_t *)vg(t); if (s[a] != s[b]) R s[a] < s[b] ? (f ? -1 : 1) : (f ? 1 : -1); } break;
    default: hgo_sort_err = E_NOT_IMPL; break;
    }
#undef CMP_T
    R 0;
}

/* lib_quicksort_cmp: h_libs.cc:449-453 */
L hgo_cmp_list(V val, L a, L b, B *isUp) {
    for (L i = 0; i < vn(val); i++) {
        B f = isUp ? isUp[i] : 1;
        L x = hgo_cmp_item(vV(val, i), a, b, &f);
        if (x != 0) R x;
    }
    R 0;
}

typedef L (*CmpFn)(V, L, L, B *);

/* ------------------------------------------------------------ radix sorts */
/* lib_radixsort_core_int: h_libs.cc:1184-1207 — four stable LSD passes over the
 * unsigned bytes of the 32-bit pattern. */
static void radix_core_int(I *kx, L *ki, L len) {
    L cnt[256];
    I *tx = malloc(sizeof(I) * (len > 0 ? len : 1));
    L *ti = malloc(sizeof(L) * (len > 0 ? len : 1));
    for (int j = 0; j < 32; j += 8) {
        memset(cnt, 0, sizeof(cnt));
        for (L i = 0; i < len; i++) cnt[((uint32_t)kx[i] >> j) & 255]++;
        for (int i = 1; i < 256; i++) cnt[i] += cnt[i - 1];
        for (L i = len - 1; i >= 0; i--) { L k = ((uint32_t)kx[i] >> j) & 255; L p = --cnt[k]; tx[p] = kx[i]; ti[p] = ki[i]; }
        memcpy(kx, tx, sizeof(I) * len); memcpy(ki, ti, sizeof(L) * len);
    }
    free(tx); free(ti);
}

/* lib_radixsort_core_long: h_libs.cc:1243-1274 — 32 bits unless some key has
 * (key >> 32) > 0, then 64; digits are unsigned bytes. */
static void radix_core_long(L *kx, L *ki, L len) {
    L cnt[256];
    int maxSize = 32;
    for (L i = 0; i < len; i++) if ((kx[i] >> 32) > 0) { maxSize = 64; break; }
    L *tx = malloc(sizeof(L) * (len > 0 ? len : 1));
    L *ti = malloc(sizeof(L) * (len > 0 ? len : 1));
    for (int j = 0; j < maxSize; j += 8) {
        memset(cnt, 0, sizeof(cnt));
        for (L i = 0; i < len; i++) cnt[((uint64_t)kx[i] >> j) & 255]++;
        for (int i = 1; i < 256; i++) cnt[i] += cnt[i - 1];
        for (L i = len - 1; i >= 0; i--) { L k = ((uint64_t)kx[i] >> j) & 255; L p = --cnt[k]; tx[p] = kx[i]; ti[p] = ki[i]; }
        memcpy(kx, tx, sizeof(L) * len); memcpy(ki, ti, sizeof(L) * len);
    }
    free(tx); free(ti);
}

/* lib_radixsort_int / lib_radixsort_long (h_libs.cc:1215-1240, 1276-1293),
 * returning indices; descending is the ascending result reversed. */
static void radixsort_int(L *rtn, V val, L len, B *isUp) {
    B f0 = isUp ? *isUp : 1;
    I *kx = malloc(sizeof(I) * (len > 0 ? len : 1));
    L *ki = malloc(sizeof(L) * (len > 0 ? len : 1));
    for (L i = 0; i < len; i++) { kx[i] = sI(val)[i]; ki[i] = i; }
    radix_core_int(kx, ki, len);
    if (f0) for (L i = 0; i < len; i++) rtn[i] = ki[i];
    else for (L i = 0; i < len; i++) rtn[i] = ki[len - i - 1];
    free(kx); free(ki);
}
static void radixsort_long_keys(L *rtn, L *keys, L len, B f0) {
    L *kx = malloc(sizeof(L) * (len > 0 ? len : 1));
    L *ki = malloc(sizeof(L) * (len > 0 ? len : 1));
    for (L i = 0; i < len; i++) { kx[i] = keys[i]; ki[i] = i; }
    radix_core_long(kx, ki, len);
    if (f0) for (L i = 0; i < len; i++) rtn[i] = ki[i];
    else for (L i = 0; i < len; i++) rtn[i] = ki[len - i - 1];
    free(kx); free(ki);
}

/* ------------------------------------------------------- comparison sorts */
/* lib_quicksort_char: h_libs.cc:386-407.  Fewer than ten rows go through the
 * all-pairs exchange at :388-390, which leaves them in DESCENDING byte order;
 * longer ranges use a stable counting sort.  The descending reversal at
 * :402-404 indexes past the range (rtn[high-i+1]) and is not restated: it
 * sets E_NOT_IMPL.  Bytes index the count table as unsigned (the reference
 * indexes with a signed char, undefined for bytes >= 128). */
static void quicksort_char(L *rtn, V val, L low, L high, B *isUp) {
    int8_t *str = (int8_t *)vg(val);
    L len = high - low;
    B f0 = isUp ? *isUp : 1;
    if (len < 10) {
        for (L i = low; i < high; i++)
            for (L j = low; j < high; j++)
                if (str[rtn[i]] > str[rtn[j]]) { L t = rtn[i]; rtn[i] = rtn[j]; rtn[j] = t; }
    } else {
        L cnt[256] = {0}, step[256] = {0}, cursor = 0;
        L *temp = malloc(sizeof(L) * len);
        for (L i = low; i < high; i++) cnt[(uint8_t)str[rtn[i]]]++;
        for (int i = 0; i < 256; i++) { if (cnt[i] != 0) step[i] = cursor; cursor += cnt[i]; }
        for (L i = low; i < high; i++) temp[step[(uint8_t)str[rtn[i]]]++] = rtn[i];
        memcpy(rtn + low, temp, sizeof(L) * len);
        free(temp);
    }
    if (!f0) hgo_sort_err = E_NOT_IMPL;
}

/* lib_partition / lib_quicksort_other: h_libs.cc:409-442 (the second
 * recursive call is a loop here; the visiting order is unchanged). */
static L partition(L *rtn, V val, L low, L high, B *isUp, CmpFn cmp, B *leftSame) {
    L pivot = low, i = low, j = high, t;
    for (;;) {
        while (++i && i < high) {
            L temp = cmp(val, rtn[i], rtn[pivot], isUp);
            if (temp != 0) *leftSame = 0;
            if (temp > 0) break;
        }
        do { --j; } while (j >= 0 && (cmp(val, rtn[j], rtn[pivot], isUp) > 0));
        if (i >= j) break;
        t = rtn[i]; rtn[i] = rtn[j]; rtn[j] = t;
    }
    if (!(*leftSame)) { t = rtn[low]; rtn[low] = rtn[j]; rtn[j] = t; }
    R j;
}
static void quicksort_other(L *rtn, V val, L low, L high, B *isUp, CmpFn cmp) {
    while (low < high) {
        B leftSame = 1;
        L pos = partition(rtn, val, low, high, isUp, cmp, &leftSame);
        if (!leftSame) quicksort_other(rtn, val, low, pos, isUp, cmp);
        if (pos < high) low = pos + 1; else break;
    }
}

/* lib_quicksort: h_libs.cc:375-384 */
static void quicksort_dispatch(L *rtn, V val, L low, L high, B *isUp, CmpFn cmp) {
    switch (vp(val)) {
    case H_C: quicksort_char(rtn, val, low, high, isUp); break;
    case H_I: radixsort_int(rtn, val, high, isUp); break;
    case H_L: { B f0 = isUp ? *isUp : 1; radixsort_long_keys(rtn, sL(val), high, f0); } break;
    default: quicksort_other(rtn, val, low, high, isUp, cmp); break;
    }
}

/* lib_mergesort: h_libs.cc:490-536 (stable top-down merge; the two-element
 * case swaps only on a strict inversion).  The merge of [low, high) uses
 * merge_buf[low, high) (the reference uses LARGE_BUFF from 0; the output is the
 * same), so the two halves of a large range can sort as parallel OpenMP tasks
 * with the same result.  merge_buf holds one slot per row of the column and is
 * allocated once per @order (the reference mallocs LARGE_BUFF per range). */
static L *merge_buf;
static void mergesort_rec(L *rtn, V val, L low, L high, B *isUp, CmpFn cmp) {
    if (low < high - 1) {
        if (low + 1 == high - 1) {
            if (cmp(val, rtn[low], rtn[high - 1], isUp) > 0) { L t = rtn[low]; rtn[low] = rtn[high - 1]; rtn[high - 1] = t; }
        } else {
            L mid = (low + high) >> 1, len = high - low;
            if (len > (1 << 16)) {
#pragma omp task default(shared) firstprivate(low, mid)
                mergesort_rec(rtn, val, low, mid, isUp, cmp);
                mergesort_rec(rtn, val, mid, high, isUp, cmp);
#pragma omp taskwait
            } else {
                mergesort_rec(rtn, val, low, mid, isUp, cmp);
                mergesort_rec(rtn, val, mid, high, isUp, cmp);
            }
            if (cmp(val, rtn[mid - 1], rtn[mid], isUp) > 0) {
                L cl = low, cr = mid, *buf = merge_buf + low;
                for (L i = 0; i < len; i++) {
                    if (cl == mid) buf[i] = rtn[cr++];
                    else if (cr == high) buf[i] = rtn[cl++];
                    else if (cmp(val, rtn[cl], rtn[cr], isUp) > 0) buf[i] = rtn[cr++];
                    else buf[i] = rtn[cl++];
                }
                memcpy(rtn + low, buf, sizeof(L) * len);
            }
        }
    }
}
static void mergesort_top(L *rtn, V val, L low, L high, B *isUp, CmpFn cmp) {
    if (high - low > (1 << 16)) {
#pragma omp parallel
#pragma omp single
        mergesort_rec(rtn, val, low, high, isUp, cmp);
    } else mergesort_rec(rtn, val, low, high, isUp, cmp);
}

/* lib_order_by_sorted: h_libs.cc:604-617 — an already ordered range is kept;
 * for a descending request, a range that is ascending is reversed. */
static B order_by_sorted(L *targ, V val, B *isUp, L low, L high, CmpFn cmp) {
    L rtn = 0;
    for (L i = low + 1; i < high; i++) {
        L t = cmp(val, targ[i - 1], targ[i], isUp);
        rtn = rtn == 0 ? t : rtn == -1 ? (t == 1 ? -2 : rtn) : (t == -1 ? -2 : rtn);
        if (rtn == -2) R 0;
    }
    B isOrder = rtn == (*isUp ? -1 : 1);
    if (isOrder && !(*isUp)) {
        for (L i = low; i < (low + high) / 2; i++) { L pos = high - (i - low) - 1, t = targ[i]; targ[i] = targ[pos]; targ[pos] = t; }
    }
    R isOrder;
}

/* lib_quicksort_list: h_libs.cc:637-697 — sort the range on column colId
 * (merge sort for i32/i64 columns, lib_quicksort otherwise), then recurse on
 * each run of equal values with the next column.  The run search of
 * :667-694 (a short scan, then a binary search over the sorted range) is
 * restated as a linear scan, which finds the same run ends. */
static void quicksort_list(L *targ, V val, B *isUp, L low, L high, L colId) {
    if (colId >= vn(val)) R;
    V curV = vV(val, colId);
    B *curB = isUp + colId;
    if (!order_by_sorted(targ, curV, curB, low, high, hgo_cmp_item)) {
        if (vp(curV) == H_I || vp(curV) == H_L) mergesort_top(targ, curV, low, high, curB, hgo_cmp_item);
        else quicksort_dispatch(targ, curV, low, high, curB, hgo_cmp_item);
    }
    L pos = low;
    while (pos < high) {
        L end = pos + 1;
        while (end < high && hgo_cmp_item(curV, targ[end - 1], targ[end], curB) == 0) end++;
        quicksort_list(targ, val, isUp, pos, end, colId + 1);
        pos = end;
    }
}

/* ------------------------------------------------------------ dict output */
/* lib_get_group_by_other / _order: h_libs.cc:776-848 — runs of equal rows in
 * `index` order become groups; the key is the run's first row. */
static I group_by_index(V z, V val, L *index, L iLen, CmpFn cmp) {
    L lenZ = iLen > 0 ? 1 : 0;
#define IX(i) (index ? index[i] : (i))
    for (L i = 1; i < iLen; i++) if (0 != cmp(val, IX(i - 1), IX(i), NULL)) lenZ++;
    initV(z, H_N, 2);
    V zKey = vV(z, 0), zVal = vV(z, 1);
    initV(zKey, H_L, lenZ);
    initV(zVal, H_G, lenZ);
    L g = 0, start = 0;
    for (L i = 1; i <= iLen; i++) {
        if (i == iLen || 0 != cmp(val, IX(i - 1), IX(i), NULL)) {
            V d = vV(zVal, g);
            initV(d, H_L, i - start);
            for (L k = start; k < i; k++) sL(d)[k - start] = IX(k);
            sL(zKey)[g] = IX(start);
            g++;
            start = i;
        }
    }
#undef IX
    R 0;
}

/* lib_group_by_normal_int / _long: h_libs.cc:1295-1329, 1369-1403 — radix
 * order, groups split where adjacent sorted values differ. */
static I group_by_sorted(V z, L *sortedVal, L *sortedIdx, L n) {
    L lenZ = n > 0 ? 1 : 0;
    for (L i = 1; i < n; i++) if (sortedVal[i - 1] != sortedVal[i]) lenZ++;
    initV(z, H_N, 2);
    V zKey = vV(z, 0), zVal = vV(z, 1);
    initV(zKey, H_L, lenZ);
    initV(zVal, H_G, lenZ);
    L g = 0, start = 0;
    for (L i = 1; i <= n; i++) {
        if (i == n || sortedVal[i - 1] != sortedVal[i]) {
            V d = vV(zVal, g);
            initV(d, H_L, i - start);
            for (L k = start; k < i; k++) sL(d)[k - start] = sortedIdx[k];
            sL(zKey)[g] = sortedIdx[start];
            g++;
            start = i;
        }
    }
    R 0;
}
static I group_normal_int(V z, V x) {
    L n = vn(x);
    I *kx = malloc(sizeof(I) * (n > 0 ? n : 1));
    L *ki = malloc(sizeof(L) * (n > 0 ? n : 1)), *kv = malloc(sizeof(L) * (n > 0 ? n : 1));
    for (L i = 0; i < n; i++) { kx[i] = sI(x)[i]; ki[i] = i; }
    radix_core_int(kx, ki, n);
    for (L i = 0; i < n; i++) kv[i] = kx[i];
    I r = group_by_sorted(z, kv, ki, n);
    free(kx); free(ki); free(kv);
    R r;
}
static I group_normal_long(V z, V x) {
    L n = vn(x);
    L *kx = malloc(sizeof(L) * (n > 0 ? n : 1)), *ki = malloc(sizeof(L) * (n > 0 ? n : 1));
    for (L i = 0; i < n; i++) { kx[i] = sL(x)[i]; ki[i] = i; }
    radix_core_long(kx, ki, n);
    I r = group_by_sorted(z, kx, ki, n);
    free(kx); free(ki);
    R r;
}

/* pfnGroupTrie: h_primitive.cc:2656-2681 — counting on (c0<<8)+c1; groups in
 * ascending code order, rows ascending, key = first row.  Bytes are taken as
 * unsigned (the reference's signed-char code is undefined for bytes >= 128). */
I pfnGroupTrie(V z, V x) {
    V c0 = vV(x, 0), c1 = vV(x, 1);
    L n = vn(c0);
    L *charMap = calloc(65536, sizeof(L)), *charId = malloc(sizeof(L) * 65536);
    uint8_t *a = (uint8_t *)vg(c0), *b = (uint8_t *)vg(c1);
    for (L i = 0; i < n; i++) charMap[(a[i] << 8) + b[i]]++;
    L lenZ = 0;
    for (L i = 0; i < 65536; i++) if (charMap[i] != 0) charId[i] = lenZ++;
    initV(z, H_N, 2);
    V keys = vV(z, 0), vals = vV(z, 1);
    initV(vals, H_G, lenZ);
    L c = 0;
    for (L i = 0; i < 65536; i++) if (charMap[i] != 0) initV(vV(vals, c++), H_L, charMap[i]);
    L *count = calloc(lenZ > 0 ? lenZ : 1, sizeof(L));
    for (L i = 0; i < n; i++) { L id = charId[(a[i] << 8) + b[i]]; sL(vV(vals, id))[count[id]++] = i; }
    initV(keys, H_L, lenZ);
    for (L i = 0; i < lenZ; i++) sL(keys)[i] = sL(vV(vals, i))[0];
    free(count); free(charMap); free(charId);
    R 0;
}

/* checkOrderCase1: h_libs.cc:1912-1940 — two i32 columns with one direction:
 * pack ((i64)x0 << 32) | (i64)x1 (x1 sign-extended, as in the reference) and
 * radix sort the packed keys. */
static B order_case1(V z, V x, V f) {
    if (!(vn(x) == 2 && vp(vV(x, 0)) == H_I && vp(vV(x, 1)) == H_I && sB(f)[0] == sB(f)[1])) R 0;
    V x0 = vV(x, 0), x1 = vV(x, 1);
    L size = vn(x0);
    L *temp = malloc(sizeof(L) * (size > 0 ? size : 1));
    for (L i = 0; i < size; i++) temp[i] = (L)(((uint64_t)(L)sI(x0)[i] << 32) | (uint64_t)(L)sI(x1)[i]);
    initV(z, H_L, size);
    radixsort_long_keys(sL(z), temp, size, sB(f)[0]);
    free(temp);
    R 1;
}

/* lib_order_basic + lib_order_by_vector: h_primitive.cc:1760-1767, h_libs.cc:730-736 */
static I order_basic(V z, V x, V y) {
    if (hgo_is_basic(vp(x)) && vp(y) == H_B && vn(y) == 1) {
        L n = vn(x);
        initV(z, H_L, n);
        L *t = sL(z);
        if (!(vp(x) == H_I || vp(x) == H_L)) for (L i = 0; i < n; i++) t[i] = i;
        hgo_sort_err = 0;
        quicksort_dispatch(t, x, 0, n, sB(y), hgo_cmp_item);
        R hgo_sort_err;
    }
    R 1;
}

/* pfnOrderBy: h_primitive.cc:1769-1816 */
I pfnOrderBy(V z, V x, V y) {
    if (vp(x) == H_G && vp(y) == H_B && vn(x) == vn(y)) {
        for (L i = 0; i < vn(x); i++) if (!hgo_is_basic(vp(vV(x, i)))) R E_DOMAIN;
        if (order_case1(z, x, y)) R 0;
        if (vn(x) == 1) R order_basic(z, vV(x, 0), y);
        L lenZ = vn(x) == 0 ? 0 : vn(vV(x, 0));
        initV(z, H_L, lenZ);
        hgo_sort_err = 0;
        for (L i = 0; i < lenZ; i++) sL(z)[i] = i;
        merge_buf = malloc(sizeof(L) * (lenZ > 0 ? lenZ : 1));
        quicksort_list(sL(z), x, sB(y), 0, lenZ, 0);
        free(merge_buf);
        merge_buf = NULL;
        R hgo_sort_err;
    }
    R order_basic(z, x, y);
}

/* pfnGroupBasic: h_primitive.cc:1002-1057 */
I pfnGroupBasic(V z, V x) {
    L lenZ = vp(x) == H_G ? vn(x) : 1;
    L *order_list = NULL;
    V0 t;
    if (hgo_is_ordered(x) || vp(x) == H_I || vp(x) == H_L) order_list = NULL;
    else {
        V0 y;
        initV(&y, H_B, lenZ);
        for (L i = 0; i < lenZ; i++) sB(&y)[i] = 1;
        CHECKE(pfnOrderBy(&t, x, &y));
        order_list = sL(&t);
    }
    if (vp(x) == H_G) {
        L numRow = vn(x) == 0 ? 0 : vn(vV(x, 0));
        R group_by_index(z, x, order_list, numRow, hgo_cmp_list);
    }
    if (vp(x) == H_I) R group_normal_int(z, x);
    if (vp(x) == H_L) R group_normal_long(z, x);
    if (hgo_is_basic(vp(x))) R group_by_index(z, x, order_list, vn(x), hgo_cmp_item);
    R E_DOMAIN;
}

/* pfnGroup: h_primitive.cc:992-999 (isGroupTrie: two equal-length char columns) */
I pfnGroup(V z, V x) {
    if (vp(x) == H_G && vn(x) == 2 && vp(vV(x, 0)) == H_C && vp(vV(x, 1)) == H_C && vn(vV(x, 0)) == vn(vV(x, 1)))
        R pfnGroupTrie(z, x);
    R pfnGroupBasic(z, x);
}
