/*
 * hgo.h — internal header of the CPU oracle (test infrastructure).
 *
 * THIS IS TEST INFRASTRUCTURE, NOT THE PRODUCT.  liboracle.so is a CPU
 * restatement, in plain C with OpenMP, of the HorsePower builtin algorithms
 * on the accelerated path.  It exports the same C ABI as the product
 * (include/hgpu.h), so the tests can drive the reference library, this
 * oracle and the GPU library through one harness.  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg may load it.
 *
 * Each function cites the reference file:line it restates (paths relative to
 * the HorsePower tree, src/horseir/v3/...).  Behaviour that is undefined in
 * the reference (out-of-bounds reads, exit() on unsupported types) is
 * replaced by an error return and listed in the function's comment.
 */
#ifndef HGO_H
#define HGO_H
#include "hgpu.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include <float.h>
#include <math.h>
#include <omp.h>

#define R return
#define MIN(a, b) (((a) < (b)) ? (a) : (b))
#define MAX(a, b) (((a) > (b)) ? (a) : (b))

#define vp(x) ((x)->typ)
#define vn(x) ((x)->len)
#define vg(x) ((x)->g)
#define sB(x) ((B *)vg(x))
#define sJ(x) ((J *)vg(x))
#define sH(x) ((H *)vg(x))
#define sI(x) ((I *)vg(x))
#define sL(x) ((L *)vg(x))
#define sF(x) ((F *)vg(x))
#define sE(x) ((E *)vg(x))
#define sC(x) ((C *)vg(x))
#define sV(x) ((V)vg(x))
#define vV(x, k) (sV(x) + (k))

#define CHECKE(e) do { I e_ = (e); if (e_) R e_; } while (0)

extern L hgo_cores;        /* H_CORE: h_system.cc:14-24 */
extern const E H_EPSILON;  /* h_system.cc:9 */

G    hgo_alloc(L bytes);   /* arena allocation, 16-byte rounded: h_memory.cc:93-112 */
B    hgo_is_int(I t);      /* isTypeGroupInt:   h_system.cc:922-924 */
B    hgo_is_float(I t);    /* isTypeGroupFloat: h_system.cc:926-928 */
B    hgo_is_real(I t);     /* isTypeGroupReal:  h_system.cc:930-932 */
B    hgo_is_basic(I t);    /* isTypeGroupBasic: h_system.cc:967-969 */
I    hgo_promote(V z, V x, I typMax);   /* promoteValueWithIndex(.., NULL): h_system.cc:168-252 */
B    hgo_is_ordered(V x);  /* isOrdered: h_system.cc:678-698 */
I    hgo_copyV(V z, V x);  /* copyV: h_system.cc:70-73 */
void hgo_swap2(V z);       /* swap2: h_system.cc:47-56 */

/* hgo_io.c: readCSV / serializeV / readSerializeV restated (h_io.cc) */
I    hgoReadCSV(V z, S fileName, L numCols, L *types, Q *symList);
I    hgoWriteSerialized(V x, FILE *fp);
I    hgoReadSerialized(V x, FILE *fp);

/* hgo_sort.c */
L    hgo_cmp_item(V t, L a, L b, B *isUp);   /* lib_quicksort_cmp_item: h_libs.cc:455-488 */
L    hgo_cmp_list(V val, L a, L b, B *isUp); /* lib_quicksort_cmp:      h_libs.cc:448-453 */

#endif
