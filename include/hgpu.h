/*
 * hgpu.h — C ABI of the GB300 HorseIR builtin library (libhgpu.so).
 *
 * libhgpu is a link-time drop-in for the builtin ("primitive") library of
 * HorsePower's HorseIR engine: it exports the same `I pfnXxx(V z, V x, ...)`
 * entry points over the same `V0` value node, so the interpreter
 * (src/horseir/v3/translator/interpreter.cc:42-60,278-294) and generated C
 * code (src/horseir/v3/translator/compiler.cc:338-368) can link against it in
 * place of libcore.a (src/horseir/v3/make.sh:30-43).
 *
 * Every declaration below cites the reference interface it replaces.  Paths
 * are relative to the HorsePower source tree.  Entry points prefixed `hgpu`
 * are extensions with no counterpart in the reference (device residency,
 * timing, fused chains, batched plans, serving).
 *
 * Conventions kept from the reference (src/horseir/v3/backend/h_primitive.cc:6-14):
 *   - z is allocated by the caller; the callee fills it (initV semantics).
 *   - return 0 on success or an E_* code; outputs may alias inputs.
 *   - vectors of length <= 1 store their element inline in the node
 *     (src/horseir/v3/backend/h_memory.cc:182-196).
 *
 * GB300 additions:
 *   - Vector payloads (`g`) may live in host memory or in HBM.  Inputs are
 *     accepted from either; outputs are placed according to the residency
 *     mode (hgpuSetResidency), HBM by default.  Node structs and list/dict
 *     node arrays always live in host memory so host code can walk them.
 *   - Device failures never exit(): they return E_DEVICE-class codes >= 100.
 */
#ifndef HGPU_H
#define HGPU_H

#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Scalar typedefs: src/horseir/v3/backend/common.h:9-22 */
typedef bool      B;
typedef char      C, *S, *G;
typedef int8_t    J;
typedef int16_t   H;
typedef int32_t   I, M, D, U, W, T;
typedef long long L, Q, Z;
typedef float     F;
typedef double    E;
typedef struct { F real, imag; } X;
/* Enum header: the reference's Y0 (common.h:19).  `source` names the enum's
 * table column (-1 for one made by pfnEnum), `ek` is the key node (the
 * primary-key column, a V stored as G) and `ev` the value node (the
 * foreign-key column).  An H_Y node holds the header in its union member `y`
 * and its i64 index into ek in `g`, always out of line (initV,
 * h_memory.cc:184-194). */
struct hgpu_enum_s { Q source; G ek, ev; };
typedef struct hgpu_enum_s Y0, *Y;
/* Table header: the reference's A0 (common.h:21): row and column counts and
 * its foreign-key list (always NULL here).  An H_A node holds it in `a` and
 * its two nodes {keys (symbols), values (list of columns)} in `g`. */
struct hgpu_table_s { L row, col; void *fkey; };
typedef struct hgpu_table_s A0, *A;

/* Value node: field order and union members of src/horseir/v3/backend/common.h:31-55.
 * sizeof(V0) == 32 on LP64. */
typedef struct NodeValue {
    L len; G g; I typ;
    union {
        B b; J j; H h; I i32; L i64; F f32; E f64; C c; Q q; S s;
        M m; D d; Z z; U u; W w; T t; X x;
        struct hgpu_enum_s *y; struct hgpu_table_s *a;
        struct NodeValue *g2;
    };
} V0, *V;

/* Type codes: src/horseir/v3/backend/h_type.h:1-23 */
#define H_B 0
#define H_J 1
#define H_H 2
#define H_I 3
#define H_L 4
#define H_F 5
#define H_E 6
#define H_X 7
#define H_C 8
#define H_Q 9
#define H_S 10
#define H_M 11
#define H_D 12
#define H_Z 13
#define H_U 14
#define H_W 15
#define H_T 16
#define H_G 17
#define H_N 18
#define H_Y 19
#define H_A 90
#define H_K 91
#define H_V 93

/* Error codes: src/horseir/v3/backend/h_system.h:128-142 */
#define E_DOMAIN          1
#define E_GENERAL         2
#define E_INDEX           3
#define E_DIV_ZERO        4
#define E_LENGTH          5
#define E_TYPE            6
#define E_NULL_VALUE      7
#define E_LIKE_PATTERN    8
#define E_MATCH           9
#define E_ENUM_INDEX      10
#define E_RAZE_LIST       11
#define E_UNKNOWN         12
#define E_TABLE_NOT_FOUND 50
#define E_COL_NOT_FOUND   51
#define E_NOT_IMPL        99
/* Extensions (no counterpart in the reference, which exit()s instead:
 * h_memory.cc:110,448, h_hash_v3.cc:27,259). */
#define E_DEVICE          100  /* a CUDA call failed; the library stays usable if the context does */
#define E_DEVICE_OOM      101  /* device or pinned-host arena exhausted */
#define E_DEVICE_TIMEOUT  102  /* a bounded device-side wait gave up (look-back, work queue) */
#define E_NO_DEVICE       103  /* no CUDA device / library not initialised */
#define E_ADMISSION       104  /* serving loop refused a request (footprint larger than the pool) */
#define E_CANCELLED       105  /* serving loop request cancelled before it ran */

/* ---------------- memory / values (src/horseir/v3/backend/h_memory.h:21-45) -------------- */
/* initBackend: src/horseir/v3/global.cc:26-35 (arena + symbols + cores).  Also creates the
 * CUDA context, library stream and arenas; safe to call more than once. */
void initBackend(void);
V    allocNode(void);                       /* h_memory.cc:160-162 */
V    initV(V x, I typ, L len);              /* h_memory.cc:182-196 (payload in the output arena) */
L    getHeapOffset(void);                   /* h_memory.cc:155-157 (both output arenas, in 256-byte units) */
L    setHeapOffset(L cur);                  /* h_memory.cc:159-161 (rewinds device + host arenas) */
L    getTypeSize(I typ, L len);             /* h_memory.cc:124-153 */
/* Symbols: src/horseir/v3/backend/h_symbol.h:38-56 (interning used by @join_index's op list) */
L    getSymbol(S name);
S    getSymbolStr(L x);

/* ---------------- builtins on the accelerated path ---------------- */
/* Stream compaction */
I pfnCompress(V z, V x, V y);   /* h_primitive.cc:1479-1521 (@compress) */
I pfnWhere   (V z, V x);        /* h_primitive.cc:728-762  (@where) */
/* Elementwise compare (h_primitive.cc:1073-1200; float compares use eps=1e-13, h_system.cc:9) */
I pfnCompare(V z, V x, V y, I op);
I pfnLt (V z, V x, V y);
I pfnLeq(V z, V x, V y);
I pfnGt (V z, V x, V y);
I pfnGeq(V z, V x, V y);
I pfnEq (V z, V x, V y);
I pfnNeq(V z, V x, V y);
/* Elementwise arithmetic (h_primitive.cc:1227-1309) */
I pfnArith(V z, V x, V y, I op);
I pfnPlus (V z, V x, V y);
I pfnMinus(V z, V x, V y);
I pfnMul  (V z, V x, V y);
I pfnDiv  (V z, V x, V y);
/* Elementwise logic (h_primitive.cc:1315-1357, functions h_system.cc:898-916) */
I pfnAnd (V z, V x, V y);
I pfnNand(V z, V x, V y);
I pfnOr  (V z, V x, V y);
I pfnNor (V z, V x, V y);
I pfnXor (V z, V x, V y);
I pfnNot (V z, V x);            /* h_primitive.cc:606-615 */
/* Reductions (h_primitive.cc:764-847) */
I pfnSum(V z, V x);
I pfnAvg(V z, V x);
I pfnReduce(V z, V x, I op);
I pfnMin(V z, V x);
I pfnMax(V z, V x);
I pfnLen(V z, V x);             /* h_primitive.cc:656-662 */
/* Gather / search */
I pfnIndex  (V z, V x, V y);    /* h_primitive.cc:43-94 */
I pfnIndexOf(V z, V x, V y);    /* h_primitive.cc:1523-1579 (vectors, or two lists of integer columns) */
I pfnMember (V z, V y, V x);    /* h_primitive.cc:2287-2336 (note argument order) */
/* @like (h_primitive.cc:1670-1758): x chars / symbols / strings against one
 * SQL pattern y ('%' any run, '_' any byte; neither matches '\n', as the
 * reference's translated PCRE2 pattern); z bool, one per row (one for chars).
 * Patterns holding other regex metacharacters, and one pattern per row:
 * E_NOT_IMPL. */
I pfnLike   (V z, V x, V y);
/* Enum / foreign-key path: pfnEnum builds the enum of y (foreign-key column)
 * over x (primary-key column) as index_of(x, y), E_ENUM_INDEX when some y has
 * no key; pfnFetch returns y back.  pfnAddFKey (h_primitive.cc:2425-2466) is
 * pfnEnum over two table columns plus table metadata. */
I pfnEnum   (V z, V x, V y);    /* h_primitive.cc:2198-2222 */
I pfnFetch  (V z, V x);         /* h_primitive.cc:219-225 */
I pfnJoinIndex(V z, V x, V y, V f); /* h_primitive.cc:2122-2155; several columns: pfnJoinIndexMultiple :2094-2110 */
/* Grouping and ordering */
I pfnGroup    (V z, V x);       /* h_primitive.cc:993-999 */
I pfnGroupTrie(V z, V x);       /* h_primitive.cc:2656-2681 */
I pfnGroupBasic(V z, V x);      /* h_primitive.cc:1002-1057 */
I pfnOrderBy  (V z, V x, V y);  /* h_primitive.cc:1769-1816 */
/* List plumbing used by the segmented-reduction chain (each_right @index -> each @sum -> raze) */
I pfnList (V z, L n, V x[]);    /* h_primitive.cc:32-36 */
I pfnKeys (V z, V x);           /* h_primitive.cc:191-203 (dict, table, enum key) */
I pfnValues(V z, V x);          /* h_primitive.cc:205-217 (dict, table, enum index) */
I pfnEach     (V z, V x, I (*foo)(V, V));        /* h_primitive.cc:1818-1832 */
I pfnEachRight(V z, V x, V y, I (*foo)(V, V, V)); /* h_primitive.cc:1882-1904 */
I pfnRaze (V z, V x);           /* h_primitive.cc:935-955 */

/* ---------------- fused segmented reductions ----------------
 * GB300 counterparts of the peephole functions the pattern pass emits for
 * raze(each(@sum|@avg|@min|@max|@len, each_right(@index, x, groups)))
 * (src/horseir/v3/optimizer/pattern.cc:63-105 FP1/2/5/6/7, emitter :180-219),
 * same (V z, V x, V y) convention: x = column, y = list of i64 index vectors
 * (the values of a @group dict), z = one aggregate per group.  Aggregation
 * semantics follow the interpreter (pfnSum/pfnAvg/pfnReduce per group). */
I hgpuGroupSum(V z, V x, V y);
I hgpuGroupAvg(V z, V x, V y);
I hgpuGroupMin(V z, V x, V y);
I hgpuGroupMax(V z, V x, V y);
I hgpuGroupLen(V z, V x, V y);
/* Several aggregates over one grouping (no counterpart in the reference: the
 * common-index pattern, pattern.cc:558-672, applied to the segmented
 * reductions of pattern.cc:63-105).  z[k] = hgpuGroupSum / Avg / Min / Max /
 * Len (x[k], y) for aggs[k] = HGPU_AGG_SUM .. HGPU_AGG_LEN, bit for bit; f64
 * sums and averages over a @group whose groups are all longer than 4096 rows
 * read the groups' row ids once for all of them. */
#define HGPU_AGG_SUM 0
#define HGPU_AGG_AVG 1
#define HGPU_AGG_MIN 2
#define HGPU_AGG_MAX 3
#define HGPU_AGG_LEN 4
I hgpuGroupAggMany(V *z, V *x, V y, const I *aggs, L n);

/* ---------------- fused chains ----------------
 * GB300 counterpart of the fused loops emitted by the loop-fusion passes
 * (src/horseir/v3/optimizer/autofusion.cc:770-935 genCodeAuto,
 *  elementwise.cc:239-281 genCodeElem, pattern.cc:482-520 genPatternCompress),
 * called with the same `(V z, V *x)` / `(V *z, V x, V *y)` conventions.
 * A chain is described by a small text program (grammar in fused.cu) and
 * compiled once into a single kernel. */
typedef struct hgpu_chain_s *hgpuChain;
I hgpuChainCreate(hgpuChain *out, const char *program);
I hgpuChainRun(hgpuChain c, V z, V *x);           /* autofusion-style: inputs x[0..n) -> z */
I hgpuChainRunMany(hgpuChain c, V *z, V *x);      /* compress sinks: one output node per expression */
I hgpuChainDestroy(hgpuChain c);
/* Multi-column compress sharing one mask: pattern.cc:452-520 (V *z, V x, V *y) */
I hgpuCompressMany(V *z, V x, V *y, L n);
/* Several columns gathered by one index, the "common index" pattern:
 * pattern.cc:558-672 (genPatternIndex, `static I qN_patternindex_K(V *z, V *x,
 * V y)`).  z[k] = x[k][y] as n pfnIndex calls on basic-typed columns; any
 * index outside any column gives E_INDEX and no output. */
I hgpuIndexMany(V *z, V *x, V y, L n);

/* ---------------- batched plans ----------------
 * Many independent filter-join-aggregate queries run stage by stage in shared
 * launches (no counterpart in the reference, which runs one query at a time).
 * Each plan is the join + group-by query of plans.join_group: filter the
 * dimension on date in [lo, hi), join its pk to the fact fk, group the matches
 * on (flag, status) and aggregate sum(qty), avg(price), sum(disc), count.
 * Per-plan results are bit-identical to running the plan's builtins alone.
 * Columns must be device or pinned host memory. */
typedef struct {
    const I *dim_pk, *dim_date; L ndim;
    const I *fk; const C *flag, *status; const E *qty, *price, *disc; L nfact;
    I lo, hi;
} hgpuJoinGroupPlan;
#define HGPU_PLAN_MAX_GROUPS 256
typedef struct {
    I status;                         /* 0, or the error code of the plan's builtins */
    L ngroups;                        /* groups in ascending (flag<<8 | status) order */
    C flag[HGPU_PLAN_MAX_GROUPS], st[HGPU_PLAN_MAX_GROUPS];
    E sum_qty[HGPU_PLAN_MAX_GROUPS], avg_price[HGPU_PLAN_MAX_GROUPS], sum_disc[HGPU_PLAN_MAX_GROUPS];
    L count[HGPU_PLAN_MAX_GROUPS];
} hgpuJoinGroupResult;
I hgpuBatchJoinGroup(const hgpuJoinGroupPlan *plans, L nplans, hgpuJoinGroupResult *out);
/* Seeded synthetic join tables generated on the device (benchmarks): dim is
 * filled with a 2-node list (pk = a permutation of 0..ndim-1, date), fact with
 * a 6-node list (fk, flag, status, qty, price, disc). */
I hgpuSynthJoinTables(unsigned long long seed, L nfact, L ndim, V dim, V fact);
/* Seeded synthetic order table on the device: a 2-node list (key i64 Zipf(s)
 * over 1..nranks, sec i32 uniform over [0, 2^20]). */
I hgpuSynthOrderTable(unsigned long long seed, L n, L nranks, E s, V order);

/* ---------------- served form ----------------
 * A request loop over tables resident in HBM (no counterpart in the
 * reference).  Requests arrive over time; each step of the loop admits the
 * waiting requests in arrival order while their HBM footprints fit the
 * server's budget, runs them together (all filter-aggregates in one
 * shared-scan launch, all join + group-bys through hgpuBatchJoinGroup, the
 * top-k orders one after another), and stamps their completion.  Requests
 * that arrive while a step runs join the next one.  A request's result does
 * not depend on which other requests share its step. */
typedef struct {
    /* filter-aggregate table: q6-shaped lineitem columns */
    const I *l_shipdate, *l_qty; const E *l_disc, *l_price; L nline;
    /* join tables (as hgpuJoinGroupPlan) */
    const I *dim_pk, *dim_date; L ndim;
    const I *fk; const C *flag, *status; const E *qty, *price, *disc; L nfact;
    /* order table: i64 key, i32 secondary */
    const L *o_key; const I *o_sec; L norder;
} hgpuServeTables;
#define HGPU_REQ_FILTER_AGG 0   /* sum(price*disc) where shipdate in [lo,hi) and the q6 predicate */
#define HGPU_REQ_JOIN_GROUP 1   /* the hgpuJoinGroupPlan query with dim.date in [lo,hi) */
#define HGPU_REQ_TOPK_ORDER 2   /* first k rows of the stable ascending @order on (key, sec) among key in [klo,khi) */
#define HGPU_TOPK 1000
typedef struct {
    I kind;
    I lo, hi;                 /* date window */
    L klo, khi;               /* key range */
    double arrival_s;         /* seconds from the start of the stream; requests sorted by it */
} hgpuRequest;
typedef struct {
    I status;                 /* 0, E_ADMISSION (footprint above the budget) or a builtin's error */
    E value;                  /* filter-aggregate result */
    hgpuJoinGroupResult *group;  /* join + group-by result: caller-owned, may be NULL */
    L *rows;                  /* top-k row ids (caller-owned, HGPU_TOPK entries), may be NULL */
    L nrows;
    double admit_s, done_s;   /* seconds from the start of the stream */
    L step;                   /* loop step that ran the request */
    L footprint;              /* HBM bytes the request was admitted with */
} hgpuResponse;
typedef struct {
    L steps, rejected, max_step_requests;
    L max_step_bytes;         /* largest admitted footprint of one step */
    double wall_s, qps, p50_ms, p99_ms, mean_ms, max_ms;
} hgpuServeStats;
typedef struct hgpu_server_s *hgpuServer;
#define HGPU_SERVE_BATCHED 0  /* continuous batching (the served form) */
#define HGPU_SERVE_PLAIN   1  /* one request at a time through its builtins, in arrival order */
I hgpuServerCreate(hgpuServer *out, const hgpuServeTables *tables, L hbm_budget_bytes, L max_step_requests);
L hgpuServerFootprint(hgpuServer s, const hgpuRequest *r);   /* admission estimate, bytes */
I hgpuServerRun(hgpuServer s, const hgpuRequest *req, L n, hgpuResponse *out, I mode, hgpuServeStats *stats);
I hgpuServerDestroy(hgpuServer s);

/* ---------------- runtime extensions ---------------- */
#define HGPU_RESIDENT_DEVICE 0   /* outputs stay in HBM (default) */
#define HGPU_RESIDENT_HOST   1   /* outputs are copied to pinned host memory on return */
I    hgpuInit(L device_arena_bytes, L host_arena_bytes);
I    hgpuSetResidency(I mode);
I    hgpuGetResidency(void);
/* Deep copies: device->host (result usable by plain host code) and host->device. */
I    hgpuToHost(V z, V x);
I    hgpuToDevice(V z, V x);
I    hgpuIsDevice(V x);               /* 1 when x's payload lives in HBM */
/* Asynchronous upload of a vector: the copy runs on a second stream, and the
 * library stream waits for it only when a builtin first reads z (or at
 * hgpuWait(z), hgpuSync, setHeapOffset), so kernels on inputs already in HBM
 * overlap the copy.  x's host memory must stay unchanged until then.  The
 * batched and served entry points take device pointers: call hgpuWait on
 * their inputs first. */
I    hgpuToDeviceAsync(V z, V x);
I    hgpuWait(V z);
I    hgpuSync(void);                  /* wait for the library stream; returns sticky device errors */
void*hgpuStream(void);                /* the cudaStream_t every kernel is launched on */
const char *hgpuLastError(void);      /* text of the last error (thread-local) */
/* Deterministic reductions: 1 (default) = fixed-order tile tree, bit-exact run to run. */
I    hgpuSetReduceMode(I mode);
/* Kernel timing on the library stream (CUDA events around each launch when enabled). */
I    hgpuProfile(I enable);
I    hgpuProfileReset(void);
/* Returns the number of distinct kernels recorded; fills names/ms/launches up to cap. */
I    hgpuProfileRead(I cap, const char **names, double *total_ms, L *launches);
L    hgpuLaunchCount(void);           /* kernels launched by this library since load */
L    hgpuSyncCount(void);             /* waits of the host on the library stream since load */
/* Event timer on the library stream */
I    hgpuTimerStart(void);
double hgpuTimerStop(void);
/* Autotuner knobs.  None of them changes a result: every setting gives the
 * same bits (stable sorts, order-preserving compaction, fixed-order sums).
 * Values outside a knob's range are clamped; hgpuGetTuning returns the
 * value in force. */
#define HGPU_TUNE_HASH_LOAD  0   /* hash-table load factor, 0.5 - 0.8 (default 0.5) */
#define HGPU_TUNE_RADIX_BITS 1   /* LSD radix digit width of @group/@order, 4 - 8 bits (default 8) */
#define HGPU_TUNE_TILE_ROWS  2   /* probe rows per thread of the tiled join probes: 8, 16, 32
                                    (tile = 256 x that; default 8) */
#define HGPU_TUNE_L2_FETCH   3   /* largest L2 fetch from DRAM, bytes: 32, 64 or 128 (default 64;
                                    32 suits sparse sorted gathers, 64 random probes and scatters) */
#define HGPU_TUNE_JOIN_FILTER 4 /* @join_index presence bitmap on dense i32 keys: 0 read through L2
                                    (default), 1 held in the shared memory of a 16-CTA cluster */
#define HGPU_TUNE_RADIX_PASS 5  /* radix pass of @group/@order: 0 tile offsets by a decoupled look-back,
                                    1 by a counting pass and one scan before the scatter, 2 (default)
                                    1 for 32-bit keys and 0 for 64-bit ones */
I    hgpuSetTuning(I knob, E value);
E    hgpuGetTuning(I knob);

/* Self-test of the bounded device waits (no counterpart in the reference):
 * runs a four-tile look-back whose first tile never publishes, so the other
 * tiles' waits give up after `limit` polls (1 .. 2^20).  Returns
 * E_DEVICE_TIMEOUT, as any builtin whose wait gave up does, and leaves the
 * library usable.  mode 0: the scans' look-back; 1: the radix passes' chain
 * look-back.  Arena caps for out-of-memory handling come from the
 * environment at first use: HGPU_DEVICE_LIMIT_MB, HGPU_SCRATCH_LIMIT_MB,
 * HGPU_HOST_LIMIT_MB (a call that needs more returns E_DEVICE_OOM). */
I    hgpuSelfTestWait(I mode, L limit);

/* Allocation-free f64 sum (no counterpart in the reference).  For callers that
 * cannot allocate device memory where they need a sum: an engine that works in
 * a fixed device-memory budget reserved up front, or a path that cannot take
 * the synchronisation an allocation may cause.  Same
 * fixed-point tile sum as pfnSum on f64 data (the same bits).  x and result are
 * device pointers the caller owns; the tile partials live in a static device
 * array (~512 KiB, held by every GPU that loads the library), so the call
 * makes no cudaMalloc/cudaFree and uses no arena.  n is limited to
 * 268,435,456 (E_LENGTH beyond).  Calls share the array: calls overlapping
 * on the GPU race, so issue them on one stream.  The first call on a device
 * looks up the array's address.  A device reset (cudaDeviceReset) is not
 * supported afterwards. */
I    hgpuSumF64Static(const double *x, L n, double *result, void *stream);

/* ---------------- ingest: binary tables and CSV (h_io.cc) ----------------
 * The reference's table loaders with column payloads landing in HBM (or in
 * pinned host memory under HGPU_RESIDENT_HOST).
 *
 * Binary format (serializeV / readSerializeV, h_io.cc:626-772): each node is
 * its 32-byte V0 followed by its payload; basic vectors as raw elements (char
 * vectors with a trailing NUL), symbols and strings as len(x) i64 lengths
 * then NUL-terminated texts, lists and tables as their nodes in order (a
 * table writes its 24-byte A0 first).  Files written by either library read
 * back in the other.  Payloads stream through pinned staging buffers, the
 * file read of one chunk overlapping the host-to-device copy of the last.
 *
 * CSV (readCSV / loadCSV / getField / loadItem, h_io.cc:50-188): the file is
 * copied to HBM once; lines, fields and every column are parsed on the GPU
 * with the reference's conversions (atoi, atol, strtof, strtod bit-exact,
 * including the slow decimal cases; %d-%d-%d dates as yyyymmdd; first
 * character; symbols interned in first-occurrence order; strings copied to
 * pinned host memory).  LINE_SEP / LINE_HEADER / LINE_MAX_CHAR are the
 * reference's format globals (h_io.cc:8-11). */
I    hgpuWriteSerialized(V x, FILE *fp);   /* serializeV, h_io.cc:672-697 */
I    hgpuReadSerialized(V x, FILE *fp);    /* readSerializeV, h_io.cc:748-772 */
I    hgpuReadCSV(V z, S fileName, L numCols, L *types, Q *symList);  /* readCSV, h_io.cc:50-71 */
/* The reference's own entry points: like its EP, they print the error and
 * exit the process when the file cannot be read or parsed; a device failure
 * (E_DEVICE and above) is printed and kept for hgpuLastError without ending
 * the process (readCSV then returns NULL). */
void serializeV(V x, FILE *fp);
void readSerializeV(V x, FILE *fp);
V    readCSV(S fileName, L numCols, L *types, Q *symList);
extern C LINE_SEP;                         /* field separator, '|' (h_io.cc:9) */
extern B LINE_HEADER;                      /* true: the first line is skipped (h_io.cc:11) */
extern L LINE_MAX_CHAR;                    /* fgets buffer: lines of up to LINE_MAX_CHAR-1 characters (h_io.cc:8) */

#ifdef __cplusplus
}
#endif
#endif /* HGPU_H */
