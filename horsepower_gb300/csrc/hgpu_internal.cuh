// Internal declarations shared by the libhgpu translation units.
//
// Memory model
//   * output arena  : device memory, bump allocated in chunks, rewound only by
//                     setHeapOffset (the reference's arena, h_memory.cc:93-112).
//   * scratch arena : device memory for per-call temporaries (hash tables,
//                     sort buffers, tile status words); every entry point
//                     rewinds it on return (the reference's hash heap,
//                     h_memory.cc:425-466).
//   * host arena    : pinned host memory for list/dict node arrays and for
//                     HOST-residency outputs; kernels write nodes there
//                     directly through unified addressing.
// All kernels run on one library stream, so a rewound scratch region is only
// reused by work ordered after the work that used it.
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include "hgpu.h"

namespace hg {

// ------------------------------------------------------------------ errors
I set_error(I code, const char* fmt, ...);
I cuda_fail(cudaError_t e, const char* what, const char* file, int line);
#define HG_CU(...)                                                                   \
    do {                                                                             \
        cudaError_t e_ = (__VA_ARGS__);                                              \
        if (e_ != cudaSuccess) return ::hg::cuda_fail(e_, #__VA_ARGS__, __FILE__, __LINE__); \
    } while (0)
#define HG_CHECK(...)           \
    do {                        \
        I e_ = (__VA_ARGS__);   \
        if (e_) return e_;      \
    } while (0)

// Device error word bits (atomicOr'd by kernels, read by the host after a sync)
enum : unsigned {
    DERR_INDEX = 1u,       // an index fell outside its vector
    DERR_TIMEOUT = 2u,     // a bounded spin-wait gave up
    DERR_DIVZERO = 4u,     // a divisor was zero
    DERR_CAPACITY = 8u,    // a hash table or buffer ran out of slots
};
extern unsigned* g_derr;   // device word
I check_device_errors();   // syncs, reads and clears g_derr, maps to E_* codes
// iteration limit for every device-side spin-wait
constexpr long long SPIN_LIMIT = 1LL << 24;

// ---------------------------------------------------------------- runtime
extern cudaStream_t g_stream;
// waits for the library stream, counts the wait (hgpuSyncCount) and
// delivers the reads queued by rb_queue
cudaError_t stream_sync();
// queues a read of `bytes` of device memory into host_dst, performed by the
// next stream_sync (or check_device_errors) in the same round trip
constexpr int RB_ITEMS = 8;
constexpr unsigned RB_BYTES = 16384;
I rb_queue(void* host_dst, const void* dev, size_t bytes);
cudaError_t rb_init();
extern int g_sms;
I ensure_init();
I sync();

// arenas
void* dalloc(size_t bytes);                    // output arena; nullptr when exhausted
bool dshrink(void* p, size_t new_bytes);       // shrink the LAST output allocation

// autotuner knobs (hgpuSetTuning)
extern int g_tile_rows;                         // rows per lane of the tiled probe kernels: 8, 16, 32
extern int g_join_filter;                       // join presence bitmap: 0 through L2, 1 in a cluster's shared memory
void set_hash_load_factor(double f);
double get_hash_load_factor();
void set_radix_digit_bits(int b);
int get_radix_digit_bits();
void set_radix_pass_mode(int m);
int get_radix_pass_mode();
long long out_mark();                          // output-arena cursor (for undoing a failed call)
void out_rewind(long long m);
void* salloc(size_t bytes);                    // scratch arena
I scratch_reserve(size_t bytes);               // pre-allocates a scratch chunk of that size
I out_reserve(size_t bytes);                   // ... an output-arena chunk
I host_reserve(size_t bytes);                  // ... a pinned host-arena chunk
void* halloc(size_t bytes);                    // pinned host arena
struct ScratchScope {                          // rewinds the scratch arena on exit
    long long mark;
    ScratchScope();
    ~ScratchScope();
};
bool is_device_ptr(const void* p);             // payload readable by kernels without staging
void wait_pending(const void* p);              // library stream waits for an upload into p, if one is in flight
bool host_readable(const void* p);             // payload readable by host code without a copy
int residency();                               // HGPU_RESIDENT_DEVICE or HGPU_RESIDENT_HOST

// ------------------------------------------------------------- value model
inline bool is_int(I t) { return t == H_B || t == H_J || t == H_H || t == H_I || t == H_L; }
inline bool is_float(I t) { return t == H_F || t == H_E; }
inline bool is_real(I t) { return is_int(t) || is_float(t); }
inline bool is_date(I t) { return t == H_M || t == H_D || t == H_Z; }
inline bool is_time(I t) { return t == H_U || t == H_W || t == H_T; }
inline bool is_string(I t) { return t == H_C || t == H_Q || t == H_S; }
inline bool is_dtime(I t) { return is_date(t) || is_time(t); }
inline bool is_basic(I t) { return is_real(t) || is_string(t) || t == H_X || is_dtime(t); }
inline bool is_comparable(I t) { return is_real(t) || t == H_C || t == H_Q || is_dtime(t); }
int esize(I t);                                 // element bytes of a basic type
inline bool is_inline(V x) { return x->len <= 1 && is_basic(x->typ) && x->g == (G)&x->b; }

// Device-readable payload of x: device/pinned memory as is, pageable host
// memory staged into scratch.  len<=1 vectors return a scratch copy too.
I in_ptr(V x, const void** p);
// Element 0 of x as raw little-endian bits (scalars are passed to kernels by value)
I read_elem0(V x, uint64_t* bits);
// Output vector: allocates the payload (device arena for len>1, a scratch
// slot for len<=1) and sets z's header.  finish_out() moves a len<=1 result
// into the node (synchronous) and applies HOST residency.
I alloc_out(V z, I typ, L len, void** dptr);
I finish_out(V z, void* dptr);
I init_list(V z, I typ, L n);                   // list/dict node array in the host arena
I apply_residency(V z);                         // HOST mode: copy the payload to pinned host memory
V0* host_nodes(V x);                            // list nodes readable by the host (always)
I promote_to(V x, I typ, const void** out);     // device payload of x converted to a real type
I gather_into(const void* x, long long nx, int es, const void* y, I ytyp, void* z, long long n);

// ---------------------------------------------------------------- launches
struct LaunchScope {
    const char* name;
    cudaEvent_t e0, e1;
    bool on;
    explicit LaunchScope(const char* n);
    ~LaunchScope();
};
#define HG_LAUNCH(name, grid, block, smem, kern, ...)                           \
    do {                                                                        \
        ::hg::LaunchScope ls_(name);                                            \
        kern<<<(grid), (block), (smem), ::hg::g_stream>>>(__VA_ARGS__);         \
    } while (0)
I last_launch_error();

inline unsigned grid_for(long long n, int per_block) {
    long long b = (n + per_block - 1) / per_block;
    return (unsigned)(b < 1 ? 1 : b);
}

// Lists produced by this library keep a device-side description, so a
// later builtin over the same list need not read its host nodes:
//   LIST_SEGMENTS: element g = data[starts[g] .. starts[g+1]) (ng+1-th bound = total),
//                  e.g. @group's row lists or each_right(@index)'s gathered vectors
//   LIST_SCALARS : element g = the one value data[g] (each(@sum) and friends)
enum { LIST_SEGMENTS = 0, LIST_SCALARS = 1 };
// One 4096-element chunk of a long segment as a reduction CTA takes it: its
// first element, its length and its index among the chunks (where its
// partial goes), in launch order.
struct ChunkDesc {
    long long first;
    unsigned len;
    unsigned chunk;
};
struct ListInfo {
    const V0* nodes;          // host node array of the list
    long long ng;             // number of elements
    int kind;
    I typ;                    // element type of the payload
    const long long* starts;  // device, ng entries (LIST_SEGMENTS)
    long long total;          // sum of lengths (LIST_SEGMENTS)
    const void* data;         // device payload
    int group_rows;           // 1: @group row lists (a permutation of 0..total-1, no empty group)
    // cached split of the segments longer than one reduction tile (output arena)
    int planned;
    long long nbig;
    unsigned long long nchunks;
    const long long* big;
    const unsigned long long* chunk0;
    const long long* pstarts;
    const struct ChunkDesc* corder;  // chunk launch order (nullptr: in segment order)
    // cached segment ids by size class and the class counts (output arena)
    const unsigned* cls_ids;
    const unsigned* cls_cnt;
    // host copy of the 8 class counts (cls_known), so empty classes launch nothing
    int cls_known;
    unsigned cls_host[8];
};
void register_list(const ListInfo& g);
// The size classes and the long-segment plan of a list of at most
// SEG_PLAN_SMALL segments, made by one launch queued on the library stream;
// the caller queues the read of hdr_dev into hdr (rb_queue) with its own
// next wait and then hands the plan to seg_plan_adopt, which puts it into
// the list's ListInfo, so that aggregations over the list need no round
// trip of their own.  Lists with more segments get nothing (hdr == nullptr).
constexpr long long SEG_PLAN_SMALL = 4096;
constexpr size_t SEG_PLAN_HDR_BYTES = 10 * 8;  // 8 class counts, nbig, nchunks
struct SmallPlan {
    unsigned* cc = nullptr;
    unsigned* ids = nullptr;
    long long* big = nullptr;
    unsigned long long* c0 = nullptr;
    long long* ps = nullptr;
    ChunkDesc* order = nullptr;
    unsigned long long* hdr = nullptr;      // host: 8 class counts, nbig, nchunks (after the wait)
    const unsigned long long* hdr_dev = nullptr;  // the same on the device, for the caller to queue
};
I seg_plan_small(const long long* starts, long long ng, long long total, SmallPlan* p);
void seg_plan_adopt(ListInfo& li, const SmallPlan& p);
ListInfo* find_list(const V0* nodes, long long ng);

// Index vectors produced by this library carry a known value range: every
// element of the i64 vector at `data` (length len) lies in [0, bound).  An
// @index with such a vector cannot go out of range when bound <= len(x), so
// it needs no synchronous bounds check.
void register_bound(const void* data, long long len, long long bound);
bool known_in_range(const void* data, long long len, long long limit);

// String columns whose texts also live in HBM as one blob, each text's span
// = (offset << 16) | length (the CSV reader registers the columns it makes).
void register_strings(const void* ptrs, long long n, const char* blob, const unsigned long long* spans);
bool find_strings(const void* ptrs, long long n, const char** blob, const unsigned long long** spans);
// The host symbol table: ids are 0 .. symbol_count() - 1 in order of interning.
L symbol_count();
const char* symbol_text(L id);

// pfnCompare on two symbol operands (k_string.cu)
I compare_symbols(V z, V x, V y, I op);

// reduction mode (1 = fixed-order deterministic tile tree)
extern int g_reduce_mode;

}  // namespace hg
