// libhgpu runtime: initialisation, arenas, residency, staging, errors,
// launch accounting and the value/symbol entry points of the C ABI.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <dlfcn.h>
#include <string>
#include <unordered_map>
#include <vector>

#include "hgpu_internal.cuh"

// the symbol table (getSymbol / getSymbolStr): texts by id, ids by text
static std::unordered_map<std::string, L>* g_sym_ids;
static std::vector<std::string>* g_sym_names;

namespace hg {

cudaStream_t g_stream = nullptr;
static cudaStream_t g_copy_stream = nullptr;  // asynchronous uploads (hgpuToDeviceAsync)
int g_sms = 0;
unsigned* g_derr = nullptr;
int g_reduce_mode = 1;
static int g_residency = -1;  // decided at first use (residency())
static bool g_inited = false;
static std::mutex g_init_mu;
static long long g_launches = 0;
static long long g_syncs = 0;

// ------------------------------------------------------------------ errors
static thread_local char t_err[512];

static void rb_drop();
I set_error(I code, const char* fmt, ...) {
    rb_drop();
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof t_err, fmt, ap);
    va_end(ap);
    return code;
}

I cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    rb_drop();
    const char* base = strrchr(file, '/');
    set_error(e == cudaErrorMemoryAllocation ? E_DEVICE_OOM : E_DEVICE, "%s failed: %s (%s:%d)", what,
              cudaGetErrorString(e), base ? base + 1 : file, line);
    return e == cudaErrorMemoryAllocation ? E_DEVICE_OOM : E_DEVICE;
}

int g_tile_rows = 8;  // autotuner knob: probe rows per thread of the tiled join probes
// Autotuner knob: cudaLimitMaxL2FetchGranularity (bytes).  32 B speeds a
// gather of 8-byte values by sorted row ids at 14% density by ~20% (fewer
// bytes over-fetched) but slows scattered writes and random probes by
// 12-18%; streaming kernels read whole lines either way.  The default keeps
// the device's 64 B.
static int g_l2_fetch = 64;

// ------------------------------------------------------------------ arenas
// A bump arena over a list of chunks.  A mark is (chunk index, cursor).
struct Arena {
    struct Chunk { char* base; size_t cap, cur; };
    std::vector<Chunk> chunks;
    size_t cur_chunk = 0;
    size_t chunk_bytes;
    bool host;
    size_t limit;                          // most bytes of chunks held at once (0: no limit)
    size_t last_off = 0, last_bytes = 0;  // last allocation (for shrinking)
    long long last_chunk = -1;

    Arena(size_t cb, bool h, size_t lim = 0) : chunk_bytes(cb), host(h), limit(lim) {}
    size_t held() const {
        size_t t = 0;
        for (const Chunk& c : chunks) t += c.cap;
        return t;
    }

    void* alloc(size_t bytes) {
        size_t need = (bytes + 255) & ~(size_t)255;
        if (need == 0) need = 256;
        for (;;) {
            if (cur_chunk < chunks.size()) {
                Chunk& c = chunks[cur_chunk];
                if (c.cur + need <= c.cap) {
                    void* p = c.base + c.cur;
                    last_chunk = (long long)cur_chunk; last_off = c.cur; last_bytes = need;
                    c.cur += need;
                    return p;
                }
                if (cur_chunk + 1 < chunks.size()) {
                    // skip to the next chunk only if the request fits there
                    if (chunks[cur_chunk + 1].cap >= need) { cur_chunk++; chunks[cur_chunk].cur = 0; continue; }
                    // otherwise drop the smaller tail chunks and grow a larger one
                    for (size_t k = cur_chunk + 1; k < chunks.size(); k++) free_chunk(chunks[k]);
                    chunks.resize(cur_chunk + 1);
                }
            }
            size_t cap = need > chunk_bytes ? need : chunk_bytes;
            if (limit) {  // a capped arena grows only up to its limit
                const size_t h = held();
                if (h + need > limit) {
                    set_error(E_DEVICE_OOM, "%s arena: %zu more bytes would pass its limit of %zu bytes",
                              host ? "host" : "device", need, limit);
                    return nullptr;
                }
                if (h + cap > limit) cap = limit - h;
            }
            char* base = nullptr;
            cudaError_t e = host ? cudaHostAlloc((void**)&base, cap, cudaHostAllocPortable | cudaHostAllocMapped)
                                 : cudaMalloc((void**)&base, cap);
            if (e != cudaSuccess) {
                cudaGetLastError();
                set_error(E_DEVICE_OOM, "%s arena: cannot allocate %zu bytes (%s)", host ? "host" : "device", cap,
                          cudaGetErrorString(e));
                return nullptr;
            }
            chunks.push_back({base, cap, 0});
            cur_chunk = chunks.size() - 1;
        }
    }
    void free_chunk(Chunk& c) {
        stream_sync();  // queued work may still use the chunk
        if (host) cudaFreeHost(c.base); else cudaFree(c.base);
    }
    long long mark() const {
        if (chunks.empty()) return 0;
        return ((long long)cur_chunk << 40) | (long long)chunks[cur_chunk].cur;
    }
    // bytes in use: the capacity of every chunk before the current one plus
    // the current chunk's cursor (chunks before the cursor are never dropped,
    // so a value taken earlier maps back to the same chunk and offset)
    size_t used() const {
        if (chunks.empty()) return 0;
        size_t u = 0;
        for (size_t k = 0; k < cur_chunk; k++) u += chunks[k].cap;
        return u + chunks[cur_chunk].cur;
    }
    // rewinds to a used() value no larger than the current one
    void rewind_used(size_t u) {
        if (chunks.empty() || u > used()) return;
        size_t k = 0;
        while (k < cur_chunk && u >= chunks[k].cap) u -= chunks[k++].cap;
        cur_chunk = k;
        chunks[k].cur = u;
        last_chunk = -1;
    }
    void rewind(long long m) {
        size_t c = (size_t)(m >> 40), off = (size_t)(m & ((1LL << 40) - 1));
        if (chunks.empty()) return;
        if (c >= chunks.size()) return;
        cur_chunk = c;
        chunks[c].cur = off;
        last_chunk = -1;
    }
    bool shrink(void* p, size_t new_bytes) {
        if (last_chunk < 0) return false;
        Chunk& c = chunks[(size_t)last_chunk];
        if ((char*)p != c.base + last_off || (size_t)last_chunk != cur_chunk) return false;
        size_t need = (new_bytes + 255) & ~(size_t)255;
        if (need == 0) need = 256;
        if (need > last_bytes) return false;
        c.cur = last_off + need;
        last_bytes = need;
        return true;
    }
    // makes sure a chunk of at least `bytes` exists after the current one, so
    // that a later request of that size finds memory without a cudaMalloc
    bool reserve(size_t bytes) {
        for (size_t k = cur_chunk; k < chunks.size(); k++)
            if (chunks[k].cap >= bytes) return true;
        char* base = nullptr;
        cudaError_t e = host ? cudaHostAlloc((void**)&base, bytes, cudaHostAllocPortable | cudaHostAllocMapped)
                             : cudaMalloc((void**)&base, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        chunks.push_back({base, bytes, 0});
        return true;
    }
    bool contains(const void* p) const {
        for (auto& c : chunks)
            if ((const char*)p >= c.base && (const char*)p < c.base + c.cap) return true;
        return false;
    }
    // false when p is an allocation of this arena at or after the cursor
    // (released by a rewind); memory the arena does not own counts as live
    bool live(const void* p) const {
        for (size_t k = 0; k < chunks.size(); k++) {
            const Chunk& c = chunks[k];
            if ((const char*)p >= c.base && (const char*)p < c.base + c.cap)
                return k < cur_chunk || (k == cur_chunk && (size_t)((const char*)p - c.base) < c.cur);
        }
        return true;
    }
};

static size_t env_mb(const char* name, size_t dflt_mb) {
    const char* s = getenv(name);
    return (size_t)(s ? atoll(s) : (long long)dflt_mb) << 20;
}
static Arena* g_out = nullptr;      // output arena (device)
static Arena* g_scratch = nullptr;  // scratch arena (device)
static Arena* g_host = nullptr;     // pinned host arena

// heap-offset tokens: token -> (output mark, host mark)

I ensure_init() {
    if (g_inited) return 0;
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_inited) return 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return set_error(E_NO_DEVICE, "libhgpu: no CUDA device (%s)", cudaGetErrorString(e));
    }
    HG_CU(cudaSetDevice(0));
    HG_CU(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, 0));
    HG_CU(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
    HG_CU(cudaStreamCreateWithFlags(&g_copy_stream, cudaStreamNonBlocking));
    HG_CU(cudaMalloc((void**)&g_derr, 256));
    HG_CU(cudaMemset(g_derr, 0, 256));
    HG_CU(rb_init());
    HG_CU(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)g_l2_fetch));
    // HGPU_RADIX_PASS=0/1/2 starts the process with that radix pass mode (HGPU_TUNE_RADIX_PASS)
    if (const char* rp = getenv("HGPU_RADIX_PASS")) set_radix_pass_mode(atoi(rp));
    // HGPU_*_LIMIT_MB caps an arena's total size (0 or unset: no cap); a call
    // that needs more returns E_DEVICE_OOM
    if (!g_out) g_out = new Arena(env_mb("HGPU_DEVICE_CHUNK_MB", 4096), false, env_mb("HGPU_DEVICE_LIMIT_MB", 0));
    if (!g_scratch) g_scratch = new Arena(env_mb("HGPU_SCRATCH_CHUNK_MB", 4096), false, env_mb("HGPU_SCRATCH_LIMIT_MB", 0));
    if (!g_host) g_host = new Arena(env_mb("HGPU_HOST_CHUNK_MB", 256), true, env_mb("HGPU_HOST_LIMIT_MB", 0));
    g_inited = true;
    return 0;
}

I sync() {
    HG_CU(stream_sync());
    return 0;
}

void* dalloc(size_t bytes) { return g_out->alloc(bytes); }
bool dshrink(void* p, size_t new_bytes) { return g_out->shrink(p, new_bytes); }
long long out_mark() { return g_out->mark(); }
static void prune_registries();
void wait_all_pending();
void out_rewind(long long m) {
    wait_all_pending();
    g_out->rewind(m);
    prune_registries();
}
void* salloc(size_t bytes) { return g_scratch->alloc(bytes); }
I scratch_reserve(size_t bytes) {
    return g_scratch->reserve(bytes) ? 0 : set_error(E_DEVICE_OOM, "scratch arena: cannot reserve %zu bytes", bytes);
}
void* halloc(size_t bytes) { return g_host->alloc(bytes); }
I out_reserve(size_t bytes) {
    return g_out->reserve(bytes) ? 0 : set_error(E_DEVICE_OOM, "output arena: cannot reserve %zu bytes", bytes);
}
I host_reserve(size_t bytes) {
    return g_host->reserve(bytes) ? 0 : set_error(E_DEVICE_OOM, "host arena: cannot reserve %zu bytes", bytes);
}
ScratchScope::ScratchScope() : mark(g_scratch ? g_scratch->mark() : 0) {}
ScratchScope::~ScratchScope() {
    if (g_scratch) g_scratch->rewind(mark);
}

bool is_device_ptr(const void* p) {
    if (!p) return true;
    if (g_out->contains(p) || g_scratch->contains(p) || g_host->contains(p)) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeHost;
}

// memory the host can read directly (pinned arena, other pinned or pageable memory)
bool host_readable(const void* p) {
    if (!p || g_host->contains(p)) return true;
    if (g_out->contains(p) || g_scratch->contains(p)) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type != cudaMemoryTypeDevice;
}
// Default residency.  When the process also holds another builtin library
// (the reference's libcore linked after libhgpu supplies every builtin
// libhgpu does not export, h_primitive.h:72-211), that library's builtins
// dereference payloads on the host, so outputs are copied to pinned host
// memory by default; alone, outputs stay in HBM.  HGPU_RESIDENCY=host|device
// in the environment, or hgpuSetResidency, decides instead.
static const char* const k_foreign_builtins[] = {"pfnUnique", "pfnVector", "pfnAppend", "pfnDateYear"};
bool foreign_builtins_linked() {
    for (const char* name : k_foreign_builtins)
        if (dlsym(RTLD_DEFAULT, name)) return true;
    return false;
}
int residency() {
    if (g_residency < 0) {
        const char* e = getenv("HGPU_RESIDENCY");
        if (e && !strcmp(e, "host")) g_residency = HGPU_RESIDENT_HOST;
        else if (e && !strcmp(e, "device")) g_residency = HGPU_RESIDENT_DEVICE;
        else g_residency = foreign_builtins_linked() ? HGPU_RESIDENT_HOST : HGPU_RESIDENT_DEVICE;
    }
    return g_residency;
}

int esize(I t) {
    switch (t) {
    case H_B: case H_J: case H_C: return 1;
    case H_H: return 2;
    case H_I: case H_F: case H_M: case H_D: case H_U: case H_W: case H_T: return 4;
    case H_L: case H_E: case H_Q: case H_Z: case H_S: case H_X: case H_Y: return 8;
    default: return 8;
    }
}

// ------------------------------------------------------- asynchronous uploads
// hgpuToDeviceAsync copies on a second stream; the library stream waits on a
// copy's event only when a builtin first reads its destination (in_ptr,
// read_elem0, a copy out), or at hgpuWait / hgpuSync / setHeapOffset, so
// kernels on other inputs run while the copy is in flight.
struct Pending { const char* p; size_t bytes; cudaEvent_t ev; };
static std::vector<Pending> g_pending;
static std::vector<cudaEvent_t> g_upload_events;
static cudaEvent_t pool_event() {
    if (!g_upload_events.empty()) {
        cudaEvent_t e = g_upload_events.back();
        g_upload_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return e;
}
void wait_pending(const void* p) {
    if (g_pending.empty() || !p) return;
    for (size_t i = 0; i < g_pending.size();) {
        const Pending& q = g_pending[i];
        if ((const char*)p >= q.p && (const char*)p < q.p + q.bytes) {
            cudaStreamWaitEvent(g_stream, q.ev, 0);
            g_upload_events.push_back(q.ev);
            g_pending.erase(g_pending.begin() + (long)i);
        } else {
            i++;
        }
    }
}
void wait_all_pending() {
    for (const Pending& q : g_pending) {
        cudaStreamWaitEvent(g_stream, q.ev, 0);
        g_upload_events.push_back(q.ev);
    }
    g_pending.clear();
}

I in_ptr(V x, const void** p) {
    size_t nb = (size_t)x->len * esize(x->typ);
    if (x->len == 0) { *p = nullptr; return 0; }
    if (!is_inline(x)) wait_pending(x->g);
    if (!is_inline(x) && is_device_ptr(x->g)) { *p = x->g; return 0; }
    void* d = salloc(nb);
    if (!d) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(d, x->g, nb, cudaMemcpyHostToDevice, g_stream));
    *p = d;
    return 0;
}

I read_elem0(V x, uint64_t* bits) {
    *bits = 0;
    if (x->len < 1) return E_LENGTH;
    if (!is_inline(x)) wait_pending(x->g);
    int es = esize(x->typ);
    if (is_inline(x) || !is_device_ptr(x->g) || g_host->contains(x->g)) {
        memcpy(bits, x->g, es);
        return 0;
    }
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, x->g) == cudaSuccess && a.type == cudaMemoryTypeHost) {
        memcpy(bits, x->g, es);
        return 0;
    }
    cudaGetLastError();
    HG_CHECK(rb_queue(bits, x->g, es));
    HG_CU(stream_sync());
    return 0;
}

I alloc_out(V z, I typ, L len, void** dptr) {
    z->typ = typ;
    z->len = len;
    if (len > 1) {
        void* d = dalloc((size_t)len * esize(typ));
        if (!d) return E_DEVICE_OOM;
        z->g = (G)d;
        *dptr = d;
    } else {
        z->g = (G)&z->b;
        z->i64 = 0;
        void* d = salloc(16);
        if (!d) return E_DEVICE_OOM;
        *dptr = d;
    }
    return 0;
}

I finish_out(V z, void* dptr) {
    if (z->len == 1 && is_basic(z->typ)) {
        HG_CHECK(rb_queue(&z->b, dptr, esize(z->typ)));
        HG_CU(stream_sync());
        z->g = (G)&z->b;
    }
    return apply_residency(z);
}

I init_list(V z, I typ, L n) {
    z->typ = typ;
    z->len = n;
    z->g = (G)halloc((size_t)(n > 0 ? n : 1) * sizeof(V0));
    if (!z->g) return E_DEVICE_OOM;
    return 0;
}

V0* host_nodes(V x) { return (V0*)x->g; }

static I to_host_rec(V z, V x, bool in_place) {
    if (x->typ == H_G || x->typ == H_N || x->typ == H_A) {
        V0* src = (V0*)x->g;
        if (!in_place) {
            V0 hdr = *x;
            HG_CHECK(init_list(z, hdr.typ, hdr.len));
            if (hdr.typ == H_A) z->a = hdr.a;  // the table header is host memory already
            for (L i = 0; i < hdr.len; i++) HG_CHECK(to_host_rec((V0*)z->g + i, src + i, false));
        } else {
            for (L i = 0; i < x->len; i++) HG_CHECK(to_host_rec(src + i, src + i, true));
        }
        return 0;
    }
    if (x->typ == H_Y) {  // enum: the i64 index moves, the header stays shared
        V0 hdr = *x;
        if (z != x) *z = hdr;
        if (g_host->contains(hdr.g)) return 0;
        size_t nb = (size_t)(hdr.len > 0 ? hdr.len : 1) * 8;
        void* h = g_host->alloc(nb);
        if (!h) return E_DEVICE_OOM;
        if (hdr.len > 0) HG_CU(cudaMemcpyAsync(h, hdr.g, (size_t)hdr.len * 8, cudaMemcpyDefault, g_stream));
        HG_CU(stream_sync());
        z->g = (G)h;
        return 0;
    }
    if (!is_basic(x->typ)) return set_error(E_NOT_IMPL, "hgpuToHost: type %d", x->typ);
    if (!is_inline(x)) wait_pending(x->g);
    V0 hdr = *x;
    if (z != x) *z = hdr;
    if (is_inline(x)) {
        z->g = (G)&z->b;
        return 0;
    }
    if (hdr.len <= 1) {  // a one-element vector stored out of line
        uint64_t bits = 0;
        if (hdr.len == 1) HG_CHECK(read_elem0(&hdr, &bits));
        z->i64 = (L)bits;
        z->g = (G)&z->b;
        return 0;
    }
    size_t nb = (size_t)hdr.len * esize(hdr.typ);
    if (g_host->contains(hdr.g)) { z->g = hdr.g; return 0; }
    void* h = g_host->alloc(nb);
    if (!h) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(h, hdr.g, nb, cudaMemcpyDefault, g_stream));
    HG_CU(stream_sync());
    z->g = (G)h;
    return 0;
}

I apply_residency(V z) {
    if (residency() != HGPU_RESIDENT_HOST) return 0;
    return to_host_rec(z, z, true);
}

// ----------------------------------------------------------- list registry
static std::vector<ListInfo> g_lists;
void register_list(const ListInfo& g) {
    if (g_lists.size() > 256) g_lists.erase(g_lists.begin());
    g_lists.push_back(g);
}
ListInfo* find_list(const V0* nodes, long long ng) {
    for (size_t i = g_lists.size(); i-- > 0;)
        if (g_lists[i].nodes == nodes && g_lists[i].ng == ng) return &g_lists[i];
    return nullptr;
}

struct Bound { const void* data; long long len, bound; };
static std::vector<Bound> g_bounds;
void register_bound(const void* data, long long len, long long bound) {
    if (!data || len <= 1) return;
    if (g_bounds.size() > 256) g_bounds.erase(g_bounds.begin());
    g_bounds.push_back({data, len, bound});
}
bool known_in_range(const void* data, long long len, long long limit) {
    for (size_t i = g_bounds.size(); i-- > 0;)
        if (g_bounds[i].data == data && g_bounds[i].len == len) return g_bounds[i].bound <= limit;
    return false;
}

// --------------------------------------------------------------- read-back
// Small values a call needs on the host before it returns (counts, flags,
// the device error word) come back through one one-block kernel that copies
// them into mapped pinned memory, launched just before the host waits: a
// copy into pageable memory blocks by itself, and a copy operation costs
// more than such a launch (GB300: two pageable 8-byte reads and the wait
// 33 us per round trip, the copy kernel and the wait 18 us, the wait alone
// 15 us).  rb_queue records a read; the next stream_sync performs every
// recorded read and copies each value to its host destination, which must
// stay valid until then (the callers queue right before they wait).
struct RbList {
    const unsigned char* src[RB_ITEMS];
    unsigned bytes[RB_ITEMS];
    unsigned off[RB_ITEMS];
    int n;
};
static RbList g_rbl{};
static void* g_rbdst[RB_ITEMS];
static unsigned char* g_rbhost = nullptr;  // mapped pinned host memory
static unsigned char* g_rbmap = nullptr;   // its device address
static unsigned g_rbused = 0;

__global__ void k_read_back(RbList l, unsigned char* dst) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (w >= l.n) return;
    const unsigned char* src = l.src[w];
    const unsigned nb = l.bytes[w];
    if ((((uintptr_t)src) & 3) == 0 && (nb & 3) == 0) {  // destinations are 16-byte aligned
        const unsigned* s4 = (const unsigned*)src;
        volatile unsigned* d4 = (volatile unsigned*)(dst + l.off[w]);
        for (unsigned k = lane; k < nb / 4; k += 32) d4[k] = s4[k];
    } else {
        for (unsigned b = lane; b < nb; b += 32) ((volatile unsigned char*)dst)[l.off[w] + b] = src[b];
    }
}

// an error return abandons the reads queued by the failing call
static void rb_drop() {
    g_rbl.n = 0;
    g_rbused = 0;
}

cudaError_t rb_init() {
    if (g_rbhost) return cudaSuccess;
    cudaError_t e = cudaHostAlloc((void**)&g_rbhost, RB_BYTES, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) return e;
    return cudaHostGetDevicePointer((void**)&g_rbmap, g_rbhost, 0);
}

I rb_queue(void* host_dst, const void* dev, size_t bytes) {
    if (!g_rbmap) return set_error(E_DEVICE, "read-back: no mapped host area");
    const unsigned off = (g_rbused + 15u) & ~15u;
    if (g_rbl.n == RB_ITEMS || bytes > RB_BYTES || off + bytes > RB_BYTES)
        return set_error(E_DEVICE, "read-back: more than %d values or %u bytes queued before a wait", RB_ITEMS,
                         RB_BYTES);
    g_rbl.src[g_rbl.n] = (const unsigned char*)dev;
    g_rbl.bytes[g_rbl.n] = (unsigned)bytes;
    g_rbl.off[g_rbl.n] = off;
    g_rbdst[g_rbl.n] = host_dst;
    g_rbl.n++;
    g_rbused = off + (unsigned)bytes;
    return 0;
}

cudaError_t stream_sync() {
    g_syncs++;
    const int n = g_rbl.n;
    if (n > 0) {
        ::hg::LaunchScope ls_("read_back");
        k_read_back<<<1, 32 * RB_ITEMS, 0, g_stream>>>(g_rbl, g_rbmap);
    }
    g_rbl.n = 0;
    g_rbused = 0;
    cudaError_t e = n > 0 ? cudaGetLastError() : cudaSuccess;
    const cudaError_t w = cudaStreamSynchronize(g_stream);
    if (e == cudaSuccess) e = w;
    if (e != cudaSuccess) return e;
    for (int i = 0; i < n; i++) memcpy(g_rbdst[i], g_rbhost + g_rbl.off[i], g_rbl.bytes[i]);
    return cudaSuccess;
}

// ------------------------------------------------------------ device errors
I check_device_errors() {
    unsigned h = 0;
    HG_CHECK(rb_queue(&h, g_derr, sizeof h));
    HG_CU(stream_sync());
    if (!h) return 0;
    HG_CU(cudaMemsetAsync(g_derr, 0, sizeof h, g_stream));
    if (h & DERR_TIMEOUT) return set_error(E_DEVICE_TIMEOUT, "a device-side wait exceeded its iteration limit");
    if (h & DERR_CAPACITY) return set_error(E_DEVICE_OOM, "a device hash table or buffer ran out of capacity");
    if (h & DERR_INDEX) return set_error(E_INDEX, "index out of range");
    if (h & DERR_DIVZERO) return set_error(E_DIV_ZERO, "division by zero");
    return set_error(E_DEVICE, "device error flags 0x%x", h);
}

// ---------------------------------------------------------------- profiling
static bool g_prof = false;
struct ProfRec { const char* name; cudaEvent_t e0, e1; };
static std::vector<ProfRec> g_recs;
static std::vector<cudaEvent_t> g_event_pool;
static std::vector<std::string> g_prof_names;

static cudaEvent_t get_event() {
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

LaunchScope::LaunchScope(const char* n) : name(n), e0(nullptr), e1(nullptr), on(g_prof) {
    g_launches++;
    if (on) {
        e0 = get_event();
        e1 = get_event();
        cudaEventRecord(e0, g_stream);
    }
}
LaunchScope::~LaunchScope() {
    if (on) {
        cudaEventRecord(e1, g_stream);
        g_recs.push_back({name, e0, e1});
    }
}

I last_launch_error() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch", __FILE__, __LINE__);
    return 0;
}

// forget the lists and index ranges whose memory was released by a rewind;
// a list that survives drops a segment plan allocated after the mark
// String columns whose texts also sit in HBM (written by the CSV reader):
// the host pointer array -> the device blob and each text's span.
struct StrCols { const void* ptrs; long long n; const char* blob; const unsigned long long* spans; };
static std::vector<StrCols> g_strcols;
void register_strings(const void* ptrs, long long n, const char* blob, const unsigned long long* spans) {
    if (g_strcols.size() > 64) g_strcols.erase(g_strcols.begin());
    g_strcols.push_back({ptrs, n, blob, spans});
}
bool find_strings(const void* ptrs, long long n, const char** blob, const unsigned long long** spans) {
    for (size_t i = g_strcols.size(); i-- > 0;)
        if (g_strcols[i].ptrs == ptrs && g_strcols[i].n == n) {
            *blob = g_strcols[i].blob;
            *spans = g_strcols[i].spans;
            return true;
        }
    return false;
}

// The symbol table as seen by host code: count and texts by id.
L symbol_count() { return g_sym_names ? (L)g_sym_names->size() : 0; }
const char* symbol_text(L id) { return (*g_sym_names)[(size_t)id].c_str(); }

static void prune_registries() {
    auto live = [](const void* p) { return !p || (g_out->live(p) && g_host->live(p)); };
    {
        std::vector<StrCols> keep;
        for (StrCols& c : g_strcols)
            if (live(c.ptrs) && live(c.blob) && live(c.spans)) keep.push_back(c);
        g_strcols.swap(keep);
    }
    std::vector<ListInfo> keep;
    for (ListInfo& li : g_lists) {
        if (!live(li.nodes) || !live(li.starts) || !live(li.data)) continue;
        if (li.planned && (!live(li.big) || !live(li.chunk0) || !live(li.pstarts) || (li.corder && !live(li.corder))))
            li.planned = 0;
        if (li.cls_ids && (!live(li.cls_ids) || !live(li.cls_cnt))) li.cls_ids = li.cls_cnt = nullptr;
        keep.push_back(li);
    }
    g_lists.swap(keep);
    std::vector<Bound> kb;
    for (const Bound& b : g_bounds)
        if (live(b.data)) kb.push_back(b);
    g_bounds.swap(kb);
}

}  // namespace hg

using namespace hg;

// ======================================================================
// C ABI
// ======================================================================
extern "C" {

void initBackend(void) { ensure_init(); }

I hgpuInit(L device_arena_bytes, L host_arena_bytes) {
    HG_CHECK(ensure_init());
    if (device_arena_bytes > 0) { void* p = dalloc((size_t)device_arena_bytes); if (!p) return E_DEVICE_OOM; }
    if (host_arena_bytes > 0) { void* p = g_host->alloc((size_t)host_arena_bytes); if (!p) return E_DEVICE_OOM; }
    setHeapOffset(0);
    return 0;
}

V allocNode(void) {
    if (ensure_init()) return nullptr;
    V x = (V)halloc(sizeof(V0));
    if (x) memset(x, 0, sizeof(V0));
    return x;
}

// Caller-facing allocation (literals, interpreter temporaries): payloads go
// to the pinned host arena, which host code can fill and kernels can read.
V initV(V x, I typ, L len) {
    if (ensure_init()) return nullptr;
    x->typ = typ;
    x->len = len;
    if (is_basic(typ)) x->g = (len > 1) ? (G)halloc((size_t)getTypeSize(typ, len)) : (G)&x->b;
    else if (typ == H_Y) {  // i64 index out of line plus a header (h_memory.cc:184-194)
        x->g = (G)halloc((size_t)(len > 0 ? len : 1) * 8);
        x->y = (Y)halloc(sizeof(Y0));
        if (x->y) memset(x->y, 0, sizeof(Y0));
    } else x->g = (G)halloc((size_t)(len > 0 ? len : 1) * sizeof(V0));
    return x;
}

// The heap offset (h_memory.cc:155-161 returns the arena's byte cursor) covers
// both arenas that outputs come from, in their 256-byte allocation units:
// bits 62..32 = device output arena bytes in use / 256 (up to 512 GiB),
// bits 31..0 = pinned host arena bytes in use / 256 (up to 1 TiB).  It grows
// as outputs are allocated, reading it allocates nothing, and
// setHeapOffset(v) rewinds both arenas to where they were when v was read.
L getHeapOffset(void) {
    if (ensure_init()) return 0;
    return (L)(((unsigned long long)(g_out->used() >> 8) << 32) | (unsigned long long)(g_host->used() >> 8));
}

L setHeapOffset(L cur) {
    if (ensure_init()) return cur;
    if (cur < 0) return cur;
    // work already queued (and uploads in flight) may still use the region being released
    wait_all_pending();
    stream_sync();
    g_out->rewind_used((size_t)((unsigned long long)cur >> 32) << 8);
    g_host->rewind_used((size_t)((unsigned long long)cur & 0xffffffffull) << 8);
    prune_registries();
    return cur;
}

L getTypeSize(I typ, L len) {
    if (typ == H_G || typ == H_N || typ == H_A || typ == H_K || typ == H_V) return (L)sizeof(V0) * len;
    return (L)esize(typ) * len + (typ == H_C ? 1 : 0);
}

L getSymbol(S name) {
    if (!g_sym_ids) { g_sym_ids = new std::unordered_map<std::string, L>(); g_sym_names = new std::vector<std::string>(); }
    auto it = g_sym_ids->find(name);
    if (it != g_sym_ids->end()) return it->second;
    L id = (L)g_sym_names->size();
    g_sym_names->push_back(name);
    (*g_sym_ids)[name] = id;
    return id;
}
S getSymbolStr(L x) {
    if (!g_sym_names || x < 0 || (size_t)x >= g_sym_names->size()) return (S) "";
    return (S)(*g_sym_names)[(size_t)x].c_str();
}

I hgpuSetResidency(I mode) {
    if (mode != HGPU_RESIDENT_DEVICE && mode != HGPU_RESIDENT_HOST) return E_DOMAIN;
    g_residency = mode;
    return 0;
}
I hgpuGetResidency(void) { return residency(); }

I hgpuToHost(V z, V x) {
    HG_CHECK(ensure_init());
    return to_host_rec(z, x, false);
}

static I to_device_rec(V z, V x) {
    if (x->typ == H_G || x->typ == H_N || x->typ == H_A) {
        V0 hdr = *x;
        HG_CHECK(init_list(z, hdr.typ, hdr.len));
        if (hdr.typ == H_A) z->a = hdr.a;
        for (L i = 0; i < hdr.len; i++) HG_CHECK(to_device_rec((V0*)z->g + i, (V0*)hdr.g + i));
        return 0;
    }
    if (x->typ == H_Y) {  // enum payloads are never inline (initV, h_memory.cc:184-194)
        V0 hdr = *x;
        *z = hdr;
        void* d = dalloc((size_t)(hdr.len > 1 ? hdr.len : 2) * 8);
        if (!d) return E_DEVICE_OOM;
        if (hdr.len > 0) HG_CU(cudaMemcpyAsync(d, hdr.g, (size_t)hdr.len * 8, cudaMemcpyDefault, g_stream));
        z->g = (G)d;
        return 0;
    }
    if (!is_basic(x->typ)) return set_error(E_NOT_IMPL, "hgpuToDevice: type %d", x->typ);
    V0 hdr = *x;
    *z = hdr;
    if (hdr.len <= 1) {
        uint64_t bits = 0;
        if (hdr.len == 1) HG_CHECK(read_elem0(&hdr, &bits));
        z->i64 = (L)bits;
        z->g = (G)&z->b;
        return 0;
    }
    size_t nb = (size_t)hdr.len * esize(hdr.typ);
    void* d = dalloc(nb);
    if (!d) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(d, hdr.g, nb, cudaMemcpyDefault, g_stream));
    z->g = (G)d;
    return 0;
}

I hgpuToDevice(V z, V x) {
    HG_CHECK(ensure_init());
    return to_device_rec(z, x);
}

I hgpuToDeviceAsync(V z, V x) {
    HG_CHECK(ensure_init());
    if (!is_basic(x->typ) || x->len <= 1) return to_device_rec(z, x);
    const size_t nb = (size_t)x->len * esize(x->typ);
    void* d = dalloc(nb);
    if (!d) return E_DEVICE_OOM;
    cudaEvent_t before = pool_event(), done = pool_event();
    if (!before || !done) return set_error(E_DEVICE, "hgpuToDeviceAsync: no event");
    // the destination may be arena memory that queued library work still uses
    HG_CU(cudaEventRecord(before, g_stream));
    HG_CU(cudaStreamWaitEvent(g_copy_stream, before, 0));
    HG_CU(cudaMemcpyAsync(d, x->g, nb, cudaMemcpyDefault, g_copy_stream));
    HG_CU(cudaEventRecord(done, g_copy_stream));
    g_upload_events.push_back(before);
    g_pending.push_back({(const char*)d, nb, done});
    *z = *x;
    z->g = (G)d;
    return 0;
}

I hgpuWait(V z) {
    HG_CHECK(ensure_init());
    if (z && !is_inline(z)) wait_pending(z->g);
    return 0;
}

I hgpuIsDevice(V x) {
    if (ensure_init()) return 0;
    if (!(is_basic(x->typ) || x->typ == H_Y) || is_inline(x) || x->len < 1) return 0;
    if (g_host->contains(x->g)) return 0;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, x->g) != cudaSuccess) { cudaGetLastError(); return 0; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

I hgpuSync(void) {
    HG_CHECK(ensure_init());
    wait_all_pending();
    HG_CU(stream_sync());
    return check_device_errors();
}

void* hgpuStream(void) {
    if (ensure_init()) return nullptr;
    return (void*)g_stream;
}

const char* hgpuLastError(void) { return t_err; }

I hgpuSetReduceMode(I mode) {
    if (mode != 0 && mode != 1) return E_DOMAIN;
    g_reduce_mode = mode;
    return 0;
}

I hgpuProfile(I enable) {
    g_prof = enable != 0;
    return 0;
}

I hgpuProfileReset(void) {
    if (g_stream) stream_sync();
    for (auto& r : g_recs) { g_event_pool.push_back(r.e0); g_event_pool.push_back(r.e1); }
    g_recs.clear();
    return 0;
}

I hgpuProfileRead(I cap, const char** names, double* total_ms, L* launches) {
    if (g_stream) stream_sync();
    std::vector<std::pair<const char*, std::pair<double, L>>> acc;
    for (auto& r : g_recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.e0, r.e1);
        size_t k = 0;
        for (; k < acc.size(); k++)
            if (!strcmp(acc[k].first, r.name)) break;
        if (k == acc.size()) acc.push_back({r.name, {0.0, 0}});
        acc[k].second.first += ms;
        acc[k].second.second += 1;
    }
    for (size_t k = 0; k < acc.size() && (I)k < cap; k++) {
        if (names) names[k] = acc[k].first;
        if (total_ms) total_ms[k] = acc[k].second.first;
        if (launches) launches[k] = acc[k].second.second;
    }
    return (I)acc.size();
}

L hgpuLaunchCount(void) { return g_launches; }
L hgpuSyncCount(void) { return g_syncs; }

I hgpuSetTuning(I knob, E value) {
    switch (knob) {
    case HGPU_TUNE_HASH_LOAD: set_hash_load_factor(value); return 0;
    case HGPU_TUNE_RADIX_BITS: set_radix_digit_bits((int)value); return 0;
    case HGPU_TUNE_TILE_ROWS: g_tile_rows = value <= 8 ? 8 : (value <= 16 ? 16 : 32); return 0;
    case HGPU_TUNE_JOIN_FILTER: g_join_filter = value >= 0.5 ? 1 : 0; return 0;
    case HGPU_TUNE_RADIX_PASS: set_radix_pass_mode((int)(value + 0.5)); return 0;
    case HGPU_TUNE_L2_FETCH:
        g_l2_fetch = value <= 32 ? 32 : (value <= 64 ? 64 : 128);
        if (g_inited) {
            HG_CU(stream_sync());
            HG_CU(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)g_l2_fetch));
        }
        return 0;
    default: return E_DOMAIN;
    }
}

E hgpuGetTuning(I knob) {
    switch (knob) {
    case HGPU_TUNE_HASH_LOAD: return get_hash_load_factor();
    case HGPU_TUNE_RADIX_BITS: return (E)get_radix_digit_bits();
    case HGPU_TUNE_TILE_ROWS: return (E)g_tile_rows;
    case HGPU_TUNE_L2_FETCH: return (E)g_l2_fetch;
    case HGPU_TUNE_JOIN_FILTER: return (E)g_join_filter;
    case HGPU_TUNE_RADIX_PASS: return (E)get_radix_pass_mode();
    default: return -1.0;
    }
}

static cudaEvent_t g_t0 = nullptr, g_t1 = nullptr;
I hgpuTimerStart(void) {
    HG_CHECK(ensure_init());
    if (!g_t0) { cudaEventCreate(&g_t0); cudaEventCreate(&g_t1); }
    HG_CU(cudaEventRecord(g_t0, g_stream));
    return 0;
}
double hgpuTimerStop(void) {
    if (!g_t0) return -1.0;
    cudaEventRecord(g_t1, g_stream);
    cudaEventSynchronize(g_t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g_t0, g_t1);
    return ms;
}

}  // extern "C"
