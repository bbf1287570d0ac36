// Table ingest: the reference's binary table format (serializeV /
// readSerializeV, h_io.cc:626-772) and its CSV reader (readCSV, loadCSV,
// getField, loadItem; h_io.cc:50-188), with column payloads landing in HBM.
//
// Binary: payloads stream from the file through two pinned staging buffers;
// the fread of one chunk overlaps the host-to-device copy of the previous.
//
// CSV: the whole file is copied to HBM once, then
//   1. line ends: per-tile newline counts, a scan, an ordered scatter;
//   2. one warp per 32 lines: the warp trims each line as getField does and
//      finds its separators with ballots, then converts column by column,
//      lane i taking line i, with loadItem's function for the column's type
//      (strtol semantics for atoi/atol, sscanf %d-%d-%d, first char);
//   3. floats: decimal significand and exponent in one pass; Clinger's exact
//      fast path (significand <= 2^53 and |exponent| <= 22: one correctly
//      rounded IEEE operation on exact operands) covers decimals such as
//      TPC-H's; every other input goes to a slow pass that decides the
//      rounding exactly with big-integer arithmetic, so values equal glibc's
//      correctly rounded strtod / strtof bit for bit;
//   4. symbols: FNV-1a hashes, a first-occurrence table, the distinct texts
//      interned on the host in first-occurrence order, ids mapped back on the
//      GPU and every row's text checked against its representative's;
//   5. strings: lengths scanned to offsets, texts and their pointers written
//      straight into pinned host memory by the GPU.
#include <unistd.h>

#include <atomic>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "dev_common.cuh"
#include "hgpu_internal.cuh"

extern "C" {
C LINE_SEP = '|';        // h_io.cc:9
B LINE_HEADER = false;   // h_io.cc:11
L LINE_MAX_CHAR = 1024;  // h_io.cc:8 (fgets buffer size)
}

namespace hg {

I compact_rows(const uint8_t* mask, long long n, long long* out, long long* count);
I scan_exclusive(const unsigned* in, long long n, unsigned long long* out, unsigned long long* total_h);
I scan_counts(const unsigned* counts, long long n, unsigned long long* offs);

namespace {

// ------------------------------------------------------------------ staging
constexpr size_t STAGE_BYTES = 32u << 20;
struct Staging {
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2];
    bool ready = false;
};
Staging g_stage;

I stage_init() {
    if (g_stage.ready) return 0;
    for (int k = 0; k < 2; k++) {
        HG_CU(cudaHostAlloc(&g_stage.buf[k], STAGE_BYTES, cudaHostAllocDefault));
        HG_CU(cudaEventCreateWithFlags(&g_stage.ev[k], cudaEventDisableTiming));
    }
    g_stage.ready = true;
    return 0;
}

I io_fail(const char* what) { return set_error(E_GENERAL, "%s", what); }

// fp -> dst (device), `bytes` bytes, double-buffered
I stream_in(FILE* fp, void* dst, size_t bytes) {
    HG_CHECK(stage_init());
    size_t done = 0;
    int k = 0;
    while (done < bytes) {
        const size_t c = bytes - done < STAGE_BYTES ? bytes - done : STAGE_BYTES;
        HG_CU(cudaEventSynchronize(g_stage.ev[k]));  // the copy out of this buffer has finished
        if (fread(g_stage.buf[k], 1, c, fp) != c) {
            stream_sync();
            return io_fail("fread: unexpected end of file");
        }
        HG_CU(cudaMemcpyAsync((char*)dst + done, g_stage.buf[k], c, cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaEventRecord(g_stage.ev[k], g_stream));
        done += c;
        k ^= 1;
    }
    HG_CU(stream_sync());
    return 0;
}

// Large reads from a regular file: worker threads pread disjoint chunks into
// their own pinned buffers and copy them to HBM on their own streams, so file
// reads (memory copies out of the page cache) run on several cores at once.
constexpr size_t PAR_CHUNK = 8u << 20;
constexpr int PAR_THREADS = 16;
struct ParWorker {
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2];
    cudaStream_t st;
    bool ready = false;
};
ParWorker g_par[PAR_THREADS];

I par_init(int t) {
    ParWorker& w = g_par[t];
    if (w.ready) return 0;
    for (int k = 0; k < 2; k++) {
        HG_CU(cudaHostAlloc(&w.buf[k], PAR_CHUNK, cudaHostAllocDefault));
        HG_CU(cudaEventCreateWithFlags(&w.ev[k], cudaEventDisableTiming));
    }
    HG_CU(cudaStreamCreateWithFlags(&w.st, cudaStreamNonBlocking));
    w.ready = true;
    return 0;
}

I stream_in_par(FILE* fp, void* dst, size_t bytes) {
    const off_t pos = ftello(fp);
    if (pos < 0 || bytes < 4 * PAR_CHUNK) return stream_in(fp, dst, bytes);
    int dev = 0;
    HG_CU(cudaGetDevice(&dev));
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)(hw > 1 ? hw : 1);
    if (nt > PAR_THREADS) nt = PAR_THREADS;
    for (int t = 0; t < nt; t++) HG_CHECK(par_init(t));
    const int fd = fileno(fp);
    std::atomic<size_t> next(0);
    std::atomic<int> bad(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) {
        th.emplace_back([&, t]() {
            cudaSetDevice(dev);
            ParWorker& w = g_par[t];
            int k = 0;
            for (;;) {
                const size_t c0 = next.fetch_add(PAR_CHUNK);
                if (c0 >= bytes || bad.load()) break;
                const size_t c = bytes - c0 < PAR_CHUNK ? bytes - c0 : PAR_CHUNK;
                if (cudaEventSynchronize(w.ev[k]) != cudaSuccess) { bad = 2; break; }
                size_t got = 0;
                while (got < c) {
                    const ssize_t r = pread(fd, (char*)w.buf[k] + got, c - got, pos + (off_t)(c0 + got));
                    if (r <= 0) break;
                    got += (size_t)r;
                }
                if (got != c) { bad = 1; break; }
                if (cudaMemcpyAsync((char*)dst + c0, w.buf[k], c, cudaMemcpyHostToDevice, w.st) != cudaSuccess ||
                    cudaEventRecord(w.ev[k], w.st) != cudaSuccess) { bad = 2; break; }
                k ^= 1;
            }
            if (cudaStreamSynchronize(w.st) != cudaSuccess) bad = 2;
        });
    }
    for (auto& x : th) x.join();
    if (bad.load() == 1) return io_fail("pread: unexpected end of file");
    if (bad.load() == 2) return set_error(E_DEVICE, "copying file chunks to the device");
    if (fseeko(fp, pos + (off_t)bytes, SEEK_SET) != 0) return io_fail("fseek failed");
    return 0;
}

// fp -> host memory: the same disjoint-chunk preads, straight into dst
I read_par_host(FILE* fp, void* dst, size_t bytes) {
    const off_t pos = ftello(fp);
    if (pos < 0 || bytes < 4 * PAR_CHUNK) {
        if (bytes && fread(dst, 1, bytes, fp) != bytes) return io_fail("fread: unexpected end of file");
        return 0;
    }
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)(hw > 1 ? hw : 1);
    if (nt > PAR_THREADS) nt = PAR_THREADS;
    const int fd = fileno(fp);
    std::atomic<size_t> next(0);
    std::atomic<int> bad(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) {
        th.emplace_back([&]() {
            for (;;) {
                const size_t c0 = next.fetch_add(PAR_CHUNK);
                if (c0 >= bytes || bad.load()) break;
                const size_t c = bytes - c0 < PAR_CHUNK ? bytes - c0 : PAR_CHUNK;
                size_t got = 0;
                while (got < c) {
                    const ssize_t r = pread(fd, (char*)dst + c0 + got, c - got, pos + (off_t)(c0 + got));
                    if (r <= 0) break;
                    got += (size_t)r;
                }
                if (got != c) { bad = 1; break; }
            }
        });
    }
    for (auto& x : th) x.join();
    if (bad.load()) return io_fail("pread: unexpected end of file");
    if (fseeko(fp, pos + (off_t)bytes, SEEK_SET) != 0) return io_fail("fseek failed");
    return 0;
}

// src (device) -> fp, double-buffered
I stream_out(FILE* fp, const void* src, size_t bytes) {
    HG_CHECK(stage_init());
    const size_t nchunks = (bytes + STAGE_BYTES - 1) / STAGE_BYTES;
    auto issue = [&](size_t j) -> I {
        const size_t off = j * STAGE_BYTES, c = bytes - off < STAGE_BYTES ? bytes - off : STAGE_BYTES;
        HG_CU(cudaMemcpyAsync(g_stage.buf[j & 1], (const char*)src + off, c, cudaMemcpyDeviceToHost, g_stream));
        HG_CU(cudaEventRecord(g_stage.ev[j & 1], g_stream));
        return 0;
    };
    if (nchunks) HG_CHECK(issue(0));
    for (size_t j = 0; j < nchunks; j++) {
        if (j + 1 < nchunks) HG_CHECK(issue(j + 1));
        HG_CU(cudaEventSynchronize(g_stage.ev[j & 1]));
        const size_t off = j * STAGE_BYTES, c = bytes - off < STAGE_BYTES ? bytes - off : STAGE_BYTES;
        if (fwrite(g_stage.buf[j & 1], 1, c, fp) != c) {
            stream_sync();
            return io_fail("fwrite failed");
        }
    }
    return 0;
}

#define RD(p, n)                                                                              \
    do {                                                                                      \
        if ((n) > 0 && fread((p), 1, (size_t)(n), fp) != (size_t)(n)) return io_fail("fread: unexpected end of file"); \
    } while (0)
#define WR(p, n)                                                                              \
    do {                                                                                      \
        if ((n) > 0 && fwrite((p), 1, (size_t)(n), fp) != (size_t)(n)) return io_fail("fwrite failed"); \
    } while (0)

bool raw_payload(I t) { return is_real(t) || t == H_C || is_dtime(t) || t == H_X; }

// An i64 payload (symbol ids) from host memory into a node of type typ.
I put_words(V x, I typ, const std::vector<L>& w) {
    x->typ = typ;
    x->len = (L)w.size();
    if (w.size() <= 1) {
        x->g = (G)&x->b;
        x->i64 = w.empty() ? 0 : w[0];
        return 0;
    }
    void* d = dalloc(w.size() * 8);
    if (!d) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(d, w.data(), w.size() * 8, cudaMemcpyHostToDevice, g_stream));
    HG_CU(stream_sync());
    x->g = (G)d;
    return 0;
}

// ------------------------------------------------------- binary: read side
I csv_symbols(const char* dbuf, const unsigned long long* spans, long long rows, long long* out);
unsigned grid_of(long long n);

__global__ void k_text_lengths(const long long* __restrict__ sz, long long n, unsigned* __restrict__ lens) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        lens[i] = (unsigned)sz[i] + 1u;
}
// span of text i = (offset << 16) | strlen; the text must end at its stored length
__global__ void k_text_spans(const char* __restrict__ blob, const long long* __restrict__ sz,
                             const unsigned long long* __restrict__ offs, long long n,
                             unsigned long long* __restrict__ spans, unsigned* bad) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long o = offs[i];
        const int k = (int)sz[i];
        if (blob[o + k] != 0) atomicOr(bad, 1u);
        int l = 0;
        while (l < k && blob[o + l] != 0) l++;
        spans[i] = (o << 16) | (unsigned long long)l;
    }
}

I read_node(V x, FILE* fp) {
    V0 hdr;
    RD(&hdr, sizeof(V0));
    const I typ = hdr.typ;
    const L len = hdr.len;
    if (len < 0) return set_error(E_GENERAL, "serialized node: negative length %lld", len);
    if (raw_payload(typ)) {
        const size_t nb = (size_t)getTypeSize(typ, len);
        x->typ = typ;
        x->len = len;
        if (len <= 1) {  // inline, as initV leaves it (h_memory.cc:184-187)
            x->i64 = hdr.i64;
            x->g = (G)&x->b;
            RD(&x->b, nb);
            return 0;
        }
        void* d = dalloc(nb);
        if (!d) return E_DEVICE_OOM;
        x->g = (G)d;
        return stream_in_par(fp, d, nb);
    }
    switch (typ) {
    case H_Q: {  // readSerializeQ (h_io.cc:716-722): lengths, then NUL-terminated texts
        std::vector<L> sz((size_t)len);
        RD(sz.data(), 8 * len);
        size_t total = 0;
        bool short_texts = true;
        for (L i = 0; i < len; i++) {
            if (sz[i] < 0) return set_error(E_GENERAL, "serialized symbol: negative length");
            total += (size_t)sz[i] + 1;
            short_texts = short_texts && sz[i] < 0xffff;
        }
        if (len <= 1 || !short_texts) {  // interned one by one, in order
            std::vector<char> blob(total > 0 ? total : 1);
            RD(blob.data(), total);
            std::vector<L> ids((size_t)len);
            size_t o = 0;
            for (L i = 0; i < len; i++) {
                if (blob[o + (size_t)sz[i]] != 0) return set_error(E_GENERAL, "serialized text without its NUL");
                ids[i] = getSymbol(blob.data() + o);
                o += (size_t)sz[i] + 1;
            }
            return put_words(x, H_Q, ids);
        }
        // on the GPU: texts straight into HBM, distinct ones interned in first-occurrence order
        char* dblob = (char*)salloc(total);
        long long* dsz = (long long*)salloc((size_t)len * 8);
        unsigned* lens = (unsigned*)salloc((size_t)len * 4);
        unsigned long long* offs = (unsigned long long*)salloc((size_t)(len + 1) * 8);
        unsigned long long* dspans = (unsigned long long*)salloc((size_t)len * 8);
        unsigned* bad = (unsigned*)salloc(16);
        long long* ids = (long long*)dalloc((size_t)len * 8);
        if (!dblob || !dsz || !lens || !offs || !dspans || !bad || !ids) return E_DEVICE_OOM;
        HG_CHECK(stream_in_par(fp, dblob, total));
        HG_CU(cudaMemcpyAsync(dsz, sz.data(), (size_t)len * 8, cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaMemsetAsync(bad, 0, 4, g_stream));
        HG_LAUNCH("text_lengths", grid_of(len), 256, 0, k_text_lengths, dsz, len, lens);
        HG_CHECK(scan_exclusive(lens, len, offs, nullptr));
        HG_LAUNCH("text_spans", grid_of(len), 256, 0, k_text_spans, dblob, dsz, offs, len, dspans, bad);
        unsigned hb = 0;
        HG_CHECK(rb_queue(&hb, bad, 4));
        HG_CU(stream_sync());
        if (hb) return set_error(E_GENERAL, "serialized text without its NUL");
        HG_CHECK(csv_symbols(dblob, dspans, len, ids));
        x->typ = H_Q;
        x->len = len;
        x->g = (G)ids;
        return 0;
    }
    case H_S: {  // readSerializeS (h_io.cc:724-729): the texts land in one pinned block
        std::vector<L> sz((size_t)len);
        RD(sz.data(), 8 * len);
        size_t total = 0;
        for (L i = 0; i < len; i++) {
            if (sz[i] < 0) return set_error(E_GENERAL, "serialized string: negative length");
            total += (size_t)sz[i] + 1;
        }
        char* blob = (char*)halloc(total > 0 ? total : 1);
        S* ptrs = len <= 1 ? (S*)&x->b : (S*)halloc((size_t)len * sizeof(S));
        if (!blob || !ptrs) return E_DEVICE_OOM;
        HG_CHECK(read_par_host(fp, blob, total));
        size_t o = 0;
        for (L i = 0; i < len; i++) {
            if (blob[o + (size_t)sz[i]] != 0) return set_error(E_GENERAL, "serialized string without its NUL");
            ptrs[i] = blob + o;
            o += (size_t)sz[i] + 1;
        }
        x->typ = H_S;
        x->len = len;
        x->g = (G)ptrs;
        if (len == 0) x->g = (G)&x->b;
        return 0;
    }
    case H_G: {  // readSerializeG (h_io.cc:731-733)
        HG_CHECK(init_list(x, H_G, len));
        V0* e = (V0*)x->g;
        memset(e, 0, (size_t)(len > 0 ? len : 1) * sizeof(V0));
        for (L i = 0; i < len; i++) HG_CHECK(read_node(e + i, fp));
        return 0;
    }
    case H_A: {  // readSerializeA (h_io.cc:735-745): A0, keys, values
        if (len != 2) return set_error(E_GENERAL, "serialized table: %lld nodes, not 2", len);
        HG_CHECK(init_list(x, H_A, 2));
        V0* e = (V0*)x->g;
        memset(e, 0, 2 * sizeof(V0));
        A a = (A)halloc(sizeof(A0));
        if (!a) return E_DEVICE_OOM;
        RD(a, sizeof(A0));
        a->fkey = nullptr;  // a pointer of the writing process
        x->a = a;
        HG_CHECK(read_node(e + 0, fp));
        HG_CHECK(read_node(e + 1, fp));
        return 0;
    }
    default:
        return set_error(E_NOT_IMPL, "serialized node of type %d", typ);  // EP in the reference
    }
}

// ------------------------------------------------------ binary: write side
I host_words(V x, std::vector<L>* w) {  // an 8-byte payload as host words
    w->resize((size_t)x->len);
    if (x->len == 0) return 0;
    if (host_readable(x->g)) {
        memcpy(w->data(), x->g, (size_t)x->len * 8);
        return 0;
    }
    HG_CU(cudaMemcpyAsync(w->data(), x->g, (size_t)x->len * 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(stream_sync());
    return 0;
}

I write_node(V x, FILE* fp) {
    WR(x, sizeof(V0));
    const I typ = x->typ;
    const L len = x->len;
    if (raw_payload(typ)) {  // serializeBasic (h_io.cc:640-643)
        const size_t nb = (size_t)esize(typ) * (size_t)len;
        if (nb > 0) {
            if (host_readable(x->g)) WR(x->g, nb);
            else HG_CHECK(stream_out(fp, x->g, nb));
        }
        if (typ == H_C) {
            const char nul = 0;
            WR(&nul, 1);
        }
        return 0;
    }
    switch (typ) {
    case H_Q: {  // serializeQ (h_io.cc:645-648)
        std::vector<L> ids;
        HG_CHECK(host_words(x, &ids));
        for (L id : ids) {
            const L n = (L)strlen(getSymbolStr(id));
            WR(&n, 8);
        }
        for (L id : ids) {
            S s = getSymbolStr(id);
            WR(s, strlen(s) + 1);
        }
        return 0;
    }
    case H_S: {  // serializeS (h_io.cc:650-654)
        std::vector<L> w;
        HG_CHECK(host_words(x, &w));
        for (L p : w) {
            const L n = (L)strlen((S)p);
            WR(&n, 8);
        }
        for (L p : w) WR((S)p, strlen((S)p) + 1);
        return 0;
    }
    case H_G: {  // serializeG (h_io.cc:656-658)
        V0* e = host_nodes(x);
        for (L i = 0; i < len; i++) HG_CHECK(write_node(e + i, fp));
        return 0;
    }
    case H_A: {  // serializeA (h_io.cc:660-668)
        A0 a{};
        if (x->a) a = *x->a;
        a.fkey = nullptr;
        WR(&a, sizeof(A0));
        V0* e = host_nodes(x);
        HG_CHECK(write_node(e + 0, fp));
        HG_CHECK(write_node(e + 1, fp));
        return 0;
    }
    default:
        return set_error(E_NOT_IMPL, "serializing a node of type %d", typ);  // EP in the reference
    }
}

// ====================================================================== CSV
constexpr int NL_TILE = 1 << 16;   // bytes per newline-count tile
constexpr int NL_THREADS = 256;    // 256 bytes per thread per tile
constexpr int CSV_MAXLINE = 65535;  // largest LINE_MAX_CHAR accepted (16-bit field offsets)
constexpr int CSV_MAXCOLS = 256;

enum : unsigned {
    CSV_FIELDS = 1u,     // a line with another number of fields than columns
    CSV_LONG = 2u,       // a line longer than LINE_MAX_CHAR - 1 (fgets would split it)
    CSV_NUL = 4u,        // a NUL byte inside a line
    CSV_DATE = 8u,       // a date field sscanf cannot read completely
    CSV_HEXNAN = 16u,    // hexadecimal float or nan(...) payload: not accepted
    CSV_SLOWFULL = 32u,  // more slow-path floats than the slow list holds
};

// newlines in the PER bytes of one thread (16-byte loads when the segment is whole)
constexpr int NL_PER = NL_TILE / NL_THREADS;
__device__ __forceinline__ unsigned nl_in_word(unsigned w) { return __popc(__vcmpeq4(w, 0x0a0a0a0au)) >> 3; }
__device__ unsigned nl_count_seg(const char* __restrict__ buf, long long n, long long t0) {
    unsigned c = 0;
    if (t0 + NL_PER <= n) {
        const uint4* p = (const uint4*)(buf + t0);
#pragma unroll 4
        for (int k = 0; k < NL_PER / 16; k++) {
            const uint4 v = p[k];
            c += nl_in_word(v.x) + nl_in_word(v.y) + nl_in_word(v.z) + nl_in_word(v.w);
        }
    } else {
        for (long long i = t0; i < n && i < t0 + NL_PER; i++) c += buf[i] == '\n';
    }
    return c;
}
__global__ void k_nl_count(const char* __restrict__ buf, long long n, unsigned* __restrict__ counts) {
    const long long t0 = (long long)blockIdx.x * NL_TILE + (long long)threadIdx.x * NL_PER;
    unsigned c = nl_count_seg(buf, n, t0);
    c = __reduce_add_sync(0xffffffffu, c);
    __shared__ unsigned ws[NL_THREADS / 32];
    if (lane_id() == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < NL_THREADS / 32; w++) t += ws[w];
        counts[blockIdx.x] = t;
    }
}

// positions of the newlines of each tile, in order (offs: exclusive tile prefix)
__global__ void k_nl_scatter(const char* __restrict__ buf, long long n, const unsigned long long* __restrict__ offs,
                             long long* __restrict__ pos) {
    const long long t0 = (long long)blockIdx.x * NL_TILE + (long long)threadIdx.x * NL_PER;
    const unsigned c = nl_count_seg(buf, n, t0);
    // exclusive prefix of c over the block (thread order = byte order)
    const unsigned incl = warp_incl_scan(c);
    __shared__ unsigned ws[NL_THREADS / 32];
    if (lane_id() == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    unsigned before = 0;
    for (unsigned w = 0; w < (threadIdx.x >> 5); w++) before += ws[w];
    unsigned long long o = offs[blockIdx.x] + before + (incl - c);
    if (c == 0) return;
    if (t0 + NL_PER <= n) {
        const uint4* p = (const uint4*)(buf + t0);
        for (int k = 0; k < NL_PER / 16; k++) {
            const uint4 v = p[k];
            const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int q = 0; q < 4; q++) {
                unsigned m = __vcmpeq4(w[q], 0x0a0a0a0au);  // 0xff in each newline byte
                while (m) {
                    const int b = __ffs(m) - 1;
                    pos[o++] = t0 + 16 * k + 4 * q + (b >> 3);
                    m &= ~(0xffu << (b & ~7));
                }
            }
        }
    } else {
        for (long long i = t0; i < n && i < t0 + NL_PER; i++)
            if (buf[i] == '\n') pos[o++] = i;
    }
}

struct CsvCol {
    int typ;
    void* out;                 // column payload (device), or the span array for symbols and strings
};
struct CsvArgs {
    const char* buf;
    long long size;            // file bytes
    const long long* nl;       // newline positions
    long long nnl;
    long long first_line;      // 1 when the first line is a header
    long long rows;
    int ncols;
    char sep;
    int maxline;               // LINE_MAX_CHAR
    const CsvCol* cols;
    unsigned* err;             // [0] codes, [1] first bad row (atomicMin)
    unsigned long long* slow;  // (span, row << 16 | col) pairs of floats for the slow pass
    unsigned* nslow;
    unsigned slow_cap;
};

__device__ __forceinline__ unsigned row32(long long r) { return r < 0xffffffffll ? (unsigned)r : 0xfffffffeu; }
__device__ __forceinline__ bool c_space(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }
__device__ __forceinline__ bool c_digit(unsigned char c) { return c >= '0' && c <= '9'; }
__device__ __forceinline__ bool c_skip(unsigned char c) { return c == ' ' || c == '\r' || c == '\n'; }

// strtol(s, NULL, 10): whitespace, sign, decimal digits; clamps to the long range
__device__ long long dev_strtol(const char* p, int n, int* end = nullptr) {
    int i = 0;
    while (i < n && c_space(p[i])) i++;
    bool neg = false;
    if (i < n && (p[i] == '+' || p[i] == '-')) { neg = p[i] == '-'; i++; }
    const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
    unsigned long long acc = 0;
    bool ovf = false, any = false;
    for (; i < n && c_digit(p[i]); i++) {
        const unsigned d = p[i] - '0';
        any = true;
        if (!ovf) {
            if (acc > (lim - d) / 10) ovf = true;
            else acc = acc * 10 + d;
        }
    }
    if (end) *end = any ? i : -1;
    if (ovf) return neg ? LLONG_MIN : LLONG_MAX;
    return neg ? (long long)(0ull - acc) : (long long)acc;
}

// one %d of sscanf: whitespace, sign, at least one digit; stored as int
__device__ bool scan_int(const char* p, int n, int* pos, int* v) {
    int end;
    long long x = dev_strtol(p + *pos, n - *pos, &end);
    if (end < 0) return false;
    *pos += end;
    *v = (int)(unsigned)(unsigned long long)x;
    return true;
}

// strtod front end: sign, up to 19 significant digits in w, decimal exponent
struct Dec {
    unsigned long long w;
    long long e10;
    bool neg, trunc;
    int kind;  // 0 number, 1 inf, 2 nan, 3 no conversion, 4 unsupported (hex, nan payload)
};
__device__ __forceinline__ unsigned char lower(unsigned char c) { return (c >= 'A' && c <= 'Z') ? c + 32 : c; }
__device__ bool match_word(const char* p, int n, int i, const char* w) {
    for (int k = 0; w[k]; k++)
        if (i + k >= n || lower(p[i + k]) != (unsigned char)w[k]) return false;
    return true;
}
__device__ Dec parse_dec(const char* p, int n) {
    Dec d{0ull, 0, false, false, 3};
    int i = 0;
    while (i < n && c_space(p[i])) i++;
    if (i < n && (p[i] == '+' || p[i] == '-')) { d.neg = p[i] == '-'; i++; }
    if (match_word(p, n, i, "inf")) { d.kind = 1; return d; }
    if (match_word(p, n, i, "nan")) { d.kind = (i + 3 < n && p[i + 3] == '(') ? 4 : 2; return d; }
    if (i + 1 < n && p[i] == '0' && (p[i + 1] == 'x' || p[i + 1] == 'X')) {
        const int j = i + 2;
        const bool hex = j < n && (c_digit(p[j]) || (lower(p[j]) >= 'a' && lower(p[j]) <= 'f') ||
                                   (p[j] == '.' && j + 1 < n && (c_digit(p[j + 1]) || (lower(p[j + 1]) >= 'a' && lower(p[j + 1]) <= 'f'))));
        if (hex) { d.kind = 4; return d; }
    }
    int nd = 0;
    long long eadj = 0;
    bool any = false;
    for (; i < n && c_digit(p[i]); i++) {
        any = true;
        const unsigned v = p[i] - '0';
        if (d.w == 0 && v == 0) continue;
        if (nd < 19) { d.w = d.w * 10 + v; nd++; }
        else { eadj++; if (v) d.trunc = true; }
    }
    if (i < n && p[i] == '.') {
        i++;
        for (; i < n && c_digit(p[i]); i++) {
            any = true;
            const unsigned v = p[i] - '0';
            if (d.w == 0 && v == 0) { eadj--; continue; }
            if (nd < 19) { d.w = d.w * 10 + v; nd++; eadj--; }
            else if (v) d.trunc = true;
        }
    }
    if (!any) return d;  // no conversion: 0.0
    d.kind = 0;
    if (i < n && (p[i] == 'e' || p[i] == 'E')) {
        int j = i + 1;
        bool eneg = false;
        if (j < n && (p[j] == '+' || p[j] == '-')) { eneg = p[j] == '-'; j++; }
        if (j < n && c_digit(p[j])) {
            long long ex = 0;
            for (; j < n && c_digit(p[j]); j++) ex = ex < 100000000 ? ex * 10 + (p[j] - '0') : ex;
            eadj += eneg ? -ex : ex;
        }
    }
    d.e10 = eadj;
    return d;
}

__device__ __forceinline__ double pow10_exact(int k) {  // 10^k for 0 <= k <= 22, exact in binary64
    double r = 1.0;
    for (int j = 0; j < k; j++) r *= 10.0;
    return r;
}
__device__ __forceinline__ float pow10f_exact(int k) {  // 10^k for 0 <= k <= 10, exact in binary32
    float r = 1.0f;
    for (int j = 0; j < k; j++) r *= 10.0f;
    return r;
}

// Clinger's fast path for doubles: true and *out when exact
__device__ bool fast_f64(const Dec& d, double* out) {
    if (d.kind == 1) { *out = d.neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll); return true; }
    if (d.kind == 2) { *out = __longlong_as_double(d.neg ? (long long)0xfff8000000000000ull : 0x7ff8000000000000ll); return true; }
    if (d.kind == 3) { *out = 0.0; return true; }
    if (d.w == 0) { *out = d.neg ? -0.0 : 0.0; return true; }
    if (d.trunc || d.w > (1ull << 53) || d.e10 < -22 || d.e10 > 22) return false;
    const double w = (double)d.w;
    double r = d.e10 >= 0 ? __dmul_rn(w, pow10_exact((int)d.e10)) : __ddiv_rn(w, pow10_exact((int)-d.e10));
    *out = d.neg ? -r : r;
    return true;
}
__device__ bool fast_f32(const Dec& d, float* out) {
    if (d.kind == 1) { *out = __int_as_float(d.neg ? (int)0xff800000u : 0x7f800000); return true; }
    if (d.kind == 2) { *out = __int_as_float(d.neg ? (int)0xffc00000u : 0x7fc00000); return true; }
    if (d.kind == 3) { *out = 0.0f; return true; }
    if (d.w == 0) { *out = d.neg ? -0.0f : 0.0f; return true; }
    if (d.trunc) return false;
    if (d.w <= (1ull << 24) && d.e10 >= -10 && d.e10 <= 10) {
        const float w = (float)d.w;
        float r = d.e10 >= 0 ? __fmul_rn(w, pow10f_exact((int)d.e10)) : __fdiv_rn(w, pow10f_exact((int)-d.e10));
        *out = d.neg ? -r : r;
        return true;
    }
    // exact double, then one rounding to float unless the double is a float midpoint
    double x;
    if (!fast_f64(d, &x)) return false;
    const float f = __double2float_rn(x);
    if (isinf(f) && !isinf(x)) return false;  // next to the overflow threshold: decide exactly
    if ((double)f != x) {
        const float g = nextafterf(f, (double)f < x ? INFINITY : -INFINITY);
        if (isfinite(g) && __dadd_rn((double)f, (double)g) * 0.5 == x) return false;
    }
    *out = f;
    return true;
}

// Field conversion by column type (loadItem, h_io.cc:164-181).
__device__ __forceinline__ void csv_convert(const CsvArgs& a, const CsvCol& c, int j, long long r, const char* f, int n,
                                            unsigned long long off) {
    switch (c.typ) {
    case H_B: ((bool*)c.out)[r] = (int)(unsigned)(unsigned long long)dev_strtol(f, n) != 0; break;
    case H_J: ((int8_t*)c.out)[r] = (int8_t)(int)(unsigned)(unsigned long long)dev_strtol(f, n); break;
    case H_H: ((int16_t*)c.out)[r] = (int16_t)(int)(unsigned)(unsigned long long)dev_strtol(f, n); break;
    case H_I: ((int32_t*)c.out)[r] = (int32_t)(unsigned)(unsigned long long)dev_strtol(f, n); break;
    case H_L: ((long long*)c.out)[r] = dev_strtol(f, n); break;
    case H_C: ((char*)c.out)[r] = n > 0 ? f[0] : 0; break;
    case H_D: {  // sscanf(s, "%d-%d-%d") -> a*10000 + b*100 + c
        int pos = 0, y, m, dd;
        bool ok = scan_int(f, n, &pos, &y) && pos < n && f[pos] == '-' && (pos++, scan_int(f, n, &pos, &m)) &&
                  pos < n && f[pos] == '-' && (pos++, scan_int(f, n, &pos, &dd));
        if (!ok) { atomicOr(a.err, CSV_DATE); atomicMin(a.err + 1, row32(r)); break; }
        ((int32_t*)c.out)[r] = (int32_t)((unsigned)y * 10000u + (unsigned)m * 100u + (unsigned)dd);
        break;
    }
    case H_E:
    case H_F: {
        const Dec d = parse_dec(f, n);
        if (d.kind == 4) { atomicOr(a.err, CSV_HEXNAN); atomicMin(a.err + 1, row32(r)); break; }
        bool done;
        if (c.typ == H_E) { double v; done = fast_f64(d, &v); if (done) ((double*)c.out)[r] = v; }
        else { float v; done = fast_f32(d, &v); if (done) ((float*)c.out)[r] = v; }
        if (!done) {
            const unsigned k = atomicAdd(a.nslow, 1u);
            if (k < a.slow_cap) {
                a.slow[2 * k] = (off << 16) | (unsigned long long)n;
                a.slow[2 * k + 1] = ((unsigned long long)r << 16) | (unsigned long long)j;
            } else {
                atomicOr(a.err, CSV_SLOWFULL);
            }
        }
        break;
    }
    default:  // H_Q, H_S: the field's span for the symbol and string passes
        ((unsigned long long*)c.out)[r] = (off << 16) | (unsigned long long)n;
        break;
    }
}

// One warp per batch of 32 consecutive lines.  Phase A: lane i scans line i
// in aligned 16-byte words, finding separators (and NULs) four bytes at a
// time with byte-wise compares, and records each field's (start, length) in
// shared memory.  Phase B converts column by column, lane i taking line i,
// so every lane runs the same conversion and a column's stores are
// contiguous.  A separator that getField's trimming could remove (' ',
// '\r', '\n') needs the line's trimmed bounds first, so such lines are
// scanned twice.
__device__ __forceinline__ unsigned byte_mask(long long o, long long lo, long long hi) {
    // 0xff in each byte k of the word at offset o with lo <= o + k < hi
    const long long a = lo - o > 0 ? lo - o : 0, b = hi - o < 4 ? hi - o : 4;
    if (b <= a) return 0u;
    const unsigned long long top = (1ull << (8 * b)) - 1ull, low = (1ull << (8 * a)) - 1ull;
    return (unsigned)(top & ~low);
}

__global__ void k_csv_parse(CsvArgs a) {
    extern __shared__ unsigned csv_fields[];
    const int warp = threadIdx.x >> 5, lane = lane_id();
    const int nc = a.ncols;
    unsigned* fld = csv_fields + (size_t)warp * 32 * nc;  // [32][nc]: start << 16 | length (within the line)
    const int warps = (int)((blockDim.x >> 5) * gridDim.x);
    const unsigned sep4 = 0x01010101u * (unsigned char)a.sep;
    const bool sep_trimmed = a.sep == ' ' || a.sep == '\r' || a.sep == '\n';
    for (long long base = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * 32; base < a.rows; base += (long long)warps * 32) {
        const long long myrow = base + lane;
        long long ms = 0, me = 0;
        bool ok = myrow < a.rows;
        if (ok) {
            const long long li = myrow + a.first_line;
            ms = li == 0 ? 0 : a.nl[li - 1] + 1;
            const bool has_nl = li < a.nnl;
            me = has_nl ? a.nl[li] : a.size;
            if (me - ms + (has_nl ? 1 : 0) > a.maxline - 1) {
                atomicOr(a.err, CSV_LONG);
                atomicMin(a.err + 1, row32(myrow));
                ok = false;
            }
        }
        // ---- phase A
        if (ok) {
            long long ls = ms, le = me;  // getField's trimmed bounds, needed only when the separator is trimmable
            if (sep_trimmed) {
                long long first = me, last = ms - 1;
                for (long long q = ms & ~15LL; q < me; q += 16) {
                    const uint4 v = *(const uint4*)(a.buf + q);
                    const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int t = 0; t < 4; t++) {
                        const long long o = q + 4 * t;
                        const unsigned valid = byte_mask(o, ms, me);
                        const unsigned notsp = ~__vcmpeq4(w[t], 0x20202020u) & valid;
                        const unsigned notskip = ~(__vcmpeq4(w[t], 0x20202020u) | __vcmpeq4(w[t], 0x0d0d0d0du) |
                                                   __vcmpeq4(w[t], 0x0a0a0a0au)) & valid;
                        if (notsp && first == me) first = o + ((__ffs(notsp) - 1) >> 3);
                        if (notskip) last = o + ((31 - __clz(notskip)) >> 3);
                    }
                }
                ls = first;
                le = last + 1;
                if (ls >= le) { ls = ms; le = ms; }
            }
            int nf = 0;
            long long start = ls;
            bool nul = false;
            for (long long q = ms & ~15LL; q < me; q += 16) {
                const uint4 v = *(const uint4*)(a.buf + q);
                const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const long long o = q + 4 * t;
                    nul |= (__vcmpeq4(w[t], 0u) & byte_mask(o, ms, me)) != 0u;
                    unsigned m = __vcmpeq4(w[t], sep4) & byte_mask(o, ls, le);
                    while (m) {
                        const int bb = __ffs(m) - 1;
                        const long long pos = o + (bb >> 3);
                        if (nf < nc) fld[lane * nc + nf] = ((unsigned)(start - ms) << 16) | (unsigned)(pos - start);
                        nf++;
                        start = pos + 1;
                        m &= ~(0xffu << (bb & ~7));
                    }
                }
            }
            if (a.sep == ' ') {  // getField also loads the remainder after the last ' '
                if (nf < nc) fld[lane * nc + nf] = ((unsigned)(start - ms) << 16) | (unsigned)(le > start ? le - start : 0);
                nf++;
            }
            if (nul) {
                atomicOr(a.err, CSV_NUL);
                atomicMin(a.err + 1, row32(myrow));
                ok = false;
            } else if (nf != nc) {
                atomicOr(a.err, CSV_FIELDS);
                atomicMin(a.err + 1, row32(myrow));
                ok = false;
            }
        }
        __syncwarp();
        // ---- phase B
        for (int j = 0; j < nc; j++) {
            const CsvCol c = a.cols[j];
            if (ok) {
                const unsigned f = fld[lane * nc + j];
                int fb = (int)(f >> 16), fe = fb + (int)(f & 0xffffu);
                const char* p = a.buf + ms;
                while (fb < fe && p[fb] == ' ') fb++;  // trimSelf
                while (fe > fb && c_skip((unsigned char)p[fe - 1])) fe--;
                csv_convert(a, c, j, myrow, p + fb, fe - fb, (unsigned long long)(ms + fb));
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------- exact decimal conversion
// Big unsigned integers of up to BIG_LIMBS 32-bit limbs, little endian.  A
// decimal of up to 800 significant digits (more only add a sticky bit: a
// binary64 midpoint has at most 767 significant digits, so digits beyond the
// 800th cannot move the value across one) scaled by 2^s or 10^k fits 4096 bits.
constexpr int BIG_LIMBS = 128;
constexpr int MAX_SIG = 800;
struct Big {
    unsigned v[BIG_LIMBS];
    int n;  // limbs in use (v[n-1] != 0 unless n == 0)
};
__device__ void big_set(Big& b, unsigned long long x) {
    b.n = 0;
    while (x) { b.v[b.n++] = (unsigned)x; x >>= 32; }
}
__device__ void big_mul_small(Big& b, unsigned m) {
    unsigned long long carry = 0;
    for (int i = 0; i < b.n; i++) {
        const unsigned long long t = (unsigned long long)b.v[i] * m + carry;
        b.v[i] = (unsigned)t;
        carry = t >> 32;
    }
    if (carry && b.n < BIG_LIMBS) b.v[b.n++] = (unsigned)carry;
}
__device__ void big_add_small(Big& b, unsigned a) {
    unsigned long long carry = a;
    for (int i = 0; i < b.n && carry; i++) {
        const unsigned long long t = (unsigned long long)b.v[i] + carry;
        b.v[i] = (unsigned)t;
        carry = t >> 32;
    }
    if (carry && b.n < BIG_LIMBS) b.v[b.n++] = (unsigned)carry;
}
__device__ void big_mul_pow10(Big& b, int k) {
    while (k >= 9) { big_mul_small(b, 1000000000u); k -= 9; }
    unsigned m = 1;
    while (k-- > 0) m *= 10;
    if (m != 1) big_mul_small(b, m);
}
__device__ int big_bitlen(const Big& b) { return b.n == 0 ? 0 : 32 * (b.n - 1) + (32 - __clz(b.v[b.n - 1])); }
__device__ void big_shl(Big& b, int s) {
    if (b.n == 0 || s == 0) return;
    const int w = s >> 5, r = s & 31;
    int nn = b.n + w + 1;
    if (nn > BIG_LIMBS) nn = BIG_LIMBS;
    for (int i = nn - 1; i >= 0; i--) {
        const int j = i - w;
        unsigned hi = (j >= 0 && j < b.n) ? b.v[j] : 0u;
        unsigned lo = (j - 1 >= 0 && j - 1 < b.n) ? b.v[j - 1] : 0u;
        b.v[i] = r ? (hi << r) | (lo >> (32 - r)) : hi;
    }
    b.n = nn;
    while (b.n > 0 && b.v[b.n - 1] == 0) b.n--;
}
__device__ void big_shr1(Big& b) {
    for (int i = 0; i < b.n; i++) b.v[i] = (b.v[i] >> 1) | (i + 1 < b.n ? b.v[i + 1] << 31 : 0u);
    while (b.n > 0 && b.v[b.n - 1] == 0) b.n--;
}
__device__ int big_cmp(const Big& a, const Big& b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (int i = a.n - 1; i >= 0; i--)
        if (a.v[i] != b.v[i]) return a.v[i] < b.v[i] ? -1 : 1;
    return 0;
}
__device__ void big_sub(Big& a, const Big& b) {  // a -= b, a >= b
    long long borrow = 0;
    for (int i = 0; i < a.n; i++) {
        long long t = (long long)a.v[i] - (i < b.n ? (long long)b.v[i] : 0) - borrow;
        borrow = t < 0;
        a.v[i] = (unsigned)(t + (borrow << 32));
    }
    while (a.n > 0 && a.v[a.n - 1] == 0) a.n--;
}
__device__ bool big_low_bits_nonzero(const Big& b, int k) {  // any of bits [0, k)
    for (int i = 0; i < b.n && 32 * i < k; i++) {
        const int take = k - 32 * i;
        const unsigned m = take >= 32 ? 0xffffffffu : ((1u << take) - 1u);
        if (b.v[i] & m) return true;
    }
    return false;
}
__device__ unsigned long long big_bits(const Big& b, int lo, int cnt) {  // bits [lo, lo + cnt), cnt <= 64
    unsigned long long r = 0;
    for (int k = 0; k < cnt; k++) {
        const int bit = lo + k, i = bit >> 5;
        if (i < b.n && ((b.v[i] >> (bit & 31)) & 1u)) r |= 1ull << k;
    }
    return r;
}

// value = m * 2^u, m < 2^(p+1) already rounded to p bits (or fewer when subnormal)
__device__ unsigned long long encode(unsigned long long m, int u, int p, int bias, bool* inf) {
    *inf = false;
    if (m == 0) return 0;
    const int top = 63 - __clzll(m), lead = top + u;  // exponent of the leading bit
    if (lead > bias) { *inf = true; return 0; }
    if (lead < 1 - bias) return m;  // subnormal: u is the subnormal unit, m < 2^(p-1)
    if (top < p - 1) m <<= (p - 1 - top);  // leading bit to the implicit position
    const unsigned long long frac = m & ((1ull << (p - 1)) - 1ull);
    return ((unsigned long long)(lead + bias) << (p - 1)) | frac;
}

// Correctly rounded binary64 (p = 53) or binary32 (p = 24) value of the
// decimal text, returned as its bit pattern (round to nearest, ties to even).
__device__ unsigned long long exact_decimal(const char* p_, int n, int p, Big& D, Big& A, Big& T) {
    const int bias = p == 53 ? 1023 : 127, emin = 1 - bias;
    const unsigned long long sign_bit = p == 53 ? (1ull << 63) : (1ull << 31);
    const unsigned long long inf_bits = p == 53 ? 0x7ff0000000000000ull : 0x7f800000ull;
    int i = 0;
    while (i < n && c_space(p_[i])) i++;
    bool neg = false;
    if (i < n && (p_[i] == '+' || p_[i] == '-')) { neg = p_[i] == '-'; i++; }
    const unsigned long long sgn = neg ? sign_bit : 0ull;
    // digits into D (in 9-digit chunks), exponent, sticky
    big_set(D, 0);
    int nd = 0;
    long long e10 = 0;
    bool trunc = false;
    unsigned chunk = 0;
    int cl = 0;
    auto push = [&](unsigned v) {
        chunk = chunk * 10 + v;
        if (++cl == 9) { big_mul_small(D, 1000000000u); big_add_small(D, chunk); chunk = 0; cl = 0; }
    };
    for (; i < n && c_digit(p_[i]); i++) {
        const unsigned v = p_[i] - '0';
        if (nd == 0 && v == 0) continue;
        if (nd < MAX_SIG) { push(v); nd++; }
        else { e10++; if (v) trunc = true; }
    }
    if (i < n && p_[i] == '.') {
        i++;
        for (; i < n && c_digit(p_[i]); i++) {
            const unsigned v = p_[i] - '0';
            if (nd == 0 && v == 0) { e10--; continue; }
            if (nd < MAX_SIG) { push(v); nd++; e10--; }
            else if (v) trunc = true;
        }
    }
    if (cl) {
        unsigned m = 1;
        for (int k = 0; k < cl; k++) m *= 10;
        big_mul_small(D, m);
        big_add_small(D, chunk);
    }
    if (i < n && (p_[i] == 'e' || p_[i] == 'E')) {
        int j = i + 1;
        bool eneg = false;
        if (j < n && (p_[j] == '+' || p_[j] == '-')) { eneg = p_[j] == '-'; j++; }
        if (j < n && c_digit(p_[j])) {
            long long ex = 0;
            for (; j < n && c_digit(p_[j]); j++) ex = ex < 100000000 ? ex * 10 + (p_[j] - '0') : ex;
            e10 += eneg ? -ex : ex;
        }
    }
    if (nd == 0) return sgn;  // zero
    const long long dexp = nd + e10;  // value in [10^(dexp-1), 10^dexp)
    if (dexp > (p == 53 ? 310 : 40)) return sgn | inf_bits;
    if (dexp < (p == 53 ? -324 : -46)) return sgn;
    bool inf;
    unsigned long long bits;
    if (e10 >= 0) {
        big_mul_pow10(D, (int)e10);
        const int L = big_bitlen(D);
        if (L <= p) {  // exact integer (no truncated digits possible here)
            bits = encode(big_bits(D, 0, L), 0, p, bias, &inf);
        } else {
            const int sh = L - p - 1;
            const unsigned long long q = big_bits(D, sh, p + 1);
            const bool sticky = trunc || big_low_bits_nonzero(D, sh);
            unsigned long long m = q >> 1;
            if ((q & 1ull) && (sticky || (m & 1ull))) m++;
            int u = sh + 1;
            if (m == (1ull << p)) { m >>= 1; u++; }
            bits = encode(m, u, p, bias, &inf);
        }
        return inf ? (sgn | inf_bits) : (sgn | bits);
    }
    // value = D / 10^k: q = floor(D * 2^s / 10^k) with p + 1 bits (fewer when subnormal)
    const int k = (int)-e10;
    const int smax = p - emin;  // result unit 2^(1 - s) never below the subnormal unit
    big_set(T, 1);
    big_mul_pow10(T, k);  // T = 10^k
    const int bq = big_bitlen(T);
    int s = p + bq - big_bitlen(D);
    if (s > smax) s = smax;
    unsigned long long q = 0;
    for (int attempt = 0; attempt < 3; attempt++) {
        // A = D * 2^max(s,0); T' = 10^k * 2^max(-s,0) * 2^(p+2)
        A = D;
        if (s > 0) big_shl(A, s);
        big_set(T, 1);
        big_mul_pow10(T, k);
        if (s < 0) big_shl(T, -s);
        big_shl(T, p + 2);
        q = 0;
        for (int b = p + 2; b >= 0; b--) {
            if (big_cmp(A, T) >= 0) { big_sub(A, T); q |= 1ull << b; }
            big_shr1(T);
        }
        if (s < smax && q < (1ull << p)) { s++; continue; }
        if (q >= (1ull << (p + 1))) { s--; continue; }
        break;
    }
    const bool sticky = trunc || A.n != 0;
    unsigned long long m = q >> 1;
    if ((q & 1ull) && (sticky || (m & 1ull))) m++;
    int u = 1 - s;
    if (m == (1ull << p)) { m >>= 1; u++; }
    bits = encode(m, u, p, bias, &inf);
    return inf ? (sgn | inf_bits) : (sgn | bits);
}

__global__ void k_csv_slow(const char* __restrict__ buf, const unsigned long long* __restrict__ slow, unsigned nslow,
                           const CsvCol* __restrict__ cols, Big* __restrict__ work) {
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < nslow; t += gridDim.x * blockDim.x) {
        const unsigned long long span = slow[2 * t], meta = slow[2 * t + 1];
        const char* f = buf + (span >> 16);
        const int n = (int)(span & 0xffffull);
        const long long r = (long long)(meta >> 16);
        const int j = (int)(meta & 0xffffull);
        const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
        Big* w = work + 3ull * g;
        if (cols[j].typ == H_E) ((unsigned long long*)cols[j].out)[r] = exact_decimal(f, n, 53, w[0], w[1], w[2]);
        else ((unsigned*)cols[j].out)[r] = (unsigned)exact_decimal(f, n, 24, w[0], w[1], w[2]);
    }
}

// ---------------------------------------------------------- symbols, strings
__device__ __forceinline__ unsigned long long span_hash(const char* buf, unsigned long long span) {
    // FNV-1a, 64-bit
    const char* f = buf + (span >> 16);
    const int n = (int)(span & 0xffffull);
    unsigned long long h = 0xcbf29ce484222325ull;
    for (int k = 0; k < n; k++) h = (h ^ (unsigned char)f[k]) * 0x100000001b3ull;
    return h == ~0ull ? h - 1 : h;
}
// first-occurrence table: key = text hash, value = smallest row
__global__ void k_sym_insert(const char* __restrict__ buf, const unsigned long long* __restrict__ spans, long long rows,
                             unsigned long long* __restrict__ keys, unsigned long long* __restrict__ first,
                             unsigned long long mask, unsigned* derr) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = span_hash(buf, spans[r]);
        unsigned long long sl = (h * 0x9e3779b97f4a7c15ull) >> 20 & mask;
        for (unsigned long long p = 0; p <= mask; p++) {
            unsigned long long cur = *(volatile unsigned long long*)(keys + sl);
            if (cur == ~0ull) cur = atomicCAS(keys + sl, ~0ull, h);
            if (cur == ~0ull || cur == h) {
                // most rows of a repeated text find a smaller row there already
                if (*(volatile unsigned long long*)(first + sl) > (unsigned long long)r) atomicMin(first + sl, (unsigned long long)r);
                break;
            }
            sl = (sl + 1) & mask;
            if (p == mask) atomicOr(derr, DERR_CAPACITY);
        }
    }
}
__global__ void k_sym_rep(const char* __restrict__ buf, const unsigned long long* __restrict__ spans, long long rows,
                          const unsigned long long* __restrict__ keys, const unsigned long long* __restrict__ first,
                          unsigned long long mask, long long* __restrict__ rep, uint8_t* __restrict__ is_first) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = span_hash(buf, spans[r]);
        unsigned long long sl = (h * 0x9e3779b97f4a7c15ull) >> 20 & mask;
        long long f = r;
        for (unsigned long long p = 0; p <= mask; p++) {
            if (keys[sl] == h) { f = (long long)first[sl]; break; }
            sl = (sl + 1) & mask;
        }
        rep[r] = f;
        is_first[r] = f == r;
    }
}
// distinct texts, NUL-terminated, packed at offs[k] (pinned host blob)
__global__ void k_sym_pack(const char* __restrict__ buf, const unsigned long long* __restrict__ spans,
                           const long long* __restrict__ drows, long long nd, const unsigned long long* __restrict__ offs,
                           char* __restrict__ blob, unsigned* __restrict__ dpos) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nd; k += (long long)gridDim.x * blockDim.x) {
        const long long r = drows[k];
        const unsigned long long sp = spans[r];
        const char* f = buf + (sp >> 16);
        const int n = (int)(sp & 0xffffull);
        char* o = blob + offs[k];
        for (int i = 0; i < n; i++) o[i] = f[i];
        o[n] = 0;
        dpos[r] = (unsigned)k;
    }
}
__global__ void k_sym_lengths(const unsigned long long* __restrict__ spans, const long long* __restrict__ drows, long long nd,
                              unsigned* __restrict__ lens) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nd; k += (long long)gridDim.x * blockDim.x)
        lens[k] = (unsigned)(spans[drows[k]] & 0xffffull) + 1u;
}
// ids per row, and the row's text checked against its representative's
__global__ void k_sym_ids(const char* __restrict__ buf, const unsigned long long* __restrict__ spans, long long rows,
                          const long long* __restrict__ rep, const unsigned* __restrict__ dpos,
                          const long long* __restrict__ ids, long long* __restrict__ out, unsigned* __restrict__ bad) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
        const long long f = rep[r];
        out[r] = ids[dpos[f]];
        if (f != r) {
            const unsigned long long a = spans[r], b = spans[f];
            bool same = (a & 0xffffull) == (b & 0xffffull);
            const char *pa = buf + (a >> 16), *pb = buf + (b >> 16);
            for (int i = 0; same && i < (int)(a & 0xffffull); i++) same = pa[i] == pb[i];
            if (!same) atomicOr(bad, 1u);
        }
    }
}
__global__ void k_str_lengths(const unsigned long long* __restrict__ spans, long long rows, unsigned* __restrict__ lens) {
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x)
        lens[r] = (unsigned)(spans[r] & 0xffffull) + 1u;
}
// texts packed NUL-terminated into a device blob (one warp per 32 rows, a
// lane per byte of each text), and each row's pointer into the host copy
__global__ void k_str_pack(const char* __restrict__ buf, const unsigned long long* __restrict__ spans, long long rows,
                           const unsigned long long* __restrict__ offs, char* __restrict__ dblob,
                           unsigned long long host_base, unsigned long long* __restrict__ ptrs,
                           unsigned long long* __restrict__ bspans) {
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = lane_id();
    for (long long base = w0 * 32; base < rows; base += nw * 32) {
        const long long mine = base + lane;
        if (mine < rows) {
            ptrs[mine] = host_base + offs[mine];
            bspans[mine] = (offs[mine] << 16) | (spans[mine] & 0xffffull);  // the text within the device blob
        }
        const long long last = base + 32 < rows ? base + 32 : rows;
        for (long long r = base; r < last; r++) {
            const unsigned long long sp = spans[r];
            const char* f = buf + (sp >> 16);
            const int n = (int)(sp & 0xffffull);
            char* o = dblob + offs[r];
            for (int i = lane; i <= n; i += 32) o[i] = i < n ? f[i] : 0;
        }
    }
}

unsigned grid_of(long long n) {
    unsigned g = grid_for(n, 256);
    return g > (unsigned)g_sms * 16 ? (unsigned)g_sms * 16 : g;
}

I csv_symbols(const char* dbuf, const unsigned long long* spans, long long rows, long long* out) {
    unsigned long long cap = 1024;
    while (cap < 2ull * (unsigned long long)rows) cap <<= 1;
    unsigned long long* keys = (unsigned long long*)salloc(cap * 8);
    unsigned long long* first = (unsigned long long*)salloc(cap * 8);
    long long* rep = (long long*)salloc((size_t)rows * 8);
    uint8_t* isf = (uint8_t*)salloc((size_t)rows);
    long long* drows = (long long*)salloc((size_t)rows * 8);
    unsigned* dpos = (unsigned*)salloc((size_t)rows * 4);
    unsigned* bad = (unsigned*)salloc(16);
    if (!keys || !first || !rep || !isf || !drows || !dpos || !bad) return E_DEVICE_OOM;
    HG_CU(cudaMemsetAsync(keys, 0xff, cap * 8, g_stream));
    HG_CU(cudaMemsetAsync(first, 0xff, cap * 8, g_stream));
    HG_CU(cudaMemsetAsync(bad, 0, 4, g_stream));
    HG_LAUNCH("sym_insert", grid_of(rows), 256, 0, k_sym_insert, dbuf, spans, rows, keys, first, cap - 1, g_derr);
    HG_LAUNCH("sym_rep", grid_of(rows), 256, 0, k_sym_rep, dbuf, spans, rows, keys, first, cap - 1, rep, isf);
    HG_CHECK(last_launch_error());
    long long nd = 0;
    HG_CHECK(compact_rows(isf, rows, drows, &nd));
    unsigned* lens = (unsigned*)salloc((size_t)(nd > 0 ? nd : 1) * 4);
    unsigned long long* offs = (unsigned long long*)salloc((size_t)(nd + 1) * 8);
    if (!lens || !offs) return E_DEVICE_OOM;
    unsigned long long total = 0;
    if (nd > 0) {
        HG_LAUNCH("sym_lengths", grid_of(nd), 256, 0, k_sym_lengths, spans, drows, nd, lens);
        HG_CHECK(scan_exclusive(lens, nd, offs, &total));
    }
    char* blob = (char*)halloc(total > 0 ? total : 1);
    if (!blob) return E_DEVICE_OOM;
    if (nd > 0) HG_LAUNCH("sym_pack", grid_of(nd), 256, 0, k_sym_pack, dbuf, spans, drows, nd, offs, blob, dpos);
    std::vector<unsigned long long> hoffs((size_t)nd);
    if (nd > 0) HG_CU(cudaMemcpyAsync(hoffs.data(), offs, (size_t)nd * 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(stream_sync());
    HG_CHECK(last_launch_error());
    // interning in first-occurrence order, as loadItem's getSymbol calls meet the texts
    std::vector<L> ids((size_t)nd);
    for (long long k = 0; k < nd; k++) ids[k] = getSymbol(blob + hoffs[k]);
    long long* dids = (long long*)salloc((size_t)(nd > 0 ? nd : 1) * 8);
    if (!dids) return E_DEVICE_OOM;
    if (nd > 0) HG_CU(cudaMemcpyAsync(dids, ids.data(), (size_t)nd * 8, cudaMemcpyHostToDevice, g_stream));
    HG_LAUNCH("sym_ids", grid_of(rows), 256, 0, k_sym_ids, dbuf, spans, rows, rep, dpos, dids, out, bad);
    unsigned hb = 0;
    HG_CHECK(rb_queue(&hb, bad, 4));
    HG_CHECK(check_device_errors());
    if (hb) return set_error(E_GENERAL, "readCSV: two symbol texts share a 64-bit hash");
    return 0;
}

I csv_strings(const char* dbuf, const unsigned long long* spans, long long rows, S** ptrs_out) {
    unsigned* lens = (unsigned*)salloc((size_t)rows * 4);
    unsigned long long* offs = (unsigned long long*)salloc((size_t)(rows + 1) * 8);
    if (!lens || !offs) return E_DEVICE_OOM;
    HG_LAUNCH("str_lengths", grid_of(rows), 256, 0, k_str_lengths, spans, rows, lens);
    unsigned long long total = 0;
    HG_CHECK(scan_exclusive(lens, rows, offs, &total));
    char* blob = (char*)halloc(total > 0 ? total : 1);
    S* ptrs = (S*)halloc((size_t)rows * sizeof(S));
    // the device copy stays (output arena) so @like can read the column in HBM
    char* dblob = (char*)dalloc(total > 0 ? total : 1);
    unsigned long long* bspans = (unsigned long long*)dalloc((size_t)rows * 8);
    unsigned long long* dptrs = (unsigned long long*)salloc((size_t)rows * 8);
    if (!blob || !ptrs || !dblob || !bspans || !dptrs) return E_DEVICE_OOM;
    HG_LAUNCH("str_pack", grid_of(rows * 32), 256, 0, k_str_pack, dbuf, spans, rows, offs, dblob,
              (unsigned long long)(uintptr_t)blob, dptrs, bspans);
    HG_CU(cudaMemcpyAsync(blob, dblob, total, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(cudaMemcpyAsync(ptrs, dptrs, (size_t)rows * 8, cudaMemcpyDeviceToHost, g_stream));
    HG_CU(stream_sync());
    HG_CHECK(last_launch_error());
    if (rows > 1) register_strings(ptrs, rows, dblob, bspans);
    *ptrs_out = ptrs;
    return 0;
}

I read_csv(V z, S fileName, L numCols, L* types, Q* symList) {
    if (numCols <= 0 || numCols > CSV_MAXCOLS) return set_error(E_NOT_IMPL, "readCSV: %lld columns", numCols);
    if (LINE_MAX_CHAR < 2 || LINE_MAX_CHAR > CSV_MAXLINE)
        return set_error(E_NOT_IMPL, "readCSV: LINE_MAX_CHAR %lld outside [2, %d]", LINE_MAX_CHAR, CSV_MAXLINE);
    for (L j = 0; j < numCols; j++) {
        const I t = (I)types[j];
        if (!(t == H_B || t == H_J || t == H_H || t == H_I || t == H_L || t == H_F || t == H_E || t == H_C || t == H_Q ||
              t == H_S || t == H_D))
            return set_error(E_NOT_IMPL, "readCSV: column %lld of type %d (loadItem has no conversion)", j, t);
    }
    FILE* fp = fopen(fileName, "rb");
    if (!fp) return set_error(E_GENERAL, "readCSV: cannot open %s", fileName);
    fseek(fp, 0, SEEK_END);
    const long long size = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (size < 0) { fclose(fp); return io_fail("readCSV: cannot size the file"); }
    char* dbuf = (char*)salloc((size_t)size + 64);
    if (!dbuf) { fclose(fp); return E_DEVICE_OOM; }
    I e = stream_in_par(fp, dbuf, (size_t)size);
    fclose(fp);
    if (e) return e;
    // newline positions
    const long long ntiles = (size + NL_TILE - 1) / NL_TILE;
    unsigned* counts = (unsigned*)salloc((size_t)(ntiles > 0 ? ntiles : 1) * 4);
    unsigned long long* toffs = (unsigned long long*)salloc((size_t)(ntiles + 1) * 8);
    if (!counts || !toffs) return E_DEVICE_OOM;
    long long nnl = 0;
    long long* nl = nullptr;
    if (ntiles > 0) {
        HG_LAUNCH("csv_nl_count", (unsigned)ntiles, NL_THREADS, 0, k_nl_count, dbuf, size, counts);
        HG_CHECK(scan_counts(counts, ntiles, toffs));
        unsigned long long h = 0;
        HG_CHECK(rb_queue(&h, toffs + ntiles, 8));
        HG_CU(stream_sync());
        nnl = (long long)h;
        nl = (long long*)salloc((size_t)(nnl > 0 ? nnl : 1) * 8);
        if (!nl) return E_DEVICE_OOM;
        HG_LAUNCH("csv_nl_scatter", (unsigned)ntiles, NL_THREADS, 0, k_nl_scatter, dbuf, size, toffs, nl);
        HG_CHECK(last_launch_error());
    }
    char last = '\n';
    if (size > 0) HG_CU(cudaMemcpy(&last, dbuf + size - 1, 1, cudaMemcpyDeviceToHost));
    const long long lines = nnl + (size > 0 && last != '\n' ? 1 : 0);
    const long long first_line = (LINE_HEADER && lines > 0) ? 1 : 0;
    const long long rows = lines - first_line;
    // columns
    std::vector<CsvCol> hc((size_t)numCols);
    std::vector<void*> spans((size_t)numCols, nullptr);
    for (L j = 0; j < numCols; j++) {
        const I t = (I)types[j];
        const size_t es = (t == H_Q || t == H_S) ? 8 : (size_t)esize(t);
        void* d = (t == H_Q || t == H_S) ? salloc((size_t)(rows > 0 ? rows : 1) * 8)
                                         : dalloc((size_t)(rows > 1 ? rows : 2) * es + (t == H_C ? 1 : 0));
        if (!d) return E_DEVICE_OOM;
        hc[j].typ = t;
        hc[j].out = d;
        if (t == H_Q || t == H_S) spans[j] = d;
    }
    CsvCol* dcols = (CsvCol*)salloc(sizeof(CsvCol) * (size_t)numCols);
    unsigned* err = (unsigned*)salloc(16);
    const unsigned slow_cap = 1u << 22;
    unsigned long long* slow = (unsigned long long*)salloc((size_t)slow_cap * 16);
    unsigned* nslow = (unsigned*)salloc(16);
    if (!dcols || !err || !slow || !nslow) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(dcols, hc.data(), sizeof(CsvCol) * (size_t)numCols, cudaMemcpyHostToDevice, g_stream));
    const unsigned init_err[2] = {0u, 0xffffffffu};
    HG_CU(cudaMemcpyAsync(err, init_err, 8, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemsetAsync(nslow, 0, 4, g_stream));
    if (rows > 0) {
        CsvArgs a{dbuf, size, nl, nnl, first_line, rows, (int)numCols, (char)LINE_SEP, (int)LINE_MAX_CHAR, dcols,
                  err, slow, nslow, slow_cap};
        const size_t per_warp = (size_t)(32 * numCols) * 4;
        int wpb = (int)(98304 / per_warp);
        wpb = wpb > 8 ? 8 : wpb < 1 ? 1 : wpb;
        const size_t smem = per_warp * (size_t)wpb;
        HG_CU(cudaFuncSetAttribute(k_csv_parse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        long long blocks = (rows + 32LL * wpb - 1) / (32LL * wpb);
        if (blocks > (long long)g_sms * 16) blocks = (long long)g_sms * 16;
        HG_LAUNCH("csv_parse", (unsigned)blocks, wpb * 32, smem, k_csv_parse, a);
        HG_CHECK(last_launch_error());
    }
    unsigned herr[2], hslow = 0;
    HG_CHECK(rb_queue(herr, err, 8));
    HG_CHECK(rb_queue(&hslow, nslow, 4));
    HG_CU(stream_sync());
    if (herr[0]) {
        const long long line = (long long)herr[1] + first_line + 1;
        const char* why = (herr[0] & CSV_FIELDS)   ? "a line whose field count differs from the column count"
                          : (herr[0] & CSV_LONG)   ? "a line longer than LINE_MAX_CHAR - 1 characters"
                          : (herr[0] & CSV_NUL)    ? "a NUL byte"
                          : (herr[0] & CSV_DATE)   ? "a date that %d-%d-%d cannot read"
                          : (herr[0] & CSV_HEXNAN) ? "a hexadecimal float or a nan(...) payload"
                                                   : "too many long decimals";
        return set_error(herr[0] & (CSV_HEXNAN | CSV_SLOWFULL) ? E_NOT_IMPL : E_GENERAL, "readCSV: %s (line %lld)", why, line);
    }
    if (hslow > 0) {
        const unsigned want = hslow < 65536u ? hslow : 65536u, blocks = (want + 127) / 128;
        Big* work = (Big*)salloc((size_t)blocks * 128 * 3 * sizeof(Big));  // three per launched thread
        if (!work) return E_DEVICE_OOM;
        HG_LAUNCH("csv_slow", blocks, 128, 0, k_csv_slow, dbuf, slow, hslow, dcols, work);
        HG_CHECK(last_launch_error());
    }
    // symbols and strings
    std::vector<V0> colv((size_t)numCols);
    for (L j = 0; j < numCols; j++) {
        const I t = (I)types[j];
        V0& c = colv[j];
        memset(&c, 0, sizeof(V0));
        c.typ = t;
        c.len = rows;
        if (t == H_Q) {
            long long* ids = (long long*)dalloc((size_t)(rows > 1 ? rows : 2) * 8);
            if (!ids) return E_DEVICE_OOM;
            if (rows > 0) HG_CHECK(csv_symbols(dbuf, (const unsigned long long*)spans[j], rows, ids));
            c.g = (G)ids;
        } else if (t == H_S) {
            S* ptrs = nullptr;
            if (rows > 0) HG_CHECK(csv_strings(dbuf, (const unsigned long long*)spans[j], rows, &ptrs));
            c.g = (G)ptrs;
        } else {
            c.g = (G)hc[j].out;
        }
        if (rows <= 1) {  // length-0/1 vectors are inline (initV)
            uint64_t bits = 0;
            if (rows == 1) {
                if (t == H_S) bits = (uint64_t)(uintptr_t)((S*)c.g)[0];
                else HG_CU(cudaMemcpy(&bits, c.g, (size_t)esize(t), cudaMemcpyDeviceToHost));
            }
            c.i64 = (L)bits;
            c.g = (G)&c.b;
        }
    }
    HG_CHECK(check_device_errors());
    // the table: A0 {rows, cols}, keys = symList, values = the columns (allocTable, h_memory.cc:168-172)
    HG_CHECK(init_list(z, H_A, 2));
    V0* e2 = (V0*)z->g;
    memset(e2, 0, 2 * sizeof(V0));
    A hdr = (A)halloc(sizeof(A0));
    if (!hdr) return E_DEVICE_OOM;
    hdr->row = rows;
    hdr->col = numCols;
    hdr->fkey = nullptr;
    z->a = hdr;
    V0& keys = e2[0];
    keys.typ = H_Q;
    keys.len = numCols;
    if (numCols == 1) { keys.g = (G)&keys.b; keys.i64 = symList[0]; }
    else {
        L* kp = (L*)halloc((size_t)numCols * 8);
        if (!kp) return E_DEVICE_OOM;
        memcpy(kp, symList, (size_t)numCols * 8);
        keys.g = (G)kp;
    }
    HG_CHECK(init_list(&e2[1], H_G, numCols));
    V0* cols = (V0*)e2[1].g;
    for (L j = 0; j < numCols; j++) {
        cols[j] = colv[j];
        if (colv[j].len <= 1) cols[j].g = (G)&cols[j].b;
    }
    return apply_residency(z);
}

}  // namespace
}  // namespace hg

using namespace hg;

extern "C" {

I hgpuReadSerialized(V x, FILE* fp) {
    HG_CHECK(ensure_init());
    if (!x || !fp) return E_DOMAIN;
    ScratchScope ss;
    const long long mark = out_mark();
    I e = read_node(x, fp);
    if (!e) e = apply_residency(x);
    if (e) out_rewind(mark);
    return e;
}

I hgpuWriteSerialized(V x, FILE* fp) {
    HG_CHECK(ensure_init());
    if (!x || !fp) return E_DOMAIN;
    return write_node(x, fp);
}

I hgpuReadCSV(V z, S fileName, L numCols, L* types, Q* symList) {
    HG_CHECK(ensure_init());
    if (!z || !fileName || !types || !symList) return E_DOMAIN;
    ScratchScope ss;
    const long long mark = out_mark();
    I e = read_csv(z, fileName, numCols, types, symList);
    if (e) out_rewind(mark);
    return e;
}

// The reference's void / V-returning loaders stop the process on a bad file
// (EP, exit codes 1 and 99); they still do for those cases.  A device
// failure (E_DEVICE and above) does not end the process: the error is
// printed, kept for hgpuLastError, and the node is left empty (readCSV
// returns NULL).  hgpuReadCSV / hgpuReadSerialized / hgpuWriteSerialized
// return every status instead.
static void loader_failed(const char* what, I rc, int code) {
    fprintf(stderr, "[ERROR] %s: %s\n", what, hgpuLastError());
    if (rc < E_DEVICE) exit(code);
}

void serializeV(V x, FILE* fp) {
    const I rc = hgpuWriteSerialized(x, fp);
    if (rc) loader_failed("serializeV", rc, 1);
}

void readSerializeV(V x, FILE* fp) {
    const I rc = hgpuReadSerialized(x, fp);
    if (rc) {
        loader_failed("readSerializeV", rc, 1);
        memset(x, 0, sizeof(V0));
    }
}

V readCSV(S fileName, L numCols, L* types, Q* symList) {
    V z = allocNode();
    if (!z) {
        loader_failed("readCSV", E_DEVICE_OOM, 99);
        return nullptr;
    }
    const I rc = hgpuReadCSV(z, fileName, numCols, types, symList);
    if (rc) {
        loader_failed("readCSV", rc, 99);
        return nullptr;
    }
    return z;
}

}  // extern "C"
