// Symbols and strings on the GPU: symbol compares (compareSymbol,
// h_symbol.cc:241-243, under COMPFN, h_primitive.cc:1068-1071) and @like
// (pfnLike, h_primitive.cc:1670-1758).
//
// The symbol table stays on the host (ids are interned texts).  Two device
// copies of it are kept and extended as symbols are added: the texts (one
// blob plus each id's span) for @like over symbol columns, and each id's
// rank in strcmp order for the ordered compares (equal ids compare equal,
// distinct ids differ in text, so rank order is strcmp order).
//
// @like: the reference turns the SQL pattern into a regex ('%' -> ".*",
// '_' -> ".", '.' and '\' escaped; genLikeString, h_system.cc:319-334) and
// matches it anchored with PCRE2.  That regex has literals, '.' and '.*'
// only, so it is an NFA over the pattern positions, run bit-parallel: bit i
// of the state word says "the first i tokens matched".  Per text byte c the
// state advances through the tokens that accept c (a literal c, or '_' when
// c is not '\n') and stays on the '%' tokens (when c is not '\n'); '%' also
// passes for free (closure).  PCRE2's '$' matches at the end or before a
// final '\n'.  Symbol columns evaluate the pattern once per symbol of the
// table and gather; string columns match each row's text.
#include <algorithm>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "hgpu_internal.cuh"

namespace hg {
namespace {

// ------------------------------------------------------ device symbol table
struct SymTable {
    L n = 0;                      // symbols copied
    char* blob = nullptr;         // texts, NUL-terminated
    size_t blob_cap = 0, blob_len = 0;
    unsigned long long* spans = nullptr;  // (offset << 16) | length per id
    long long* rank = nullptr;    // strcmp rank per id
    L span_cap = 0, rank_n = 0;
};
SymTable g_symtab;

I grow(void** p, size_t old_bytes, size_t new_bytes) {
    void* q = nullptr;
    HG_CU(cudaMalloc(&q, new_bytes));
    if (*p && old_bytes) HG_CU(cudaMemcpyAsync(q, *p, old_bytes, cudaMemcpyDeviceToDevice, g_stream));
    HG_CU(stream_sync());
    if (*p) cudaFree(*p);
    *p = q;
    return 0;
}

// texts and spans of every symbol interned so far
I sym_texts(SymTable** out) {
    SymTable& t = g_symtab;
    const L n = symbol_count();
    if (n > t.n) {
        std::vector<char> add;
        std::vector<unsigned long long> sp((size_t)(n - t.n));
        size_t off = t.blob_len;
        for (L id = t.n; id < n; id++) {
            const char* s = symbol_text(id);
            const size_t k = strlen(s);
            if (k >= 0xffff) return set_error(E_NOT_IMPL, "a symbol of %zu characters", k);
            sp[(size_t)(id - t.n)] = ((unsigned long long)(off + add.size()) << 16) | k;
            add.insert(add.end(), s, s + k + 1);
        }
        if (t.blob_len + add.size() > t.blob_cap) {
            size_t cap = t.blob_cap ? t.blob_cap : 1 << 16;
            while (cap < t.blob_len + add.size()) cap *= 2;
            HG_CHECK(grow((void**)&t.blob, t.blob_len, cap));
            t.blob_cap = cap;
        }
        if (n > t.span_cap) {
            L cap = t.span_cap ? t.span_cap : 1024;
            while (cap < n) cap *= 2;
            HG_CHECK(grow((void**)&t.spans, (size_t)t.n * 8, (size_t)cap * 8));
            t.span_cap = cap;
        }
        HG_CU(cudaMemcpyAsync(t.blob + t.blob_len, add.data(), add.size(), cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaMemcpyAsync(t.spans + t.n, sp.data(), sp.size() * 8, cudaMemcpyHostToDevice, g_stream));
        HG_CU(stream_sync());
        t.blob_len += add.size();
        t.n = n;
    }
    *out = &t;
    return 0;
}

// strcmp rank of every symbol (the dictionary's order, rebuilt when it grows)
I sym_ranks(const long long** rank, L* n_out) {
    SymTable& t = g_symtab;
    const L n = symbol_count();
    if (n != t.rank_n) {
        std::vector<L> ids((size_t)n);
        for (L i = 0; i < n; i++) ids[(size_t)i] = i;
        std::sort(ids.begin(), ids.end(), [](L a, L b) { return strcmp(symbol_text(a), symbol_text(b)) < 0; });
        std::vector<long long> r((size_t)(n > 0 ? n : 1));
        for (L k = 0; k < n; k++) r[(size_t)ids[(size_t)k]] = k;
        if (t.rank) cudaFree(t.rank);
        t.rank = nullptr;
        HG_CU(cudaMalloc((void**)&t.rank, r.size() * 8));
        HG_CU(cudaMemcpyAsync(t.rank, r.data(), r.size() * 8, cudaMemcpyHostToDevice, g_stream));
        HG_CU(stream_sync());
        t.rank_n = n;
    }
    *rank = t.rank;
    *n_out = n;
    return 0;
}

__global__ void k_cmp_sym(const long long* __restrict__ x, long long xs, bool xone, const long long* __restrict__ y,
                          long long ys, bool yone, long long n, const long long* __restrict__ rank, long long nsym, int op,
                          bool* __restrict__ z, unsigned* derr) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long a = xone ? xs : x[i], b = yone ? ys : y[i];
        bool r;
        if (op == 4) r = a == b;
        else if (op == 5) r = a != b;
        else {
            int c = 0;
            if (a != b) {
                if (a < 0 || a >= nsym || b < 0 || b >= nsym) { flag_error(derr, DERR_INDEX); c = 0; }
                else c = rank[a] < rank[b] ? -1 : 1;
            }
            r = op == 0 ? c < 0 : op == 1 ? c <= 0 : op == 2 ? c > 0 : c >= 0;
        }
        z[i] = r;
    }
}

// ------------------------------------------------------------------- @like
struct LikeProg {
    unsigned long long cls[256];  // tokens accepting byte c
    unsigned long long star;      // '%' tokens
    int m;                        // tokens
};

I like_compile(const char* pat, LikeProg* p) {
    memset(p, 0, sizeof(*p));
    int m = 0;
    unsigned long long any = 0;
    for (const unsigned char* c = (const unsigned char*)pat; *c; c++) {
        if (m >= 63) return set_error(E_NOT_IMPL, "@like: a pattern of more than 63 tokens");
        if (*c == '%') p->star |= 1ull << m;
        else if (*c == '_') any |= 1ull << m;
        else if (strchr("()[]{}*+?|^$", *c))
            return set_error(E_NOT_IMPL, "@like: '%c' would be a regex operator in the reference's pattern", *c);
        else p->cls[*c] |= 1ull << m;
        m++;
    }
    for (int c = 0; c < 256; c++)
        if (c != '\n') p->cls[c] |= any;
    p->m = m;
    return 0;
}

__device__ __forceinline__ unsigned long long like_closure(unsigned long long s, unsigned long long star) {
    for (;;) {
        const unsigned long long t = s | ((s & star) << 1);
        if (t == s) return s;
        s = t;
    }
}
__device__ bool like_match(const LikeProg& p, const unsigned char* s, int n) {
    unsigned long long st = like_closure(1ull, p.star), before_last = 0;
    for (int k = 0; k < n && st; k++) {
        const unsigned c = s[k];
        if (k == n - 1) before_last = st;
        st = ((st & p.cls[c]) << 1) | (c != '\n' ? (st & p.star) : 0ull);
        st = like_closure(st, p.star);
    }
    const unsigned long long fin = 1ull << p.m;
    return (st & fin) || (n > 0 && s[n - 1] == '\n' && (before_last & fin));
}

// one text per thread: texts given by (offset << 16 | length) spans into blob
__global__ void k_like_spans(LikeProg prog, const char* __restrict__ blob, const unsigned long long* __restrict__ spans,
                             long long n, bool* __restrict__ z) {
    __shared__ LikeProg p;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) p.cls[i] = prog.cls[i];
    if (threadIdx.x == 0) { p.star = prog.star; p.m = prog.m; }
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long sp = spans[i];
        const unsigned char* t = (const unsigned char*)blob + (sp >> 16);
        int len = (int)(sp & 0xffffull);
        z[i] = like_match(p, t, len);
    }
}
// symbol columns: the per-id result gathered by the column's ids
__global__ void k_like_gather(const bool* __restrict__ by_id, long long nsym, const long long* __restrict__ ids, long long n,
                              bool* __restrict__ z, unsigned* derr) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long id = ids[i];
        if (id < 0 || id >= nsym) { flag_error(derr, DERR_INDEX); z[i] = false; }
        else z[i] = by_id[id];
    }
}

unsigned grid_n(long long n) {
    unsigned g = grid_for(n, 256);
    return g > (unsigned)g_sms * 16 ? (unsigned)g_sms * 16 : g;
}

// Host string vector -> (device blob, spans): the CSV reader's columns are
// found in HBM already; others are gathered once into scratch.
I string_spans(V x, const char** blob, const unsigned long long** spans) {
    const long long n = x->len;
    if (n > 1 && find_strings(x->g, n, blob, spans)) return 0;
    std::vector<S> ptrs((size_t)n);
    if (n == 1) {
        uint64_t p;
        HG_CHECK(read_elem0(x, &p));
        ptrs[0] = (S)(uintptr_t)p;
    } else if (n > 1) {
        if (host_readable(x->g)) memcpy(ptrs.data(), x->g, (size_t)n * sizeof(S));
        else {
            HG_CU(cudaMemcpyAsync(ptrs.data(), x->g, (size_t)n * sizeof(S), cudaMemcpyDeviceToHost, g_stream));
            HG_CU(stream_sync());
        }
    }
    std::vector<unsigned long long> sp((size_t)n);
    size_t total = 0;
    for (long long i = 0; i < n; i++) {
        const size_t k = strlen(ptrs[(size_t)i]);
        if (k >= 0xffff) return set_error(E_NOT_IMPL, "@like: a text of %zu characters", k);
        sp[(size_t)i] = ((unsigned long long)total << 16) | k;
        total += k;
    }
    char* hb = (char*)halloc(total > 0 ? total : 1);
    if (!hb) return E_DEVICE_OOM;
    for (long long i = 0; i < n; i++) memcpy(hb + (sp[(size_t)i] >> 16), ptrs[(size_t)i], sp[(size_t)i] & 0xffffull);
    char* db = (char*)salloc(total > 0 ? total : 1);
    unsigned long long* ds = (unsigned long long*)salloc((size_t)(n > 0 ? n : 1) * 8);
    if (!db || !ds) return E_DEVICE_OOM;
    HG_CU(cudaMemcpyAsync(db, hb, total, cudaMemcpyHostToDevice, g_stream));
    HG_CU(cudaMemcpyAsync(ds, sp.data(), (size_t)n * 8, cudaMemcpyHostToDevice, g_stream));
    *blob = db;
    *spans = ds;
    return 0;
}

}  // namespace

// Symbol compares for pfnCompare (both operands H_Q, lengths already checked).
I compare_symbols(V z, V x, V y, I op) {
    const bool xone = x->len == 1, yone = y->len == 1;
    const long long n = xone ? y->len : x->len;
    uint64_t xs = 0, ys = 0;
    const void *px = nullptr, *py = nullptr;
    if (xone) HG_CHECK(read_elem0(x, &xs)); else HG_CHECK(in_ptr(x, &px));
    if (yone) HG_CHECK(read_elem0(y, &ys)); else HG_CHECK(in_ptr(y, &py));
    const long long* rank = nullptr;
    L nsym = 0;
    if (op < 4) HG_CHECK(sym_ranks(&rank, &nsym));
    void* dz;
    HG_CHECK(alloc_out(z, H_B, n, &dz));
    if (n > 0)
        HG_LAUNCH("cmp_sym", grid_n(n), 256, 0, k_cmp_sym, (const long long*)px, (long long)xs, xone, (const long long*)py,
                  (long long)ys, yone, n, rank, nsym, (int)op, (bool*)dz, g_derr);
    HG_CHECK(last_launch_error());
    HG_CHECK(check_device_errors());
    return finish_out(z, dz);
}

}  // namespace hg

using namespace hg;

extern "C" {

// pfnLike (h_primitive.cc:1670-1758): one pattern y over chars / symbols / strings x
I pfnLike(V z, V x, V y) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    if (!is_string(x->typ) || !is_string(y->typ)) return E_DOMAIN;
    if (y->len != 1)
        return (x->typ == H_C || x->len == y->len) ? set_error(E_NOT_IMPL, "@like with one pattern per row") : E_LENGTH;
    // the pattern text: sC(y), vs(y) or getSymbolStr(vq(y))
    std::vector<char> pat;
    if (y->typ == H_Q) {
        uint64_t id;
        HG_CHECK(read_elem0(y, &id));
        const char* s = getSymbolStr((L)id);
        pat.assign(s, s + strlen(s) + 1);
    } else if (y->typ == H_S) {
        uint64_t p;
        HG_CHECK(read_elem0(y, &p));
        const char* s = (const char*)(uintptr_t)p;
        pat.assign(s, s + strlen(s) + 1);
    } else {
        uint64_t c;
        HG_CHECK(read_elem0(y, &c));
        pat.push_back((char)c);
        pat.push_back(0);
    }
    if (!pat[0]) return E_NULL_VALUE;  // genLikeString gives NULL for an empty pattern
    LikeProg prog;
    HG_CHECK(like_compile(pat.data(), &prog));
    if (x->typ == H_C) {  // one text: the char vector up to its first NUL
        const void* px;
        HG_CHECK(in_ptr(x, &px));
        std::vector<char> h((size_t)x->len + 1, 0);
        if (x->len > 0) HG_CU(cudaMemcpy(h.data(), px, (size_t)x->len, cudaMemcpyDefault));
        const size_t k = strlen(h.data());
        char* db = (char*)salloc(k + 1);
        unsigned long long* ds = (unsigned long long*)salloc(16);
        void* dz;
        if (!db || !ds) return E_DEVICE_OOM;
        const unsigned long long sp = k;
        HG_CU(cudaMemcpyAsync(db, h.data(), k + 1, cudaMemcpyHostToDevice, g_stream));
        HG_CU(cudaMemcpyAsync(ds, &sp, 8, cudaMemcpyHostToDevice, g_stream));
        HG_CHECK(alloc_out(z, H_B, 1, &dz));
        HG_LAUNCH("like", 1, 32, 0, k_like_spans, prog, db, ds, 1LL, (bool*)dz);
        HG_CHECK(last_launch_error());
        return finish_out(z, dz);
    }
    const long long n = x->len;
    void* dz;
    HG_CHECK(alloc_out(z, H_B, n, &dz));
    if (n == 0) return finish_out(z, dz);
    if (x->typ == H_Q) {
        SymTable* t;
        HG_CHECK(sym_texts(&t));
        bool* by_id = (bool*)salloc((size_t)(t->n > 0 ? t->n : 1));
        const void* px;
        if (!by_id) return E_DEVICE_OOM;
        HG_CHECK(in_ptr(x, &px));
        if (t->n > 0) HG_LAUNCH("like_symbols", grid_n(t->n), 256, 0, k_like_spans, prog, t->blob, t->spans, (long long)t->n, by_id);
        HG_LAUNCH("like_gather", grid_n(n), 256, 0, k_like_gather, by_id, (long long)t->n, (const long long*)px, n, (bool*)dz, g_derr);
    } else {
        const char* blob;
        const unsigned long long* spans;
        HG_CHECK(string_spans(x, &blob, &spans));
        HG_LAUNCH("like", grid_n(n), 256, 0, k_like_spans, prog, blob, spans, n, (bool*)dz);
    }
    HG_CHECK(last_launch_error());
    HG_CHECK(check_device_errors());
    return finish_out(z, dz);
}

}  // extern "C"
