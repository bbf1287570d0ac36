// Fused elementwise + compress + reduce chains, one kernel per chain.
//
// The reference's loop-fusion passes turn chains of builtins into single C
// loops (optimizer/autofusion.cc:770-935 genCodeAuto: masked reductions
// `if(cond) c += expr` with reduction(op:c) at :907, scan/compress at
// :888-900; elementwise.cc:239-281 genCodeElem; pattern.cc:482-520
// multi-column compress sharing one mask).  Here a chain is written as a
// small S-expression program, and each (program, input types) pair is
// compiled once with NVRTC into one sm_103a kernel:
//
//   (sum   VALUE MASK)          masked reduction (also min, max)
//   (count MASK)                number of selected rows
//   (compress MASK E1 E2 ...)   one output per expression, rows where MASK
//   (map   E)                   elementwise result
//
//   E := xK | literal | (lt|leq|gt|geq|eq|neq E E) | (plus|minus|mul|div E E)
//        | (and E E ...) | (or E E ...) | (not E)
//   literal := 24:i32 | 0.05:f64 | 3:i64 | 1:bool ...
//
// Each operation has the interpreter's semantics (the oracle): operands are
// promoted to the larger type code, f32/f64 compares use compareFloat's
// 1e-13 epsilon (h_primitive.cc:1061), integer arithmetic wraps, sums of
// integers accumulate in i64.  Reductions use the fixed-order tile tree over
// the full row range (unselected rows contribute nothing), so a fused sum is
// deterministic; it differs from compress-then-sum only in rounding order.
#include <dlfcn.h>

#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "dev_common.cuh"

namespace hg {

I compact_rows(const uint8_t* mask, long long n, long long* out, long long* count);

// ------------------------------------------------------------------ NVRTC
// libnvrtc is opened at run time so libhgpu loads without it; only chain
// compilation needs it.
typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;
struct Nvrtc {
    void* h = nullptr;
    nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*, const char* const*);
    nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*);
    nvrtcResult_t (*logsize)(nvrtcProgram_t, size_t*);
    nvrtcResult_t (*log)(nvrtcProgram_t, char*);
    nvrtcResult_t (*cubinsize)(nvrtcProgram_t, size_t*);
    nvrtcResult_t (*cubin)(nvrtcProgram_t, char*);
    nvrtcResult_t (*destroy)(nvrtcProgram_t*);
};
static Nvrtc* nvrtc() {
    static Nvrtc n;
    static bool tried = false;
    if (tried) return n.h ? &n : nullptr;
    tried = true;
    const char* cands[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                           "/usr/local/cuda/targets/sbsa-linux/lib/libnvrtc.so.13",
                           "/usr/local/cuda/targets/x86_64-linux/lib/libnvrtc.so.13"};
    for (const char* c : cands)
        if ((n.h = dlopen(c, RTLD_NOW | RTLD_LOCAL))) break;
    if (!n.h) return nullptr;
    n.create = (decltype(n.create))dlsym(n.h, "nvrtcCreateProgram");
    n.compile = (decltype(n.compile))dlsym(n.h, "nvrtcCompileProgram");
    n.logsize = (decltype(n.logsize))dlsym(n.h, "nvrtcGetProgramLogSize");
    n.log = (decltype(n.log))dlsym(n.h, "nvrtcGetProgramLog");
    n.cubinsize = (decltype(n.cubinsize))dlsym(n.h, "nvrtcGetCUBINSize");
    n.cubin = (decltype(n.cubin))dlsym(n.h, "nvrtcGetCUBIN");
    n.destroy = (decltype(n.destroy))dlsym(n.h, "nvrtcDestroyProgram");
    if (!n.create || !n.compile || !n.cubin) { n.h = nullptr; return nullptr; }
    return &n;
}

// ------------------------------------------------------------------ parse
struct Node {
    std::string op;           // "x", "lit", or an operation name
    int col = -1;             // for "x"
    std::string lit;          // literal text
    int typ = -1;             // result type code
    std::vector<std::unique_ptr<Node>> kids;
};

static const char* skip(const char* p) { while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') p++; return p; }

static std::unique_ptr<Node> parse(const char*& p, std::string& err) {
    p = skip(p);
    auto n = std::make_unique<Node>();
    if (*p == '(') {
        p++;
        p = skip(p);
        const char* s = p;
        while (*p && *p != ' ' && *p != ')' && *p != '(') p++;
        n->op.assign(s, p);
        for (;;) {
            p = skip(p);
            if (*p == ')') { p++; break; }
            if (!*p) { err = "unbalanced parenthesis"; return nullptr; }
            auto k = parse(p, err);
            if (!k) return nullptr;
            n->kids.push_back(std::move(k));
        }
        return n;
    }
    const char* s = p;
    while (*p && *p != ' ' && *p != ')' && *p != '(' && *p != '\n') p++;
    std::string tok(s, p);
    if (tok.empty()) { err = "empty token"; return nullptr; }
    if (tok[0] == 'x') { n->op = "x"; n->col = atoi(tok.c_str() + 1); return n; }
    n->op = "lit";
    n->lit = tok;
    return n;
}

static const char* ctype(int t) {
    switch (t) {
    case H_B: return "bool";
    case H_J: case H_C: return "signed char";
    case H_H: return "short";
    case H_I: case H_D: case H_M: case H_U: case H_W: case H_T: return "int";
    case H_L: case H_Z: return "long long";
    case H_F: return "float";
    default: return "double";
    }
}
static int arith_rank(int t) { return (t == H_D || t == H_M || t == H_U || t == H_W || t == H_T) ? H_I : (t == H_Z ? H_L : (t == H_C ? H_J : t)); }

struct Gen {
    std::vector<int> in_typ;   // input column types
    std::vector<bool> used;
    std::string err;
    std::string vsuffix;       // appended to the input variables (v0, v1, ...) of the expressions made

    // returns a C++ expression; sets n->typ
    std::string expr(Node* n) {
        if (n->op == "x") {
            if (n->col < 0 || n->col >= (int)in_typ.size()) { err = "input x" + std::to_string(n->col) + " not given"; return ""; }
            used[n->col] = true;
            n->typ = in_typ[n->col];
            return "v" + std::to_string(n->col) + vsuffix;
        }
        if (n->op == "lit") {
            size_t c = n->lit.find(':');
            std::string num = n->lit.substr(0, c), ty = c == std::string::npos ? "" : n->lit.substr(c + 1);
            bool isf = num.find('.') != std::string::npos || num.find('e') != std::string::npos;
            int t = ty == "bool" ? H_B : ty == "i8" ? H_J : ty == "i16" ? H_H : ty == "i32" ? H_I : ty == "i64" ? H_L
                  : ty == "f32" ? H_F : ty == "f64" ? H_E : ty == "date" ? H_D : (isf ? H_E : H_L);
            n->typ = t;
            return std::string("((") + ctype(t) + ")(" + num + (t == H_F && isf ? "f" : "") + "))";
        }
        std::vector<std::string> a;
        for (auto& k : n->kids) { a.push_back(expr(k.get())); if (!err.empty()) return ""; }
        const std::string& o = n->op;
        auto need = [&](size_t k) { if (a.size() != k) err = o + " takes " + std::to_string(k) + " operands"; return err.empty(); };
        if (o == "and" || o == "or") {
            if (a.size() < 2) { err = o + " takes at least two operands"; return ""; }
            std::string s = "(";
            for (size_t i = 0; i < a.size(); i++) {
                if (n->kids[i]->typ != H_B) { err = o + " needs bool operands"; return ""; }
                s += (i ? (o == "and" ? " & " : " | ") : "") + std::string("(int)") + a[i];
            }
            n->typ = H_B;
            return s + ")";
        }
        if (o == "not") {
            if (!need(1)) return "";
            n->typ = H_B;
            return "(!" + a[0] + ")";
        }
        static const std::map<std::string, int> cmp = {{"lt", 0}, {"leq", 1}, {"gt", 2}, {"geq", 3}, {"eq", 4}, {"neq", 5}};
        static const std::map<std::string, int> ari = {{"plus", 0}, {"minus", 1}, {"mul", 2}, {"div", 3}};
        if (cmp.count(o) || ari.count(o)) {
            if (!need(2)) return "";
            int ta = arith_rank(n->kids[0]->typ), tb = arith_rank(n->kids[1]->typ);
            int t = ta > tb ? ta : tb;
            std::string ca = std::string("((") + ctype(t) + ")" + a[0] + ")", cb = std::string("((") + ctype(t) + ")" + a[1] + ")";
            if (cmp.count(o)) {
                n->typ = H_B;
                const bool la = n->kids[0]->op == "lit", lb = n->kids[1]->op == "lit";
                if (t == H_E && la != lb) {
                    // f64 against a literal: compareFloat by integer thresholds (no FP64 subtraction)
                    const std::string& lt = (la ? n->kids[0] : n->kids[1])->lit;
                    const double sv = strtod(lt.substr(0, lt.find(':')).c_str(), nullptr);
                    const F64Cmp th = f64_cmp_thresholds(sv, la);
                    return "hg_cmpf_fixed(" + (la ? cb : ca) + ", " + std::to_string(th.ta) + "LL, " +
                           std::to_string(th.tb) + "LL, " + std::to_string(th.ca) + ", " + std::to_string(th.cb) +
                           ", " + std::to_string(th.cc) + ", " + std::to_string(cmp.at(o)) + ")";
                }
                return "hg_cmp<" + std::string(ctype(t)) + ">(" + std::to_string(cmp.at(o)) + ", " + ca + ", " + cb + ")";
            }
            if (ari.at(o) == 3) uses_div = true;
            n->typ = t;
            return "hg_arith<" + std::string(ctype(t)) + ">(" + std::to_string(ari.at(o)) + ", " + ca + ", " + cb + ", dz)";
        }
        err = "unknown operation " + o;
        return "";
    }
    bool uses_div = false;
};

// Device helpers shared by every generated kernel (same semantics as
// k_elementwise.cu and k_reduce.cu).
static const char* kPrelude = R"(
template <typename T> struct hg_is_f { static const bool v = false; };
template <> struct hg_is_f<float> { static const bool v = true; };
template <> struct hg_is_f<double> { static const bool v = true; };
__device__ __forceinline__ bool hg_cmpf_fixed(double v, long long ta, long long tb, int ca, int cb, int cc, int op) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    int c;
    if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) c = 1;
    else {
        const long long o = (b >> 63) ? -(long long)(b & 0x7fffffffffffffffull) : (long long)b;
        c = o < ta ? ca : (o < tb ? cb : cc);
    }
    return op == 0 ? c < 0 : op == 1 ? c <= 0 : op == 2 ? c > 0 : op == 3 ? c >= 0 : op == 4 ? c == 0 : c != 0;
}
template <typename T> __device__ __forceinline__ bool hg_cmp(int op, T a, T b) {
    if (hg_is_f<T>::v) {
        int c = a < b ? ((double)(b - a) < 1e-13 ? 0 : -1) : ((double)(a - b) < 1e-13 ? 0 : 1);
        return op == 0 ? c < 0 : op == 1 ? c <= 0 : op == 2 ? c > 0 : op == 3 ? c >= 0 : op == 4 ? c == 0 : c != 0;
    }
    return op == 0 ? a < b : op == 1 ? a <= b : op == 2 ? a > b : op == 3 ? a >= b : op == 4 ? a == b : a != b;
}
__device__ __forceinline__ double hg_ar(int op, double a, double b, bool& dz) {
    if (op == 0) return __dadd_rn(a, b); if (op == 1) return __dsub_rn(a, b); if (op == 2) return __dmul_rn(a, b);
    if (b == 0.0) dz = true; return __ddiv_rn(a, b); }
__device__ __forceinline__ float hg_ar(int op, float a, float b, bool& dz) {
    if (op == 0) return __fadd_rn(a, b); if (op == 1) return __fsub_rn(a, b); if (op == 2) return __fmul_rn(a, b);
    if (b == 0.0f) dz = true; return __fdiv_rn(a, b); }
__device__ __forceinline__ long long hg_ar(int op, long long a, long long b, bool& dz) {
    unsigned long long x = a, y = b;
    if (op == 0) return (long long)(x + y); if (op == 1) return (long long)(x - y); if (op == 2) return (long long)(x * y);
    if (b == 0) { dz = true; return 0; } if (b == -1) return (long long)(0ull - x); return a / b; }
__device__ __forceinline__ int hg_ar(int op, int a, int b, bool& dz) {
    unsigned x = a, y = b;
    if (op == 0) return (int)(x + y); if (op == 1) return (int)(x - y); if (op == 2) return (int)(x * y);
    if (b == 0) { dz = true; return 0; } if (b == -1) return (int)(0u - x); return a / b; }
template <typename T> __device__ __forceinline__ T hg_arith(int op, T a, T b, bool& dz) {
    int x = a, y = b, r;
    if (op == 0) r = x + y; else if (op == 1) r = x - y; else if (op == 2) r = x * y;
    else { if (y == 0) { dz = true; r = 0; } else r = x / y; }
    return (T)r; }
template <> __device__ __forceinline__ bool hg_arith<bool>(int op, bool a, bool b, bool& dz) {
    int x = a, y = b, r;
    if (op == 0) r = x + y; else if (op == 1) r = x - y; else if (op == 2) r = x * y;
    else { if (y == 0) { dz = true; r = 0; } else r = x / y; }
    return r != 0; }
template <> __device__ __forceinline__ int hg_arith<int>(int op, int a, int b, bool& dz) { return hg_ar(op, a, b, dz); }
template <> __device__ __forceinline__ long long hg_arith<long long>(int op, long long a, long long b, bool& dz) { return hg_ar(op, a, b, dz); }
template <> __device__ __forceinline__ float hg_arith<float>(int op, float a, float b, bool& dz) { return hg_ar(op, a, b, dz); }
template <> __device__ __forceinline__ double hg_arith<double>(int op, double a, double b, bool& dz) { return hg_ar(op, a, b, dz); }
)";

struct Compiled {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kern = nullptr;
    std::string sink;       // sum|min|max|count|compress|map
    int acc_typ = H_E;      // accumulator / result type
    std::vector<int> out_typ;
    bool may_fail = false;  // some operation can flag an error (division by zero)
};

}  // namespace hg

struct hgpu_chain_s {
    std::string text;
    std::unique_ptr<hg::Node> root;
    std::map<std::string, std::shared_ptr<hg::Compiled>> cache;  // by input type signature
};

namespace hg {

static I compile_chain(hgpu_chain_s* c, const std::vector<int>& types, std::shared_ptr<Compiled>* out) {
    std::string key;
    for (int t : types) key += std::to_string(t) + ",";
    auto it = c->cache.find(key);
    if (it != c->cache.end()) { *out = it->second; return 0; }
    Node* r = c->root.get();
    Gen g;
    g.in_typ = types;
    g.used.assign(types.size(), false);
    auto cm = std::make_shared<Compiled>();
    cm->sink = r->op;
    std::string body, red;
    const int nin = (int)types.size();
    std::string loads;
    auto gen_loads = [&]() {
        loads.clear();
        for (int k = 0; k < nin; k++)
            if (g.used[k])
                loads += std::string("        ") + ctype(types[k]) + " v" + std::to_string(k) + " = ((const " + ctype(types[k]) +
                         "*)cols[" + std::to_string(k) + "])[i];\n";
    };
    std::string src = kPrelude;
    if (r->op == "sum" || r->op == "min" || r->op == "max" || r->op == "count") {
        std::string val, mask;
        if (r->op == "count") {
            if (r->kids.size() != 1) return set_error(E_DOMAIN, "count takes (count MASK)");
            mask = g.expr(r->kids[0].get());
            val = "1LL";
        } else {
            if (r->kids.size() != 2) return set_error(E_DOMAIN, "%s takes (%s VALUE MASK)", r->op.c_str(), r->op.c_str());
            val = g.expr(r->kids[0].get());
            mask = g.expr(r->kids[1].get());
        }
        if (!g.err.empty()) return set_error(E_DOMAIN, "chain: %s", g.err.c_str());
        // columns the mask reads are loaded for every row; columns only the
        // value reads are loaded for selected rows only
        std::vector<bool> in_mask(nin, false), in_val(nin, false);
        {
            std::vector<Node*> st;
            if (r->op == "count") st.push_back(r->kids[0].get()); else st.push_back(r->kids[1].get());
            while (!st.empty()) { Node* q = st.back(); st.pop_back(); if (q->op == "x") in_mask[q->col] = true; for (auto& k : q->kids) st.push_back(k.get()); }
            if (r->op != "count") {
                st.push_back(r->kids[0].get());
                while (!st.empty()) { Node* q = st.back(); st.pop_back(); if (q->op == "x") in_val[q->col] = true; for (auto& k : q->kids) st.push_back(k.get()); }
            }
        }
        std::string vloads, hoist, preload, unpack;
        for (int k = 0; k < nin; k++) {
            const std::string K = std::to_string(k), T = ctype(types[k]);
            if (in_mask[k] || in_val[k]) hoist += "    const " + T + "* __restrict__ c" + K + " = (const " + T + "*)cols[" + K + "];\n";
            if (in_val[k] && !in_mask[k]) vloads += "                " + T + " v" + K + " = c" + K + "[i];\n";
            if (in_mask[k]) {
                preload += "        a" + K + "[k] = in ? c" + K + "[i] : (" + T + ")0;\n";
                hoist += "    " + T + " a" + K + "[16];\n";
                unpack += "            " + T + " v" + K + " = a" + K + "[k];\n";
            }
        }
        int vt = r->op == "count" ? H_L : arith_rank(r->kids[0]->typ);
        int at = r->op == "count" ? H_L : (r->op == "sum" ? (vt == H_F ? H_F : vt == H_E ? H_E : H_L) : vt);
        cm->acc_typ = at;
        const char* A = ctype(at);
        std::string opf = r->op == "min" ? "(a < b ? a : b)" : r->op == "max" ? "(a > b ? a : b)"
                        : (at == H_E ? "__dadd_rn(a, b)" : at == H_F ? "__fadd_rn(a, b)" : "(long long)((unsigned long long)a + (unsigned long long)b)");
        std::string ident = r->op == "min" ? "ident" : r->op == "max" ? "ident" : std::string("(") + A + ")0";
        // Each block reduces one 4096-row tile in the tile-tree order: lane t
        // takes rows t, t+256, ..., t+3840 (the mask columns of all 16 rows
        // are loaded before the first is used, so the loads overlap), then a
        // xor butterfly and the pairwise combine of the 8 warps.  With
        // `result` set, the block that finishes last reduces the tile
        // partials by the same tree (one tile of partials: at most 4096
        // blocks) and writes the result, so the chain is one launch.
        auto tree = [&](const std::string& dest) {
            return std::string("    {\n") +
                   "    for (int o = 16; o > 0; o >>= 1) acc = hg_op(acc, __shfl_xor_sync(0xffffffffu, acc, o));\n"
                   "    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;\n"
                   "    __syncthreads();\n"
                   "    if (threadIdx.x == 0) " + dest + " = hg_op(hg_op(hg_op(ws[0], ws[1]), hg_op(ws[2], ws[3])),"
                   " hg_op(hg_op(ws[4], ws[5]), hg_op(ws[6], ws[7])));\n"
                   "    }\n";
        };
        src += std::string("__device__ __forceinline__ ") + A + " hg_op(" + A + " a, " + A + " b) { return " + opf + "; }\n";
        src += std::string("extern \"C\" __global__ void __launch_bounds__(256) chain_kernel(const void* const* cols, long long n, ") + A +
               "* part, " + A + " ident, unsigned* derr, unsigned* done, " + A + "* result) {\n"
               "    __shared__ " + A + " ws[8];\n"
               "    __shared__ bool last;\n"
               "    const long long base = (long long)blockIdx.x * 4096;\n" + hoist +
               "    #pragma unroll\n"
               "    for (int k = 0; k < 16; k++) {\n"
               "        const long long i = base + k * 256 + threadIdx.x;\n"
               "        const bool in = i < n;\n" + preload +
               "    }\n"
               "    " + A + " acc = " + ident + ";\n    bool dz = false;\n"
               "    #pragma unroll\n"
               "    for (int k = 0; k < 16; k++) {\n"
               "        const long long i = base + k * 256 + threadIdx.x;\n"
               "        if (i < n) {\n" + unpack +
               "            if (" + mask + ") {\n" + vloads + "                acc = hg_op(acc, (" + A + ")(" + val + "));\n            }\n"
               "        }\n"
               "    }\n" + tree("part[blockIdx.x]") +
               "    if (dz) atomicOr(derr, 4u);\n"
               "    if (!result) return;\n"
               "    __threadfence();\n"
               "    __syncthreads();\n"
               "    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;\n"
               "    __syncthreads();\n"
               "    if (!last) return;\n"
               "    __threadfence();\n"
               "    acc = " + ident + ";\n"
               "    for (int k = 0; k < 16; k++) {\n"
               "        const long long i = k * 256 + threadIdx.x;\n"
               "        acc = hg_op(acc, i < gridDim.x ? ((volatile " + A + "*)part)[i] : ident);\n"
               "    }\n"
               "    __syncthreads();\n" + tree("*result") + "}\n";
    } else if (r->op == "compress" || r->op == "map") {
        if (r->kids.empty()) return set_error(E_DOMAIN, "chain: %s needs operands", r->op.c_str());
        bool isc = r->op == "compress";
        // mask (compress) or values (map) are produced row by row, CH_UNROLL
        // rows per thread and round with all their loads issued before the
        // first store (the outputs are fresh buffers, never the inputs);
        // compress writes the mask and the values into scratch and compacts
        // afterwards
        constexpr int CH_UNROLL = 4;
        std::string body;
        for (int u = 0; u < CH_UNROLL; u++) {
            g.vsuffix = "_" + std::to_string(u);
            const std::string iu = "i" + std::to_string(u);
            const std::string mask = isc ? g.expr(r->kids[0].get()) : "";
            std::vector<std::string> outs;
            for (size_t k = isc ? 1 : 0; k < r->kids.size(); k++) {
                outs.push_back(g.expr(r->kids[k].get()));
                if (u == 0) cm->out_typ.push_back(r->kids[k]->typ);
            }
            body += "        if (" + iu + " < n) {\n" +
                    (isc ? "            const bool m = " + mask + ";\n            mask[" + iu + "] = m;\n" : "");
            for (size_t k = 0; k < outs.size(); k++)
                body += std::string("            ") + (isc ? "if (m) " : "") + "((" + ctype(cm->out_typ[k]) + "*)outs[" +
                        std::to_string(k) + "])[" + iu + "] = " + outs[k] + ";\n";
            body += "        }\n";
        }
        g.vsuffix.clear();
        if (!g.err.empty()) return set_error(E_DOMAIN, "chain: %s", g.err.c_str());
        if (isc && r->kids[0]->typ != H_B) return set_error(E_DOMAIN, "chain: compress mask must be bool");
        std::string ld;
        for (int u = 0; u < CH_UNROLL; u++) {
            const std::string iu = "i" + std::to_string(u);
            ld += "        const long long " + iu + " = i + " + std::to_string(u) + " * stride;\n";
            for (int k = 0; k < nin; k++)
                if (g.used[k])
                    ld += std::string("        const ") + ctype(types[k]) + " v" + std::to_string(k) + "_" + std::to_string(u) +
                          " = " + iu + " < n ? ((const " + ctype(types[k]) + "*)cols[" + std::to_string(k) + "])[" + iu +
                          "] : (" + ctype(types[k]) + ")0;\n";
        }
        src += "extern \"C\" __global__ void __launch_bounds__(256) chain_kernel(const void* const* cols, long long n, "
               "unsigned char* mask, void* const* outs, unsigned* derr) {\n    bool dz = false;\n"
               "    const long long stride = (long long)gridDim.x * blockDim.x;\n"
               "    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += " +
               std::to_string(CH_UNROLL) + " * stride) {\n" + ld + body + "    }\n    if (dz) atomicOr(derr, 4u);\n}\n";
    } else {
        return set_error(E_DOMAIN, "chain: unknown sink %s (sum|min|max|count|compress|map)", r->op.c_str());
    }
    cm->may_fail = g.uses_div;
    Nvrtc* nv = nvrtc();
    if (!nv) return set_error(E_NOT_IMPL, "chain compilation needs libnvrtc, which could not be opened");
    nvrtcProgram_t prog;
    if (nv->create(&prog, src.c_str(), "chain.cu", 0, nullptr, nullptr)) return set_error(E_DEVICE, "nvrtcCreateProgram failed");
    const char* opts[] = {"--gpu-architecture=sm_103a", "-default-device", "-std=c++17", "--fmad=false"};
    int rc = nv->compile(prog, 4, opts);
    if (rc) {
        size_t ls = 0;
        nv->logsize(prog, &ls);
        std::string log(ls, '\0');
        nv->log(prog, &log[0]);
        nv->destroy(&prog);
        return set_error(E_DEVICE, "chain compile failed: %.400s", log.c_str());
    }
    size_t cs = 0;
    nv->cubinsize(prog, &cs);
    std::vector<char> cubin(cs);
    nv->cubin(prog, cubin.data());
    nv->destroy(&prog);
    HG_CU(cudaLibraryLoadData(&cm->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    HG_CU(cudaLibraryGetKernel(&cm->kern, cm->lib, "chain_kernel"));
    c->cache[key] = cm;
    *out = cm;
    return 0;
}

I tree_reduce_any(int typ, int op, const void* part, long long n, void* result);

static I run_chain(hgpu_chain_s* c, V z, V* zs_many, V* x) {
    std::vector<int> types;
    size_t nin = 0;
    {  // inputs referenced by the program decide how many x[] entries are read
        std::vector<Node*> st{c->root.get()};
        int mx = -1;
        while (!st.empty()) {
            Node* n = st.back();
            st.pop_back();
            if (n->op == "x" && n->col > mx) mx = n->col;
            for (auto& k : n->kids) st.push_back(k.get());
        }
        nin = (size_t)(mx + 1);
    }
    long long n = -1;
    std::vector<const void*> ptrs(nin);
    for (size_t k = 0; k < nin; k++) {
        if (!is_basic(x[k]->typ)) return E_DOMAIN;
        types.push_back(x[k]->typ);
        if (x[k]->len != 1) {
            if (n >= 0 && n != x[k]->len) return E_LENGTH;
            n = x[k]->len;
        }
    }
    if (n < 0) n = 1;
    for (size_t k = 0; k < nin; k++) {
        if (x[k]->len == 1 && n > 1) return set_error(E_NOT_IMPL, "chain: pass scalars as literals");
        HG_CHECK(in_ptr(x[k], &ptrs[k]));
    }
    std::shared_ptr<Compiled> cm;
    HG_CHECK(compile_chain(c, types, &cm));
    const void** dcols = (const void**)salloc(16 + nin * sizeof(void*));
    if (!dcols) return E_DEVICE_OOM;
    if (nin) HG_CU(cudaMemcpyAsync(dcols, ptrs.data(), nin * sizeof(void*), cudaMemcpyHostToDevice, g_stream));
    if (cm->sink == "map") {
        // the values go straight into the outputs; with no operation that
        // can fail there is nothing to read back, so no wait
        V single[1] = {z};
        V* zs = zs_many ? zs_many : single;
        const size_t no = cm->out_typ.size();
        if (no > 1 && !zs_many) return set_error(E_DOMAIN, "chain: map writes several outputs; use hgpuChainRunMany");
        std::vector<void*> outs(no);
        const long long mark = out_mark();
        for (size_t k = 0; k < no; k++) HG_CHECK(alloc_out(zs[k], cm->out_typ[k], n, &outs[k]));
        void** douts = (void**)salloc(16 + no * sizeof(void*));
        if (!douts) return E_DEVICE_OOM;
        HG_CU(cudaMemcpyAsync(douts, outs.data(), no * sizeof(void*), cudaMemcpyHostToDevice, g_stream));
        long long nn = n;
        unsigned char* nomask = nullptr;
        void* args[] = {&dcols, &nn, &nomask, &douts, &g_derr};
        unsigned grid = grid_for(n, 256);
        if (grid > (unsigned)g_sms * 16) grid = g_sms * 16;
        {
            LaunchScope ls("chain");
            HG_CU(cudaLaunchKernel((const void*)cm->kern, dim3(grid), dim3(256), args, 0, g_stream));
        }
        HG_CHECK(last_launch_error());
        if (cm->may_fail) {  // a division by zero fails the call, as the builtin's checkZero does
            const I e = check_device_errors();
            if (e) {
                out_rewind(mark);
                return e;
            }
        }
        for (size_t k = 0; k < no; k++) HG_CHECK(finish_out(zs[k], outs[k]));
        return 0;
    }
    if (cm->sink == "compress") {
        size_t no = cm->out_typ.size();
        std::vector<void*> outs(no);
        for (size_t k = 0; k < no; k++) {
            outs[k] = salloc((size_t)(n > 0 ? n : 1) * esize(cm->out_typ[k]));
            if (!outs[k]) return E_DEVICE_OOM;
        }
        void** douts = (void**)salloc(16 + no * sizeof(void*));
        uint8_t* mask = (uint8_t*)salloc((size_t)(n > 0 ? n : 1));
        if (!douts || !mask) return E_DEVICE_OOM;
        HG_CU(cudaMemcpyAsync(douts, outs.data(), no * sizeof(void*), cudaMemcpyHostToDevice, g_stream));
        long long nn = n;
        void* args[] = {&dcols, &nn, &mask, &douts, &g_derr};
        unsigned grid = grid_for(n, 256);
        if (grid > (unsigned)g_sms * 16) grid = g_sms * 16;
        {
            LaunchScope ls("chain");
            HG_CU(cudaLaunchKernel((const void*)cm->kern, dim3(grid), dim3(256), args, 0, g_stream));
        }
        HG_CHECK(check_device_errors());
        if (!zs_many) return set_error(E_DOMAIN, "chain: compress writes several outputs; use hgpuChainRunMany");
        V* zs = zs_many;
        long long* rows = (long long*)salloc((size_t)(n > 0 ? n : 1) * 8);
        long long cnt = 0;
        if (!rows) return E_DEVICE_OOM;
        HG_CHECK(compact_rows(mask, n, rows, &cnt));
        for (size_t k = 0; k < no; k++) {
            void* d;
            HG_CHECK(alloc_out(zs[k], cm->out_typ[k], cnt, &d));
            HG_CHECK(gather_into(outs[k], n, esize(cm->out_typ[k]), rows, H_L, d, cnt));
            HG_CHECK(finish_out(zs[k], d));
        }
        return 0;
    }
    // reductions
    long long tiles = (n + TILE_SUM - 1) / TILE_SUM;
    if (tiles < 1) tiles = 1;
    int es = esize(cm->acc_typ);
    void* part = salloc((size_t)tiles * es);
    void* res = salloc(16);
    if (!part || !res) return E_DEVICE_OOM;
    long long nn = n;
    union { double d; float f; long long l; int i; short s; signed char c; bool b; } ident;
    ident.l = 0;
    if (cm->sink == "min" || cm->sink == "max") {
        bool mn = cm->sink == "min";
        switch (cm->acc_typ) {
        case H_E: ident.d = mn ? __builtin_huge_val() : -__builtin_huge_val(); break;
        case H_F: ident.f = mn ? __builtin_huge_valf() : -__builtin_huge_valf(); break;
        case H_L: ident.l = mn ? LLONG_MAX : LLONG_MIN; break;
        case H_I: ident.i = mn ? INT32_MAX : INT32_MIN; break;
        case H_H: ident.s = mn ? INT16_MAX : INT16_MIN; break;
        case H_J: ident.c = mn ? INT8_MAX : INT8_MIN; break;
        default: ident.b = mn; break;
        }
    }
    // up to one tile of tile partials: the last block reduces them in the
    // same launch; more: a separate tree over the partials
    const bool one_launch = tiles <= TILE_SUM;
    unsigned* done = (unsigned*)salloc(16);
    if (!done) return E_DEVICE_OOM;
    void* rptr = one_launch ? res : nullptr;
    if (one_launch) HG_CU(cudaMemsetAsync(done, 0, 4, g_stream));
    void* args[] = {&dcols, &nn, &part, &ident, &g_derr, &done, &rptr};
    {
        LaunchScope ls("chain");
        HG_CU(cudaLaunchKernel((const void*)cm->kern, dim3((unsigned)tiles), dim3(256), args, 0, g_stream));
    }
    if (!one_launch) {
        int op = cm->sink == "min" ? 1 : cm->sink == "max" ? 2 : 0;
        HG_CHECK(tree_reduce_any(cm->acc_typ, op, part, tiles, res));
    }
    HG_CHECK(check_device_errors());
    z->typ = cm->acc_typ;
    z->len = 1;
    return finish_out(z, res);
}

}  // namespace hg

using namespace hg;

extern "C" {

I hgpuChainCreate(hgpuChain* out, const char* program) {
    HG_CHECK(ensure_init());
    auto c = new hgpu_chain_s();
    c->text = program;
    std::string err;
    const char* p = c->text.c_str();
    c->root = parse(p, err);
    if (!c->root) { delete c; return set_error(E_DOMAIN, "chain parse error: %s", err.c_str()); }
    *out = c;
    return 0;
}

I hgpuChainRun(hgpuChain c, V z, V* x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    return run_chain(c, z, nullptr, x);
}

I hgpuChainRunMany(hgpuChain c, V* z, V* x) {
    HG_CHECK(ensure_init());
    ScratchScope ss;
    return run_chain(c, z[0], z, x);
}

I hgpuChainDestroy(hgpuChain c) {
    if (c) {
        for (auto& kv : c->cache)
            if (kv.second->lib) cudaLibraryUnload(kv.second->lib);
        delete c;
    }
    return 0;
}

}  // extern "C"
