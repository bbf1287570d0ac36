/*
 * hgo_str.c — CPU oracle for @like (pfnLike, src/horseir/v3/backend/
 * h_primitive.cc:1670-1758).
 *
 * THIS IS TEST INFRASTRUCTURE, NOT THE PRODUCT (see hgo.h).  The reference
 * turns the SQL pattern into a regex (genLikeString, h_system.cc:319-334:
 * '%' -> ".*", '_' -> ".", '.' and '\' escaped, "^...$" around it) and runs
 * PCRE2 anchored (getLikePatten / LIKEMATCH, h_system.cc:478-496,
 * h_primitive.cc:1650-1654).  Such a regex holds literals, '.', '.*' and the
 * anchors only; this restatement decides it with a dynamic program over
 * (pattern position, text position): '.' is any byte but '\n' (PCRE2's
 * default newline), '$' also matches before a final '\n'.  A pattern with
 * other regex metacharacters would need a regex engine: E_NOT_IMPL.  One
 * pattern per call (y of length 1); one pattern per row: E_NOT_IMPL.  An
 * empty pattern is E_NULL_VALUE, the reference's check after
 * getLikePatten (which it reaches only after PCRE2 has crashed on it).
 */
#include "hgo.h"

enum { T_LIT = 0, T_ANY = 1, T_STAR = 2 };
typedef struct { int kind; unsigned char c; } Tok;

/* genLikeString's translation, as tokens; -1 when a regex metacharacter passes through */
static int like_tokens(const char *pat, Tok *t, int cap) {
    int m = 0;
    for (const unsigned char *p = (const unsigned char *)pat; *p; p++) {
        if (m >= cap) return -1;
        if (*p == '%') t[m++] = (Tok){T_STAR, 0};
        else if (*p == '_') t[m++] = (Tok){T_ANY, 0};
        else if (strchr("()[]{}*+?|^$", *p)) return -1;
        else t[m++] = (Tok){T_LIT, *p};
    }
    return m;
}

static B like_match(const Tok *t, int m, const unsigned char *s, L n, unsigned char *dp) {
    /* dp[i * (n + 1) + j]: tokens i.. match text j.. up to the end (or a final '\n') */
    for (int i = m; i >= 0; i--) {
        for (L j = n; j >= 0; j--) {
            B r;
            if (i == m) r = j == n || (j == n - 1 && s[j] == '\n');
            else if (t[i].kind == T_STAR) r = dp[(i + 1) * (n + 1) + j] || (j < n && s[j] != '\n' && dp[i * (n + 1) + j + 1]);
            else if (j == n) r = 0;
            else if (t[i].kind == T_ANY) r = s[j] != '\n' && dp[(i + 1) * (n + 1) + j + 1];
            else r = s[j] == t[i].c && dp[(i + 1) * (n + 1) + j + 1];
            dp[i * (n + 1) + j] = r;
        }
    }
    R dp[0];
}

static B like_one(const Tok *t, int m, const char *s) {
    L n = (L)strlen(s);
    unsigned char *dp = (unsigned char *)malloc((size_t)(m + 1) * (size_t)(n + 1));
    B r = like_match(t, m, (const unsigned char *)s, n, dp);
    free(dp);
    R r;
}

I pfnLike(V z, V x, V y) {
    I tx = vp(x), ty = vp(y);
    if (!(tx == H_C || tx == H_Q || tx == H_S) || !(ty == H_C || ty == H_Q || ty == H_S)) R E_DOMAIN;
    if (vn(y) != 1) R (tx == H_C || vn(x) == vn(y)) ? E_NOT_IMPL : E_LENGTH;
    const char *pat = ty == H_C ? (const char *)vg(y) : ty == H_S ? ((S *)vg(y))[0] : getSymbolStr(sL(y)[0]);
    if (!pat[0]) R E_NULL_VALUE;  /* genLikeString returns NULL; the reference then crashes in PCRE2 */
    Tok t[64];
    int m = like_tokens(pat, t, 64);
    if (m < 0) R E_NOT_IMPL;
    L lenZ = tx == H_C ? 1 : vn(x);
    initV(z, H_B, lenZ);
    if (tx == H_C) { sB(z)[0] = like_one(t, m, (const char *)vg(x)); R 0; }
#pragma omp parallel for
    for (L i = 0; i < lenZ; i++)
        sB(z)[i] = like_one(t, m, tx == H_Q ? getSymbolStr(sL(x)[i]) : ((S *)vg(x))[i]);
    R 0;
}
