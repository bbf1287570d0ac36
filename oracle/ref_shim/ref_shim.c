/* Link shim for building the reference builtin library as oracle/_ref/libref.so.
 *
 * Oracle test infrastructure only.  The reference's library sources
 * (src/horseir/v3/backend, util, global.cc, frontend/pretty.cc — the file set
 * of src/horseir/v3/make.sh:30-43) reference a few symbols from the parser /
 * optimizer, which are not part of that file set, and PCRE2 for @like.  None
 * of them is reached by the builtins exercised here, so they are defined as
 * inert placeholders; the PCRE2 ones abort if ever reached.
 */
#include <stdio.h>
#include <stdlib.h>
#include <stddef.h>
#include <stdint.h>

void *compiledMethodList = 0;
int findDefByName(void *chain, char *name) { (void)chain; (void)name; return 0; }
void *getNodeParams(void *n) { (void)n; return 0; }
void *getNodeFunc(void *n) { (void)n; return 0; }

#ifndef REF_PCRE2_SYSTEM
static void no_pcre(const char *f) {
    fprintf(stderr, "oracle/_ref: %s reached (PCRE2 is stubbed; @like is outside the path)\n", f);
    abort();
}
#define STUB(ret, name, ...) ret name(__VA_ARGS__) { no_pcre(#name); return (ret)0; }
STUB(void *, pcre2_compile, const unsigned char *a, size_t b, uint32_t c, int *d, size_t *e, void *f)
STUB(int, pcre2_config, uint32_t a, void *b)
STUB(int, pcre2_pattern_info, const void *a, uint32_t b, void *c)
STUB(int, pcre2_jit_compile, void *a, uint32_t b)
STUB(int, pcre2_jit_match, const void *a, const unsigned char *b, size_t c, size_t d, uint32_t e, void *f, void *g)
STUB(int, pcre2_match, const void *a, const unsigned char *b, size_t c, size_t d, uint32_t e, void *f, void *g)
STUB(void *, pcre2_match_data_create_from_pattern, const void *a, void *b)
STUB(void *, pcre2_match_context_create, void *a)
STUB(void *, pcre2_jit_stack_create, size_t a, size_t b, void *c)
void pcre2_code_free(void *a) { (void)a; no_pcre("pcre2_code_free"); }
void pcre2_match_data_free(void *a) { (void)a; no_pcre("pcre2_match_data_free"); }
void pcre2_match_context_free(void *a) { (void)a; no_pcre("pcre2_match_context_free"); }
void pcre2_jit_stack_assign(void *a, void *b, void *c) { (void)a; (void)b; (void)c; no_pcre("pcre2_jit_stack_assign"); }
void pcre2_jit_stack_free(void *a) { (void)a; no_pcre("pcre2_jit_stack_free"); }
#endif
