/* Prototype-only stand-in for the PCRE2 8-bit API header.
 *
 * Oracle test infrastructure: used only to compile the reference builtin
 * library into oracle/_ref/ for golden vectors.  The reference's @like
 * builtin is the only PCRE2 user.  Where the system has libpcre2-8 the
 * Makefile defines REF_PCRE2_SYSTEM and links it (the names below map to its
 * _8 exports), so @like runs as in the reference; elsewhere ref_shim.c
 * defines the functions as stubs that abort if ever called.  Names and
 * signatures follow the public PCRE2 10.x API.
 */
#ifndef HGPU_REF_PCRE2_STUB_H
#define HGPU_REF_PCRE2_STUB_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#ifdef REF_PCRE2_SYSTEM
/* the system's libpcre2-8 exports the 8-bit API with a _8 suffix */
#define pcre2_compile pcre2_compile_8
#define pcre2_code_free pcre2_code_free_8
#define pcre2_config pcre2_config_8
#define pcre2_pattern_info pcre2_pattern_info_8
#define pcre2_jit_compile pcre2_jit_compile_8
#define pcre2_jit_match pcre2_jit_match_8
#define pcre2_match pcre2_match_8
#define pcre2_match_data_create_from_pattern pcre2_match_data_create_from_pattern_8
#define pcre2_match_data_free pcre2_match_data_free_8
#define pcre2_match_context_create pcre2_match_context_create_8
#define pcre2_match_context_free pcre2_match_context_free_8
#define pcre2_jit_stack_create pcre2_jit_stack_create_8
#define pcre2_jit_stack_assign pcre2_jit_stack_assign_8
#define pcre2_jit_stack_free pcre2_jit_stack_free_8
#endif
typedef const unsigned char *PCRE2_SPTR;
typedef size_t PCRE2_SIZE;
typedef struct pcre2_code_8 pcre2_code;
typedef struct pcre2_match_data_8 pcre2_match_data;
typedef struct pcre2_match_context_8 pcre2_match_context;
typedef struct pcre2_general_context_8 pcre2_general_context;
typedef struct pcre2_compile_context_8 pcre2_compile_context;
typedef struct pcre2_jit_stack_8 pcre2_jit_stack;
#define PCRE2_ANCHORED 0x80000000u
#define PCRE2_NO_UTF_CHECK 0x40000000u
#define PCRE2_JIT_COMPLETE 0x00000001u
#define PCRE2_CONFIG_JIT 1
#define PCRE2_INFO_JITSIZE 13
pcre2_code *pcre2_compile(PCRE2_SPTR, PCRE2_SIZE, uint32_t, int *, PCRE2_SIZE *, pcre2_compile_context *);
void pcre2_code_free(pcre2_code *);
int pcre2_config(uint32_t, void *);
int pcre2_pattern_info(const pcre2_code *, uint32_t, void *);
int pcre2_jit_compile(pcre2_code *, uint32_t);
int pcre2_jit_match(const pcre2_code *, PCRE2_SPTR, PCRE2_SIZE, PCRE2_SIZE, uint32_t, pcre2_match_data *, pcre2_match_context *);
int pcre2_match(const pcre2_code *, PCRE2_SPTR, PCRE2_SIZE, PCRE2_SIZE, uint32_t, pcre2_match_data *, pcre2_match_context *);
pcre2_match_data *pcre2_match_data_create_from_pattern(const pcre2_code *, pcre2_general_context *);
void pcre2_match_data_free(pcre2_match_data *);
pcre2_match_context *pcre2_match_context_create(pcre2_general_context *);
void pcre2_match_context_free(pcre2_match_context *);
pcre2_jit_stack *pcre2_jit_stack_create(PCRE2_SIZE, PCRE2_SIZE, pcre2_general_context *);
void pcre2_jit_stack_assign(pcre2_match_context *, void *, void *);
void pcre2_jit_stack_free(pcre2_jit_stack *);
#ifdef __cplusplus
}
#endif
#endif
