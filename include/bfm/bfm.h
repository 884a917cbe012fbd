/* libbfm core state and allocator hooks.
 * ABI-identical to the reference's libbfm/src/bfm/bfm.h:6-34: same structs,
 * same prototypes, so existing C callers and the pybfm cffi binding link
 * against this library unchanged. */
#pragma once

#include <stdbool.h>
#include <stdlib.h>

/* Error record.  The GPU path fills it (has/msg/file/func/line) whenever an
 * entry point returns -1. */
typedef struct {
	bool has;
	char* msg;
	char const* file;
	char const* func;
	size_t line;
} bfm_err_t;

typedef void* (*bfm_alloc_t)(size_t size);
typedef void* (*bfm_realloc_t)(void* ptr, size_t size);
typedef void (*bfm_free_t)(void* ptr);

/* Every host-side buffer of the library is obtained through these hooks. */
typedef struct {
	bfm_err_t err;
	bfm_alloc_t alloc;
	bfm_realloc_t realloc;
	bfm_free_t free;
} bfm_state_t;

int bfm_state_create(bfm_state_t* state);                   /* ref state.c:6-14  */
int bfm_state_destroy(bfm_state_t* state);                  /* ref state.c:16-19 */
int bfm_set_alloc(bfm_state_t* state, bfm_alloc_t alloc);   /* ref state.c:21-24 */
int bfm_set_realloc(bfm_state_t* state, bfm_realloc_t realloc); /* ref state.c:26-29 */
int bfm_set_free(bfm_state_t* state, bfm_free_t free);      /* ref state.c:31-34 */
int bfm_err_print(bfm_state_t* state);                      /* ref state.c:36-46 */
