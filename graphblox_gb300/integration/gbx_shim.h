/* Helpers shared by the cuda integration shims (the GraphBlox algorithm
 * symbols implemented on libgbx.so). */
#ifndef GBX_SHIM_H
#define GBX_SHIM_H
#include <stddef.h>
#include <stdint.h>

#include "gbx.h"
#include "graphCSR.h"

/* Device copy of a GraphCSR, uploaded on first use and cached (a few most
 * recent graphs, keyed by the GraphCSR pointer, its array pointers and a
 * fingerprint of its contents: every word of arrays up to 2^20 entries,
 * an even sample of 65,536 words plus both ends of larger ones). A graph
 * rewritten in place is uploaded again; a caller that changes only a few
 * entries of a large graph calls gbx_shim_release first.
 * Returns NULL and prints the library's message on failure. */
gbx_graph *gbx_shim_graph(struct GraphCSR *graph);
/* Drop the cached device copy of `graph` (call before freeing it). */
void gbx_shim_release(struct GraphCSR *graph);
/* 4 KiB-aligned zeroed host allocation, freed with free() like the
 * reference's my_malloc (01_host/src/utils_graph/myMalloc.c:54-66). */
void *gbx_shim_alloc(size_t bytes);
double gbx_shim_now(void);
/* prints "| <what> failed: <status> <message>" and returns NULL */
void *gbx_shim_fail(const char *what, int status);
void gbx_shim_not_available(const char *algorithm);
#endif
