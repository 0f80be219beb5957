/*
 * Minimal stand-in for the libJudy "JudyL" word->word map, used only to
 * compile the reference host (connectedComponents.c) in this container,
 * where libJudy is not installed.
 *
 * Test infrastructure, not product code: only the oracle build recipe
 * (oracle/build_ref.sh) puts this directory on the include path.
 *
 * Semantics kept from the published Judy API (judy.sourceforge.net,
 * JudyL(3)):
 *   JudyLIns(&A, k)       -> pointer to the value slot of key k (inserted as 0)
 *   JudyLFirst(A, &k)     -> first key >= k, or NULL
 *   JudyLNext(A, &k)      -> first key >  k, or NULL
 *   JudyLFreeArray(&A)    -> frees A, sets it to NULL, returns bytes freed
 * Keys iterate in ascending order, which is the only property the
 * reference relies on (Afforest's "most frequent sampled component" picks
 * the first maximum in key order).
 *
 * The reference frees its JudyL array with the JudySL macro JSLFA; here
 * both free routines release the same ordered map.
 */
#ifndef GBX_JUDY_SHIM_H
#define GBX_JUDY_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long Word_t;
typedef Word_t *PWord_t;
typedef void *Pvoid_t;
typedef const void *Pcvoid_t;
typedef void *PJError_t;

#define PJE0 ((PJError_t)0)

void *JudyLIns(Pvoid_t *array, Word_t index, PJError_t err);
void *JudyLFirst(Pcvoid_t array, Word_t *index, PJError_t err);
void *JudyLNext(Pcvoid_t array, Word_t *index, PJError_t err);
Word_t JudyLFreeArray(Pvoid_t *array, PJError_t err);

#define JLI(PV, PArray, Index) (PV) = (Word_t *)JudyLIns(&(PArray), (Index), PJE0)
#define JLF(PV, PArray, Index) (PV) = (Word_t *)JudyLFirst((PArray), &(Index), PJE0)
#define JLN(PV, PArray, Index) (PV) = (Word_t *)JudyLNext((PArray), &(Index), PJE0)
#define JLFA(Rc, PArray) (Rc) = JudyLFreeArray(&(PArray), PJE0)
#define JSLFA(Rc, PArray) (Rc) = JudyLFreeArray(&(PArray), PJE0)

#ifdef __cplusplus
}
#endif

#endif
