// Ordered-map implementation of the JudyL subset declared in Judy.h.
// Test infrastructure for the oracle build only.
#include "Judy.h"

#include <map>

namespace {
typedef std::map<Word_t, Word_t> WordMap;
}

extern "C" void *JudyLIns(Pvoid_t *array, Word_t index, PJError_t) {
    if (*array == nullptr) *array = new WordMap();
    WordMap *m = static_cast<WordMap *>(*array);
    return &(*m)[index];
}

extern "C" void *JudyLFirst(Pcvoid_t array, Word_t *index, PJError_t) {
    if (array == nullptr) return nullptr;
    const WordMap *m = static_cast<const WordMap *>(array);
    auto it = m->lower_bound(*index);
    if (it == m->end()) return nullptr;
    *index = it->first;
    return const_cast<Word_t *>(&it->second);
}

extern "C" void *JudyLNext(Pcvoid_t array, Word_t *index, PJError_t) {
    if (array == nullptr) return nullptr;
    const WordMap *m = static_cast<const WordMap *>(array);
    auto it = m->upper_bound(*index);
    if (it == m->end()) return nullptr;
    *index = it->first;
    return const_cast<Word_t *>(&it->second);
}

extern "C" Word_t JudyLFreeArray(Pvoid_t *array, PJError_t) {
    if (*array == nullptr) return 0;
    WordMap *m = static_cast<WordMap *>(*array);
    Word_t bytes = (Word_t)(m->size() * 2 * sizeof(Word_t));
    delete m;
    *array = nullptr;
    return bytes;
}
