/* Layout-identical declaration of the reference's mt19937state
 * (01_host/include/utils_graph/mt19937.h:58-62), needed because
 * struct Arguments embeds it. Used only where the reference's own headers
 * are not on the include path. */
#ifndef MT19937_H
#define MT19937_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct mt19937_stateStruct {
    unsigned long mt[624];
    int mti;
} mt19937state;
#ifdef __cplusplus
}
#endif
#endif
