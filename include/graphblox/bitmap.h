/* Layout-identical declaration of the reference's struct Bitmap
 * (01_host/include/structures/bitmap.h:23-30): bit v of the set is bit
 * v % 32 of bitarray[v / 32]. Needed by the BFS step prototypes; used only
 * where the reference's own headers are not on the include path. */
#ifndef BITMAP_H
#define BITMAP_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
struct Bitmap {
    uint32_t real_size;
    uint32_t size;
    uint32_t numSetBits;
    uint32_t *bitarray;
};
#ifdef __cplusplus
}
#endif
#endif
