/* Layout-identical declaration of the reference's struct ArrayQueue
 * (01_host/include/structures/arrayQueue.h:11-20): the current frontier is
 * queue[head, tail), the next one grows from tail_next. Needed by the BFS
 * step prototypes; used only where the reference's own headers are not on
 * the include path. */
#ifndef ARRAYQUEUE_H
#define ARRAYQUEUE_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "bitmap.h"
struct ArrayQueue {
    uint32_t head;
    uint32_t tail;
    uint32_t tail_next;
    uint32_t size;
    uint32_t *queue;
    struct Bitmap *q_bitmap;
    struct Bitmap *q_bitmap_next;
};
#ifdef __cplusplus
}
#endif
#endif
