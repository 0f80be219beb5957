/* Layout-identical declaration of the reference's struct Arguments
 * (01_host/include/config/graphConfig.h:18-63) and its build macros, for
 * building the cuda integration without the reference tree. Inside the
 * reference build (INTEGRATION=cuda) the reference's own header is used. */
#ifndef GRAPHCONFIG_H
#define GRAPHCONFIG_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "mt19937.h"

#ifndef GBX_WEIGHTED
#define GBX_WEIGHTED 0
#endif
#ifndef GBX_DIRECTED
#define GBX_DIRECTED 0
#endif
#define WEIGHTED GBX_WEIGHTED
#define DIRECTED GBX_DIRECTED
#define DYNAMIC 0

struct Arguments {
    int wflag, xflag, sflag, Sflag, dflag;
    uint32_t binSize, verbosity, iterations, trials;
    double epsilon;
    uint32_t source, algorithm, datastructure, pushpull, sort;
    uint32_t lmode, lmode_l2, lmode_l3, mmode;
    uint32_t symmetric, weighted, delta;
    int pre_numThreads, algo_numThreads, ker_numThreads;
    char *fnameb;
    char *fnamel;
    uint32_t fnameb_format, convert_format;
    mt19937state mt19937var;
    uint32_t cache_size;
    char *kernel_name;
    int cu_id, device_index;
    char *xclbin_path;
    char *overlay_path;
    int ctrl_mode, endian_read, endian_write, flush_cache, bankGroupIndex;
};
#ifdef __cplusplus
}
#endif
#endif
