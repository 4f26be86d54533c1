/* Test-infrastructure shim: the libsharp calls of src/healpix_extra.c:44-130,
 * implemented in oracle/jt_shim.c over the oracle's FP64 transforms. */
#ifndef SHIM_SHARP_H
#define SHIM_SHARP_H
typedef struct sharp_alm_info sharp_alm_info;
typedef struct sharp_geom_info sharp_geom_info;
typedef enum { SHARP_MAP2ALM = 0, SHARP_ALM2MAP = 1 } sharp_jobtype;
enum { SHARP_DP = 1 << 4 };
void sharp_execute(sharp_jobtype type, int spin, void *alm, void *map, const sharp_geom_info *geom_info,
                   const sharp_alm_info *alm_info, int ntrans, int flags, double *time,
                   unsigned long long *opcnt);
#endif
