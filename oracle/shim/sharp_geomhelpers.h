/* Test-infrastructure shim (see sharp.h) */
#ifndef SHIM_SHARP_GEOMHELPERS_H
#define SHIM_SHARP_GEOMHELPERS_H
#include "sharp.h"
void sharp_make_weighted_healpix_geom_info(int nside, int stride, const double *weight,
                                           sharp_geom_info **geom_info);
void sharp_destroy_geom_info(sharp_geom_info *info);
#endif
