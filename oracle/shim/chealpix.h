/* Test-infrastructure shim: the chealpix calls of src/pixelize.c and
 * src/io_gh.c, backed by the oracle's restatement of the RING scheme. */
#ifndef SHIM_CHEALPIX_H
#define SHIM_CHEALPIX_H
void vec2pix_ring(long nside, const double *vec, long *ipix);
long nside2npix(long nside);
#endif
