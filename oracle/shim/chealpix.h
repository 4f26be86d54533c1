/* Test-infrastructure shim: the chealpix calls of src/pixelize.c, src/io_gh.c,
 * src/healpix_extra.c and src/main_jt.c, backed by the oracle's restatement of
 * the RING and NESTED schemes. */
#ifndef SHIM_CHEALPIX_H
#define SHIM_CHEALPIX_H
void vec2pix_ring(long nside, const double *vec, long *ipix);
long nside2npix(long nside);
void ring2nest(long nside, long ipring, long *ipnest);
void nest2ring(long nside, long ipnest, long *ipring);
#endif
