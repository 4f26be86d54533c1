/* Test-infrastructure shim: src/io_gh.c includes this; maps are dumped by the driver instead. */
#ifndef SHIM_FITSIO_H
#define SHIM_FITSIO_H
#endif
