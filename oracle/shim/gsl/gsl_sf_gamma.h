/* Test-infrastructure shim: included by src/cosmo_mad.h, nothing used. */
#ifndef SHIM_GSL_SF_GAMMA_H
#define SHIM_GSL_SF_GAMMA_H
#endif
