/* Test-infrastructure shim: types named in src/cosmo_mad.h:58-61 (unused on the path). */
#ifndef SHIM_GSL_SPLINE_H
#define SHIM_GSL_SPLINE_H
typedef struct gsl_interp_accel gsl_interp_accel;
typedef struct gsl_spline gsl_spline;
#endif
