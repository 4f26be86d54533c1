/* Test-infrastructure shim: status codes named by src/cosmo.c:88-125. */
#ifndef SHIM_GSL_ERRNO_H
#define SHIM_GSL_ERRNO_H
enum { GSL_SUCCESS = 0, GSL_EDOM = 1, GSL_EMAXITER = 11, GSL_ETOL = 14, GSL_EUNDRFLW = 15,
       GSL_EROUND = 18, GSL_ESING = 21, GSL_EDIVERGE = 22 };
typedef void gsl_error_handler_t(const char *reason, const char *file, int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler_off(void);
#endif
