/* Test-infrastructure shim: the cfitsio calls of src/healpix_extra.c:132-224
 * (one binary-table HDU of float columns), implemented in oracle/jt_shim.c.
 * src/io_gh.c also includes this header; the GetHI driver never calls it. */
#ifndef SHIM_FITSIO_H
#define SHIM_FITSIO_H
typedef struct shim_fitsfile fitsfile;
#define READONLY 0
#define READWRITE 1
#define BINARY_TBL 2
#define TSTRING 16
#define TLONG 41
#define TFLOAT 42
#define TDOUBLE 82
int fits_open_file(fitsfile **f, const char *name, int mode, int *status);
int fits_movabs_hdu(fitsfile *f, int hdu, int *hdutype, int *status);
int fits_read_key_lng(fitsfile *f, const char *key, long *value, char *comment, int *status);
int fits_read_keys_lng(fitsfile *f, const char *root, int nstart, int nmax, long *value, int *nfound,
                       int *status);
int fits_read_key(fitsfile *f, int datatype, const char *key, void *value, char *comment, int *status);
int fits_read_col(fitsfile *f, int datatype, int colnum, long long firstrow, long long firstelem,
                  long long nelem, void *nulval, void *array, int *anynul, int *status);
int fits_close_file(fitsfile *f, int *status);
int fits_create_file(fitsfile **f, const char *name, int *status);
int fits_create_tbl(fitsfile *f, int tbltype, long long naxis2, int tfields, char **ttype, char **tform,
                    char **tunit, const char *extname, int *status);
int fits_write_key(fitsfile *f, int datatype, const char *key, void *value, const char *comment,
                   int *status);
int fits_write_comment(fitsfile *f, const char *comment, int *status);
int fits_write_col(fitsfile *f, int datatype, int colnum, long long firstrow, long long firstelem,
                   long long nelem, void *array, int *status);
#endif
