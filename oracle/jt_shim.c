/*
 * Test-infrastructure shim implementations that let the reference's JoinT
 * sources (src/main_jt.c, io_jt.c, common_jt.c, common.c, healpix_extra.c)
 * build and run here: GSL RNG -> oracle MT19937; chealpix RING/NESTED ->
 * oracle restatement; libsharp map2alm/alm2map -> oracle FP64 transforms
 * (float maps and a_lm in and out, as the reference's single-precision build
 * asks); cfitsio -> a minimal reader/writer of one binary-table HDU of float or
 * double columns (big-endian, 2880-byte blocks, FITS standard 4.0).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "common_jt.h"
#include <fitsio.h>
#include <chealpix.h>
#include "sharp.h"
#include "sharp_almhelpers.h"
#include "sharp_geomhelpers.h"
#include "orc.h"

/* ---- GSL RNG ---- */
struct gsl_rng { orc_mt mt; };
static const gsl_rng_type mt_type = {"mt19937"};
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) { (void)T; return (gsl_rng *)calloc(1, sizeof(gsl_rng)); }
void gsl_rng_set(const gsl_rng *r, unsigned long int s) { orc_mt_seed((orc_mt *)&r->mt, (uint32_t)s); }
double gsl_rng_uniform(const gsl_rng *r) { return orc_mt_uniform((orc_mt *)&r->mt); }
void gsl_rng_free(gsl_rng *r) { free(r); }
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu)
{
  (void)r; (void)mu;
  fprintf(stderr, "shim: gsl_ran_poisson is not on the JoinT path\n");
  abort();
}

/* ---- chealpix ---- */
long nside2npix(long nside) { return 12 * nside * nside; }
void ring2nest(long nside, long ipring, long *ipnest) { *ipnest = orc_ring2nest(nside, ipring); }
void nest2ring(long nside, long ipnest, long *ipring) { *ipring = orc_nest2ring(nside, ipnest); }

/* ---- libsharp ---- */
struct sharp_alm_info { int lmax; };
struct sharp_geom_info { int nside; };
void sharp_make_triangular_alm_info(int lmax, int mmax, int stride, sharp_alm_info **alm_info)
{
  if (mmax != lmax || stride != 1) { fprintf(stderr, "shim: only triangular a_lm\n"); abort(); }
  *alm_info = malloc(sizeof(sharp_alm_info));
  (*alm_info)->lmax = lmax;
}
void sharp_destroy_alm_info(sharp_alm_info *info) { free(info); }
void sharp_make_weighted_healpix_geom_info(int nside, int stride, const double *weight,
                                           sharp_geom_info **geom_info)
{
  if (stride != 1 || weight) { fprintf(stderr, "shim: only unit ring weights\n"); abort(); }
  *geom_info = malloc(sizeof(sharp_geom_info));
  (*geom_info)->nside = nside;
}
void sharp_destroy_geom_info(sharp_geom_info *info) { free(info); }
void sharp_execute(sharp_jobtype type, int spin, void *alm, void *map, const sharp_geom_info *geom_info,
                   const sharp_alm_info *alm_info, int ntrans, int flags, double *time,
                   unsigned long long *opcnt)
{
  (void)time; (void)opcnt;
  if (spin != 0 || (flags & SHARP_DP)) { fprintf(stderr, "shim: only spin-0 single-precision jobs\n"); abort(); }
  const long nside = geom_info->nside, npix = 12 * nside * nside;
  const int lmax = alm_info->lmax;
  const long nalm = orc_nalms(lmax);
  float **maps = (float **)map, **alms = (float **)alm; /* float complex a_lm as (re, im) pairs */
  double *md = malloc(sizeof(double) * npix), *ad = malloc(sizeof(double) * 2 * nalm);
  for (int t = 0; t < ntrans; t++) {
    if (type == SHARP_MAP2ALM) {
      for (long i = 0; i < npix; i++) md[i] = maps[t][i];
      orc_map2alm(nside, lmax, md, ad);
      for (long i = 0; i < 2 * nalm; i++) alms[t][i] = (float)ad[i];
    } else {
      for (long i = 0; i < 2 * nalm; i++) ad[i] = alms[t][i];
      orc_alm2map(nside, lmax, ad, md);
      for (long i = 0; i < npix; i++) maps[t][i] = (float)md[i];
    }
  }
  free(md);
  free(ad);
}

/* ---- cfitsio (one binary table of E/D columns) ---- */
#define NCARD_MAX 256
#define NCOL_MAX 8
struct shim_fitsfile {
  char name[512];
  int writing;
  /* reader: the extension's header cards and its data */
  char cards[NCARD_MAX][81];
  int ncards;
  unsigned char *data;
  long row_bytes, nrows;
  int ncols, repeat[NCOL_MAX], size[NCOL_MAX], offset[NCOL_MAX];
  char type[NCOL_MAX];
  /* writer */
  int wcols;
  char ttype[NCOL_MAX][32], tform[NCOL_MAX][16], tunit[NCOL_MAX][16], extname[32];
  char wcards[NCARD_MAX][81];
  int nwcards;
  float *wdata[NCOL_MAX];
  long wrows;
};

static const char *card_value(fitsfile *f, const char *key)
{
  size_t kl = strlen(key);
  for (int i = 0; i < f->ncards; i++)
    if (!strncmp(f->cards[i], key, kl) && (f->cards[i][kl] == ' ' || f->cards[i][kl] == '=') &&
        f->cards[i][8] == '=')
      return f->cards[i] + 10;
  return NULL;
}

static int read_header(FILE *fp, char cards[][81], int *ncards)
{
  char block[2880];
  *ncards = 0;
  for (;;) {
    if (fread(block, 1, 2880, fp) != 2880) return -1;
    for (int i = 0; i < 36; i++) {
      const char *c = block + 80 * i;
      if (!strncmp(c, "END     ", 8)) return 0;
      if (*ncards < NCARD_MAX) {
        memcpy(cards[*ncards], c, 80);
        cards[*ncards][80] = 0;
        (*ncards)++;
      }
    }
  }
}

int fits_open_file(fitsfile **fo, const char *name, int mode, int *status)
{
  (void)mode;
  if (*status) return *status;
  FILE *fp = fopen(name, "rb");
  if (!fp) return *status = 104;
  fitsfile *f = calloc(1, sizeof(fitsfile));
  snprintf(f->name, sizeof(f->name), "%s", name);
  char prim[NCARD_MAX][81];
  int np;
  if (read_header(fp, prim, &np) || read_header(fp, f->cards, &f->ncards)) {
    fclose(fp);
    free(f);
    return *status = 107;
  }
  const char *v;
  f->row_bytes = (v = card_value(f, "NAXIS1")) ? atol(v) : 0;
  f->nrows = (v = card_value(f, "NAXIS2")) ? atol(v) : 0;
  f->ncols = (v = card_value(f, "TFIELDS")) ? atoi(v) : 0;
  int off = 0;
  for (int c = 0; c < f->ncols && c < NCOL_MAX; c++) {
    char key[16];
    snprintf(key, sizeof(key), "TFORM%d", c + 1);
    v = card_value(f, key);
    const char *q = v ? strchr(v, '\'') : NULL;
    int rep = 1;
    char t = 'E';
    if (q) {
      q++;
      if (*q >= '0' && *q <= '9') rep = atoi(q);
      while (*q >= '0' && *q <= '9') q++;
      t = *q;
    }
    f->repeat[c] = rep;
    f->type[c] = t;
    f->size[c] = t == 'D' ? 8 : 4;
    f->offset[c] = off;
    off += rep * f->size[c];
  }
  f->data = malloc((size_t)f->row_bytes * f->nrows + 1);
  if (fread(f->data, 1, (size_t)f->row_bytes * f->nrows, fp) != (size_t)f->row_bytes * f->nrows) *status = 107;
  fclose(fp);
  *fo = f;
  return *status;
}

int fits_movabs_hdu(fitsfile *f, int hdu, int *hdutype, int *status)
{
  (void)f;
  if (hdu != 2) return *status = 301;
  if (hdutype) *hdutype = BINARY_TBL;
  return *status;
}

int fits_read_key_lng(fitsfile *f, const char *key, long *value, char *comment, int *status)
{
  (void)comment;
  if (*status) return *status;
  const char *v = card_value(f, key);
  if (!v) return *status = 202;
  *value = atol(v);
  return 0;
}

int fits_read_keys_lng(fitsfile *f, const char *root, int nstart, int nmax, long *value, int *nfound,
                       int *status)
{
  if (*status) return *status;
  *nfound = 0;
  for (int i = 0; i < nmax; i++) {
    char key[16];
    snprintf(key, sizeof(key), "%s%d", root, nstart + i);
    const char *v = card_value(f, key);
    if (v) {
      value[i] = atol(v);
      (*nfound)++;
    }
  }
  return 0;
}

int fits_read_key(fitsfile *f, int datatype, const char *key, void *value, char *comment, int *status)
{
  (void)comment;
  if (*status) return *status;
  const char *v = card_value(f, key);
  if (!v) return *status = 202;
  if (datatype == TSTRING) {
    const char *a = strchr(v, '\'');
    const char *b = a ? strchr(a + 1, '\'') : NULL;
    if (!a || !b) return *status = 204;
    int n = (int)(b - a - 1);
    while (n > 0 && a[n] == ' ') n--;
    memcpy(value, a + 1, n);
    ((char *)value)[n] = 0;
  } else if (datatype == TLONG) {
    *(long *)value = atol(v);
  } else {
    return *status = 410;
  }
  return 0;
}

static double be_value(const unsigned char *p, char type)
{
  if (type == 'D') {
    uint64_t u = 0;
    for (int i = 0; i < 8; i++) u = (u << 8) | p[i];
    double d;
    memcpy(&d, &u, 8);
    return d;
  }
  uint32_t u = 0;
  for (int i = 0; i < 4; i++) u = (u << 8) | p[i];
  float x;
  memcpy(&x, &u, 4);
  return x;
}

int fits_read_col(fitsfile *f, int datatype, int colnum, long long firstrow, long long firstelem,
                  long long nelem, void *nulval, void *array, int *anynul, int *status)
{
  (void)nulval;
  if (*status) return *status;
  if (colnum < 1 || colnum > f->ncols) return *status = 302;
  const int c = colnum - 1, rep = f->repeat[c];
  if (anynul) *anynul = 0;
  for (long long e = 0; e < nelem; e++) {
    const long long g = (firstrow - 1) * rep + (firstelem - 1) + e;
    const long long row = g / rep, k = g % rep;
    if (row >= f->nrows) return *status = 307;
    const double v = be_value(f->data + row * f->row_bytes + f->offset[c] + k * f->size[c], f->type[c]);
    if (datatype == TFLOAT) ((float *)array)[e] = (float)v;
    else if (datatype == TDOUBLE) ((double *)array)[e] = v;
    else return *status = 410;
  }
  return 0;
}

int fits_create_file(fitsfile **fo, const char *name, int *status)
{
  if (*status) return *status;
  fitsfile *f = calloc(1, sizeof(fitsfile));
  snprintf(f->name, sizeof(f->name), "%s", name[0] == '!' ? name + 1 : name);
  f->writing = 1;
  *fo = f;
  return 0;
}

int fits_create_tbl(fitsfile *f, int tbltype, long long naxis2, int tfields, char **ttype, char **tform,
                    char **tunit, const char *extname, int *status)
{
  (void)tbltype; (void)naxis2;
  if (*status) return *status;
  if (tfields > NCOL_MAX) return *status = 216;
  f->wcols = tfields;
  for (int i = 0; i < tfields; i++) {
    snprintf(f->ttype[i], sizeof(f->ttype[i]), "%s", ttype[i]);
    snprintf(f->tform[i], sizeof(f->tform[i]), "%s", tform[i]);
    snprintf(f->tunit[i], sizeof(f->tunit[i]), "%s", tunit ? tunit[i] : "");
  }
  snprintf(f->extname, sizeof(f->extname), "%s", extname ? extname : "");
  return 0;
}

static void add_card(char cards[][81], int *n, const char *text)
{
  if (*n >= NCARD_MAX) return;
  snprintf(cards[*n], 81, "%-80s", text);
  (*n)++;
}

int fits_write_key(fitsfile *f, int datatype, const char *key, void *value, const char *comment, int *status)
{
  if (*status) return *status;
  char buf[128], val[80];
  if (datatype == TSTRING) {
    char s[72];
    snprintf(s, sizeof(s), "'%-8s'", (const char *)value);
    snprintf(val, sizeof(val), "%-20s", s);
  } else if (datatype == TLONG) {
    snprintf(val, sizeof(val), "%20ld", *(long *)value);
  } else {
    return *status = 410;
  }
  snprintf(buf, sizeof(buf), "%-8.8s= %s / %s", key, val, comment ? comment : "");
  buf[80] = 0;
  add_card(f->wcards, &f->nwcards, buf);
  return 0;
}

int fits_write_comment(fitsfile *f, const char *comment, int *status)
{
  if (*status) return *status;
  char buf[128];
  snprintf(buf, sizeof(buf), "COMMENT %s", comment);
  buf[80] = 0;
  add_card(f->wcards, &f->nwcards, buf);
  return 0;
}

int fits_write_col(fitsfile *f, int datatype, int colnum, long long firstrow, long long firstelem,
                   long long nelem, void *array, int *status)
{
  if (*status) return *status;
  if (datatype != TFLOAT || firstrow != 1 || firstelem != 1 || colnum < 1 || colnum > f->wcols)
    return *status = 410;
  free(f->wdata[colnum - 1]);
  f->wdata[colnum - 1] = malloc(sizeof(float) * nelem);
  memcpy(f->wdata[colnum - 1], array, sizeof(float) * nelem);
  if (nelem > f->wrows) f->wrows = nelem;
  return 0;
}

static void put_block_pad(FILE *fp, long written, int fill)
{
  long pad = (2880 - written % 2880) % 2880;
  for (long i = 0; i < pad; i++) fputc(fill, fp);
}

static void put_header(FILE *fp, char cards[][81], int n)
{
  for (int i = 0; i < n; i++) fwrite(cards[i], 1, 80, fp);
  char end[81];
  snprintf(end, sizeof(end), "%-80s", "END");
  fwrite(end, 1, 80, fp);
  put_block_pad(fp, 80L * (n + 1), ' ');
}

int fits_close_file(fitsfile *f, int *status)
{
  if (!f->writing) {
    free(f->data);
    free(f);
    return *status;
  }
  FILE *fp = fopen(f->name, "wb");
  if (!fp) return *status = 105;
  char cards[NCARD_MAX][81];
  int n = 0;
  char buf[128];
  add_card(cards, &n, "SIMPLE  =                    T / file does conform to FITS standard");
  add_card(cards, &n, "BITPIX  =                    8 / number of bits per data pixel");
  add_card(cards, &n, "NAXIS   =                    0 / number of data axes");
  add_card(cards, &n, "EXTEND  =                    T / FITS dataset may contain extensions");
  put_header(fp, cards, n);
  n = 0;
  add_card(cards, &n, "XTENSION= 'BINTABLE'           / binary table extension");
  add_card(cards, &n, "BITPIX  =                    8 / 8-bit bytes");
  add_card(cards, &n, "NAXIS   =                    2 / 2-dimensional binary table");
  snprintf(buf, sizeof(buf), "NAXIS1  = %20d / width of table in bytes", 4 * f->wcols);
  add_card(cards, &n, buf);
  snprintf(buf, sizeof(buf), "NAXIS2  = %20ld / number of rows in table", f->wrows);
  add_card(cards, &n, buf);
  add_card(cards, &n, "PCOUNT  =                    0 / size of special data area");
  add_card(cards, &n, "GCOUNT  =                    1 / one data group (required keyword)");
  snprintf(buf, sizeof(buf), "TFIELDS = %20d / number of fields in each row", f->wcols);
  add_card(cards, &n, buf);
  for (int c = 0; c < f->wcols; c++) {
    char s[48];
    snprintf(s, sizeof(s), "'%-8s'", f->ttype[c]);
    snprintf(buf, sizeof(buf), "TTYPE%-3d= %-20s", c + 1, s);
    add_card(cards, &n, buf);
    snprintf(s, sizeof(s), "'%-8s'", f->tform[c]);
    snprintf(buf, sizeof(buf), "TFORM%-3d= %-20s", c + 1, s);
    add_card(cards, &n, buf);
    snprintf(s, sizeof(s), "'%-8s'", f->tunit[c]);
    snprintf(buf, sizeof(buf), "TUNIT%-3d= %-20s", c + 1, s);
    add_card(cards, &n, buf);
  }
  if (f->extname[0]) {
    char s[48];
    snprintf(s, sizeof(s), "'%-8s'", f->extname);
    snprintf(buf, sizeof(buf), "EXTNAME = %-20s", s);
    add_card(cards, &n, buf);
  }
  for (int i = 0; i < f->nwcards; i++) add_card(cards, &n, f->wcards[i]);
  put_header(fp, cards, n);
  for (long r = 0; r < f->wrows; r++)
    for (int c = 0; c < f->wcols; c++) {
      float v = f->wdata[c] ? f->wdata[c][r] : 0.f;
      uint32_t u;
      memcpy(&u, &v, 4);
      unsigned char b[4] = {(unsigned char)(u >> 24), (unsigned char)(u >> 16), (unsigned char)(u >> 8),
                            (unsigned char)u};
      fwrite(b, 1, 4, fp);
    }
  put_block_pad(fp, 4L * f->wcols * f->wrows, 0);
  fclose(fp);
  for (int c = 0; c < NCOL_MAX; c++) free(f->wdata[c]);
  free(f);
  return *status;
}
