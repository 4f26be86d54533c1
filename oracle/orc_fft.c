/*
 * Oracle (test infrastructure only): FP64 mixed-radix FFT and the 3D c2r the
 * reference obtains from FFTW (src/fourier.c:78-99, fftwf_plan_dft_c2r_3d,
 * sign +1, unnormalised).
 *
 * c2r semantics (FFTW documents only Hermitian input): inverse c2c along z
 * and y, then a 1D c2r along x that uses Re(X[0]) and Re(X[N/2]) and the
 * Hermitian extension X[N-k] = conj(X[k]).  The reference draws the kx=0 and
 * kx=N/2 planes without Hermitian symmetry (src/fourier.c:275-299); this
 * definition is the real part of the full complex inverse DFT of the
 * half-spectrum extended that way.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

typedef struct { double re, im; } cplx;

typedef struct {
  int n, nf;
  int fac[40];
  cplx *tw; /* exp(+2 pi i j / n) */
} fplan;

static void plan_init(fplan *p, int n)
{
  p->n = n;
  p->nf = 0;
  int m = n;
  while (m % 4 == 0) { p->fac[p->nf++] = 4; m /= 4; }
  while (m % 2 == 0) { p->fac[p->nf++] = 2; m /= 2; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) { p->fac[p->nf++] = f; m /= f; }
  p->fac[p->nf] = 1;
  p->tw = (cplx *)malloc(sizeof(cplx) * n);
  for (int j = 0; j < n; j++) {
    double a = 2 * M_PI * (double)j / n;
    p->tw[j].re = cos(a);
    p->tw[j].im = sin(a);
  }
}

static void plan_free(fplan *p) { free(p->tw); }

/* recursive decimation in time; out has n entries, in is read with stride is */
static void fft_rec(const fplan *P, cplx *out, const cplx *in, int n, int is, const int *f, int ts)
{
  if (n == 1) { out[0] = in[0]; return; }
  int p = f[0], m = n / p;
  for (int r = 0; r < p; r++) fft_rec(P, out + r * m, in + (size_t)r * is, m, is * p, f + 1, ts * p);
  cplx t[64], s[64];
  for (int k = 0; k < m; k++) {
    for (int r = 0; r < p; r++) {
      cplx a = out[r * m + k];
      cplx w = P->tw[((long)r * k * ts) % P->n];
      t[r].re = a.re * w.re - a.im * w.im;
      t[r].im = a.re * w.im + a.im * w.re;
    }
    for (int q = 0; q < p; q++) {
      double sr = 0, si = 0;
      for (int r = 0; r < p; r++) {
        cplx w = P->tw[((long)r * q * m * ts) % P->n];
        sr += t[r].re * w.re - t[r].im * w.im;
        si += t[r].re * w.im + t[r].im * w.re;
      }
      s[q].re = sr;
      s[q].im = si;
    }
    for (int q = 0; q < p; q++) out[q * m + k] = s[q];
  }
}

/* inverse (sign +1) unnormalised complex DFT of v (length n), via buffer tmp */
static void ifft(const fplan *P, cplx *v, cplx *tmp)
{
  fft_rec(P, tmp, v, P->n, 1, P->fac, 1);
  memcpy(v, tmp, sizeof(cplx) * P->n);
}

void orc_c2r_to_double(int n, const float *spec, double *out)
{
  int h = n / 2 + 1;
  size_t nh = (size_t)n * n * h;
  cplx *buf = (cplx *)malloc(sizeof(cplx) * nh);
  for (size_t i = 0; i < nh; i++) { buf[i].re = spec[2 * i]; buf[i].im = spec[2 * i + 1]; }
  fplan P;
  plan_init(&P, n);

  /* z axis: columns (y, kx), stride n*h */
#pragma omp parallel
  {
    cplx *v = (cplx *)malloc(sizeof(cplx) * n), *t = (cplx *)malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
    for (long c = 0; c < (long)n * h; c++) {
      for (int z = 0; z < n; z++) v[z] = buf[(size_t)z * n * h + c];
      ifft(&P, v, t);
      for (int z = 0; z < n; z++) buf[(size_t)z * n * h + c] = v[z];
    }
    /* y axis: columns (z, kx), stride h */
#pragma omp for schedule(static)
    for (long c = 0; c < (long)n * h; c++) {
      long z = c / h, kx = c % h;
      cplx *base = buf + (size_t)z * n * h + kx;
      for (int y = 0; y < n; y++) v[y] = base[(size_t)y * h];
      ifft(&P, v, t);
      for (int y = 0; y < n; y++) base[(size_t)y * h] = v[y];
    }
    /* x axis: Hermitian extension of each row, real part of the inverse */
#pragma omp for schedule(static)
    for (long row = 0; row < (long)n * n; row++) {
      const cplx *x = buf + (size_t)row * h;
      v[0].re = x[0].re; v[0].im = 0;
      for (int k = 1; k < n / 2; k++) {
        v[k] = x[k];
        v[n - k].re = x[k].re;
        v[n - k].im = -x[k].im;
      }
      v[n / 2].re = x[n / 2].re; v[n / 2].im = 0;
      ifft(&P, v, t);
      for (int i = 0; i < n; i++) out[(size_t)row * n + i] = v[i].re;
    }
    free(v);
    free(t);
  }
  plan_free(&P);
  free(buf);
}

void orc_c2r_inplace(int n, float *data)
{
  int h = n / 2 + 1;
  double *out = (double *)malloc(sizeof(double) * (size_t)n * n * n);
  orc_c2r_to_double(n, data, out);
  size_t pitch = 2 * (size_t)h;
  for (size_t row = 0; row < (size_t)n * n; row++) {
    for (int i = 0; i < n; i++) data[row * pitch + i] = (float)out[row * n + i];
    data[row * pitch + n] = 0;
    data[row * pitch + n + 1] = 0;
  }
  free(out);
}

void orc_normalize(int n, double l_box, float *data)
{
  long tot = 2 * (long)(n / 2 + 1) * n * n;
  double norm = pow(sqrt(2 * M_PI) / l_box, 3);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < tot; i++) data[i] *= norm;
}
