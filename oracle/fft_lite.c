/*
 * fft_lite.c -- double-precision real FFTs behind the FFTW 3 calls declared
 * in oracle/shim/fftw3.h.
 *
 * TEST INFRASTRUCTURE ONLY (part of the oracle; the product never links it).
 * FFTW itself is not available here.  The relxill reference uses it only for
 * the convolution of Relbase.cpp:119-188 (one r2c per input, a complex
 * product, one c2r), always with n = N_ENER_CONV = 4096.  This file restates
 * the published algorithm: an iterative radix-2 Cooley-Tukey transform with
 * directly evaluated twiddles, wrapped with FFTW's conventions:
 *   r2c: out[k] = sum_j in[j] exp(-2 pi i j k / n), k = 0..n/2, with the
 *        imaginary parts of out[0] and out[n/2] set to exactly zero;
 *   c2r: out[j] = sum_k X[k] exp(+2 pi i j k / n) over the Hermitian
 *        extension of in[0..n/2] (imaginary parts of in[0], in[n/2] ignored),
 *        unnormalised (a c2r after an r2c multiplies by n).
 * Results agree with FFTW to rounding (~1e-15 relative to the largest term).
 */
#include "shim/fftw3.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct fftw_plan_s {
  int n;
  int kind;  /* 0 = r2c, 1 = c2r */
  double *rin;
  fftw_complex *cin;
  double *rout;
  fftw_complex *cout;
};

static void fft_inplace(double *re, double *im, int n, int sign) {
  /* bit reversal */
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1;
    for (int k = 0; k < half; k++) {
      double ang = sign * 2.0 * M_PI * (double) k / (double) len;
      double wr = cos(ang), wi = sin(ang);
      for (int s = 0; s < n; s += len) {
        int a = s + k, b = s + k + half;
        double xr = re[b] * wr - im[b] * wi;
        double xi = re[b] * wi + im[b] * wr;
        re[b] = re[a] - xr;
        im[b] = im[a] - xi;
        re[a] += xr;
        im[a] += xi;
      }
    }
  }
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* plain O(n^2) DFT for lengths that are not powers of two (not used by relxill) */
static void dft(const double *re, const double *im, double *ore, double *oim, int n, int sign) {
  for (int k = 0; k < n; k++) {
    double sr = 0, si = 0;
    for (int j = 0; j < n; j++) {
      double ang = sign * 2.0 * M_PI * (double) ((long long) j * k % n) / (double) n;
      sr += re[j] * cos(ang) - im[j] * sin(ang);
      si += re[j] * sin(ang) + im[j] * cos(ang);
    }
    ore[k] = sr;
    oim[k] = si;
  }
}

static void transform(double *re, double *im, int n, int sign) {
  if (is_pow2(n)) {
    fft_inplace(re, im, n, sign);
  } else {
    double *r2 = malloc(sizeof(double) * n), *i2 = malloc(sizeof(double) * n);
    dft(re, im, r2, i2, n, sign);
    memcpy(re, r2, sizeof(double) * n);
    memcpy(im, i2, sizeof(double) * n);
    free(r2);
    free(i2);
  }
}

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags) {
  (void) flags;
  fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
  p->n = n;
  p->kind = 0;
  p->rin = in;
  p->cout = out;
  return p;
}

fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags) {
  (void) flags;
  fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
  p->n = n;
  p->kind = 1;
  p->cin = in;
  p->rout = out;
  return p;
}

void fftw_execute(const fftw_plan p) {
  int n = p->n;
  double *re = malloc(sizeof(double) * n), *im = malloc(sizeof(double) * n);
  if (p->kind == 0) {
    for (int j = 0; j < n; j++) { re[j] = p->rin[j]; im[j] = 0.0; }
    transform(re, im, n, -1);
    for (int k = 0; k <= n / 2; k++) {
      p->cout[k][0] = re[k];
      p->cout[k][1] = im[k];
    }
    p->cout[0][1] = 0.0;
    if (n % 2 == 0) p->cout[n / 2][1] = 0.0;
  } else {
    for (int k = 0; k <= n / 2; k++) {
      re[k] = p->cin[k][0];
      im[k] = p->cin[k][1];
    }
    im[0] = 0.0;
    if (n % 2 == 0) im[n / 2] = 0.0;
    for (int k = n / 2 + 1; k < n; k++) {
      re[k] = p->cin[n - k][0];
      im[k] = -p->cin[n - k][1];
    }
    transform(re, im, n, +1);
    for (int j = 0; j < n; j++) p->rout[j] = re[j];
  }
  free(re);
  free(im);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

/* The reference hands memory from new[] to fftw_free (Relbase.cpp:52 vs :668);
 * releasing it here would be undefined behaviour, so this is a no-op. */
void fftw_free(void *p) { (void) p; }
