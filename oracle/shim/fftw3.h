/*
 * fftw3.h -- stand-in for the subset of FFTW 3 (double precision) that the
 * relxill reference calls (Relbase.cpp:55,153-167,182,638-670): real-to-
 * complex and complex-to-real transforms of one dimension with FFTW's
 * conventions (forward sign -1, unnormalised inverse, n/2+1 complex outputs).
 * The transform is a plain mixed radix-2 Cooley-Tukey FFT in double
 * precision (oracle/fft_lite.c).  Test infrastructure only.
 */
#ifndef RELX_ORACLE_FFTW_LITE_H
#define RELX_ORACLE_FFTW_LITE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE 0U

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void fftw_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
