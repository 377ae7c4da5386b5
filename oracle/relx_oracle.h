/*
 * relx_oracle.h -- C restatement of relxill's relativistic convolution path
 * (double precision).  TEST INFRASTRUCTURE ONLY: the checker for the GPU
 * path; the product never links it.
 */
#ifndef RELX_ORACLE_H
#define RELX_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { RELXO_RELLINE = 0, RELXO_RELCONV = 1, RELXO_RELXILL = 2, RELXO_RELXILLLP = 3, RELXO_RELLINELP = 4,
       RELXO_RELCONVLP = 5, RELXO_XILLVER = 6, RELXO_XILLVERCP = 7, RELXO_RELXILLCP = 8, RELXO_RELXILLLPCP = 9 };

int relxo_set_table_path(const char *path);
/* one model evaluation; params in lmodel.dat order; returns 0 on success */
int relxo_eval(int model, const double *params, const double *energy, int n_flux, double *flux);
/* relxilllp with the hidden ionisation-gradient switch (0 const, 1 PL, 2 ALPHA) */
int relxo_eval_ext(int model, const double *params, int ion_grad_type, double iongrad_index, const double *energy,
                   int n_flux, double *flux);

/* components, for pinning against the reference's known-answer tests */
double relxo_interp_lin_1d(double f, double lo, double hi);
double relxo_interp_lin_2d(double f1, double f2, double r11, double r12, double r21, double r22);
double relxo_interp_lin_2d_float(double f1, double f2, float r11, float r12, float r21, float r22);
void relxo_rebin_spectrum(const double *ener, double *flu, int nbins, const double *ener0, const double *flu0,
                          int nbins0);
double relxo_kerr_rms(double a);
double relxo_gi_potential_lp(double r, double a, double h, double bet, double del);
double relxo_norm_wrt_xillver(const double *flux, const double *ener, int n);
double relxo_primary_norm_factor(double ect, double gam);
double relxo_norm_change(double energy_shift, double ect, double gam);
void relxo_conv_spectrum_normalized(const double *ener, const double *fxill, const double *frel, double *fout, int n);
void relxo_conv_grid(double *out);
/* nthcomp photon spectrum per bin (kTbb 0.05 keV, disk-blackbody seed) on ear[0..ne] */
void relxo_nthcomp(const double *ear, int ne, double gamma, double kte, double z, double *photar);
int relxo_relline_profile_zones(int model, const double *params, const double *ener, int n_ener, int *nzones_out,
                                double *flux, int n_incl, double *dist);
/* integrand evaluations (relb_func, one branch each) since the last reset; reset != 0 resets */
long long relxo_relb_calls(int reset);

#ifdef __cplusplus
}
#endif
#endif
