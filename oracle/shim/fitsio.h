/*
 * fitsio.h -- stand-in for the subset of the cfitsio API that the relxill
 * reference code calls (reltable.c, xilltable.c, Relreturn_Table.cpp,
 * Relreturn_BlackBody.cpp, relutility.c).  Only reading of BINTABLE
 * extensions with E/D/J/I/A columns is implemented (oracle/fitsio_lite.c);
 * the write calls return an error status.  Test infrastructure only: it lets
 * the unmodified reference sources and the oracle read the synthetic tables.
 */
#ifndef RELX_ORACLE_FITSIO_LITE_H
#define RELX_ORACLE_FITSIO_LITE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef long long LONGLONG;
typedef struct fitsfile fitsfile;

#define READONLY 0
#define READWRITE 1
#define IMAGE_HDU 0
#define ASCII_TBL 1
#define BINARY_TBL 2
#define ANY_HDU -1
#define CASESEN 1
#define CASEINSEN 0
#define TBYTE 11
#define TSTRING 16
#define TSHORT 21
#define TINT 31
#define TLONG 41
#define TFLOAT 42
#define TLONGLONG 81
#define TDOUBLE 82
#define FLEN_STATUS 31
#define FLEN_ERRMSG 81

int fits_open_table(fitsfile **fptr, const char *filename, int mode, int *status);
int fits_open_file(fitsfile **fptr, const char *filename, int mode, int *status);
int fits_close_file(fitsfile *fptr, int *status);
int fits_movnam_hdu(fitsfile *fptr, int hdutype, const char *extname, int extver, int *status);
int fits_movabs_hdu(fitsfile *fptr, int hdunum, int *exttype, int *status);
int fits_get_colnum(fitsfile *fptr, int casesen, const char *templt, int *colnum, int *status);
int fits_get_num_rows(fitsfile *fptr, long *nrows, int *status);
int fits_read_col(fitsfile *fptr, int datatype, int colnum, LONGLONG firstrow, LONGLONG firstelem,
                  LONGLONG nelem, void *nulval, void *array, int *anynul, int *status);
void fits_get_errstatus(int status, char *err_text);

/* write side: not implemented (only used by debug output of out-of-scope models) */
int fits_create_file(fitsfile **fptr, const char *filename, int *status);
int fits_create_tbl(fitsfile *fptr, int tbltype, LONGLONG naxis2, int tfields, char **ttype, char **tform,
                    char **tunit, const char *extname, int *status);
int fits_write_col(fitsfile *fptr, int datatype, int colnum, LONGLONG firstrow, LONGLONG firstelem,
                   LONGLONG nelem, void *array, int *status);
int fits_write_key(fitsfile *fptr, int datatype, const char *keyname, void *value, const char *comment,
                   int *status);

#ifdef __cplusplus
}
#endif
#endif
