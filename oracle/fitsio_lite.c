/*
 * fitsio_lite.c -- a small FITS binary-table reader behind the cfitsio calls
 * declared in oracle/shim/fitsio.h.
 *
 * TEST INFRASTRUCTURE ONLY.  This file belongs to the oracle (the CPU checker
 * of the GPU path); the product never links it.  It implements what the
 * relxill table loaders need (reltable.c:121-448, xilltable.c:169-276,
 * 513-564): moving between HDUs by number or EXTNAME, looking up columns by
 * name, counting rows and reading E/D/J/I/A columns with cfitsio's
 * element-wise addressing (firstrow, firstelem, nelem running across rows).
 * Semantics follow the cfitsio reference manual for these routines; numeric
 * conversions are plain C casts, as cfitsio does for unscaled columns.
 */
#define _FILE_OFFSET_BITS 64
#define _POSIX_C_SOURCE 200809L
#include "shim/fitsio.h"

#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define BLOCK 2880
#define MAXCOL 1024
#define MAXHDU 4096

typedef struct {
  long long hdr_off;   /* byte offset of the header */
  long long data_off;  /* byte offset of the data */
  int is_table;
  long long width;     /* NAXIS1 */
  long long nrows;     /* NAXIS2 */
  int ncol;
  char extname[72];
  char (*ttype)[72];
  char *code;          /* E, D, J, I, A, B, K */
  long long *repeat;
  long long *coloff;
} hdu_t;

struct fitsfile {
  FILE *fp;
  int nhdu;
  int cur;             /* 0-based current HDU */
  hdu_t *hdu;
};

static int elem_size(char c) {
  switch (c) {
    case 'E': case 'J': return 4;
    case 'D': case 'K': return 8;
    case 'I': return 2;
    case 'A': case 'B': case 'L': return 1;
    default: return 0;
  }
}

static void trim(char *s) {
  size_t n = strlen(s);
  while (n > 0 && (s[n - 1] == ' ' || s[n - 1] == '\'')) s[--n] = 0;
  char *p = s;
  while (*p == ' ' || *p == '\'') p++;
  if (p != s) memmove(s, p, strlen(p) + 1);
}

static void card_value(const char *card, char *out) {
  /* value part of an 80-char card (after "= "), string quotes removed */
  char buf[81];
  memcpy(buf, card + 10, 70);
  buf[70] = 0;
  char *p = buf;
  while (*p == ' ') p++;
  if (*p == '\'') {
    p++;
    char *q = out;
    while (*p) {
      if (*p == '\'') {
        if (p[1] == '\'') { *q++ = '\''; p += 2; continue; }
        break;
      }
      *q++ = *p++;
    }
    *q = 0;
    size_t n = strlen(out);
    while (n > 0 && out[n - 1] == ' ') out[--n] = 0;
  } else {
    char *slash = strchr(p, '/');
    if (slash) *slash = 0;
    strcpy(out, p);
    trim(out);
  }
}

static int scan_file(fitsfile *f) {
  long long pos = 0;
  f->hdu = (hdu_t *) calloc(MAXHDU, sizeof(hdu_t));
  f->nhdu = 0;
  char block[BLOCK];
  while (f->nhdu < MAXHDU) {
    if (fseeko(f->fp, pos, SEEK_SET) != 0) break;
    hdu_t *h = &f->hdu[f->nhdu];
    memset(h, 0, sizeof(*h));
    h->hdr_off = pos;
    long long naxis = 0, naxis1 = 0, naxis2 = 0, pcount = 0, tfields = 0;
    int xt_bintable = 0, ended = 0;
    long long nbytes = 0;
    char (*ttype)[72] = NULL;
    char (*tform)[72] = NULL;
    while (!ended) {
      if (fread(block, 1, BLOCK, f->fp) != BLOCK) return f->nhdu > 0 ? 0 : 104;
      nbytes += BLOCK;
      for (int i = 0; i < BLOCK; i += 80) {
        const char *card = block + i;
        char key[9];
        memcpy(key, card, 8);
        key[8] = 0;
        trim(key);
        if (strcmp(key, "END") == 0) { ended = 1; break; }
        if (card[8] != '=') continue;
        char val[81];
        card_value(card, val);
        if (strcmp(key, "XTENSION") == 0) xt_bintable = (strcmp(val, "BINTABLE") == 0);
        else if (strcmp(key, "NAXIS") == 0) naxis = atoll(val);
        else if (strcmp(key, "NAXIS1") == 0) naxis1 = atoll(val);
        else if (strcmp(key, "NAXIS2") == 0) naxis2 = atoll(val);
        else if (strcmp(key, "PCOUNT") == 0) pcount = atoll(val);
        else if (strcmp(key, "TFIELDS") == 0) {
          tfields = atoll(val);
          if (tfields > MAXCOL) return 104;
          ttype = calloc(tfields + 1, sizeof(*ttype));
          tform = calloc(tfields + 1, sizeof(*tform));
        } else if (strcmp(key, "EXTNAME") == 0) {
          strncpy(h->extname, val, 71);
        } else if (strncmp(key, "TTYPE", 5) == 0 && ttype) {
          int k = atoi(key + 5);
          if (k >= 1 && k <= tfields) strncpy(ttype[k], val, 71);
        } else if (strncmp(key, "TFORM", 5) == 0 && tform) {
          int k = atoi(key + 5);
          if (k >= 1 && k <= tfields) strncpy(tform[k], val, 71);
        }
      }
    }
    h->data_off = pos + nbytes;
    long long datasize = 0;
    if (xt_bintable && naxis == 2) {
      h->is_table = 1;
      h->width = naxis1;
      h->nrows = naxis2;
      h->ncol = (int) tfields;
      h->ttype = calloc(tfields + 1, sizeof(*h->ttype));
      h->code = calloc(tfields + 1, 1);
      h->repeat = calloc(tfields + 1, sizeof(long long));
      h->coloff = calloc(tfields + 1, sizeof(long long));
      long long off = 0;
      for (int k = 1; k <= tfields; k++) {
        strcpy(h->ttype[k], ttype[k]);
        const char *tf = tform[k];
        long long rep = 1;
        int j = 0;
        if (isdigit((unsigned char) tf[0])) {
          rep = atoll(tf);
          while (isdigit((unsigned char) tf[j])) j++;
        }
        h->code[k] = tf[j];
        h->repeat[k] = rep;
        h->coloff[k] = off;
        off += rep * elem_size(tf[j]);
      }
      datasize = naxis1 * naxis2 + pcount;
    }
    free(ttype);
    free(tform);
    f->nhdu++;
    pos = h->data_off + ((datasize + BLOCK - 1) / BLOCK) * BLOCK;
  }
  return 0;
}

int fits_open_file(fitsfile **fptr, const char *filename, int mode, int *status) {
  if (*status) return *status;
  (void) mode;
  FILE *fp = fopen(filename, "rb");
  if (!fp) { *fptr = NULL; return *status = 104; }
  fitsfile *f = (fitsfile *) calloc(1, sizeof(fitsfile));
  f->fp = fp;
  int st = scan_file(f);
  if (st) { fclose(fp); free(f); *fptr = NULL; return *status = st; }
  f->cur = 0;
  *fptr = f;
  return 0;
}

int fits_open_table(fitsfile **fptr, const char *filename, int mode, int *status) {
  if (fits_open_file(fptr, filename, mode, status)) return *status;
  fitsfile *f = *fptr;
  for (int i = 0; i < f->nhdu; i++) {
    if (f->hdu[i].is_table) { f->cur = i; return 0; }
  }
  return *status = 235;
}

int fits_close_file(fitsfile *f, int *status) {
  if (!f) return *status;
  fclose(f->fp);
  for (int i = 0; i < f->nhdu; i++) {
    free(f->hdu[i].ttype);
    free(f->hdu[i].code);
    free(f->hdu[i].repeat);
    free(f->hdu[i].coloff);
  }
  free(f->hdu);
  free(f);
  return *status;
}

static int streq_ci(const char *a, const char *b) {
  while (*a && *b) {
    if (tolower((unsigned char) *a) != tolower((unsigned char) *b)) return 0;
    a++;
    b++;
  }
  return *a == 0 && *b == 0;
}

int fits_movnam_hdu(fitsfile *f, int hdutype, const char *extname, int extver, int *status) {
  if (*status) return *status;
  (void) hdutype;
  (void) extver;
  for (int i = 0; i < f->nhdu; i++) {
    if (streq_ci(f->hdu[i].extname, extname)) { f->cur = i; return 0; }
  }
  return *status = 301;  /* BAD_HDU_NUM */
}

int fits_movabs_hdu(fitsfile *f, int hdunum, int *exttype, int *status) {
  if (*status) return *status;
  if (hdunum < 1 || hdunum > f->nhdu) return *status = 107;
  f->cur = hdunum - 1;
  if (exttype) *exttype = f->hdu[f->cur].is_table ? BINARY_TBL : IMAGE_HDU;
  return 0;
}

int fits_get_colnum(fitsfile *f, int casesen, const char *templt, int *colnum, int *status) {
  if (*status) return *status;
  hdu_t *h = &f->hdu[f->cur];
  for (int k = 1; k <= h->ncol; k++) {
    int eq = casesen ? (strcmp(h->ttype[k], templt) == 0) : streq_ci(h->ttype[k], templt);
    if (eq) { *colnum = k; return 0; }
  }
  return *status = 219;  /* COL_NOT_FOUND */
}

int fits_get_num_rows(fitsfile *f, long *nrows, int *status) {
  if (*status) return *status;
  *nrows = (long) f->hdu[f->cur].nrows;
  return 0;
}

static double get_be(const unsigned char *p, char code) {
  switch (code) {
    case 'E': {
      uint32_t u = ((uint32_t) p[0] << 24) | ((uint32_t) p[1] << 16) | ((uint32_t) p[2] << 8) | p[3];
      float v;
      memcpy(&v, &u, 4);
      return v;
    }
    case 'D': {
      uint64_t u = 0;
      for (int i = 0; i < 8; i++) u = (u << 8) | p[i];
      double v;
      memcpy(&v, &u, 8);
      return v;
    }
    case 'J': {
      uint32_t u = ((uint32_t) p[0] << 24) | ((uint32_t) p[1] << 16) | ((uint32_t) p[2] << 8) | p[3];
      return (double) (int32_t) u;
    }
    case 'K': {
      uint64_t u = 0;
      for (int i = 0; i < 8; i++) u = (u << 8) | p[i];
      return (double) (int64_t) u;
    }
    case 'I': {
      uint16_t u = (uint16_t) (((uint16_t) p[0] << 8) | p[1]);
      return (double) (int16_t) u;
    }
    case 'B': return (double) p[0];
    default: return 0.0;
  }
}

static float get_be_float(const unsigned char *p) {
  uint32_t u = ((uint32_t) p[0] << 24) | ((uint32_t) p[1] << 16) | ((uint32_t) p[2] << 8) | p[3];
  float v;
  memcpy(&v, &u, 4);
  return v;
}

int fits_read_col(fitsfile *f, int datatype, int colnum, LONGLONG firstrow, LONGLONG firstelem,
                  LONGLONG nelem, void *nulval, void *array, int *anynul, int *status) {
  if (*status) return *status;
  (void) nulval;
  if (anynul) *anynul = 0;
  hdu_t *h = &f->hdu[f->cur];
  if (!h->is_table || colnum < 1 || colnum > h->ncol) return *status = 302;
  char code = h->code[colnum];
  long long rep = h->repeat[colnum];
  int esz = elem_size(code);
  if (datatype == TSTRING) {
    /* one string of 'rep' characters per row */
    char **out = (char **) array;
    unsigned char *buf = malloc(rep + 1);
    for (LONGLONG i = 0; i < nelem; i++) {
      long long row = firstrow - 1 + i;
      if (row >= h->nrows) { free(buf); return *status = 307; }
      fseeko(f->fp, h->data_off + row * h->width + h->coloff[colnum], SEEK_SET);
      if ((long long) fread(buf, 1, rep, f->fp) != rep) { free(buf); return *status = 108; }
      buf[rep] = 0;
      size_t n = strlen((char *) buf);
      while (n > 0 && buf[n - 1] == ' ') buf[--n] = 0;
      strcpy(out[i], (char *) buf);
    }
    free(buf);
    return 0;
  }
  /* numeric: element index e (0-based) runs across rows */
  long long e = (firstrow - 1) * rep + (firstelem - 1);
  long long done = 0;
  unsigned char *buf = malloc(rep * esz);
  while (done < nelem) {
    long long row = e / rep;
    long long el = e % rep;
    if (row >= h->nrows) { free(buf); return *status = 307; }
    long long take = rep - el;
    if (take > nelem - done) take = nelem - done;
    fseeko(f->fp, h->data_off + row * h->width + h->coloff[colnum] + el * esz, SEEK_SET);
    if ((long long) fread(buf, esz, take, f->fp) != take) { free(buf); return *status = 108; }
    for (long long i = 0; i < take; i++) {
      const unsigned char *p = buf + i * esz;
      long long o = done + i;
      switch (datatype) {
        case TFLOAT:
          ((float *) array)[o] = (code == 'E') ? get_be_float(p) : (float) get_be(p, code);
          break;
        case TDOUBLE: ((double *) array)[o] = get_be(p, code); break;
        case TINT: ((int *) array)[o] = (int) get_be(p, code); break;
        case TLONG: ((long *) array)[o] = (long) get_be(p, code); break;
        case TSHORT: ((short *) array)[o] = (short) get_be(p, code); break;
        default: free(buf); return *status = 410;
      }
    }
    done += take;
    e += take;
  }
  free(buf);
  return 0;
}

void fits_get_errstatus(int status, char *err_text) {
  snprintf(err_text, FLEN_STATUS, "fitsio_lite status %d", status);
}

int fits_create_file(fitsfile **fptr, const char *filename, int *status) {
  (void) filename;
  *fptr = NULL;
  return *status = 105;
}

int fits_create_tbl(fitsfile *fptr, int tbltype, LONGLONG naxis2, int tfields, char **ttype, char **tform,
                    char **tunit, const char *extname, int *status) {
  (void) fptr; (void) tbltype; (void) naxis2; (void) tfields; (void) ttype; (void) tform; (void) tunit;
  (void) extname;
  return *status = 105;
}

int fits_write_col(fitsfile *fptr, int datatype, int colnum, LONGLONG firstrow, LONGLONG firstelem,
                   LONGLONG nelem, void *array, int *status) {
  (void) fptr; (void) datatype; (void) colnum; (void) firstrow; (void) firstelem; (void) nelem; (void) array;
  return *status = 105;
}

int fits_write_key(fitsfile *fptr, int datatype, const char *keyname, void *value, const char *comment,
                   int *status) {
  (void) fptr; (void) datatype; (void) keyname; (void) value; (void) comment;
  return *status = 105;
}
