/*
 * Reader of SW2 case files (`<case>.sw`), for running the reference's own
 * cases on the GPU step. It restates what the reference's `initialize()`
 * reads (init.c:48-237), in the same order, through the same layers:
 *   1. a subset of the m4 preprocessor the reference shells out to
 *      (sppde/sppde_parser.c:177-210): define(NAME,VALUE), include(FILE),
 *      macro replacement with rescanning, '#' comments copied verbatim;
 *   2. line cleaning and '<expression>' evaluation (sppde_parser.c:64-157):
 *      comments cut at '#', empty lines skipped, each <...> replaced by its
 *      value printed with "%.15e" ('\<' and '\>' are literal);
 *   3. tagged values and tables (sppde_parser.c:160-320).
 * Reference-field comparison (reftype 1) is read but not run.
 */
#ifndef SWCASE_H
#define SWCASE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWC_GAUSS_COLS 12   /* N_COLS_GAUSS (sw.h) */
#define SWC_VORTEX_COLS 7   /* N_COLS_VORTICES (sw.h) */

typedef struct {
  int sch, polar;
  /* band limits in radians, as the sw struct holds them (init.c:56-59) */
  double lon0, lon1, lat0, lat1;
  int nx, ny;
  double t0, t1, Dt, CFL;
  int N;                  /* (int)((t1 - t0) / Dt), init.c:107 */
  double tau;             /* Tau as entered */
  double sigma_dis;       /* 0 if Tau > 1e10, else 1/Tau (init.c:108-113) */
  double nu2, nu4, nu6;   /* as entered (positive); the reference stores -nu4 */
  int IteInfo, saveEvery, loadFrom;
  int reftype;
  double Omega, rE, rP, gE, depth;
  double epsilon2;        /* (rE/rP)^2 */
  int geoeq;
  int num_vortices;
  double *vortices;       /* num_vortices x 7, rows contiguous */
  int num_gaussians;
  double *gaussians;      /* num_gaussians x 12, rows contiguous */
  double tracer_dis;
  int wind_rows;
  double *wind;           /* wind_rows latitudes (deg), then wind_rows values (transposed table) */
  double beta_sponge;     /* BetaSp as entered (degrees), polar caps only */
  double sigma_sponge;    /* SigSp, polar caps only */
} swcase;

/* Reads `path` (the .sw file; includes are resolved against its directory).
 * Returns 0 on success; otherwise nonzero with a message in err. */
int swcase_read(const char *path, swcase *c, char *err, size_t errlen);
void swcase_free(swcase *c);

/* The m4 subset alone: expands `path` into a malloc'ed string (NULL on error). */
char *swcase_m4(const char *path, char *err, size_t errlen);

/* Evaluates one '<...>' expression (the grammar of the reference's tinyexpr:
 * + - * / % ^ (left-associative), unary signs, parentheses, numbers, pi, e
 * and the functions abs acos asin atan atan2 ceil cos cosh exp fac floor ln
 * log (base 10) log10 ncr npr pow sin sinh sqrt tan tanh). Returns 0 on
 * success. */
int swcase_eval(const char *expr, double *value);

#ifdef __cplusplus
}
#endif
#endif
