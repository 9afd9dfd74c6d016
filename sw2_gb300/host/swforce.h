/*
 * Time-dependent forcing of SW2 cases, restated on the host: the Gaussian
 * mass injections (add_Gaussians, add_Gaussian_core, get_Gaussian_field,
 * perturbs.c:22-364) and the vortices in geostrophic balance (add_vortices,
 * add_vortex_core, perturbs.c:366-477). Everything that decides a value is
 * computed here with the reference's expressions in its operation order
 * (compiled with -ffp-contract=off, the host libm), so the fields handed to
 * the GPU step are the reference's bit for bit; the step applies them with
 * the same arithmetic (field += scale * delta).
 * Polar 0 geometry only.
 */
#ifndef SWFORCE_H
#define SWFORCE_H

#include "swcase.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Padded fields ((nx+4)*(ny+4), x fastest) the forcing of one step produces. */
typedef struct {
  int nx, ny;
  double *pert;        /* Gaussian field of one injection (perturb_field) */
  double *tracer;      /* tracer values set inside the injection radius */
  unsigned char *mask; /* cells inside the radius (where TRACER and PERTURBS are set) */
  double *perturbs;    /* the reference's PERTURBS field (1 inside any radius this step) */
  double *deta, *du, *dv;  /* one vortex: increments of eta, u, v */
  /* The cells inside the radius of the last injection: ncells padded
   * indices, increasing, with their Gaussian (cell_pert) and tracer
   * (cell_tracer) values, the same numbers as pert/tracer hold there. */
  int *cells;
  int ncells;
  double *cell_pert, *cell_tracer;
  /* per-case tables, filled on first use: planetocentric latitude of row j
   * and its sine and cosine, area element DXC*DYC of row j, longitude of
   * column i (index j or i, 0..n+1) */
  double *row_pl, *row_sin, *row_cos, *row_surf, *col_lonc;
  int tables_ready;
} swforce;

int swforce_init(swforce *w, int nx, int ny);
void swforce_free(swforce *w);

/* Geometry of the case (sw.h:108-193 macros on the case's planet). */
double swf_lone(const swcase *c, int i);
double swf_lonc(const swcase *c, int i);
double swf_latn(const swcase *c, int j);
double swf_latc(const swcase *c, int j);
double swf_rZ(const swcase *c, double lat);
double swf_rM(const swcase *c, double lat);
double swf_lat2pclat(const swcase *c, double lat);
double swf_g_eff(const swcase *c, double pclat);
double swf_DXC(const swcase *c, int j);
double swf_DYC(const swcase *c, int j);

/* The per-step scalars of Gaussian row g at time t (add_Gaussians and the
 * start of add_Gaussian_core, perturbs.c:56-258): the centre moved and
 * wrapped into [lon0, lon1], sigma and radius in metres, the ramped volume
 * Dt*Q(t), the peak before rescaling, and which periodic images the field
 * needs (bit 0: lon - (lon1 - lon0), bit 1: lon + (lon1 - lon0)). Returns 0,
 * 1 if the row is not active at t, or -1 on an error of the case. */
typedef struct {
  double lon, lat, amp, sigma, radius, inject, volume;
  int images;
} swf_gplan;
int swforce_gaussian_plan(const swcase *c, int g, double Dt, double t, swf_gplan *p, char *err, size_t errlen);

/* One Gaussian injection that is active at time t (t0 <= t <= t1 of row g):
 * fills w->pert (zeroed first), sets w->tracer/w->mask for the cells inside
 * the radius (mask zeroed first), sets w->perturbs to 1 there, lists those
 * cells in w->cells/cell_pert/cell_tracer, and returns in *scale the rescale
 * factor volume/V (perturbs.c:303-309), or 0 when the volume is below the
 * reference's 1e-7 threshold (no eta change). Only cells that can lie inside
 * the radius are evaluated (see swforce.c); the others keep zero, as the
 * reference's evaluation of them gives.
 * Returns 0, 1 if row g is not active at t, or -1 on an error of the case
 * (message in err). */
int swforce_gaussian(const swcase *c, int g, double Dt, double t, swforce *w, double *scale, char *err,
                     size_t errlen);

/* Whether vortex row k starts in the step ending at t (perturbs.c:388). */
int swforce_vortex_due(const swcase *c, int k, double Dt, double t);
/* Increments of eta, u, v of vortex row k (add_vortex_core) into w->deta/du/dv. */
void swforce_vortex(const swcase *c, int k, swforce *w);

/* windx over all padded cells by linear interpolation of the wind table at
 * latc(j) (io.c:199-206), followed by the single-rank halo wrap
 * (init.c:232-235). Returns -1 if the table does not cover the rows. */
int swforce_windx(const swcase *c, double *windx, char *err, size_t errlen);

/* windx and windy of the case over all padded cells as read_wind leaves them:
 * the band's zonal wind (swforce_windx, windy zero), or a polar cap's wind
 * turned around the pole and damped beyond the sponge (io.c:207-240);
 * beta_sponge_deg is the case's BetaSp in degrees (c->beta_sponge). */
int swforce_winds(const swcase *c, double beta_sponge_deg, double *windx, double *windy, char *err,
                  size_t errlen);

/* Single-rank halo update of a padded field (sppde_hupdate.c:274-342). */
void swf_halo_wrap(double *x, int nx, int ny);

#ifdef __cplusplus
}
#endif
#endif
