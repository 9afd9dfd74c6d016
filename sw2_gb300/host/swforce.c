/*
 * Host restatement of the reference's time-dependent forcing; see swforce.h.
 * Compiled with -ffp-contract=off: every expression keeps the operand order
 * of the reference expression named beside it.
 */
#include "swforce.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static double PI_(void) { return 4.0 * atan(1.0); }                       /* sw.h:16 */
static double deg2rad(double a) { return a * (PI_() / 180.0); }          /* sw.h:108 */
static double rad2deg(double b) { return b * (180.0 / PI_()); }          /* sw.h:109 */
static double sq(double a) { return a * a; }                             /* POW2, sw.h:105 */
static double linspace(int i, double x0, double x1, int n) {             /* tools.c:256-273 */
  return x0 + (double)i * (x1 - x0) / ((double)n);
}

static void set_err(char *err, size_t errlen, const char *fmt, ...) {
  if (!err || !errlen) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, errlen, fmt, ap);
  va_end(ap);
}

double swf_lone(const swcase *c, int i) { return linspace(i, c->lon0, c->lon1, c->nx); }           /* sw.h:113 */
double swf_lonc(const swcase *c, int i) { return (swf_lone(c, i) + swf_lone(c, i - 1)) / 2.; }     /* sw.h:114 */
double swf_latn(const swcase *c, int j) { return linspace(j, c->lat0, c->lat1, c->ny); }           /* sw.h:116 */
double swf_latc(const swcase *c, int j) { return (swf_latn(c, j) + swf_latn(c, j - 1)) / 2.; }     /* sw.h:117 */
double swf_rZ(const swcase *c, double lat) {                                                        /* sw.h:174 */
  return c->rE / sqrt(1.0 + sq(tan(lat)) / c->epsilon2);
}
double swf_rM(const swcase *c, double lat) {                                                        /* sw.h:175 */
  const double q = swf_rZ(c, lat) / (c->rE * cos(lat));
  return c->rE / c->epsilon2 * (q * q * q);
}
double swf_lat2pclat(const swcase *c, double lat) { return atan(1.0 / c->epsilon2 * tan(lat)); }   /* sw.h:170 */
static double r_pc(const swcase *c, double pc) {                                                    /* sw.h:172 */
  return c->rE * c->rP / sqrt(sq(c->rE * sin(pc)) + sq(c->rP * cos(pc)));
}
double swf_g_eff(const swcase *c, double pc) {                                                      /* sw.h:178-179 */
  const double g0 = (c->gE + sq(c->Omega) * c->rE) * sq(c->rE / r_pc(c, pc));
  return g0 - sq(c->Omega) * r_pc(c, pc) * cos(pc);
}
static double fcor(const swcase *c, double lat) { return 2.0 * c->Omega * sin(lat); }              /* sw.h:193 */
double swf_DXC(const swcase *c, int j) {                                                            /* coords.c:60-65 */
  return ((c->lon1 - c->lon0) / ((double)c->nx)) * swf_rZ(c, swf_latc(c, j));
}
double swf_DYC(const swcase *c, int j) {
  return ((c->lat1 - c->lat0) / ((double)c->ny)) * swf_rM(c, swf_latn(c, j - 1));
}

static size_t IXP(int nx, int i, int j) { return (size_t)(i + 1) + (size_t)(j + 1) * (size_t)(nx + 4); }

int swforce_init(swforce *w, int nx, int ny) {
  memset(w, 0, sizeof *w);
  w->nx = nx;
  w->ny = ny;
  const size_t S = (size_t)(nx + 4) * (ny + 4);
  w->pert = (double *)calloc(S, sizeof(double));
  w->tracer = (double *)calloc(S, sizeof(double));
  w->mask = (unsigned char *)calloc(S, 1);
  w->perturbs = (double *)calloc(S, sizeof(double));
  w->deta = (double *)calloc(S, sizeof(double));
  w->du = (double *)calloc(S, sizeof(double));
  w->dv = (double *)calloc(S, sizeof(double));
  const size_t N = (size_t)nx * ny;
  w->cells = (int *)calloc(N, sizeof(int));
  w->cell_pert = (double *)calloc(N, sizeof(double));
  w->cell_tracer = (double *)calloc(N, sizeof(double));
  w->row_pl = (double *)calloc((size_t)ny + 2, sizeof(double));
  w->row_sin = (double *)calloc((size_t)ny + 2, sizeof(double));
  w->row_cos = (double *)calloc((size_t)ny + 2, sizeof(double));
  w->row_surf = (double *)calloc((size_t)ny + 2, sizeof(double));
  w->col_lonc = (double *)calloc((size_t)nx + 2, sizeof(double));
  if (!w->pert || !w->tracer || !w->mask || !w->perturbs || !w->deta || !w->du || !w->dv || !w->cells ||
      !w->cell_pert || !w->cell_tracer || !w->row_pl || !w->row_sin || !w->row_cos || !w->row_surf ||
      !w->col_lonc) {
    swforce_free(w);
    return -1;
  }
  return 0;
}

void swforce_free(swforce *w) {
  free(w->pert);
  free(w->tracer);
  free(w->mask);
  free(w->perturbs);
  free(w->deta);
  free(w->du);
  free(w->dv);
  free(w->cells);
  free(w->cell_pert);
  free(w->cell_tracer);
  free(w->row_pl);
  free(w->row_sin);
  free(w->row_cos);
  free(w->row_surf);
  free(w->col_lonc);
  memset(w, 0, sizeof *w);
}

/* Per-case tables of the values the Gaussian loops use per row and column:
 * the same functions of the same arguments as the reference evaluates per
 * cell, so the cached numbers are its numbers. */
static void tables(const swcase *c, swforce *w) {
  if (w->tables_ready) return;
  for (int j = 1; j <= c->ny; j++) {
    const double pl = swf_lat2pclat(c, swf_latc(c, j));
    w->row_pl[j] = pl;
    w->row_sin[j] = sin(pl);
    w->row_cos[j] = cos(pl);
    w->row_surf[j] = swf_DXC(c, j) * swf_DYC(c, j);
  }
  for (int i = 1; i <= c->nx; i++) w->col_lonc[i] = swf_lonc(c, i);
  w->tables_ready = 1;
}

static int cmp_int(const void *a, const void *b) {
  const int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* Margin (radians of central angle) of the test that skips cells outside
 * the radius. The reference's computed distance differs from the exact
 * central angle of its inputs by far less than this (about 1e-15 / sin of
 * the angle: a few 1e-9 at angles of 1e-6), so a cell whose exact angle
 * exceeds radius/R + kSkipMargin is one where the reference finds
 * r >= radius and changes nothing. */
#define kSkipMargin 1e-6

/* get_Gaussian_field, fill mode 1 (perturbs.c:333-364): every interior cell
 * whose great-circle distance (tools.c:104-119, on the mean radius, between
 * planetocentric latitudes) is below the radius. Cells that cannot be inside
 * are skipped before that expression is evaluated: the central angle to the
 * centre is at least the difference of latitudes, and in a row at latitude
 * pl it exceeds th = radius/R + margin wherever the longitude difference
 * (mod 2 pi, as the cosine in the distance sees it) exceeds
 * acos((cos th - sin(plat) sin(pl)) / (cos(plat) cos(pl))). */
static void gaussian_field(const swcase *c, double lon, double lat, double amp, double sigma, double radius,
                           double inject, swforce *w) {
  const double R = (c->rE + c->rP) / 2.0;
  const double plat = swf_lat2pclat(c, lat);
  const double sp = sin(plat), cp = cos(plat);
  const double th = radius / R + kSkipMargin;
  const double two_pi = 8.0 * atan(1.0);
  const int skip = (th < 3.0);  /* otherwise every cell can be inside (or radius is not a number) */
  const double cth = cos(th);
  for (int j = 1; j <= c->ny; j++) {
    const double pl = w->row_pl[j];
    double dl = 4.0;  /* largest longitude difference that can be inside; >= pi: all */
    if (skip) {
      if (fabs(pl - plat) > th) continue;
      const double cmin = (cth - sp * w->row_sin[j]) / (cp * w->row_cos[j]);
      if (cmin > 1.0) continue;
      if (cmin > -1.0) dl = acos(cmin) + kSkipMargin;
    }
    for (int i = 1; i <= c->nx; i++) {
      if (dl < 3.14) {
        double d = w->col_lonc[i] - lon;
        d -= two_pi * nearbyint(d / two_pi);
        if (fabs(d) > dl) continue;
      }
      const double r = (R)*acos(sin(plat) * w->row_sin[j] + cos(plat) * w->row_cos[j] * cos(w->col_lonc[i] - lon));
      if (r < radius) {
        const size_t q = IXP(c->nx, i, j);
        w->pert[q] += amp * exp(-sq(r) / (2.0 * sq(sigma)));
        w->tracer[q] = (inject)*exp(-sq(r) / (2.0 * sq(sigma)));
        if (!w->mask[q]) w->cells[w->ncells++] = (int)q;
        w->mask[q] = 1;
        w->perturbs[q] = 1.0;
      }
    }
  }
}

int swforce_gaussian_plan(const swcase *c, int g, double Dt, double t, swf_gplan *p, char *err, size_t errlen) {
  const double *G = c->gaussians + (size_t)g * SWC_GAUSS_COLS;
  const double t0 = G[0], t1 = G[1];
  if (!((t0 <= t) && (t1 >= t))) return 1;  /* perturbs.c:63 */
  const double tau = G[2];
  if (tau < 0) {
    set_err(err, errlen, "Gaussian %d: tau is %e and should be positive", g, tau);
    return -1;
  }
  double lon = deg2rad(G[3]);
  const double lat = deg2rad(G[4]);
  const int isdegvel = (int)G[5];
  const double vel = G[6];
  if (isdegvel < 0 || isdegvel > 1) {
    set_err(err, errlen, "Gaussian %d: isdegvel should be 0 or 1", g);
    return -1;
  }
  const double tt = (t - t0);
  double Om = 0.0;
  if (isdegvel == 0) Om = vel / swf_rZ(c, lat);
  if (isdegvel == 1) Om = deg2rad(vel);
  lon = lon + Om * tt;  /* perturbs.c:92-94, polar 0 */
  const double Q = G[7];
  const int isdegsize = (int)G[8];
  double sigma = G[9], radius = G[10];
  const double inject = G[11];
  if (isdegsize < 0 || isdegsize > 1) {
    set_err(err, errlen, "Gaussian %d: isdegsize should be 0 or 1", g);
    return -1;
  }
  if (isdegsize == 1) {  /* perturbs.c:127-130 */
    sigma = sigma / 360.0 * 2 * PI_() * (c->rE + c->rP) / 2.0;
    radius = radius / 360.0 * 2 * PI_() * (c->rE + c->rP) / 2.0;
  }
  /* injected flow rate: first-order rise, plateau, first-order decay (perturbs.c:141-186);
   * a time covered by none of the three keeps no injection */
  double Qexp = 0.0;
  const double tauTH = 6 * tau;
  const double t_int = tau * log(exp((t1 - tauTH) / tau) + exp(t0 / tau));
  if ((t < tauTH + t0) && (t < t_int)) Qexp = Q * (1.0 - exp(-(t - t0) / tau));
  if ((t0 + tauTH <= t) && (t <= t1 - tauTH)) Qexp = Q;
  if ((t > t1 - tauTH) && (t > t_int)) Qexp = Q * exp(-(t - (t1 - tauTH)) / tau);
  const double volume = Dt * Qexp;

  /* add_Gaussian_core (perturbs.c:199-330) */
  while (lon < c->lon0) lon += (c->lon1 - c->lon0);
  while (lon > c->lon1) lon -= (c->lon1 - c->lon0);
  p->lon = lon;
  p->lat = lat;
  p->sigma = sigma;
  p->radius = radius;
  p->inject = inject;
  p->volume = volume;
  p->amp = volume / (2.0 * PI_() * sq(sigma) * (1.0 - exp(-sq(radius) / (2.0 * sq(sigma)))));
  p->images = 0;
  if ((lon + radius / swf_rZ(c, lat)) >= c->lon1) p->images |= 1;  /* perturbs.c:250-258 */
  if ((lon - radius / swf_rZ(c, lat)) <= c->lon0) p->images |= 2;
  return 0;
}

int swforce_gaussian(const swcase *c, int g, double Dt, double t, swforce *w, double *scale, char *err,
                     size_t errlen) {
  *scale = 0.0;
  swf_gplan p;
  const int prc = swforce_gaussian_plan(c, g, Dt, t, &p, err, errlen);
  if (prc != 0) return prc;
  const double lon = p.lon, lat = p.lat, sigma = p.sigma, radius = p.radius, inject = p.inject;
  const double volume = p.volume, amp = p.amp;
  tables(c, w);
  /* the previous injection's cells back to zero (the reference starts from a
   * zeroed perturb_field, perturbs.c:237-238) */
  for (int k = 0; k < w->ncells; k++) {
    w->pert[w->cells[k]] = 0.0;
    w->mask[w->cells[k]] = 0;
  }
  w->ncells = 0;
  gaussian_field(c, lon, lat, amp, sigma, radius, inject, w);
  const double lonRight = lon + (c->lon1 - c->lon0);
  const double lonLeft = lon - (c->lon1 - c->lon0);
  if (p.images & 1) gaussian_field(c, lonLeft, lat, amp, sigma, radius, inject, w);
  if (p.images & 2) gaussian_field(c, lonRight, lat, amp, sigma, radius, inject, w);
  /* padded index order is the reference's loop order (j outer, i inner) */
  qsort(w->cells, (size_t)w->ncells, sizeof(int), cmp_int);
  const int W = c->nx + 4;
  for (int k = 0; k < w->ncells; k++) {
    w->cell_pert[k] = w->pert[w->cells[k]];
    w->cell_tracer[k] = w->tracer[w->cells[k]];
  }
  /* injected volume, summed in the reference's loop order; the cells off the
   * list add +0.0, which changes no sum that starts at +0.0 */
  double V = 0.0;
  for (int k = 0; k < w->ncells; k++) V += w->cell_pert[k] * w->row_surf[w->cells[k] / W - 1];
  if (fabs(volume) > 1e-7) {
    if (V == 0.0) {
      set_err(err, errlen, "Gaussian %d: total injected volume is 0", g);
      return -1;
    }
    const double rf = (volume / V);
    /* the reference's own check of the rescaled volume (perturbs.c:310-326) */
    double Vc = 0.0;
    for (int k = 0; k < w->ncells; k++) Vc += (rf * w->cell_pert[k]) * w->row_surf[w->cells[k] / W - 1];
    if (fabs(Vc - volume) / volume > 1e-1) {
      set_err(err, errlen, "Gaussian %d: injected volume %e does not match %e", g, Vc, volume);
      return -1;
    }
    *scale = rf;
  }
  return 0;
}

int swforce_vortex_due(const swcase *c, int k, double Dt, double t) {
  const double t0 = c->vortices[(size_t)k * SWC_VORTEX_COLS + 0];
  return (t0 < t) && (t0 >= (t - Dt));  /* perturbs.c:388 */
}

void swforce_vortex(const swcase *c, int k, swforce *w) {
  const double *V = c->vortices + (size_t)k * SWC_VORTEX_COLS;
  const double lonc = V[1], latc = V[2], as = V[3], bs = V[4], Umax = V[5], n = V[6];
  /* perturbs.c:401 (g_eff of the planetographic latitude, as written there) */
  const double amp = 0.5 * Umax * swf_rM(c, deg2rad(latc)) * deg2rad(bs) * fcor(c, deg2rad(latc)) *
                     pow((1.0 - 1.0 / (2.0 * n)), ((1.0 - 2.0 * n) / (2.0 * n))) * exp(1.0 - 1.0 / (2.0 * n)) /
                     (swf_g_eff(c, deg2rad(latc)) * n);
  const size_t S = (size_t)(c->nx + 4) * (c->ny + 4);
  memset(w->deta, 0, S * sizeof(double));
  memset(w->du, 0, S * sizeof(double));
  memset(w->dv, 0, S * sizeof(double));
  /* add_vortex_core (perturbs.c:418-441) */
  for (int j = 1; j <= c->ny; j++) {
    const double LATC = swf_latc(c, j), LATE = swf_latc(c, j), LATN = swf_latn(c, j);
    const double GE = swf_g_eff(c, swf_lat2pclat(c, LATE)), GN = swf_g_eff(c, swf_lat2pclat(c, LATN));
    for (int i = 1; i <= c->nx; i++) {
      const double LONC = swf_lonc(c, i), LONE = swf_lone(c, i), LONN = swf_lonc(c, i);
      const double exponent = pow(sq((rad2deg(LONC) - lonc) / as) + sq((rad2deg(LATC) - latc) / bs), n);
      const double eta_ij = amp * exp(-exponent);
      const double psi_u = sq((rad2deg(LONE) - lonc) / as) + sq((rad2deg(LATE) - latc) / bs);
      const double du = 2.0 * (n)*GE / (fcor(c, deg2rad(latc)) * sq(deg2rad(bs)) * swf_rM(c, deg2rad(latc))) *
                        (LATE - deg2rad(latc)) * pow(psi_u, n - 1.0) * eta_ij;
      const double psi_v = sq((rad2deg(LONN) - lonc) / as) + sq((rad2deg(LATN) - latc) / bs);
      const double dv = -2.0 * (n)*GN / (fcor(c, deg2rad(latc)) * sq(deg2rad(as)) * swf_rZ(c, deg2rad(latc))) *
                        (LONN - deg2rad(lonc)) * pow(psi_v, n - 1.0) * eta_ij;
      const size_t q = IXP(c->nx, i, j);
      w->deta[q] = eta_ij;
      w->du[q] = du;
      w->dv[q] = dv;
    }
  }
}

/* linterp_core over the whole table (tools.c:21-74); at the last abscissa the
 * reference's extra term multiplies a zero, leaving y[n-1]. */
static double linterp(double xi, const double *x, const double *y, int n) {
  int i = 0;
  while (i < n - 1 && x[i + 1] <= xi) i++;
  if (i >= n - 1) return y[n - 1];
  return (y[i + 1] - y[i]) * (xi - x[i]) / (x[i + 1] - x[i]) + y[i];
}

void swf_halo_wrap(double *x, int nx, int ny) {
  const int W = nx + 4;
  for (int i = 1; i <= nx; i++) {  /* y pass, interior columns */
    x[IXP(nx, i, -1)] = x[IXP(nx, i, ny - 1)];
    x[IXP(nx, i, 0)] = x[IXP(nx, i, ny)];
    x[IXP(nx, i, ny + 1)] = x[IXP(nx, i, 1)];
    x[IXP(nx, i, ny + 2)] = x[IXP(nx, i, 2)];
  }
  for (int j = -1; j <= ny + 2; j++) {  /* x pass, all rows */
    x[IXP(nx, -1, j)] = x[IXP(nx, nx - 1, j)];
    x[IXP(nx, 0, j)] = x[IXP(nx, nx, j)];
    x[IXP(nx, nx + 1, j)] = x[IXP(nx, 1, j)];
    x[IXP(nx, nx + 2, j)] = x[IXP(nx, 2, j)];
  }
  (void)W;
}

int swforce_windx(const swcase *c, double *windx, char *err, size_t errlen) {
  const int n = c->wind_rows;
  const double *x = c->wind, *y = c->wind + n;
  if (n < 2) {
    set_err(err, errlen, "wind table needs at least 2 rows");
    return -1;
  }
  if (rad2deg(swf_latc(c, -1)) < x[0] || rad2deg(swf_latc(c, c->ny + 2)) > x[n - 1]) {  /* io.c:201 */
    set_err(err, errlen, "wind table (%e .. %e) does not cover the band's rows", x[0], x[n - 1]);
    return -1;
  }
  for (int j = -1; j <= c->ny + 2; j++) {
    const double w = linterp(rad2deg(swf_latc(c, j)), x, y, n);
    for (int i = -1; i <= c->nx + 2; i++) windx[IXP(c->nx, i, j)] = w;
  }
  swf_halo_wrap(windx, c->nx, c->ny);
  return 0;
}

static double great_angle(double lon0, double lat0, double lon1, double lat1) {  /* tools.c:122-136 */
  return acos(sin(lat0) * sin(lat1) + cos(lat0) * cos(lat1) * cos(lon1 - lon0));
}

/* read_wind for a polar cap (io.c:207-240): the zonal wind of the table at
 * each point's polar latitude, turned around the pole, and damped beyond the
 * sponge; no halo update follows (init.c:232-235). */
static void polar_winds(const swcase *c, double beta, double *windx, double *windy) {
  const int n = c->wind_rows;
  const double *x = c->wind, *y = c->wind + n;
  const double mlon = ((c->lon0) + (c->lon1)) / 2.0, mlat = ((c->lat0) + (c->lat1)) / 2.0;
  const double k = log(0.01) / (sqrt(2.0) * c->lat1 - beta);
  for (int j = -1; j <= c->ny + 2; j++)
    for (int i = -1; i <= c->nx + 2; i++) {
      const double LONC = swf_lonc(c, i), LATC = swf_latc(c, j);
      const double plat = (c->polar) * (PI_() / 2.0 - great_angle(LONC, LATC, mlon, mlat));  /* sw.h:130 */
      const size_t q = IXP(c->nx, i, j);
      if (rad2deg(plat) < x[0] || rad2deg(plat) > x[n - 1]) {
        windx[q] = 0;
        windy[q] = 0;
        continue;
      }
      double ang = acos((LATC - mlat) / sqrt(sq(LATC - mlat) + sq(LONC - mlon)));
      if (!((LONC - mlon) >= 0)) ang = -ang;
      const double w = linterp(rad2deg(plat), x, y, n);
      if (c->polar == 1) {
        windx[q] = -cos(ang) * w;
        windy[q] = sin(ang) * w;
      } else {
        windx[q] = cos(ang) * w;
        windy[q] = -sin(ang) * w;
      }
      const double dist = fabs(great_angle(mlon, mlat, LONC, LATC)) - beta;
      if (dist >= 0) {
        windx[q] = windx[q] * exp(k * dist);
        windy[q] = windy[q] * exp(k * dist);
      }
    }
}

int swforce_winds(const swcase *c, double beta_sponge_deg, double *windx, double *windy, char *err,
                  size_t errlen) {
  const int n = c->wind_rows;
  if (n < 2) {
    set_err(err, errlen, "wind table needs at least 2 rows");
    return -1;
  }
  if (c->polar != 0) {
    polar_winds(c, deg2rad(beta_sponge_deg), windx, windy);
    return 0;
  }
  memset(windy, 0, (size_t)(c->nx + 4) * (c->ny + 4) * sizeof(double));
  return swforce_windx(c, windx, err, errlen);
}

