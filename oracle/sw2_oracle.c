/*
 * CPU oracle for the SW2 shallow-water step (TEST INFRASTRUCTURE ONLY; see
 * sw2_oracle.h). Every expression below keeps the association and operand
 * order of the reference expression it restates, so that with
 * -ffp-contract=off the results are bit-identical to the reference's own
 * single-rank run. Build: oracle/Makefile.
 */
#include "sw2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NTAB 11

struct sw2o {
  sw2o_params p;
  int nx, ny, W, S;
  /* physical constants as the reference stores them (init.c:56-161) */
  double lon0, lon1, lat0, lat1, eps2, sigma, nu2, nu4, nu6;
  /* per-row tables, index j+1 */
  double *row[NTAB];
  double *rmc, *rzc, *rmn, *rzn, *sinc, *sinn;
  /* state */
  double *f[7]; /* eta u v tracer windx windy hB */
  /* histories and scratch (core.c:55-81) */
  double *dtr[3], *deta[3], *du[3], *dv[3]; /* [0]=n [1]=n-1 [2]=n-2 */
  double *dtrAB, *detaAB, *duAB, *dvAB;
  double *duadv, *dvadv, *dupres, *dvpres;
  double *L[6];   /* Lu Lv LLu LLv LLLu LLLv */
  double *Le[3];  /* Le LLe LLLe */
  double *psi, *xi, *ze, *di;
  int k; /* AB index n - nstart */
};

enum { F_ETA, F_U, F_V, F_TR, F_WX, F_WY, F_HB };
enum { T_DXE, T_DXC, T_DXV, T_DYN, T_DYC, T_DYV, T_GE, T_GN, T_GC, T_FE, T_FN };

#define IX(i, j) ((i) + 1 + ((j) + 1) * W)
#define R(t, j) (s->row[t][(j) + 1])

/* ---------------------------------------------------------------- geometry */
/* sw.h:16,108 */
static double ref_pi(void) { return 4.0 * atan(1.0); }
static double deg2rad(double a) { return a * (ref_pi() / 180.0); }
/* tools.c:256-273 */
static double linspace_val(int i, double x0, double x1, int n) { return x0 + (double)i * (x1 - x0) / ((double)n); }
/* sw.h:174 */
static double rZ(const sw2o *s, double lat) { return s->p.rE / sqrt(1.0 + (tan(lat) * tan(lat)) / s->eps2); }
/* sw.h:175 */
static double rM(const sw2o *s, double lat) {
  double q = rZ(s, lat) / (s->p.rE * cos(lat));
  return s->p.rE / s->eps2 * (q * q * q);
}
/* sw.h:170 */
static double lat2pclat(const sw2o *s, double lat) { return atan(1.0 / s->eps2 * tan(lat)); }
/* sw.h:172 */
static double rad(const sw2o *s, double pc) {
  double a = s->p.rE * sin(pc), b = s->p.rP * cos(pc);
  return s->p.rE * s->p.rP / sqrt(a * a + b * b);
}
/* sw.h:178-179 */
static double g_eff(const sw2o *s, double pc) {
  double Om = s->p.Omega, r = rad(s, pc);
  double g0 = (s->p.gE + Om * Om * s->p.rE) * ((s->p.rE / r) * (s->p.rE / r));
  return g0 - Om * Om * r * cos(pc);
}
/* sw.h:193 */
static double fcor(const sw2o *s, double lat) { return 2.0 * s->p.Omega * sin(lat); }
static double latn(const sw2o *s, int j) { return linspace_val(j, s->lat0, s->lat1, s->ny); }
static double latc(const sw2o *s, int j) { return (latn(s, j) + latn(s, j - 1)) / 2.; }

/* coords.c:35-96 and init.c:279-297, reduced to one value per row (polar 0) */
static void build_rows(sw2o *s) {
  int ny = s->ny;
  double dlon = (s->lon1 - s->lon0) / ((double)s->nx);
  double dlat = (s->lat1 - s->lat0) / ((double)ny);
  for (int j = -1; j <= ny + 2; j++) {
    double lc = latc(s, j), ln = latn(s, j);
    R(T_DXE, j) = dlon * rZ(s, lc);
    R(T_DXC, j) = dlon * rZ(s, lc);
    R(T_DXV, j) = dlon * rZ(s, ln);
    R(T_DYN, j) = dlat * rM(s, lc);
    R(T_DYC, j) = dlat * rM(s, latn(s, j - 1));
    R(T_DYV, j) = dlat * rM(s, lc);
    R(T_GE, j) = g_eff(s, lat2pclat(s, lc));
    R(T_GN, j) = g_eff(s, lat2pclat(s, ln));
    R(T_GC, j) = g_eff(s, lat2pclat(s, lc));
    R(T_FE, j) = fcor(s, lc);
    R(T_FN, j) = fcor(s, ln);
    s->rmc[j + 1] = rM(s, lc);
    s->rzc[j + 1] = rZ(s, lc);
    s->rmn[j + 1] = rM(s, ln);
    s->rzn[j + 1] = rZ(s, ln);
    s->sinc[j + 1] = sin(lc);
    s->sinn[j + 1] = sin(ln);
  }
}

/* ---------------------------------------------------------------- plumbing */
static double *zalloc(int n) { return (double *)calloc((size_t)n, sizeof(double)); }

sw2o *sw2o_create(const sw2o_params *p) {
  if (p->nx < 3 || p->ny < 3 || p->sch < 0 || p->sch > 9) return NULL;
  sw2o *s = (sw2o *)calloc(1, sizeof(sw2o));
  s->p = *p;
  s->nx = p->nx;
  s->ny = p->ny;
  s->W = p->nx + 4;
  s->S = (p->nx + 4) * (p->ny + 4);
  s->lon0 = deg2rad(p->lon0);
  s->lon1 = deg2rad(p->lon1);
  s->lat0 = deg2rad(p->lat0);
  s->lat1 = deg2rad(p->lat1);
  s->eps2 = (p->rE / p->rP) * (p->rE / p->rP);   /* init.c:150 */
  s->sigma = p->tau > 1e10 ? 0 : 1.0 / p->tau;    /* init.c:110-114 */
  s->nu2 = p->hypernu[0];
  s->nu4 = -p->hypernu[1];                         /* init.c:120 */
  s->nu6 = p->hypernu[2];
  int nr = p->ny + 4;
  for (int t = 0; t < NTAB; t++) s->row[t] = zalloc(nr);
  s->rmc = zalloc(nr); s->rzc = zalloc(nr); s->rmn = zalloc(nr); s->rzn = zalloc(nr);
  s->sinc = zalloc(nr); s->sinn = zalloc(nr);
  for (int q = 0; q < 7; q++) s->f[q] = zalloc(s->S);
  for (int q = 0; q < 3; q++) {
    s->dtr[q] = zalloc(s->S); s->deta[q] = zalloc(s->S); s->du[q] = zalloc(s->S); s->dv[q] = zalloc(s->S);
  }
  s->dtrAB = zalloc(s->S); s->detaAB = zalloc(s->S); s->duAB = zalloc(s->S); s->dvAB = zalloc(s->S);
  s->duadv = zalloc(s->S); s->dvadv = zalloc(s->S); s->dupres = zalloc(s->S); s->dvpres = zalloc(s->S);
  for (int q = 0; q < 6; q++) s->L[q] = zalloc(s->S);
  for (int q = 0; q < 3; q++) s->Le[q] = zalloc(s->S);
  s->psi = zalloc(s->S); s->xi = zalloc(s->S); s->ze = zalloc(s->S); s->di = zalloc(s->S);
  build_rows(s);
  return s;
}

void sw2o_destroy(sw2o *s) {
  if (!s) return;
  for (int t = 0; t < NTAB; t++) free(s->row[t]);
  free(s->rmc); free(s->rzc); free(s->rmn); free(s->rzn); free(s->sinc); free(s->sinn);
  for (int q = 0; q < 7; q++) free(s->f[q]);
  for (int q = 0; q < 3; q++) { free(s->dtr[q]); free(s->deta[q]); free(s->du[q]); free(s->dv[q]); }
  free(s->dtrAB); free(s->detaAB); free(s->duAB); free(s->dvAB);
  free(s->duadv); free(s->dvadv); free(s->dupres); free(s->dvpres);
  for (int q = 0; q < 6; q++) free(s->L[q]);
  for (int q = 0; q < 3; q++) free(s->Le[q]);
  free(s->psi); free(s->xi); free(s->ze); free(s->di);
  free(s);
}

int sw2o_padded_size(const sw2o *s) { return s->S; }
double *sw2o_field(sw2o *s, int which) { return (which >= 0 && which < 7) ? s->f[which] : NULL; }
const double *sw2o_row_table(const sw2o *s, int which) { return (which >= 0 && which < NTAB) ? s->row[which] : NULL; }
void sw2o_reset_ab(sw2o *s) { s->k = 0; }

int sw2o_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* sppde_hupdate.c:274-342: y first (interior columns, rows wrap even though y
 * is a wall), then x over every row including the y halos (corners). */
void sw2o_halo_update(int nx, int ny, double *x) {
  int W = nx + 4;
  for (int i = 1; i <= nx; i++) {
    x[IX(i, -1)] = x[IX(i, ny - 1)];
    x[IX(i, 0)] = x[IX(i, ny)];
    x[IX(i, ny + 1)] = x[IX(i, 1)];
    x[IX(i, ny + 2)] = x[IX(i, 2)];
  }
  for (int j = -1; j <= ny + 2; j++) {
    x[IX(-1, j)] = x[IX(nx - 1, j)];
    x[IX(0, j)] = x[IX(nx, j)];
    x[IX(nx + 1, j)] = x[IX(1, j)];
    x[IX(nx + 2, j)] = x[IX(2, j)];
  }
}

static void halo(sw2o *s, double *x) { sw2o_halo_update(s->nx, s->ny, x); }

static void interior_copy(sw2o *s, double *dst, const double *src) {
  int W = s->W;
  for (int j = 1; j <= s->ny; j++) memcpy(dst + IX(1, j), src + IX(1, j), sizeof(double) * (size_t)s->nx);
}

void sw2o_load(sw2o *s, const double *eta, const double *u, const double *v, const double *tracer,
               const double *windx, const double *windy, const double *hB) {
  const double *in[4] = {eta, u, v, tracer};
  for (int q = 0; q < 4; q++) {
    memset(s->f[q], 0, sizeof(double) * (size_t)s->S);
    interior_copy(s, s->f[q], in[q]);
    halo(s, s->f[q]);
  }
  memcpy(s->f[F_WX], windx, sizeof(double) * (size_t)s->S);
  memcpy(s->f[F_WY], windy, sizeof(double) * (size_t)s->S);
  memcpy(s->f[F_HB], hB, sizeof(double) * (size_t)s->S);
  s->k = 0;
}

void sw2o_load_raw(sw2o *s, const double *eta, const double *u, const double *v, const double *tracer,
                   const double *windx, const double *windy, const double *hB) {
  const double *in[7] = {eta, u, v, tracer, windx, windy, hB};
  for (int q = 0; q < 7; q++) memcpy(s->f[q], in[q], sizeof(double) * (size_t)s->S);
  s->k = 0;
}

/* ---------------------------------------------------------------- limiters */
/* calc.c:54-63 with sw.h:104-105 MIN/MAX (ternaries, NaN-order as written) */
#define MN(a, b) (((a) < (b)) ? (a) : (b))
#define MX(a, b) (((a) > (b)) ? (a) : (b))
static inline __attribute__((always_inline)) double limiter(int sch, double r) {
  switch (sch) {
    case 0: return MX(0, MN(MN((1 + r) / 2.0, 2.0 * r), 2.0));
    case 1: return MX(MX(0, MN(2.0 * r, 1.0)), MX(0, MN(r, 2.0)));
    case 2: return MN(r, 1);
    case 3: return (r + fabs(r)) / (1.0 + r);
    case 4: return MX(0, MN(2.0 * r, MN((1 + 2.0 * r) / 3.0, 2.0)));
    case 5: return (1.5 * (r * r + r)) / (r * r + r + 1.0);
    case 6: return (r * r + r) / (r * r + 1.0);
    case 7: return MX(0, MN(MN(2.0, 2.0 * r), MN(0.25 + 0.75 * r, 0.75 + 0.25 * r)));
    case 8: return 0;
    default: return 1.0;
  }
}

/* One face between cells q0|q1 with outer neighbours qm, q2 (calc.c:41-49):
 * r2rP/r2rM slope ratios, then the two limited face values. */
typedef struct { double P, M; } face2;
static inline __attribute__((always_inline)) face2 tvd_face(int sch, double qm, double q0, double q1, double q2,
                                                            double cP, double cM) {
  double d = q1 - q0;
  double rP = (d != 0) ? ((q0 - qm) / d) : 0;
  double rM = (d != 0) ? ((q2 - q1) / d) : 0;
  face2 b;
  b.P = q0 + limiter(sch, rP) * 0.5 * (1 - cP) * d;
  b.M = q1 - limiter(sch, rM) * 0.5 * (1 + cM) * d;
  return b;
}

/* Courant numbers of one upwind-split face (calc.c:72-79) */
static inline double cpos(double a, double dt, double dx) { return 0.5 * (a + fabs(a)) * dt / dx; }
static inline double cneg(double a, double dt, double dx) { return 0.5 * (a - fabs(a)) * dt / dx; }
/* averaged Courant numbers of the momentum bodies (calc.c:170-177, 207-214) */
static inline double cpos2(double a, double b, double dt, double dx) {
  return 0.5 * (0.5 * (a + fabs(a)) + 0.5 * (b + fabs(b))) * dt / dx;
}
static inline double cneg2(double a, double b, double dt, double dx) {
  return 0.5 * (0.5 * (a - fabs(a)) + 0.5 * (b - fabs(b))) * dt / dx;
}

/* ------------------------------------------------- flux-form TVD sweep body */
/* Given the 5-point x and y stencils of a scalar q at a cell and the eight
 * Courant numbers, returns Sum C*B in the reference's order (calc.c:100). */
static inline __attribute__((always_inline)) double tvd_sum(int sch, const double *qx, const double *qy,
                                                            double cwP, double cwM, double ceP, double ceM,
                                                            double csP, double csM, double cnP, double cnM) {
  /* qx/qy: index 0..4 = offsets -2..+2 */
  face2 w = tvd_face(sch, qx[0], qx[1], qx[2], qx[3], cwP, cwM);
  face2 e = tvd_face(sch, qx[1], qx[2], qx[3], qx[4], ceP, ceM);
  face2 so = tvd_face(sch, qy[0], qy[1], qy[2], qy[3], csP, csM);
  face2 n = tvd_face(sch, qy[1], qy[2], qy[3], qy[4], cnP, cnM);
  return cwP * w.P + cwM * w.M - ceP * e.P - ceM * e.M + csP * so.P + csM * so.M - cnP * n.P - cnM * n.M;
}

#define UW(i, j) (u[IX(i, j)] + wx[IX(i, j)]) /* sw.h:216 */
#define VW(i, j) (v[IX(i, j)] + wy[IX(i, j)]) /* sw.h:217 */
#define HH(i, j) (eta[IX(i, j)] + depth - hb[IX(i, j)]) /* sw.h:213 */

/* BODYH / solve_cons_h first part (calc.c:70-113, 289-321) */
static inline __attribute__((always_inline)) void mass_sweep_s(sw2o *s, int sch, double *out) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  const double *eta = s->f[F_ETA], *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY], *hb = s->f[F_HB];
  const double depth = s->p.depth, Dt = s->p.Dt, sig = s->sigma;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double dxe = R(T_DXE, j), dyn = R(T_DYN, j);
    for (int i = 1; i <= nx; i++) {
      double qx[5], qy[5];
      for (int o = -2; o <= 2; o++) { qx[o + 2] = HH(i + o, j); qy[o + 2] = HH(i, j + o); }
      double a = UW(i - 1, j), b = UW(i, j), c = VW(i, j - 1), d = VW(i, j);
      double acc = tvd_sum(sch, qx, qy, cpos(a, Dt, dxe), cneg(a, Dt, dxe), cpos(b, Dt, dxe), cneg(b, Dt, dxe),
                           cpos(c, Dt, dyn), cneg(c, Dt, dyn), cpos(d, Dt, dyn), cneg(d, Dt, dyn));
      acc -= 2.0 * Dt * (sig)*eta[IX(i, j)];
      out[IX(i, j)] = acc;
    }
  }
}

/* BODYTRACER (calc.c:117-163) */
static inline __attribute__((always_inline)) void tracer_sweep_s(sw2o *s, int sch, double *out) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  const double *tr = s->f[F_TR], *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY];
  const double Dt = s->p.Dt, sig = s->p.tracer_dis;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double dxe = R(T_DXE, j), dyn = R(T_DYN, j);
    for (int i = 1; i <= nx; i++) {
      double qx[5], qy[5];
      for (int o = -2; o <= 2; o++) { qx[o + 2] = tr[IX(i + o, j)]; qy[o + 2] = tr[IX(i, j + o)]; }
      double a = UW(i - 1, j), b = UW(i, j), c = VW(i, j - 1), d = VW(i, j);
      double pv1 = tvd_sum(sch, qx, qy, cpos(a, Dt, dxe), cneg(a, Dt, dxe), cpos(b, Dt, dxe), cneg(b, Dt, dxe),
                           cpos(c, Dt, dyn), cneg(c, Dt, dyn), cpos(d, Dt, dyn), cneg(d, Dt, dyn));
      double t = tr[IX(i, j)];
      double pv2 = Dt * t * (b - a) / dxe;
      pv2 += Dt * t * (d - c) / dyn;
      double acc = pv1 + pv2;
      acc -= 2.0 * Dt * (sig)*t;
      out[IX(i, j)] = acc;
    }
  }
}

/* BODYU (calc.c:168-200) */
static inline __attribute__((always_inline)) void adv_u_s(sw2o *s, int sch, double *out) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  const double *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY];
  const double Dt = s->p.Dt;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double dxc = R(T_DXC, j), dyv = R(T_DYV, j), dxe = R(T_DXE, j);
    for (int i = 1; i <= nx; i++) {
      double qx[5], qy[5];
      for (int o = -2; o <= 2; o++) { qx[o + 2] = UW(i + o, j); qy[o + 2] = UW(i, j + o); }
      double uwm = qx[1], u0 = qx[2], uep = qx[3];
      double vs0 = VW(i, j - 1), vs1 = VW(i + 1, j - 1), vn0 = VW(i, j), vn1 = VW(i + 1, j);
      double p1 = tvd_sum(sch, qx, qy, cpos2(uwm, u0, Dt, dxc), cneg2(uwm, u0, Dt, dxc), cpos2(u0, uep, Dt, dxc),
                          cneg2(u0, uep, Dt, dxc), cpos2(vs0, vs1, Dt, dyv), cneg2(vs0, vs1, Dt, dyv),
                          cpos2(vn0, vn1, Dt, dyv), cneg2(vn0, vn1, Dt, dyv));
      double p2 = Dt * (u0 * (uep - uwm) / (dxe + dxe) + u0 * ((vn0 + vn1) / 2. - (vs0 + vs1) / 2.) / dyv);
      out[IX(i, j)] = p1 + p2;
    }
  }
}

/* BODYV (calc.c:205-237) */
static inline __attribute__((always_inline)) void adv_v_s(sw2o *s, int sch, double *out) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  const double *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY];
  const double Dt = s->p.Dt;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double dxv = R(T_DXV, j), dyc = R(T_DYC, j), dyn0 = R(T_DYN, j), dyn1 = R(T_DYN, j + 1);
    for (int i = 1; i <= nx; i++) {
      double qx[5], qy[5];
      for (int o = -2; o <= 2; o++) { qx[o + 2] = VW(i + o, j); qy[o + 2] = VW(i, j + o); }
      double vsm = qy[1], v0 = qy[2], vnp = qy[3];
      double uw1 = UW(i - 1, j + 1), uw0 = UW(i - 1, j), ue1 = UW(i, j + 1), ue0 = UW(i, j);
      double p1 = tvd_sum(sch, qx, qy, cpos2(uw1, uw0, Dt, dxv), cneg2(uw1, uw0, Dt, dxv), cpos2(ue1, ue0, Dt, dxv),
                          cneg2(ue1, ue0, Dt, dxv), cpos2(vsm, v0, Dt, dyc), cneg2(vsm, v0, Dt, dyc),
                          cpos2(v0, vnp, Dt, dyc), cneg2(v0, vnp, Dt, dyc));
      double p2 = Dt * (v0 * ((ue0 + ue1) / 2. - (uw0 + uw1) / 2.) / dxv + v0 * (vnp - vsm) / (dyn0 + dyn1));
      out[IX(i, j)] = p1 + p2;
    }
  }
}

#define SCHEME_SWITCH(fn, s, out)          \
  switch ((s)->p.sch) {                    \
    case 0: fn(s, 0, out); break;          \
    case 1: fn(s, 1, out); break;          \
    case 2: fn(s, 2, out); break;          \
    case 3: fn(s, 3, out); break;          \
    case 4: fn(s, 4, out); break;          \
    case 5: fn(s, 5, out); break;          \
    case 6: fn(s, 6, out); break;          \
    case 7: fn(s, 7, out); break;          \
    case 8: fn(s, 8, out); break;          \
    default: fn(s, 9, out); break;         \
  }

/* ------------------------------------------------------------- laplacians */
/* laplacian_eta (laplacian.c:114-151). psi/xi halos read as zero. */
static void lap_eta(sw2o *s, const double *e_in, double *e_out) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  double *psi = s->psi, *xi = s->xi;
  memset(psi, 0, sizeof(double) * (size_t)s->S);
  memset(xi, 0, sizeof(double) * (size_t)s->S);
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double kx = s->rmc[j + 1] / s->rzc[j + 1], ky = s->rzn[j + 1] / s->rmn[j + 1];
    double dxc = R(T_DXC, j), dyc = R(T_DYC, j);
    for (int i = 1; i <= nx; i++) {
      psi[IX(i, j)] = kx * (e_in[IX(i + 1, j)] - e_in[IX(i, j)]) / (dxc);
      xi[IX(i, j)] = ky * (e_in[IX(i, j + 1)] - e_in[IX(i, j)]) / (dyc);
    }
  }
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double kc = 1.0 / (s->rmc[j + 1] * s->rzc[j + 1]);
    double dxe = R(T_DXE, j), dyn = R(T_DYN, j);
    for (int i = 1; i <= nx; i++)
      e_out[IX(i, j)] =
          kc * ((psi[IX(i, j)] - psi[IX(i - 1, j)]) / (dxe) + (xi[IX(i, j)] - xi[IX(i, j - 1)]) / (dyn));
  }
  halo(s, e_out);
  for (int i = 1; i <= nx; i++) {
    e_out[IX(i, ny + 1)] = e_out[IX(i, ny)];
    e_out[IX(i, ny + 2)] = e_out[IX(i, ny + 1)];
    e_out[IX(i, 0)] = e_out[IX(i, 1)];
  }
}

/* laplacian_vels (laplacian.c:51-111) */
static void lap_vels(sw2o *s, const double *uu, const double *vv, double *lu, double *lv) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  double *ze = s->ze, *di = s->di;
  memset(ze, 0, sizeof(double) * (size_t)s->S);
  memset(di, 0, sizeof(double) * (size_t)s->S);
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double dxv = R(T_DXV, j), dxv_s = R(T_DXV, j - 1), dyc1 = R(T_DYC, j + 1), dxc = R(T_DXC, j),
           dxc1 = R(T_DXC, j + 1), dxe = R(T_DXE, j), dyn = R(T_DYN, j);
    for (int i = 1; i <= nx; i++) {
      double a = (1.0 / dxv), b = -(1.0 / dyc1);
      ze[IX(i, j)] = a * ((vv[IX(i + 1, j)] - vv[IX(i, j)]) + b * (dxc1 * uu[IX(i, j + 1)] - dxc * uu[IX(i, j)]));
      a = (1.0 / dxe);
      b = (1.0 / dyn);
      di[IX(i, j)] = a * ((uu[IX(i, j)] - uu[IX(i - 1, j)]) + b * (dxv * vv[IX(i, j)] - dxv_s * vv[IX(i, j - 1)]));
    }
  }
  halo(s, ze);
  halo(s, di);
  for (int i = 1; i <= nx; i++) {
    di[IX(i, ny + 1)] = (uu[IX(i, ny)] - uu[IX(i - 1, ny)]) / R(T_DXE, ny);
    ze[IX(i, 0)] = 0;
  }
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++) {
    double dyn = R(T_DYN, j), dxc = R(T_DXC, j), dxv = R(T_DXV, j), dyc1 = R(T_DYC, j + 1);
    for (int i = 1; i <= nx; i++) {
      double a = -(1.0 / dyn), b = (1.0 / dxc);
      lu[IX(i, j)] = a * (ze[IX(i, j)] - ze[IX(i, j - 1)]) + b * (di[IX(i + 1, j)] - di[IX(i, j)]);
      a = (1.0 / dxv);
      b = (1.0 / dyc1);
      lv[IX(i, j)] = a * (ze[IX(i, j)] - ze[IX(i - 1, j)]) + b * (di[IX(i, j + 1)] - di[IX(i, j)]);
    }
  }
  halo(s, lu);
  halo(s, lv);
  for (int i = 1; i <= nx; i++) {
    lu[IX(i, ny + 1)] = lu[IX(i, ny)];
    lv[IX(i, ny + 1)] = 0;
    lu[IX(i, 0)] = lu[IX(i, 1)];
    lv[IX(i, 0)] = 0;
  }
}

/* ------------------------------------------------------------ small phases */
/* do_AdamsBashforth with linop_scaf/copy_scaf (calc.c:651-699; sppde_core.c:247-298) */
static void adams_bashforth(sw2o *s, double *ab, const double *dn, const double *dm1, const double *dm2) {
  const int W = s->W, nx = s->nx, ny = s->ny, k = s->k;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      int q = IX(i, j);
      if (k == 0) {
        ab[q] = dn[q];
      } else if (k == 1) {
        ab[q] = (3.0 / 2.0) * dn[q] + -(1.0 / 2.0) * dm1[q];
      } else {
        double t = -(4.0 / 3.0) * dm1[q] + +(5.0 / 12.0) * dm2[q];
        ab[q] = (23.0 / 12.0) * dn[q] + 1.0 * t;
      }
    }
}

/* history shift by rotation: contents after the reference's two copy_scaf calls */
static void rotate(double **h) {
  double *t = h[2];
  h[2] = h[1];
  h[1] = h[0];
  h[0] = t;
}

static void add_interior(sw2o *s, double *x, const double *dx) {
  const int W = s->W;
  for (int j = 1; j <= s->ny; j++)
    for (int i = 1; i <= s->nx; i++) x[IX(i, j)] = x[IX(i, j)] + dx[IX(i, j)];
}

/* do_channel (calc.c:600-649), polar 0: interior columns only */
static void channel(sw2o *s) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  double *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY];
  for (int i = 1; i <= nx; i++) {
    v[IX(i, 0)] = 0; v[IX(i, -1)] = 0;
    wy[IX(i, 0)] = 0; wy[IX(i, -1)] = 0;
    u[IX(i, 0)] = u[IX(i, 1)]; u[IX(i, -1)] = u[IX(i, 0)];
    wx[IX(i, 0)] = wx[IX(i, 1)]; wx[IX(i, -1)] = wx[IX(i, 0)];
  }
  for (int i = 1; i <= nx; i++) {
    v[IX(i, ny)] = 0; v[IX(i, ny + 1)] = 0; v[IX(i, ny + 2)] = 0;
    wy[IX(i, ny)] = 0; wy[IX(i, ny + 1)] = 0; wy[IX(i, ny + 2)] = 0;
    u[IX(i, ny + 1)] = u[IX(i, ny)]; u[IX(i, ny + 2)] = u[IX(i, ny + 1)];
    wx[IX(i, ny + 1)] = wx[IX(i, ny)]; wx[IX(i, ny + 2)] = wx[IX(i, ny + 1)];
  }
}

/* compute_Dt (calc.c:701-738) */
static double cfl_dt(sw2o *s) {
  const int W = s->W;
  const double *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY];
  double mx = 0, my = 0;
  for (int j = 1; j <= s->ny; j++)
    for (int i = 1; i <= s->nx; i++) {
      double dxe = R(T_DXE, j), dyn = R(T_DYN, j);
      if (fabs(UW(i, j) / dxe) > mx) mx = fabs(UW(i, j)) / dxe;
      if (fabs(VW(i, j) / dyn) > my) my = fabs(VW(i, j)) / dyn;
    }
  if (mx + my == 0) {
    for (int j = 1; j <= s->ny; j++)
      for (int i = 1; i <= s->nx; i++) {
        double dxe = R(T_DXE, j), dyn = R(T_DYN, j);
        double cx = sqrt((s->p.depth) * (R(T_GE, j))), cy = sqrt((s->p.depth) * (R(T_GN, j)));
        if (fabs(cx / dxe) > mx) mx = fabs(cx) / dxe;
        if (fabs(cy / dyn) > my) my = fabs(cy) / dyn;
      }
  }
  return (s->p.courant / (mx + my));
}

/* get_stats_scaf / check_stats_scaf (sppde_core.c:346-395) */
static int stats_bad(sw2o *s, const double *x) {
  const int W = s->W;
  double n = 0, mn = 0, mx = 0;
  for (int j = 1; j <= s->ny; j++)
    for (int i = 1; i <= s->nx; i++) {
      double r = x[IX(i, j)];
      n = n + 1;
      if (r < mn || n == 1.0) mn = r;
      if (r > mx || n == 1.0) mx = r;
    }
  return (mn < -1e10 || mx > 1e10 || isfinite(mn) == 0 || isfinite(mx) == 0);
}

/* ------------------------------------------------------------------- step */
static void one_step(sw2o *s) {
  const int W = s->W, nx = s->nx, ny = s->ny;
  const double Dt = s->p.Dt;
  double *eta = s->f[F_ETA], *u = s->f[F_U], *v = s->f[F_V], *hb = s->f[F_HB];
  double *wx = s->f[F_WX], *wy = s->f[F_WY];
  const double depth = s->p.depth;

  /* tracer (core.c:161-182) */
  SCHEME_SWITCH(tracer_sweep_s, s, s->dtr[0]);
  adams_bashforth(s, s->dtrAB, s->dtr[0], s->dtr[1], s->dtr[2]);
  rotate(s->dtr);
  add_interior(s, s->f[F_TR], s->dtrAB);
  halo(s, s->f[F_TR]);

  /* mass (core.c:184-210; calc.c:289-355) */
  double *dn = s->deta[0];
  SCHEME_SWITCH(mass_sweep_s, s, dn);
  if (s->nu2 != 0 || s->nu4 != 0 || s->nu6 != 0) {
    for (int q = 0; q < 3; q++) memset(s->Le[q], 0, sizeof(double) * (size_t)s->S);
    lap_eta(s, s->p.lape_eta ? eta : u, s->Le[0]); /* the reference applies it to u (calc.c:332) */
    if (s->nu4 != 0 || s->nu6 != 0) {
      lap_eta(s, s->Le[0], s->Le[1]);
      if (s->nu6 != 0) lap_eta(s, s->Le[1], s->Le[2]);
    }
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        int q = IX(i, j);
        dn[q] += (s->nu2) * (Dt)*s->Le[0][q];
        dn[q] += (s->nu4) * (Dt)*s->Le[1][q];
        dn[q] += (s->nu6) * (Dt)*s->Le[2][q];
      }
  }
  adams_bashforth(s, s->detaAB, dn, s->deta[1], s->deta[2]);
  /* do_eta_geofactor (calc.c:403-422), after AB */
  for (int j = 1; j <= ny; j++) {
    double g = Dt * s->sinc[j + 1] / s->rzc[j + 1];
    for (int i = 1; i <= nx; i++)
      s->detaAB[IX(i, j)] -= (g * HH(i, j) * 0.5 * (VW(i, j) + VW(i, j - 1)));
  }
  rotate(s->deta);
  add_interior(s, eta, s->detaAB);
  halo(s, eta);

  /* momentum (core.c:212-280) */
  SCHEME_SWITCH(adv_u_s, s, s->duadv);
  SCHEME_SWITCH(adv_v_s, s, s->dvadv);
  for (int j = 1; j <= ny; j++) {
    double ge = R(T_GE, j), gn = R(T_GN, j), dxc = R(T_DXC, j), dyc1 = R(T_DYC, j + 1);
    for (int i = 1; i <= nx; i++) {
      s->dupres[IX(i, j)] = -ge * Dt * (eta[IX(i + 1, j)] - eta[IX(i, j)]) / dxc;
      s->dvpres[IX(i, j)] = -gn * Dt * (eta[IX(i, j + 1)] - eta[IX(i, j)]) / dyc1;
    }
  }
  double *dun = s->du[0], *dvn = s->dv[0];
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      int q = IX(i, j);
      dun[q] = s->duadv[q] + s->dupres[q];
      dvn[q] = s->dvadv[q] + s->dvpres[q];
    }
  /* dissipation_effect (calc.c:357-400), polar 0 */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      int q = IX(i, j);
      dun[q] -= u[q] * s->sigma * Dt;
      dvn[q] -= v[q] * s->sigma * Dt;
    }
  if (s->nu2 != 0 || s->nu4 != 0 || s->nu6 != 0) {
    for (int q = 0; q < 6; q++) memset(s->L[q], 0, sizeof(double) * (size_t)s->S);
    lap_vels(s, u, v, s->L[0], s->L[1]);
    if (s->nu4 != 0 || s->nu6 != 0) {
      lap_vels(s, s->L[0], s->L[1], s->L[2], s->L[3]);
      if (s->nu6 != 0) lap_vels(s, s->L[2], s->L[3], s->L[4], s->L[5]);
    }
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        int q = IX(i, j);
        dun[q] += (s->nu2) * (Dt)*s->L[0][q];
        dun[q] += (s->nu4) * (Dt)*s->L[2][q];
        dun[q] += (s->nu6) * (Dt)*s->L[4][q];
        dvn[q] += (s->nu2) * (Dt)*s->L[1][q];
        dvn[q] += (s->nu4) * (Dt)*s->L[3][q];
        dvn[q] += (s->nu6) * (Dt)*s->L[5][q];
      }
  }
  adams_bashforth(s, s->duAB, dun, s->du[1], s->du[2]);
  adams_bashforth(s, s->dvAB, dvn, s->dv[1], s->dv[2]);
  rotate(s->du);
  rotate(s->dv);

  /* semi-implicit Coriolis, in place, u then v (calc.c:542-598) */
  for (int j = 1; j <= ny; j++) {
    double fe = R(T_FE, j), sc = s->sinc[j + 1], rz = s->rzc[j + 1];
    for (int i = 1; i <= nx; i++) {
      int q = IX(i, j);
      double semi = 0.25 * (v[IX(i, j)] + v[IX(i + 1, j)] + v[IX(i, j - 1)] + v[IX(i + 1, j - 1)]);
      double al = Dt * fe + (Dt * u[q] * sc) / rz;
      double be = 0.25 * al * al;
      u[q] = (u[q] + s->duAB[q] - be * u[q] + al * semi) / (1.0 + be);
    }
  }
  for (int j = 1; j <= ny; j++) {
    double fn = R(T_FN, j), sn = s->sinn[j + 1], rz = s->rzn[j + 1];
    for (int i = 1; i <= nx; i++) {
      int q = IX(i, j);
      double semi = 0.25 * (u[IX(i - 1, j + 1)] + u[IX(i, j + 1)] + u[IX(i, j)] + u[IX(i - 1, j)]);
      double al = Dt * fn + (Dt * semi * sn) / rz;
      double be = 0.25 * al * al;
      v[q] = (v[q] + s->dvAB[q] - be * v[q] - al * semi) / (1.0 + be);
    }
  }
  /* core.c:288-307 (no perturbations; the tracer/eta halo refresh is idempotent) */
  halo(s, u);
  halo(s, v);
  halo(s, s->f[F_TR]);
  halo(s, eta);
  channel(s);
  (void)hb; (void)wx; (void)wy; (void)depth;
}

int sw2o_step(sw2o *s, int nsteps, int *bad_step) {
  for (int n = 0; n < nsteps; n++) {
    if (s->p.Dt > cfl_dt(s)) { if (bad_step) *bad_step = n; return 1; }
    one_step(s);
    s->k++;
    if (stats_bad(s, s->f[F_TR]) || stats_bad(s, s->f[F_ETA]) || stats_bad(s, s->f[F_U]) ||
        stats_bad(s, s->f[F_V])) {
      if (bad_step) *bad_step = n;
      return 2;
    }
  }
  return 0;
}

/* calc_energy_balance (energy.c:25-55), sequential sums in forall order */
void sw2o_energy(const sw2o *s, double *ke, double *ape, double *mass) {
  const int W = s->W;
  const double *eta = s->f[F_ETA], *u = s->f[F_U], *v = s->f[F_V], *wx = s->f[F_WX], *wy = s->f[F_WY],
               *hb = s->f[F_HB];
  const double depth = s->p.depth;
  double k = 0, a = 0, m = 0;
  for (int j = 1; j <= s->ny; j++)
    for (int i = 1; i <= s->nx; i++) {
      double uc = 0.5 * (UW(i, j) + UW(i - 1, j));
      double vc = 0.5 * (VW(i, j) + VW(i, j - 1));
      double surf = R(T_DXC, j) * R(T_DYC, j);
      double w0 = wx[IX(i, j)], w1 = wy[IX(i, j)];
      k += 0.5 * HH(i, j) * (uc * uc + vc * vc) * surf - 0.5 * ((w0 * w0) + (w1 * w1)) * surf;
      a += 0.5 * R(T_GC, j) * (HH(i, j) * HH(i, j)) * surf - 0.5 * R(T_GC, j) * (depth * depth) * surf;
      m += HH(i, j) * surf;
    }
  *ke = k;
  *ape = a;
  *mass = m;
}
