/*
 * sw2g-run: runs an SW2 case file on the GPU step, as the reference's
 * executable runs it on one rank:
 *
 *     sw2g-run [--fp32] [--quiet] [--checkpoint] [--resume F] [--device-forcing] NPX NPY CASE OUTDIR
 *
 * (NPX = NPY = 1). --device-forcing evaluates the Gaussian injections on the
 * GPU (sw2g_add_gaussian: results within rounding of the reference's); by
 * default the host evaluates them with the reference's expressions and libm
 * and only the cells inside each radius cross to the GPU (bit for bit).
 * --timing prints the time loop's step count and wall time on stderr
 * ("LOOP n steps t s"). --checkpoint writes, next to each frame, an exact-restart
 * checkpoint (full padded state, Adams-Bashforth histories and index);
 * --resume F continues from the checkpoint of frame F bit for bit as the
 * uninterrupted run would (the reference's LoadFrom restarts with an Euler
 * step from a frame, and departs from it).
 *
 * reads CASE.sw (swcase.c), builds the initial fields of initialize() and
 * loop() (init.c:48-237, core.c:88-131: zero state, zonal wind from the
 * table, the forcing at t0, LoadFrom or frame 0), then runs the time loop of
 * core.c:131-338 with the step on the GPU (include/sw2g.h) and, after each
 * step, the reference's forcing (swforce.c), frames every SaveEvery steps
 * (MAGICSW2, io.c:27-58) and "ENERGY t ke ape ke+ape" lines every IteInfo
 * steps (energy.c:21-23).
 *
 * Differences from the reference: energy sums are compensated (the printed
 * digits agree); the range check of a step runs before that step's forcing
 * (the reference checks after it); a flow-rate ramp that covers none of its
 * three phases injects nothing (the reference leaves the rate unset).
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include "sw2g.h"
#include "swcase.h"
#include "swforce.h"

#define MAGIC_SW1 27
#define MAGIC_SW2 28
#define MAGIC_FIELD 15

static const char *base_name(const char *p) {
  const char *s = strrchr(p, '/');
  return s ? s + 1 : p;
}

/* save_binary_sw (io.c:27-58): the reference writes the gathered interior of
 * each field with zero halos (sppde_binary_files.c:36-60); so does this. */
static int write_frame(const char *outdir, const char *bname, int frame, int nstep, double t, int nx, int ny,
                       double *const f[5]) {
  for (int k = 0; k < 5; k++)
    for (int j = -1; j <= ny + 2; j++)
      for (int i = -1; i <= nx + 2; i++)
        if (i < 1 || i > nx || j < 1 || j > ny) f[k][(size_t)(i + 1) + (size_t)(j + 1) * (nx + 4)] = 0.0;
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.%04d.bin", outdir, base_name(bname), frame);
  FILE *fo = fopen(path, "wb");
  if (!fo) {
    fprintf(stderr, "sw2g-run: cannot write %s\n", path);
    return -1;
  }
  const int magic = MAGIC_SW2, fm = MAGIC_FIELD;
  const size_t S = (size_t)(nx + 4) * (ny + 4);
  int ok = fwrite(&magic, sizeof(int), 1, fo) == 1 && fwrite(&nstep, sizeof(int), 1, fo) == 1 &&
           fwrite(&t, sizeof(double), 1, fo) == 1 && fwrite(&nx, sizeof(int), 1, fo) == 1 &&
           fwrite(&ny, sizeof(int), 1, fo) == 1;
  for (int k = 0; k < 5 && ok; k++)
    ok = fwrite(&fm, sizeof(int), 1, fo) == 1 && fwrite(f[k], sizeof(double), S, fo) == S;
  fclose(fo);
  if (!ok) fprintf(stderr, "sw2g-run: short write on %s\n", path);
  return ok ? 0 : -1;
}

/* Frames are written by a background thread while the GPU steps on: two sets
 * of host fields alternate, the step loop fills one while the writer drains
 * the other, and waits only when the writer is still busy with the set it
 * needs. */
typedef struct {
  pthread_t th;
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int started, pending, quit, failed;
  const char *outdir, *bname;
  int frame, nstep, nx, ny;
  double t;
  double *f[5];
} frame_writer;

static void *writer_main(void *arg) {
  frame_writer *w = (frame_writer *)arg;
  pthread_mutex_lock(&w->mu);
  for (;;) {
    while (!w->pending && !w->quit) pthread_cond_wait(&w->cv, &w->mu);
    if (!w->pending && w->quit) break;
    pthread_mutex_unlock(&w->mu);
    const int rc = write_frame(w->outdir, w->bname, w->frame, w->nstep, w->t, w->nx, w->ny, w->f);
    pthread_mutex_lock(&w->mu);
    if (rc) w->failed = 1;
    w->pending = 0;
    pthread_cond_broadcast(&w->cv);
  }
  pthread_mutex_unlock(&w->mu);
  return NULL;
}

static int writer_start(frame_writer *w) {
  memset(w, 0, sizeof *w);
  pthread_mutex_init(&w->mu, NULL);
  pthread_cond_init(&w->cv, NULL);
  if (pthread_create(&w->th, NULL, writer_main, w)) return -1;
  w->started = 1;
  return 0;
}

/* Waits until the writer is idle; returns -1 if a write failed. */
static int writer_wait(frame_writer *w) {
  pthread_mutex_lock(&w->mu);
  while (w->pending) pthread_cond_wait(&w->cv, &w->mu);
  const int failed = w->failed;
  pthread_mutex_unlock(&w->mu);
  return failed ? -1 : 0;
}

static int writer_submit(frame_writer *w, const char *outdir, const char *bname, int frame, int nstep, double t,
                         int nx, int ny, double *const f[5]) {
  if (writer_wait(w)) return -1;
  pthread_mutex_lock(&w->mu);
  w->outdir = outdir;
  w->bname = bname;
  w->frame = frame;
  w->nstep = nstep;
  w->t = t;
  w->nx = nx;
  w->ny = ny;
  for (int k = 0; k < 5; k++) w->f[k] = f[k];
  w->pending = 1;
  pthread_cond_broadcast(&w->cv);
  pthread_mutex_unlock(&w->mu);
  return 0;
}

static int writer_stop(frame_writer *w) {
  if (!w->started) return 0;
  const int rc = writer_wait(w);
  pthread_mutex_lock(&w->mu);
  w->quit = 1;
  pthread_cond_broadcast(&w->cv);
  pthread_mutex_unlock(&w->mu);
  pthread_join(w->th, NULL);
  pthread_mutex_destroy(&w->mu);
  pthread_cond_destroy(&w->cv);
  w->started = 0;
  return rc;
}

/* load_binary_sw (io.c:115-171): fields eta, u, v, tracer, perturbs (tracer
 * absent in MAGICSW1 frames); returns 1 if the file does not exist. */
static int read_frame(const char *outdir, const char *bname, int frame, int nx, int ny, int *nstep, double *t,
                      double *const f[5]) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.%04d.bin", outdir, base_name(bname), frame);
  FILE *fi = fopen(path, "rb");
  if (!fi) return 1;
  int magic = 0, nxr = 0, nyr = 0;
  int ok = fread(&magic, sizeof(int), 1, fi) == 1 && fread(nstep, sizeof(int), 1, fi) == 1 &&
           fread(t, sizeof(double), 1, fi) == 1 && fread(&nxr, sizeof(int), 1, fi) == 1 &&
           fread(&nyr, sizeof(int), 1, fi) == 1;
  if (!ok || (magic != MAGIC_SW1 && magic != MAGIC_SW2) || nxr != nx || nyr != ny) {
    fprintf(stderr, "sw2g-run: %s is not a frame of this grid\n", path);
    fclose(fi);
    return -1;
  }
  const size_t S = (size_t)(nx + 4) * (ny + 4);
  const int order2[5] = {0, 1, 2, 3, 4}, order1[4] = {0, 1, 2, 4};
  const int nf = (magic == MAGIC_SW2) ? 5 : 4;
  for (int k = 0; k < nf && ok; k++) {
    int fm = 0;
    ok = fread(&fm, sizeof(int), 1, fi) == 1 && fread(f[magic == MAGIC_SW2 ? order2[k] : order1[k]], sizeof(double), S, fi) == S;
  }
  if (magic == MAGIC_SW1) memset(f[3], 0, S * sizeof(double));
  fclose(fi);
  if (!ok) fprintf(stderr, "sw2g-run: %s is truncated\n", path);
  return ok ? 0 : -1;
}

/* Exact-restart checkpoint next to a frame: "<case>.NNNN.ckp" holds the int
 * 0x43325753 ("SW2C"), the step number, t, the length n of the library's
 * checkpoint buffer (sw2g_checkpoint_save) as a 64-bit count, and the buffer. */
#define MAGIC_CKP 0x43325753
static int write_checkpoint(const char *outdir, const char *bname, int frame, int nstep, double t, sw2g_ctx *g) {
  const size_t n = sw2g_checkpoint_doubles(g);
  double *buf = (double *)malloc(n * sizeof(double));
  if (!buf) {
    fprintf(stderr, "sw2g-run: out of host memory for the checkpoint\n");
    return -1;
  }
  const sw2g_status st = sw2g_checkpoint_save(g, buf, n);
  if (st != SW2G_OK) {
    fprintf(stderr, "sw2g-run: checkpoint: %s\n", sw2g_status_string(st));
    free(buf);
    return -1;
  }
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.%04d.ckp", outdir, base_name(bname), frame);
  FILE *fo = fopen(path, "wb");
  int ok = fo != NULL;
  const int magic = MAGIC_CKP;
  const unsigned long long nn = n;
  ok = ok && fwrite(&magic, sizeof(int), 1, fo) == 1 && fwrite(&nstep, sizeof(int), 1, fo) == 1 &&
       fwrite(&t, sizeof(double), 1, fo) == 1 && fwrite(&nn, sizeof nn, 1, fo) == 1 &&
       fwrite(buf, sizeof(double), n, fo) == n;
  if (fo) fclose(fo);
  free(buf);
  if (!ok) fprintf(stderr, "sw2g-run: cannot write %s\n", path);
  return ok ? 0 : -1;
}

static int read_checkpoint(const char *outdir, const char *bname, int frame, int *nstep, double *t, sw2g_ctx *g) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.%04d.ckp", outdir, base_name(bname), frame);
  FILE *fi = fopen(path, "rb");
  if (!fi) {
    fprintf(stderr, "sw2g-run: checkpoint %s not found\n", path);
    return -1;
  }
  const size_t n = sw2g_checkpoint_doubles(g);
  double *buf = (double *)malloc(n * sizeof(double));
  int magic = 0;
  unsigned long long nn = 0;
  int ok = buf && fread(&magic, sizeof(int), 1, fi) == 1 && magic == MAGIC_CKP &&
           fread(nstep, sizeof(int), 1, fi) == 1 && fread(t, sizeof(double), 1, fi) == 1 &&
           fread(&nn, sizeof nn, 1, fi) == 1 && nn == n && fread(buf, sizeof(double), n, fi) == n;
  fclose(fi);
  sw2g_status st = SW2G_OK;
  if (ok) st = sw2g_checkpoint_load(g, buf, n);
  free(buf);
  if (!ok || st != SW2G_OK) {
    fprintf(stderr, "sw2g-run: %s is not a checkpoint of this case\n", path);
    return -1;
  }
  return 0;
}

static int ck(sw2g_status st, const char *what) {
  if (st == SW2G_OK) return 0;
  fprintf(stderr, "sw2g-run: %s: %s\n", what, sw2g_status_string(st));
  return -1;
}

/* The cells of the PERTURBS field (w->perturbs) set to 1 since it was last
 * cleared, so that clearing it (core.c:94, 292) touches those cells only;
 * `all` when its content came from elsewhere (a loaded frame). */
typedef struct {
  int *idx;
  size_t n, cap;
  int all;
} marks;

static int marks_add(marks *m, const int *idx, int n) {
  if (m->n + (size_t)n > m->cap) {
    size_t cap = m->cap ? m->cap : 1024;
    while (cap < m->n + (size_t)n) cap *= 2;
    int *p = (int *)realloc(m->idx, cap * sizeof(int));
    if (!p) return -1;
    m->idx = p;
    m->cap = cap;
  }
  memcpy(m->idx + m->n, idx, (size_t)n * sizeof(int));
  m->n += (size_t)n;
  return 0;
}

static void perturbs_clear(swforce *w, marks *m) {
  if (m->all) memset(w->perturbs, 0, (size_t)(w->nx + 4) * (w->ny + 4) * sizeof(double));
  else
    for (size_t k = 0; k < m->n; k++) w->perturbs[m->idx[k]] = 0.0;
  m->n = 0;
  m->all = 0;
}

/* The forcing of the step that ends at time t (core.c:292-302, perturbs.c):
 * Gaussians, then vortices. During the run it is applied between
 * sw2g_step_open and sw2g_step_close, where the reference applies it (after
 * the velocity halos, before do_channel); at t0 it is followed by
 * sw2g_apply_channel (core.c:96-101). A Gaussian sends only the cells inside
 * its radius to the GPU (sw2g_set_cells, sw2g_add_cells). */
static int apply_forcing(const swcase *c, sw2g_ctx *g, swforce *w, marks *pm, double Dt, double t, int device,
                         int need_mask, char *err, size_t errlen) {
  perturbs_clear(w, pm);
  for (int k = 0; k < c->num_gaussians; k++) {
    if (device) {
      /* the field, the volume and its rescale evaluated on the GPU; the host
       * evaluates the cells inside the radius only for a frame's PERTURBS */
      swf_gplan p;
      const int prc = swforce_gaussian_plan(c, k, Dt, t, &p, err, errlen);
      if (prc < 0) return -1;
      if (prc == 1) continue;
      const sw2g_gaussian dg = {p.lon, p.lat, p.amp, p.sigma, p.radius, p.inject, p.volume, p.images};
      const sw2g_status st = sw2g_add_gaussian(g, &dg);
      if (st == SW2G_ERR_FORCING) {
        snprintf(err, errlen, "Gaussian %d: total injected volume is 0 or missed its target", k);
        return -1;
      }
      if (ck(st, "Gaussian")) return -1;
      if (need_mask) {
        double rf_unused = 0;
        if (swforce_gaussian(c, k, Dt, t, w, &rf_unused, err, errlen) < 0) return -1;
        if (marks_add(pm, w->cells, w->ncells)) {
          snprintf(err, errlen, "out of host memory");
          return -1;
        }
      }
      continue;
    }
    double rf = 0;
    const int rc = swforce_gaussian(c, k, Dt, t, w, &rf, err, errlen);
    if (rc < 0) return -1;
    if (rc == 1) continue;
    if (marks_add(pm, w->cells, w->ncells)) {
      snprintf(err, errlen, "out of host memory");
      return -1;
    }
    if (ck(sw2g_set_cells(g, 3, w->cells, w->cell_tracer, w->ncells), "tracer")) return -1;
    if (rf != 0.0 && ck(sw2g_add_cells(g, 0, w->cells, w->cell_pert, w->ncells, rf), "eta")) return -1;
  }
  for (int k = 0; k < c->num_vortices; k++) {
    if (!swforce_vortex_due(c, k, Dt, t)) continue;
    swforce_vortex(c, k, w);
    if (ck(sw2g_add_field(g, 0, w->deta, 1.0), "eta") || ck(sw2g_add_field(g, 1, w->du, 1.0), "u") ||
        ck(sw2g_add_field(g, 2, w->dv, 1.0), "v"))
      return -1;
  }
  return 0;
}

static int forcing_active(const swcase *c, double Dt, double t) {
  for (int k = 0; k < c->num_gaussians; k++) {
    const double *G = c->gaussians + (size_t)k * SWC_GAUSS_COLS;
    if (G[0] <= t && G[1] >= t) return 1;
  }
  for (int k = 0; k < c->num_vortices; k++)
    if (swforce_vortex_due(c, k, Dt, t)) return 1;
  return 0;
}

static int print_energy(sw2g_ctx *g, double t) {
  double ke, ape, mass;
  if (ck(sw2g_diag(g, &ke, &ape, &mass), "energy")) return -1;
  printf("ENERGY %e %e %e %e\n", t, ke, ape, ke + ape);
  fflush(stdout);
  return 0;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int sw2g_run_case(const char *bname, const char *outdir, int fp32, int quiet, int checkpoint, int resume,
                  int device_forcing, int timing) {
  char err[512] = {0}, path[4096];
  snprintf(path, sizeof path, "%s.sw", bname);
  swcase c;
  if (swcase_read(path, &c, err, sizeof err)) {
    fprintf(stderr, "sw2g-run: %s: %s\n", path, err);
    return 2;
  }
  int rc = 1;
  sw2g_ctx *g = NULL;
  swforce w = {0};
  marks pm = {0};
  double *f[5] = {NULL, NULL, NULL, NULL, NULL}, *windx = NULL, *windy = NULL, *zero = NULL;
  double *f2[5] = {NULL, NULL, NULL, NULL, NULL};
  frame_writer wr;
  memset(&wr, 0, sizeof wr);
  int set = 0;  /* the host frame set the loop fills next */
  if (c.polar != 0 && (c.num_gaussians || c.num_vortices)) {
    fprintf(stderr, "sw2g-run: forcing on a polar cap is not supported\n");
    goto done;
  }
  if (c.reftype != 0 && !quiet) fprintf(stderr, "sw2g-run: reftype %d: the comparison is not run\n", c.reftype);
  if (fp32 && (checkpoint || resume >= 0)) {
    fprintf(stderr, "sw2g-run: checkpoints are written and read by the FP64 step only\n");
    goto done;
  }
  mkdir(outdir, 0775);
  const int nx = c.nx, ny = c.ny;
  const size_t S = (size_t)(nx + 4) * (ny + 4);
  for (int k = 0; k < 5; k++) f[k] = (double *)calloc(S, sizeof(double));
  for (int k = 0; k < 5; k++) f2[k] = (double *)calloc(S, sizeof(double));
  if (!f2[0] || !f2[1] || !f2[2] || !f2[3] || !f2[4] || writer_start(&wr)) {
    fprintf(stderr, "sw2g-run: out of host memory\n");
    goto done;
  }
  windx = (double *)calloc(S, sizeof(double));
  zero = (double *)calloc(S, sizeof(double));
  if (!f[0] || !f[1] || !f[2] || !f[3] || !f[4] || !windx || !zero || swforce_init(&w, nx, ny)) {
    fprintf(stderr, "sw2g-run: out of host memory\n");
    goto done;
  }
  windy = (double *)calloc(S, sizeof(double));
  if (!windy || swforce_winds(&c, c.beta_sponge, windx, windy, err, sizeof err)) {
    fprintf(stderr, "sw2g-run: %s\n", err[0] ? err : "out of host memory");
    goto done;
  }
  sw2g_case sc;
  memset(&sc, 0, sizeof sc);
  sc.nx = nx;
  sc.ny = ny;
  sc.sch = c.sch;
  sc.lon0 = c.lon0;
  sc.lon1 = c.lon1;
  sc.lat0 = c.lat0;
  sc.lat1 = c.lat1;
  sc.Omega = c.Omega;
  sc.rE = c.rE;
  sc.rP = c.rP;
  sc.gE = c.gE;
  sc.depth = c.depth;
  sc.Dt = c.Dt;
  sc.courant = c.CFL;
  sc.tau = c.sigma_dis;
  sc.tracer_dis = c.tracer_dis;
  sc.hypernu[0] = c.nu2;
  sc.hypernu[1] = c.nu4;
  sc.hypernu[2] = c.nu6;
  sc.flags = SW2G_FLAG_RADIANS | SW2G_FLAG_SIGMA | (fp32 ? SW2G_FLAG_VANLEER_SAFE : 0u);
  sc.polar = c.polar;
  sc.beta_sponge = c.beta_sponge * ((4.0 * atan(1.0)) / 180.0);  /* init.c:155, radians like the angles */
  sc.sigma_sponge = c.sigma_sponge;
  if (ck(sw2g_create(&sc, fp32 ? SW2G_FP32 : SW2G_FP64, 0, &g), "create")) goto done;
  /* zero state, winds, zero bottom, all halos already wrapped (core.c:88-94) */
  if (ck(sw2g_upload(g, zero, zero, zero, zero, windx, windy, zero, SW2G_UPLOAD_RAW), "upload")) goto done;
  const double Dt = c.Dt;
  double t = c.t0;
  /* forcing at t0 and the wall fixes (core.c:96-101) */
  if (resume < 0) {
    if (apply_forcing(&c, g, &w, &pm, Dt, t, device_forcing, 1, err, sizeof err)) {
      if (err[0]) fprintf(stderr, "sw2g-run: %s\n", err);
      goto done;
    }
    if (ck(sw2g_apply_channel(g), "channel")) goto done;
  }
  int frame = 0, nstart = 0;
  if (resume >= 0) {  /* exact restart from this runner's own checkpoint */
    frame = resume;
    if (read_checkpoint(outdir, bname, frame, &nstart, &t, g)) goto done;
  } else if (c.loadFrom != 0) {  /* core.c:115-118 */
    frame = c.loadFrom;
    int ns = 0;
    const int lr = read_frame(outdir, bname, frame, nx, ny, &ns, &t, f);
    if (lr != 0) {
      if (lr == 1) fprintf(stderr, "sw2g-run: frame %d to be loaded not found\n", frame);
      goto done;
    }
    nstart = ns;
    memcpy(w.perturbs, f[4], S * sizeof(double));
    pm.all = 1;
    if (ck(sw2g_upload(g, f[0], f[1], f[2], f[3], windx, windy, zero, SW2G_UPLOAD_FRAME), "load")) goto done;
  } else {
    if (ck(sw2g_download(g, f[0], f[1], f[2], f[3]), "download")) goto done;
    memcpy(f[4], w.perturbs, S * sizeof(double));
    if (write_frame(outdir, bname, frame, 0, t, nx, ny, f)) goto done;
  }
  if (print_energy(g, t)) goto done;
  frame++;
  nstart++;
  if (!quiet)
    fprintf(stderr, "sw2g-run: %s %dx%d, steps %d..%d, Dt %g, %s%s\n", bname, nx, ny, nstart, c.N, Dt,
            fp32 ? "FP32 form" : "FP64", device_forcing ? ", Gaussians evaluated on the GPU" : "");
  const double loop_t0 = now_s();
  const int loop_n0 = nstart;
  for (int n = nstart; n <= c.N;) {
    /* steps without output or forcing are run in one call */
    int k = 1;
    double tk = t + Dt;
    while (n + k <= c.N && !(n + k - 1 == nstart || (n + k - 1) % c.IteInfo == 0) &&
           (n + k - 1) % c.saveEvery != 0 && !forcing_active(&c, Dt, tk)) {
      /* step n+k-1 ends without output and forcing: it can join the next */
      tk += Dt;
      k++;
    }
    /* the last step of the group takes its forcing between its two halves */
    const int forced = forcing_active(&c, Dt, tk);
    sw2g_status st = SW2G_OK;
    if (k > 1 || !forced) st = sw2g_step(g, forced ? k - 1 : k);
    if (st == SW2G_OK && forced) {
      st = sw2g_step_open(g);
      if (st == SW2G_OK) {
        /* the step ending at tk writes a frame: its PERTURBS are needed */
        const int frame_step = ((n + k - 1) % c.saveEvery == 0);
        if (apply_forcing(&c, g, &w, &pm, Dt, tk, device_forcing, frame_step, err, sizeof err)) {
          if (err[0]) fprintf(stderr, "sw2g-run: %s\n", err);
          goto done;
        }
        st = sw2g_step_close(g);
      }
    }
    if (st == SW2G_ERR_CFL || st == SW2G_ERR_NONFINITE || st == SW2G_ERR_FORCING) {
      /* error steps count from the last upload, which preceded step nstart */
      fprintf(stderr, "sw2g-run: %s at step %d\n",
              st == SW2G_ERR_CFL        ? "Dt exceeds the CFL bound"
              : st == SW2G_ERR_FORCING ? "a Gaussian's injected volume is 0 or missed its target"
                                       : "nonsense value detected",
              nstart + sw2g_error_step(g));
      rc = 3;
      goto done;
    }
    if (ck(st, "step")) goto done;
    for (int q = 0; q < k; q++) t += Dt;  /* core.c:145 */
    n += k;
    const int m = n - 1;  /* the step just finished */
    if (!forced) perturbs_clear(&w, &pm);  /* core.c:292 */
    if (m % c.saveEvery == 0) {  /* core.c:315-320 */
      /* the writer holds at most the other set: submitting it waited for this one */
      double *const *fs = set ? f2 : f;
      if (ck(sw2g_download(g, fs[0], fs[1], fs[2], fs[3]), "download")) goto done;
      memcpy(fs[4], w.perturbs, S * sizeof(double));
      if (writer_submit(&wr, outdir, bname, frame, m, t, nx, ny, fs)) goto done;
      set ^= 1;
      if (checkpoint && write_checkpoint(outdir, bname, frame, m, t, g)) goto done;
      frame++;
    }
    if (m == nstart || m % c.IteInfo == 0) {  /* core.c:136, 329-332 */
      if (print_energy(g, t)) goto done;
    }
  }
  if (timing) /* the time loop's wall time: steps, forcing, frames and ENERGY lines */
    fprintf(stderr, "LOOP %d steps %.6f s\n", c.N - loop_n0 + 1, now_s() - loop_t0);
  rc = 0;
done:
  if (writer_stop(&wr) && rc == 0) rc = 1;
  if (g) sw2g_destroy(g);
  swforce_free(&w);
  free(pm.idx);
  for (int k = 0; k < 5; k++) free(f[k]);
  for (int k = 0; k < 5; k++) free(f2[k]);
  free(windx);
  free(windy);
  free(zero);
  swcase_free(&c);
  return rc;
}
