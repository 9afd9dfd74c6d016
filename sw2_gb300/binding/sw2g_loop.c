/*
 * The reference's time loop on the GPU: a replacement of loop() (core.c:22,
 * declared in sw.h:223) for a build of the reference that links libsw2g.so.
 *
 * The reference's core.c is compiled unchanged with -Dloop=loop_cpu, so its
 * own loop stays available as loop_cpu(); main() (main/Main.c:77) then calls
 * this loop(). It keeps the reference's set-up, frames and ENERGY lines by
 * calling the reference's own functions for them (core.c:83-138), and moves
 * the body of every step (core.c:134-338) to the GPU through include/sw2g.h.
 * Steps that carry forcing are split where the reference applies it
 * (sw2g_step_open / sw2g_step_close around add_Gaussians and add_vortices,
 * core.c:292-303): the state comes back to the reference's arrays, its own
 * forcing routines run on them, and the state goes back with the history kept.
 *
 * Runs on the CPU loop instead: several ranks (the library reproduces the
 * single-rank halos), polar caps (the sw struct no longer holds the case's
 * radii after init_polar_region, init.c:273-276), or SW2G_CPU set in the
 * environment.
 *
 * Build (oracle/Makefile, target binding): the reference's sources where they
 * lie plus this file, -I include/, linked with -lsw2g.
 */
#include <stdlib.h>

#include "mpi.h"
#include "sppde.h"
#include "sw.h"
#include "sw2g.h"

void loop_cpu(char *bname, char *output_folder, sw *SW);

static void gpu_ok(sw2g_status st, const char *what) {
  if (st != SW2G_OK) CRASH("%s: %s", what, sw2g_status_string(st));
}

/* Whether the forcing of the step ending at t does anything (perturbs.c:63, 388). */
static int forced_at(const sw *SW, double Dt, double t) {
  for (int g = 0; g < SW->num_Gaussians; g++) {
    const double *G = SW->Gaussians + g * N_COLS_GAUSS;
    if (G[0] <= t && G[1] >= t) return 1;
  }
  for (int k = 0; k < SW->num_vortices; k++) {
    const double t0 = SW->vortices[k * N_COLS_VORTICES];
    if (t0 < t && t0 >= t - Dt) return 1;
  }
  return 0;
}

void loop(char *bname, char *output_folder, sw *SW) {
  if (quants() != 1 || SW->polar != 0 || getenv("SW2G_CPU")) {
    loop_cpu(bname, output_folder, SW);
    return;
  }
  const double Dt = SW->Dt;
  double t = SW->t0, ke, ape;

  /* set-up of the reference's loop (core.c:83-138), by its own routines */
  halo_update(SW->tracer, SW->M);
  halo_update(SW->u, SW->M);
  halo_update(SW->v, SW->M);
  halo_update(SW->eta, SW->M);
  halo_update(SW->hB, SW->M);
  setzero_scaf(SW->perturbs, SW->M);
  add_Gaussians(Dt, t, SW);
  add_vortices(Dt, t, SW);
  halo_update(SW->tracer, SW->M);
  halo_update(SW->eta, SW->M);
  do_channel(SW);
  int frame = 0, nstart = 0;
  if (SW->loadFrom != 0) {
    frame = SW->loadFrom;
    if (load_binary_sw(frame, &nstart, &t, bname, output_folder, SW)) CRASH("File to be loaded not found");
  } else {
    save_binary_sw(frame, 0, t, bname, output_folder, SW);
  }
  calc_energy_balance(&ke, &ape, SW);
  print_energy(t, ke, ape);
  frame++;
  nstart++;

  /* the case as initialize() left it: angles in radians, sigma_dis, nu4 negated */
  sw2g_case c = {0};
  c.nx = SW->nx;
  c.ny = SW->ny;
  c.sch = SW->sch;
  c.lon0 = SW->lon0;
  c.lon1 = SW->lon1;
  c.lat0 = SW->lat0;
  c.lat1 = SW->lat1;
  c.Omega = SW->Omega;
  c.rE = SW->rE;
  c.rP = SW->rP;
  c.gE = SW->gE;
  c.depth = SW->depth;
  c.Dt = Dt;
  c.courant = SW->Courant_max;
  c.tau = SW->sigma_dis;
  c.tracer_dis = SW->tracer_dis;
  c.hypernu[0] = SW->nu2;
  c.hypernu[1] = -SW->nu4;
  c.hypernu[2] = SW->nu6;
  c.flags = SW2G_FLAG_RADIANS | SW2G_FLAG_SIGMA;
  sw2g_ctx *g = NULL;
  gpu_ok(sw2g_create(&c, SW2G_FP64, 0, &g), "sw2g_create");
  gpu_ok(sw2g_upload(g, SW->eta, SW->u, SW->v, SW->tracer, SW->windx, SW->windy, SW->hB, SW2G_UPLOAD_RAW),
        "sw2g_upload");

  for (int n = nstart; n <= SW->N;) {
    /* steps without output or forcing run in one call; the last step of a
     * group is the one that prints, saves or is forced */
    int k = 1;
    double tk = t + Dt;
    while (n + k <= SW->N && !(n + k - 1 == nstart || (n + k - 1) % SW->IteInfo == 0) &&
           (n + k - 1) % SW->saveEvery != 0 && !forced_at(SW, Dt, tk)) {
      tk += Dt;
      k++;
    }
    const int forced = forced_at(SW, Dt, tk);
    sw2g_status st = SW2G_OK;
    if (k > 1 || !forced) st = sw2g_step(g, forced ? k - 1 : k);
    if (st == SW2G_OK && forced) {
      gpu_ok(sw2g_step_open(g), "sw2g_step_open");
      gpu_ok(sw2g_download(g, SW->eta, SW->u, SW->v, SW->tracer), "sw2g_download");
      setzero_scaf(SW->perturbs, SW->M);  /* core.c:292-294 */
      add_Gaussians(Dt, tk, SW);
      add_vortices(Dt, tk, SW);
      halo_update(SW->tracer, SW->M);
      halo_update(SW->eta, SW->M);
      gpu_ok(sw2g_upload(g, SW->eta, SW->u, SW->v, SW->tracer, NULL, NULL, NULL, SW2G_UPLOAD_CONTINUE),
            "sw2g_upload");
      st = sw2g_step_close(g);
    } else if (!forced) {
      setzero_scaf(SW->perturbs, SW->M);
    }
    if (st == SW2G_ERR_CFL || st == SW2G_ERR_NONFINITE)
      CRASH("step %d: %s", nstart + sw2g_error_step(g), sw2g_status_string(st));
    gpu_ok(st, "sw2g_step");
    for (int q = 0; q < k; q++) t += Dt; /* core.c:145 */
    n += k;
    const int m = n - 1;
    if (m % SW->saveEvery == 0) { /* core.c:315-320 */
      gpu_ok(sw2g_download(g, SW->eta, SW->u, SW->v, SW->tracer), "sw2g_download");
      save_binary_sw(frame, m, t, bname, output_folder, SW);
      frame++;
    }
    if (m == nstart || m % SW->IteInfo == 0) { /* core.c:136, 328-331 */
      double mass;
      gpu_ok(sw2g_diag(g, &ke, &ape, &mass), "sw2g_diag");
      print_energy(t, ke, ape);
    }
  }
  gpu_ok(sw2g_download(g, SW->eta, SW->u, SW->v, SW->tracer), "sw2g_download");
  sw2g_destroy(g);
  pprintf("Core loop ended.\n");
}
