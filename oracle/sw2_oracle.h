/*
 * CPU oracle for the SW2 shallow-water step (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of the reference's per-step hot path (core.c:134-338
 * with calc.c, laplacian.c, energy.c and the single-rank halo update of
 * sppde/sppde_hupdate.c:274-363). It exists to check the CUDA implementation:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. Nothing in the product links or calls it.
 *
 * Pinning: the restatement is checked bit-for-bit against frames written by
 * the reference itself (built from its own sources by oracle/Makefile into
 * oracle/_ref, with a one-rank MPI stand-in and zeroed allocations) on the
 * committed fixtures in tests/golden/, generated by tests/golden/make_golden.py.
 *
 * Field layout is the reference's (sppde/sppde.h:131-142): every field is a
 * padded (nx+4) x (ny+4) array of doubles, halo width 2, x (longitude)
 * fastest; cell (i,j), i in [-1,nx+2], j in [-1,ny+2], lives at
 * (i+1) + (j+1)*(nx+4).
 */
#ifndef SW2_ORACLE_H
#define SW2_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny;
  int sch;                       /* limiter index 0..9 (calc.c:262-273) */
  double lon0, lon1, lat0, lat1; /* degrees, as in the .sw file */
  double Omega, rE, rP, gE, depth;
  double Dt, courant;
  double tau;                    /* Tau: sigma = 0 when tau > 1e10 (init.c:110-114) */
  double tracer_dis;
  double hypernu[3];             /* as entered (nu4 is negated internally, init.c:117-122) */
  int lape_eta;                  /* 1: laplacian_eta takes eta as its source; the reference
                                    passes u (calc.c:332), which is 0 here */
} sw2o_params;

typedef struct sw2o sw2o;

sw2o *sw2o_create(const sw2o_params *p);
void sw2o_destroy(sw2o *s);

/* Padded field sizes and pointers (eta, u, v, tracer, windx, windy, hB). */
int sw2o_padded_size(const sw2o *s);
double *sw2o_field(sw2o *s, int which);

/* Frame-load semantics (io.c:115-171, sppde_binary_files.c:147-180): copy the
 * interior of the given padded arrays and refresh all halos by the single-rank
 * wrap. Winds and hB are taken verbatim (all cells). Resets the AB index. */
void sw2o_load(sw2o *s, const double *eta, const double *u, const double *v, const double *tracer,
               const double *windx, const double *windy, const double *hB);
/* Raw semantics: every padded cell of every field is taken verbatim. */
void sw2o_load_raw(sw2o *s, const double *eta, const double *u, const double *v, const double *tracer,
                   const double *windx, const double *windy, const double *hB);

/* Advance nsteps. Returns 0, or 1 if the CFL check (core.c:156-158) failed,
 * 2 if the field range check (core.c:309-312) failed; *bad_step gets the step. */
int sw2o_step(sw2o *s, int nsteps, int *bad_step);
void sw2o_reset_ab(sw2o *s);

/* Energy exactly as energy.c:25-55 (sequential sums), plus mass = sum H*DXC*DYC. */
void sw2o_energy(const sw2o *s, double *ke, double *ape, double *mass);

/* Per-row geometry tables (ny+4 entries, row j at index j+1):
 * 0 dxe 1 dxc 2 dxv 3 dyn 4 dyc 5 dyv 6 ge 7 gn 8 gc 9 fe 10 fn */
const double *sw2o_row_table(const sw2o *s, int which);

/* Single-rank halo update of any padded field (sppde_hupdate.c:274-342). */
void sw2o_halo_update(int nx, int ny, double *x);

/* Threads used by sw2o_step (1 unless built with OpenMP). */
int sw2o_threads(void);

#ifdef __cplusplus
}
#endif
#endif
