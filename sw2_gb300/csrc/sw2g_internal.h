// Internal declarations shared by the sw2g translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "sw2g.h"

namespace sw2g {

// Per-row tables (one value per latitude row j = -1..ny+2, stored at j+1).
// The first group restates the reference's metric and physics fields, which
// for polar 0 depend on j only (coords.c:35-96, init.c:279-297, sw.h:174-193);
// the second holds per-row subexpressions that the reference evaluates per
// cell with identical operands, precomputed here with the same operations.
enum Row {
  R_DXE, R_DXC, R_DXV, R_DYN, R_DYC, R_DYV,
  R_GE, R_GN, R_GC, R_FE, R_FN,
  R_RMC, R_RZC, R_RMN, R_RZN, R_SINC, R_SINN,
  R_KX,    // rM(latc)/rZ(latc)            laplacian.c:121
  R_KY,    // rZ(latn)/rM(latn)            laplacian.c:122
  R_KC,    // 1.0/(rM(latc)*rZ(latc))      laplacian.c:126
  R_GEO,   // Dt*sin(latc)/rZ(latc)        calc.c:419
  R_IDXE, R_IDXC, R_IDXV, R_IDYN, R_IDYC,  // 1.0/x   laplacian.c:60-87
  R_DTFE,  // Dt*FE                        calc.c:563
  R_DTFN,  // Dt*FN                        calc.c:592
  R_MGEDT, // -GE*Dt                       calc.c:517
  R_MGNDT, // -GN*Dt                       calc.c:538
  R_DXE2,  // DXE+DXE                      calc.c:197
  R_DYNS,  // DYN(j)+DYN(j+1)              calc.c:234
  R_SURF,  // DXC*DYC                      energy.c:40
  R_IDYV, R_IDXE2, R_IDYNS, R_IRZC, R_IRZN,  // 1.0/x of DYV, DXE2, DYNS, rZ(latc), rZ(latn): divisors of div_rcp
  R_NUM
};

// Internal limiter index: 0..9 as the reference, 10 = Van Leer made safe at r = -1.
constexpr int kVanLeerSafe = 10;

// Two-dimensional fields of a polar cap (padded, pitch W), index P_* * W*H:
// gravity at E, N and C points, Coriolis at E and N points (init.c:243-261),
// and the damping rates of h, tracer, u and v with the sponge
// (calc.c:102-111, 152-161, 374-394).
enum Polar { P_GE, P_GN, P_GC, P_FE, P_FN, P_SH, P_STR, P_SU, P_SV, P_NUM };

struct DevState {
  int nx, ny, W, H;  // W = nx+4 (row pitch), H = ny+4
  const double* rows;  // R_NUM * H
  double depth, Dt, sigma, sigma_tr, nu2, nu4, nu6;
  double nu2dt, nu4dt, nu6dt;  // (nu)*(Dt) as the reference forms it (calc.c:346-348)
  int plain;           // windx, windy and hB are +0.0 in every padded cell
  int lape_eta;        // laplacian_eta of eta instead of u (SW2G_FLAG_LAPE_ETA)
  int fk;              // rows per strip of the fast TVD bodies (set per launch)
  unsigned* strips;    // the fast bodies' strip queue: next strip, warps done (zero between launches)
  int polar;           // 0: band; +-1: polar cap, with the fields below
  const double* pf;    // P_NUM * W * H (polar only)
};

struct Ctx;

// Checks of a case's grid shared by every entry point that takes one: at least
// 3x3 cells, padded cell indices within 32 bits, positive radii, increasing
// bounds, latitudes strictly between the poles, known flags.
bool grid_ok(const sw2g_case* c);

// Host geometry (geometry.cpp): fills rows[R_NUM*H]; returns the at-rest CFL
// maxima used by compute_Dt when the flow is at rest (calc.c:715-725).
void build_rows(const sw2g_case& c, std::vector<double>& rows, double* rest_mx, double* rest_my);
// The fields of a polar cap (P_NUM x (nx+4)(ny+4)) and the at-rest CFL maxima
// computed with them.
void polar_fields(const sw2g_case& c, std::vector<double>& f, double* rest_mx, double* rest_my);
// Tables of the Gaussian forcing (perturbs.c:333-364, tools.c:104-119), with
// the reference's expressions: rows3[3*j..] = {sin, cos of the planetocentric
// latitude of latc(j), DXC(j)*DYC(j)} and pl[j] that latitude, j = 0..ny+1;
// lonc[i] = lonc(i), i = 0..nx+1. forcing_pclat: the planetocentric latitude
// of a planetographic one (sw.h:170).
void forcing_tables(const sw2g_case& c, std::vector<double>& rows3, std::vector<double>& pl,
                    std::vector<double>& lonc);
double forcing_pclat(const sw2g_case& c, double lat);
// lon1 - lon0 in radians (the shift of a Gaussian's periodic images, perturbs.c:250-251).
double forcing_lon_span(const sw2g_case& c);

// A Gaussian injection on the device (forcing.cu): rows j0 .. j0+nrows-1
// (1 <= j0, j0+nrows-1 <= ny) hold every cell that can be inside the radius.
struct GaussJob {
  int nx, j0, nrows, nimg;
  double lon[3];           // the centre and its periodic images, in evaluation order
  double sp, cp;           // sin, cos of the centre's planetocentric latitude
  double R;                // mean radius (rE + rP) / 2
  double amp, den;         // peak before the rescale; 2 * sigma^2
  double radius, inject, volume;
};
// Device scratch of the injections: per-cell field, tracer value and mask
// (padded), partial volumes (one per block: ceil(nx/128) * ny), the rescale
// factor and the error word (nonzero after a failed volume check).
struct GaussScratch {
  double* gp = nullptr;
  double* gt = nullptr;
  unsigned char* gm = nullptr;
  double* part = nullptr;
  double* rf = nullptr;
  int* err = nullptr;
};
void gauss_inject(const GaussJob& g, const double* rows, const double* lonc, GaussScratch& sc, double* eta,
                  double* tracer, cudaStream_t st);

// FP64 reference-exact step (step_fp64.cu).
struct Fp64Buffers {
  double* f[7];  // eta u v tracer windx windy hB (padded)
  double* deta[3]; double* du[3]; double* dv[3]; double* dtr[3];
  double* detaAB; double* duAB; double* dvAB; double* dtrAB;
  double* duadv; double* dvadv;
  double* Le[3]; double* L[6];
  double* psi; double* xi; double* ze; double* di;
};

struct StepChecks {
  unsigned long long* cfl;  // 2 per step: bit patterns of max|u|/dx, max|v|/dy
  int* bad;                 // 1 per step: range check failed
};

// Named device timers (the role of the reference's cr_start/cr_end channels,
// sppde_cr.c:38-217): while enabled, every tagged launch is bracketed by a
// pair of CUDA events on the launching stream; collect() (after the stream has
// been synchronised) adds the elapsed times per tag.
class Timers {
 public:
  struct Entry {
    const char* name;
    long long launches;
    double ms;
  };
  bool on = false;
  void begin(const char* tag, cudaStream_t st);
  void end(cudaStream_t st);
  void collect();
  void reset();
  void release();
  const std::vector<Entry>& entries() const { return entries_; }

 private:
  struct Pending {
    int entry;
    cudaEvent_t a, b;
  };
  cudaEvent_t take();
  std::vector<cudaEvent_t> free_;
  std::vector<Pending> pending_;
  std::vector<Entry> entries_;
  int open_ = -1;
  cudaEvent_t open_ev_ = nullptr;
};

// Parts of one step: the head runs through the velocity halos (core.c:134-290),
// the tail the wall fixes and range checks (core.c:303-312); the reference's
// forcing goes between them.
constexpr int STEP_HEAD = 1, STEP_TAIL = 2, STEP_FULL = 3;
// Events within a step, for callers that overlap host copies with it: the
// stream waits for v_in before the first kernel that reads v (the eta
// Laplacians, which read only u, come first), for eta_in before the first
// kernel that reads eta (the advection of u and v, which do not read it, come
// first), records eta_out as soon as eta holds the step's result, and u_out
// once the interior of u does (its halo columns and wall rows are still
// rewritten at the end of the step). Null events are skipped.
struct StepHooks {
  cudaEvent_t v_in = nullptr;
  cudaEvent_t eta_in = nullptr;
  cudaEvent_t eta_out = nullptr;
  cudaEvent_t u_out = nullptr;
};
int fp64_step(const DevState& s, Fp64Buffers& b, int sch, int k, bool tracer, StepChecks chk, int step_slot,
              cudaStream_t st, Timers* tm, int parts = STEP_FULL, StepHooks hk = StepHooks{});
// Forcing between steps on FP64 fields (interior cells, then the halo wrap;
// fp64_channel is do_channel on u, v and the winds).
void fp64_add_scaled(double* f, const double* d, double scale, int nx, int ny, cudaStream_t st);
void fp64_set_where(double* f, const double* val, const unsigned char* mask, int nx, int ny, cudaStream_t st);
void fp64_channel(double* u, double* v, double* wx, double* wy, int nx, int ny, cudaStream_t st);
// The reference's range check (check_stats_scaf, sppde_core.c:386-395) of n
// padded fields of the grid; sets *bad (device) to 1 when one fails.
void fp64_range(const DevState& s, const double* const* fields, int n, int* bad, cudaStream_t st);
// f[cells[k]] = values[k] (values NULL: 0.0) for k < n; the cells are distinct.
void fp64_scatter_cells(double* f, const int* cells, const double* values, int n, cudaStream_t st);
// Compares the step's division by a row metric (div_rcp) with IEEE division
// on `samples` random numerators per divisor; returns the mismatch count in
// *bad (device pointer) once the stream is done.
void fp64_check_division(const double* d_div, int n, long long samples, unsigned long long seed,
                         unsigned long long* bad, cudaStream_t st);
// Compares the step's integer-pipe additions (sadd, ssub) with the FP64
// unit's on `samples` operand pairs; mismatch count in *bad (device pointer).
void fp64_check_add(long long samples, unsigned long long seed, unsigned long long* bad, cudaStream_t st);
// FP32 precision form (step_fp32.cu). Per-row FP32 constants, index j+1.
enum Q32 {
  Q_KXE, Q_KYN, Q_KXC, Q_KYV, Q_KXV, Q_KYC,  // Dt/DXE, Dt/DYN, Dt/DXC, Dt/DYV, Dt/DXV, Dt/DYC
  Q_K2XE,   // Dt/(DXE+DXE)
  Q_KDYNS,  // Dt/(DYN(j)+DYN(j+1))
  Q_GEX,    // -GE*Dt/DXC
  Q_GNY,    // -GN*Dt/DYC(j+1)
  Q_GEO,    // Dt*sin(latc)/rZ(latc)
  Q_CV,     // Dt*sin(latn)/rZ(latn)
  Q_DTFE, Q_DTFN,
  Q_HB,     // reference height of the row: eta_ref(j) + depth
  Q_EREF,   // eta_ref(j)
  Q_DHBM2, Q_DHBM1, Q_DHBP1, Q_DHBP2,  // eta_ref(j+k) - eta_ref(j), k = -2,-1,1,2
  Q_IDXV, Q_IDYC, Q_DXC, Q_IDXE, Q_IDYN, Q_DXV, Q_IDXC,
  Q_NUM
};

// Tracer of an FP32-form member (device-resident, one per context with an
// active tracer): FP64 state and FP32 shadow (double-buffered like eta), the
// three-slot history ring of its tendency, and 2*Dt*TracerDis.
struct TracerDesc {
  double* tr[2];
  float* ts[2];
  float* h[3];
  float sig2dt;
};

// Per-cell FP32 fields of a polar cap in the FP32 form (layout of the FP32
// arrays, one after another): -GE*Dt/DXC and -GN*Dt/DYC(j+1) of the pressure
// terms (calc.c:517, 538), Dt*FE and Dt*FN of the Coriolis updates
// (calc.c:563, 592), and the damping with the sponge (calc.c:102-111,
// 152-161, 374-394): 2*Dt*sigma of height and tracer, sigma*Dt of u and v.
enum PolarQ { PQ_GEX, PQ_GNY, PQ_DTFE, PQ_DTFN, PQ_SH2, PQ_SU, PQ_SV, PQ_STR2, PQ_NUM };

struct Fp32Ctx {
  int nx, ny, sch, extra;
  int polar = 0;             // 0 band, +-1 polar cap (single contexts only)
  const float* pf = nullptr;  // PQ_NUM fields of P*R floats (polar caps)
  int P, R;  // FP32 arrays: row pitch and rows (padded so tile windows stay in bounds)
  const float* q;
  float sig2dt, sigdt, nu2dt, nu4dt, nu6dt;
  const float* wx; const float* wy; const float* hb;
  // Test of the failure path (sw2g_test_tile_timeout): > 0 makes the tile
  // loads of the next steps also wait for a barrier phase that never
  // completes, giving up after that many tries; 0 in normal use.
  int tile_test = 0;
  // 1 while a step is run for sw2g_step_open: the step writes u and v with
  // the plain halo update only (core.c:287-288), leaving do_channel and the
  // range checks to sw2g_step_close, after the forcing (core.c:292-312).
  int open_step = 0;
};

struct Fp32Engine {
  double* eta[2] = {nullptr, nullptr};  // eta - eta_ref(j), double-buffered
  double* u[2] = {nullptr, nullptr};
  double* v[2] = {nullptr, nullptr};
  float* es[2] = {nullptr, nullptr};  // FP32 shadows of the state (pitch P)
  float* us[2] = {nullptr, nullptr};
  float* vs[2] = {nullptr, nullptr};
  int cur = 0;
  // Adams-Bashforth histories: a ring of three slots; the next step writes
  // slot w, step n-1 is in slot (w+2)%3 and step n-2 in slot (w+1)%3.
  float* heta[3] = {nullptr, nullptr, nullptr};
  float* hu[3] = {nullptr, nullptr, nullptr};
  float* hv[3] = {nullptr, nullptr, nullptr};
  int w = 0;
  float* Lu = nullptr; float* Lv = nullptr;
  float* LLu = nullptr; float* LLv = nullptr;  // second Laplacian level (only with nu6)
  // tracer (allocated when a nonzero tracer is uploaded; advected while active)
  double* tr[2] = {nullptr, nullptr};
  float* ts[2] = {nullptr, nullptr};
  float* htr[3] = {nullptr, nullptr, nullptr};
  TracerDesc* d_trd = nullptr;
  bool tracer = false;
  float* dup = nullptr; float* dvp = nullptr;
  unsigned* cfl = nullptr;  // 2 per step (float bits)
  int* bad = nullptr;       // 1 per step
  void* maps = nullptr;     // TM_NUM tensor maps (device memory) of the FP32 fields, see Fp32Map
  // host view after nsteps more steps: state buffer and history ring position
  void advance_host(long long nsteps);
};

// Tensor maps of a member's FP32 fields (rows of a strip, for the TMA
// engine), by field: the two buffers of the eta, u, v and tracer shadows, the
// Laplacian levels, the winds and the bottom height.
enum Fp32Map {
  TM_ES = 0, TM_US = 2, TM_VS = 4, TM_LU = 6, TM_LV = 7, TM_LLU = 8, TM_LLV = 9, TM_TS = 10,
  TM_WX = 12, TM_WY = 13, TM_HB = 14, TM_NUM = 15
};

// Steps whose checks are kept on the device before the host reads them back.
constexpr int kCheckSlots = 1024;
// Bits of a step's check word: 1 a value out of range, 2 a device wait that
// ran out of iterations (the FP32 form's tile loads).
constexpr int kCheckTimeout = 2;

// Descriptor of one member of an FP32-form batch (a context is a batch of
// one), passed to the kernels in their launch parameters. Pointers are fixed;
// the per-step rotation is derived in-kernel from a device step counter n:
// state buffer cur0 ^ (n & 1), history slot (w0 + n) % 3 written, AB index
// min(k0 + n, 2), checks in slot n % kCheckSlots.
struct MemberDesc {
  int nx, ny, P;
  int extra;
  float sig2dt, sigdt, nu2dt, nu4dt, nu6dt;
  const float* q;
  double* eta[2]; double* u[2]; double* v[2];
  float* es[2]; float* us[2]; float* vs[2];
  float* heta[3]; float* hu[3]; float* hv[3];
  float* Lu; float* Lv; float* dup; float* dvp;
  float* LLu; float* LLv;
  const TracerDesc* trd;  // nullptr: no tracer advected
  const CUtensorMap* tm;  // TM_NUM tensor maps of this member's FP32 fields
  unsigned* cfl; int* bad;
  int cur0, w0, k0, tile_test;
  int open_step;  // Fp32Ctx::open_step
  int polar;      // Fp32Ctx::polar
  const float* pf;  // Fp32Ctx::pf
};

// Most members of one batch: their descriptors fill at most ~28 KB of the
// 32 KB kernel parameter space.
constexpr int kMaxBatch = 96;

// Descriptor of a context's engine at its current step (counter n = 0).
MemberDesc fp32_desc(const Fp32Ctx& c, const Fp32Engine& e, int k);
// The same descriptor seen n steps after it was taken (what the kernels derive).
MemberDesc fp32_desc_after(const MemberDesc& d, int n);
// Strips of the FP32 kernels: kStripWidth cells wide (a warp, four cells per
// lane), kTileRows[s] rows high (the shapes the batch tuner picks from).
constexpr int kStripWidth = 128;
constexpr int kTileShapes = 3;
constexpr int kTileRows[kTileShapes] = {16, 32, 64};
// Strip height of a single context's steps.
constexpr int kTileRowsSolo = 32;
// Strips of a grid for strips th rows high.
void fp32_tiles(int nx, int ny, int th, int* nbx, int* nby);
// Enqueues one step of a batch of nmem members (host descriptors, passed by
// value) with strips th rows high; tiles is the device strip table (unused
// for one member, whose strips are nbx x nby in row order); queue is the
// launches' strip queue (2 words, zero between launches). Returns the number
// of kernel launches.
int fp32_batch_step(int sch, int th, const MemberDesc* desc, int nmem, const int4* tiles, int ntiles, int nbx,
                    int nby, int* counter, unsigned* queue, cudaStream_t st, Timers* tm);
// Shared-memory limits and occupancy of every FP32 kernel on the current
// device; called before any step can be captured into a graph.
void fp32_prepare();
// Bytes of a member's tensor-map table, and writing it (after the buffers
// exist; rewritten when the tracer buffers are made). False if the driver
// does not provide the tensor-map encoder or refuses a map.
size_t fp32_map_bytes();
bool fp32_write_maps(void* d_maps, const Fp32Ctx& c, const Fp32Engine& e, cudaStream_t st);

// FP32 shadow (pitch P) of an FP64 padded field (pitch nx+4), all padded cells.
void fp32_shadow(float* dst, const double* src, int nx, int ny, int P, cudaStream_t st);
// Pitch and row count of the FP32 arrays for a grid.
void fp32_geometry(int nx, int ny, int* P, int* R);

// dst = src + ref(j) row by row over a padded field (eta perturbation -> eta)
void add_row_ref(double* dst, const double* src, const double* ref_rows, int nx, int ny, cudaStream_t st);

void halo_wrap(double* x, int nx, int ny, cudaStream_t st);
void energy_rows(const DevState& s, const double* const* f, double* row_out, cudaStream_t st);
void energy_sum(const double* row_in, int ny, double* out3, cudaStream_t st);

}  // namespace sw2g
