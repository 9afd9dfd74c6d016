// C-ABI of the GB300 SW2 step (declared in include/sw2g.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "sw2g_internal.h"

using namespace sw2g;

namespace {

constexpr int kChunk = kCheckSlots;  // steps per check read-back

// Launch state of an FP32-form batch: the tile table (the sweep schedule),
// the device step counter, the member descriptors a one-step CUDA graph was
// captured with, and that graph.
struct BatchExec {
  int4* d_tiles = nullptr;
  int ntiles = 0, nbx = 0, nby = 0;  // nbx x nby: the grid of a single member
  int th = kTileRowsSolo;            // tile height of the kernels
  int per_step = 0;                  // launches per step of the captured graph
  int* d_counter = nullptr;
  unsigned* d_queue = nullptr;       // the kernels' strip queue (2 words, zero between launches)
  int n_dev = 0;                     // device counter: steps since cap was taken
  std::vector<MemberDesc> cap;
  cudaGraphExec_t exec = nullptr;
  int sch = 0;

  cudaError_t alloc(int ntile) {
    ntiles = ntile;
    cudaError_t e = cudaMalloc((void**)&d_counter, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_queue, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(d_queue, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess && ntile > 0) e = cudaMalloc((void**)&d_tiles, sizeof(int4) * ntile);
    return e;
  }
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (d_tiles) cudaFree(d_tiles);
    if (d_counter) cudaFree(d_counter);
    if (d_queue) cudaFree(d_queue);
    exec = nullptr;
    d_tiles = nullptr;
    d_counter = nullptr;
    d_queue = nullptr;
    cap.clear();
  }
  // Brings the launch state in line with the members' descriptors at their
  // current step. The captured graph and the counter are kept when every
  // member is where the counter says (only this launch state has stepped
  // it); otherwise the new descriptors are taken and the counter restarts.
  cudaError_t sync_to(const std::vector<MemberDesc>& now, cudaStream_t st) {
    bool same = cap.size() == now.size() && n_dev < (1 << 30);
    for (size_t m = 0; same && m < now.size(); m++) {
      const MemberDesc a = fp32_desc_after(cap[m], n_dev);
      same = std::memcmp(&a, &now[m], sizeof a) == 0;
    }
    if (same) return cudaSuccess;
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    cap = now;
    n_dev = 0;
    return cudaMemsetAsync(d_counter, 0, sizeof(int), st);
  }
  // Another tile shape: the captured graph (its grid size and kernels) no longer applies.
  void set_shape(int tile_rows, int n_tiles, int nbx1, int nby1) {
    if (tile_rows != th || n_tiles != ntiles) {
      if (exec) cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    th = tile_rows;
    ntiles = n_tiles;
    nbx = nbx1;
    nby = nby1;
  }
  // Check slot of the next step, and the steps left before the slots wrap.
  int slot() const { return n_dev & (kCheckSlots - 1); }
  int room() const { return kCheckSlots - slot(); }
  // Enqueues n steps: replays of a captured one-step graph, or direct
  // launches while per-kernel timers are on.
  cudaError_t enqueue(int n, cudaStream_t st, Timers* tm, long long& launches) {
    const int M = (int)cap.size();
    if (tm && tm->on) {
      for (int s = 0; s < n; s++)
        launches += fp32_batch_step(sch, th, cap.data(), M, d_tiles, ntiles, nbx, nby, d_counter, d_queue, st, tm);
      n_dev += n;
      return cudaGetLastError();
    }
    if (!exec) {
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return e;
      per_step = fp32_batch_step(sch, th, cap.data(), M, d_tiles, ntiles, nbx, nby, d_counter, d_queue, st, nullptr);
      e = cudaStreamEndCapture(st, &g);
      if (e != cudaSuccess) return e;
      e = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return e;
    }
    for (int s = 0; s < n; s++) {
      cudaError_t e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) return e;
    }
    n_dev += n;
    launches += (long long)per_step * n;
    return cudaSuccess;
  }
};

// Tile tables (sweep schedules) over members given as (nbx, nby) pairs.
enum Schedule { SCHED_ROWS = 0, SCHED_COLS = 1, SCHED_INTERLEAVE = 2, SCHED_BANDS = 3, SCHED_COUNT = 4 };

std::vector<int4> tile_table(const std::vector<int2>& nb, int sched) {
  std::vector<int4> t;
  const int M = (int)nb.size();
  if (sched == SCHED_INTERLEAVE) {
    std::vector<int> next(M, 0);
    bool more = true;
    while (more) {
      more = false;
      for (int m = 0; m < M; m++) {
        const int total = nb[m].x * nb[m].y;
        if (next[m] < total) {
          const int k = next[m]++;
          t.push_back(make_int4(m, k % nb[m].x, k / nb[m].x, 0));
          more = true;
        }
      }
    }
    return t;
  }
  for (int m = 0; m < M; m++) {
    const int nbx = nb[m].x, nby = nb[m].y;
    if (sched == SCHED_COLS) {
      for (int bx = 0; bx < nbx; bx++)
        for (int by = 0; by < nby; by++) t.push_back(make_int4(m, bx, by, 0));
    } else if (sched == SCHED_BANDS) {  // vertical bands of 8 tile columns, rows inside a band
      for (int b0 = 0; b0 < nbx; b0 += 8)
        for (int by = 0; by < nby; by++)
          for (int bx = b0; bx < nbx && bx < b0 + 8; bx++) t.push_back(make_int4(m, bx, by, 0));
    } else {
      for (int by = 0; by < nby; by++)
        for (int bx = 0; bx < nbx; bx++) t.push_back(make_int4(m, bx, by, 0));
    }
  }
  return t;
}

}  // namespace

struct sw2g_ctx {
  sw2g_case c{};
  int precision = SW2G_FP64;
  int device = 0;
  int sch = 0;
  DevState s{};
  std::vector<double> rows;
  double rest_mx = 0, rest_my = 0;
  double* d_rows = nullptr;
  Fp64Buffers b{};
  std::vector<double*> allocs;
  unsigned long long* d_cfl = nullptr;
  int* d_bad = nullptr;
  unsigned* d_strips = nullptr;  // DevState::strips
  double* d_energy = nullptr;  // 3*ny row partials + 3 totals
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double last_step_ms = 0;
  Timers timers;
  bool uploaded = false;
  bool tracer_active = false;
  bool aux_zero[3] = {true, true, true};  // windx, windy, hB hold +0.0 in every padded cell
  int k = 0;  // Adams-Bashforth index n - nstart
  long long steps = 0;
  int err_step = -1;
  long long last_launches = 0;
  bool open = false;  // between sw2g_step_open and sw2g_step_close
  int open_slot = 0;  // FP32 form: check slot of the opened step
  unsigned forced = 0;  // FP32 form, opened step: fields changed by forcing (bit per field)
  // FP32 precision form
  Fp32Engine e32;
  Fp32Ctx c32{};
  std::vector<void*> allocs32;
  float* d_q32 = nullptr;
  double* d_ref = nullptr;         // eta_ref(j), ny+4 rows
  std::vector<double> ref;         // host copy
  double* d_aux64[3] = {nullptr, nullptr, nullptr};  // windx, windy, hB (FP64) for the diagnostic
  float* d_aux32[3] = {nullptr, nullptr, nullptr};   // the same in FP32 for the stencils
  double* d_tmp = nullptr;         // full eta for download and diagnostics
  BatchExec run32;                 // this context as a batch of one
  // forcing between steps (FP64 form): staging of one padded field and a mask
  double* d_force = nullptr;
  void* d_mask = nullptr;
  // forcing on listed cells: a ring of pinned staging slots for the caller's
  // index and value lists (used in turn, each free again once its event has
  // completed: with 8 slots the calls of one forced step do not wait for the
  // step), the lists on the device, and a padded field that is zero outside
  // the cells of the call in progress
  struct CellSlot {
    int* idx = nullptr;
    double* val = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
  } cell_slot[8];
  int cell_next = 0;
  int* d_cells = nullptr;
  double* d_cellv = nullptr;
  size_t d_cell_cap = 0;
  double* d_delta = nullptr;
  // sw2g_step_host: a second stream for the copies of v, eta and u, and the
  // events u copied in, eta copied in, eta final, side copies done, u's
  // interior final, step done, v copied in (made on first use)
  cudaStream_t side = nullptr;
  cudaEvent_t hev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // pinned host copies of a chunk's checks (CFL maxima of either form, range
  // flags), so that reading them back is one more asynchronous copy
  void* h_chk = nullptr;
  unsigned long long* h_cfl = nullptr;
  unsigned* h_cfl32 = nullptr;
  int* h_bad = nullptr;
  // Gaussians evaluated on the device (sw2g_add_gaussian, made on first use):
  // the forcing tables, the scratch, a pinned copy of the error word, and
  // whether an injection ran since that word was last read
  double* d_grows = nullptr;
  double* d_glonc = nullptr;
  std::vector<double> gpl;  // planetocentric latc(j), j = 0..ny+1
  GaussScratch gs;
  int* h_gerr = nullptr;
  bool gerr_pending = false;
  bool gerr_host = false;   // an injection whose rows hold no cell had a volume to rescale
};

namespace {

sw2g_status cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SW2G_OK;
  fprintf(stderr, "sw2g: %s: %s\n", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? SW2G_ERR_NOMEM : SW2G_ERR_CUDA;
}

#define CK(call)                                              \
  do {                                                        \
    sw2g_status _st = cuda_fail((call), #call);               \
    if (_st != SW2G_OK) return _st;                           \
  } while (0)

bool case_ok(const sw2g_case* c) {
  if (!grid_ok(c)) return false;
  if (c->sch < 0 || c->sch > 9) return false;
  if (!(c->Dt > 0) || !(c->courant > 0)) return false;
  // init.c:122: hyperviscosity coefficients are entered as non-negative
  if (c->hypernu[0] < 0 || c->hypernu[1] < 0 || c->hypernu[2] < 0) return false;
  if (c->polar != 0) {  // the square around the pole (init.c:66-79)
    if ((c->polar != 1 && c->polar != -1) || c->nx != c->ny) return false;
    if (!(c->lon1 > 0) || c->lon0 != -c->lon1 || c->lat0 != c->lon0 || c->lat1 != c->lon1) return false;
    if (!(c->sigma_sponge >= 0)) return false;
  }
  if ((c->flags & SW2G_FLAG_SIGMA) && !(c->tau >= 0)) return false;
  return true;
}

sw2g_status dalloc(sw2g_ctx* x, double** p, size_t n) {
  CK(cudaMalloc((void**)p, n * sizeof(double)));
  CK(cudaMemsetAsync(*p, 0, n * sizeof(double), x->stream));
  x->allocs.push_back(*p);
  return SW2G_OK;
}

template <typename T>
sw2g_status dalloc32(sw2g_ctx* x, T** p, size_t n) {
  CK(cudaMalloc((void**)p, n * sizeof(T)));
  CK(cudaMemsetAsync(*p, 0, n * sizeof(T), x->stream));
  x->allocs32.push_back(*p);
  return SW2G_OK;
}

// Buffers of the FP32 form: FP64 state (double-buffered, eta as a perturbation),
// FP32 histories and intermediates.
sw2g_status alloc_fp32(sw2g_ctx* x) {
  const size_t S = (size_t)x->s.W * x->s.H;
  int P = 0, R = 0;
  fp32_geometry(x->s.nx, x->s.ny, &P, &R);
  x->c32.P = P;
  x->c32.R = R;
  const size_t S32 = (size_t)P * R;
  Fp32Engine& e = x->e32;
  sw2g_status st;
  for (int q = 0; q < 2; q++) {
    if ((st = dalloc(x, &e.eta[q], S)) != SW2G_OK) return st;
    if ((st = dalloc(x, &e.u[q], S)) != SW2G_OK) return st;
    if ((st = dalloc(x, &e.v[q], S)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.es[q], S32)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.us[q], S32)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.vs[q], S32)) != SW2G_OK) return st;
  }
  for (int q = 0; q < 3; q++) {
    if ((st = dalloc32(x, &e.heta[q], S32)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.hu[q], S32)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.hv[q], S32)) != SW2G_OK) return st;
    if ((st = dalloc(x, &x->d_aux64[q], S)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &x->d_aux32[q], S32)) != SW2G_OK) return st;
  }
  if ((st = dalloc32(x, &e.Lu, S32)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &e.Lv, S32)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &e.dup, S32)) != SW2G_OK) return st;
  {
    unsigned char* maps = nullptr;
    if ((st = dalloc32(x, &maps, fp32_map_bytes())) != SW2G_OK) return st;
    e.maps = maps;
  }
  if (x->s.nu6 != 0) {
    if ((st = dalloc32(x, &e.LLu, S32)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.LLv, S32)) != SW2G_OK) return st;
  }
  if ((st = dalloc32(x, &e.dvp, S32)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &e.cfl, 2 * (size_t)kChunk)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &e.bad, (size_t)kChunk)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &x->d_q32, (size_t)Q_NUM * x->s.H)) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->d_ref, (size_t)x->s.H)) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->d_tmp, S)) != SW2G_OK) return st;
  return SW2G_OK;
}

// Per-row FP32 constants of the FP32 form, from the FP64 geometry and the
// reference profile eta_ref(j) (all arithmetic in FP64, rounded once).
void build_q32(const sw2g_ctx* x, std::vector<float>& q) {
  const int ny = x->s.ny, H = x->s.H;
  const double Dt = x->c.Dt;
  q.assign((size_t)Q_NUM * H, 0.f);
  auto R = [&](int t, int j) { return x->rows[(size_t)t * H + (j + 1)]; };
  auto ref = [&](int j) { return x->ref[j + 1]; };
  for (int j = -1; j <= ny + 2; j++) {
    auto set = [&](int t, double v) { q[(size_t)(j + 1) * Q_NUM + t] = (float)v; };
    const bool up = (j + 1 <= ny + 2), up2 = (j + 2 <= ny + 2), dn2 = (j - 2 >= -1);
    set(Q_KXE, Dt / R(R_DXE, j));
    set(Q_KYN, Dt / R(R_DYN, j));
    set(Q_KXC, Dt / R(R_DXC, j));
    set(Q_KYV, Dt / R(R_DYV, j));
    set(Q_KXV, Dt / R(R_DXV, j));
    set(Q_KYC, Dt / R(R_DYC, j));
    set(Q_K2XE, Dt / (R(R_DXE, j) + R(R_DXE, j)));
    set(Q_KDYNS, up ? Dt / (R(R_DYN, j) + R(R_DYN, j + 1)) : 0.0);
    set(Q_GEX, -R(R_GE, j) * Dt / R(R_DXC, j));
    set(Q_GNY, up ? -R(R_GN, j) * Dt / R(R_DYC, j + 1) : 0.0);
    set(Q_GEO, R(R_GEO, j));
    set(Q_CV, Dt * R(R_SINN, j) / R(R_RZN, j));
    set(Q_DTFE, R(R_DTFE, j));
    set(Q_DTFN, R(R_DTFN, j));
    set(Q_HB, ref(j) + x->c.depth);
    set(Q_EREF, ref(j));
    set(Q_DHBM2, dn2 ? ref(j - 2) - ref(j) : 0.0);
    set(Q_DHBM1, j - 1 >= -1 ? ref(j - 1) - ref(j) : 0.0);
    set(Q_DHBP1, up ? ref(j + 1) - ref(j) : 0.0);
    set(Q_DHBP2, up2 ? ref(j + 2) - ref(j) : 0.0);
    set(Q_IDXV, 1.0 / R(R_DXV, j));
    set(Q_IDYC, 1.0 / R(R_DYC, j));
    set(Q_DXC, R(R_DXC, j));
    set(Q_IDXE, 1.0 / R(R_DXE, j));
    set(Q_IDYN, 1.0 / R(R_DYN, j));
    set(Q_DXV, R(R_DXV, j));
    set(Q_IDXC, 1.0 / R(R_DXC, j));
  }
}

bool all_zero(const double* a, size_t n) {
  if (!a) return true;
  for (size_t t = 0; t < n; t++)
    if (a[t] != 0.0) return false;
  return true;
}

// Upload for the FP32 form: eta is stored as eta - eta_ref(j), with eta_ref
// the zonal mean of the uploaded interior (halo rows take the wrapped rows).
// Buffers of the FP32 form's tracer, made on the first upload of a nonzero
// tracer: FP64 state and FP32 shadow (double-buffered), the history ring and
// the device descriptor the tracer kernel reads.
sw2g_status tracer_fp32(sw2g_ctx* x) {
  Fp32Engine& e = x->e32;
  if (e.d_trd) return SW2G_OK;
  const size_t S = (size_t)x->s.W * x->s.H, S32 = (size_t)x->c32.P * x->c32.R;
  sw2g_status st;
  for (int q = 0; q < 2; q++) {
    if ((st = dalloc(x, &e.tr[q], S)) != SW2G_OK) return st;
    if ((st = dalloc32(x, &e.ts[q], S32)) != SW2G_OK) return st;
  }
  for (int q = 0; q < 3; q++)
    if ((st = dalloc32(x, &e.htr[q], S32)) != SW2G_OK) return st;
  TracerDesc td;
  for (int q = 0; q < 2; q++) {
    td.tr[q] = e.tr[q];
    td.ts[q] = e.ts[q];
  }
  for (int q = 0; q < 3; q++) td.h[q] = e.htr[q];
  td.sig2dt = (float)(2.0 * x->c.Dt * x->c.tracer_dis);  // calc.c:162
  TracerDesc* d = nullptr;
  if ((st = dalloc32(x, &d, 1)) != SW2G_OK) return st;
  CK(cudaMemcpyAsync(d, &td, sizeof td, cudaMemcpyHostToDevice, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  e.d_trd = d;
  if (!fp32_write_maps(e.maps, x->c32, e, x->stream)) {  // now with the tracer shadows
    fprintf(stderr, "sw2g: tensor maps of the FP32 fields could not be made\n");
    return SW2G_ERR_CUDA;
  }
  return SW2G_OK;
}

sw2g_status upload_fp32(sw2g_ctx* x, const double* eta, const double* u, const double* v, const double* tracer,
                        const double* windx, const double* windy, const double* hB, int mode) {
  const DevState& s = x->s;
  const int W = s.W, H = s.H, nx = s.nx, ny = s.ny;
  const size_t S = (size_t)W * H, bytes = S * sizeof(double);
  const bool cont = (mode == SW2G_UPLOAD_CONTINUE);
  Fp32Engine& e = x->e32;
  // the tracer is advected once any padded cell of it can be nonzero (a tracer
  // that is +0.0 everywhere stays so: its step then changes nothing)
  if (tracer && (e.tracer || !all_zero(tracer, S))) {
    sw2g_status st = tracer_fp32(x);
    if (st != SW2G_OK) return st;
    CK(cudaMemcpyAsync(e.tr[e.cur], tracer, bytes, cudaMemcpyHostToDevice, x->stream));
    if (mode == SW2G_UPLOAD_FRAME) halo_wrap(e.tr[e.cur], nx, ny, x->stream);
    fp32_shadow(e.ts[e.cur], e.tr[e.cur], nx, ny, x->c32.P, x->stream);
    e.tracer = true;
  } else if (!cont) {
    e.tracer = false;
  }
  if (!cont) {
    x->ref.assign(H, 0.0);
    for (int j = 1; j <= ny; j++) {
      double acc = 0, cmp = 0;
      for (int i = 1; i <= nx; i++) {  // compensated zonal sum
        const double t = eta[(i + 1) + (size_t)(j + 1) * W], a = acc + t;
        cmp += (std::fabs(acc) >= std::fabs(t)) ? ((acc - a) + t) : ((t - a) + acc);
        acc = a;
      }
      x->ref[j + 1] = (acc + cmp) / nx;
    }
    x->ref[0] = x->ref[ny];  // j = -1 <- ny - 1
    x->ref[1] = x->ref[ny + 1];
    x->ref[ny + 2] = x->ref[2];
    x->ref[ny + 3] = x->ref[3];
    CK(cudaMemcpyAsync(x->d_ref, x->ref.data(), H * sizeof(double), cudaMemcpyHostToDevice, x->stream));
    std::vector<float> q;
    build_q32(x, q);
    CK(cudaMemcpyAsync(x->d_q32, q.data(), q.size() * sizeof(float), cudaMemcpyHostToDevice, x->stream));
    CK(cudaStreamSynchronize(x->stream));
  }
  std::vector<double> ep(S);
  for (int j = -1; j <= ny + 2; j++)
    for (int i = -1; i <= nx + 2; i++) {
      const size_t t = (i + 1) + (size_t)(j + 1) * W;
      ep[t] = eta[t] - x->ref[j + 1];
    }
  CK(cudaMemcpyAsync(e.eta[e.cur], ep.data(), bytes, cudaMemcpyHostToDevice, x->stream));
  CK(cudaMemcpyAsync(e.u[e.cur], u, bytes, cudaMemcpyHostToDevice, x->stream));
  CK(cudaMemcpyAsync(e.v[e.cur], v, bytes, cudaMemcpyHostToDevice, x->stream));
  if (mode == SW2G_UPLOAD_FRAME) {
    halo_wrap(e.eta[e.cur], nx, ny, x->stream);
    halo_wrap(e.u[e.cur], nx, ny, x->stream);
    halo_wrap(e.v[e.cur], nx, ny, x->stream);
  }
  const int P = x->c32.P;
  fp32_shadow(e.es[e.cur], e.eta[e.cur], nx, ny, P, x->stream);
  fp32_shadow(e.us[e.cur], e.u[e.cur], nx, ny, P, x->stream);
  fp32_shadow(e.vs[e.cur], e.v[e.cur], nx, ny, P, x->stream);
  const double* aux[3] = {windx, windy, hB};
  if (!cont || windx || windy || hB) {
    int extra = 0;
    for (int q = 0; q < 3; q++) {
      if (aux[q]) {
        CK(cudaMemcpyAsync(x->d_aux64[q], aux[q], bytes, cudaMemcpyHostToDevice, x->stream));
        fp32_shadow(x->d_aux32[q], x->d_aux64[q], nx, ny, P, x->stream);
        if (!all_zero(aux[q], S)) extra = 1;
      } else if (!cont) {
        CK(cudaMemsetAsync(x->d_aux64[q], 0, bytes, x->stream));
        CK(cudaMemsetAsync(x->d_aux32[q], 0, (size_t)P * x->c32.R * sizeof(float), x->stream));
      }
    }
    if (!cont) x->c32.extra = extra;
    else x->c32.extra = x->c32.extra || extra;
  }
  CK(cudaStreamSynchronize(x->stream));
  return SW2G_OK;
}

}  // namespace

namespace sw2g {

bool grid_ok(const sw2g_case* c) {
  if (!c) return false;
  if (c->nx < 3 || c->ny < 3) return false;
  // cell indices are 32-bit: (i+1) + (j+1)*(nx+4) over the padded field
  if ((long long)(c->nx + 4) * (c->ny + 4) > (1LL << 31) - 1) return false;
  if (!(c->rE > 0) || !(c->rP > 0)) return false;
  if (!(c->lon1 > c->lon0) || !(c->lat1 > c->lat0)) return false;
  const double pole = (c->flags & SW2G_FLAG_RADIANS) ? 2.0 * std::atan(1.0) : 90.0;
  if (!(c->lat0 > -pole) || !(c->lat1 < pole)) return false;
  if (c->flags & ~(SW2G_FLAG_VANLEER_SAFE | SW2G_FLAG_RADIANS | SW2G_FLAG_SIGMA | SW2G_FLAG_LAPE_ETA)) return false;
  return true;
}

cudaEvent_t Timers::take() {
  if (!free_.empty()) {
    cudaEvent_t e = free_.back();
    free_.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void Timers::begin(const char* tag, cudaStream_t st) {
  int idx = -1;
  for (size_t q = 0; q < entries_.size(); q++)
    if (std::strcmp(entries_[q].name, tag) == 0) idx = (int)q;
  if (idx < 0) {
    entries_.push_back(Entry{tag, 0, 0.0});
    idx = (int)entries_.size() - 1;
  }
  open_ = idx;
  open_ev_ = take();
  cudaEventRecord(open_ev_, st);
}

void Timers::end(cudaStream_t st) {
  if (open_ < 0) return;
  cudaEvent_t e = take();
  cudaEventRecord(e, st);
  pending_.push_back(Pending{open_, open_ev_, e});
  open_ = -1;
}

void Timers::collect() {
  for (const Pending& p : pending_) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      entries_[p.entry].ms += ms;
      entries_[p.entry].launches += 1;
    }
    free_.push_back(p.a);
    free_.push_back(p.b);
  }
  pending_.clear();
}

void Timers::reset() {
  for (Entry& e : entries_) {
    e.launches = 0;
    e.ms = 0;
  }
}

void Timers::release() {
  collect();
  for (cudaEvent_t e : free_) cudaEventDestroy(e);
  free_.clear();
  entries_.clear();
}

}  // namespace sw2g

extern "C" {

const char* sw2g_status_string(sw2g_status s) {
  switch (s) {
    case SW2G_OK: return "ok";
    case SW2G_ERR_BAD_ARG: return "invalid argument";
    case SW2G_ERR_CFL: return "time step exceeds the CFL limit";
    case SW2G_ERR_NONFINITE: return "field out of range or not finite";
    case SW2G_ERR_TIMEOUT: return "device wait timed out";
    case SW2G_ERR_CUDA: return "CUDA error";
    case SW2G_ERR_NOMEM: return "out of memory";
    case SW2G_ERR_STATE: return "call out of order";
    case SW2G_ERR_FORCING: return "injected volume is zero or missed its target";
  }
  return "unknown status";
}

sw2g_status sw2g_create(const sw2g_case* c, int precision, int device, sw2g_ctx** out) {
  if (!out) return SW2G_ERR_BAD_ARG;
  *out = nullptr;
  if (!case_ok(c) || (precision != SW2G_FP64 && precision != SW2G_FP32)) return SW2G_ERR_BAD_ARG;
  // the FP32 form covers the reference's u source of the eta Laplacian
  if (precision == SW2G_FP32 && (c->flags & SW2G_FLAG_LAPE_ETA)) return SW2G_ERR_BAD_ARG;
  sw2g_ctx* x = new (std::nothrow) sw2g_ctx();
  if (!x) return SW2G_ERR_NOMEM;
  x->c = *c;
  x->precision = precision;
  x->device = device;
  x->sch = c->sch;
  if (c->sch == 3 && (c->flags & SW2G_FLAG_VANLEER_SAFE)) x->sch = kVanLeerSafe;
  sw2g_status st = SW2G_OK;
  auto fail = [&](sw2g_status e) {
    sw2g_destroy(x);
    return e;
  };
  if ((st = cuda_fail(cudaSetDevice(device), "cudaSetDevice")) != SW2G_OK) return fail(st);
  if ((st = cuda_fail(cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking), "stream")) != SW2G_OK)
    return fail(st);
  for (int e = 0; e < 2; e++)
    if ((st = cuda_fail(cudaEventCreate(&x->ev[e]), "event")) != SW2G_OK) return fail(st);
  build_rows(*c, x->rows, &x->rest_mx, &x->rest_my);
  DevState& s = x->s;
  s.nx = c->nx;
  s.ny = c->ny;
  s.W = c->nx + 4;
  s.H = c->ny + 4;
  s.depth = c->depth;
  s.Dt = c->Dt;
  if (c->flags & SW2G_FLAG_SIGMA) s.sigma = c->tau;  // already sigma_dis
  else s.sigma = c->tau > 1e10 ? 0 : 1.0 / c->tau;     // init.c:110-114
  s.sigma_tr = c->tracer_dis;
  s.nu2 = c->hypernu[0];
  s.nu4 = -c->hypernu[1];  // init.c:120
  s.nu6 = c->hypernu[2];
  s.lape_eta = (c->flags & SW2G_FLAG_LAPE_ETA) ? 1 : 0;
  s.nu2dt = s.nu2 * s.Dt;
  s.nu4dt = s.nu4 * s.Dt;
  s.nu6dt = s.nu6 * s.Dt;
  const size_t S = (size_t)s.W * s.H;
  if ((st = dalloc(x, &x->d_rows, x->rows.size())) != SW2G_OK) return fail(st);
  if ((st = cuda_fail(cudaMemcpyAsync(x->d_rows, x->rows.data(), x->rows.size() * sizeof(double),
                                      cudaMemcpyHostToDevice, x->stream), "rows")) != SW2G_OK)
    return fail(st);
  s.rows = x->d_rows;
  s.polar = c->polar;
  s.pf = nullptr;
  std::vector<double> pf;
  if (c->polar != 0) {  // gravity, Coriolis and sponge fields of the cap
    polar_fields(*c, pf, &x->rest_mx, &x->rest_my);
    double* d_pf = nullptr;
    if ((st = dalloc(x, &d_pf, pf.size())) != SW2G_OK) return fail(st);
    if ((st = cuda_fail(cudaMemcpyAsync(d_pf, pf.data(), pf.size() * sizeof(double), cudaMemcpyHostToDevice,
                                        x->stream), "polar fields")) != SW2G_OK)
      return fail(st);
    if ((st = cuda_fail(cudaStreamSynchronize(x->stream), "polar fields")) != SW2G_OK) return fail(st);
    s.pf = d_pf;
  }
  if (precision == SW2G_FP64) {
    Fp64Buffers& b = x->b;
    double** all[] = {&b.f[0], &b.f[1], &b.f[2], &b.f[3], &b.f[4], &b.f[5], &b.f[6],
                      &b.deta[0], &b.deta[1], &b.deta[2], &b.du[0], &b.du[1], &b.du[2],
                      &b.dv[0], &b.dv[1], &b.dv[2], &b.dtr[0], &b.dtr[1], &b.dtr[2],
                      &b.detaAB, &b.duAB, &b.dvAB, &b.dtrAB, &b.duadv, &b.dvadv,
                      &b.Le[0], &b.Le[1], &b.Le[2], &b.L[0], &b.L[1], &b.L[2], &b.L[3], &b.L[4], &b.L[5],
                      &b.psi, &b.xi, &b.ze, &b.di};
    for (double** p : all)
      if ((st = dalloc(x, p, S)) != SW2G_OK) return fail(st);
  } else {
    if ((st = alloc_fp32(x)) != SW2G_OK) return fail(st);
    Fp32Ctx& c32 = x->c32;
    c32.nx = c->nx;
    c32.ny = c->ny;
    c32.sch = (c->sch == 3) ? kVanLeerSafe : c->sch;  // the FP32 form always uses the safe Van Leer
    c32.q = x->d_q32;
    c32.sig2dt = (float)(2.0 * c->Dt * s.sigma);
    c32.sigdt = (float)(s.sigma * c->Dt);
    c32.nu2dt = (float)(s.nu2 * c->Dt);
    c32.nu4dt = (float)(s.nu4 * c->Dt);
    c32.nu6dt = (float)(s.nu6 * c->Dt);
    c32.wx = x->d_aux32[0];
    c32.wy = x->d_aux32[1];
    c32.hb = x->d_aux32[2];
    if (c->polar != 0) {  // the cap's per-cell factors, FP64 arithmetic rounded once
      const int P = c32.P, W = s.W, H = s.H;
      const size_t S32 = (size_t)P * c32.R;
      std::vector<float> q32((size_t)PQ_NUM * S32, 0.f);
      auto row = [&](int t, int j) { return x->rows[(size_t)t * H + (j + 1)]; };
      const double Dt = c->Dt;
      for (int j = -1; j <= c->ny + 2; j++)
        for (int i = -1; i <= c->nx + 2; i++) {
          const size_t q = (size_t)(i + 1) + (size_t)(j + 1) * W, r = (size_t)(i + 3) + (size_t)(j + 1) * P;
          auto F = [&](int t) { return pf[(size_t)t * S + q]; };
          q32[PQ_GEX * S32 + r] = (float)(-F(P_GE) * Dt / row(R_DXC, j));
          q32[PQ_GNY * S32 + r] = (float)(j + 1 <= c->ny + 2 ? -F(P_GN) * Dt / row(R_DYC, j + 1) : 0.0);
          q32[PQ_DTFE * S32 + r] = (float)(Dt * F(P_FE));
          q32[PQ_DTFN * S32 + r] = (float)(Dt * F(P_FN));
          q32[PQ_SH2 * S32 + r] = (float)(2.0 * Dt * F(P_SH));
          q32[PQ_SU * S32 + r] = (float)(F(P_SU) * Dt);
          q32[PQ_SV * S32 + r] = (float)(F(P_SV) * Dt);
          q32[PQ_STR2 * S32 + r] = (float)(2.0 * Dt * F(P_STR));
        }
      float* d_pf32 = nullptr;
      if ((st = dalloc32(x, &d_pf32, q32.size())) != SW2G_OK) return fail(st);
      if ((st = cuda_fail(cudaMemcpyAsync(d_pf32, q32.data(), q32.size() * sizeof(float), cudaMemcpyHostToDevice,
                                          x->stream), "polar fields")) != SW2G_OK)
        return fail(st);
      c32.polar = c->polar;
      c32.pf = d_pf32;
    }
    fp32_tiles(c->nx, c->ny, x->run32.th, &x->run32.nbx, &x->run32.nby);
    if ((st = cuda_fail(x->run32.alloc(0), "batch")) != SW2G_OK) return fail(st);
    x->run32.sch = c32.sch;
    fp32_prepare();
    if ((st = cuda_fail(cudaStreamSynchronize(x->stream), "alloc")) != SW2G_OK) return fail(st);
    if (!fp32_write_maps(x->e32.maps, c32, x->e32, x->stream)) {
      fprintf(stderr, "sw2g: tensor maps of the FP32 fields could not be made\n");
      return fail(SW2G_ERR_CUDA);
    }
  }
  if ((st = cuda_fail(cudaMalloc((void**)&x->d_cfl, sizeof(unsigned long long) * 2 * kChunk), "cfl")) != SW2G_OK)
    return fail(st);
  if ((st = cuda_fail(cudaMalloc((void**)&x->d_bad, sizeof(int) * kChunk), "bad")) != SW2G_OK) return fail(st);
  if ((st = cuda_fail(cudaMalloc((void**)&x->d_strips, 2 * sizeof(unsigned)), "strips")) != SW2G_OK) return fail(st);
  if ((st = cuda_fail(cudaMemsetAsync(x->d_strips, 0, 2 * sizeof(unsigned), x->stream), "strips")) != SW2G_OK)
    return fail(st);
  x->s.strips = x->d_strips;
  {
    const size_t b64 = sizeof(unsigned long long) * 2 * kChunk, b32 = sizeof(unsigned) * 2 * kChunk;
    if ((st = cuda_fail(cudaHostAlloc(&x->h_chk, b64 + b32 + sizeof(int) * kChunk, cudaHostAllocDefault),
                        "pinned checks")) != SW2G_OK)
      return fail(st);
    x->h_cfl = (unsigned long long*)x->h_chk;
    x->h_cfl32 = (unsigned*)((char*)x->h_chk + b64);
    x->h_bad = (int*)((char*)x->h_chk + b64 + b32);
  }
  if ((st = dalloc(x, &x->d_energy, 3 * (size_t)c->ny + 3)) != SW2G_OK) return fail(st);
  if ((st = cuda_fail(cudaStreamSynchronize(x->stream), "sync")) != SW2G_OK) return fail(st);
  *out = x;
  return SW2G_OK;
}

sw2g_status sw2g_upload(sw2g_ctx* x, const double* eta, const double* u, const double* v, const double* tracer,
                        const double* windx, const double* windy, const double* hB, int mode) {
  if (!x || !eta || !u || !v) return SW2G_ERR_BAD_ARG;
  if (mode != SW2G_UPLOAD_RAW && mode != SW2G_UPLOAD_FRAME && mode != SW2G_UPLOAD_CONTINUE) return SW2G_ERR_BAD_ARG;
  const bool cont = (mode == SW2G_UPLOAD_CONTINUE);
  if (cont && !x->uploaded) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  if (x->precision == SW2G_FP32) {
    sw2g_status st = upload_fp32(x, eta, u, v, tracer, windx, windy, hB, mode);
    if (st != SW2G_OK) return st;
    if (!cont) {
      x->k = 0;
      x->steps = 0;
      x->err_step = -1;
    }
    x->uploaded = true;
    return SW2G_OK;
  }
  const DevState& s = x->s;
  const size_t S = (size_t)s.W * s.H, bytes = S * sizeof(double);
  const double* src[7] = {eta, u, v, tracer, windx, windy, hB};
  for (int q = 0; q < 7; q++) {
    if (src[q]) CK(cudaMemcpyAsync(x->b.f[q], src[q], bytes, cudaMemcpyHostToDevice, x->stream));
    else if (!cont) CK(cudaMemsetAsync(x->b.f[q], 0, bytes, x->stream));  // CONTINUE: NULL keeps the field
  }
  if (mode == SW2G_UPLOAD_FRAME)
    for (int q = 0; q < 4; q++) halo_wrap(x->b.f[q], s.nx, s.ny, x->stream);
  // Winds and bottom that are +0.0 everywhere (the usual case) let the fast
  // bodies drop the additions u+windx, v+windy and the subtraction -hB
  // (fp64_step's plain form; do_channel keeps such fields +0.0).
  for (int q = 4; q < 7; q++) {
    if (src[q]) {
      bool z = true;
      for (size_t t = 0; t < S && z; t++) {
        uint64_t bits;
        std::memcpy(&bits, &src[q][t], sizeof(bits));
        z = (bits == 0);
      }
      x->aux_zero[q - 4] = z;
    } else if (!cont) {
      x->aux_zero[q - 4] = true;
    }
  }
  x->s.plain = x->aux_zero[0] && x->aux_zero[1] && x->aux_zero[2];
  if (cont) {
    // history, step count and the tracer decision carry over (unless a tracer is given)
    if (tracer) x->tracer_active = true;
    CK(cudaStreamSynchronize(x->stream));
    return SW2G_OK;
  }
  // The tracer step is skipped while the tracer is +0.0 in every cell it can
  // read: with no source the reference's tracer update then provably leaves it +0.
  bool active = false;
  if (tracer) {
    for (int j = -1; j <= s.ny + 2 && !active; j++)
      for (int i = -1; i <= s.nx + 2; i++) {
        const bool inner = (i >= 1 && i <= s.nx && j >= 1 && j <= s.ny);
        if (mode == SW2G_UPLOAD_FRAME && !inner) continue;
        uint64_t bits;
        std::memcpy(&bits, &tracer[(i + 1) + (size_t)(j + 1) * s.W], sizeof(bits));
        if (bits != 0) { active = true; break; }
      }
  }
  x->tracer_active = active;
  x->k = 0;
  x->steps = 0;
  x->err_step = -1;
  x->uploaded = true;
  CK(cudaStreamSynchronize(x->stream));
  return SW2G_OK;
}

// The caller's arrays of sw2g_step_host: copied out at the end of the last
// step, eta as soon as the step has finished it (FP64 form).
struct HostIO {
  double *eta, *u, *v;
  bool copied;
};

static sw2g_status run_steps(sw2g_ctx* x, int nsteps, HostIO* io);

sw2g_status sw2g_step(sw2g_ctx* x, int nsteps) {
  if (!x || nsteps < 0) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded || x->open) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  return run_steps(x, nsteps, nullptr);
}

sw2g_status sw2g_step_host(sw2g_ctx* x, double* eta, double* u, double* v, int nsteps) {
  if (!x || !eta || !u || !v || nsteps < 1) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded || x->open) return SW2G_ERR_STATE;
  if (x->precision == SW2G_FP32) {  // the FP32 form converts on the way in and out: in sequence
    sw2g_status st = sw2g_upload(x, eta, u, v, nullptr, nullptr, nullptr, nullptr, SW2G_UPLOAD_CONTINUE);
    if (st != SW2G_OK) return st;
    const sw2g_status ss = sw2g_step(x, nsteps);
    st = sw2g_download(x, eta, u, v, nullptr);
    return ss != SW2G_OK ? ss : st;
  }
  CK(cudaSetDevice(x->device));
  for (int e = 0; e < 7; e++)  // made on first use (and again after a failed attempt)
    if (!x->hev[e]) CK(cudaEventCreateWithFlags(&x->hev[e], cudaEventDisableTiming));
  if (!x->side) CK(cudaStreamCreateWithFlags(&x->side, cudaStreamNonBlocking));
  // u first, then v and eta on the side stream: the step's first kernels
  // (the eta Laplacians) read only u, the next ones (the CFL maxima, the
  // advection of u and v) u and v, while eta is still on its way in.
  const size_t bytes = sizeof(double) * (size_t)x->s.W * x->s.H;
  CK(cudaMemcpyAsync(x->b.f[1], u, bytes, cudaMemcpyHostToDevice, x->stream));
  CK(cudaEventRecord(x->hev[0], x->stream));
  CK(cudaStreamWaitEvent(x->side, x->hev[0], 0));
  CK(cudaMemcpyAsync(x->b.f[2], v, bytes, cudaMemcpyHostToDevice, x->side));
  CK(cudaEventRecord(x->hev[6], x->side));
  CK(cudaMemcpyAsync(x->b.f[0], eta, bytes, cudaMemcpyHostToDevice, x->side));
  CK(cudaEventRecord(x->hev[1], x->side));
  HostIO io{eta, u, v, false};
  const sw2g_status st = run_steps(x, nsteps, &io);
  if (!io.copied) {  // a failure before the last chunk of steps was queued
    // the side stream's uploads of v and eta must have landed before the
    // read-back on the main stream reads those fields
    const sw2g_status sw = cuda_fail(cudaStreamSynchronize(x->side), "cudaStreamSynchronize");
    if (sw != SW2G_OK) return st != SW2G_OK ? st : sw;
    const sw2g_status sd = sw2g_download(x, eta, u, v, nullptr);
    return st != SW2G_OK ? st : sd;
  }
  CK(cudaStreamSynchronize(x->side));
  return st;
}

static sw2g_status run_steps(sw2g_ctx* x, int nsteps, HostIO* io) {
  x->last_launches = 0;
  unsigned long long* const cfl = x->h_cfl;
  unsigned* const cfl32 = x->h_cfl32;
  int* const bad = x->h_bad;
  int done = 0;
  x->last_step_ms = 0;
  const bool f32 = (x->precision == SW2G_FP32);
  while (done < nsteps) {
    int n = (nsteps - done) < kChunk ? (nsteps - done) : kChunk;
    int slot0 = 0;  // check slot of the chunk's first step
    if (f32) {
      CK(x->run32.sync_to({fp32_desc(x->c32, x->e32, x->k)}, x->stream));
      if (n > x->run32.room()) n = x->run32.room();
      slot0 = x->run32.slot();
      CK(cudaMemsetAsync(x->e32.cfl + 2 * slot0, 0, sizeof(unsigned) * 2 * n, x->stream));
      CK(cudaMemsetAsync(x->e32.bad + slot0, 0, sizeof(int) * n, x->stream));
    } else {
      CK(cudaMemsetAsync(x->d_cfl, 0, sizeof(unsigned long long) * 2 * n, x->stream));
      CK(cudaMemsetAsync(x->d_bad, 0, sizeof(int) * n, x->stream));
    }
    StepChecks chk{x->d_cfl, x->d_bad};
    CK(cudaEventRecord(x->ev[0], x->stream));
    if (f32) {
      CK(x->run32.enqueue(n, x->stream, &x->timers, x->last_launches));
      x->e32.advance_host(n);
      x->k += n;
    } else {
      for (int t = 0; t < n; t++) {
        StepHooks hk;
        if (io && done + t == 0) {
          hk.v_in = x->hev[6];
          hk.eta_in = x->hev[1];
        }
        if (io && done + t == nsteps - 1) {
          hk.eta_out = x->hev[2];
          hk.u_out = x->hev[4];
        }
        x->last_launches += fp64_step(x->s, x->b, x->sch, x->k, x->tracer_active, chk, t, x->stream, &x->timers,
                                      STEP_FULL, hk);
        x->k++;
      }
    }
    CK(cudaEventRecord(x->ev[1], x->stream));
    CK(cudaGetLastError());
    if (io && done + n == nsteps) {
      // On the side stream, eta goes out while the step computes u and v, and
      // u while it computes v; u's halo columns and wall rows, which the end
      // of the step rewrites, follow once it is done.
      const size_t W = x->s.W, H = x->s.H, row = sizeof(double) * W, bytes = row * H;
      const int nx = x->s.nx, ny = x->s.ny;
      CK(cudaEventRecord(x->hev[5], x->stream));
      CK(cudaStreamWaitEvent(x->side, x->hev[2], 0));
      CK(cudaMemcpyAsync(io->eta, x->b.f[0], bytes, cudaMemcpyDeviceToHost, x->side));
      CK(cudaStreamWaitEvent(x->side, x->hev[4], 0));
      CK(cudaMemcpyAsync(io->u, x->b.f[1], bytes, cudaMemcpyDeviceToHost, x->side));
      CK(cudaStreamWaitEvent(x->side, x->hev[5], 0));
      const double* du = x->b.f[1];
      CK(cudaMemcpyAsync(io->u, du, 2 * row, cudaMemcpyDeviceToHost, x->side));  // rows -1, 0
      CK(cudaMemcpyAsync(io->u + (ny + 2) * W, du + (ny + 2) * W, 2 * row, cudaMemcpyDeviceToHost,
                         x->side));  // rows ny+1, ny+2
      for (size_t c : {(size_t)0, (size_t)nx + 2})  // columns -1, 0 and nx+1, nx+2 of the interior rows
        CK(cudaMemcpy2DAsync(io->u + 2 * W + c, row, du + 2 * W + c, row, 2 * sizeof(double), ny,
                             cudaMemcpyDeviceToHost, x->side));
      CK(cudaEventRecord(x->hev[3], x->side));
      CK(cudaMemcpyAsync(io->v, x->b.f[2], bytes, cudaMemcpyDeviceToHost, x->stream));
      CK(cudaStreamWaitEvent(x->stream, x->hev[3], 0));
      io->copied = true;
    }
    if (f32) {
      CK(cudaMemcpyAsync(cfl32, x->e32.cfl + 2 * slot0, sizeof(unsigned) * 2 * n, cudaMemcpyDeviceToHost,
                         x->stream));
      CK(cudaMemcpyAsync(bad, x->e32.bad + slot0, sizeof(int) * n, cudaMemcpyDeviceToHost, x->stream));
    } else {
      CK(cudaMemcpyAsync(cfl, x->d_cfl, sizeof(unsigned long long) * 2 * n, cudaMemcpyDeviceToHost, x->stream));
      CK(cudaMemcpyAsync(bad, x->d_bad, sizeof(int) * n, cudaMemcpyDeviceToHost, x->stream));
    }
    CK(cudaStreamSynchronize(x->stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, x->ev[0], x->ev[1]));
    x->last_step_ms += ms;
    if (x->timers.on) x->timers.collect();
    for (int t = 0; t < n; t++) {
      // compute_Dt (calc.c:701-738) and its check (core.c:158)
      double mx, my;
      if (f32) {
        float a, b2;
        std::memcpy(&a, &cfl32[2 * t], sizeof(float));
        std::memcpy(&b2, &cfl32[2 * t + 1], sizeof(float));
        mx = a;
        my = b2;
      } else {
        std::memcpy(&mx, &cfl[2 * t], sizeof(double));
        std::memcpy(&my, &cfl[2 * t + 1], sizeof(double));
      }
      if (mx + my == 0) { mx = x->rest_mx; my = x->rest_my; }
      const double dt_cfl = (x->c.courant / (mx + my));
      if (x->c.Dt > dt_cfl) {
        x->err_step = (int)(x->steps + t);
        x->steps += t;
        return SW2G_ERR_CFL;
      }
      if (bad[t]) {
        x->err_step = (int)(x->steps + t);
        x->steps += t + 1;
        return (bad[t] & kCheckTimeout) ? SW2G_ERR_TIMEOUT : SW2G_ERR_NONFINITE;
      }
    }
    x->steps += n;
    done += n;
  }
  return SW2G_OK;
}

namespace {
sw2g_status gauss_queue_check(sw2g_ctx* x);
bool gauss_failed(sw2g_ctx* x);

// The FP64 field a forcing call changes: the reference layout's field, or in
// the FP32 form its FP64 state (eta as eta - eta_ref(j)).
double* force_target(sw2g_ctx* x, int which) {
  if (x->precision == SW2G_FP32) {
    Fp32Engine& e = x->e32;
    return which == 0 ? e.eta[e.cur] : which == 1 ? e.u[e.cur] : which == 2 ? e.v[e.cur] : e.tr[e.cur];
  }
  return x->b.f[which];
}

// FP32 form: the FP32 shadow of a field after its FP64 state changed.
void fp32_reshadow(sw2g_ctx* x, int which) {
  Fp32Engine& e = x->e32;
  float* dst = which == 0 ? e.es[e.cur] : which == 1 ? e.us[e.cur] : which == 2 ? e.vs[e.cur] : e.ts[e.cur];
  fp32_shadow(dst, force_target(x, which), x->s.nx, x->s.ny, x->c32.P, x->stream);
}

// FP32 form: do_channel (calc.c:600-649) on the FP64 u, v and the winds, then
// their FP32 shadows.
void fp32_channel(sw2g_ctx* x) {
  Fp32Engine& e = x->e32;
  const int nx = x->s.nx, ny = x->s.ny, P = x->c32.P;
  fp64_channel(e.u[e.cur], e.v[e.cur], x->d_aux64[0], x->d_aux64[1], nx, ny, x->stream);
  fp32_reshadow(x, 1);
  fp32_reshadow(x, 2);
  fp32_shadow(x->d_aux32[0], x->d_aux64[0], nx, ny, P, x->stream);
  fp32_shadow(x->d_aux32[1], x->d_aux64[1], nx, ny, P, x->stream);
}

// FP32 form: one whole step with the plain halo update of u and v (its range
// flags are not used: the checks come after the forcing).
sw2g_status fp32_step_open(sw2g_ctx* x) {
  x->c32.open_step = 1;
  CK(x->run32.sync_to({fp32_desc(x->c32, x->e32, x->k)}, x->stream));
  x->c32.open_step = 0;
  const int slot = x->run32.slot();
  CK(cudaMemsetAsync(x->e32.cfl + 2 * slot, 0, sizeof(unsigned) * 2, x->stream));
  CK(cudaMemsetAsync(x->e32.bad + slot, 0, sizeof(int), x->stream));
  CK(cudaEventRecord(x->ev[0], x->stream));
  x->last_launches = 0;
  CK(x->run32.enqueue(1, x->stream, &x->timers, x->last_launches));
  CK(cudaGetLastError());
  x->e32.advance_host(1);
  x->k++;
  x->open_slot = slot;
  x->forced = 0;
  x->open = true;
  return SW2G_OK;
}

// FP32 form, after the forcing (core.c:297-312): the halo update of the
// forced tracer and eta, do_channel, the FP32 shadows of what changed, the
// range checks of the four fields; then the step's CFL check.
sw2g_status fp32_step_close(sw2g_ctx* x) {
  Fp32Engine& e = x->e32;
  const int nx = x->s.nx, ny = x->s.ny;
  for (int w : {3, 0})
    if (x->forced & (1u << w)) {
      halo_wrap(force_target(x, w), nx, ny, x->stream);
      fp32_reshadow(x, w);
    }
  fp32_channel(x);
  add_row_ref(x->d_tmp, e.eta[e.cur], x->d_ref, nx, ny, x->stream);  // eta itself, for its range check
  const double* f[4];
  int nf = 0;
  if (e.tracer) f[nf++] = e.tr[e.cur];
  f[nf++] = x->d_tmp;
  f[nf++] = e.u[e.cur];
  f[nf++] = e.v[e.cur];
  CK(cudaMemsetAsync(x->d_bad, 0, sizeof(int), x->stream));
  fp64_range(x->s, f, nf, x->d_bad, x->stream);
  CK(cudaEventRecord(x->ev[1], x->stream));
  CK(cudaGetLastError());
  x->open = false;
  unsigned* const cfl = x->h_cfl32;
  int* const bad = x->h_bad;
  CK(cudaMemcpyAsync(cfl, e.cfl + 2 * x->open_slot, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaMemcpyAsync(bad, e.bad + x->open_slot, sizeof(int), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaMemcpyAsync(bad + 1, x->d_bad, sizeof(int), cudaMemcpyDeviceToHost, x->stream));
  sw2g_status gst = gauss_queue_check(x);
  if (gst != SW2G_OK) return gst;
  CK(cudaStreamSynchronize(x->stream));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, x->ev[0], x->ev[1]));
  x->last_step_ms = ms;
  if (x->timers.on) x->timers.collect();
  if (gauss_failed(x)) {  // the reference stops inside add_Gaussians (perturbs.c:316-326)
    x->err_step = (int)x->steps;
    return SW2G_ERR_FORCING;
  }
  float a, b2;
  std::memcpy(&a, &cfl[0], sizeof(float));
  std::memcpy(&b2, &cfl[1], sizeof(float));
  double mx = a, my = b2;
  if (mx + my == 0) { mx = x->rest_mx; my = x->rest_my; }
  if (x->c.Dt > (x->c.courant / (mx + my))) {  // core.c:158
    x->err_step = (int)x->steps;
    return SW2G_ERR_CFL;
  }
  x->steps += 1;
  if (bad[0] & kCheckTimeout) {
    x->err_step = (int)(x->steps - 1);
    return SW2G_ERR_TIMEOUT;
  }
  if (bad[1]) {
    x->err_step = (int)(x->steps - 1);
    return SW2G_ERR_NONFINITE;
  }
  return SW2G_OK;
}
}  // namespace

sw2g_status sw2g_step_open(sw2g_ctx* x) {
  if (!x) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded || x->open) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  if (x->precision == SW2G_FP32) return fp32_step_open(x);
  CK(cudaMemsetAsync(x->d_cfl, 0, sizeof(unsigned long long) * 2, x->stream));
  CK(cudaMemsetAsync(x->d_bad, 0, sizeof(int), x->stream));
  StepChecks chk{x->d_cfl, x->d_bad};
  CK(cudaEventRecord(x->ev[0], x->stream));
  x->last_launches = fp64_step(x->s, x->b, x->sch, x->k, x->tracer_active, chk, 0, x->stream, &x->timers, STEP_HEAD);
  CK(cudaGetLastError());
  x->k++;
  x->open = true;
  return SW2G_OK;
}

sw2g_status sw2g_step_close(sw2g_ctx* x) {
  if (!x) return SW2G_ERR_BAD_ARG;
  if (!x->open) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  if (x->precision == SW2G_FP32) return fp32_step_close(x);
  StepChecks chk{x->d_cfl, x->d_bad};
  x->last_launches += fp64_step(x->s, x->b, x->sch, x->k - 1, x->tracer_active, chk, 0, x->stream, &x->timers,
                                STEP_TAIL);
  CK(cudaEventRecord(x->ev[1], x->stream));
  CK(cudaGetLastError());
  x->open = false;
  unsigned long long* const cfl = x->h_cfl;
  int* const bad = x->h_bad;
  CK(cudaMemcpyAsync(cfl, x->d_cfl, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaMemcpyAsync(bad, x->d_bad, sizeof(int), cudaMemcpyDeviceToHost, x->stream));
  sw2g_status gst = gauss_queue_check(x);
  if (gst != SW2G_OK) return gst;
  CK(cudaStreamSynchronize(x->stream));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, x->ev[0], x->ev[1]));
  x->last_step_ms = ms;
  if (x->timers.on) x->timers.collect();
  if (gauss_failed(x)) {  // the reference stops inside add_Gaussians (perturbs.c:316-326)
    x->err_step = (int)x->steps;
    return SW2G_ERR_FORCING;
  }
  double mx, my;
  std::memcpy(&mx, &cfl[0], sizeof(double));
  std::memcpy(&my, &cfl[1], sizeof(double));
  if (mx + my == 0) { mx = x->rest_mx; my = x->rest_my; }
  if (x->c.Dt > (x->c.courant / (mx + my))) {  // core.c:158
    x->err_step = (int)x->steps;
    return SW2G_ERR_CFL;
  }
  x->steps += 1;
  if (bad[0]) {
    x->err_step = (int)(x->steps - 1);
    return SW2G_ERR_NONFINITE;
  }
  return SW2G_OK;
}

int sw2g_error_step(const sw2g_ctx* x) { return x ? x->err_step : -1; }
long long sw2g_steps_done(const sw2g_ctx* x) { return x ? x->steps : 0; }
long long sw2g_last_launches(const sw2g_ctx* x) { return x ? x->last_launches : 0; }

sw2g_status sw2g_download(sw2g_ctx* x, double* eta, double* u, double* v, double* tracer) {
  if (!x) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  const size_t bytes = sizeof(double) * (size_t)x->s.W * x->s.H;
  double* dst[4] = {eta, u, v, tracer};
  if (x->precision == SW2G_FP32) {
    const Fp32Engine& e = x->e32;
    if (eta) {
      add_row_ref(x->d_tmp, e.eta[e.cur], x->d_ref, x->s.nx, x->s.ny, x->stream);
      CK(cudaMemcpyAsync(eta, x->d_tmp, bytes, cudaMemcpyDeviceToHost, x->stream));
    }
    if (u) CK(cudaMemcpyAsync(u, e.u[e.cur], bytes, cudaMemcpyDeviceToHost, x->stream));
    if (v) CK(cudaMemcpyAsync(v, e.v[e.cur], bytes, cudaMemcpyDeviceToHost, x->stream));
    if (tracer) {
      if (e.tracer) CK(cudaMemcpyAsync(tracer, e.tr[e.cur], bytes, cudaMemcpyDeviceToHost, x->stream));
      else std::memset(tracer, 0, bytes);
    }
    CK(cudaStreamSynchronize(x->stream));
    return SW2G_OK;
  }
  for (int q = 0; q < 4; q++)
    if (dst[q]) CK(cudaMemcpyAsync(dst[q], x->b.f[q], bytes, cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  return SW2G_OK;
}

sw2g_status sw2g_diag(sw2g_ctx* x, double* ke, double* ape, double* mass) {
  if (!x) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  const double* f[7];
  if (x->precision == SW2G_FP32) {
    const Fp32Engine& e = x->e32;
    add_row_ref(x->d_tmp, e.eta[e.cur], x->d_ref, x->s.nx, x->s.ny, x->stream);
    f[0] = x->d_tmp;
    f[1] = e.u[e.cur];
    f[2] = e.v[e.cur];
    f[3] = x->d_aux64[0];  // not read by the energy sum
    f[4] = x->d_aux64[0];
    f[5] = x->d_aux64[1];
    f[6] = x->d_aux64[2];
  } else {
    for (int q = 0; q < 7; q++) f[q] = x->b.f[q];
  }
  energy_rows(x->s, f, x->d_energy, x->stream);
  energy_sum(x->d_energy, x->s.ny, x->d_energy + 3 * (size_t)x->s.ny, x->stream);
  double h[3];
  CK(cudaMemcpyAsync(h, x->d_energy + 3 * (size_t)x->s.ny, sizeof(h), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  if (ke) *ke = h[0];
  if (ape) *ape = h[1];
  if (mass) *mass = h[2];
  return SW2G_OK;
}

sw2g_status sw2g_test_tile_timeout(sw2g_ctx* x, int waits) {
  if (!x || x->precision != SW2G_FP32 || waits < 0) return SW2G_ERR_BAD_ARG;
  x->c32.tile_test = waits;
  return SW2G_OK;
}

sw2g_status sw2g_reset_ab(sw2g_ctx* x) {
  if (!x) return SW2G_ERR_BAD_ARG;
  x->k = 0;
  return SW2G_OK;
}

namespace {
constexpr size_t kCkpHeader = 8;  // format, nx, ny, k, tracer flag, 3 spare
constexpr double kCkpFormat = 1.0;
// The checkpoint's device arrays in buffer order: seven fields, then the
// histories D(n-1), D(n-2) of eta, u, v, tracer (slots 1 and 2 after a step).
void ckp_arrays(sw2g_ctx* x, double* a[15]) {
  Fp64Buffers& b = x->b;
  for (int q = 0; q < 7; q++) a[q] = b.f[q];
  double** h[4] = {b.deta, b.du, b.dv, b.dtr};
  for (int f = 0; f < 4; f++) {
    a[7 + 2 * f] = h[f][1];
    a[8 + 2 * f] = h[f][2];
  }
}
}  // namespace

size_t sw2g_checkpoint_doubles(const sw2g_ctx* x) {
  if (!x || x->precision != SW2G_FP64) return 0;
  return kCkpHeader + 15 * (size_t)x->s.W * x->s.H;
}

sw2g_status sw2g_checkpoint_save(sw2g_ctx* x, double* buf, size_t n) {
  if (!x || !buf || x->precision != SW2G_FP64 || n != sw2g_checkpoint_doubles(x)) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded || x->open) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  const size_t S = (size_t)x->s.W * x->s.H;
  double* a[15];
  ckp_arrays(x, a);
  for (int q = 0; q < 15; q++)
    CK(cudaMemcpyAsync(buf + kCkpHeader + q * S, a[q], S * sizeof(double), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  const double head[kCkpHeader] = {kCkpFormat, (double)x->s.nx, (double)x->s.ny, (double)x->k,
                                   x->tracer_active ? 1.0 : 0.0, 0.0, 0.0, 0.0};
  std::memcpy(buf, head, sizeof head);
  return SW2G_OK;
}

sw2g_status sw2g_checkpoint_load(sw2g_ctx* x, const double* buf, size_t n) {
  if (!x || !buf || x->precision != SW2G_FP64 || n != sw2g_checkpoint_doubles(x)) return SW2G_ERR_BAD_ARG;
  if (x->open) return SW2G_ERR_STATE;
  if (buf[0] != kCkpFormat || buf[1] != (double)x->s.nx || buf[2] != (double)x->s.ny || !(buf[3] >= 0) ||
      !(buf[3] <= 1e9) || (buf[4] != 0.0 && buf[4] != 1.0))
    return SW2G_ERR_BAD_ARG;
  CK(cudaSetDevice(x->device));
  const size_t S = (size_t)x->s.W * x->s.H;
  double* a[15];
  ckp_arrays(x, a);
  for (int q = 0; q < 15; q++)
    CK(cudaMemcpyAsync(a[q], buf + kCkpHeader + q * S, S * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  CK(cudaStreamSynchronize(x->stream));
  // the plain form of the bodies depends on the winds and the bottom
  for (int q = 4; q < 7; q++) {
    bool z = true;
    const double* f = buf + kCkpHeader + q * S;
    for (size_t t = 0; t < S && z; t++) {
      uint64_t bits;
      std::memcpy(&bits, &f[t], sizeof(bits));
      z = (bits == 0);
    }
    x->aux_zero[q - 4] = z;
  }
  x->s.plain = x->aux_zero[0] && x->aux_zero[1] && x->aux_zero[2];
  x->k = (int)buf[3];
  x->tracer_active = (buf[4] != 0.0);
  x->steps = 0;
  x->err_step = -1;
  x->uploaded = true;
  return SW2G_OK;
}

namespace {
// Forcing calls are for uploaded contexts; the staging field is allocated on
// first use. In the FP32 form a forced tracer is advected from then on.
sw2g_status force_ready(sw2g_ctx* x, int which) {
  if (!x || which < 0 || which > 3) return SW2G_ERR_BAD_ARG;
  if (!x->uploaded) return SW2G_ERR_STATE;
  CK(cudaSetDevice(x->device));
  if (!x->d_force) {
    sw2g_status st = dalloc(x, &x->d_force, (size_t)x->s.W * x->s.H);
    if (st != SW2G_OK) return st;
  }
  if (x->precision == SW2G_FP32 && which == 3 && !x->e32.tracer) {
    Fp32Engine& e = x->e32;
    sw2g_status st = tracer_fp32(x);
    if (st != SW2G_OK) return st;
    const size_t S = (size_t)x->s.W * x->s.H, S32 = (size_t)x->c32.P * x->c32.R;
    CK(cudaMemsetAsync(e.tr[e.cur], 0, S * sizeof(double), x->stream));
    CK(cudaMemsetAsync(e.ts[e.cur], 0, S32 * sizeof(float), x->stream));
    e.tracer = true;
  }
  return SW2G_OK;
}


// After a forcing call: the FP32 form refreshes the shadow at once between
// steps, or at sw2g_step_close inside an opened step.
void forced_field(sw2g_ctx* x, int which) {
  if (x->precision != SW2G_FP32) return;
  if (x->open) x->forced |= 1u << which;
  else fp32_reshadow(x, which);
}

// FP32 form, setting eta: the values are heights, the state holds eta - eta_ref(j).
double eta_ref_of_cell(const sw2g_ctx* x, int q) { return x->ref[q / x->s.W]; }
}  // namespace

sw2g_status sw2g_add_field(sw2g_ctx* x, int which, const double* delta, double scale) {
  sw2g_status st = force_ready(x, which);
  if (st != SW2G_OK) return st;
  if (!delta) return SW2G_ERR_BAD_ARG;
  const size_t S = (size_t)x->s.W * x->s.H;
  CK(cudaMemcpyAsync(x->d_force, delta, S * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  fp64_add_scaled(force_target(x, which), x->d_force, scale, x->s.nx, x->s.ny, x->stream);
  forced_field(x, which);
  CK(cudaGetLastError());
  if (which == 3 && !x->tracer_active) {
    // the tracer step runs once any interior tracer value can be nonzero
    for (int j = 1; j <= x->s.ny && !x->tracer_active; j++)
      for (int i = 1; i <= x->s.nx; i++)
        if (delta[(i + 1) + (size_t)(j + 1) * x->s.W] != 0.0 || std::signbit(delta[(i + 1) + (size_t)(j + 1) * x->s.W])) {
          x->tracer_active = true;
          break;
        }
  }
  CK(cudaStreamSynchronize(x->stream));
  return SW2G_OK;
}

sw2g_status sw2g_set_field_where(sw2g_ctx* x, int which, const double* value, const unsigned char* mask) {
  sw2g_status st = force_ready(x, which);
  if (st != SW2G_OK) return st;
  if (!value || !mask) return SW2G_ERR_BAD_ARG;
  const size_t S = (size_t)x->s.W * x->s.H;
  if (!x->d_mask) CK(cudaMalloc(&x->d_mask, S));
  std::vector<double> pert;
  if (x->precision == SW2G_FP32 && which == 0) {  // heights -> eta - eta_ref(j)
    pert.resize(S);
    for (size_t q = 0; q < S; q++) pert[q] = value[q] - eta_ref_of_cell(x, (int)q);
  }
  CK(cudaMemcpyAsync(x->d_force, pert.empty() ? value : pert.data(), S * sizeof(double), cudaMemcpyHostToDevice,
                     x->stream));
  CK(cudaMemcpyAsync(x->d_mask, mask, S, cudaMemcpyHostToDevice, x->stream));
  fp64_set_where(force_target(x, which), x->d_force, (const unsigned char*)x->d_mask, x->s.nx, x->s.ny, x->stream);
  forced_field(x, which);
  CK(cudaGetLastError());
  if (which == 3 && !x->tracer_active) {
    for (int j = 1; j <= x->s.ny && !x->tracer_active; j++)
      for (int i = 1; i <= x->s.nx; i++) {
        const size_t q = (i + 1) + (size_t)(j + 1) * x->s.W;
        if (mask[q] && (value[q] != 0.0 || std::signbit(value[q]))) {
          x->tracer_active = true;
          break;
        }
      }
  }
  CK(cudaStreamSynchronize(x->stream));
  return SW2G_OK;
}

namespace {
// Checks a cell list (strictly increasing padded indices of interior cells)
// and queues its copy to the device through the next staging slot; returns
// with d_cells/d_cellv holding the list in stream order.
sw2g_status stage_cells(sw2g_ctx* x, const int* cells, const double* values, int n) {
  const DevState& s = x->s;
  if (n < 0 || (long long)n > (long long)s.nx * s.ny) return SW2G_ERR_BAD_ARG;
  if (n > 0 && (!cells || !values)) return SW2G_ERR_BAD_ARG;
  for (int k = 0; k < n; k++) {
    const int q = cells[k], j = q / s.W - 1, i = q - (j + 1) * s.W - 1;
    if (q < 0 || i < 1 || i > s.nx || j < 1 || j > s.ny) return SW2G_ERR_BAD_ARG;
    if (k > 0 && q <= cells[k - 1]) return SW2G_ERR_BAD_ARG;
  }
  if (!x->d_delta) {
    sw2g_status st = dalloc(x, &x->d_delta, (size_t)s.W * s.H);  // zeroed
    if (st != SW2G_OK) return st;
  }
  if (n == 0) return SW2G_OK;
  if ((size_t)n > x->d_cell_cap) {  // grows rarely: cudaFree orders itself after the queued work
    if (x->d_cells) CK(cudaFree(x->d_cells));
    if (x->d_cellv) CK(cudaFree(x->d_cellv));
    x->d_cells = nullptr;
    x->d_cellv = nullptr;
    x->d_cell_cap = 0;
    CK(cudaMalloc((void**)&x->d_cells, sizeof(int) * (size_t)n));
    CK(cudaMalloc((void**)&x->d_cellv, sizeof(double) * (size_t)n));
    x->d_cell_cap = (size_t)n;
  }
  auto& sl = x->cell_slot[x->cell_next];
  x->cell_next = (x->cell_next + 1) % 8;
  if (!sl.done) CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
  if (sl.pending) CK(cudaEventSynchronize(sl.done));  // the copy that last used this slot
  sl.pending = false;
  if ((size_t)n > sl.cap) {
    if (sl.idx) CK(cudaFreeHost(sl.idx));
    if (sl.val) CK(cudaFreeHost(sl.val));
    sl.idx = nullptr;
    sl.val = nullptr;
    sl.cap = 0;
    CK(cudaHostAlloc((void**)&sl.idx, sizeof(int) * (size_t)n, cudaHostAllocDefault));
    CK(cudaHostAlloc((void**)&sl.val, sizeof(double) * (size_t)n, cudaHostAllocDefault));
    sl.cap = (size_t)n;
  }
  std::memcpy(sl.idx, cells, sizeof(int) * (size_t)n);
  std::memcpy(sl.val, values, sizeof(double) * (size_t)n);
  CK(cudaMemcpyAsync(x->d_cells, sl.idx, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, x->stream));
  CK(cudaMemcpyAsync(x->d_cellv, sl.val, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, x->stream));
  CK(cudaEventRecord(sl.done, x->stream));
  sl.pending = true;
  return SW2G_OK;
}

void tracer_from_list(sw2g_ctx* x, int which, const double* values, int n) {
  if (which != 3 || x->tracer_active) return;
  for (int k = 0; k < n; k++)
    if (values[k] != 0.0 || std::signbit(values[k])) {
      x->tracer_active = true;
      return;
    }
}
}  // namespace

sw2g_status sw2g_add_cells(sw2g_ctx* x, int which, const int* cells, const double* values, int n, double scale) {
  sw2g_status st = force_ready(x, which);
  if (st != SW2G_OK) return st;
  if ((st = stage_cells(x, cells, values, n)) != SW2G_OK) return st;
  // every interior cell gets field += scale * delta, as the reference's loop
  // over the whole grid does (perturbs.c:308), with delta zero off the list
  fp64_scatter_cells(x->d_delta, x->d_cells, x->d_cellv, n, x->stream);
  fp64_add_scaled(force_target(x, which), x->d_delta, scale, x->s.nx, x->s.ny, x->stream);
  fp64_scatter_cells(x->d_delta, x->d_cells, nullptr, n, x->stream);
  forced_field(x, which);
  CK(cudaGetLastError());
  tracer_from_list(x, which, values, n);
  return SW2G_OK;
}

sw2g_status sw2g_set_cells(sw2g_ctx* x, int which, const int* cells, const double* values, int n) {
  sw2g_status st = force_ready(x, which);
  if (st != SW2G_OK) return st;
  std::vector<double> pert;
  if (x->precision == SW2G_FP32 && which == 0 && n > 0 && cells && values) {  // heights -> eta - eta_ref(j)
    pert.resize((size_t)n);
    for (int k = 0; k < n; k++) pert[k] = values[k] - eta_ref_of_cell(x, cells[k]);
  }
  if ((st = stage_cells(x, cells, pert.empty() ? values : pert.data(), n)) != SW2G_OK) return st;
  fp64_scatter_cells(force_target(x, which), x->d_cells, x->d_cellv, n, x->stream);
  halo_wrap(force_target(x, which), x->s.nx, x->s.ny, x->stream);
  forced_field(x, which);
  CK(cudaGetLastError());
  tracer_from_list(x, which, values, n);
  return SW2G_OK;
}

namespace {
// Tables and scratch of the device Gaussians, made on the first injection.
sw2g_status gauss_ready(sw2g_ctx* x) {
  if (x->d_grows) return SW2G_OK;
  std::vector<double> rows3, lonc;
  forcing_tables(x->c, rows3, x->gpl, lonc);
  sw2g_status st;
  const size_t S = (size_t)x->s.W * x->s.H;
  const size_t nparts = (size_t)((x->s.nx + 127) / 128) * (size_t)x->s.ny;
  if ((st = dalloc(x, &x->d_grows, rows3.size())) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->d_glonc, lonc.size())) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->gs.gp, S)) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->gs.gt, S)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &x->gs.gm, S)) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->gs.part, nparts)) != SW2G_OK) return st;
  if ((st = dalloc(x, &x->gs.rf, 1)) != SW2G_OK) return st;
  if ((st = dalloc32(x, &x->gs.err, 1)) != SW2G_OK) return st;
  CK(cudaHostAlloc((void**)&x->h_gerr, sizeof(int), cudaHostAllocDefault));
  *x->h_gerr = 0;
  CK(cudaMemcpyAsync(x->d_grows, rows3.data(), rows3.size() * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  CK(cudaMemcpyAsync(x->d_glonc, lonc.data(), lonc.size() * sizeof(double), cudaMemcpyHostToDevice, x->stream));
  CK(cudaStreamSynchronize(x->stream));  // the host tables go out of scope
  return SW2G_OK;
}

// Queues the read-back of the device Gaussians' error word (and its reset);
// gauss_failed tells, once the stream is done, whether an injection failed.
sw2g_status gauss_queue_check(sw2g_ctx* x) {
  if (!x->gerr_pending) return SW2G_OK;
  CK(cudaMemcpyAsync(x->h_gerr, x->gs.err, sizeof(int), cudaMemcpyDeviceToHost, x->stream));
  CK(cudaMemsetAsync(x->gs.err, 0, sizeof(int), x->stream));
  return SW2G_OK;
}
bool gauss_failed(sw2g_ctx* x) {
  const bool f = x->gerr_host || (x->gerr_pending && *x->h_gerr != 0);
  x->gerr_pending = false;
  x->gerr_host = false;
  if (x->h_gerr) *x->h_gerr = 0;
  return f;
}
}  // namespace

sw2g_status sw2g_add_gaussian(sw2g_ctx* x, const sw2g_gaussian* g) {
  if (!x || !g) return SW2G_ERR_BAD_ARG;
  if (x->s.polar != 0) return SW2G_ERR_BAD_ARG;  // the reference's Gaussians are placed on the band
  if (!std::isfinite(g->lon) || !std::isfinite(g->lat) || !std::isfinite(g->amp) || !(g->sigma > 0) ||
      !std::isfinite(g->sigma) || std::isnan(g->radius) || !std::isfinite(g->inject) ||
      !std::isfinite(g->volume) || g->images < 0 || g->images > 3)
    return SW2G_ERR_BAD_ARG;
  sw2g_status st = force_ready(x, 0);
  if (st != SW2G_OK) return st;
  if ((st = force_ready(x, 3)) != SW2G_OK) return st;
  if ((st = gauss_ready(x)) != SW2G_OK) return st;
  const sw2g_case& c = x->c;
  const int nx = x->s.nx, ny = x->s.ny;
  GaussJob job{};
  job.nx = nx;
  job.R = (c.rE + c.rP) / 2.0;  // perturbs.c:377
  const double plat = forcing_pclat(c, g->lat);
  job.sp = std::sin(plat);
  job.cp = std::cos(plat);
  job.amp = g->amp;
  job.den = 2.0 * (g->sigma * g->sigma);
  job.radius = g->radius;
  job.inject = g->inject;
  job.volume = g->volume;
  const double span = forcing_lon_span(c);
  job.lon[job.nimg++] = g->lon;
  if (g->images & 1) job.lon[job.nimg++] = g->lon - span;  // lonLeft
  if (g->images & 2) job.lon[job.nimg++] = g->lon + span;  // lonRight
  // Rows that can hold a cell inside the radius: the central angle to the
  // centre is at least the difference of the planetocentric latitudes. The
  // margin covers the rounding of the distance (1e-6 rad against ~1e-15).
  const double th = g->radius / job.R + 1e-6;
  int j0 = 1, j1 = ny;
  if (th < 3.0) {
    j0 = ny + 1;
    j1 = 0;
    for (int j = 1; j <= ny; j++)
      if (std::fabs(x->gpl[j] - plat) <= th) {
        if (j < j0) j0 = j;
        j1 = j;
      }
  }
  if (j0 > j1) {  // no cell can be inside: the tracer and eta keep their values
    if (std::fabs(g->volume) > 1e-7) x->gerr_host = true;  // perturbs.c:316: no volume to rescale
  } else {
    job.j0 = j0;
    job.nrows = j1 - j0 + 1;
    double* eta = force_target(x, 0);
    double* tr = force_target(x, 3);
    gauss_inject(job, x->d_grows, x->d_glonc, x->gs, eta, tr, x->stream);
    CK(cudaGetLastError());
    if (x->precision == SW2G_FP64) {  // the calls end with the halo wrap of the fields
      halo_wrap(eta, nx, ny, x->stream);
      halo_wrap(tr, nx, ny, x->stream);
    }
    forced_field(x, 0);
    forced_field(x, 3);
    x->gerr_pending = true;
    if (g->inject != 0.0 || std::signbit(g->inject)) x->tracer_active = true;
  }
  if (x->open) return SW2G_OK;  // reported by sw2g_step_close
  if ((st = gauss_queue_check(x)) != SW2G_OK) return st;
  CK(cudaStreamSynchronize(x->stream));
  return gauss_failed(x) ? SW2G_ERR_FORCING : SW2G_OK;
}

sw2g_status sw2g_apply_channel(sw2g_ctx* x) {
  sw2g_status st = force_ready(x, 0);
  if (st != SW2G_OK) return st;
  if (x->s.polar != 0) return SW2G_OK;  // periodic in y: the wall loops run over no cells (sppde_core.c:589)
  if (x->precision == SW2G_FP32) {
    fp32_channel(x);
  } else {
    fp64_channel(x->b.f[1], x->b.f[2], x->b.f[4], x->b.f[5], x->s.nx, x->s.ny, x->stream);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(x->stream));
  return SW2G_OK;
}

void* sw2g_device_field(sw2g_ctx* x, int which) {
  if (!x || which < 0 || which > 3) return nullptr;
  if (x->precision == SW2G_FP32) {
    const Fp32Engine& e = x->e32;
    // eta is held as eta - eta_ref(j) in this form; the tracer only while advected
    return which == 0 ? (void*)e.eta[e.cur] : which == 1 ? (void*)e.u[e.cur] : which == 2 ? (void*)e.v[e.cur]
                                                                            : (e.tracer ? (void*)e.tr[e.cur] : nullptr);
  }
  return x->b.f[which];
}

void* sw2g_stream(sw2g_ctx* x) { return x ? (void*)x->stream : nullptr; }

void sw2g_destroy(sw2g_ctx* x) {
  if (!x) return;
  cudaSetDevice(x->device);
  if (x->stream) cudaStreamSynchronize(x->stream);
  for (double* p : x->allocs) cudaFree(p);
  for (void* p : x->allocs32) cudaFree(p);
  if (x->d_cfl) cudaFree(x->d_cfl);
  if (x->d_bad) cudaFree(x->d_bad);
  if (x->d_strips) cudaFree(x->d_strips);
  if (x->d_mask) cudaFree(x->d_mask);
  if (x->d_cells) cudaFree(x->d_cells);
  if (x->d_cellv) cudaFree(x->d_cellv);
  for (auto& sl : x->cell_slot) {
    if (sl.idx) cudaFreeHost(sl.idx);
    if (sl.val) cudaFreeHost(sl.val);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  if (x->h_chk) cudaFreeHost(x->h_chk);
  if (x->h_gerr) cudaFreeHost(x->h_gerr);
  x->timers.release();
  x->run32.release();
  for (int e = 0; e < 2; e++)
    if (x->ev[e]) cudaEventDestroy(x->ev[e]);
  for (int e = 0; e < 7; e++)
    if (x->hev[e]) cudaEventDestroy(x->hev[e]);
  if (x->side) {
    cudaStreamSynchronize(x->side);
    cudaStreamDestroy(x->side);
  }
  if (x->stream) cudaStreamDestroy(x->stream);
  delete x;
}

double sw2g_last_step_ms(const sw2g_ctx* x) { return x ? x->last_step_ms : 0.0; }

sw2g_status sw2g_timers_enable(sw2g_ctx* x, int on) {
  if (!x) return SW2G_ERR_BAD_ARG;
  x->timers.on = (on != 0);
  return SW2G_OK;
}

void sw2g_timers_reset(sw2g_ctx* x) {
  if (x) x->timers.reset();
}

int sw2g_timers_count(const sw2g_ctx* x) { return x ? (int)x->timers.entries().size() : 0; }

sw2g_status sw2g_timer_read(const sw2g_ctx* x, int idx, const char** name, long long* launches, double* total_ms) {
  if (!x || idx < 0 || idx >= (int)x->timers.entries().size()) return SW2G_ERR_BAD_ARG;
  const Timers::Entry& e = x->timers.entries()[idx];
  if (name) *name = e.name;
  if (launches) *launches = e.launches;
  if (total_ms) *total_ms = e.ms;
  return SW2G_OK;
}

}  // extern "C"

extern "C" sw2g_status sw2g_selfcheck_division(const double* divisors, int n, long long samples,
                                              unsigned long long seed, int device, long long* mismatches) {
  if (!divisors || n < 1 || samples < 1 || !mismatches) return SW2G_ERR_BAD_ARG;
  for (int k = 0; k < n; k++)
    if (!(divisors[k] > 0) || !std::isfinite(divisors[k]) || divisors[k] < 1e-300) return SW2G_ERR_BAD_ARG;
  CK(cudaSetDevice(device));
  double* d = nullptr;
  unsigned long long* bad = nullptr;
  cudaStream_t st = nullptr;
  sw2g_status rc = SW2G_OK;
  auto run = [&]() -> sw2g_status {
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaMalloc((void**)&d, sizeof(double) * n));
    CK(cudaMalloc((void**)&bad, sizeof(unsigned long long)));
    CK(cudaMemcpyAsync(d, divisors, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st));
    fp64_check_division(d, n, samples, seed, bad, st);
    CK(cudaGetLastError());
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *mismatches = (long long)h;
    return SW2G_OK;
  };
  rc = run();
  if (d) cudaFree(d);
  if (bad) cudaFree(bad);
  if (st) cudaStreamDestroy(st);
  return rc;
}

extern "C" sw2g_status sw2g_selfcheck_add(long long samples, unsigned long long seed, int device,
                                         long long* mismatches) {
  if (samples < 1 || !mismatches) return SW2G_ERR_BAD_ARG;
  CK(cudaSetDevice(device));
  unsigned long long* bad = nullptr;
  cudaStream_t st = nullptr;
  auto run = [&]() -> sw2g_status {
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaMalloc((void**)&bad, sizeof(unsigned long long)));
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st));
    fp64_check_add(samples, seed, bad, st);
    CK(cudaGetLastError());
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *mismatches = (long long)h;
    return SW2G_OK;
  };
  const sw2g_status rc = run();
  if (bad) cudaFree(bad);
  if (st) cudaStreamDestroy(st);
  return rc;
}

// ------------------------------------------------------------------ batches
struct sw2g_batch {
  std::vector<sw2g_ctx*> mem;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  BatchExec run;
  std::vector<int2> dims;  // members' nx, ny
  int sched = SCHED_ROWS;
  int th = kTileRowsSolo;
  double last_ms = 0;
  long long last_launches = 0;
  int err_member = -1, err_step = -1;
};

namespace {

// Tile shape th rows high and sweep schedule sched: the tile table of the
// members' tiles in that order (the device table holds room for the
// smallest tiles).
sw2g_status batch_set_schedule(sw2g_batch* b, int th, int sched) {
  std::vector<int2> nb;
  for (const int2 d : b->dims) {
    int nbx = 0, nby = 0;
    fp32_tiles(d.x, d.y, th, &nbx, &nby);
    nb.push_back(make_int2(nbx, nby));
  }
  const std::vector<int4> t = tile_table(nb, sched);
  CK(cudaStreamSynchronize(b->stream));  // no queued step reads the table being replaced
  CK(cudaMemcpy(b->run.d_tiles, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice));
  b->run.set_shape(th, (int)t.size(), nb[0].x, nb[0].y);
  b->sched = sched;
  b->th = th;
  return SW2G_OK;
}

}  // namespace

extern "C" {

sw2g_status sw2g_batch_create(sw2g_ctx* const* members, int n, sw2g_batch** out) {
  if (!out || !members || n < 1 || n > SW2G_BATCH_MAX) return SW2G_ERR_BAD_ARG;
  *out = nullptr;
  for (int m = 0; m < n; m++) {
    const sw2g_ctx* x = members[m];
    if (!x || x->precision != SW2G_FP32 || x->device != members[0]->device) return SW2G_ERR_BAD_ARG;
    if (x->c32.sch != members[0]->c32.sch) return SW2G_ERR_BAD_ARG;
    if (x->c32.polar != 0 && n > 1) return SW2G_ERR_BAD_ARG;  // polar caps step alone
    if (!x->uploaded) return SW2G_ERR_STATE;
    for (int q = 0; q < m; q++)
      if (members[q] == x) return SW2G_ERR_BAD_ARG;
  }
  sw2g_batch* b = new (std::nothrow) sw2g_batch();
  if (!b) return SW2G_ERR_NOMEM;
  b->mem.assign(members, members + n);
  b->device = members[0]->device;
  auto fail = [&](sw2g_status e) {
    sw2g_batch_destroy(b);
    return e;
  };
  sw2g_status st;
  if ((st = cuda_fail(cudaSetDevice(b->device), "cudaSetDevice")) != SW2G_OK) return fail(st);
  if ((st = cuda_fail(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream")) != SW2G_OK)
    return fail(st);
  for (int e = 0; e < 2; e++)
    if ((st = cuda_fail(cudaEventCreate(&b->ev[e]), "event")) != SW2G_OK) return fail(st);
  int ntiles = 0;  // for the smallest tiles, the most of them
  for (sw2g_ctx* x : b->mem) {
    int nbx = 0, nby = 0;
    fp32_tiles(x->c32.nx, x->c32.ny, kTileRows[0], &nbx, &nby);
    b->dims.push_back(make_int2(x->c32.nx, x->c32.ny));
    ntiles += nbx * nby;
  }
  if ((st = cuda_fail(b->run.alloc(ntiles), "batch")) != SW2G_OK) return fail(st);
  b->run.sch = members[0]->c32.sch;
  if ((st = batch_set_schedule(b, kTileRowsSolo, SCHED_ROWS)) != SW2G_OK) return fail(st);
  *out = b;
  return SW2G_OK;
}

sw2g_status sw2g_batch_step(sw2g_batch* b, int nsteps) {
  if (!b || nsteps < 0) return SW2G_ERR_BAD_ARG;
  CK(cudaSetDevice(b->device));
  const int M = (int)b->mem.size();
  b->last_ms = 0;
  b->last_launches = 0;
  b->err_member = -1;
  b->err_step = -1;
  std::vector<unsigned> cfl((size_t)M * 2 * kChunk);
  std::vector<int> bad((size_t)M * kChunk);
  int done = 0;
  std::vector<MemberDesc> now(M);
  while (done < nsteps) {
    int n = (nsteps - done) < kChunk ? (nsteps - done) : kChunk;
    for (int m = 0; m < M; m++) now[m] = fp32_desc(b->mem[m]->c32, b->mem[m]->e32, b->mem[m]->k);
    CK(b->run.sync_to(now, b->stream));
    if (n > b->run.room()) n = b->run.room();
    const int slot0 = b->run.slot();
    for (int m = 0; m < M; m++) {
      sw2g_ctx* x = b->mem[m];
      CK(cudaMemsetAsync(x->e32.cfl + 2 * slot0, 0, sizeof(unsigned) * 2 * n, b->stream));
      CK(cudaMemsetAsync(x->e32.bad + slot0, 0, sizeof(int) * n, b->stream));
    }
    CK(cudaEventRecord(b->ev[0], b->stream));
    CK(b->run.enqueue(n, b->stream, nullptr, b->last_launches));
    CK(cudaEventRecord(b->ev[1], b->stream));
    for (int m = 0; m < M; m++) {
      sw2g_ctx* x = b->mem[m];
      CK(cudaMemcpyAsync(&cfl[(size_t)m * 2 * kChunk], x->e32.cfl + 2 * slot0, sizeof(unsigned) * 2 * n,
                         cudaMemcpyDeviceToHost, b->stream));
      CK(cudaMemcpyAsync(&bad[(size_t)m * kChunk], x->e32.bad + slot0, sizeof(int) * n, cudaMemcpyDeviceToHost,
                         b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
    b->last_ms += ms;
    for (sw2g_ctx* x : b->mem) {
      x->e32.advance_host(n);
      x->k += n;
    }
    // first failing step over all members, in step order (compute_Dt then the range check)
    for (int t = 0; t < n && b->err_member < 0; t++) {
      for (int m = 0; m < M; m++) {
        sw2g_ctx* x = b->mem[m];
        float a, c;
        std::memcpy(&a, &cfl[(size_t)m * 2 * kChunk + 2 * t], sizeof(float));
        std::memcpy(&c, &cfl[(size_t)m * 2 * kChunk + 2 * t + 1], sizeof(float));
        double mx = a, my = c;
        if (mx + my == 0) { mx = x->rest_mx; my = x->rest_my; }
        const bool cfl_bad = x->c.Dt > (x->c.courant / (mx + my));
        if (cfl_bad || bad[(size_t)m * kChunk + t]) {
          b->err_member = m;
          b->err_step = done + t;
          x->err_step = (int)(x->steps + t);
          for (sw2g_ctx* y : b->mem) y->steps += (y == x) ? t : n;
          if (cfl_bad) return SW2G_ERR_CFL;
          return (bad[(size_t)m * kChunk + t] & kCheckTimeout) ? SW2G_ERR_TIMEOUT : SW2G_ERR_NONFINITE;
        }
      }
    }
    for (sw2g_ctx* x : b->mem) x->steps += n;
    done += n;
  }
  return SW2G_OK;
}

sw2g_status sw2g_batch_tune(sw2g_batch* b, int steps_per_candidate, double* ms_per_step) {
  if (!b || steps_per_candidate < 1) return SW2G_ERR_BAD_ARG;
  static_assert(SW2G_TILE_SHAPES == kTileShapes && SW2G_SCHEDULES == SCHED_COUNT, "candidates of the header");
  double best = 0;
  int best_th = kTileRowsSolo, best_s = SCHED_ROWS;
  for (int shape = 0; shape < kTileShapes; shape++) {
    for (int s = 0; s < SCHED_COUNT; s++) {
      sw2g_status st = batch_set_schedule(b, kTileRows[shape], s);
      if (st != SW2G_OK) return st;
      // the first steps of a shape capture its graph: one untimed step first
      if (s == 0 && (st = sw2g_batch_step(b, 1)) != SW2G_OK) return st;
      st = sw2g_batch_step(b, steps_per_candidate);
      if (st != SW2G_OK) return st;
      const double ms = b->last_ms / steps_per_candidate;
      if (ms_per_step) ms_per_step[shape * SCHED_COUNT + s] = ms;
      if ((shape == 0 && s == 0) || ms < best) {
        best = ms;
        best_th = kTileRows[shape];
        best_s = s;
      }
    }
  }
  return batch_set_schedule(b, best_th, best_s);
}

sw2g_status sw2g_batch_set_schedule(sw2g_batch* b, int tile_rows, int schedule) {
  if (!b || schedule < 0 || schedule >= SCHED_COUNT) return SW2G_ERR_BAD_ARG;
  bool known = false;
  for (int k = 0; k < kTileShapes; k++) known = known || (kTileRows[k] == tile_rows);
  if (!known) return SW2G_ERR_BAD_ARG;
  CK(cudaSetDevice(b->device));
  return batch_set_schedule(b, tile_rows, schedule);
}

int sw2g_batch_schedule(const sw2g_batch* b) { return b ? b->sched : -1; }
int sw2g_batch_tile_rows(const sw2g_batch* b) { return b ? b->th : -1; }
int sw2g_batch_error_member(const sw2g_batch* b) { return b ? b->err_member : -1; }
int sw2g_batch_error_step(const sw2g_batch* b) { return b ? b->err_step : -1; }
double sw2g_batch_last_step_ms(const sw2g_batch* b) { return b ? b->last_ms : 0.0; }
long long sw2g_batch_last_launches(const sw2g_batch* b) { return b ? b->last_launches : 0; }

void sw2g_batch_destroy(sw2g_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  b->run.release();
  for (int e = 0; e < 2; e++)
    if (b->ev[e]) cudaEventDestroy(b->ev[e]);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // extern "C"
