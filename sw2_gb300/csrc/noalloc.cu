// Energy diagnostic that allocates nothing (sw2g_energy_noalloc, include/sw2g.h).
//
// sw2g_diag sums the energy through per-row partials kept in a buffer that the
// context allocates. Some callers have fields on the GPU but cannot let a
// library allocate: a host loop whose device memory is fully reserved by its
// own pool allocator, a step loop where cudaMalloc/cudaFree would synchronise
// the device in the middle of a time step, or a post-processing tool that owns
// its field buffers and never creates a sw2g context. For them this variant
// keeps its scratch (per-row geometry and row partials) in one file-scope
// __device__ array of fixed size, so the call needs no cudaMalloc, cudaFree or
// any other allocating routine.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "sw2g_internal.h"

namespace sw2g {
void energy_row_geometry(const sw2g_case& c, int j0, int n, double* surf, double* gc);
}

namespace {

constexpr int kMaxDevices = 64;
constexpr int kStage = 256;  // rows of geometry staged on the host stack per copy

// Scratch for the no-allocation energy sum: per interior row, the area element
// and gravity (2 * SW2G_NOALLOC_MAX_ROWS doubles), then three row partials
// (3 * SW2G_NOALLOC_MAX_ROWS doubles): 320 KiB in all. Every GPU on which the
// library's module is loaded holds this array until the process exits.
__device__ __align__(256) double g_energy_scratch[5 * SW2G_NOALLOC_MAX_ROWS];

// Device address of g_energy_scratch per device, looked up once per device.
// In host code the symbol itself is only a host-side stand-in, never a device
// address, so kernels are always given this looked-up pointer.
double* g_scratch_addr[kMaxDevices];
std::mutex g_setup;

cudaError_t scratch_on_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_energy_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

__device__ __forceinline__ int IXn(int W, int i, int j) { return (i + 1) + (j + 1) * W; }

// One block per interior row; the same per-cell terms (energy.c:36-41) and the
// same compensated summation order as sw2g_diag.
__global__ void k_energy_rows_noalloc(int nx, int ny, double depth, const double* eta, const double* u,
                                      const double* v, const double* wx, const double* wy, const double* hb,
                                      const double* scratch) {
  const int W = nx + 4;
  const int j = blockIdx.x + 1;
  const double* surf_rows = scratch;
  const double* gc_rows = scratch + SW2G_NOALLOC_MAX_ROWS;
  double* part = const_cast<double*>(scratch) + 2 * SW2G_NOALLOC_MAX_ROWS;
  const double surf = surf_rows[j - 1], gc = gc_rows[j - 1];
  double acc[3] = {0, 0, 0}, cmp[3] = {0, 0, 0};
  for (int i = threadIdx.x + 1; i <= nx; i += blockDim.x) {
    const int q = IXn(W, i, j), qw = IXn(W, i - 1, j), qs = IXn(W, i, j - 1);
    const double wxq = wx ? wx[q] : 0.0, wxw = wx ? wx[qw] : 0.0;
    const double wyq = wy ? wy[q] : 0.0, wys = wy ? wy[qs] : 0.0;
    const double hbq = hb ? hb[q] : 0.0;
    const double uc = 0.5 * ((u[q] + wxq) + (u[qw] + wxw));
    const double vc = 0.5 * ((v[q] + wyq) + (v[qs] + wys));
    const double h = eta[q] + depth - hbq;
    const double term[3] = {0.5 * h * (uc * uc + vc * vc) * surf - 0.5 * ((wxq * wxq) + (wyq * wyq)) * surf,
                            0.5 * gc * (h * h) * surf - 0.5 * gc * (depth * depth) * surf, h * surf};
    for (int c = 0; c < 3; c++) {
      const double t = acc[c] + term[c];
      cmp[c] += (fabs(acc[c]) >= fabs(term[c])) ? ((acc[c] - t) + term[c]) : ((term[c] - t) + acc[c]);
      acc[c] = t;
    }
  }
  __shared__ double sh[3][2][256];
  for (int c = 0; c < 3; c++) {
    sh[c][0][threadIdx.x] = acc[c];
    sh[c][1][threadIdx.x] = cmp[c];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int c = threadIdx.x;
    double a = 0, e = 0;
    for (int t = 0; t < (int)blockDim.x; t++) {
      const double term = sh[c][0][t];
      const double s = a + term;
      e += (fabs(a) >= fabs(term)) ? ((a - s) + term) : ((term - s) + a);
      a = s;
      e += sh[c][1][t];
    }
    part[3 * (j - 1) + c] = a + e;
  }
}

__global__ void k_energy_sum_noalloc(int ny, const double* scratch, double* out3) {
  const double* part = scratch + 2 * SW2G_NOALLOC_MAX_ROWS;
  const int c = threadIdx.x;
  if (c >= 3) return;
  double a = 0, e = 0;
  for (int j = 0; j < ny; j++) {
    const double term = part[3 * j + c];
    const double s = a + term;
    e += (fabs(a) >= fabs(term)) ? ((a - s) + term) : ((term - s) + a);
    a = s;
  }
  out3[c] = a + e;
}

}  // namespace

extern "C" sw2g_status sw2g_energy_noalloc(const sw2g_case* c, const double* eta, const double* u,
                                           const double* v, const double* windx, const double* windy,
                                           const double* hB, double* out3, void* stream) {
  if (!c || !eta || !u || !v || !out3) return SW2G_ERR_BAD_ARG;
  if (c->nx < 3 || c->ny < 3 || !(c->rE > 0) || !(c->rP > 0) || !(c->lon1 > c->lon0) || !(c->lat1 > c->lat0))
    return SW2G_ERR_BAD_ARG;
  if (c->flags & ~(SW2G_FLAG_VANLEER_SAFE | SW2G_FLAG_RADIANS | SW2G_FLAG_SIGMA | SW2G_FLAG_LAPE_ETA))
    return SW2G_ERR_BAD_ARG;
  if (c->polar != 0) return SW2G_ERR_BAD_ARG;  // its gravity is two-dimensional: sw2g_diag covers caps
  if (c->ny > SW2G_NOALLOC_MAX_ROWS) {
    fprintf(stderr,
            "sw2g_energy_noalloc: ny=%d exceeds the fixed scratch of this entry point (at most %d rows); "
            "use sw2g_diag instead\n",
            c->ny, SW2G_NOALLOC_MAX_ROWS);
    return SW2G_ERR_BAD_ARG;
  }
  double* scratch = nullptr;
  cudaError_t e = scratch_on_current_device(&scratch);
  if (e != cudaSuccess) {
    fprintf(stderr, "sw2g_energy_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
    return SW2G_ERR_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Per-row geometry, staged through a small buffer on the host stack. Each
  // call rewrites rows 0..ny-1 of the geometry and of the partials before
  // reading them, so nothing in the scratch needs clearing first.
  double stage[2][kStage];
  for (int j0 = 1; j0 <= c->ny; j0 += kStage) {
    const int n = (c->ny - j0 + 1) < kStage ? (c->ny - j0 + 1) : kStage;
    sw2g::energy_row_geometry(*c, j0, n, stage[0], stage[1]);
    e = cudaMemcpyAsync(scratch + (j0 - 1), stage[0], sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(scratch + SW2G_NOALLOC_MAX_ROWS + (j0 - 1), stage[1], sizeof(double) * n,
                          cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the stage buffer is reused next round
    if (e != cudaSuccess) {
      fprintf(stderr, "sw2g_energy_noalloc: geometry copy: %s\n", cudaGetErrorString(e));
      return SW2G_ERR_CUDA;
    }
  }
  k_energy_rows_noalloc<<<c->ny, 256, 0, st>>>(c->nx, c->ny, c->depth, eta, u, v, windx, windy, hB, scratch);
  k_energy_sum_noalloc<<<1, 32, 0, st>>>(c->ny, scratch, out3);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "sw2g_energy_noalloc: launch: %s\n", cudaGetErrorString(e));
    return SW2G_ERR_CUDA;
  }
  return SW2G_OK;
}
