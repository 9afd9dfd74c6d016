// Energy diagnostic that allocates nothing (sw2g_energy_noalloc, include/sw2g.h).
//
// sw2g_diag sums the energy through per-row partials kept in a buffer that the
// context allocates. Some callers have fields on the GPU but cannot let a
// library allocate: a host loop whose device memory is fully reserved by its
// own pool allocator, a step loop where cudaMalloc/cudaFree would synchronise
// the device in the middle of a time step, or a post-processing tool that owns
// its field buffers and never creates a sw2g context. For them this variant
// keeps its scratch (the row partials) in one file-scope __device__ array of
// fixed size, so the call needs no cudaMalloc, cudaFree or any other
// allocating routine.
//
// The per-row geometry (area element and gravity) is computed on the host with
// the same expressions as the context's tables and travels to the GPU inside
// the kernel parameters, in chunks of kRowsPerLaunch rows: no host buffer is
// copied and nothing waits for the stream, so a call only queues work.
#include <cuda_runtime.h>

#include <cstdio>

#include "sw2g_internal.h"

namespace sw2g {
void energy_row_geometry(const sw2g_case& c, int j0, int n, double* surf, double* gc);
}

namespace {

// Rows whose geometry one launch carries in its parameters (16 KiB).
constexpr int kRowsPerLaunch = 1024;

struct RowGeometry {
  double surf[kRowsPerLaunch];  // DXC*DYC (energy.c:40)
  double gc[kRowsPerLaunch];    // GC, gravity at the cell centre (init.c:289)
};
static_assert(sizeof(RowGeometry) + 128 <= 32760, "kernel parameters are limited to 32 KB");

// Scratch of the no-allocation energy sum: three compensated partials per
// interior row (3 * SW2G_NOALLOC_MAX_ROWS doubles, 192 KiB). Every GPU on
// which the library's module is loaded holds this array until the process
// exits.
__device__ __align__(256) double g_energy_scratch[3 * SW2G_NOALLOC_MAX_ROWS];

// Device address of g_energy_scratch on the current device. In host code the
// symbol itself is only a host-side stand-in, never a device address, so the
// kernels are given the address looked up here. The lookup is repeated on
// every call (it allocates nothing and costs a table lookup once the module is
// loaded), so a device reset or a reloaded module never leaves a stale pointer.
cudaError_t scratch_on_current_device(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_energy_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<double*>(p);
  return cudaSuccess;
}

__device__ __forceinline__ int IXn(int W, int i, int j) { return (i + 1) + (j + 1) * W; }

// One block per interior row j = j0 + blockIdx.x; the same per-cell terms
// (energy.c:36-41) and the same compensated summation order as sw2g_diag.
__global__ void k_energy_rows_noalloc(int nx, int j0, double depth, const double* eta, const double* u,
                                      const double* v, const double* wx, const double* wy, const double* hb,
                                      const __grid_constant__ RowGeometry geo, double* part) {
  const int W = nx + 4;
  const int j = j0 + blockIdx.x;
  const double surf = geo.surf[blockIdx.x], gc = geo.gc[blockIdx.x];
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

__global__ void k_energy_sum_noalloc(int ny, const double* part, double* out3) {
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
  // the grid checks of sw2g_create: sizes, 32-bit cell indices, the poles
  if (!sw2g::grid_ok(c)) return SW2G_ERR_BAD_ARG;
  if (c->polar != 0) return SW2G_ERR_BAD_ARG;  // its gravity is two-dimensional: sw2g_diag covers caps
  if (c->ny > SW2G_NOALLOC_MAX_ROWS) {
    fprintf(stderr,
            "sw2g_energy_noalloc: ny=%d exceeds the fixed scratch of this entry point (at most %d rows); "
            "use sw2g_diag instead\n",
            c->ny, SW2G_NOALLOC_MAX_ROWS);
    return SW2G_ERR_BAD_ARG;
  }
  double* part = nullptr;
  cudaError_t e = scratch_on_current_device(&part);
  if (e != cudaSuccess) {
    fprintf(stderr, "sw2g_energy_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
    return SW2G_ERR_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Each call rewrites the partials of rows 1..ny before the sum reads them,
  // so nothing in the scratch needs clearing first. The geometry is part of
  // each launch's parameters, copied when the launch is queued.
  RowGeometry geo;
  for (int j0 = 1; j0 <= c->ny; j0 += kRowsPerLaunch) {
    const int n = (c->ny - j0 + 1) < kRowsPerLaunch ? (c->ny - j0 + 1) : kRowsPerLaunch;
    sw2g::energy_row_geometry(*c, j0, n, geo.surf, geo.gc);
    k_energy_rows_noalloc<<<n, 256, 0, st>>>(c->nx, j0, c->depth, eta, u, v, windx, windy, hB, geo, part);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
  }
  if (e == cudaSuccess) {
    k_energy_sum_noalloc<<<1, 32, 0, st>>>(c->ny, part, out3);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "sw2g_energy_noalloc: launch: %s\n", cudaGetErrorString(e));
    return SW2G_ERR_CUDA;
  }
  return SW2G_OK;
}
