// Gaussian injections evaluated on the device: get_Gaussian_field (fill mode
// 1, perturbs.c:333-364) for a centre and its periodic images, the injected
// volume summed over the cells inside the radius and the rescale to the
// step's volume (perturbs.c:299-326), eta += rf * pert (perturbs.c:305-309)
// and the tracer set inside the radius (perturbs.c:356).
//
// Compiled with -fmad=false: the products and sums keep the reference's
// operand order and rounding (it is built with -ffp-contract=off); only the
// distance's cos and acos and the Gaussian's exp come from the GPU's FP64
// library, so a cell's values are within a few ulps of the reference's.
// The volume is summed in a fixed order (per block of a row, then over the
// blocks row by row), so a run is reproducible, in another order than the
// reference's loop.
#include "sw2g_internal.h"

namespace sw2g {
namespace {

constexpr int GT = 128;  // threads per block, one cell each along a row

__device__ __forceinline__ int IXg(int W, int i, int j) { return (i + 1) + (j + 1) * W; }

// Sum over the block in a fixed order (warp shuffles, then the warps in order).
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
  return s;
}

// One cell per thread, rows g.j0 .. g.j0 + gridDim.y - 1, every interior
// column. rows: {sin, cos of the planetocentric latc(j), DXC*DYC} for j =
// 0..ny+1; lonc: lonc(i) for i = 0..nx+1. Writes every cell of its rows (a
// cell outside the radius gets zeros), and the block's share of the volume.
__global__ void __launch_bounds__(GT) k_gauss_field(GaussJob g, const double* __restrict__ rows,
                                                    const double* __restrict__ lonc, double* gp, double* gt,
                                                    unsigned char* gm, double* part) {
  __shared__ double sh[GT / 32];
  const int j = g.j0 + blockIdx.y;
  const int i = blockIdx.x * GT + threadIdx.x + 1;
  double contrib = 0.0;
  if (i <= g.nx) {
    const double sj = rows[3 * j], cj = rows[3 * j + 1], lc = lonc[i];
    double p = 0.0, tr = 0.0;
    bool hit = false;
    for (int k = 0; k < g.nimg; k++) {
      // tools.c:104-119 on the mean radius: R*acos(sin*sin + cos*cos*cos(dlon))
      const double r = (g.R) * acos(g.sp * sj + g.cp * cj * cos(lc - g.lon[k]));
      if (r < g.radius) {
        const double e = exp(-(r * r) / g.den);  // exp(-r^2 / (2 sigma^2))
        p += g.amp * e;
        tr = (g.inject) * e;
        hit = true;
      }
    }
    const int q = IXg(g.nx + 4, i, j);
    gp[q] = p;
    gt[q] = tr;
    gm[q] = hit ? 1 : 0;
    contrib = p * rows[3 * j + 2];  // pert * DXC * DYC (perturbs.c:306-309)
  }
  const double s = block_sum(contrib, sh);
  if (threadIdx.x == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// The injected volume (the partial sums in order), the rescale factor
// rf = volume / V (perturbs.c:299-304) and the reference's check of the
// rescaled volume (perturbs.c:310-326, here rf * V). |volume| <= 1e-7: rf = 0
// (no rescale; eta is left unchanged). Failures set *err (1: V = 0, 2: the
// rescaled volume off by more than 10 %).
__global__ void __launch_bounds__(256) k_gauss_total(const double* part, int n, double volume, double* rf,
                                                    int* err) {
  __shared__ double sh[8];
  double v = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v += part[k];
  const double V = block_sum(v, sh);
  if (threadIdx.x == 0) {
    double f = 0.0;
    if (fabs(volume) > 1e-7) {
      if (V == 0.0) {
        *err = 1;
      } else {
        f = volume / V;
        const double Vc = f * V;
        if (fabs(Vc - volume) / volume > 1e-1) *err = 2;
      }
    }
    *rf = f;
  }
}

// eta += rf * pert and tracer = inject * exp(...) inside the radius.
__global__ void __launch_bounds__(GT) k_gauss_apply(GaussJob g, const double* __restrict__ gp,
                                                    const double* __restrict__ gt,
                                                    const unsigned char* __restrict__ gm, const double* rf,
                                                    double* eta, double* tracer) {
  const int j = g.j0 + blockIdx.y;
  const int i = blockIdx.x * GT + threadIdx.x + 1;
  if (i > g.nx) return;
  const int q = IXg(g.nx + 4, i, j);
  if (!gm[q]) return;
  const double f = *rf;
  if (f != 0.0) eta[q] += f * gp[q];
  tracer[q] = gt[q];
}

}  // namespace

void gauss_inject(const GaussJob& g, const double* rows, const double* lonc, GaussScratch& sc, double* eta,
                  double* tracer, cudaStream_t st) {
  const int bx = (g.nx + GT - 1) / GT;
  constexpr int kMaxRows = 65535;  // grid y limit; the partial sums stay in row order across chunks
  for (int r0 = 0; r0 < g.nrows; r0 += kMaxRows) {
    GaussJob c = g;
    c.j0 = g.j0 + r0;
    c.nrows = (g.nrows - r0 < kMaxRows) ? g.nrows - r0 : kMaxRows;
    k_gauss_field<<<dim3(bx, c.nrows), GT, 0, st>>>(c, rows, lonc, sc.gp, sc.gt, sc.gm, sc.part + (size_t)r0 * bx);
  }
  k_gauss_total<<<1, 256, 0, st>>>(sc.part, bx * g.nrows, g.volume, sc.rf, sc.err);
  for (int r0 = 0; r0 < g.nrows; r0 += kMaxRows) {
    GaussJob c = g;
    c.j0 = g.j0 + r0;
    c.nrows = (g.nrows - r0 < kMaxRows) ? g.nrows - r0 : kMaxRows;
    k_gauss_apply<<<dim3(bx, c.nrows), GT, 0, st>>>(c, sc.gp, sc.gt, sc.gm, sc.rf, eta, tracer);
  }
}

}  // namespace sw2g
