// FP32 precision form of the SW2 step: strip kernels (device code and the
// launch helpers shared by step_fp32.cu and step_fp32_limiters.cu).
//
// Same algorithm and step order as the reference (core.c:134-338), including
// its halo and wall semantics, but the stencils, limiters and Laplacians run
// in FP32 while the state is accumulated in FP64:
//   * eta is kept in FP64 as a perturbation about a per-row reference profile
//     (the zonal mean of the uploaded eta), so the FP32 stencil sees small
//     numbers and row-to-row differences of the reference are exact FP64
//     differences rounded once;
//   * u, v are FP64; each step adds an FP32 increment to them in FP64;
//   * the Adams-Bashforth histories and the intermediate fields are FP32.
// Kernels of one step:
//   kb_tracer: tracer advection, AB and update (calc.c:117-163, core.c:161-182),
//              only for members with an active tracer;
//   kb_lap1  : first Laplacian level of (u, v) (laplacian.c:51-111) -> L, with
//              the reference's halo images and wall fixes;
//   kb_main1 : mass sweep + AB + geofactor -> eta (calc.c:70-113, 403-422),
//              second Laplacian level from L, momentum advection and
//              dissipation -> partial tendencies, CFL maxima;
//   kb_lap3  : third Laplacian level (nu6), added to the partial tendencies;
//   kb_main2 : pressure, AB, semi-implicit Coriolis u then v (calc.c:500-598),
//              halo images and do_channel (calc.c:600-649) of u and v.
//
// Work decomposition. A strip is 128 columns (one warp, four consecutive
// cells per lane) by `SR` rows; a warp marches down its strip row by row.
// Each row of each FP32 input field (the strip's 128 columns plus four on
// either side) is fetched by the TMA engine with one 2-D tensor copy into a
// per-warp ring of shared-memory rows, completed on that ring slot's
// mbarrier; copies run up to two rows ahead of the row being computed. Lanes
// read their four cells with one 16-byte shared load and their x neighbours
// with two 8-byte loads. The y faces of the TVD sweeps and the intermediate
// zeta/divergence rows of the Laplacians are carried from row to row in
// registers. Warps take strips from a queue (the launch's last warp resets it),
// so a launch has at most as many blocks as are resident.
//
// Every face value is computed with the same operations wherever it is
// evaluated (carried, recomputed at a strip's first row, or on either side of
// a lane or strip boundary): the file is compiled without contraction and the
// fused multiply-adds are written out, so results do not depend on the strip
// height, the sweep order or the batch a member is stepped in.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sw2g_internal.h"

namespace sw2g {
namespace f32 {

constexpr int SW = kStripWidth;  // strip width in cells: a warp, four cells per lane
constexpr int NWARP = 4;         // warps (independent strips) per block
constexpr int NT = 32 * NWARP;
constexpr int BOXW = SW + 8;     // staged row: columns i0-4 .. i0+SW+3
constexpr int ROWB = BOXW * 4;   // bytes of one staged row
constexpr int RS = 160;          // floats per ring slot row: 640 bytes, keeping every copy 128-byte aligned
constexpr unsigned FULL = 0xffffffffu;
// Ring depths (staged rows per warp): kb_main1 and kb_tracer read rows j-1..j+2
// for row j and prefetch one row; kb_main2 reads j..j+1 and prefetches two;
// the Laplacian kernels, whose rows are short, prefetch three.
constexpr int kDMain1 = 5, kDMain2 = 4, kDLap = 5;
constexpr int NONE = INT_MIN;
static_assert(ROWB % 16 == 0, "tensor rows are whole 16-byte units");
static_assert((RS * 4) % 128 == 0 && RS >= BOXW, "tensor copies land on 128-byte boundaries");

// Layout of the FP32 arrays: column i at offset i + 3 (interior column 1 on a
// 16-byte boundary), row j at j + 1, row pitch P (a multiple of 4).
__host__ __device__ __forceinline__ int IX32(int P, int i, int j) { return (i + 3) + (j + 1) * P; }
__device__ __forceinline__ int IX(int W, int i, int j) { return (i + 1) + (j + 1) * W; }

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ float Qr(const float* q, int t, int j) { return __ldg(q + (j + 1) * Q_NUM + t); }

// The bit pattern of a double through an opaque move, so that tests on it
// stay integer operations instead of being turned back into FP64 compares.
__device__ __forceinline__ long long dbits(double x) {
  long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}

// FP64 <-> FP32 conversions on the integer pipe. On GB300 the hardware
// conversions issue on the FP64 unit, whose throughput (~1/64 of FP32) would
// otherwise bound these kernels; here only the state additions use it.
// d2f: round to nearest (ties away), magnitudes below 2^-126 flush to zero,
// overflow gives inf, NaN stays NaN.
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long b = (unsigned long long)dbits(x);
  const unsigned long long mag = b & 0x7fffffffffffffffULL;
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  unsigned r;
  if (mag < (897ULL << 52)) r = 0u;
  else if (mag >= (1151ULL << 52)) r = (mag > (2047ULL << 52)) ? 0x7fc00000u : 0x7f800000u;
  else r = (unsigned)(((mag + (1ULL << 28)) >> 29) - (896ULL << 23));
  return __uint_as_float(r | sign);
}
__device__ __forceinline__ float d2f(float x) { return x; }

// The hardware conversions (cvt on the FP64 unit), for a kernel whose FP64
// unit is otherwise nearly idle: kb_main1 issues on two thirds of its cycles
// with the FP64 unit busy on under a tenth of them, and runs 2-5 % faster
// with these than with the integer-pipe forms; kb_main2, whose FP64 unit
// carries two state additions per cell, runs slower with them.
__device__ __forceinline__ double f2d_unit(float f) { return (double)f; }
__device__ __forceinline__ float d2f_unit(double x) { return __double2float_rn(x); }

// f2d: exact widening; FP32 subnormals flush to zero.
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  unsigned long long r;
  if (e == 0u) r = 0ULL;
  else if (e == 255u) r = 0x7ff0000000000000ULL | ((unsigned long long)(b & 0x7fffffu) << 29);
  else r = ((unsigned long long)(b & 0x7fffffffu) << 29) + (896ULL << 52);
  r |= (unsigned long long)(b & 0x80000000u) << 32;
  return __longlong_as_double((long long)r);
}

// |x| <= 1e10 and not NaN, tested on the bits (the reference's range check,
// sppde_core.c:386-395, without an FP64 compare).
__device__ __forceinline__ bool in_range(double x) {
  const unsigned long long mag = (unsigned long long)dbits(x) & 0x7fffffffffffffffULL;
  return mag <= 0x4202a05f20000000ULL;  // bits of 1e10
}

// ------------------------------------------------------------------ limiters
// calc.c:54-63 in FP32; SCH 10 is Van Leer with the limit 0 at r = -1.
template <int SCH>
__device__ __forceinline__ float psi(float r) {
  if constexpr (SCH == 0) return fmaxf(0.f, fminf(fminf((1.f + r) * 0.5f, 2.f * r), 2.f));
  else if constexpr (SCH == 1) return fmaxf(fmaxf(0.f, fminf(2.f * r, 1.f)), fmaxf(0.f, fminf(r, 2.f)));
  else if constexpr (SCH == 2) return (r < 1.f) ? r : 1.f;
  else if constexpr (SCH == 3) return (r + fabsf(r)) / (1.f + r);
  else if constexpr (SCH == 4) return fmaxf(0.f, fminf(2.f * r, fminf(fmaf(2.f, r, 1.f) * (1.f / 3.f), 2.f)));
  else if constexpr (SCH == 5) {
    const float rr = fmaf(r, r, r);
    return __fdividef(1.5f * rr, rr + 1.f);
  } else if constexpr (SCH == 6) return __fdividef(fmaf(r, r, r), fmaf(r, r, 1.f));
  else if constexpr (SCH == 7) return fmaxf(0.f, fminf(fminf(2.f, 2.f * r), fminf(fmaf(0.75f, r, 0.25f), fmaf(0.25f, r, 0.75f))));
  else if constexpr (SCH == 8) return 0.f;
  else if constexpr (SCH == 9) return 1.f;
  else return (r > 0.f) ? __fdividef(2.f * r, 1.f + r) : 0.f;
}

constexpr float kTiny = 1.17549435e-38f;  // differences below the smallest normal count as zero

// One upwind face with a single Courant number c (mass): c*B of calc.c:41-49,100
// with B_P (c > 0) or B_M (c < 0) reconstructed from q0|q1, outer neighbours qm, q2.
template <int SCH>
__device__ __forceinline__ float face1(float qm, float q0, float q1, float q2, float c) {
  const float d = q1 - q0;
  const bool pos = c > 0.f;
  const float n = pos ? (q0 - qm) : (q2 - q1);
  const float r = (d != 0.f) ? __fdividef(n, d) : 0.f;
  const float x = ((pos ? 0.5f : -0.5f) * psi<SCH>(r)) * (1.f - fabsf(c));
  return c * fmaf(x, d, pos ? q0 : q1);
}

// A face with both split Courant numbers (momentum and tracer bodies, calc.c:170-177).
template <int SCH>
__device__ __forceinline__ float face2(float qm, float q0, float q1, float q2, float cP, float cM) {
  const float d = q1 - q0;
  const float inv = (fabsf(d) >= kTiny) ? __fdividef(1.f, d) : 0.f;
  const float rP = (q0 - qm) * inv, rM = (q2 - q1) * inv;
  const float bP = fmaf((0.5f * psi<SCH>(rP)) * (1.f - cP), d, q0);
  const float bM = fmaf(-((0.5f * psi<SCH>(rM)) * (1.f + cM)), d, q1);
  return fmaf(cP, bP, cM * bM);
}

__device__ __forceinline__ float cpos2(float a, float b, float k) { return (0.5f * (fmaxf(a, 0.f) + fmaxf(b, 0.f))) * k; }
__device__ __forceinline__ float cneg2(float a, float b, float k) { return (0.5f * (fminf(a, 0.f) + fminf(b, 0.f))) * k; }

// y faces: the two cells of a face divide by their own row metric, so their
// Courant numbers differ, while the limited slope is shared. For a mass face
// (one Courant number, whose sign is that of v): g = +-psi(r)/2*(q1-q0) and the
// upwind value; the cell's term is c*(base + g*(1-|c|)).
template <int SCH>
__device__ __forceinline__ float2 face1_shared(float qm, float q0, float q1, float q2, bool pos) {
  const float d = q1 - q0;
  const float n = pos ? (q0 - qm) : (q2 - q1);
  const float r = (fabsf(d) >= kTiny) ? __fdividef(n, d) : 0.f;
  return make_float2(((pos ? 0.5f : -0.5f) * psi<SCH>(r)) * d, pos ? q0 : q1);
}
__device__ __forceinline__ float face1_term(float2 gb, float c) { return c * fmaf(gb.x, 1.f - fabsf(c), gb.y); }

// A momentum or tracer y face: gP = psi(rP)/2*(q1-q0), gM = psi(rM)/2*(q1-q0);
// the cell's term is cP*(q0 + gP*(1-cP)) + cM*(q1 - gM*(1+cM)).
template <int SCH>
__device__ __forceinline__ float2 face2_shared(float qm, float q0, float q1, float q2) {
  const float d = q1 - q0;
  const float inv = (fabsf(d) >= kTiny) ? __fdividef(1.f, d) : 0.f;
  return make_float2((0.5f * psi<SCH>((q0 - qm) * inv)) * d, (0.5f * psi<SCH>((q2 - q1) * inv)) * d);
}
__device__ __forceinline__ float face2_term(float2 g, float q0, float q1, float cP, float cM) {
  return fmaf(cP, fmaf(g.x, 1.f - cP, q0), cM * fmaf(-g.y, 1.f + cM, q1));
}

__device__ __forceinline__ float ab3(int k, float d, float h1, float h2) {
  if (k == 0) return d;
  if (k == 1) return fmaf(1.5f, d, -0.5f * h1);
  return fmaf(23.f / 12.f, d, fmaf(-4.f / 3.f, h1, (5.f / 12.f) * h2));
}

// ---------------------------------------------------------- halo images
enum Img { IMG_ETA, IMG_U, IMG_V, IMG_LU, IMG_LV };

// Writes the value of interior cell (i,j) and every halo cell whose final
// value in the reference comes from it: the single-rank halo update
// (sppde_hupdate.c:274-342, y pass then x pass) followed by do_channel for
// u and v (calc.c:600-649) or the wall fixes of laplacian_vels
// (laplacian.c:94-107). OFF is the array's column offset (1 for the FP64
// arrays in the reference layout, 3 for the FP32 arrays).
template <Img M, int OFF, typename T>
__device__ __forceinline__ void put1(T* f, int pitch, int nx, int ny, int i, int j, T val) {
  auto at = [&](int ii, int jj) -> T& { return f[(ii + OFF) + (jj + 1) * pitch]; };
  const T zero = T(0);
  at(i, j) = (M == IMG_V && j == ny) ? zero : val;
  const int xa = (i <= 2) ? i + nx : NONE, xb = (i >= nx - 1) ? i - nx : NONE;
  const int ya = (j <= 2) ? j + ny : NONE, yb = (j >= ny - 1) ? j - ny : NONE;
  if (xa != NONE) at(xa, j) = val;
  if (xb != NONE) at(xb, j) = val;
  if (ya != NONE) {
    if (xa != NONE) at(xa, ya) = val;
    if (xb != NONE) at(xb, ya) = val;
  }
  if (yb != NONE) {
    if (xa != NONE) at(xa, yb) = val;
    if (xb != NONE) at(xb, yb) = val;
  }
  if constexpr (M == IMG_ETA) {
    if (ya != NONE) at(i, ya) = val;
    if (yb != NONE) at(i, yb) = val;
  } else if constexpr (M == IMG_U) {
    if (j == 1) { at(i, 0) = val; at(i, -1) = val; }
    if (j == ny) { at(i, ny + 1) = val; at(i, ny + 2) = val; }
  } else if constexpr (M == IMG_V) {
    if (j == 1) { at(i, 0) = zero; at(i, -1) = zero; }
    if (j == ny) { at(i, ny + 1) = zero; at(i, ny + 2) = zero; }
  } else {
    if (j == 2) at(i, ny + 2) = val;
    if (j == ny - 1) at(i, -1) = val;
    if (j == 1) at(i, 0) = (M == IMG_LU) ? val : zero;
    if (j == ny) at(i, ny + 1) = (M == IMG_LU) ? val : zero;
  }
}

// The lane's cells near an edge, with their images.
template <Img M, int OFF, typename T>
__device__ __forceinline__ void put4_edge(T* f, int pitch, int nx, int ny, int i, int j, T v0, T v1, T v2, T v3) {
  if (i <= nx) put1<M, OFF>(f, pitch, nx, ny, i, j, v0);
  if (i + 1 <= nx) put1<M, OFF>(f, pitch, nx, ny, i + 1, j, v1);
  if (i + 2 <= nx) put1<M, OFF>(f, pitch, nx, ny, i + 2, j, v2);
  if (i + 3 <= nx) put1<M, OFF>(f, pitch, nx, ny, i + 3, j, v3);
}

// The four cells (i..i+3, j) of a lane with their images; cells beyond nx
// are not written. Cells with no images are stored with vector stores.
template <Img M, int OFF, typename T>
__device__ __forceinline__ void put4(T* f, int pitch, int nx, int ny, int i, int j, const T (&v)[4]) {
  if (i > 2 && i + 3 < nx - 1 && j > 2 && j < ny - 1) {
    T* p = f + (i + OFF) + (j + 1) * pitch;
    if constexpr (sizeof(T) == 4) {
      *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
        reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
      } else {
        p[0] = v[0]; p[1] = v[1]; p[2] = v[2]; p[3] = v[3];
      }
    }
    return;
  }
  put4_edge<M, OFF, T>(f, pitch, nx, ny, i, j, v[0], v[1], v[2], v[3]);
}

// FP64 values of the lane's four cells (pitch W); cells beyond nx read 0.
__device__ __forceinline__ void ld4d(const double* f, int W, int nx, int i, int j, double (&v)[4]) {
  const double* p = f + IX(W, i, j);
  if (i + 3 <= nx) {
    if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
      const double2 a = __ldg(reinterpret_cast<const double2*>(p));
      const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
      v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    } else {
#pragma unroll
      for (int c = 0; c < 4; c++) v[c] = __ldg(p + c);
    }
  } else {
#pragma unroll
    for (int c = 0; c < 4; c++) v[c] = (i + c <= nx) ? __ldg(p + c) : 0.0;
  }
}
// FP32 values of the lane's four cells: one aligned 16-byte load (the FP32
// arrays are padded, so the columns beyond nx are in bounds).
__device__ __forceinline__ float4 ld4f(const float* f, int P, int i, int j) {
  return __ldg(reinterpret_cast<const float4*>(f + IX32(P, i, j)));
}
__device__ __forceinline__ void st4f(float* f, int P, int i, int j, const float (&v)[4]) {
  *reinterpret_cast<float4*>(f + IX32(P, i, j)) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void arr(float4 a, float (&v)[4]) { v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; }

// ------------------------------------------------------ staged row windows
// A staged row holds columns i0-4 .. i0+SW+3 (smem index s <-> column i0-4+s).
// win8: columns ib-2 .. ib+5 of the lane (ib = i0 + 4*lane), i.e. w[c+2] is
// the lane's cell c; own4: the lane's four cells.
__device__ __forceinline__ void win8(const float* r, float (&w)[8]) {
  const int l = lane_id();
  const float2 a = *reinterpret_cast<const float2*>(r + 4 * l + 2);
  const float4 b = *reinterpret_cast<const float4*>(r + 4 * l + 4);
  const float2 c = *reinterpret_cast<const float2*>(r + 4 * l + 8);
  w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y; w[4] = b.z; w[5] = b.w; w[6] = c.x; w[7] = c.y;
}
__device__ __forceinline__ void own4(const float* r, float (&w)[4]) {
  const float4 b = *reinterpret_cast<const float4*>(r + 4 * lane_id() + 4);
  w[0] = b.x; w[1] = b.y; w[2] = b.z; w[3] = b.w;
}
template <int K>
__device__ __forceinline__ void addw(float (&w)[K], const float (&x)[K], float s) {
#pragma unroll
  for (int m = 0; m < K; m++) w[m] = fmaf(s, x[m], w[m]);
}

// ------------------------------------------------------------- row rings
// Bounded waits: each try suspends the thread for at most TILE_WAIT_HINT_NS,
// so a wait gives up after about 1.3 s; a warp that gives up sets
// CHECK_TIMEOUT in the step's check word (SW2G_ERR_TIMEOUT on the host),
// waits (again bounded) for its copies in flight and leaves the launch.
constexpr int TILE_WAIT_LIMIT = 1 << 16;
constexpr int TILE_DRAIN_LIMIT = 1 << 12;
constexpr unsigned TILE_WAIT_HINT_NS = 20000;
constexpr int CHECK_TIMEOUT = kCheckTimeout;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool phase_wait(unsigned bar, unsigned parity, int limit) {
  unsigned done = 0;
  for (int it = 0; it < limit && !done; it++) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, "
        "p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity), "r"(TILE_WAIT_HINT_NS)
        : "memory");
  }
  return done != 0;
}

// A warp's ring of D staged rows of NF fields. Row t of a strip (t = 0, 1, ...
// in order) goes to slot (base + t) % D; `base` counts the rows of the warp's
// earlier strips, so barrier phases continue across strips without re-init.
template <int NF, int D>
struct Ring {
  float* buf;               // [D][NF][BOXW]
  unsigned long long* bar;  // [D]
  unsigned long long map[NF];  // generic addresses of the fields' tensor maps
  int x, y0, T;             // tensor column and row of the strip's row 0, rows of the strip
  int base, issued;

  __device__ __forceinline__ const float* row(int t, int f) const {
    return buf + (((base + t) % D) * NF + f) * RS;
  }
  // lane 0: one tensor copy per field of row t into its slot
  __device__ __forceinline__ void issue(int t) const {
    const int s = (base + t) % D;
    const unsigned b = smem_u32(&bar[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(NF * ROWB) : "memory");
#pragma unroll
    for (int f = 0; f < NF; f++) {
      const unsigned dst = smem_u32(buf + (s * NF + f) * RS);
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
          "[%4];" ::"r"(dst),
          "l"(map[f]), "r"(x), "r"(y0 + t), "r"(b)
          : "memory");
    }
  }
  __device__ __forceinline__ bool try_row(int t, int limit) const {
    const int g = base + t;
    return phase_wait(smem_u32(&bar[g % D]), (unsigned)((g / D) & 1), limit);
  }
};

// Dynamic shared memory of a block: the warps' barriers, then their rings,
// from a 128-byte boundary (the launch adds 128 bytes of slack).
template <int D>
__host__ __device__ constexpr int bar_bytes() { return (NWARP * D * 8 + 127) / 128 * 128; }

// The block's dynamic shared memory from its first 128-byte boundary.
__device__ __forceinline__ unsigned char* smem_base(unsigned char* sm) {
  return sm + ((128u - (smem_u32(sm) & 127u)) & 127u);
}

// Carves the warp's ring out of the block's dynamic shared memory (the
// blocks' barriers of this ring at bar_off, their rows at row_off, both
// byte offsets from smem_base) and initialises its barriers (one arrival
// each: the expect_tx of lane 0).
template <int NF, int D>
__device__ __forceinline__ void ring_init_at(unsigned char* a, int bar_off, int row_off, Ring<NF, D>& r) {
  const int w = threadIdx.x >> 5;
  r.bar = reinterpret_cast<unsigned long long*>(a + bar_off) + w * D;
  r.buf = reinterpret_cast<float*>(a + row_off) + w * D * NF * RS;
  r.base = 0;
  r.issued = 0;
  if (lane_id() == 0) {
    for (int s = 0; s < D; s++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&r.bar[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
}
template <int NF, int D>
__device__ __forceinline__ void ring_init(unsigned char* sm, Ring<NF, D>& r) {
  ring_init_at(smem_base(sm), 0, bar_bytes<D>(), r);
}

// Starts a strip: the first min(D, T) rows. The slots were last read with
// generic loads, so the async proxy is fenced behind them first.
template <int NF, int D>
__device__ __forceinline__ void ring_begin(Ring<NF, D>& r) {
  __syncwarp();
  const int n = r.T < D ? r.T : D;
  if (lane_id() == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int t = 0; t < n; t++) r.issue(t);
  }
  r.issued = n;
}
// Row t is no longer read: its slot takes row t + D.
template <int NF, int D>
__device__ __forceinline__ void ring_refill(Ring<NF, D>& r, int t) {
  if (t + D < r.T) {
    __syncwarp();
    if (lane_id() == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      r.issue(t + D);
    }
    r.issued = t + D + 1;
  }
}
// Waits for row t; false (and the timeout flag set) if the warp gave up.
template <int NF, int D>
__device__ __forceinline__ bool ring_wait(const Ring<NF, D>& r, int t, int* bad) {
  const bool ok = r.try_row(t, TILE_WAIT_LIMIT);
  if (__all_sync(FULL, ok)) return true;
  if (lane_id() == 0) atomicOr(bad, CHECK_TIMEOUT);
  for (int u = t; u < r.issued; u++) r.try_row(u, TILE_DRAIN_LIMIT);
  return false;
}
// Failure-path test: after row 0 has arrived, also wait for the next phase
// of its slot, which nothing completes before row D is issued; gives up
// after `waits` tries like a real timeout.
template <int NF, int D>
__device__ __forceinline__ bool ring_test(const Ring<NF, D>& r, int waits, int* bad) {
  const int g = r.base;
  const bool ok = phase_wait(smem_u32(&r.bar[g % D]), (unsigned)(((g / D) & 1) ^ 1), waits);
  if (__all_sync(FULL, ok)) return true;
  if (lane_id() == 0) atomicOr(bad, CHECK_TIMEOUT);
  for (int u = 0; u < r.issued; u++) r.try_row(u, TILE_DRAIN_LIMIT);
  return false;
}
template <int NF, int D>
__device__ __forceinline__ void ring_end(Ring<NF, D>& r) {
  r.base += r.T;
}

// ------------------------------------------------ own-cell staging (cp.async)
// The own-cell inputs of a row (FP64 state, FP32 histories) are copied by
// each lane into a per-warp double-buffered staging area with cp.async one
// row ahead, and each lane waits for its own copies a row later
// (cp.async.wait_group): the loads are issued a full row before their use
// without holding registers.
__device__ __forceinline__ void cpa16(unsigned dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
// 8 bytes, or 8 zero bytes (nothing read) when !ok
__device__ __forceinline__ void cpa8(unsigned dst, const void* src, bool ok) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(ok ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cpa4(unsigned dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpa_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cpa_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// The lane's four FP64 cells of row j (pitch W), cells beyond nx as zeros.
__device__ __forceinline__ void cpa_d4(unsigned dst, const double* f, int W, int nx, int i, int j) {
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const bool ok = (i + c <= nx);
    cpa8(dst + 8 * c, ok ? f + IX(W, i + c, j) : f, ok);
  }
}

// ------------------------------------------------------------ strip queue
// Warps take strips in the order of the launch's strip table until none is
// left; the last warp of the launch to find the queue empty resets it
// (queue[0] next strip, queue[1] warps done), so the next launch starts at 0.
__device__ __forceinline__ int take_strip(unsigned* queue) {
  unsigned v = 0;
  if (lane_id() == 0) v = atomicAdd(&queue[0], 1u);
  return (int)__shfl_sync(FULL, v, 0);
}
__device__ __forceinline__ void warp_done(unsigned* queue) {
  if (lane_id() == 0) {
    const unsigned total = gridDim.x * NWARP;
    if (atomicAdd(&queue[1], 1u) == total - 1) {
      atomicExch(&queue[0], 0u);
      atomicExch(&queue[1], 0u);
    }
  }
}

// ------------------------------------------- Laplacian pieces (laplacian.c)
// Operands of the wrapped ZE(0, j) = ZE(nx, j) and DI(nx+1, j) = DI(1, j) at
// their source columns (only the strips at the seam need them).
__device__ __forceinline__ float4 ze_source(const float* gU, const float* gV, int P, int nx, int j) {
  return make_float4(gV[IX32(P, nx + 1, j)], gV[IX32(P, nx, j)], gU[IX32(P, nx, j + 1)], gU[IX32(P, nx, j)]);
}
__device__ __forceinline__ float4 di_source(const float* gU, const float* gV, int P, int j) {
  return make_float4(gU[IX32(P, 1, j)], gU[IX32(P, 0, j)], gV[IX32(P, 1, j)], gV[IX32(P, 1, j - 1)]);
}

// ZE(i, j) at columns ib-1+k, k = 0..4 (laplacian.c:77-79): zero outside rows
// 1..ny and beyond column nx; ZE(0, j) is the wrapped ZE(nx, j), evaluated at
// its source column from the global arrays gU, gV (pitch P). ua, ub: u rows j,
// j+1; va: v row j (windows).
// A polar cap has no walls: its halo rows wrap, so ZE(i, 0) is ZE(i, ny),
// evaluated at its source row from the global arrays.
template <bool POLAR = false>
__device__ __forceinline__ void ze5(const float* q, int nx, int ny, int P, int ib, int j, const float (&ua)[8],
                                    const float (&ub)[8], const float (&va)[8], const float* gU, const float* gV,
                                    float (&ze)[5]) {
  if constexpr (POLAR) {
    if (j == 0) {
      const float idxv = Qr(q, Q_IDXV, ny), idyc = Qr(q, Q_IDYC, ny + 1);
      const float dxc1 = Qr(q, Q_DXC, ny + 1), dxc0 = Qr(q, Q_DXC, ny);
#pragma unroll
      for (int k = 0; k < 5; k++) {
        const int i = ib - 1 + k, is = (i == 0) ? nx : i;
        float z = 0.f;
        if (i <= nx) {
          const float v1 = gV[IX32(P, is + 1, ny)], v0 = gV[IX32(P, is, ny)];
          const float u1 = gU[IX32(P, is, ny + 1)], u0 = gU[IX32(P, is, ny)];
          z = idxv * ((v1 - v0) - idyc * (dxc1 * u1 - dxc0 * u0));
        }
        ze[k] = z;
      }
      return;
    }
  }
  const bool rowok = (j >= 1 && j <= ny);
  const float idxv = Qr(q, Q_IDXV, j), idyc = Qr(q, Q_IDYC, j + 1);
  const float dxc1 = Qr(q, Q_DXC, j + 1), dxc0 = Qr(q, Q_DXC, j);
#pragma unroll
  for (int k = 0; k < 5; k++) {
    const int i = ib - 1 + k;
    float v1 = va[k + 2], v0 = va[k + 1], u1 = ub[k + 1], u0 = ua[k + 1];
    if (i == 0) {
      const float4 g = ze_source(gU, gV, P, nx, j);
      v1 = g.x; v0 = g.y; u1 = g.z; u0 = g.w;
    }
    const float z = idxv * ((v1 - v0) - idyc * (dxc1 * u1 - dxc0 * u0));
    ze[k] = (rowok && i <= nx) ? z : 0.f;
  }
}
// DI(i, jd) at columns ib+k, k = 0..4 (laplacian.c:66-74): rows 1..ny from the
// stencil, DI(nx+1, jd) the wrapped DI(1, jd) from the source column, the
// north wall row ny+1 the difference of u along row ny, zero elsewhere.
// uj, vj: u, v rows jd; vjm, ujm: v, u rows jd-1 (windows).
// A polar cap: DI(i, ny+1) is DI(i, 1), evaluated at its source row.
template <bool POLAR = false>
__device__ __forceinline__ void di5(const float* q, int nx, int ny, int P, int ib, int jd, const float (&uj)[8],
                                    const float (&vj)[8], const float (&vjm)[8], const float (&ujm)[8],
                                    const float* gU, const float* gV, float (&di)[5]) {
  if constexpr (POLAR) {
    if (jd == ny + 1) {
      const float idxe = Qr(q, Q_IDXE, 1), idyn = Qr(q, Q_IDYN, 1);
      const float dxv1 = Qr(q, Q_DXV, 1), dxv0 = Qr(q, Q_DXV, 0);
#pragma unroll
      for (int k = 0; k < 5; k++) {
        const int i = ib + k, is = (i == nx + 1) ? 1 : i;
        float r = 0.f;
        if (i >= 1 && i <= nx + 1) {
          const float uc = gU[IX32(P, is, 1)], uw = gU[IX32(P, is - 1, 1)];
          const float vc = gV[IX32(P, is, 1)], vs = gV[IX32(P, is, 0)];
          r = idxe * ((uc - uw) + idyn * (dxv1 * vc - dxv0 * vs));
        }
        di[k] = r;
      }
      return;
    }
  }
  const bool rowok = (jd >= 1 && jd <= ny), wall = !POLAR && (jd == ny + 1);
  const float idxe = Qr(q, Q_IDXE, jd), idyn = Qr(q, Q_IDYN, jd);
  const float dxv1 = Qr(q, Q_DXV, jd), dxv0 = Qr(q, Q_DXV, jd - 1), idxew = Qr(q, Q_IDXE, ny);
#pragma unroll
  for (int k = 0; k < 5; k++) {
    const int i = ib + k;
    float uc = uj[k + 2], uw = uj[k + 1], vc = vj[k + 2], vs = vjm[k + 2];
    if (i == nx + 1) {
      const float4 g = di_source(gU, gV, P, jd);
      uc = g.x; uw = g.y; vc = g.z; vs = g.w;
    }
    const float dv = idxe * ((uc - uw) + idyn * (dxv1 * vc - dxv0 * vs));
    const float dw = (ujm[k + 2] - ujm[k + 1]) * idxew;
    di[k] = (rowok && i >= 1 && i <= nx + 1) ? dv : ((wall && i >= 1 && i <= nx) ? dw : 0.f);
  }
}
// Second pass at the lane's cells of row j (laplacian.c:83-89): zj = ZE row j
// (columns ib-1..ib+3), zm = ZE row j-1 (ib..ib+3), dj = DI row j (ib..ib+4),
// dn = DI row j+1 (ib..ib+4).
__device__ __forceinline__ void lap_out4(const float* q, int j, const float (&zj)[5], const float (&zm)[4],
                                         const float (&dj)[5], const float (&dn)[5], float (&lu)[4], float (&lv)[4]) {
  const float idyn = Qr(q, Q_IDYN, j), idxc = Qr(q, Q_IDXC, j), idxv = Qr(q, Q_IDXV, j), idyc = Qr(q, Q_IDYC, j + 1);
#pragma unroll
  for (int c = 0; c < 4; c++) {
    lu[c] = -idyn * (zj[c + 1] - zm[c]) + idxc * (dj[c + 1] - dj[c]);
    lv[c] = idxv * (zj[c + 1] - zj[c]) + idyc * (dn[c] - dj[c]);
  }
}

// ------------------------------------------------------------ member views
// One launch per phase covers every strip of every member of a batch (a
// single context is a batch of one). The member descriptors travel by value
// in the launch parameters (the constant bank). Buffer rotation is derived
// from a device step counter n, which a one-thread kernel advances after each
// step, so a captured graph of one step can be replayed for any number of steps.
template <int N>
struct DescSet {
  MemberDesc m[N];
};

struct View {
  int cur, w, h1, h2, slot, k;
};

static_assert((kCheckSlots & (kCheckSlots - 1)) == 0, "check slots are indexed with a mask");
static_assert(kMaxBatch == SW2G_BATCH_MAX, "batch limit of the header");

__device__ __forceinline__ View view_of(const MemberDesc& d, int n) {
  View v;
  v.k = (n >= 2 - d.k0) ? 2 : d.k0 + n;
  v.cur = d.cur0 ^ (n & 1);
  const int r = (int)(((unsigned)d.w0 + (unsigned)n % 3u) % 3u);
  v.w = r;
  v.h1 = (r == 0) ? 2 : r - 1;
  v.h2 = (r == 2) ? 0 : r + 1;
  v.slot = n & (kCheckSlots - 1);
  return v;
}

template <int N>
__device__ __forceinline__ int4 strip_at(const int4* __restrict__ tiles, int s, int nbx) {
  if constexpr (N == 1) return make_int4(0, s % nbx, s / nbx, 0);
  else return tiles[s];
}

__device__ __forceinline__ unsigned long long map_of(const MemberDesc& d, int which) {
  return reinterpret_cast<unsigned long long>(d.tm) + (unsigned long long)which * sizeof(CUtensorMap);
}

// Maxima of the CFL quotients and the range flag of a strip, to the member's slot.
__device__ __forceinline__ void flush_checks(const MemberDesc& d, const View& v, float mxu, float mxv, bool oor) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    mxu = fmaxf(mxu, __shfl_xor_sync(FULL, mxu, s));
    mxv = fmaxf(mxv, __shfl_xor_sync(FULL, mxv, s));
  }
  const bool any = __any_sync(FULL, oor);
  if (lane_id() == 0) {
    if (d.cfl) {
      if (mxu > 0.f) atomicMax(d.cfl + 2 * v.slot, __float_as_uint(mxu));
      if (mxv > 0.f) atomicMax(d.cfl + 2 * v.slot + 1, __float_as_uint(mxv));
    }
    if (any) atomicOr(d.bad + v.slot, 1);
  }
}

// ------------------------------------------------ Laplacian levels of (u, v)
// ACC = false: the first level L of (u, v) (kb_lap1), written with its halo
// images. ACC = true: the Laplacian of the second level LL, i.e. the third
// level LLL (kb_lap3), added as nu6*Dt*LLL to the partial tendencies
// (core.c:233-268). Rows j0-1 .. j1+1 are staged (ring row t <-> j0-1+t).
template <bool ACC, bool POLAR>
__device__ __forceinline__ bool strip_lap(const MemberDesc& d, const View& vw, int sx, int sy, int SR,
                                          Ring<2, kDLap>& rg, bool test) {
  const int nx = d.nx, ny = d.ny, P = d.P;
  const float* q = d.q;
  const int i0 = sx * SW + 1, j0 = sy * SR + 1, j1 = min(j0 + SR - 1, ny);
  const int ib = i0 + 4 * lane_id();
  const float* gU = ACC ? d.LLu : d.us[vw.cur];
  const float* gV = ACC ? d.LLv : d.vs[vw.cur];
  int* bad = d.bad + vw.slot;
  rg.map[0] = map_of(d, ACC ? TM_LLU : TM_US + vw.cur);
  rg.map[1] = map_of(d, ACC ? TM_LLV : TM_VS + vw.cur);
  rg.x = sx * SW;
  rg.y0 = j0;  // tensor row of j0 - 1
  rg.T = j1 - j0 + 3;
  ring_begin(rg);
  if (!ring_wait(rg, 0, bad) || !ring_wait(rg, 1, bad)) return false;
  if (test && !ring_test(rg, d.tile_test, bad)) return false;
  float zm[4], dj[5];
  {
    float ua[8], ub[8], va[8], vb[8], zt[5];
    win8(rg.row(0, 0), ua); win8(rg.row(1, 0), ub);
    win8(rg.row(0, 1), va); win8(rg.row(1, 1), vb);
    ze5<POLAR>(q, nx, ny, P, ib, j0 - 1, ua, ub, va, gU, gV, zt);
#pragma unroll
    for (int c = 0; c < 4; c++) zm[c] = zt[c + 1];
    di5<POLAR>(q, nx, ny, P, ib, j0, ub, vb, va, ua, gU, gV, dj);
  }
  const float nu6dt = d.nu6dt;
  for (int j = j0; j <= j1; j++) {
    const int k = j - j0, t = k + 1;
    ring_refill(rg, k);
    if (!ring_wait(rg, t + 1, bad)) return false;
    float ua[8], ub[8], va[8], vb[8], zj[5], dn[5];
    win8(rg.row(t, 0), ua); win8(rg.row(t + 1, 0), ub);
    win8(rg.row(t, 1), va); win8(rg.row(t + 1, 1), vb);
    ze5<POLAR>(q, nx, ny, P, ib, j, ua, ub, va, gU, gV, zj);
    di5<POLAR>(q, nx, ny, P, ib, j + 1, ub, vb, va, ua, gU, gV, dn);
    float lu[4], lv[4];
    lap_out4(q, j, zj, zm, dj, dn, lu, lv);
    if constexpr (ACC) {
      float* du = d.dup + IX32(P, ib, j);
      float* dv = d.dvp + IX32(P, ib, j);
      float4 a = *reinterpret_cast<float4*>(du), b = *reinterpret_cast<float4*>(dv);
      a.x = fmaf(nu6dt, lu[0], a.x); a.y = fmaf(nu6dt, lu[1], a.y); a.z = fmaf(nu6dt, lu[2], a.z); a.w = fmaf(nu6dt, lu[3], a.w);
      b.x = fmaf(nu6dt, lv[0], b.x); b.y = fmaf(nu6dt, lv[1], b.y); b.z = fmaf(nu6dt, lv[2], b.z); b.w = fmaf(nu6dt, lv[3], b.w);
      *reinterpret_cast<float4*>(du) = a;
      *reinterpret_cast<float4*>(dv) = b;
    } else {
      put4<POLAR ? IMG_ETA : IMG_LU, 3>(d.Lu, P, nx, ny, ib, j, lu);
      put4<POLAR ? IMG_ETA : IMG_LV, 3>(d.Lv, P, nx, ny, ib, j, lv);
    }
#pragma unroll
    for (int c = 0; c < 4; c++) zm[c] = zj[c + 1];
#pragma unroll
    for (int c = 0; c < 5; c++) dj[c] = dn[c];
  }
  ring_end(rg);
  return true;
}

// ---------------------------------------------------------------- kb_main1
// Two rings per warp: rows j0-2 .. j1+2 (ring row t <-> j0-2+t) of the eta,
// u and v shadows, and with EXTRA the winds and the bottom height (UWINDX,
// VWINDY of sw.h:216-217 and H = eta + depth - hB, sw.h:213); and rows
// j0-1 .. j1+1 (ring row t <-> j0-1+t) of the first Laplacian level Lu, Lv,
// of which row j needs only j and j+1.
constexpr int kDLapIn = 3;  // depth of the Laplacian-level ring of kb_main1
template <bool EXTRA>
__host__ __device__ constexpr int main1_fields() { return EXTRA ? 6 : 3; }
template <bool EXTRA>
__host__ __device__ constexpr int main1_bars() {
  return (NWARP * (kDMain1 + kDLapIn) * 8 + 127) / 128 * 128;
}
template <bool EXTRA>
__host__ __device__ constexpr int main1_lrows() {
  return main1_bars<EXTRA>() + NWARP * kDMain1 * main1_fields<EXTRA>() * RS * 4;
}
// own-cell staging of a warp: two rows of [eta (32 lanes x 4 doubles), h1, h2 (32 x 4 floats)]
constexpr int kStageMain1 = 2 * 2048;
template <bool EXTRA>
__host__ __device__ constexpr int main1_stage() {
  return main1_lrows<EXTRA>() + NWARP * kDLapIn * 2 * RS * 4;
}

// Sections of a row are separated by a compiler fence, so that windows are
// read again from shared memory where a section needs them instead of being
// held in registers across the row.
__device__ __forceinline__ void section() { asm volatile("" ::: "memory"); }

template <int SCH, bool EXTRA, bool POLAR>
__device__ __forceinline__ bool strip_main1(const MemberDesc& d, const View& vw, int sx, int sy, int SR,
                                            Ring<main1_fields<EXTRA>(), kDMain1>& rg, Ring<2, kDLapIn>& rl,
                                            unsigned stg, bool test) {
  enum { FE, FU, FV, FWX, FWY, FHB };
  const int nx = d.nx, ny = d.ny, P = d.P, W = nx + 4;
  const float* q = d.q;
  const int i0 = sx * SW + 1, j0 = sy * SR + 1, j1 = min(j0 + SR - 1, ny);
  const int ib = i0 + 4 * lane_id();
  int* bad = d.bad + vw.slot;
  rg.map[FE] = map_of(d, TM_ES + vw.cur);
  rg.map[FU] = map_of(d, TM_US + vw.cur);
  rg.map[FV] = map_of(d, TM_VS + vw.cur);
  if constexpr (EXTRA) {
    rg.map[FWX] = map_of(d, TM_WX);
    rg.map[FWY] = map_of(d, TM_WY);
    rg.map[FHB] = map_of(d, TM_HB);
  }
  rg.x = sx * SW;
  rg.y0 = j0 - 1;  // tensor row of j0 - 2
  rg.T = j1 - j0 + 5;
  rl.map[0] = map_of(d, TM_LU);
  rl.map[1] = map_of(d, TM_LV);
  rl.x = sx * SW;
  rl.y0 = j0;  // tensor row of j0 - 1
  rl.T = j1 - j0 + 3;
  ring_begin(rg);
  ring_begin(rl);
  for (int t = 0; t < 4; t++)
    if (!ring_wait(rg, t, bad)) return false;
  if (!ring_wait(rl, 0, bad) || !ring_wait(rl, 1, bad)) return false;
  if (test && !ring_test(rg, d.tile_test, bad)) return false;

  // windows of the stencil fields, with the winds added to u, v and the
  // bottom height taken from eta when the member has them
  auto E8 = [&](int t, float (&w)[8]) {
    win8(rg.row(t, FE), w);
    if constexpr (EXTRA) { float x[8]; win8(rg.row(t, FHB), x); addw(w, x, -1.f); }
  };
  auto E4 = [&](int t, float (&w)[4]) {
    own4(rg.row(t, FE), w);
    if constexpr (EXTRA) { float x[4]; own4(rg.row(t, FHB), x); addw(w, x, -1.f); }
  };
  auto U8 = [&](int t, float (&w)[8]) {
    win8(rg.row(t, FU), w);
    if constexpr (EXTRA) { float x[8]; win8(rg.row(t, FWX), x); addw(w, x, 1.f); }
  };
  auto U4 = [&](int t, float (&w)[4]) {
    own4(rg.row(t, FU), w);
    if constexpr (EXTRA) { float x[4]; own4(rg.row(t, FWX), x); addw(w, x, 1.f); }
  };
  auto V8 = [&](int t, float (&w)[8]) {
    win8(rg.row(t, FV), w);
    if constexpr (EXTRA) { float x[8]; win8(rg.row(t, FWY), x); addw(w, x, 1.f); }
  };
  auto V4 = [&](int t, float (&w)[4]) {
    own4(rg.row(t, FV), w);
    if constexpr (EXTRA) { float x[4]; own4(rg.row(t, FWY), x); addw(w, x, 1.f); }
  };

  // carried from row to row: the y faces south of the row (mass: limited
  // slope and upwind value relative to the reference of the row below; u, v:
  // limited slopes), ZE of the row below and DI of the row
  float2 ysm[4], ysu[4], ysv[4];
  float zm[4], dj[5];
  {
    const int jm = j0 - 1;
    float ea[4], eb[4], ec[4], ed[4], vb[4];
    E4(0, ea); E4(1, eb); E4(2, ec); E4(3, ed); V4(1, vb);
    const float dm1 = Qr(q, Q_DHBM1, jm), dp1 = Qr(q, Q_DHBP1, jm), dp2 = Qr(q, Q_DHBP2, jm);
#pragma unroll
    for (int c = 0; c < 4; c++) ysm[c] = face1_shared<SCH>(ea[c] + dm1, eb[c], ec[c] + dp1, ed[c] + dp2, vb[c] > 0.f);
    float a[4], b[4], cc[4], dd[4];
    U4(0, a); U4(1, b); U4(2, cc); U4(3, dd);
#pragma unroll
    for (int c = 0; c < 4; c++) ysu[c] = face2_shared<SCH>(a[c], b[c], cc[c], dd[c]);
    V4(0, a); V4(2, cc); V4(3, dd);
#pragma unroll
    for (int c = 0; c < 4; c++) ysv[c] = face2_shared<SCH>(a[c], vb[c], cc[c], dd[c]);
    float la[8], lb[8], ma[8], mb[8], zt[5];
    win8(rl.row(0, 0), la); win8(rl.row(1, 0), lb);
    win8(rl.row(0, 1), ma); win8(rl.row(1, 1), mb);
    ze5<POLAR>(q, nx, ny, P, ib, jm, la, lb, ma, d.Lu, d.Lv, zt);
#pragma unroll
    for (int c = 0; c < 4; c++) zm[c] = zt[c + 1];
    di5<POLAR>(q, nx, ny, P, ib, j0, lb, mb, ma, la, d.Lu, d.Lv, dj);
  }

  const float sig2dt = d.sig2dt, sigdt = d.sigdt, nu2dt = d.nu2dt, nu4dt = d.nu4dt;
  const bool keep_ll = (d.nu6dt != 0.f);
  const int PR = P * (ny + 4);  // stride of a cap's per-cell fields
  const double* eta_in = d.eta[vw.cur];
  double* eta_out = d.eta[1 - vw.cur];
  float* es_out = d.es[1 - vw.cur];
  const float* h1p = d.heta[vw.h1];
  const float* h2p = d.heta[vw.h2];
  float* hw = d.heta[vw.w];
  const int kab = vw.k;
  float mxu = 0.f, mxv = 0.f;
  bool oor = false;
  // own-cell inputs of a row, staged a row ahead (slot k & 1 of the row j0 + k)
  const int l = lane_id();
  auto stage = [&](int jr, int slot) {
    const unsigned b = stg + slot * 2048;
    cpa_d4(b + l * 32, eta_in, W, nx, ib, jr);
    if (kab >= 1) cpa16(b + 1024 + l * 16, h1p + IX32(P, ib, jr));
    if (kab >= 2) cpa16(b + 1536 + l * 16, h2p + IX32(P, ib, jr));
  };
  stage(j0, 0);
  cpa_commit();

  for (int j = j0; j <= j1; j++) {
    const int k = j - j0, t = k + 2;  // ring row of j (the Laplacian ring: k + 1)
    ring_refill(rg, k);
    ring_refill(rl, k);
    if (j < j1) stage(j + 1, (k + 1) & 1);
    cpa_commit();
    if (!ring_wait(rg, t + 2, bad) || !ring_wait(rl, k + 2, bad)) {
      cpa_wait0();
      return false;
    }
    cpa_wait1();  // this lane's copies of row j
    float h1[4] = {0.f, 0.f, 0.f, 0.f}, h2[4] = {0.f, 0.f, 0.f, 0.f};
    double ec[4];
    {
      const unsigned b = stg + (k & 1) * 2048;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        asm volatile("ld.shared.f64 %0, [%1];" : "=d"(ec[c]) : "r"(b + l * 32 + 8 * c) : "memory");
      }
      if (kab >= 1) asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(h1[0]), "=f"(h1[1]), "=f"(h1[2]), "=f"(h1[3]) : "r"(b + 1024 + l * 16) : "memory");
      if (kab >= 2) asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(h2[0]), "=f"(h2[1]), "=f"(h2[2]), "=f"(h2[3]) : "r"(b + 1536 + l * 16) : "memory");
    }

    // ---- mass (BODYH, calc.c:70-113), H relative to the row reference Hb(j)
    {
      float e0[8], u0[8], vm[4], v0[4], em[4], e1[4], e2[4];
      E8(t, e0); U8(t, u0); V4(t - 1, vm); V4(t, v0);
      E4(t - 1, em); E4(t + 1, e1); E4(t + 2, e2);
      const float kx = Qr(q, Q_KXE, j), ky = Qr(q, Q_KYN, j), hb = Qr(q, Q_HB, j), eref = Qr(q, Q_EREF, j);
      const float geo = Qr(q, Q_GEO, j), dm1 = Qr(q, Q_DHBM1, j), dp1 = Qr(q, Q_DHBP1, j), dp2 = Qr(q, Q_DHBP2, j);
      float fx[5];
#pragma unroll
      for (int m = 0; m < 5; m++) fx[m] = face1<SCH>(e0[m], e0[m + 1], e0[m + 2], e0[m + 3], u0[m + 1] * kx);
      float eraw[4];
      if constexpr (EXTRA) own4(rg.row(t, FE), eraw);
      float damp[4] = {sig2dt, sig2dt, sig2dt, sig2dt};  // 2*Dt*sigma; per cell with a cap's sponge
      if constexpr (POLAR) arr(ld4f(d.pf + PQ_SH2 * PR, P, ib, j), damp);
      float hist[4], esn[4];
      double en[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        float2 fs = ysm[c];
        fs.y += dm1;  // the south face's upwind value relative to Hb(j)
        const float2 fn = face1_shared<SCH>(em[c] + dm1, e0[c + 2], e1[c] + dp1, e2[c] + dp2, v0[c] > 0.f);
        ysm[c] = fn;
        const float cw = u0[c + 1] * kx, ce = u0[c + 2] * kx, cs = vm[c] * ky, cn = v0[c] * ky;
        float de = (fx[c] - fx[c + 1]) + (face1_term(fs, cs) - face1_term(fn, cn));
        de = fmaf(hb, (cw - ce) + (cs - cn), de);
        de = fmaf(-damp[c], eref + (EXTRA ? eraw[c] : e0[c + 2]), de);
        // Adams-Bashforth (calc.c:651-699) then the geofactor (calc.c:403-422)
        float ab = ab3(kab, de, h1[c], h2[c]);
        ab = fmaf(-(geo * (hb + e0[c + 2])), 0.5f * (v0[c] + vm[c]), ab);
        hist[c] = de;
        en[c] = ec[c] + f2d_unit(ab);
        esn[c] = d2f_unit(en[c]);
        oor = oor || ((ib + c <= nx) && !in_range(en[c]));
      }
      st4f(hw, P, ib, j, hist);
      put4<IMG_ETA, 1>(eta_out, W, nx, ny, ib, j, en);
      put4<IMG_ETA, 3>(es_out, P, nx, ny, ib, j, esn);
    }
    section();

    // ---- second Laplacian level of (u, v) from L (laplacian.c:51-111),
    // and the hyperviscosity terms nu2*Dt*L + nu4*Dt*LL of both tendencies
    float visu[4], visv[4];
    {
      float la[8], lb[8], ma[8], mb[8], zj[5], dn[5], llu[4], llv[4];
      win8(rl.row(k + 1, 0), la); win8(rl.row(k + 2, 0), lb);
      win8(rl.row(k + 1, 1), ma); win8(rl.row(k + 2, 1), mb);
      ze5<POLAR>(q, nx, ny, P, ib, j, la, lb, ma, d.Lu, d.Lv, zj);
      di5<POLAR>(q, nx, ny, P, ib, j + 1, lb, mb, ma, la, d.Lu, d.Lv, dn);
      lap_out4(q, j, zj, zm, dj, dn, llu, llv);
#pragma unroll
      for (int c = 0; c < 4; c++) {
        zm[c] = zj[c + 1];
        visu[c] = fmaf(nu4dt, llu[c], nu2dt * la[c + 2]);
        visv[c] = fmaf(nu4dt, llv[c], nu2dt * ma[c + 2]);
      }
#pragma unroll
      for (int c = 0; c < 5; c++) dj[c] = dn[c];
      if (keep_ll) {  // with its halo images, for the third level
        put4<POLAR ? IMG_ETA : IMG_LU, 3>(d.LLu, P, nx, ny, ib, j, llu);
        put4<POLAR ? IMG_ETA : IMG_LV, 3>(d.LLv, P, nx, ny, ib, j, llv);
      }
    }
    section();

    // ---- BODYU (calc.c:168-200)
    {
      float u0[8], u1[4], um[4], u2[4], vm[8], v0[8];
      U8(t, u0); U4(t + 1, u1); U4(t - 1, um); U4(t + 2, u2); V8(t - 1, vm); V8(t, v0);
      const float kc = Qr(q, Q_KXC, j), kv = Qr(q, Q_KYV, j), k2xe = Qr(q, Q_K2XE, j), idxe = Qr(q, Q_IDXE, j);
      float xu[5];
#pragma unroll
      for (int m = 0; m < 5; m++)
        xu[m] = face2<SCH>(u0[m], u0[m + 1], u0[m + 2], u0[m + 3], cpos2(u0[m + 1], u0[m + 2], kc),
                           cneg2(u0[m + 1], u0[m + 2], kc));
      float uraw[4];
      if constexpr (EXTRA) own4(rg.row(t, FU), uraw);
      float damp[4] = {sigdt, sigdt, sigdt, sigdt};
      if constexpr (POLAR) arr(ld4f(d.pf + PQ_SU * PR, P, ib, j), damp);
      float du[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const float uc = u0[c + 2];
        const float2 yn = face2_shared<SCH>(um[c], uc, u1[c], u2[c]);
        const float vs0 = vm[c + 2], vs1 = vm[c + 3], vn0 = v0[c + 2], vn1 = v0[c + 3];
        const float p1 = (xu[c] - xu[c + 1]) +
                         (face2_term(ysu[c], um[c], uc, cpos2(vs0, vs1, kv), cneg2(vs0, vs1, kv)) -
                          face2_term(yn, uc, u1[c], cpos2(vn0, vn1, kv), cneg2(vn0, vn1, kv)));
        ysu[c] = yn;
        const float p2 = fmaf(uc * (u0[c + 3] - u0[c + 1]), k2xe, (uc * (0.5f * (vn0 + vn1) - 0.5f * (vs0 + vs1))) * kv);
        du[c] = fmaf(-(EXTRA ? uraw[c] : uc), damp[c], p1 + p2) + visu[c];
        if (ib + c <= nx) mxu = fmaxf(mxu, fabsf(uc) * idxe);
      }
      st4f(d.dup, P, ib, j, du);
    }
    section();

    // ---- BODYV (calc.c:205-237)
    {
      float v0[8], vm[4], v1[4], v2[4], u0[8], u1[8];
      V8(t, v0); V4(t - 1, vm); V4(t + 1, v1); V4(t + 2, v2); U8(t, u0); U8(t + 1, u1);
      const float kxv = Qr(q, Q_KXV, j), kyc = Qr(q, Q_KYC, j), kdyns = Qr(q, Q_KDYNS, j), idyn = Qr(q, Q_IDYN, j);
      float xv[5];
#pragma unroll
      for (int m = 0; m < 5; m++)
        xv[m] = face2<SCH>(v0[m], v0[m + 1], v0[m + 2], v0[m + 3], cpos2(u1[m + 1], u0[m + 1], kxv),
                           cneg2(u1[m + 1], u0[m + 1], kxv));
      float vraw[4];
      if constexpr (EXTRA) own4(rg.row(t, FV), vraw);
      float damp[4] = {sigdt, sigdt, sigdt, sigdt};
      if constexpr (POLAR) arr(ld4f(d.pf + PQ_SV * PR, P, ib, j), damp);
      float dv[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const float vsm = vm[c], vc = v0[c + 2], vnp = v1[c];
        const float2 yn = face2_shared<SCH>(vsm, vc, vnp, v2[c]);
        const float p1 = (xv[c] - xv[c + 1]) +
                         (face2_term(ysv[c], vsm, vc, cpos2(vsm, vc, kyc), cneg2(vsm, vc, kyc)) -
                          face2_term(yn, vc, vnp, cpos2(vc, vnp, kyc), cneg2(vc, vnp, kyc)));
        ysv[c] = yn;
        const float uw1 = u1[c + 1], uw0 = u0[c + 1], ue1 = u1[c + 2], ue0 = u0[c + 2];
        const float p2 = fmaf(vc * (0.5f * (ue0 + ue1) - 0.5f * (uw0 + uw1)), kxv, (vc * (vnp - vsm)) * kdyns);
        dv[c] = fmaf(-(EXTRA ? vraw[c] : vc), damp[c], p1 + p2) + visv[c];
        if (ib + c <= nx) mxv = fmaxf(mxv, fabsf(vc) * idyn);
      }
      st4f(d.dvp, P, ib, j, dv);
    }
    section();
  }
  ring_end(rg);
  ring_end(rl);
  cpa_wait0();
  flush_checks(d, vw, mxu, mxv, oor);
  return true;
}

// --------------------------------------------------------------- kb_tracer
// BODYTRACER (calc.c:117-163): TVD fluxes of the tracer on the four faces,
// each with both split Courant numbers of its face velocity (winds
// included), the compression term and the damping -2*Dt*TracerDis*T; then the
// Adams-Bashforth combination (calc.c:651-699) and the update with the
// single-rank halo wrap (core.c:161-182). Staged rows j0-2 .. j1+2 of the
// tracer shadow, u and v (and the winds with EXTRA).
template <int SCH, bool EXTRA, bool POLAR>
__device__ __forceinline__ bool strip_tracer(const MemberDesc& d, const View& vw, int sx, int sy, int SR,
                                             Ring<EXTRA ? 5 : 3, kDMain1>& rg, bool test) {
  enum { FT, FU, FV, FWX, FWY };
  const TracerDesc& td = *d.trd;
  const int nx = d.nx, ny = d.ny, P = d.P, W = nx + 4;
  const float* q = d.q;
  const int i0 = sx * SW + 1, j0 = sy * SR + 1, j1 = min(j0 + SR - 1, ny);
  const int ib = i0 + 4 * lane_id();
  int* bad = d.bad + vw.slot;
  rg.map[FT] = map_of(d, TM_TS + vw.cur);
  rg.map[FU] = map_of(d, TM_US + vw.cur);
  rg.map[FV] = map_of(d, TM_VS + vw.cur);
  if constexpr (EXTRA) {
    rg.map[FWX] = map_of(d, TM_WX);
    rg.map[FWY] = map_of(d, TM_WY);
  }
  rg.x = sx * SW;
  rg.y0 = j0 - 1;
  rg.T = j1 - j0 + 5;
  ring_begin(rg);
  for (int t = 0; t < 4; t++)
    if (!ring_wait(rg, t, bad)) return false;
  if (test && !ring_test(rg, d.tile_test, bad)) return false;
  auto U8 = [&](int t, float (&w)[8]) {
    win8(rg.row(t, FU), w);
    if constexpr (EXTRA) { float x[8]; win8(rg.row(t, FWX), x); addw(w, x, 1.f); }
  };
  auto V4 = [&](int t, float (&w)[4]) {
    own4(rg.row(t, FV), w);
    if constexpr (EXTRA) { float x[4]; own4(rg.row(t, FWY), x); addw(w, x, 1.f); }
  };
  float2 yst[4];
  {
    float a[4], b[4], c4[4], e[4];
    own4(rg.row(0, FT), a); own4(rg.row(1, FT), b); own4(rg.row(2, FT), c4); own4(rg.row(3, FT), e);
#pragma unroll
    for (int c = 0; c < 4; c++) yst[c] = face2_shared<SCH>(a[c], b[c], c4[c], e[c]);
  }
  const float sig2dt = td.sig2dt;
  const double* tin = td.tr[vw.cur];
  double* tout = td.tr[1 - vw.cur];
  float* tsout = td.ts[1 - vw.cur];
  const float* h1p = td.h[vw.h1];
  const float* h2p = td.h[vw.h2];
  float* hw = td.h[vw.w];
  const int kab = vw.k;
  bool oor = false;
  double to[4];
  float4 g1 = make_float4(0.f, 0.f, 0.f, 0.f), g2 = g1;
  ld4d(tin, W, nx, ib, j0, to);
  if (kab >= 1) g1 = ld4f(h1p, P, ib, j0);
  if (kab >= 2) g2 = ld4f(h2p, P, ib, j0);
  for (int j = j0; j <= j1; j++) {
    const int k = j - j0, t = k + 2;
    ring_refill(rg, k);
    if (!ring_wait(rg, t + 2, bad)) return false;
    float h1[4], h2[4];
    double tc[4];
    arr(g1, h1); arr(g2, h2);
#pragma unroll
    for (int c = 0; c < 4; c++) tc[c] = to[c];
    if (j < j1) {
      ld4d(tin, W, nx, ib, j + 1, to);
      if (kab >= 1) g1 = ld4f(h1p, P, ib, j + 1);
      if (kab >= 2) g2 = ld4f(h2p, P, ib, j + 1);
    }
    float tw[8], tm[4], t1[4], t2[4], uw[8], vm[4], vc[4];
    win8(rg.row(t, FT), tw); own4(rg.row(t - 1, FT), tm); own4(rg.row(t + 1, FT), t1); own4(rg.row(t + 2, FT), t2);
    U8(t, uw); V4(t - 1, vm); V4(t, vc);
    const float kx = Qr(q, Q_KXE, j), ky = Qr(q, Q_KYN, j);
    float damp[4] = {sig2dt, sig2dt, sig2dt, sig2dt};  // 2*Dt*TracerDis; per cell with a cap's sponge
    if constexpr (POLAR) arr(ld4f(d.pf + PQ_STR2 * P * (ny + 4), P, ib, j), damp);
    float fx[5];
#pragma unroll
    for (int m = 0; m < 5; m++)
      fx[m] = face2<SCH>(tw[m], tw[m + 1], tw[m + 2], tw[m + 3], fmaxf(uw[m + 1], 0.f) * kx, fminf(uw[m + 1], 0.f) * kx);
    float hist[4], tsn[4];
    double tn[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float T = tw[c + 2];
      const float2 yn = face2_shared<SCH>(tm[c], T, t1[c], t2[c]);
      const float fs = face2_term(yst[c], tm[c], T, fmaxf(vm[c], 0.f) * ky, fminf(vm[c], 0.f) * ky);
      const float fn = face2_term(yn, T, t1[c], fmaxf(vc[c], 0.f) * ky, fminf(vc[c], 0.f) * ky);
      yst[c] = yn;
      float dtr = (fx[c] - fx[c + 1]) + (fs - fn);
      dtr = fmaf(T, fmaf(uw[c + 2] - uw[c + 1], kx, (vc[c] - vm[c]) * ky), dtr);
      dtr = fmaf(-damp[c], T, dtr);
      const float ab = ab3(kab, dtr, h1[c], h2[c]);
      hist[c] = dtr;
      tn[c] = tc[c] + f2d(ab);
      tsn[c] = d2f(tn[c]);
      oor = oor || ((ib + c <= nx) && !in_range(tn[c]));
    }
    st4f(hw, P, ib, j, hist);
    put4<IMG_ETA, 1>(tout, W, nx, ny, ib, j, tn);  // the tracer's halo update wraps (core.c:180-181)
    put4<IMG_ETA, 3>(tsout, P, nx, ny, ib, j, tsn);
  }
  ring_end(rg);
  flush_checks(d, vw, 0.f, 0.f, oor);
  return true;
}

// ---------------------------------------------------------------- kb_main2
// Pressure on the new eta (calc.c:500-540), AB, Coriolis u then v
// (calc.c:542-598). v at (i, j) needs the new u at (i-1..i, j..j+1): each
// row computes the new u of the next row at the lane's columns and the one
// west of them, and the halo column 0 and the halo row ny+1 keep the old u
// (the v update reads them before the halo refresh, core.c:283-289). Staged
// rows j0-1 .. j1+1 of the new eta shadow and the old u, v shadows.
struct UnewIn {
  float dup[5], h1[5], h2[5];  // columns ib-1 .. ib+3
  double uo[4];                // old u at ib .. ib+3
};

__device__ __forceinline__ void load_unew(const MemberDesc& d, const View& vw, int ib, int jr, UnewIn& o) {
  const int P = d.P;
  float a[4];
  arr(ld4f(d.dup, P, ib, jr), a);
  o.dup[0] = __ldg(d.dup + IX32(P, ib - 1, jr));
#pragma unroll
  for (int c = 0; c < 4; c++) o.dup[c + 1] = a[c];
  if (vw.k >= 1) {
    arr(ld4f(d.hu[vw.h1], P, ib, jr), a);
    o.h1[0] = __ldg(d.hu[vw.h1] + IX32(P, ib - 1, jr));
#pragma unroll
    for (int c = 0; c < 4; c++) o.h1[c + 1] = a[c];
  } else {
#pragma unroll
    for (int c = 0; c < 5; c++) o.h1[c] = 0.f;
  }
  if (vw.k >= 2) {
    arr(ld4f(d.hu[vw.h2], P, ib, jr), a);
    o.h2[0] = __ldg(d.hu[vw.h2] + IX32(P, ib - 1, jr));
#pragma unroll
    for (int c = 0; c < 4; c++) o.h2[c + 1] = a[c];
  } else {
#pragma unroll
    for (int c = 0; c < 5; c++) o.h2[c] = 0.f;
  }
  ld4d(d.u[vw.cur], d.nx + 4, d.nx, ib, jr, o.uo);
}

// New u of row jr at columns ib-1+k, k = 0..4 (calc.c:542-573); with `own`
// the lane's four cells are written (tendency history, FP64 state and shadow
// with their images).
// The per-cell -GE*Dt/DXC and Dt*FE of a polar cap at columns ib-1..ib+3 of row jr.
__device__ __forceinline__ void cap5(const MemberDesc& d, int t, int ib, int jr, float (&v)[5]) {
  const float* f = d.pf + t * d.P * (d.ny + 4);
  float a[4];
  arr(ld4f(f, d.P, ib, jr), a);
  v[0] = __ldg(f + IX32(d.P, ib - 1, jr));
#pragma unroll
  for (int c = 0; c < 4; c++) v[c + 1] = a[c];
}

template <bool POLAR>
__device__ __forceinline__ void unew5(const MemberDesc& d, const View& vw, int ib, int jr, bool own,
                                      const float (&ew)[8], const float (&uw)[8], const float (&vr)[8],
                                      const float (&vrm)[8], const UnewIn& in, float (&un)[5], bool& oor) {
  const int nx = d.nx, ny = d.ny, P = d.P;
  const float* q = d.q;
  const bool rowok = (jr <= ny);
  const float geo = Qr(q, Q_GEO, jr);
  float gex[5], dtfe[5];
  if constexpr (POLAR) {
    cap5(d, PQ_GEX, ib, jr, gex);
    cap5(d, PQ_DTFE, ib, jr, dtfe);
  } else {
    const float g = Qr(q, Q_GEX, jr), f = Qr(q, Q_DTFE, jr);
#pragma unroll
    for (int k = 0; k < 5; k++) { gex[k] = g; dtfe[k] = f; }
  }
  float dun[5], du[5];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    const int i = ib - 1 + k, m = k + 1;
    const float uu = uw[m];
    const float dn = fmaf(gex[k], ew[m + 1] - ew[m], in.dup[k]);
    const float ab = ab3(vw.k, dn, in.h1[k], in.h2[k]);
    const float semi = 0.25f * (((vr[m] + vr[m + 1]) + vrm[m]) + vrm[m + 1]);
    const float al = fmaf(uu, geo, dtfe[k]);
    const float be = 0.25f * (al * al);
    const float dd = __fdividef(fmaf(al, semi, fmaf(-2.f * be, uu, ab)), 1.f + be);
    const bool live = rowok && i >= 1 && i <= nx;
    dun[k] = dn;
    du[k] = dd;
    un[k] = live ? uu + dd : uu;
  }
  if (own) {
    float hist[4], usn[4];
    double unw[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      hist[c] = dun[c + 1];
      unw[c] = in.uo[c] + f2d(du[c + 1]);
      usn[c] = d2f(unw[c]);
      oor = oor || ((ib + c <= nx) && !in_range(unw[c]));
    }
    st4f(d.hu[vw.w], P, ib, jr, hist);
    if (POLAR || d.open_step) {  // the plain halo update only (no walls, or do_channel after the forcing)
      put4<IMG_ETA, 1>(d.u[1 - vw.cur], nx + 4, nx, ny, ib, jr, unw);
      put4<IMG_ETA, 3>(d.us[1 - vw.cur], P, nx, ny, ib, jr, usn);
    } else {
      put4<IMG_U, 1>(d.u[1 - vw.cur], nx + 4, nx, ny, ib, jr, unw);
      put4<IMG_U, 3>(d.us[1 - vw.cur], P, nx, ny, ib, jr, usn);
    }
  }
}

template <bool POLAR>
__device__ __forceinline__ bool strip_main2(const MemberDesc& d, const View& vw, int sx, int sy, int SR,
                                            Ring<3, kDMain2>& rg, bool test) {
  enum { FE, FU, FV };
  const int nx = d.nx, ny = d.ny, P = d.P, W = nx + 4;
  const float* q = d.q;
  const int i0 = sx * SW + 1, j0 = sy * SR + 1, j1 = min(j0 + SR - 1, ny);
  const int ib = i0 + 4 * lane_id();
  int* bad = d.bad + vw.slot;
  rg.map[FE] = map_of(d, TM_ES + (1 - vw.cur));
  rg.map[FU] = map_of(d, TM_US + vw.cur);
  rg.map[FV] = map_of(d, TM_VS + vw.cur);
  rg.x = sx * SW;
  rg.y0 = j0;  // tensor row of j0 - 1
  rg.T = j1 - j0 + 3;
  ring_begin(rg);
  if (!ring_wait(rg, 0, bad) || !ring_wait(rg, 1, bad)) return false;
  if (test && !ring_test(rg, d.tile_test, bad)) return false;
  bool oor = false;
  float unc[5];
  UnewIn in;
  load_unew(d, vw, ib, j0, in);
  {  // the new u of row j0
    float ew[8], uw[8], vr[8], vrm[8];
    win8(rg.row(1, FE), ew); win8(rg.row(1, FU), uw); win8(rg.row(1, FV), vr); win8(rg.row(0, FV), vrm);
    unew5<POLAR>(d, vw, ib, j0, true, ew, uw, vr, vrm, in, unc, oor);
  }
  const float* hv1p = d.hv[vw.h1];
  const float* hv2p = d.hv[vw.h2];
  const int kab = vw.k;
  // own-cell inputs of the v update of row j and of the new u of row j+1
  float4 gd, g1 = make_float4(0.f, 0.f, 0.f, 0.f), g2 = g1;
  double vo[4];
  gd = ld4f(d.dvp, P, ib, j0);
  if (kab >= 1) g1 = ld4f(hv1p, P, ib, j0);
  if (kab >= 2) g2 = ld4f(hv2p, P, ib, j0);
  ld4d(d.v[vw.cur], W, nx, ib, j0, vo);
  if (j0 + 1 <= ny + 1) load_unew(d, vw, ib, min(j0 + 1, ny), in);
  for (int j = j0; j <= j1; j++) {
    const int k = j - j0, t = k + 1;  // ring row of j
    ring_refill(rg, k);
    if (!ring_wait(rg, t + 1, bad)) return false;
    float dvpv[4], h1[4], h2[4];
    double vc[4];
    arr(gd, dvpv); arr(g1, h1); arr(g2, h2);
#pragma unroll
    for (int c = 0; c < 4; c++) vc[c] = vo[c];
    const UnewIn cur_in = in;
    if (j < j1) {
      gd = ld4f(d.dvp, P, ib, j + 1);
      if (kab >= 1) g1 = ld4f(hv1p, P, ib, j + 1);
      if (kab >= 2) g2 = ld4f(hv2p, P, ib, j + 1);
      ld4d(d.v[vw.cur], W, nx, ib, j + 1, vo);
      load_unew(d, vw, ib, min(j + 2, ny), in);
    }
    // the new u of row j+1 (the halo row ny+1 keeps the old u)
    float unn[5];
    {
      float ew[8], uw[8], vr[8], vrm[8];
      win8(rg.row(t + 1, FE), ew); win8(rg.row(t + 1, FU), uw); win8(rg.row(t + 1, FV), vr); win8(rg.row(t, FV), vrm);
      unew5<POLAR>(d, vw, ib, j + 1, j + 1 <= j1, ew, uw, vr, vrm, cur_in, unn, oor);
    }
    // v of row j
    float e0[4], e1[4], vv[4];
    own4(rg.row(t, FE), e0); own4(rg.row(t + 1, FE), e1); own4(rg.row(t, FV), vv);
    const float dp1 = Qr(q, Q_DHBP1, j), cv = Qr(q, Q_CV, j);
    float gny[4], dtfn[4];
    if constexpr (POLAR) {
      const int PR = P * (ny + 4);
      arr(ld4f(d.pf + PQ_GNY * PR, P, ib, j), gny);
      arr(ld4f(d.pf + PQ_DTFN * PR, P, ib, j), dtfn);
    } else {
      const float g = Qr(q, Q_GNY, j), f = Qr(q, Q_DTFN, j);
#pragma unroll
      for (int c = 0; c < 4; c++) { gny[c] = g; dtfn[c] = f; }
    }
    float hist[4], vsn[4];
    double vn[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float dvn = fmaf(gny[c], (e1[c] - e0[c]) + dp1, dvpv[c]);
      const float ab = ab3(kab, dvn, h1[c], h2[c]);
      // new u at (i-1, j+1), (i, j+1), (i, j), (i-1, j)
      const float semi = 0.25f * (((unn[c] + unn[c + 1]) + unc[c + 1]) + unc[c]);
      const float al = fmaf(semi, cv, dtfn[c]);
      const float be = 0.25f * (al * al);
      const float dv = __fdividef(fmaf(-al, semi, fmaf(-2.f * be, vv[c], ab)), 1.f + be);
      hist[c] = dvn;
      vn[c] = vc[c] + f2d(dv);
      vsn[c] = d2f(vn[c]);
      // a band's row ny is a wall: do_channel zeroes it before the check
      oor = oor || ((ib + c <= nx) && (POLAR || j != ny) && !in_range(vn[c]));
    }
    st4f(d.hv[vw.w], P, ib, j, hist);
    if (POLAR || d.open_step) {
      put4<IMG_ETA, 1>(d.v[1 - vw.cur], W, nx, ny, ib, j, vn);
      put4<IMG_ETA, 3>(d.vs[1 - vw.cur], P, nx, ny, ib, j, vsn);
    } else {
      put4<IMG_V, 1>(d.v[1 - vw.cur], W, nx, ny, ib, j, vn);
      put4<IMG_V, 3>(d.vs[1 - vw.cur], P, nx, ny, ib, j, vsn);
    }
#pragma unroll
    for (int c = 0; c < 5; c++) unc[c] = unn[c];
  }
  ring_end(rg);
  flush_checks(d, vw, 0.f, 0.f, oor);
  return true;
}

// ------------------------------------------------------------------ kernels
// Each warp of a block is an independent strip worker with its own ring.
// A warp that gave up on a wait (timeout) takes no further strips.
#define SW2G_STRIP_LOOP(NF, D, CALL)                                   \
  extern __shared__ __align__(128) unsigned char sm[];                  \
  Ring<NF, D> rg;                                                      \
  ring_init(sm, rg);                                                   \
  const int n = *counter;                                              \
  bool first = true;                                                   \
  for (;;) {                                                           \
    const int s = take_strip(queue);                                   \
    if (s >= nstrips) break;                                           \
    const int4 tl = strip_at<N>(tiles, s, nbx);                        \
    const MemberDesc& d = ds.m[N == 1 ? 0 : tl.x];                     \
    const View v = view_of(d, n);                                      \
    const bool test = first && d.tile_test > 0;                        \
    first = false;                                                     \
    if (!(CALL)) break;                                                \
  }                                                                    \
  warp_done(queue);

#define SW2G_KPARAMS                                                                                       \
  const __grid_constant__ DescSet<N> ds, const int4* __restrict__ tiles, int nstrips, int nbx, int SR, \
      const int* __restrict__ counter, unsigned* queue

template <int N, bool POLAR = false>
__global__ void __launch_bounds__(NT, 6) kb_lap1(SW2G_KPARAMS) {
  SW2G_STRIP_LOOP(2, kDLap, (strip_lap<false, POLAR>(d, v, tl.y, tl.z, SR, rg, test)))
}

// Third Laplacian level (nu6): members without it skip their strips.
template <int N, bool POLAR = false>
__global__ void __launch_bounds__(NT, 6) kb_lap3(SW2G_KPARAMS) {
  SW2G_STRIP_LOOP(2, kDLap, (d.nu6dt == 0.f || strip_lap<true, POLAR>(d, v, tl.y, tl.z, SR, rg, test)))
}

// Tracer advection: members without an active tracer skip their strips.
template <int SCH, bool EXTRA, int N, bool POLAR = false>
__global__ void __launch_bounds__(NT) kb_tracer(SW2G_KPARAMS) {
  SW2G_STRIP_LOOP(EXTRA ? 5 : 3, kDMain1,
                  (!d.trd || strip_tracer<SCH, EXTRA, POLAR>(d, v, tl.y, tl.z, SR, rg, test)))
}

template <int SCH, bool EXTRA, int N, bool POLAR = false>
__global__ void __launch_bounds__(NT, EXTRA ? 2 : 3) kb_main1(SW2G_KPARAMS) {
  extern __shared__ __align__(128) unsigned char sm[];
  Ring<main1_fields<EXTRA>(), kDMain1> rg;
  Ring<2, kDLapIn> rl;
  unsigned char* a = smem_base(sm);
  ring_init_at(a, 0, main1_bars<EXTRA>(), rg);
  ring_init_at(a, NWARP * kDMain1 * 8, main1_lrows<EXTRA>(), rl);
  const unsigned stg = smem_u32(a + main1_stage<EXTRA>() + (threadIdx.x >> 5) * kStageMain1);
  const int n = *counter;
  bool first = true;
  for (;;) {
    const int s = take_strip(queue);
    if (s >= nstrips) break;
    const int4 tl = strip_at<N>(tiles, s, nbx);
    const MemberDesc& d = ds.m[N == 1 ? 0 : tl.x];
    const View v = view_of(d, n);
    const bool test = first && d.tile_test > 0;
    first = false;
    if (!strip_main1<SCH, EXTRA, POLAR>(d, v, tl.y, tl.z, SR, rg, rl, stg, test)) break;
  }
  warp_done(queue);
}

template <int N, bool POLAR = false>
__global__ void __launch_bounds__(NT, 4) kb_main2(SW2G_KPARAMS) {
  SW2G_STRIP_LOOP(3, kDMain2, (strip_main2<POLAR>(d, v, tl.y, tl.z, SR, rg, test)))
}
#undef SW2G_STRIP_LOOP
#undef SW2G_KPARAMS

template <int NF, int D>
constexpr int smem_bytes() {
  return 128 + bar_bytes<D>() + NWARP * D * NF * RS * 4;
}
constexpr int kSmemLap = smem_bytes<2, kDLap>();
constexpr int kSmemMain2 = smem_bytes<3, kDMain2>();
template <bool EX>
constexpr int smem_main1() { return 128 + main1_stage<EX>() + NWARP * kStageMain1; }
template <bool EX>
constexpr int smem_tracer() { return smem_bytes<EX ? 5 : 3, kDMain1>(); }

// Dynamic shared memory and the number of resident blocks of a kernel on the
// current device (set once per device; fp32_prepare does it for every kernel
// before any launch can be captured into a graph).
constexpr int kMaxDevices = 64;
template <auto K>
int grid_cap(int smem) {
  static int cap[kMaxDevices] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  if (!cap[dev]) {
    cudaFuncSetAttribute(reinterpret_cast<const void*>(K), cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int b = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, K, NT, smem);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cap[dev] = (b > 0 ? b : 1) * (sms > 0 ? sms : 1);
  }
  return cap[dev];
}

// Arguments of one phase launch over a batch's strips (a single member: its
// grid of nbx strip columns and ny rows).
template <int N>
struct PhaseArgs {
  const DescSet<N>* ds;
  const int4* tiles;
  int nstrips, nbx, sr, ny;
  int* counter;
  unsigned* queue;
  cudaStream_t st;
  Timers* tm;
};

// One launch of kernel K over the strips: at most as many blocks as are
// resident (the warps take the strips from the queue), under the named timer.
// A single member's strips are as high as makes their number a whole
// multiple (or just under) of the kernel's resident warps, so that no round
// of strips runs on a few warps only: at 4096 x 2048 and 1824 resident warps,
// 57 strip rows of 36 rows rather than 64 of 32 (2048 strips, the last 224 of
// them running alone).
template <auto K, int N>
void run_phase(const char* tag, int smem, const PhaseArgs<N>& a, int& nl) {
  if (a.tm && a.tm->on) a.tm->begin(tag, a.st);
  const int cap = grid_cap<K>(smem);
  int nstrips = a.nstrips, sr = a.sr;
  if constexpr (N == 1) {
    const int slots = cap * NWARP, rows = slots / a.nbx > 0 ? slots / a.nbx : 1;
    sr = (a.ny + rows - 1) / rows;
    nstrips = a.nbx * ((a.ny + sr - 1) / sr);
  }
  const int want = (nstrips + NWARP - 1) / NWARP;
  K<<<want < cap ? want : cap, NT, smem, a.st>>>(*a.ds, a.tiles, nstrips, a.nbx, sr, a.counter, a.queue);
  if (a.tm && a.tm->on) a.tm->end(a.st);
  nl++;
}

// The limiter-dependent phases (mass and momentum sweeps, tracer), one
// instantiation per limiter in step_fp32_limiters.cu.
// polar: a single polar-cap member (N = 1; its kernels always read the winds)
template <int SCH, int N>
void sch_main1(bool extra, bool polar, const PhaseArgs<N>& a, int& nl);
template <int SCH, int N>
void sch_tracer(bool extra, bool polar, const PhaseArgs<N>& a, int& nl);
template <int SCH>
void sch_prepare();

}  // namespace f32
}  // namespace sw2g
