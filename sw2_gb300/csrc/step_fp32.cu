// FP32 precision form of the SW2 step.
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
// Three kernels per step:
//   k_lap1   : first Laplacian of (u, v) (laplacian.c:51-111) -> L, with the
//              reference's halo images and wall fixes written by each producer;
//   k_main1  : mass sweep + AB + geofactor -> eta (calc.c:70-113, 403-422),
//              second Laplacian of (u, v) from L, momentum advection and
//              dissipation -> partial tendencies, CFL maxima;
//   k_main2  : pressure, AB, semi-implicit Coriolis u then v (calc.c:500-598),
//              halo images and do_channel (calc.c:600-649) of u and v.
// Halos of intermediate fields at the periodic seam are computed at their
// source column ("ghosts"), because the reference's wrapped halo of a field
// is not the value its stencil would give at the halo column near the walls.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>

#include "sw2g_internal.h"

namespace sw2g {
namespace f32 {

// Tiles are TW = 32 cells wide (a warp per tile row) and TH rows high, TH a
// template parameter in {4, 8, 16} (the tile shapes the batch tuner picks
// from); a block has one thread per tile cell.
constexpr int TW = 32;
constexpr int NONE = INT_MIN;
static_assert(kTileRowsMax == 16, "the FP32 layout pads rows for tiles up to 16 rows high");
template <int TH>
__host__ __device__ constexpr int nthreads() { return TW * TH; }

__device__ __forceinline__ int IX(int W, int i, int j) { return (i + 1) + (j + 1) * W; }

struct KP {
  int nx, ny, W, H, P;
  const float* q;  // Q_NUM x H per-row FP32 table
  float sig2dt, sigdt, nu2dt, nu4dt, nu6dt;
  int k;           // Adams-Bashforth index
  int extra;       // winds / bottom present
  const float* wx; const float* wy; const float* hb;  // FP32 copies (pitch P) when extra
};

// Per-row constants of the rows a block touches (j0-2 .. j0+TH+2), staged in
// shared memory once per block from the row-major table p.q[(j+1)*Q_NUM + t].
template <int TH>
using RowCache = float[TH + 5][Q_NUM];
struct Rows {
  const float (*r)[Q_NUM];
  int j0;
};
__device__ __forceinline__ float Q(const Rows& c, int t, int j) { return c.r[j - c.j0 + 2][t]; }
template <int TH>
__device__ __forceinline__ void fill_rows(const KP& p, int j0, RowCache<TH>& sq) {
  for (int t = threadIdx.x; t < (TH + 5) * Q_NUM; t += nthreads<TH>()) {
    const int r = t / Q_NUM, c = t - r * Q_NUM;
    const int row = min(j0 - 2 + r, p.ny + 2);
    sq[r][c] = p.q[(size_t)(row + 1) * Q_NUM + c];
  }
}

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
template <int SCH>
__device__ __forceinline__ float psi(float r) {
  if constexpr (SCH == 0) return fmaxf(0.f, fminf(fminf((1.f + r) * 0.5f, 2.f * r), 2.f));
  else if constexpr (SCH == 1) return fmaxf(fmaxf(0.f, fminf(2.f * r, 1.f)), fmaxf(0.f, fminf(r, 2.f)));
  else if constexpr (SCH == 2) return (r < 1.f) ? r : 1.f;
  else if constexpr (SCH == 3) return (r + fabsf(r)) / (1.f + r);
  else if constexpr (SCH == 4) return fmaxf(0.f, fminf(2.f * r, fminf((1.f + 2.f * r) * (1.f / 3.f), 2.f)));
  else if constexpr (SCH == 5) return __fdividef(1.5f * (r * r + r), r * r + r + 1.f);
  else if constexpr (SCH == 6) return __fdividef(r * r + r, r * r + 1.f);
  else if constexpr (SCH == 7) return fmaxf(0.f, fminf(fminf(2.f, 2.f * r), fminf(0.25f + 0.75f * r, 0.75f + 0.25f * r)));
  else if constexpr (SCH == 8) return 0.f;
  else if constexpr (SCH == 9) return 1.f;
  else return (r > 0.f) ? __fdividef(2.f * r, 1.f + r) : 0.f;  // Van Leer, 0 for r <= 0 (its limit at -1)
}

// One upwind face with a single Courant number c (mass): c*B of calc.c:41-49,100
// with B_P (c > 0) or B_M (c < 0) reconstructed from q0|q1, outer neighbours qm, q2.
template <int SCH>
__device__ __forceinline__ float face1(float qm, float q0, float q1, float q2, float c) {
  const float d = q1 - q0;
  const bool pos = c > 0.f;
  const float n = pos ? (q0 - qm) : (q2 - q1);
  const float base = pos ? q0 : q1;
  const float r = (d != 0.f) ? __fdividef(n, d) : 0.f;
  const float s = pos ? 0.5f : -0.5f;
  return c * (base + s * psi<SCH>(r) * (1.f - fabsf(c)) * d);
}

// A face with both split Courant numbers (momentum bodies, calc.c:170-177).
template <int SCH>
__device__ __forceinline__ float face2(float qm, float q0, float q1, float q2, float cP, float cM) {
  const float d = q1 - q0;
  // approximate reciprocal (relative error below 2^-22); differences below the
  // smallest normal count as zero, like a zero difference
  const float inv = (fabsf(d) >= 1.17549435e-38f) ? __fdividef(1.f, d) : 0.f;
  const float rP = (q0 - qm) * inv, rM = (q2 - q1) * inv;
  const float bP = q0 + 0.5f * psi<SCH>(rP) * (1.f - cP) * d;
  const float bM = q1 - 0.5f * psi<SCH>(rM) * (1.f + cM) * d;
  return cP * bP + cM * bM;
}

__device__ __forceinline__ float cpos2(float a, float b, float k) { return 0.5f * (fmaxf(a, 0.f) + fmaxf(b, 0.f)) * k; }
__device__ __forceinline__ float cneg2(float a, float b, float k) { return 0.5f * (fminf(a, 0.f) + fminf(b, 0.f)) * k; }

// y faces: the two cells of a face divide by their own row metric, so their
// Courant numbers differ, while the limited slope is shared. For a mass face
// (one Courant number, whose sign is that of v): g = +-psi(r)/2*(q1-q0) and the
// upwind value; the cell's term is c*(base + g*(1-|c|)).
template <int SCH>
__device__ __forceinline__ float2 face1_shared(float qm, float q0, float q1, float q2, bool pos) {
  const float d = q1 - q0;
  const float n = pos ? (q0 - qm) : (q2 - q1);
  const float r = (fabsf(d) >= 1.17549435e-38f) ? __fdividef(n, d) : 0.f;
  return make_float2((pos ? 0.5f : -0.5f) * psi<SCH>(r) * d, pos ? q0 : q1);
}
__device__ __forceinline__ float face1_term(float2 gb, float c) { return c * (gb.y + gb.x * (1.f - fabsf(c))); }

// A momentum y face: gP = psi(rP)/2*(q1-q0), gM = psi(rM)/2*(q1-q0); the
// cell's term is cP*(q0 + gP*(1-cP)) + cM*(q1 - gM*(1+cM)).
template <int SCH>
__device__ __forceinline__ float2 face2_shared(float qm, float q0, float q1, float q2) {
  const float d = q1 - q0;
  const float inv = (fabsf(d) >= 1.17549435e-38f) ? __fdividef(1.f, d) : 0.f;
  return make_float2(0.5f * psi<SCH>((q0 - qm) * inv) * d, 0.5f * psi<SCH>((q2 - q1) * inv) * d);
}
__device__ __forceinline__ float face2_term(float2 g, float q0, float q1, float cP, float cM) {
  return cP * (q0 + g.x * (1.f - cP)) + cM * (q1 - g.y * (1.f + cM));
}

// ---------------------------------------------------------- halo images
enum Img { IMG_ETA, IMG_U, IMG_V, IMG_LU, IMG_LV };

// Writes the value of interior cell (i,j) and every halo cell whose final
// value in the reference comes from it: the single-rank halo update
// (sppde_hupdate.c:274-342, y pass then x pass) followed by do_channel for
// u and v (calc.c:600-649) or the wall fixes of laplacian_vels (laplacian.c:94-107).
template <Img M, typename T>
__device__ __forceinline__ void put(T* f, int W, int nx, int ny, int i, int j, T val) {
  // cells at least three columns and rows from every edge have no images
  if (i > 2 && i < nx - 1 && j > 2 && j < ny - 1) {
    f[IX(W, i, j)] = val;
    return;
  }
  const T zero = T(0);
  f[IX(W, i, j)] = (M == IMG_V && j == ny) ? zero : val;
  const int xa = (i <= 2) ? i + nx : NONE, xb = (i >= nx - 1) ? i - nx : NONE;
  const int ya = (j <= 2) ? j + ny : NONE, yb = (j >= ny - 1) ? j - ny : NONE;
  if (xa != NONE) f[IX(W, xa, j)] = val;
  if (xb != NONE) f[IX(W, xb, j)] = val;
  if (ya != NONE) {
    if (xa != NONE) f[IX(W, xa, ya)] = val;
    if (xb != NONE) f[IX(W, xb, ya)] = val;
  }
  if (yb != NONE) {
    if (xa != NONE) f[IX(W, xa, yb)] = val;
    if (xb != NONE) f[IX(W, xb, yb)] = val;
  }
  if constexpr (M == IMG_ETA) {
    if (ya != NONE) f[IX(W, i, ya)] = val;
    if (yb != NONE) f[IX(W, i, yb)] = val;
  } else if constexpr (M == IMG_U) {
    if (j == 1) { f[IX(W, i, 0)] = val; f[IX(W, i, -1)] = val; }
    if (j == ny) { f[IX(W, i, ny + 1)] = val; f[IX(W, i, ny + 2)] = val; }
  } else if constexpr (M == IMG_V) {
    if (j == 1) { f[IX(W, i, 0)] = zero; f[IX(W, i, -1)] = zero; }
    if (j == ny) { f[IX(W, i, ny + 1)] = zero; f[IX(W, i, ny + 2)] = zero; }
  } else {
    if (j == 2) f[IX(W, i, ny + 2)] = val;
    if (j == ny - 1) f[IX(W, i, -1)] = val;
    if (j == 1) f[IX(W, i, 0)] = (M == IMG_LU) ? val : zero;
    if (j == ny) f[IX(W, i, ny + 1)] = (M == IMG_LU) ? val : zero;
  }
}

// ------------------------------------------------------------- tile loads
// FP32 fields of this form use a row pitch P (a multiple of 4) and enough
// padding rows and columns that the ring-2 window of any tile is in bounds.
// The window [i0-2, i0+TW+1] x [j0-2, j0+TH+1] starts on a 16-byte boundary
// (padded column i0-1 = TW*bx), so it is read with 16-byte loads.
template <int TH>
using Tile = float[TH + 4][TW + 4];

__device__ __forceinline__ int IX32(int P, int i, int j) { return (i + 1) + (j + 1) * P; }

// Window loads by the threads: 16-byte loads of each row, spread over the block.
template <int TH>
__device__ __forceinline__ void load_tile(const float* __restrict__ f, int P, int i0, int j0, Tile<TH>& t) {
  constexpr int C4 = (TW + 4) / 4;
  const float* base = f + (size_t)(j0 - 1) * P + (i0 - 1);
  for (int q = threadIdx.x; q < (TH + 4) * C4; q += nthreads<TH>()) {
    const int r = q / C4, c = q - r * C4;
    const float4 v = __ldg(reinterpret_cast<const float4*>(base + (size_t)r * P) + c);
    *reinterpret_cast<float4*>(&t[r][4 * c]) = v;
  }
}

// Window loads by the TMA engine (kb_main2; measured: 8-10 % faster there,
// while kb_main1's five windows and kb_lap1's two load faster by threads):
// each of a window's TH+4 rows
// (TW+4 floats, 144 bytes, 16-byte aligned at both ends) is one bulk copy
// from global to shared memory, issued by one thread after it has registered
// the row's bytes on the block's mbarrier; every thread then waits for the
// barrier's first phase with an iteration limit. A wait that runs out sets
// CHECK_TIMEOUT in the step's check word (SW2G_ERR_TIMEOUT on the host) and
// the whole block returns without computing.
constexpr int TILE_ROW_BYTES = (TW + 4) * 4;
// Each wait suspends the thread for at most TILE_WAIT_HINT_NS, so the limit
// bounds a wait to about 1.3 s.
constexpr int TILE_WAIT_LIMIT = 1 << 16;
constexpr unsigned TILE_WAIT_HINT_NS = 20000;
constexpr int CHECK_TIMEOUT = kCheckTimeout;
static_assert(TILE_ROW_BYTES % 16 == 0, "bulk copies move multiples of 16 bytes");

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Barrier for `copies` row copies (one arrival each); ends with a block barrier.
__device__ __forceinline__ void tiles_init(unsigned long long* bar, int copies) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(copies) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// Row r of the window of field f (pitch P) at tile (i0, j0) into t[r].
template <int TH>
__device__ __forceinline__ void tile_row_copy(unsigned long long* bar, const float* f, int P, int i0, int j0,
                                              Tile<TH>& t, int r) {
  const float* src = f + (size_t)(j0 - 1 + r) * P + (i0 - 1);
  unsigned long long g;
  asm("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(src));
  const unsigned b = smem_u32(bar), d = smem_u32(&t[r][0]);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(TILE_ROW_BYTES) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
               "l"(g), "r"(TILE_ROW_BYTES), "r"(b)
               : "memory");
}

// One thread's bounded wait for the completion of the barrier phase of the
// given parity; true if it completed.
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

// True when every row arrived; all threads of the block return the same
// answer. test_waits > 0 (the failure-path test): after the rows have
// arrived, also wait for the next phase, which nothing completes, giving up
// after test_waits tries; no copy is then in flight when the block leaves.
__device__ __forceinline__ bool tiles_wait(unsigned long long* bar, int* bad, int test_waits) {
  const unsigned b = smem_u32(bar);
  bool done = phase_wait(b, 0u, TILE_WAIT_LIMIT);
  if (test_waits > 0 && done) done = phase_wait(b, 1u, test_waits);
  const int failed = __syncthreads_or(!done);
  if (failed && threadIdx.x == 0 && bad) atomicOr(bad, CHECK_TIMEOUT);
  return !failed;
}

// ------------------------------------------------ Laplacian of (u,v), one level
// Tiles U, V in ring-2 layout: local (a,b) <-> global (i0-2+a, j0-2+b).
// Produces ZE at (i0-1+a, j0-1+b) and DI at (i0+a, j0+b), a in [0,TW], b in [0,TH],
// following laplacian.c:59-81: ZE(i,0) = 0 and DI(i,ny+1) fixed at the walls;
// ZE(0,j) and DI(nx+1,j) are the wrapped values ZE(nx,j) and DI(1,j),
// evaluated at their source column from the global arrays gU, gV.
template <int TH>
__device__ __forceinline__ void zeta_div(const KP& p, const Rows& rc, int i0, int j0, const Tile<TH>& su,
                                         const Tile<TH>& sv, const float* gU, const float* gV, float (*ze)[TW + 1],
                                         float (*di)[TW + 1]) {
  const int P = p.P, nx = p.nx, ny = p.ny;
  for (int t = threadIdx.x; t < (TW + 1) * (TH + 1); t += nthreads<TH>()) {
    const int a = t % (TW + 1), b = t / (TW + 1);
    {  // ZE at (i, j) = (i0 - 1 + a, j0 - 1 + b)
      const int i = i0 - 1 + a, j = j0 - 1 + b;
      float z = 0.f;
      if (j >= 1 && j <= ny && i <= nx) {
        float v1, v0, u1, u0;
        if (i >= 1) {
          v1 = sv[b + 1][a + 2]; v0 = sv[b + 1][a + 1]; u1 = su[b + 2][a + 1]; u0 = su[b + 1][a + 1];
        } else {  // i == 0: ZE(nx, j) from the source column
          v1 = gV[IX32(P, nx + 1, j)]; v0 = gV[IX32(P, nx, j)];
          u1 = gU[IX32(P, nx, j + 1)]; u0 = gU[IX32(P, nx, j)];
        }
        z = Q(rc, Q_IDXV, j) * ((v1 - v0) - Q(rc, Q_IDYC, j + 1) * (Q(rc, Q_DXC, j + 1) * u1 - Q(rc, Q_DXC, j) * u0));
      }
      ze[b][a] = z;
    }
    {  // DI at (i, j) = (i0 + a, j0 + b)
      const int i = i0 + a, j = j0 + b;
      float d = 0.f;
      if (j >= 1 && j <= ny && i >= 1 && i <= nx + 1) {
        float uc, uw, vc, vs;
        if (i <= nx) {
          uc = su[b + 2][a + 2]; uw = su[b + 2][a + 1]; vc = sv[b + 2][a + 2]; vs = sv[b + 1][a + 2];
        } else {  // i == nx + 1: DI(1, j) from the source column
          uc = gU[IX32(P, 1, j)]; uw = gU[IX32(P, 0, j)];
          vc = gV[IX32(P, 1, j)]; vs = gV[IX32(P, 1, j - 1)];
        }
        d = Q(rc, Q_IDXE, j) * ((uc - uw) + Q(rc, Q_IDYN, j) * (Q(rc, Q_DXV, j) * vc - Q(rc, Q_DXV, j - 1) * vs));
      } else if (j == ny + 1 && i >= 1 && i <= nx) {
        d = (su[b + 1][a + 2] - su[b + 1][a + 1]) * Q(rc, Q_IDXE, ny);  // laplacian.c:73
      }
      di[b][a] = d;
    }
  }
}

// Second pass at tile cell (a,b) (laplacian.c:83-89).
__device__ __forceinline__ void lap_out(const Rows& rc, int j, int a, int b, const float (*ze)[TW + 1],
                                        const float (*di)[TW + 1], float& lu, float& lv) {
  lu = -Q(rc, Q_IDYN, j) * (ze[b + 1][a + 1] - ze[b][a + 1]) + Q(rc, Q_IDXC, j) * (di[b][a + 1] - di[b][a]);
  lv = Q(rc, Q_IDXV, j) * (ze[b + 1][a + 1] - ze[b + 1][a]) + Q(rc, Q_IDYC, j + 1) * (di[b + 1][a] - di[b][a]);
}

// ------------------------------------------------------------------ kernels
// ACC = false: the first Laplacian level L of (u, v), written with its halo
// images. ACC = true: the Laplacian of the second level LL, i.e. the third
// level LLL, added as nu6*Dt*LLL to the partial tendencies Lu, Lv (core.c:233-268).
template <int TH, bool ACC = false>
__device__ __forceinline__ void d_lap1(const KP& p, int bx, int by, const float* __restrict__ u,
                                       const float* __restrict__ v, float* Lu, float* Lv) {
  __shared__ __align__(16) Tile<TH> su, sv;
  __shared__ float ze[TH + 1][TW + 1], di[TH + 1][TW + 1];
  __shared__ RowCache<TH> sq;
  const int i0 = bx * TW + 1, j0 = by * TH + 1;
  fill_rows<TH>(p, j0, sq);
  const Rows rc{sq, j0};
  load_tile<TH>(u, p.P, i0, j0, su);
  load_tile<TH>(v, p.P, i0, j0, sv);
  __syncthreads();
  zeta_div<TH>(p, rc, i0, j0, su, sv, u, v, ze, di);
  __syncthreads();
  const int a = threadIdx.x % TW, b = threadIdx.x / TW;
  const int i = i0 + a, j = j0 + b;
  if (i > p.nx || j > p.ny) return;
  float lu, lv;
  lap_out(rc, j, a, b, ze, di, lu, lv);
  if constexpr (ACC) {
    const int q32 = IX32(p.P, i, j);
    Lu[q32] += p.nu6dt * lu;
    Lv[q32] += p.nu6dt * lv;
  } else {
    put<IMG_LU>(Lu, p.P, p.nx, p.ny, i, j, lu);
    put<IMG_LV>(Lv, p.P, p.nx, p.ny, i, j, lv);
  }
}

struct Main1Io {
  const double* eta;        // FP64 perturbation (pitch W)
  const float* es; const float* us; const float* vs;  // FP32 shadows (pitch P)
  const float* Lu; const float* Lv;
  const float* h1; const float* h2;
  double* eta_next; float* es_next;
  float* hist_eta;          // slot for Deta_n
  float* dup; float* dvp;
  float* LLu; float* LLv;   // second Laplacian level, written only when nu6 != 0
  unsigned* cfl;            // 2 floats as bits (max |u|/dx, max |v|/dy)
  int* bad;
};

// Faces of the three TVD bodies in tile-local ring-2 coordinates (column A,
// row B; global (i0-2+A, j0-2+B)). An x face lies west of column A and is
// shared whole by its two cells (their Courant numbers use the same row
// metric); a y face lies north of row B and shares its limited slopes.
template <int SCH, int TH>
__device__ __forceinline__ float mass_xface(const Tile<TH>& se, const Tile<TH>& su, float kx, int A, int B) {
  return face1<SCH>(se[B][A - 2], se[B][A - 1], se[B][A], se[B][A + 1], su[B][A - 1] * kx);
}
template <int SCH, int TH>
__device__ __forceinline__ float u_xface(const Tile<TH>& su, float kc, int A, int B) {
  const float uw = su[B][A - 1], ue = su[B][A];
  return face2<SCH>(su[B][A - 2], uw, ue, su[B][A + 1], cpos2(uw, ue, kc), cneg2(uw, ue, kc));
}
template <int SCH, int TH>
__device__ __forceinline__ float v_xface(const Tile<TH>& sv, const Tile<TH>& su, float kxv, int A, int B) {
  const float u1 = su[B + 1][A - 1], u0 = su[B][A - 1];
  return face2<SCH>(sv[B][A - 2], sv[B][A - 1], sv[B][A], sv[B][A + 1], cpos2(u1, u0, kxv), cneg2(u1, u0, kxv));
}
// Heights relative to the reference of row B (global row j).
template <int SCH, int TH>
__device__ __forceinline__ float2 mass_yface(const Tile<TH>& se, const Tile<TH>& sv, const Rows& rc, int A, int B,
                                             int j) {
  return face1_shared<SCH>(se[B - 1][A] + Q(rc, Q_DHBM1, j), se[B][A], se[B + 1][A] + Q(rc, Q_DHBP1, j),
                           se[B + 2][A] + Q(rc, Q_DHBP2, j), sv[B][A] > 0.f);
}
template <int SCH, int TH>
__device__ __forceinline__ float2 mom_yface(const Tile<TH>& t, int A, int B) {
  return face2_shared<SCH>(t[B - 1][A], t[B][A], t[B + 1][A], t[B + 2][A]);
}

template <int SCH, int TH>
__device__ __forceinline__ void d_main1(const KP& p, int bx, int by, const Main1Io& o) {
  constexpr int NT = nthreads<TH>();
  __shared__ __align__(16) Tile<TH> se, su, sv, sl, sm;
  __shared__ float ze[TH + 1][TW + 1], di[TH + 1][TW + 1];
  // x faces [b][a]: west of tile column a (a = 0..TW); y faces [b][a]: south of
  // tile row b (b = 0..TH)
  __shared__ float xm[TH][TW + 1], xu[TH][TW + 1], xv[TH][TW + 1];
  __shared__ float2 ym[TH + 1][TW], yu[TH + 1][TW], yv[TH + 1][TW];
  __shared__ float red[2][NT / 32];
  __shared__ RowCache<TH> sq;
  const int W = p.W, P = p.P, nx = p.nx, ny = p.ny;
  const int i0 = bx * TW + 1, j0 = by * TH + 1;
  // this thread's own cell: issue its global loads before the tile traffic
  const int ta = threadIdx.x % TW, tb = threadIdx.x / TW;  // tile coordinates
  const int a = ta + 2, b = tb + 2;                          // ring-2 local coordinates
  const int i = i0 + ta, j = j0 + tb;
  const bool live = (i <= nx && j <= ny);
  const int q = IX(W, live ? i : 1, live ? j : 1), q32 = IX32(P, i, j);
  const double eta_old = o.eta[q];
  const float h1v = (p.k >= 1) ? o.h1[q32] : 0.f, h2v = (p.k >= 2) ? o.h2[q32] : 0.f;
  const float e_raw = p.extra ? o.es[q32] : 0.f;  // eta without the bottom, for the damping
  fill_rows<TH>(p, j0, sq);
  const Rows rc{sq, j0};
  load_tile<TH>(o.es, P, i0, j0, se);
  load_tile<TH>(o.us, P, i0, j0, su);
  load_tile<TH>(o.vs, P, i0, j0, sv);
  load_tile<TH>(o.Lu, P, i0, j0, sl);
  load_tile<TH>(o.Lv, P, i0, j0, sm);
  __syncthreads();
  if (p.extra) {  // UWINDX, VWINDY (sw.h:216-217) and H = eta + depth - hB (sw.h:213)
    for (int t = threadIdx.x; t < (TH + 4) * (TW + 4); t += NT) {
      const int c = t % (TW + 4), r = t / (TW + 4);
      const int qq = IX32(P, i0 - 2 + c, j0 - 2 + r);
      su[r][c] += p.wx[qq];
      sv[r][c] += p.wy[qq];
      se[r][c] -= p.hb[qq];
    }
    __syncthreads();
  }
  zeta_div<TH>(p, rc, i0, j0, sl, sm, o.Lu, o.Lv, ze, di);
  {  // faces: each thread the x faces west of its cell and the y faces north of it
    xm[tb][ta] = mass_xface<SCH, TH>(se, su, Q(rc, Q_KXE, j), a, b);
    xu[tb][ta] = u_xface<SCH, TH>(su, Q(rc, Q_KXC, j), a, b);
    xv[tb][ta] = v_xface<SCH, TH>(sv, su, Q(rc, Q_KXV, j), a, b);
    ym[tb + 1][ta] = mass_yface<SCH, TH>(se, sv, rc, a, b, j);
    yu[tb + 1][ta] = mom_yface<SCH, TH>(su, a, b);
    yv[tb + 1][ta] = mom_yface<SCH, TH>(sv, a, b);
    // and the tile's south row (3 x TW faces) and east column (3 x TH) of
    // faces, counted from the last warp backwards (the first warps carry the
    // extra items of zeta_div); the south-row items fill whole warps
    const int e = (NT / 32 - 1 - tb) * 32 + ta;
    if (e < TW) ym[0][e] = mass_yface<SCH, TH>(se, sv, rc, e + 2, 1, j0 - 1);
    else if (e < 2 * TW) yu[0][e - TW] = mom_yface<SCH, TH>(su, e - TW + 2, 1);
    else if (e < 3 * TW) yv[0][e - 2 * TW] = mom_yface<SCH, TH>(sv, e - 2 * TW + 2, 1);
    else if (e < 3 * TW + 3 * TH) {
      const int l = e - 3 * TW, r = l % TH, B = r + 2, jr = j0 + r;
      if (l < TH) xm[r][TW] = mass_xface<SCH, TH>(se, su, Q(rc, Q_KXE, jr), TW + 2, B);
      else if (l < 2 * TH) xu[r][TW] = u_xface<SCH, TH>(su, Q(rc, Q_KXC, jr), TW + 2, B);
      else xv[r][TW] = v_xface<SCH, TH>(sv, su, Q(rc, Q_KXV, jr), TW + 2, B);
    }
  }
  __syncthreads();

  float mxu = 0.f, mxv = 0.f;
  if (live) {
    // ---- mass (BODYH, calc.c:70-113), H relative to the row reference Hb(j)
    const float kx = Q(rc, Q_KXE, j), ky = Q(rc, Q_KYN, j);
    const float cw = su[b][a - 1] * kx, ce = su[b][a] * kx, cs = sv[b - 1][a] * ky, cn = sv[b][a] * ky;
    float2 fs = ym[tb][ta];
    fs.y += Q(rc, Q_DHBM1, j);  // the south face's upwind value relative to Hb(j)
    float deta = xm[tb][ta] - xm[tb][ta + 1] + face1_term(fs, cs) - face1_term(ym[tb + 1][ta], cn);
    deta += Q(rc, Q_HB, j) * ((cw - ce) + (cs - cn));
    deta -= p.sig2dt * (Q(rc, Q_EREF, j) + (p.extra ? e_raw : se[b][a]));
    // Adams-Bashforth (calc.c:651-699) then the geofactor (calc.c:403-422)
    float ab;
    if (p.k == 0) ab = deta;
    else if (p.k == 1) ab = 1.5f * deta - 0.5f * h1v;
    else ab = (23.f / 12.f) * deta - (4.f / 3.f) * h1v + (5.f / 12.f) * h2v;
    const float hcell = Q(rc, Q_HB, j) + se[b][a];
    ab -= Q(rc, Q_GEO, j) * hcell * 0.5f * (sv[b][a] + sv[b - 1][a]);
    o.hist_eta[q32] = deta;
    const double en = eta_old + f2d(ab);
    put<IMG_ETA>(o.eta_next, W, nx, ny, i, j, en);
    put<IMG_ETA>(o.es_next, P, nx, ny, i, j, d2f(en));
    if (!in_range(en)) atomicOr(o.bad, 1);

    // ---- second Laplacian of (u, v) from L (laplacian.c:83-89)
    float llu, llv;
    lap_out(rc, j, ta, tb, ze, di, llu, llv);
    if (p.nu6dt != 0.f) {  // kept with its halo images for the third level
      put<IMG_LU>(o.LLu, P, nx, ny, i, j, llu);
      put<IMG_LV>(o.LLv, P, nx, ny, i, j, llv);
    }

    // ---- BODYU (calc.c:168-200)
    {
      const float uwm = su[b][a - 1], u0 = su[b][a], uep = su[b][a + 1];
      const float vs0 = sv[b - 1][a], vs1 = sv[b - 1][a + 1], vn0 = sv[b][a], vn1 = sv[b][a + 1];
      const float kv = Q(rc, Q_KYV, j);
      const float p1 = xu[tb][ta] - xu[tb][ta + 1] +
                       face2_term(yu[tb][ta], su[b - 1][a], u0, cpos2(vs0, vs1, kv), cneg2(vs0, vs1, kv)) -
                       face2_term(yu[tb + 1][ta], u0, su[b + 1][a], cpos2(vn0, vn1, kv), cneg2(vn0, vn1, kv));
      const float p2 = u0 * (uep - uwm) * Q(rc, Q_K2XE, j) + u0 * (0.5f * (vn0 + vn1) - 0.5f * (vs0 + vs1)) * kv;
      const float ul = p.extra ? o.us[q32] : u0;  // dissipation acts on U without the wind
      float du = p1 + p2 - ul * p.sigdt;
      du += p.nu2dt * sl[b][a] + p.nu4dt * llu;
      o.dup[q32] = du;
      mxu = fabsf(u0) * Q(rc, Q_IDXE, j);
    }
    // ---- BODYV (calc.c:205-237)
    {
      const float vsm = sv[b - 1][a], v0 = sv[b][a], vnp = sv[b + 1][a];
      const float uw1 = su[b + 1][a - 1], uw0 = su[b][a - 1], ue1 = su[b + 1][a], ue0 = su[b][a];
      const float kxv = Q(rc, Q_KXV, j), kyc = Q(rc, Q_KYC, j);
      const float p1 = xv[tb][ta] - xv[tb][ta + 1] +
                       face2_term(yv[tb][ta], vsm, v0, cpos2(vsm, v0, kyc), cneg2(vsm, v0, kyc)) -
                       face2_term(yv[tb + 1][ta], v0, vnp, cpos2(v0, vnp, kyc), cneg2(v0, vnp, kyc));
      const float p2 = v0 * (0.5f * (ue0 + ue1) - 0.5f * (uw0 + uw1)) * kxv + v0 * (vnp - vsm) * Q(rc, Q_KDYNS, j);
      const float vl = p.extra ? o.vs[q32] : v0;
      float dv = p1 + p2 - vl * p.sigdt;
      dv += p.nu2dt * sm[b][a] + p.nu4dt * llv;
      o.dvp[q32] = dv;
      mxv = fabsf(v0) * Q(rc, Q_IDYN, j);
    }
  }
  // CFL maxima of this block (calc.c:705-712)
  for (int s = 16; s > 0; s >>= 1) {
    mxu = fmaxf(mxu, __shfl_xor_sync(0xffffffffu, mxu, s));
    mxv = fmaxf(mxv, __shfl_xor_sync(0xffffffffu, mxv, s));
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = mxu; red[1][threadIdx.x >> 5] = mxv; }
  __syncthreads();
  if (threadIdx.x < 2) {
    float m = 0.f;
    for (int w = 0; w < NT / 32; w++) m = fmaxf(m, red[threadIdx.x][w]);
    if (m > 0.f) atomicMax(o.cfl + threadIdx.x, __float_as_uint(m));
  }
}

// BODYTRACER (calc.c:117-163): TVD fluxes of the tracer on the four faces,
// each with both split Courant numbers of its face velocity (winds
// included), the compression term and the damping -2*Dt*TracerDis*T; then the
// Adams-Bashforth combination (calc.c:651-699) and the update with the
// single-rank halo wrap (core.c:161-182). One cell per thread, faces per cell.
template <int SCH, int TH>
__device__ __forceinline__ void d_tracer(const KP& p, int bx, int by, const TracerDesc& td, int cur, int w, int h1,
                                         int h2, const float* __restrict__ us, const float* __restrict__ vs,
                                         int* bad) {
  __shared__ __align__(16) Tile<TH> st, su, sv;
  __shared__ RowCache<TH> sq;
  const int W = p.W, P = p.P, nx = p.nx, ny = p.ny;
  const int i0 = bx * TW + 1, j0 = by * TH + 1;
  fill_rows<TH>(p, j0, sq);
  const Rows rc{sq, j0};
  load_tile<TH>(td.ts[cur], P, i0, j0, st);
  load_tile<TH>(us, P, i0, j0, su);
  load_tile<TH>(vs, P, i0, j0, sv);
  __syncthreads();
  if (p.extra) {  // UWINDX, VWINDY (sw.h:216-217)
    for (int t = threadIdx.x; t < (TH + 4) * (TW + 4); t += nthreads<TH>()) {
      const int c = t % (TW + 4), r = t / (TW + 4);
      const int qq = IX32(P, i0 - 2 + c, j0 - 2 + r);
      su[r][c] += p.wx[qq];
      sv[r][c] += p.wy[qq];
    }
    __syncthreads();
  }
  const int ta = threadIdx.x % TW, tb = threadIdx.x / TW;
  const int a = ta + 2, b = tb + 2, i = i0 + ta, j = j0 + tb;
  if (i > nx || j > ny) return;
  const float kx = Q(rc, Q_KXE, j), ky = Q(rc, Q_KYN, j);
  const float uw = su[b][a - 1], ue = su[b][a], vsb = sv[b - 1][a], vn = sv[b][a];
  const float T = st[b][a];
  const float fw = face2<SCH>(st[b][a - 2], st[b][a - 1], T, st[b][a + 1], fmaxf(uw, 0.f) * kx, fminf(uw, 0.f) * kx);
  const float fe = face2<SCH>(st[b][a - 1], T, st[b][a + 1], st[b][a + 2], fmaxf(ue, 0.f) * kx, fminf(ue, 0.f) * kx);
  const float fs = face2<SCH>(st[b - 2][a], st[b - 1][a], T, st[b + 1][a], fmaxf(vsb, 0.f) * ky, fminf(vsb, 0.f) * ky);
  const float fn = face2<SCH>(st[b - 1][a], T, st[b + 1][a], st[b + 2][a], fmaxf(vn, 0.f) * ky, fminf(vn, 0.f) * ky);
  float dtr = (fw - fe) + (fs - fn);
  dtr += T * ((ue - uw) * kx + (vn - vsb) * ky);
  dtr -= td.sig2dt * T;
  const int q32 = IX32(P, i, j);
  float ab;
  if (p.k == 0) ab = dtr;
  else if (p.k == 1) ab = 1.5f * dtr - 0.5f * td.h[h1][q32];
  else ab = (23.f / 12.f) * dtr - (4.f / 3.f) * td.h[h1][q32] + (5.f / 12.f) * td.h[h2][q32];
  td.h[w][q32] = dtr;
  const double tn = td.tr[cur][IX(W, i, j)] + f2d(ab);
  put<IMG_ETA>(td.tr[1 - cur], W, nx, ny, i, j, tn);
  put<IMG_ETA>(td.ts[1 - cur], P, nx, ny, i, j, d2f(tn));
  if (!in_range(tn)) atomicOr(bad, 1);
}

struct Main2Io {
  const float* es;                        // new eta shadow
  const double* u; const double* v;       // FP64 state at step start (pitch W)
  const float* us; const float* vs;       // and its shadows (pitch P)
  double* u_next; double* v_next;
  float* us_next; float* vs_next;
  const float* dup; const float* dvp;
  const float* hu1; const float* hu2; const float* hv1; const float* hv2;
  float* hu0; float* hv0;                 // slots for Du_n, Dv_n
  int* bad;
};

// Pressure (calc.c:500-540), AB, Coriolis u then v (calc.c:542-598).
template <int TH>
__device__ __forceinline__ void d_main2(const KP& p, int bx, int by, const Main2Io& io, int tile_test) {
  constexpr int NT = nthreads<TH>(), TILE_ROWS = TH + 4;
  __shared__ __align__(16) Tile<TH> se, su, sv;  // ring-2 windows, ring 1 used
  __shared__ float un[TH + 1][TW + 1];       // new u at (i0-1+a, j0+b)
  __shared__ RowCache<TH> sq;
  const int W = p.W, P = p.P, nx = p.nx, ny = p.ny;
  const int i0 = bx * TW + 1, j0 = by * TH + 1;
  // own cell of the v update: issue its global loads first
  const int ac = threadIdx.x % TW, bc = threadIdx.x / TW;
  const int ic = i0 + ac, jc = j0 + bc;
  const bool livec = (ic <= nx && jc <= ny);
  const int qc = IX(W, livec ? ic : 1, livec ? jc : 1), qc32 = IX32(P, ic, jc);
  const double v_old = io.v[qc];
  const float dvp_c = io.dvp[qc32];
  const float hv1_c = (p.k >= 1) ? io.hv1[qc32] : 0.f, hv2_c = (p.k >= 2) ? io.hv2[qc32] : 0.f;
  // the (at most two) positions of the new-u region this thread updates:
  // their global operands are loaded now as well
  constexpr int NU = (TW + 1) * (TH + 1);
  static_assert(2 * NT >= NU, "two items of the new-u region per thread");
  float pre_dup[2], pre_h1[2], pre_h2[2];
  double pre_u[2];
#pragma unroll
  for (int s2 = 0; s2 < 2; s2++) {
    const int t = threadIdx.x + s2 * NT;
    const int a = t % (TW + 1), b = t / (TW + 1);
    const int i = i0 - 1 + a, j = j0 + b;
    const bool comp = (t < NU) && (i >= 1 && i <= nx && j <= ny);
    const bool own = comp && a >= 1 && b < TH;
    const int q32 = IX32(P, comp ? i : 1, comp ? j : 1);
    pre_dup[s2] = comp ? io.dup[q32] : 0.f;
    pre_h1[s2] = (comp && p.k >= 1) ? io.hu1[q32] : 0.f;
    pre_h2[s2] = (comp && p.k >= 2) ? io.hu2[q32] : 0.f;
    pre_u[s2] = own ? io.u[IX(W, i, j)] : 0.0;
  }
  __shared__ __align__(8) unsigned long long tbar;
  static_assert(3 * TILE_ROWS <= NT, "one thread per row copy");
  tiles_init(&tbar, 3 * TILE_ROWS);
  if (threadIdx.x < 3 * TILE_ROWS) {  // Coriolis uses U and V without the winds
    const int t = threadIdx.x / TILE_ROWS, r = threadIdx.x - t * TILE_ROWS;
    if (t == 0) tile_row_copy<TH>(&tbar, io.es, P, i0, j0, se, r);
    else if (t == 1) tile_row_copy<TH>(&tbar, io.us, P, i0, j0, su, r);
    else tile_row_copy<TH>(&tbar, io.vs, P, i0, j0, sv, r);
  }
  fill_rows<TH>(p, j0, sq);
  const Rows rc{sq, j0};
  if (!tiles_wait(&tbar, io.bad, tile_test)) return;
  // new u on [i0-1, i0+TW-1] x [j0, j0+TH]: interior cells recomputed, the
  // halo column 0 and the halo row ny+1 keep the old u (the v update reads
  // them before the halo refresh, core.c:283-289)
#pragma unroll
  for (int s2 = 0; s2 < 2; s2++) {
    const int t = threadIdx.x + s2 * NT;
    if (t >= NU) break;
    const int a = t % (TW + 1), b = t / (TW + 1);
    const int i = i0 - 1 + a, j = j0 + b;
    const int la = a + 1, lb = b + 2;  // ring-2 local of (i, j)
    float val = 0.f;
    if (i <= nx && j <= ny + 1) {
      if (i >= 1 && j <= ny) {
        const int q32 = IX32(P, i, j);
        const float dun = pre_dup[s2] + Q(rc, Q_GEX, j) * (se[lb][la + 1] - se[lb][la]);
        float ab;
        if (p.k == 0) ab = dun;
        else if (p.k == 1) ab = 1.5f * dun - 0.5f * pre_h1[s2];
        else ab = (23.f / 12.f) * dun - (4.f / 3.f) * pre_h1[s2] + (5.f / 12.f) * pre_h2[s2];
        const float uu = su[lb][la];
        const float semi = 0.25f * (sv[lb][la] + sv[lb][la + 1] + sv[lb - 1][la] + sv[lb - 1][la + 1]);
        const float al = Q(rc, Q_DTFE, j) + uu * Q(rc, Q_GEO, j);
        const float be = 0.25f * al * al;
        const float du = __fdividef(ab - 2.f * be * uu + al * semi, 1.f + be);
        val = uu + du;
        if (a >= 1 && b < TH) {  // a cell of this tile: accumulate in FP64 and write
          io.hu0[q32] = dun;
          const double unew = pre_u[s2] + f2d(du);
          put<IMG_U>(io.u_next, W, nx, ny, i, j, unew);
          put<IMG_U>(io.us_next, P, nx, ny, i, j, d2f(unew));
          if (!in_range(unew)) atomicOr(io.bad, 1);
        }
      } else {
        val = su[lb][la];
      }
    }
    un[b][a] = val;
  }
  __syncthreads();
  if (!livec) return;
  const int a = ac, b = bc, i = ic, j = jc, q32 = qc32;
  const int la = a + 2, lb = b + 2;
  const float dvn = dvp_c + Q(rc, Q_GNY, j) * (se[lb + 1][la] - se[lb][la] + Q(rc, Q_DHBP1, j));
  float ab;
  if (p.k == 0) ab = dvn;
  else if (p.k == 1) ab = 1.5f * dvn - 0.5f * hv1_c;
  else ab = (23.f / 12.f) * dvn - (4.f / 3.f) * hv1_c + (5.f / 12.f) * hv2_c;
  const float vv = sv[lb][la];
  // un local: (i-1, j+1) -> (a, b+1), (i, j+1) -> (a+1, b+1), (i, j) -> (a+1, b), (i-1, j) -> (a, b)
  const float semi = 0.25f * (un[b + 1][a] + un[b + 1][a + 1] + un[b][a + 1] + un[b][a]);
  const float al = Q(rc, Q_DTFN, j) + semi * Q(rc, Q_CV, j);
  const float be = 0.25f * al * al;
  const float dv = __fdividef(ab - 2.f * be * vv - al * semi, 1.f + be);
  io.hv0[q32] = dvn;
  const double vnew = v_old + f2d(dv);
  put<IMG_V>(io.v_next, W, nx, ny, i, j, vnew);
  put<IMG_V>(io.vs_next, P, nx, ny, i, j, d2f(vnew));
  if (!in_range(vnew)) atomicOr(io.bad, 1);
}

// ------------------------------------------------------------ batched launch
// One launch per phase covers every tile of every member of a batch (a single
// context is a batch of one). The member descriptors travel by value in the
// launch parameters (the constant bank), so their fields are read like kernel
// arguments: uniform over the block and loaded where they are used rather than
// held in registers. With one member the grid is the member's nbx x nby tiles;
// otherwise block b works on tiles[b] = (member, bx, by).
// Buffer rotation is derived from a device step counter n, which a one-thread
// kernel advances after each step (see MemberDesc), so a captured graph of one
// step can be replayed for any number of steps.
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

__device__ __forceinline__ KP kp_of(const MemberDesc& d, int k) {
  KP p;
  p.nx = d.nx; p.ny = d.ny; p.W = d.nx + 4; p.H = d.ny + 4; p.P = d.P;
  p.q = d.q;
  p.sig2dt = d.sig2dt; p.sigdt = d.sigdt; p.nu2dt = d.nu2dt; p.nu4dt = d.nu4dt; p.nu6dt = d.nu6dt;
  p.k = k;
  p.extra = d.extra;
  p.wx = d.wx; p.wy = d.wy; p.hb = d.hb;
  return p;
}

template <int N>
__device__ __forceinline__ int4 tile_of(const int4* __restrict__ tiles) {
  if constexpr (N == 1) return make_int4(0, blockIdx.x, blockIdx.y, 0);
  else return tiles[blockIdx.x];
}

// Resident blocks per SM the register allocation must allow (measured:
// kb_lap1 at 8 and kb_main2 at 6 are 9-15 % faster than at their natural 6
// and 5; kb_main1 gains nothing beyond 6).
template <int TH, int N>
__global__ void __launch_bounds__(nthreads<TH>(), 2048 / nthreads<TH>())
    kb_lap1(const __grid_constant__ DescSet<N> ds, const int4* __restrict__ tiles, const int* __restrict__ counter) {
  const int4 t = tile_of<N>(tiles);
  const int n = *counter;
  const MemberDesc& d = ds.m[N == 1 ? 0 : t.x];
  const View v = view_of(d, n);
  d_lap1<TH>(kp_of(d, v.k), t.y, t.z, d.us[v.cur], d.vs[v.cur], d.Lu, d.Lv);
}

// Tracer advection: members without an active tracer return at once.
template <int SCH, int TH, int N>
__global__ void __launch_bounds__(nthreads<TH>())
    kb_tracer(const __grid_constant__ DescSet<N> ds, const int4* __restrict__ tiles, const int* __restrict__ counter) {
  const int4 t = tile_of<N>(tiles);
  const int n = *counter;
  const MemberDesc& d = ds.m[N == 1 ? 0 : t.x];
  if (!d.trd) return;
  const View v = view_of(d, n);
  d_tracer<SCH, TH>(kp_of(d, v.k), t.y, t.z, *d.trd, v.cur, v.w, v.h1, v.h2, d.us[v.cur], d.vs[v.cur],
                    d.bad + v.slot);
}

// Third Laplacian level (nu6): members without it return at once.
template <int TH, int N>
__global__ void __launch_bounds__(nthreads<TH>(), 2048 / nthreads<TH>())
    kb_lap3(const __grid_constant__ DescSet<N> ds, const int4* __restrict__ tiles, const int* __restrict__ counter) {
  const int4 t = tile_of<N>(tiles);
  const int n = *counter;
  const MemberDesc& d = ds.m[N == 1 ? 0 : t.x];
  if (d.nu6dt == 0.f) return;
  const View v = view_of(d, n);
  d_lap1<TH, true>(kp_of(d, v.k), t.y, t.z, d.LLu, d.LLv, d.dup, d.dvp);
}

template <int SCH, int TH, int N>
__global__ void __launch_bounds__(nthreads<TH>())
    kb_main1(const __grid_constant__ DescSet<N> ds, const int4* __restrict__ tiles, const int* __restrict__ counter) {
  const int4 t = tile_of<N>(tiles);
  const int n = *counter;
  const MemberDesc& d = ds.m[N == 1 ? 0 : t.x];
  const View v = view_of(d, n);
  const Main1Io o{d.eta[v.cur], d.es[v.cur], d.us[v.cur], d.vs[v.cur], d.Lu, d.Lv, d.heta[v.h1], d.heta[v.h2],
                  d.eta[1 - v.cur], d.es[1 - v.cur], d.heta[v.w], d.dup, d.dvp, d.LLu, d.LLv,
                  d.cfl + 2 * v.slot, d.bad + v.slot};
  d_main1<SCH, TH>(kp_of(d, v.k), t.y, t.z, o);
}

template <int TH, int N>
__global__ void __launch_bounds__(nthreads<TH>(), 1536 / nthreads<TH>())
    kb_main2(const __grid_constant__ DescSet<N> ds, const int4* __restrict__ tiles, const int* __restrict__ counter) {
  const int4 t = tile_of<N>(tiles);
  const int n = *counter;
  const MemberDesc& d = ds.m[N == 1 ? 0 : t.x];
  const View v = view_of(d, n);
  const Main2Io io{d.es[1 - v.cur], d.u[v.cur], d.v[v.cur], d.us[v.cur], d.vs[v.cur], d.u[1 - v.cur],
                   d.v[1 - v.cur], d.us[1 - v.cur], d.vs[1 - v.cur], d.dup, d.dvp, d.hu[v.h1], d.hu[v.h2],
                   d.hv[v.h1], d.hv[v.h2], d.hu[v.w], d.hv[v.w], d.bad + v.slot};
  d_main2<TH>(kp_of(d, v.k), t.y, t.z, io, d.tile_test);
}

__global__ void kb_advance(int* counter) { *counter += 1; }

// FP32 shadow of an FP64 field over all padded cells (pitch W -> pitch P).
__global__ void k_shadow(float* dst, const double* src, int nx, int ny, int W, int P) {
  const int n = W * (ny + 4);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int r = t / W, c = t - r * W;
    dst[(size_t)r * P + c] = d2f(src[t]);
  }
}

}  // namespace f32

using namespace f32;

void fp32_shadow(float* dst, const double* src, int nx, int ny, int P, cudaStream_t st) {
  const int W = nx + 4, n = W * (ny + 4);
  const int blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_shadow<<<blocks, 256, 0, st>>>(dst, src, nx, ny, W, P);
}

void fp32_geometry(int nx, int ny, int* P, int* R) {
  *P = TW * ((nx + TW - 1) / TW) + 4;
  *R = kTileRowsMax * ((ny + kTileRowsMax - 1) / kTileRowsMax) + 4;  // in bounds for every tile height
}

void fp32_tiles(int nx, int ny, int th, int* nbx, int* nby) {
  *nbx = (nx + TW - 1) / TW;
  *nby = (ny + th - 1) / th;
}

MemberDesc fp32_desc(const Fp32Ctx& c, const Fp32Engine& e, int k) {
  MemberDesc d;
  std::memset(&d, 0, sizeof d);  // padding included, so descriptors compare with memcmp
  d.nx = c.nx; d.ny = c.ny; d.P = c.P;
  d.extra = c.extra;
  d.sig2dt = c.sig2dt; d.sigdt = c.sigdt; d.nu2dt = c.nu2dt; d.nu4dt = c.nu4dt; d.nu6dt = c.nu6dt;
  d.q = c.q;
  d.wx = c.wx; d.wy = c.wy; d.hb = c.hb;
  for (int q = 0; q < 2; q++) {
    d.eta[q] = e.eta[q]; d.u[q] = e.u[q]; d.v[q] = e.v[q];
    d.es[q] = e.es[q]; d.us[q] = e.us[q]; d.vs[q] = e.vs[q];
  }
  for (int q = 0; q < 3; q++) {
    d.heta[q] = e.heta[q]; d.hu[q] = e.hu[q]; d.hv[q] = e.hv[q];
  }
  d.Lu = e.Lu; d.Lv = e.Lv; d.dup = e.dup; d.dvp = e.dvp;
  d.LLu = e.LLu; d.LLv = e.LLv;
  d.trd = e.tracer ? e.d_trd : nullptr;
  d.cfl = e.cfl; d.bad = e.bad;
  d.cur0 = e.cur;
  d.w0 = e.w;
  d.k0 = k > 2 ? 2 : k;
  d.tile_test = c.tile_test;
  return d;
}

MemberDesc fp32_desc_after(const MemberDesc& d, int n) {
  MemberDesc a = d;
  a.cur0 = d.cur0 ^ (n & 1);
  a.w0 = (d.w0 + n % 3) % 3;
  a.k0 = (n >= 2 - d.k0) ? 2 : d.k0 + n;
  return a;
}

void Fp32Engine::advance_host(long long nsteps) {
  if (nsteps & 1) cur = 1 - cur;
  w = (int)((w + nsteps % 3) % 3);
}

namespace {

template <int TH, int N>
int batch_step_n(int sch, const MemberDesc* desc, int nmem, const int4* tiles, int ntiles, int nbx, int nby,
                 int* counter, cudaStream_t st, Timers* tm) {
  static_assert(sizeof(DescSet<N>) + 3 * sizeof(void*) <= 32760, "launch parameters are limited to 32 KB");
  constexpr int NT = nthreads<TH>();
  std::vector<DescSet<N>> hold(1);  // heap: up to ~28 KB
  DescSet<N>& ds = hold[0];
  std::memset(&ds, 0, sizeof ds);
  for (int m = 0; m < nmem; m++) ds.m[m] = desc[m];
  const dim3 g = (N == 1) ? dim3(nbx, nby) : dim3(ntiles);
  int nl = 0;
#define LAUNCH(tag, ...)                        \
  do {                                          \
    if (tm && tm->on) tm->begin(tag, st);       \
    __VA_ARGS__;                                \
    if (tm && tm->on) tm->end(st);              \
    nl++;                                       \
  } while (0)
#define MAIN1(S) LAUNCH("f32_main1", (kb_main1<S, TH, N><<<g, NT, 0, st>>>(ds, tiles, counter)))
#define TRACER(S) LAUNCH("f32_tracer", (kb_tracer<S, TH, N><<<g, NT, 0, st>>>(ds, tiles, counter)))
  bool tracer = false;
  for (int m = 0; m < nmem; m++) tracer = tracer || (desc[m].trd != nullptr);
  if (tracer) {  // reads the step's old u, v and tracer only (core.c:161-182)
    switch (sch) {
      case 0: TRACER(0); break;
      case 1: TRACER(1); break;
      case 2: TRACER(2); break;
      case 4: TRACER(4); break;
      case 5: TRACER(5); break;
      case 6: TRACER(6); break;
      case 7: TRACER(7); break;
      case 8: TRACER(8); break;
      case 9: TRACER(9); break;
      default: TRACER(kVanLeerSafe); break;
    }
  }
  LAUNCH("f32_lap1", (kb_lap1<TH, N><<<g, NT, 0, st>>>(ds, tiles, counter)));
  switch (sch) {
    case 0: MAIN1(0); break;
    case 1: MAIN1(1); break;
    case 2: MAIN1(2); break;
    case 3: MAIN1(3); break;
    case 4: MAIN1(4); break;
    case 5: MAIN1(5); break;
    case 6: MAIN1(6); break;
    case 7: MAIN1(7); break;
    case 8: MAIN1(8); break;
    case 9: MAIN1(9); break;
    default: MAIN1(kVanLeerSafe); break;
  }
  bool nu6 = false;
  for (int m = 0; m < nmem; m++) nu6 = nu6 || (desc[m].nu6dt != 0.f);
  if (nu6) LAUNCH("f32_lap3", (kb_lap3<TH, N><<<g, NT, 0, st>>>(ds, tiles, counter)));
  LAUNCH("f32_main2", (kb_main2<TH, N><<<g, NT, 0, st>>>(ds, tiles, counter)));
  kb_advance<<<1, 1, 0, st>>>(counter);
  nl++;
#undef MAIN1
#undef TRACER
#undef LAUNCH
  return nl;
}

template <int TH>
int batch_step_th(int sch, const MemberDesc* desc, int nmem, const int4* tiles, int ntiles, int nbx, int nby,
                  int* counter, cudaStream_t st, Timers* tm) {
  if (nmem == 1) return batch_step_n<TH, 1>(sch, desc, nmem, tiles, ntiles, nbx, nby, counter, st, tm);
  if (nmem <= 16) return batch_step_n<TH, 16>(sch, desc, nmem, tiles, ntiles, nbx, nby, counter, st, tm);
  return batch_step_n<TH, kMaxBatch>(sch, desc, nmem, tiles, ntiles, nbx, nby, counter, st, tm);
}

}  // namespace

int fp32_batch_step(int sch, int th, const MemberDesc* desc, int nmem, const int4* tiles, int ntiles, int nbx,
                    int nby, int* counter, cudaStream_t st, Timers* tm) {
  if (th == 4) return batch_step_th<4>(sch, desc, nmem, tiles, ntiles, nbx, nby, counter, st, tm);
  if (th == 16) return batch_step_th<16>(sch, desc, nmem, tiles, ntiles, nbx, nby, counter, st, tm);
  return batch_step_th<8>(sch, desc, nmem, tiles, ntiles, nbx, nby, counter, st, tm);
}

}  // namespace sw2g

namespace sw2g {
namespace {
__global__ void k_add_row_ref(double* dst, const double* src, const double* ref, int W, int H) {
  const size_t n = (size_t)W * H;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int row = (int)(t / W);
    dst[t] = src[t] + ref[row];
  }
}
}  // namespace

void add_row_ref(double* dst, const double* src, const double* ref_rows, int nx, int ny, cudaStream_t st) {
  const int W = nx + 4, H = ny + 4;
  const size_t n = (size_t)W * H;
  const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  k_add_row_ref<<<blocks, 256, 0, st>>>(dst, src, ref_rows, W, H);
}
}  // namespace sw2g
