// Reference-exact FP64 step, in core.c's order (core.c:134-338). The first
// two steps after an upload run one kernel per reference routine; from the
// third (AB3) the tails of the tendencies are fused, the Laplacian passes
// write their own halo images and wall fixes, and the range checks are made
// by the kernels that write the state. Compiled with -fmad=false so that no
// a*b+c is fused: every expression keeps the association of the reference
// expression it restates, which makes the results bit-identical to the
// reference's own single-rank run. Divisions by a per-row metric factor go
// through div_rcp (the same IEEE quotient with fewer FP64 instructions),
// scalings by powers of two, zero numerators and bit tests are answered on
// the integer pipe, since GB300 executes FP64 at 2 lanes per SM per clock,
// and so are some of the small kernels' additions (sadd, ssub: the same
// IEEE sums).
#include <cuda_runtime.h>

#include "sw2g_internal.h"

namespace sw2g {
namespace {

constexpr int TX = 128;

__device__ __forceinline__ int IX(int W, int i, int j) { return (i + 1) + (j + 1) * W; }
__device__ __forceinline__ double RW(const DevState& s, int t, int j) { return s.rows[t * s.H + j + 1]; }
// A field of a polar cap at padded index q.
__device__ __forceinline__ double PF(const DevState& s, int t, int q) { return s.pf[(size_t)t * s.W * s.H + q]; }

// The bit pattern of a double, through an opaque move: tests written on the
// integer image (sign, exponent, zero) then stay integer operations; given
// the plain reinterpretation, the compiler may turn them back into FP64
// comparisons, which issue on GB300's narrow FP64 unit.
__device__ __forceinline__ long long dbits(double x) {
  long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}

__device__ __forceinline__ int dexp(double x) {
  return (int)(((unsigned long long)dbits(x) >> 52) & 0x7ffULL);
}

// a / b with a zero numerator answered from the bits: IEEE division gives
// +-0 / b the zero whose sign is the exclusive or of the operands' signs for
// every b other than a zero or a NaN; there the hardware sequence would take
// its special-case path (about 15 FP64 instructions). Other operands divide.
// The literal cells use it: in a state at rest their velocities, Courant
// numbers and differences are zeros.
__device__ __forceinline__ double zdiv(double a, double b) {
  const long long A = dbits(a), B = dbits(b);
  const long long mb = B & 0x7fffffffffffffffLL;
  if ((A & 0x7fffffffffffffffLL) == 0 && mb != 0 && mb <= 0x7ff0000000000000LL)
    return __longlong_as_double((A ^ B) & (long long)0x8000000000000000ULL);
  return a / b;
}

// x * 2^k for k in -2..1 (p = 2^k), the same value as the FP64 product: when
// x and the product are normal numbers, the product only changes the exponent
// field, done here on the integer pipe; zeros are their own product; other
// cases (subnormal operand or result, inf, NaN) multiply, out of line.
__device__ __noinline__ double mul_pow2_fp64(double x, double p) { return x * p; }
__device__ __forceinline__ double mul_pow2(double x, int k, double p) {
  const long long b = dbits(x);
  if ((b & 0x7fffffffffffffffLL) == 0) return x;
  const int e = (int)((b >> 52) & 0x7ff);
  if (e >= 1 && e <= 2046 && e + k >= 1 && e + k <= 2046) return __longlong_as_double(b + ((long long)k << 52));
  return mul_pow2_fp64(x, p);
}
#define HALF(x) mul_pow2((x), -1, 0.5)
#define QUARTER(x) mul_pow2((x), -2, 0.25)
#define TWICE(x) mul_pow2((x), 1, 2.0)

// Correctly rounded a/b given y = RN(1/b), b a positive normal number, with
// one multiplication and two fused multiply-adds (Markstein's method:
// P. Markstein, IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et al., Handbook
// of Floating-Point Arithmetic, ch. "division with an FMA"): q0 = RN(a*y),
// r0 = a - b*q0 (exact), RN(q0 + r0*y) = RN(a/b). Markstein's theorem covers
// q0 within one ulp of a/b; RN(a*y) can be up to 1.5 ulps off, and the one
// correction still rounds correctly there by the case analysis of a/b in
// [1/2, 1) scaled (a wrong rounding would need a and b both within a few
// ulps of a power of two, a set the self-check walks exhaustively, with
// random and near-midpoint numerators on top: fp64_check_division).
// A zero numerator gives itself (+-0 / b = +-0 for b > 0); other numerators
// outside [2^-900, 2^776] (subnormals: remainders could underflow; inf, NaN)
// use the IEEE division. The row tables hold y = 1.0/b computed by IEEE
// division on the host. fp64_check_division compares this with the IEEE
// quotient on random and near-halfway numerators.
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
  if ((dbits(a) & 0x7fffffffffffffffLL) == 0) return a;
  if ((unsigned)(dexp(a) - 123) > 1799u - 123u) return a / b;
  const double q0 = __dmul_rn(a, y);
  const double r0 = __fma_rn(-b, q0, a);
  return __fma_rn(r0, y, q0);
}

// a + b rounded to nearest, ties to even, computed on the integer pipe (the
// textbook IEEE 754 adder: order the operands by magnitude, align the
// smaller significand with ten guard bits and a sticky bit, add or subtract,
// renormalise, round) when both operands and the sum are normal numbers. A
// zero operand gives the other operand (two zeros give -0 only if both are
// -0), and exact cancellation gives +0, as the FP64 unit's round-to-nearest
// does. Everything else (subnormals, inf, NaN, a sum that overflows or falls
// below the normal range) adds on the FP64 unit, out of line. fp64_check_add
// compares sadd and ssub with the FP64 unit on random and edge-case operands.
// An integer-pipe addition takes about a hundred instructions where the FP64
// unit takes one, but GB300 issues 128 integer operations per SM and clock
// against 2 FP64 lanes: the small kernels below are bound by the FP64 unit
// with most issue slots idle, so moving some of their additions off it makes
// them faster, up to the point where issue becomes the bound. Which additions
// move was measured per kernel at 2048x1024 (CUDA-event times of each mix):
// all of the Coriolis updates' and of the second velocity-Laplacian pass,
// the two outer sums of the first pass, the final sum of the second
// eta-Laplacian pass, the Adams-Bashforth and hyperviscosity sums, the two
// tendency sums of k_pres_sum; in the TVD bodies only the four-face sum of a
// cell and, in the mass body, the last sum of each side term (their 96
// registers per thread leave too few warps to hide longer chains: more
// integer-pipe additions there made them slower); none in the first
// eta-Laplacian pass (no gain).
__device__ __noinline__ double add_fp64(double a, double b) { return a + b; }
__device__ __forceinline__ double sadd(double a, double b) {
  constexpr unsigned long long MAG = 0x7fffffffffffffffULL, FRAC = 0x000fffffffffffffULL, ONE = 1ULL << 52;
  unsigned long long A = (unsigned long long)dbits(a), B = (unsigned long long)dbits(b);
  if ((A & MAG) < (B & MAG)) {  // |A| >= |B| from here on
    const unsigned long long t = A;
    A = B;
    B = t;
  }
  const int ea = (int)((A >> 52) & 0x7ff), eb = (int)((B >> 52) & 0x7ff);
  if ((B & MAG) == 0)  // the smaller is a zero: the larger (a NaN stays a NaN);
    // two zeros: -0 if both are, else +0
    return __longlong_as_double((long long)(((A & MAG) == 0) ? (A & B) : A));
  if (ea == 0x7ff || eb == 0) return add_fp64(a, b);  // inf, NaN or a subnormal operand
  const int d = ea - eb;
  const unsigned long long ma = ((A & FRAC) | ONE) << 10;  // significand at bits 62..10
  unsigned long long mb = ((B & FRAC) | ONE) << 10;
  if (d >= 63) {
    mb = 1;  // only the sticky bit is left
  } else if (d > 0) {
    mb = (mb >> d) | ((mb << (64 - d)) != 0 ? 1ULL : 0ULL);
  }
  int e = ea;
  unsigned long long m;
  if (((A ^ B) >> 63) == 0) {
    m = ma + mb;
    if (m >> 63) {  // carry: one bit right, keeping the sticky bit
      m = (m >> 1) | (m & 1ULL);
      e += 1;
    }
  } else {
    m = ma - mb;
    if (m == 0) return 0.0;
    const int lz = __clzll((long long)m) - 1;  // back to bit 62 (at most one place when bits were lost)
    m <<= lz;
    e -= lz;
  }
  unsigned long long r = m >> 10;
  const unsigned long long rem = m & 0x3ffULL;
  if (rem > 0x200ULL || (rem == 0x200ULL && (r & 1ULL))) r += 1;
  if (r >> 53) {
    r >>= 1;
    e += 1;
  }
  if (e <= 0 || e >= 0x7ff) return add_fp64(a, b);
  return __longlong_as_double((long long)((A & ~MAG) | ((unsigned long long)e << 52) | (r & FRAC)));
}
// a - b = a + (-b), exactly and for every operand (a NaN operand gives a
// NaN either way; NaN bit patterns are not compared anywhere).
__device__ __forceinline__ double ssub(double a, double b) {
  return sadd(a, __longlong_as_double(dbits(b) ^ (long long)0x8000000000000000ULL));
}

// calc.c:54-63 with sw.h:104-105 MIN/MAX as ternaries (NaN order as written).
template <int SCH>
__device__ __forceinline__ double limiter(double r) {
#define MN(a, b) (((a) < (b)) ? (a) : (b))
#define MX(a, b) (((a) > (b)) ? (a) : (b))
  if constexpr (SCH == 0) return MX(0.0, MN(MN((1 + r) / 2.0, 2.0 * r), 2.0));
  else if constexpr (SCH == 1) return MX(MX(0.0, MN(2.0 * r, 1.0)), MX(0.0, MN(r, 2.0)));
  else if constexpr (SCH == 2) return MN(r, 1.0);
  else if constexpr (SCH == 3) return zdiv(r + fabs(r), 1.0 + r);
  else if constexpr (SCH == 4) return MX(0.0, MN(2.0 * r, MN((1 + 2.0 * r) / 3.0, 2.0)));
  else if constexpr (SCH == 5) return zdiv(1.5 * (r * r + r), r * r + r + 1.0);
  else if constexpr (SCH == 6) return zdiv(r * r + r, r * r + 1.0);
  else if constexpr (SCH == 7) return MX(0.0, MN(MN(2.0, 2.0 * r), MN(0.25 + 0.75 * r, 0.75 + 0.25 * r)));
  else if constexpr (SCH == 8) return 0.0;
  else if constexpr (SCH == 9) return 1.0;
  else return (r == -1.0) ? 0.0 : zdiv(r + fabs(r), 1.0 + r);
#undef MN
#undef MX
}

// One face q0|q1 with outer neighbours qm, q2 (calc.c:41-49).
template <int SCH>
__device__ __forceinline__ void tvd_face(double qm, double q0, double q1, double q2, double cP, double cM,
                                         double& BP, double& BM) {
  const double d = q1 - q0;
  const double rP = (d != 0) ? zdiv(q0 - qm, d) : 0.0;
  const double rM = (d != 0) ? zdiv(q2 - q1, d) : 0.0;
  BP = q0 + limiter<SCH>(rP) * 0.5 * (1 - cP) * d;
  BM = q1 - limiter<SCH>(rM) * 0.5 * (1 + cM) * d;
}

// Sum C*B over the four faces in the reference's order (calc.c:100).
template <int SCH>
__device__ __forceinline__ double tvd_sum(const double* qx, const double* qy, double cwP, double cwM, double ceP,
                                          double ceM, double csP, double csM, double cnP, double cnM) {
  double wP, wM, eP, eM, sP, sM, nP, nM;
  tvd_face<SCH>(qx[0], qx[1], qx[2], qx[3], cwP, cwM, wP, wM);
  tvd_face<SCH>(qx[1], qx[2], qx[3], qx[4], ceP, ceM, eP, eM);
  tvd_face<SCH>(qy[0], qy[1], qy[2], qy[3], csP, csM, sP, sM);
  tvd_face<SCH>(qy[1], qy[2], qy[3], qy[4], cnP, cnM, nP, nM);
  return cwP * wP + cwM * wM - ceP * eP - ceM * eM + csP * sP + csM * sM - cnP * nP - cnM * nM;
}

__device__ __forceinline__ double cpos(double a, double dt, double dx) { return zdiv(0.5 * (a + fabs(a)) * dt, dx); }
__device__ __forceinline__ double cneg(double a, double dt, double dx) { return zdiv(0.5 * (a - fabs(a)) * dt, dx); }
__device__ __forceinline__ double cpos2(double a, double b, double dt, double dx) {
  return zdiv(0.5 * (0.5 * (a + fabs(a)) + 0.5 * (b + fabs(b))) * dt, dx);
}
__device__ __forceinline__ double cneg2(double a, double b, double dt, double dx) {
  return zdiv(0.5 * (0.5 * (a - fabs(a)) + 0.5 * (b - fabs(b))) * dt, dx);
}

struct F7 {
  const double *eta, *u, *v, *tr, *wx, *wy, *hb;
};

#define UW(i, j) (f.u[IX(W, i, j)] + f.wx[IX(W, i, j)])                   /* sw.h:216 */
#define VW(i, j) (f.v[IX(W, i, j)] + f.wy[IX(W, i, j)])                   /* sw.h:217 */
#define HH(i, j) (f.eta[IX(W, i, j)] + s.depth - f.hb[IX(W, i, j)])       /* sw.h:213 */

#define INTERIOR_IJ                                   \
  const int W = s.W;                                  \
  const int i = blockIdx.x * TX + threadIdx.x + 1;    \
  const int j = blockIdx.y + 1;                       \
  if (i > s.nx) return;

// BODYH + damping (calc.c:70-113), one cell
template <int SCH>
__device__ __forceinline__ double mass_cell(const DevState& s, const F7& f, int i, int j) {
  const int W = s.W;
  const double Dt = s.Dt, dxe = RW(s, R_DXE, j), dyn = RW(s, R_DYN, j);
  double qx[5], qy[5];
#pragma unroll
  for (int o = -2; o <= 2; o++) { qx[o + 2] = HH(i + o, j); qy[o + 2] = HH(i, j + o); }
  const double a = UW(i - 1, j), b = UW(i, j), c = VW(i, j - 1), d = VW(i, j);
  double acc = tvd_sum<SCH>(qx, qy, cpos(a, Dt, dxe), cneg(a, Dt, dxe), cpos(b, Dt, dxe), cneg(b, Dt, dxe),
                            cpos(c, Dt, dyn), cneg(c, Dt, dyn), cpos(d, Dt, dyn), cneg(d, Dt, dyn));
  const double sigma = s.polar ? PF(s, P_SH, IX(W, i, j)) : s.sigma;  // the sponge, calc.c:102-111
  acc -= 2.0 * Dt * (sigma) * f.eta[IX(W, i, j)];
  return acc;
}

// Programmatic dependent launch of the step's kernels: each kernel starts by
// waiting for the previous kernel of the stream to complete (a no-op for a
// kernel launched without the attribute) and then lets the next one be
// scheduled, which happens once all of its own blocks are resident; so a
// launch's scheduling overlaps the drain of the kernel before it, and no
// kernel reads or writes memory before its predecessor has finished.
#define SW2G_PDL_ENTRY()                                            \
  do {                                                              \
    asm volatile("griddepcontrol.wait;" ::: "memory");              \
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); \
  } while (0)

template <typename... KArgs, typename... Args>
void pdl_launch(void (*k)(KArgs...), dim3 g, dim3 b, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = g;
  cfg.blockDim = b;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

template <int SCH>
__global__ void k_mass(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  out[IX(W, i, j)] = mass_cell<SCH>(s, f, i, j);
}

// BODYTRACER (calc.c:117-163)
template <int SCH>
__global__ void k_tracer(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const double Dt = s.Dt, dxe = RW(s, R_DXE, j), dyn = RW(s, R_DYN, j);
  double qx[5], qy[5];
#pragma unroll
  for (int o = -2; o <= 2; o++) { qx[o + 2] = f.tr[IX(W, i + o, j)]; qy[o + 2] = f.tr[IX(W, i, j + o)]; }
  const double a = UW(i - 1, j), b = UW(i, j), c = VW(i, j - 1), d = VW(i, j);
  const double pv1 = tvd_sum<SCH>(qx, qy, cpos(a, Dt, dxe), cneg(a, Dt, dxe), cpos(b, Dt, dxe), cneg(b, Dt, dxe),
                                  cpos(c, Dt, dyn), cneg(c, Dt, dyn), cpos(d, Dt, dyn), cneg(d, Dt, dyn));
  const double t = qx[2];
  double pv2 = zdiv(Dt * t * (b - a), dxe);
  pv2 += zdiv(Dt * t * (d - c), dyn);
  double acc = pv1 + pv2;
  const double sigma = s.polar ? PF(s, P_STR, IX(W, i, j)) : s.sigma_tr;  // calc.c:152-161
  acc -= 2.0 * Dt * (sigma) * t;
  out[IX(W, i, j)] = acc;
}

// BODYU (calc.c:168-200), one cell
template <int SCH>
__device__ __forceinline__ double advu_cell(const DevState& s, const F7& f, int i, int j) {
  const int W = s.W;
  const double Dt = s.Dt, dxc = RW(s, R_DXC, j), dyv = RW(s, R_DYV, j);
  double qx[5], qy[5];
#pragma unroll
  for (int o = -2; o <= 2; o++) { qx[o + 2] = UW(i + o, j); qy[o + 2] = UW(i, j + o); }
  const double uwm = qx[1], u0 = qx[2], uep = qx[3];
  const double vs0 = VW(i, j - 1), vs1 = VW(i + 1, j - 1), vn0 = VW(i, j), vn1 = VW(i + 1, j);
  const double p1 = tvd_sum<SCH>(qx, qy, cpos2(uwm, u0, Dt, dxc), cneg2(uwm, u0, Dt, dxc), cpos2(u0, uep, Dt, dxc),
                                 cneg2(u0, uep, Dt, dxc), cpos2(vs0, vs1, Dt, dyv), cneg2(vs0, vs1, Dt, dyv),
                                 cpos2(vn0, vn1, Dt, dyv), cneg2(vn0, vn1, Dt, dyv));
  const double p2 = Dt * (zdiv(u0 * (uep - uwm), RW(s, R_DXE2, j)) + zdiv(u0 * ((vn0 + vn1) / 2. - (vs0 + vs1) / 2.), dyv));
  return p1 + p2;
}

template <int SCH>
__global__ void k_adv_u(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  out[IX(W, i, j)] = advu_cell<SCH>(s, f, i, j);
}

// BODYV (calc.c:205-237), one cell
template <int SCH>
__device__ __forceinline__ double advv_cell(const DevState& s, const F7& f, int i, int j) {
  const int W = s.W;
  const double Dt = s.Dt, dxv = RW(s, R_DXV, j), dyc = RW(s, R_DYC, j);
  double qx[5], qy[5];
#pragma unroll
  for (int o = -2; o <= 2; o++) { qx[o + 2] = VW(i + o, j); qy[o + 2] = VW(i, j + o); }
  const double vsm = qy[1], v0 = qy[2], vnp = qy[3];
  const double uw1 = UW(i - 1, j + 1), uw0 = UW(i - 1, j), ue1 = UW(i, j + 1), ue0 = UW(i, j);
  const double p1 = tvd_sum<SCH>(qx, qy, cpos2(uw1, uw0, Dt, dxv), cneg2(uw1, uw0, Dt, dxv), cpos2(ue1, ue0, Dt, dxv),
                                 cneg2(ue1, ue0, Dt, dxv), cpos2(vsm, v0, Dt, dyc), cneg2(vsm, v0, Dt, dyc),
                                 cpos2(v0, vnp, Dt, dyc), cneg2(v0, vnp, Dt, dyc));
  const double p2 = Dt * (zdiv(v0 * ((ue0 + ue1) / 2. - (uw0 + uw1) / 2.), dxv) + zdiv(v0 * (vnp - vsm), RW(s, R_DYNS, j)));
  return p1 + p2;
}

template <int SCH>
__global__ void k_adv_v(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  out[IX(W, i, j)] = advv_cell<SCH>(s, f, i, j);
}

// Literal cells for the fast kernels' fallback, kept out of line.
template <int SCH>
__device__ __noinline__ double mass_cell_ool(const DevState& s, const F7& f, int i, int j) {
  return mass_cell<SCH>(s, f, i, j);
}
template <int SCH>
__device__ __noinline__ double advu_cell_ool(const DevState& s, const F7& f, int i, int j) {
  return advu_cell<SCH>(s, f, i, j);
}
template <int SCH>
__device__ __noinline__ double advv_cell_ool(const DevState& s, const F7& f, int i, int j) {
  return advv_cell<SCH>(s, f, i, j);
}

// ------------------------------------------------------------ fast TVD bodies
// The same values as k_mass, k_adv_u and k_adv_v, bit for bit, with about a
// third of their FP64 operations. Three properties of the reference formulas
// (calc.c:41-49, 70-237) make that possible:
//  (1) x faces. With polar 0 the metric factors DXE, DXC, DXV depend on j
//      only, so the Courant numbers, limiter ratios and limited values of the
//      face between columns i-1 and i are the same operations on the same
//      operands for cell i (its west face) and cell i-1 (its east face). Each
//      lane of a warp computes the face west of its column; a warp covers 31
//      cells with 32 faces and takes the east face from the next lane.
//  (2) y faces. The ratios and limiter values of the face between rows j and
//      j+1 are shared by both cells; only the Courant numbers differ, since
//      each cell divides by its own DYN, DYV or DYC. A warp marches up its
//      rows and carries the face's shared part from one row to the next.
//  (3) Upwind split. C+ = 0.5(U+|U|)*Dt/DX is +0 when U <= 0, and C- is a
//      zero when U >= 0 (for the two-velocity averages, when both are), so
//      the term C*B of an unused side is a zero whenever B is finite, and
//      0.5(U+|U|) = U exactly when U > 0 (0.5(U-|U|) = U when U < 0). Leaving
//      zero terms out of a sum of otherwise identical terms, in the same
//      order, can change only the sign of a zero result. So the unused side
//      is skipped, and a cell is recomputed literally when its sum is zero,
//      when an input is not finite, or when the skipped side's limiter ratio
//      could exceed 2^498 (the bound under which every limiter gives a finite
//      value, squares included).
// The Van Leer limiter in its reference form (0/0 at r = -1) keeps the
// literal kernels.
constexpr int FW = 31;      // cells per strip along x (32 faces)
constexpr int FWARPS = 4;   // warps per block; each warp takes strips from the launch's queue
// Resident blocks per SM the register allocation must allow: 5 blocks (20
// warps) at 96 registers hide the FP64 unit's latency better than 4 at ~120.
#define FAST_MIN_BLOCKS 5
constexpr unsigned FULL = 0xffffffffu;


// Comparisons on the integer pipe (GB300 issues FP64 compares on its narrow
// FP64 unit). For finite values they agree with the IEEE comparisons except
// that -0 orders below +0; on the fast path that can only change the sign of
// a zero, which cannot reach a nonzero sum (see above), and non-finite inputs
// are recomputed literally.
__device__ __forceinline__ long long key(double x) {  // order-preserving integer image
  const long long b = dbits(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool nz(double x) { return (dbits(x) & 0x7fffffffffffffffLL) != 0; }
__device__ __forceinline__ bool gt0(double x) { return dbits(x) > 0; }
__device__ __forceinline__ bool lt0(double x) { return key(x) < -1; }
__device__ __forceinline__ double mn(double a, double b) { return key(a) < key(b) ? a : b; }  // sw.h MIN
__device__ __forceinline__ double mx(double a, double b) { return key(a) > key(b) ? a : b; }  // sw.h MAX

// The limiters of calc.c:54-63 with the comparisons above.
template <int SCH>
__device__ __forceinline__ double limiter_fast(double r) {
  if constexpr (SCH == 0) return mx(0.0, mn(mn(HALF(1 + r), TWICE(r)), 2.0));
  else if constexpr (SCH == 1) return mx(mx(0.0, mn(TWICE(r), 1.0)), mx(0.0, mn(r, 2.0)));
  else if constexpr (SCH == 2) return mn(r, 1.0);
  else if constexpr (SCH == 4) { const double r2 = TWICE(r); return mx(0.0, mn(r2, mn((1 + r2) / 3.0, 2.0))); }
  else if constexpr (SCH == 7) return mx(0.0, mn(mn(2.0, TWICE(r)), mn(0.25 + 0.75 * r, 0.75 + QUARTER(r))));
  else if constexpr (SCH == kVanLeerSafe)
    return (dbits(r) == dbits(-1.0)) ? 0.0 : (r + fabs(r)) / (1.0 + r);
  else return limiter<SCH>(r);
}


// n/d for d nonzero, with a zero n answered on the integer pipe: the IEEE
// quotient of +-0 by d is the zero whose sign is sign(n) xor sign(d).
__device__ __forceinline__ double div_nz(double n, double d) {
  const long long nb = dbits(n);
  if ((nb & 0x7fffffffffffffffLL) == 0)
    return __longlong_as_double((nb ^ dbits(d)) & (long long)0x8000000000000000ULL);
  return n / d;
}

template <int SCH>
__device__ __forceinline__ double half_psi(double n, double d) {
  const double r = nz(d) ? div_nz(n, d) : 0.0;  // r2rP / r2rM (calc.c:42-43)
  return HALF(limiter_fast<SCH>(r));
}

// c*B of one side: B2BP (pos) = q0 + psi*0.5*(1-c)*(q1-q0), or B2BM =
// q1 - psi*0.5*(1+c)*(q1-q0); 1 + c = 1 - (-c) and q1 - X = q1 + (-X) exactly.
// SB: the last sum on the integer pipe (measured faster in the mass body only).
template <bool SB>
__device__ __forceinline__ double side_term(bool pos, double c, double hpsi, double q0, double q1, double d) {
  const double g = 1.0 - (pos ? c : -c);
  const double X = (hpsi * g) * d;
  if constexpr (SB) return c * sadd(pos ? q0 : q1, pos ? X : -X);
  else return c * ((pos ? q0 : q1) + (pos ? X : -X));
}

// Shared part of a face q0|q1 (outer neighbours qm, q2), with the Courant
// numerators pn = 0.5(...+|...|) >= 0 and mn <= 0 before "*Dt/dx".
struct Face {
  double d, q0, q1, pn, mn, hp1, hp2;
  bool pos1, act, both, ok;
};

template <int SCH>
__device__ __forceinline__ Face make_face(double qm, double q0, double q1, double q2, double pn, double mn,
                                          bool cfin) {
  Face F;
  F.d = q1 - q0;
  F.q0 = q0;
  F.q1 = q1;
  F.pn = pn;
  F.mn = mn;
  const bool aP = nz(pn), aM = nz(mn);
  F.pos1 = aP;  // the side computed first: + if in use, else -
  F.act = aP || aM;
  F.both = aP && aM;
  F.hp1 = half_psi<SCH>(aP ? (q0 - qm) : (q2 - q1), F.d);
  F.hp2 = 0.0;
  if (__any_sync(FULL, F.both)) {
    if (F.both) F.hp2 = half_psi<SCH>(q2 - q1, F.d);
  }
  const int E = max(max(dexp(qm), dexp(q0)), max(dexp(q1), dexp(q2)));
  F.ok = cfin && (E < 0x7ff) && (!nz(F.d) || dexp(F.d) + 498 > E);
  return F;
}

// The face's two terms for a cell whose metric divisor is dx (idx = 1.0/dx).
template <bool SB>
__device__ __forceinline__ void face_terms(const Face& F, double Dt, double dx, double idx, double& tP,
                                           double& tM) {
  const double c1 = div_rcp((F.pos1 ? F.pn : F.mn) * Dt, dx, idx);
  const double t1 = F.act ? side_term<SB>(F.pos1, c1, F.hp1, F.q0, F.q1, F.d) : 0.0;
  tP = F.pos1 ? t1 : 0.0;
  tM = F.pos1 ? 0.0 : t1;
  if (__any_sync(FULL, F.both)) {
    if (F.both) tM = side_term<SB>(false, div_rcp(F.mn * Dt, dx, idx), F.hp2, F.q0, F.q1, F.d);
  }
}
#define ROW2(t, it, j) RW(s, t, j), RW(s, it, j)

// calc.c:100 over the four faces: +wP +wM -eP -eM +sP +sM -nP -nM. The term
// of an unused side is a +0 placeholder; leaving it out changes only the sign
// of a zero sum, which the literal path recomputes. Unless a face of the
// warp's cells uses both sides, each face has one term (the side in use) and
// the sum takes three additions; otherwise all eight terms are summed, out of
// line so that the common case does not carry the extra FP64 operations.
__device__ __noinline__ double sum_faces8(double wP, double wM, double eP, double eM, double sP, double sM,
                                          double nP, double nM) {
  double S = wP + wM;
  S = S - eP;
  S = S - eM;
  S = S + sP;
  S = S + sM;
  S = S - nP;
  S = S - nM;
  return S;
}
struct Side {  // a face's terms as seen by one cell, and which side is in use
  double P, M;
  bool pos, both;
};
__device__ __forceinline__ double sum_faces(const Side& w, const Side& e, const Side& so, const Side& n) {
  if (__any_sync(FULL, w.both || e.both || so.both || n.both))
    return sum_faces8(w.P, w.M, e.P, e.M, so.P, so.M, n.P, n.M);
  const double tw = w.pos ? w.P : w.M, te = e.pos ? e.P : e.M;
  const double ts = so.pos ? so.P : so.M, tn = n.pos ? n.P : n.M;
  return ssub(sadd(ssub(tw, te), ts), tn);
}
__device__ __forceinline__ Side east_of(const Side& w, int lane) {
  Side e;
  e.P = __shfl_sync(FULL, w.P, (lane + 1) & 31);
  e.M = __shfl_sync(FULL, w.M, (lane + 1) & 31);
  e.pos = __shfl_sync(FULL, (int)w.pos, (lane + 1) & 31) != 0;
  e.both = __shfl_sync(FULL, (int)w.both, (lane + 1) & 31) != 0;
  return e;
}
template <bool SB = false>
__device__ __forceinline__ Side side_of(const Face& F, double Dt, double dx, double idx) {
  Side t;
  face_terms<SB>(F, Dt, dx, idx, t.P, t.M);
  t.pos = F.pos1;
  t.both = F.both;
  return t;
}

// Upwind halves of one velocity: 0.5(a+|a|) and 0.5(a-|a|) up to the sign of a zero.
__device__ __forceinline__ double up_p(double a) { return gt0(a) ? a : 0.0; }
__device__ __forceinline__ double up_m(double a) { return lt0(a) ? a : 0.0; }
__device__ __forceinline__ bool fin(double a) { return dexp(a) != 0x7ff; }

// Values of the lane's x neighbours at one row: own value v of column i,
// aux = the value of column base-2 (lane 0), base-1 (lane 1) or base+32 (lane 31).
struct XN {
  double m2, m1, p1;
};
__device__ __forceinline__ XN x_neighbours(double v, double aux, int lane) {
  XN n;
  n.m2 = __shfl_sync(FULL, v, (lane + 30) & 31);
  n.m1 = __shfl_sync(FULL, v, (lane + 31) & 31);
  n.p1 = __shfl_sync(FULL, v, (lane + 1) & 31);
  const double a1 = __shfl_sync(FULL, aux, 1);
  if (lane < 2) n.m2 = aux;
  if (lane == 0) n.m1 = a1;
  if (lane == 31) n.p1 = aux;
  return n;
}

// A strip is 31 columns x s.fk rows (chosen per launch, see fast_launch).
// The warps of the grid (the resident warps) take strips from a queue, the
// next strip index being an atomic counter: a warp that finishes early takes
// more, so the SMs finish together. The last warp of the launch to find the
// queue empty sets both counters back to zero for the next launch (every
// other warp has made its last fetch by then). No warp ever waits.
__device__ __forceinline__ int next_strip(unsigned* q, int lane) {
  unsigned v = 0;
  if (lane == 0) v = atomicAdd(q, 1u);
  return (int)__shfl_sync(FULL, v, 0);
}
__device__ __forceinline__ void strips_done(unsigned* q, int lane) {
  if (lane == 0 && atomicAdd(q + 1, 1u) == gridDim.x * (blockDim.x >> 5) - 1) {
    atomicExch(q, 0u);
    atomicExch(q + 1, 0u);
  }
}
#define FAST_SETUP                                                                          \
  const int W = s.W, nx = s.nx, ny = s.ny;                                                  \
  const int lane = threadIdx.x & 31;                                                        \
  const int FK = s.fk;                                                                      \
  const int nsx = (nx + FW - 1) / FW, nstrips = nsx * ((ny + FK - 1) / FK);                  \
  const double Dt = s.Dt;                                                                   \
  for (int strip = next_strip(s.strips, lane); strip < nstrips; strip = next_strip(s.strips, lane)) { \
    const int j0 = (strip / nsx) * FK + 1;                                                  \
    const int jn = min(j0 + FK - 1, ny);                                                    \
    const int base = (strip % nsx) * FW + 1;                                                \
    const int i = base + lane;                                                              \
    const int ic = min(i, nx + 2);                                                          \
    const int ia = (lane == 0) ? base - 2 : (lane == 1) ? base - 1 : min(base + 32, nx + 2); \
    const bool own = (lane < FW) && (i <= nx);
#define FAST_END \
  }                \
  strips_done(s.strips, lane);
// Field values of the fast bodies. PL (plain form): windx, windy and hB are
// +0.0 everywhere, so x - hB = x exactly, and u + windx = u except that -0
// becomes +0, which the fast path cannot tell apart (see (3) above).
#define UF(i, j) (PL ? f.u[IX(W, i, j)] : UW(i, j))
#define VF(i, j) (PL ? f.v[IX(W, i, j)] : VW(i, j))
#define HF(i, j) (PL ? (f.eta[IX(W, i, j)] + s.depth) : HH(i, j))

// BODYH + damping, fast form.
template <int SCH, bool PL, bool UD>
__global__ void __launch_bounds__(32 * FWARPS, FAST_MIN_BLOCKS) k_mass_fast(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  FAST_SETUP
  const int iu = min(i - 1, nx + 2);
  const double damp = 2.0 * Dt * (s.sigma);  // calc.c:112: (2.0*Dt*sigma)*ETA
  // H at this lane's column, rows j-1 .. j+1 (window), and the face south of j0
  double h1 = HF(ic, j0 - 1), h2 = HF(ic, j0), h3 = HF(ic, j0 + 1);
  // UD (no damping: sigma = 0, a band): the product damp*eta is a zero (eta is
  // finite on the fast path), and a nonzero S minus a zero is S
  Side ts;
  bool oks;
  {
    const double b = VF(ic, j0 - 1);
    const Face F = make_face<SCH>(HF(ic, j0 - 2), h1, h2, h3, up_p(b), up_m(b), fin(b));
    ts = side_of<true>(F, Dt, ROW2(R_DYN, R_IDYN, j0));
    oks = F.ok;
  }
  for (int j = j0; j <= jn; j++) {
    const double h4 = HF(ic, j + 2);
    // x face west of column i, row j
    const XN xn = x_neighbours(h2, HF(ia, j), lane);
    const double a = UF(iu, j);
    const Face FX = make_face<SCH>(xn.m2, xn.m1, h2, xn.p1, up_p(a), up_m(a), fin(a));
    const Side tw = side_of<true>(FX, Dt, ROW2(R_DXE, R_IDXE, j));
    const Side te = east_of(tw, lane);
    const bool oke = __shfl_sync(FULL, (int)FX.ok, (lane + 1) & 31) != 0;
    // y face north of row j: shared by this cell and the cell above
    const double b = VF(ic, j);
    const Face FY = make_face<SCH>(h1, h2, h3, h4, up_p(b), up_m(b), fin(b));
    const Side tn = side_of<true>(FY, Dt, ROW2(R_DYN, R_IDYN, j));
    const Side ns = side_of<true>(FY, Dt, ROW2(R_DYN, R_IDYN, j + 1));
    const double S = sum_faces(tw, te, ts, tn);  // calc.c:100 in its order: +w -e +s -n
    const bool slow = !(FX.ok && oke && oks && FY.ok) || !nz(S);
    if (own) {
      double r;
      if (slow) r = mass_cell_ool<SCH>(s, f, i, j);
      else if (UD) r = S;
      else r = S - (s.polar ? 2.0 * Dt * PF(s, P_SH, IX(W, i, j)) : damp) * f.eta[IX(W, i, j)];
      out[IX(W, i, j)] = r;
    }
    ts = ns;
    oks = FY.ok;
    h1 = h2;
    h2 = h3;
    h3 = h4;
  }
  FAST_END
}

// BODYU, fast form.
template <int SCH, bool PL>
__global__ void __launch_bounds__(32 * FWARPS, FAST_MIN_BLOCKS) k_adv_u_fast(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  FAST_SETUP
  const int ic1 = min(i + 1, nx + 2);
  // U at this lane's column, rows j-1 .. j+1, and V at columns i, i+1 of row j-1
  double u1 = UF(ic, j0 - 1), u2 = UF(ic, j0), u3 = UF(ic, j0 + 1);
  double vs0 = VF(ic, j0 - 1), vs1 = VF(ic1, j0 - 1);
  Side ts;
  bool oks;
  {
    const Face F = make_face<SCH>(UF(ic, j0 - 2), u1, u2, u3, HALF(up_p(vs0) + up_p(vs1)),
                                  HALF(up_m(vs0) + up_m(vs1)), fin(vs0) && fin(vs1));
    ts = side_of(F, Dt, ROW2(R_DYV, R_IDYV, j0));
    oks = F.ok;
  }
  double vsh = HALF(vs0 + vs1);  // (vs0 + vs1) / 2., calc.c:198, carried from the row below
  for (int j = j0; j <= jn; j++) {
    const double u4 = UF(ic, j + 2);
    // x face west of column i, row j: velocities u(i-1), u(i)
    const XN xn = x_neighbours(u2, UF(ia, j), lane);
    const Face FX = make_face<SCH>(xn.m2, xn.m1, u2, xn.p1, HALF(up_p(xn.m1) + up_p(u2)),
                                   HALF(up_m(xn.m1) + up_m(u2)), true);
    const Side tw = side_of(FX, Dt, ROW2(R_DXC, R_IDXC, j));
    const Side te = east_of(tw, lane);
    const bool oke = __shfl_sync(FULL, (int)FX.ok, (lane + 1) & 31) != 0;
    // y face north of row j: velocities v(i, j), v(i+1, j)
    const double vn0 = VF(ic, j), vn1 = VF(ic1, j);
    const Face FY = make_face<SCH>(u1, u2, u3, u4, HALF(up_p(vn0) + up_p(vn1)), HALF(up_m(vn0) + up_m(vn1)),
                                   fin(vn0) && fin(vn1));
    const Side tn = side_of(FY, Dt, ROW2(R_DYV, R_IDYV, j));
    const Side ns = side_of(FY, Dt, ROW2(R_DYV, R_IDYV, j + 1));
    const double S = sum_faces(tw, te, ts, tn);
    const bool slow = !(FX.ok && oke && oks && FY.ok) || !nz(S);
    const double vnh = HALF(vn0 + vn1);
    if (own) {
      double r;
      if (slow) {
        r = advu_cell_ool<SCH>(s, f, i, j);
      } else {
        const double uwm = xn.m1, u0 = u2, uep = xn.p1;  // calc.c:198
        const double p2 = Dt * (div_rcp(u0 * (uep - uwm), ROW2(R_DXE2, R_IDXE2, j)) +
                                div_rcp(u0 * (vnh - vsh), ROW2(R_DYV, R_IDYV, j)));
        r = S + p2;
      }
      out[IX(W, i, j)] = r;
    }
    ts = ns;
    oks = FY.ok;
    vsh = vnh;
    u1 = u2;
    u2 = u3;
    u3 = u4;
  }
  FAST_END
}

// BODYV, fast form.
template <int SCH, bool PL>
__global__ void __launch_bounds__(32 * FWARPS, FAST_MIN_BLOCKS) k_adv_v_fast(DevState s, F7 f, double* out) {
  SW2G_PDL_ENTRY();
  FAST_SETUP
  const int iu = min(i - 1, nx + 2);
  // V at this lane's column, rows j-1 .. j+1; U at column i-1, row j
  double v1 = VF(ic, j0 - 1), v2 = VF(ic, j0), v3 = VF(ic, j0 + 1);
  double uw0 = UF(iu, j0);
  Side ts;
  bool oks;
  {
    const Face F = make_face<SCH>(VF(ic, j0 - 2), v1, v2, v3, HALF(up_p(v1) + up_p(v2)),
                                  HALF(up_m(v1) + up_m(v2)), true);
    ts = side_of(F, Dt, ROW2(R_DYC, R_IDYC, j0));
    oks = F.ok;
  }
  for (int j = j0; j <= jn; j++) {
    const double v4 = VF(ic, j + 2);
    const double uw1 = UF(iu, j + 1);
    // x face west of column i, row j: velocities u(i-1, j+1), u(i-1, j)
    const XN xn = x_neighbours(v2, VF(ia, j), lane);
    const Face FX = make_face<SCH>(xn.m2, xn.m1, v2, xn.p1, HALF(up_p(uw1) + up_p(uw0)),
                                   HALF(up_m(uw1) + up_m(uw0)), fin(uw1) && fin(uw0));
    const Side tw = side_of(FX, Dt, ROW2(R_DXV, R_IDXV, j));
    const Side te = east_of(tw, lane);
    const bool oke = __shfl_sync(FULL, (int)FX.ok, (lane + 1) & 31) != 0;
    // (u(i-1, j) + u(i-1, j+1))/2 and, from the next lane, (u(i, j) + u(i, j+1))/2 (calc.c:235)
    const double uwh = HALF(uw0 + uw1);
    const double ueh = __shfl_sync(FULL, uwh, (lane + 1) & 31);
    // y face north of row j: velocities v(i, j), v(i, j+1)
    const Face FY = make_face<SCH>(v1, v2, v3, v4, HALF(up_p(v2) + up_p(v3)), HALF(up_m(v2) + up_m(v3)), true);
    const Side tn = side_of(FY, Dt, ROW2(R_DYC, R_IDYC, j));
    const Side ns = side_of(FY, Dt, ROW2(R_DYC, R_IDYC, j + 1));
    const double S = sum_faces(tw, te, ts, tn);
    const bool slow = !(FX.ok && oke && oks && FY.ok) || !nz(S);
    if (own) {
      double r;
      if (slow) {
        r = advv_cell_ool<SCH>(s, f, i, j);
      } else {
        const double vsm = v1, v0 = v2, vnp = v3;  // calc.c:235
        const double p2 = Dt * (div_rcp(v0 * (ueh - uwh), ROW2(R_DXV, R_IDXV, j)) +
                                div_rcp(v0 * (vnp - vsm), ROW2(R_DYNS, R_IDYNS, j)));
        r = S + p2;
      }
      out[IX(W, i, j)] = r;
    }
    ts = ns;
    oks = FY.ok;
    uw0 = uw1;
    v1 = v2;
    v2 = v3;
    v3 = v4;
  }
  FAST_END
}
#undef FAST_SETUP
#undef FAST_END
#undef UF
#undef VF
#undef HF
#undef ROW2

// Self-check of div_rcp: for each divisor b, `samples` numerators a drawn
// from a SplitMix64 stream (random significands over exponents 2^-950..2^60,
// both signs, and numerators whose quotient lies within a few ulps of a
// rounding midpoint), compared bit for bit with the IEEE quotient a/b.
__device__ __forceinline__ unsigned long long splitmix(unsigned long long& x) {
  unsigned long long z = (x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__global__ void k_check_division(const double* div, int n, long long samples, unsigned long long seed,
                                 unsigned long long* bad) {
  const long long total = (long long)n * samples;
  unsigned long long miss = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const double b = div[t / samples];
    const double y = 1.0 / b;
    unsigned long long st = seed ^ (unsigned long long)t * 0xD1B54A32D192ED03ULL;
    const unsigned long long r1 = splitmix(st), r2 = splitmix(st);
    double a;
    if (r2 & 1) {  // random significand and exponent
      const unsigned long long e = 73 + (r2 >> 1) % 1010;  // 2^-950 .. 2^59
      a = __longlong_as_double((long long)((e << 52) | (r1 & 0xFFFFFFFFFFFFFULL) | (r2 & 2 ? 1ULL << 63 : 0)));
    } else {  // a = b * (q + half an ulp of q + small offset): quotient near a midpoint
      const unsigned long long e = 523 + (r2 >> 1) % 500;
      const double q = __longlong_as_double((long long)((e << 52) | (r1 & 0xFFFFFFFFFFFFFULL)));
      const double h = __longlong_as_double((long long)(((e - 53) << 52))) * (double)(((r2 >> 10) & 7) + 1) * 0.5;
      a = __dmul_rn(b, q + h);
    }
    const double want = a / b, got = div_rcp(a, b, y);
    if (dbits(want) != dbits(got)) miss++;
  }
  // every divisor against the numerators +-(2 - k ulp), k = 1..512: with the
  // divisor's significand also within a few ulps of 2 these are the pairs
  // where RN(a*y) strays more than one ulp from a/b and a wrong rounding is
  // not excluded by the case analysis alone
  const long long grid = (long long)n * 1024;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < grid;
       t += (long long)gridDim.x * blockDim.x) {
    const double b = div[t >> 10];
    const double y = 1.0 / b;
    const unsigned long long k = (unsigned long long)(t & 511), neg = (unsigned long long)((t >> 9) & 1);
    const double a = __longlong_as_double((long long)((0x3FFFFFFFFFFFFFFFULL - k) | (neg << 63)));
    const double want = a / b, got = div_rcp(a, b, y);
    if (dbits(want) != dbits(got)) miss++;
  }
  if (miss) atomicAdd(bad, miss);
}

// Self-check of sadd and ssub against the FP64 unit: operand pairs from a
// SplitMix64 stream, in classes that reach every branch of the adder: any two
// normal numbers; exponents within 64 of each other (alignment, carries,
// cancellation); b = -a give or take a few ulps (total and near-total
// cancellation); b a tie (an odd multiple of half an ulp of a); sums near
// the overflow and subnormal limits; zeros, subnormals, inf and NaN.
__device__ __forceinline__ double rnd_double(unsigned long long r, int e, bool neg) {
  return __longlong_as_double((long long)(((unsigned long long)e << 52) | (r & 0xFFFFFFFFFFFFFULL) |
                                          (neg ? 1ULL << 63 : 0ULL)));
}
__global__ void k_check_add(long long samples, unsigned long long seed, unsigned long long* bad) {
  unsigned long long miss = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < samples;
       t += (long long)gridDim.x * blockDim.x) {
    unsigned long long st = seed ^ (unsigned long long)t * 0xD1B54A32D192ED03ULL;
    const unsigned long long r1 = splitmix(st), r2 = splitmix(st), r3 = splitmix(st);
    const int cls = (int)(r3 % 8);
    double a, b;
    if (cls == 0) {
      a = rnd_double(r1, 1 + (int)((r3 >> 8) % 2046), r2 & 1);
      b = rnd_double(r2, 1 + (int)((r3 >> 20) % 2046), r2 & 2);
    } else if (cls <= 2) {
      const int e = 70 + (int)((r3 >> 8) % 1900);
      a = rnd_double(r1, e, r2 & 1);
      b = rnd_double(r2, e - (int)((r3 >> 20) % 64), r2 & 2);
    } else if (cls == 3) {
      a = rnd_double(r1, 3 + (int)((r3 >> 8) % 2040), r2 & 1);
      b = __longlong_as_double((dbits(a) ^ (long long)0x8000000000000000ULL) + (long long)((r2 >> 8) % 9) - 4);
    } else if (cls == 4) {  // |b| = k/2 ulp(a), k odd, with or without a few more low bits
      const int e = 60 + (int)((r3 >> 8) % 1900);
      a = rnd_double(r1, e, r2 & 1);
      const double k = (double)(2 * ((r2 >> 8) % 16) + 1);
      b = k * __longlong_as_double((long long)((unsigned long long)(e - 53) << 52));
      if (r2 & 4) b = __longlong_as_double(dbits(b) + (long long)((r2 >> 20) % 3) - 1);
      if (r2 & 2) b = -b;
    } else if (cls == 5) {  // near the top of the range
      a = rnd_double(r1, 2046 - (int)((r3 >> 8) % 3), r2 & 1);
      b = rnd_double(r2, 2046 - (int)((r3 >> 20) % 60), r2 & 2);
    } else if (cls == 6) {  // near the bottom: subnormal sums and operands
      a = rnd_double(r1, (int)((r3 >> 8) % 4), r2 & 1);
      b = rnd_double(r2, (int)((r3 >> 20) % 60), r2 & 2);
    } else {  // zeros, inf, NaN against anything
      const double sp[6] = {0.0, -0.0, __longlong_as_double(0x7ff0000000000000LL),
                            __longlong_as_double((long long)0xfff0000000000000ULL),
                            __longlong_as_double(0x7ff8000000000000LL), 1.0};
      a = sp[(r3 >> 8) % 6];
      b = (r2 & 1) ? sp[(r3 >> 20) % 6] : rnd_double(r2, 1 + (int)((r3 >> 24) % 2046), r2 & 2);
      if (r2 & 4) {
        const double t = a;
        a = b;
        b = t;
      }
    }
    const double s1 = a + b, s2 = sadd(a, b), d1 = a - b, d2 = ssub(a, b);
    const bool nan1 = (dbits(s1) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
    const bool nan2 = (dbits(d1) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
    if (nan1 ? !((dbits(s2) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) : dbits(s1) != dbits(s2)) miss++;
    if (nan2 ? !((dbits(d2) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) : dbits(d1) != dbits(d2)) miss++;
  }
  if (miss) atomicAdd(bad, miss);
}

// do_AdamsBashforth (calc.c:651-699) via copy_scaf/linop_scaf (sppde_core.c:247-298)
__global__ void k_ab(DevState s, int k, double* ab, const double* dn, const double* dm1, const double* dm2) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  if (k == 0) {
    ab[q] = dn[q];
  } else if (k == 1) {
    ab[q] = (3.0 / 2.0) * dn[q] + -(1.0 / 2.0) * dm1[q];
  } else {
    const double t = -(4.0 / 3.0) * dm1[q] + +(5.0 / 12.0) * dm2[q];
    ab[q] = (23.0 / 12.0) * dn[q] + 1.0 * t;
  }
}

// forall x += dx (core.c:175-177, 203-205)
__global__ void k_add(DevState s, double* x, const double* dx) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  x[q] = x[q] + dx[q];
}

// Writer-side halos. The reference refreshes a Laplacian field's halo with the
// single-rank update (every halo cell copies interior cell (wrap(i), wrap(j)))
// and then fixes the wall rows of the interior columns. Each halo cell's
// final value therefore comes from one interior cell (or is a constant), and
// the thread that computes that interior cell writes it:
//   x-halo columns and corners: the wrap;
//   halo rows of the interior columns, per field (band; a polar cap keeps the
//   wrap, it has no walls):
//     LE (laplacian_eta, laplacian.c:131-146): rows ny+1, ny+2 <- row ny,
//        row 0 <- row 1, row -1 <- row ny-1;
//     ZE (laplacian.c:79): row 0 = 0, the other rows wrap;
//     DI (laplacian.c:73): row ny+1 = the wall difference of u (written by
//        the kernel), the other rows wrap;
//     LU (laplacian.c:94-107): row ny+1 <- row ny, row 0 <- row 1, others wrap;
//     LV: rows ny+1 and 0 = 0, others wrap.
enum HaloKind { HK_WRAP, HK_LE, HK_ZE, HK_DI, HK_LU, HK_LV };
constexpr int NOIMG = -1000000;
template <int K>
__device__ __forceinline__ void put_images(const DevState& s, double* f, int i, int j, double v) {
  const int W = s.W, nx = s.nx, ny = s.ny;
  f[IX(W, i, j)] = v;
  if (i > 2 && i < nx - 1 && j > 2 && j < ny - 1) return;
  const int xa = (i <= 2) ? i + nx : NOIMG, xb = (i >= nx - 1) ? i - nx : NOIMG;
  const int ya = (j <= 2) ? j + ny : NOIMG, yb = (j >= ny - 1) ? j - ny : NOIMG;
  if (xa != NOIMG) f[IX(W, xa, j)] = v;
  if (xb != NOIMG) f[IX(W, xb, j)] = v;
  if (ya != NOIMG) {
    if (xa != NOIMG) f[IX(W, xa, ya)] = v;
    if (xb != NOIMG) f[IX(W, xb, ya)] = v;
  }
  if (yb != NOIMG) {
    if (xa != NOIMG) f[IX(W, xa, yb)] = v;
    if (xb != NOIMG) f[IX(W, xb, yb)] = v;
  }
  if (K == HK_WRAP || s.polar != 0) {
    if (ya != NOIMG) f[IX(W, i, ya)] = v;
    if (yb != NOIMG) f[IX(W, i, yb)] = v;
  } else if (K == HK_LE) {
    if (j == ny) {
      f[IX(W, i, ny + 1)] = v;
      f[IX(W, i, ny + 2)] = v;
    }
    if (j == 1) f[IX(W, i, 0)] = v;
    if (j == ny - 1) f[IX(W, i, -1)] = v;
  } else if (K == HK_ZE) {
    if (j == ny - 1) f[IX(W, i, -1)] = v;
    if (j == 1) {
      f[IX(W, i, 0)] = 0.0;
      f[IX(W, i, ny + 1)] = v;
    }
    if (j == 2) f[IX(W, i, ny + 2)] = v;
  } else if (K == HK_DI) {
    if (j == ny - 1) f[IX(W, i, -1)] = v;
    if (j == ny) f[IX(W, i, 0)] = v;
    if (j == 2) f[IX(W, i, ny + 2)] = v;
  } else if (K == HK_LU) {
    if (j == ny - 1) f[IX(W, i, -1)] = v;
    if (j == 1) f[IX(W, i, 0)] = v;
    if (j == ny) f[IX(W, i, ny + 1)] = v;
    if (j == 2) f[IX(W, i, ny + 2)] = v;
  } else {  // HK_LV
    if (j == ny - 1) f[IX(W, i, -1)] = v;
    if (j == 1) f[IX(W, i, 0)] = 0.0;
    if (j == ny) f[IX(W, i, ny + 1)] = 0.0;
    if (j == 2) f[IX(W, i, ny + 2)] = v;
  }
}

// laplacian_eta first pass (laplacian.c:120-123)
__global__ void k_lape_pass1(DevState s, const double* e, double* psi, double* xi) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  psi[q] = div_rcp(RW(s, R_KX, j) * (e[IX(W, i + 1, j)] - e[q]), RW(s, R_DXC, j), RW(s, R_IDXC, j));
  xi[q] = div_rcp(RW(s, R_KY, j) * (e[IX(W, i, j + 1)] - e[q]), RW(s, R_DYC, j), RW(s, R_IDYC, j));
}

// laplacian_eta second pass (laplacian.c:125-127)
// (with its halo update and wall rows written from here, laplacian.c:129-146)
__global__ void k_lape_pass2(DevState s, const double* psi, const double* xi, double* eo) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double v =
      RW(s, R_KC, j) * sadd(div_rcp(psi[q] - psi[IX(W, i - 1, j)], RW(s, R_DXE, j), RW(s, R_IDXE, j)),
                        div_rcp(xi[q] - xi[IX(W, i, j - 1)], RW(s, R_DYN, j), RW(s, R_IDYN, j)));
  put_images<HK_LE>(s, eo, i, j, v);
}


// Deta_n += nu*Dt*L (calc.c:346-350); Du/Dv the same (core.c:258-266), with
// nu*Dt formed once on the host by the same multiplication. A term whose nu
// is a zero adds the product nudt*L, a zero when L is finite, and adding a
// zero to a finite nonzero x gives x; only a zero x (the sign of the sum) or a
// non-finite operand needs that term's arithmetic.
__device__ __forceinline__ bool zero_term_is_exact(double x, double L) {
  const long long xb = dbits(x) & 0x7fffffffffffffffLL;
  return xb != 0 && xb < 0x7ff0000000000000LL && dexp(L) != 0x7ff;
}
// Out of line, so that the rare case is a branch and not predicated FP64 work.
__device__ __noinline__ double add_product(double x, double nd, double v) { return x + nd * v; }

// NZ: bit t set when the order-t coefficient is nonzero (chosen at compile
// time: a skipped FP64 operation under a predicate still occupies the FP64 unit).
// NZ = 8: no hyperviscosity block at all (every nu zero: the reference skips it).
constexpr int kNoHyper = 8;
template <int NZ>
__device__ __forceinline__ double hyper_terms(const DevState& s, double x, const double* l2, const double* l4,
                                              const double* l6, int q) {
  if constexpr (NZ == kNoHyper) {
    return x;
  } else {
    const double V[3] = {l2[q], l4[q], l6[q]};  // all loads issued before any branch
    const double nd[3] = {s.nu2dt, s.nu4dt, s.nu6dt};
#pragma unroll
    for (int t = 0; t < 3; t++) {
      const double v = V[t];
      if ((NZ >> t) & 1) x = sadd(x, nd[t] * v);
      else if (!zero_term_is_exact(x, v)) x = add_product(x, nd[t], v);
    }
    return x;
  }
}

template <int NZ>
__global__ void k_hyper_add(DevState s, double* d, const double* l2, const double* l4, const double* l6) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  d[q] = hyper_terms<NZ>(s, d[q], l2, l4, l6, q);
}

// The coefficient mask of the hyperviscosity terms (kNoHyper when every nu is zero).
int hyper_mask(const DevState& s) {
  if (s.nu2 == 0 && s.nu4 == 0 && s.nu6 == 0) return kNoHyper;
  return (s.nu2dt != 0.0 ? 1 : 0) | (s.nu4dt != 0.0 ? 2 : 0) | (s.nu6dt != 0.0 ? 4 : 0);
}

void hyper_add(const DevState& s, dim3 g, cudaStream_t st, double* d, const double* l2, const double* l4,
               const double* l6) {
  const int m = (s.nu2dt != 0.0 ? 1 : 0) | (s.nu4dt != 0.0 ? 2 : 0) | (s.nu6dt != 0.0 ? 4 : 0);
  switch (m) {
    case 0: pdl_launch(k_hyper_add<0>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    case 1: pdl_launch(k_hyper_add<1>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    case 2: pdl_launch(k_hyper_add<2>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    case 3: pdl_launch(k_hyper_add<3>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    case 4: pdl_launch(k_hyper_add<4>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    case 5: pdl_launch(k_hyper_add<5>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    case 6: pdl_launch(k_hyper_add<6>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
    default: pdl_launch(k_hyper_add<7>, dim3(g), dim3(TX), st, s, d, l2, l4, l6); break;
  }
}

// do_eta_geofactor (calc.c:403-422)
__global__ void k_geofactor(DevState s, F7 f, double* ab) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  ab[q] -= (RW(s, R_GEO, j) * HH(i, j) * 0.5 * (VW(i, j) + VW(i, j - 1)));
}

// solve_pres_u/v + new_vels + dissipation_effect (core.c:217-231; calc.c:500-540, 357-400)
// x - (U*0)*Dt with U finite is x - (+-0): x itself unless x is a zero.
__device__ __noinline__ double minus_damping(double x, double U, double sigma, double Dt) { return x - U * sigma * Dt; }

// UD (a band with sigma = 0): the dissipation terms are zeros, subtracted
// only where the sum is zero or an operand is not finite.
template <bool UD>
__global__ void k_pres_sum(DevState s, F7 f, const double* duadv, const double* dvadv, double* dun, double* dvn) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double* e = f.eta;
  const double mge = s.polar ? -PF(s, P_GE, q) * s.Dt : RW(s, R_MGEDT, j);  // -GE*Dt, calc.c:517
  const double mgn = s.polar ? -PF(s, P_GN, q) * s.Dt : RW(s, R_MGNDT, j);
  const double dup = div_rcp(mge * (e[IX(W, i + 1, j)] - e[q]), RW(s, R_DXC, j), RW(s, R_IDXC, j));
  const double dvp = div_rcp(mgn * (e[IX(W, i, j + 1)] - e[q]), RW(s, R_DYC, j + 1), RW(s, R_IDYC, j + 1));
  double a = sadd(duadv[q], dup);
  double b = sadd(dvadv[q], dvp);
  if constexpr (UD) {
    const double U = f.u[q], V = f.v[q];
    if (!zero_term_is_exact(a, U)) a = minus_damping(a, U, s.sigma, s.Dt);
    if (!zero_term_is_exact(b, V)) b = minus_damping(b, V, s.sigma, s.Dt);
  } else {
    const double su = s.polar ? PF(s, P_SU, q) : s.sigma, sv = s.polar ? PF(s, P_SV, q) : s.sigma;  // calc.c:374-394
    a = ssub(a, f.u[q] * su * s.Dt);
    b = ssub(b, f.v[q] * sv * s.Dt);
  }
  dun[q] = a;
  dvn[q] = b;
}

// laplacian_vels first pass (laplacian.c:59-65)
// (with the halo update and wall fixes of ze and di written from here,
// laplacian.c:67-81). A thread marches down LV_ROWS rows of its column, so
// the products DXC(j+1)*u(i,j+1) and DXV(j)*v(i,j) of one row are the
// DXC(j)*u(i,j) and DXV(j-1)*v(i,j-1) of the next: the same operands and the
// same products, formed once. Four rows (measured against 2, 8 and 16 at
// 2048x1024) keep enough threads in flight for the integer-pipe additions.
constexpr int LV_ROWS = 4;
__global__ void k_lapv_pass1(DevState s, const double* uu, const double* vv, double* ze, double* di) {
  SW2G_PDL_ENTRY();
  const int W = s.W;
  const int i = blockIdx.x * TX + threadIdx.x + 1;
  const int j0 = blockIdx.y * LV_ROWS + 1;
  if (i > s.nx) return;
  const int j1 = min(j0 + LV_ROWS - 1, s.ny);
  double pu = RW(s, R_DXC, j0) * uu[IX(W, i, j0)];
  double qv = RW(s, R_DXV, j0 - 1) * vv[IX(W, i, j0 - 1)];
  for (int j = j0; j <= j1; j++) {
    const int q = IX(W, i, j);
    const double pu1 = RW(s, R_DXC, j + 1) * uu[IX(W, i, j + 1)];
    const double qv1 = RW(s, R_DXV, j) * vv[q];
    double a = RW(s, R_IDXV, j), b = -RW(s, R_IDYC, j + 1);
    const double z = a * sadd((vv[IX(W, i + 1, j)] - vv[q]), b * (pu1 - pu));
    a = RW(s, R_IDXE, j);
    b = RW(s, R_IDYN, j);
    const double d = a * sadd((uu[q] - uu[IX(W, i - 1, j)]), b * (qv1 - qv));
    put_images<HK_ZE>(s, ze, i, j, z);
    put_images<HK_DI>(s, di, i, j, d);
    if (j == s.ny && s.polar == 0)  // laplacian.c:73
      di[IX(W, i, s.ny + 1)] = (uu[IX(W, i, s.ny)] - uu[IX(W, i - 1, s.ny)]) / RW(s, R_DXE, s.ny);
    pu = pu1;
    qv = qv1;
  }
}

// laplacian_vels second pass (laplacian.c:83-89)
// (with the halo update and wall fixes of lu and lv written from here, laplacian.c:91-107)
__global__ void k_lapv_pass2(DevState s, const double* ze, const double* di, double* lu, double* lv) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  double a = -RW(s, R_IDYN, j), b = RW(s, R_IDXC, j);
  const double vu = sadd(a * ssub(ze[q], ze[IX(W, i, j - 1)]), b * ssub(di[IX(W, i + 1, j)], di[q]));
  a = RW(s, R_IDXV, j);
  b = RW(s, R_IDYC, j + 1);
  const double vl = sadd(a * ssub(ze[q], ze[IX(W, i - 1, j)]), b * ssub(di[IX(W, i, j + 1)], di[q]));
  put_images<HK_LU>(s, lu, i, j, vu);
  put_images<HK_LV>(s, lv, i, j, vl);
}


// solve_Coriolis_u (calc.c:542-569), in place
__global__ void k_coriolis_u(DevState s, double* u, const double* v, const double* duab) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double semi = 0.25 * (v[IX(W, i, j)] + v[IX(W, i + 1, j)] + v[IX(W, i, j - 1)] + v[IX(W, i + 1, j - 1)]);
  const double dtf = s.polar ? s.Dt * PF(s, P_FE, q) : RW(s, R_DTFE, j);  // Dt*FE, calc.c:563
  const double al = sadd(dtf, div_rcp(s.Dt * u[q] * RW(s, R_SINC, j), RW(s, R_RZC, j), RW(s, R_IRZC, j)));
  const double be = 0.25 * al * al;
  u[q] = (u[q] + duab[q] - be * u[q] + al * semi) / (1.0 + be);
}

// solve_Coriolis_v (calc.c:571-598), in place, reading the new u interior
__global__ void k_coriolis_v(DevState s, const double* u, double* v, const double* dvab) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double semi = 0.25 * (u[IX(W, i - 1, j + 1)] + u[IX(W, i, j + 1)] + u[IX(W, i, j)] + u[IX(W, i - 1, j)]);
  const double dtf = s.polar ? s.Dt * PF(s, P_FN, q) : RW(s, R_DTFN, j);  // Dt*FN, calc.c:592
  const double al = sadd(dtf, div_rcp(s.Dt * semi * RW(s, R_SINN, j), RW(s, R_RZN, j), RW(s, R_IRZN, j)));
  const double be = 0.25 * al * al;
  v[q] = (v[q] + dvab[q] - be * v[q] - al * semi) / (1.0 + be);
}

// check_stats_scaf (sppde_core.c:346-395) as the reference evaluates it: min and
// max start from the first interior value and skip NaNs after it, so the step
// aborts iff the first value is not finite or some value lies outside +-1e10.
// Tested on the bits (|x| > 1e10 and not NaN), for up to four fields at once.
__device__ __forceinline__ bool range_bad(double x, bool first) {
  const long long m = dbits(x) & 0x7fffffffffffffffLL;
  if (first) return m > 0x4202a05f20000000LL;  // beyond 1e10, inf or NaN
  return m > 0x4202a05f20000000LL && m <= 0x7ff0000000000000LL;
}
// From the third step on (AB3), the tail of each tendency is fused into one
// kernel per field, with the operations of the separate kernels in their
// order: the hyperviscosity terms (into the stored tendency), the
// Adams-Bashforth combination (calc.c:651-699, linop_scaf's two passes) and
//   eta: the geofactor (calc.c:403-422) and eta += D (core.c:203-205);
//   u, v: the Coriolis update (calc.c:542-598).
__device__ __forceinline__ double ab3(double dn, double dm1, double dm2) {
  const double t = sadd(-(4.0 / 3.0) * dm1, +(5.0 / 12.0) * dm2);
  return sadd((23.0 / 12.0) * dn, t);  // 1.0 * t is t
}
// v + (+0): v, except that -0 becomes +0 (the plain form's zero winds).
__device__ __forceinline__ double plus_pos_zero(double v) {
  return (dbits(v) == (long long)0x8000000000000000ULL) ? 0.0 : v;
}

// With `bad` given (a whole step, no forcing between its halves), the range
// check of the new value (core.c:309-312) is done here as well.
__device__ __forceinline__ void check_range(int* bad, double x, int i, int j) {
  if (bad && range_bad(x, i == 1 && j == 1)) atomicOr(bad, 1);
}

template <int NZ, bool PL>
__global__ void k_eta_ab3(DevState s, F7 f, double* eta, double* dn, const double* dm1, const double* dm2,
                          const double* l2, const double* l4, const double* l6, int* bad) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double x = hyper_terms<NZ>(s, dn[q], l2, l4, l6, q);
  if constexpr (NZ != kNoHyper) dn[q] = x;
  double ab = ab3(x, dm1[q], dm2[q]);
  const double e = f.eta[q];
  if constexpr (PL) {
    const double h = e + s.depth;  // - hB with hB = +0 is exact
    ab -= (HALF(RW(s, R_GEO, j) * h) * (plus_pos_zero(f.v[q]) + plus_pos_zero(f.v[IX(W, i, j - 1)])));
  } else {
    ab -= (HALF(RW(s, R_GEO, j) * HH(i, j)) * (VW(i, j) + VW(i, j - 1)));
  }
  const double en = e + ab;
  put_images<HK_WRAP>(s, eta, i, j, en);  // with eta's halo update (core.c:206-210)
  check_range(bad, en, i, j);
}

template <int NZ>
__global__ void k_coriolis_u_ab3(DevState s, double* u, const double* v, double* dn, const double* dm1,
                                 const double* dm2, const double* l2, const double* l4, const double* l6,
                                 int* bad) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double x = hyper_terms<NZ>(s, dn[q], l2, l4, l6, q);
  if constexpr (NZ != kNoHyper) dn[q] = x;
  const double duab = ab3(x, dm1[q], dm2[q]);
  const double semi =
      QUARTER(sadd(sadd(sadd(v[IX(W, i, j)], v[IX(W, i + 1, j)]), v[IX(W, i, j - 1)]), v[IX(W, i + 1, j - 1)]));
  const double dtf = s.polar ? s.Dt * PF(s, P_FE, q) : RW(s, R_DTFE, j);
  const double al = sadd(dtf, div_rcp(s.Dt * u[q] * RW(s, R_SINC, j), RW(s, R_RZC, j), RW(s, R_IRZC, j)));
  const double be = QUARTER(al) * al;
  const double un = sadd(ssub(sadd(u[q], duab), be * u[q]), al * semi) / sadd(1.0, be);
  u[q] = un;
  check_range(bad, un, i, j);
}

template <int NZ>
__global__ void k_coriolis_v_ab3(DevState s, const double* u, double* v, double* dn, const double* dm1,
                                 const double* dm2, const double* l2, const double* l4, const double* l6,
                                 int* bad) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const double x = hyper_terms<NZ>(s, dn[q], l2, l4, l6, q);
  if constexpr (NZ != kNoHyper) dn[q] = x;
  const double dvab = ab3(x, dm1[q], dm2[q]);
  const double semi =
      QUARTER(sadd(sadd(sadd(u[IX(W, i - 1, j + 1)], u[IX(W, i, j + 1)]), u[IX(W, i, j)]), u[IX(W, i - 1, j)]));
  const double dtf = s.polar ? s.Dt * PF(s, P_FN, q) : RW(s, R_DTFN, j);
  const double al = sadd(dtf, div_rcp(s.Dt * semi * RW(s, R_SINN, j), RW(s, R_RZN, j), RW(s, R_IRZN, j)));
  const double be = QUARTER(al) * al;
  const double vn = ssub(ssub(sadd(v[q], dvab), be * v[q]), al * semi) / sadd(1.0, be);
  v[q] = vn;
  // a band's row ny is a wall: do_channel zeroes it before the range check
  // (core.c:303-312), so the check sees +0 there
  if (s.polar != 0 || j != s.ny) check_range(bad, vn, i, j);
}

template <int NZ>
void fused_tails(const DevState& s, dim3 g, cudaStream_t st, const F7& f, Fp64Buffers& b, int which, int* bad) {
  if (which == 0) {
    if (s.plain)
      pdl_launch(k_eta_ab3<NZ, true>, dim3(g), dim3(TX), st, s, f, b.f[0], b.deta[0], b.deta[1], b.deta[2], b.Le[0], b.Le[1], b.Le[2],
                                            bad);
    else
      pdl_launch(k_eta_ab3<NZ, false>, dim3(g), dim3(TX), st, s, f, b.f[0], b.deta[0], b.deta[1], b.deta[2], b.Le[0], b.Le[1],
                                             b.Le[2], bad);
  } else if (which == 1) {
    pdl_launch(k_coriolis_u_ab3<NZ>, dim3(g), dim3(TX), st, s, b.f[1], b.f[2], b.du[0], b.du[1], b.du[2], b.L[0], b.L[2], b.L[4],
                                           bad);
  } else {
    pdl_launch(k_coriolis_v_ab3<NZ>, dim3(g), dim3(TX), st, s, b.f[1], b.f[2], b.dv[0], b.dv[1], b.dv[2], b.L[1], b.L[3], b.L[5],
                                           bad);
  }
}
// which: 0 eta (hyper + AB3 + geofactor + update), 1 u, 2 v (hyper + AB3 + Coriolis);
// bad: the step's range flag when the range check is done here, else null
void fused_tail(const DevState& s, dim3 g, cudaStream_t st, const F7& f, Fp64Buffers& b, int which, int* bad) {
  switch (hyper_mask(s)) {
    case 0: fused_tails<0>(s, g, st, f, b, which, bad); break;
    case 1: fused_tails<1>(s, g, st, f, b, which, bad); break;
    case 2: fused_tails<2>(s, g, st, f, b, which, bad); break;
    case 3: fused_tails<3>(s, g, st, f, b, which, bad); break;
    case 4: fused_tails<4>(s, g, st, f, b, which, bad); break;
    case 5: fused_tails<5>(s, g, st, f, b, which, bad); break;
    case 6: fused_tails<6>(s, g, st, f, b, which, bad); break;
    case 7: fused_tails<7>(s, g, st, f, b, which, bad); break;
    default: fused_tails<kNoHyper>(s, g, st, f, b, which, bad); break;
  }
}

// Single-rank halo update (sppde_hupdate.c:274-342). The y pass then the x pass
// compose to: every halo cell copies the interior cell (wrapx(i), wrapy(j)).
// blockIdx.y selects the field: one launch wraps x and, when given, y.
__global__ void k_halo(double* x, double* y, int nx, int ny) {
  SW2G_PDL_ENTRY();
  const int W = nx + 4;
  const int nh = 4 * W + 4 * ny;  // 4 full halo rows + 4 halo columns over interior rows
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nh) return;
  if (blockIdx.y == 1) x = y;
  int i, j;
  if (t < 4 * W) {
    const int r = t / W;
    i = t - r * W - 1;
    j = (r < 2) ? r - 1 : ny + r - 1;  // rows -1, 0, ny+1, ny+2
  } else {
    const int u = t - 4 * W;
    const int c = u / ny;
    j = u - c * ny + 1;
    i = (c < 2) ? c - 1 : nx + c - 1;  // columns -1, 0, nx+1, nx+2
  }
  const int si = (i < 1) ? i + nx : ((i > nx) ? i - nx : i);
  const int sj = (j < 1) ? j + ny : ((j > ny) ? j - ny : j);
  x[IX(W, i, j)] = x[IX(W, si, sj)];
}

// do_channel (calc.c:600-649), polar 0: interior columns of the wall rows
__global__ void k_channel(int nx, int ny, double* u, double* v, double* wx, double* wy) {
  SW2G_PDL_ENTRY();
  const int W = nx + 4;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i > nx) return;
  v[IX(W, i, 0)] = 0; v[IX(W, i, -1)] = 0;
  wy[IX(W, i, 0)] = 0; wy[IX(W, i, -1)] = 0;
  u[IX(W, i, 0)] = u[IX(W, i, 1)]; u[IX(W, i, -1)] = u[IX(W, i, 0)];
  wx[IX(W, i, 0)] = wx[IX(W, i, 1)]; wx[IX(W, i, -1)] = wx[IX(W, i, 0)];
  v[IX(W, i, ny)] = 0; v[IX(W, i, ny + 1)] = 0; v[IX(W, i, ny + 2)] = 0;
  wy[IX(W, i, ny)] = 0; wy[IX(W, i, ny + 1)] = 0; wy[IX(W, i, ny + 2)] = 0;
  u[IX(W, i, ny + 1)] = u[IX(W, i, ny)]; u[IX(W, i, ny + 2)] = u[IX(W, i, ny + 1)];
  wx[IX(W, i, ny + 1)] = wx[IX(W, i, ny)]; wx[IX(W, i, ny + 2)] = wx[IX(W, i, ny + 1)];
}

// compute_Dt maxima (calc.c:705-712): max |u+wx|/DXE and |v+wy|/DYN over the
// interior; NaNs never win the comparison, as in the reference's loop. A
// correctly rounded division by a positive number is non-decreasing in the
// numerator, so the largest quotient of a row is the quotient of its largest
// magnitude: the magnitudes are compared as integers (NaNs set to 0) and each
// warp divides once.
__device__ __forceinline__ long long mag_bits(double x) {
  const long long m = dbits(x) & 0x7fffffffffffffffLL;
  return (m > 0x7ff0000000000000LL) ? 0 : m;
}
// One block per row: the row's largest magnitudes, then its two quotients and
// two atomics (atomics on the same address from every warp of the grid would
// serialise in L2).
constexpr int CFL_T = 256;
__global__ void __launch_bounds__(CFL_T) k_cfl(DevState s, F7 f, unsigned long long* out) {
  SW2G_PDL_ENTRY();
  __shared__ long long red[2][CFL_T / 32];
  const int W = s.W;
  const int j = blockIdx.x + 1;
  long long bx = 0, by = 0;
  if (s.plain) {  // |u + (+0)| = |u|
#pragma unroll 4
    for (int i = threadIdx.x + 1; i <= s.nx; i += CFL_T) {
      bx = max(bx, mag_bits(f.u[IX(W, i, j)]));
      by = max(by, mag_bits(f.v[IX(W, i, j)]));
    }
  } else {
#pragma unroll 4
    for (int i = threadIdx.x + 1; i <= s.nx; i += CFL_T) {
      bx = max(bx, mag_bits(UW(i, j)));
      by = max(by, mag_bits(VW(i, j)));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    bx = max(bx, __shfl_xor_sync(0xffffffffu, bx, o));
    by = max(by, __shfl_xor_sync(0xffffffffu, by, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = bx;
    red[1][threadIdx.x >> 5] = by;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < CFL_T / 32; w++) {
      bx = max(bx, red[0][w]);
      by = max(by, red[1][w]);
    }
    const double mx = div_rcp(__longlong_as_double(bx), RW(s, R_DXE, j), RW(s, R_IDXE, j));
    const double my = div_rcp(__longlong_as_double(by), RW(s, R_DYN, j), RW(s, R_IDYN, j));
    if (mx > 0) atomicMax(out, (unsigned long long)dbits(mx));
    if (my > 0) atomicMax(out + 1, (unsigned long long)dbits(my));
  }
}

struct RangeFields {
  const double* f[4];
  int n;
};
__global__ void k_range(DevState s, RangeFields r, int* bad) {
  SW2G_PDL_ENTRY();
  INTERIOR_IJ
  const int q = IX(W, i, j);
  const bool first = (i == 1 && j == 1);
  bool b = false;
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (k < r.n) b = b || range_bad(r.f[k][q], first);
  if (b) atomicOr(bad, 1);
}

#undef UW
#undef VW
#undef HH

// Launch of a fast body. Its warps take strips of 31 columns x fk rows from
// a queue (next_strip), and the grid is the blocks resident on the device at
// once (or fewer when there are fewer strips). Measured on the 2048x1024 and
// 4096x2048 workloads with strips dealt in turn (bodies' CUDA-event times for
// 8, 12, 16 and 24 rows): 12 rows is the best or within 0.2 % of it on both,
// 16 loses 10 % at 2048x1024, where its 1.4 rounds of strips leave most warps
// idle in the second. The queue instead of the fixed turns: the same time at
// 2048x1024, 1 % less at 4096x2048. With the queue, 8 rows beat 12 by 0.6 %
// at 2048x1024 (1.9 rounds of 12-row strips, 2.8 of 8-row ones) and lose
// 0.6 % at 4096x2048 (7.5 rounds of 12-row strips): the tallest strip that
// gives every resident warp at least 2.5 strips, down to 4 rows.
int choose_strip_rows(int nx, int ny, long long warps) {
  for (int fk : {12, 8, 6}) {
    const long long strips = (long long)((nx + FW - 1) / FW) * ((ny + fk - 1) / fk);
    if (2 * strips >= 5 * warps) return fk;
  }
  return 4;
}

template <typename K>
void fast_launch(K kernel, cudaStream_t st, const DevState& s0, const F7& f, double* out) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * FWARPS, 0);
  const long long full = (long long)(sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  DevState s = s0;
  s.fk = choose_strip_rows(s.nx, s.ny, full * FWARPS);
  const long long strips = (long long)((s.nx + FW - 1) / FW) * ((s.ny + s.fk - 1) / s.fk);
  const long long need = (strips + FWARPS - 1) / FWARPS;
  pdl_launch(kernel, dim3((int)(need < full ? need : full)), dim3(32 * FWARPS), st, s, f, out);
}

template <int SCH>
void launch_bodies(int which, dim3 g, cudaStream_t st, const DevState& s, const F7& f, double* out) {
  if constexpr (SCH != 3) {
    const bool ud = !s.polar && s.sigma == 0.0;
    if (s.plain && ud) {
      if (which == 0) { fast_launch(k_mass_fast<SCH, true, true>, st, s, f, out); return; }
    }
    if (s.plain) {
      if (which == 0) { fast_launch(k_mass_fast<SCH, true, false>, st, s, f, out); return; }
      if (which == 2) { fast_launch(k_adv_u_fast<SCH, true>, st, s, f, out); return; }
      if (which == 3) { fast_launch(k_adv_v_fast<SCH, true>, st, s, f, out); return; }
    } else {
      if (which == 0) { fast_launch(k_mass_fast<SCH, false, false>, st, s, f, out); return; }
      if (which == 2) { fast_launch(k_adv_u_fast<SCH, false>, st, s, f, out); return; }
      if (which == 3) { fast_launch(k_adv_v_fast<SCH, false>, st, s, f, out); return; }
    }
  }
  if (which == 0) pdl_launch(k_mass<SCH>, dim3(g), dim3(TX), st, s, f, out);
  else if (which == 1) pdl_launch(k_tracer<SCH>, dim3(g), dim3(TX), st, s, f, out);
  else if (which == 2) pdl_launch(k_adv_u<SCH>, dim3(g), dim3(TX), st, s, f, out);
  else pdl_launch(k_adv_v<SCH>, dim3(g), dim3(TX), st, s, f, out);
}

void body(int which, int sch, dim3 g, cudaStream_t st, const DevState& s, const F7& f, double* out) {
  switch (sch) {
    case 0: launch_bodies<0>(which, g, st, s, f, out); break;
    case 1: launch_bodies<1>(which, g, st, s, f, out); break;
    case 2: launch_bodies<2>(which, g, st, s, f, out); break;
    case 3: launch_bodies<3>(which, g, st, s, f, out); break;
    case 4: launch_bodies<4>(which, g, st, s, f, out); break;
    case 5: launch_bodies<5>(which, g, st, s, f, out); break;
    case 6: launch_bodies<6>(which, g, st, s, f, out); break;
    case 7: launch_bodies<7>(which, g, st, s, f, out); break;
    case 8: launch_bodies<8>(which, g, st, s, f, out); break;
    case 9: launch_bodies<9>(which, g, st, s, f, out); break;
    default: launch_bodies<kVanLeerSafe>(which, g, st, s, f, out); break;
  }
}

void rotate3(double** h) {
  double* t = h[2];
  h[2] = h[1];
  h[1] = h[0];
  h[0] = t;
}

}  // namespace

namespace {
// Forcing between steps (perturbs.c): field += scale * delta, or field =
// value where mask, over the interior cells.
__global__ void k_add_scaled(int nx, int ny, double* f, const double* d, double scale) {
  const int W = nx + 4;
  const int n = nx * ny;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = IX(W, t % nx + 1, t / nx + 1);
    f[q] += scale * d[q];
  }
}
__global__ void k_set_where(int nx, int ny, double* f, const double* val, const unsigned char* mask) {
  const int W = nx + 4;
  const int n = nx * ny;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = IX(W, t % nx + 1, t / nx + 1);
    if (mask[q]) f[q] = val[q];
  }
}
__global__ void k_scatter_cells(double* f, const int* __restrict__ cells, const double* __restrict__ values, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    f[cells[t]] = values ? values[t] : 0.0;
}
}  // namespace

void fp64_add_scaled(double* f, const double* d, double scale, int nx, int ny, cudaStream_t st) {
  const int n = nx * ny, blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_add_scaled<<<blocks, 256, 0, st>>>(nx, ny, f, d, scale);
  halo_wrap(f, nx, ny, st);
}

void fp64_set_where(double* f, const double* val, const unsigned char* mask, int nx, int ny, cudaStream_t st) {
  const int n = nx * ny, blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_set_where<<<blocks, 256, 0, st>>>(nx, ny, f, val, mask);
  halo_wrap(f, nx, ny, st);
}

void fp64_scatter_cells(double* f, const int* cells, const double* values, int n, cudaStream_t st) {
  if (n <= 0) return;
  const int blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_scatter_cells<<<blocks, 256, 0, st>>>(f, cells, values, n);
}

void fp64_channel(double* u, double* v, double* wx, double* wy, int nx, int ny, cudaStream_t st) {
  k_channel<<<(nx + 127) / 128, 128, 0, st>>>(nx, ny, u, v, wx, wy);
}

void fp64_range(const DevState& s, const double* const* fields, int n, int* bad, cudaStream_t st) {
  RangeFields r{};
  for (int k = 0; k < n && k < 4; k++) r.f[r.n++] = fields[k];
  const dim3 g((s.nx + TX - 1) / TX, s.ny);
  pdl_launch(k_range, g, dim3(TX), st, s, r, bad);
}

void fp64_check_add(long long samples, unsigned long long seed, unsigned long long* bad, cudaStream_t st) {
  k_check_add<<<152 * 8, 256, 0, st>>>(samples, seed, bad);
}

void fp64_check_division(const double* d_div, int n, long long samples, unsigned long long seed,
                         unsigned long long* bad, cudaStream_t st) {
  k_check_division<<<152 * 8, 256, 0, st>>>(d_div, n, samples, seed, bad);
}

void halo_wrap(double* x, int nx, int ny, cudaStream_t st) {
  const int nh = 4 * (nx + 4) + 4 * ny;
  pdl_launch(k_halo, dim3((nh + 255) / 256), dim3(256), st, x, x, nx, ny);
}
// Two fields in one launch.
void halo_wrap2(double* x, double* y, int nx, int ny, cudaStream_t st) {
  const int nh = 4 * (nx + 4) + 4 * ny;
  pdl_launch(k_halo, dim3(dim3((nh + 255) / 256, 2)), dim3(256), st, x, y, nx, ny);
}

// One reference time step; returns the number of kernels launched.
namespace {

// Launch bookkeeping shared by the two halves of a step: every tagged launch
// is timed while the timers are on, and counted.
#define LAUNCH(tag, ...)                          \
  do {                                            \
    if (tm && tm->on) tm->begin(tag, st);         \
    __VA_ARGS__;                                  \
    if (tm && tm->on) tm->end(st);                \
    nl++;                                         \
  } while (0)

// Head of a step: core.c:134-290, through the velocity halos.
// fused_checks: the range checks of eta, u and v are done by the kernels that
// write their new values (a whole step with a zero tracer, from the third step).
// The advection sweeps of u and v (core.c:212-215) run before the mass
// update: they read only u, v, the winds and the geometry, and write only
// their own tendencies, so the order changes no value, and a caller that
// copies eta in can overlap that copy with them (StepHooks).
int step_head(const DevState& s, Fp64Buffers& b, int sch, int k, bool tracer, StepChecks chk, int slot,
              cudaStream_t st, Timers* tm, bool fused_checks, StepHooks hk) {
  int* const fbad = fused_checks ? chk.bad + slot : nullptr;
  const dim3 g((s.nx + TX - 1) / TX, s.ny);
  int nl = 0;
  auto F = [&]() { return F7{b.f[0], b.f[1], b.f[2], b.f[3], b.f[4], b.f[5], b.f[6]}; };
  const bool hyper = (s.nu2 != 0 || s.nu4 != 0 || s.nu6 != 0);

  // The Laplacians of the mass equation's hyperviscosity (calc.c:325-335,
  // laplacian.c:110-146). The reference zeroes Le, psi and xi before them
  // (calc.c:325-327, laplacian.c:116-118). Here they are zeroed once at
  // allocation: every level that runs rewrites all cells of its Le
  // (interior, halo wrap, wall rows) and the interior of psi and xi, whose
  // halos stay zero; levels that do not run leave their Le zero.
  auto eta_laplacians = [&]() {
    const double* src = s.lape_eta ? b.f[0] : b.f[1];  // the reference passes u, not eta (calc.c:332)
    const int nlap = (s.nu4 != 0 || s.nu6 != 0) ? ((s.nu6 != 0) ? 3 : 2) : 1;
    for (int q = 0; q < nlap; q++) {
      LAUNCH("lape_pass1", pdl_launch(k_lape_pass1, dim3(g), dim3(TX), st, s, q == 0 ? src : b.Le[q - 1], b.psi, b.xi));
      // halo and wall rows of Le are written by the pass (a polar cap has no walls)
      LAUNCH("lape_pass2", pdl_launch(k_lape_pass2, dim3(g), dim3(TX), st, s, b.psi, b.xi, b.Le[q]));
    }
  };
  // Reading u alone, and nothing that the kernels before their place in the
  // reference's order write, they run first when a caller copies the fields
  // in, which then overlaps the copies of v and eta with them (StepHooks);
  // otherwise they keep their place after the mass body.
  const bool laplacians_first = hyper && !s.lape_eta && hk.v_in;
  if (laplacians_first) eta_laplacians();
  if (hk.v_in) cudaStreamWaitEvent(st, hk.v_in, 0);

  // compute_Dt (core.c:155-159): maxima at the start of the step
  LAUNCH("cfl", pdl_launch(k_cfl, dim3(s.ny), dim3(CFL_T), st, s, F(), chk.cfl + 2 * slot));

  // tracer (core.c:161-182); skipped while the tracer is identically +0, which
  // the step then provably leaves unchanged
  if (tracer) {
    LAUNCH("tracer", body(1, sch, g, st, s, F(), b.dtr[0]));
    LAUNCH("ab", pdl_launch(k_ab, dim3(g), dim3(TX), st, s, k, b.dtrAB, b.dtr[0], b.dtr[1], b.dtr[2]));
    rotate3(b.dtr);
    LAUNCH("add", pdl_launch(k_add, dim3(g), dim3(TX), st, s, b.f[3], b.dtrAB));
    LAUNCH("halo", halo_wrap(b.f[3], s.nx, s.ny, st));
  }

  // advection of u and v (core.c:212-215)
  LAUNCH("adv_u", body(2, sch, g, st, s, F(), b.duadv));
  LAUNCH("adv_v", body(3, sch, g, st, s, F(), b.dvadv));

  // mass (core.c:184-210; calc.c:289-355)
  if (hk.eta_in) cudaStreamWaitEvent(st, hk.eta_in, 0);
  LAUNCH("mass", body(0, sch, g, st, s, F(), b.deta[0]));
  if (hyper) {
    if (!laplacians_first) eta_laplacians();
    if (k < 2) LAUNCH("hyper_add", hyper_add(s, g, st, b.deta[0], b.Le[0], b.Le[1], b.Le[2]));
  }
  if (k >= 2) {
    LAUNCH("eta_ab3", fused_tail(s, g, st, F(), b, 0, fbad));  // writes eta's halo images too
    rotate3(b.deta);
  } else {
    LAUNCH("ab", pdl_launch(k_ab, dim3(g), dim3(TX), st, s, k, b.detaAB, b.deta[0], b.deta[1], b.deta[2]));
    LAUNCH("geofactor", pdl_launch(k_geofactor, dim3(g), dim3(TX), st, s, F(), b.detaAB));
    rotate3(b.deta);
    LAUNCH("add", pdl_launch(k_add, dim3(g), dim3(TX), st, s, b.f[0], b.detaAB));
    LAUNCH("halo", halo_wrap(b.f[0], s.nx, s.ny, st));
  }
  if (hk.eta_out) cudaEventRecord(hk.eta_out, st);  // eta is final for this step

  // momentum (core.c:212-280)
  if (s.polar == 0 && s.sigma == 0.0)
    LAUNCH("pres_sum", pdl_launch(k_pres_sum<true>, dim3(g), dim3(TX), st, s, F(), b.duadv, b.dvadv, b.du[0], b.dv[0]));
  else
    LAUNCH("pres_sum", pdl_launch(k_pres_sum<false>, dim3(g), dim3(TX), st, s, F(), b.duadv, b.dvadv, b.du[0], b.dv[0]));
  if (hyper) {
    // As above: each level rewrites every cell of ze, di and its two L fields
    // (interior, halo wraps, wall fixes), and L of levels not run stay zero.
    const int nlap = (s.nu4 != 0 || s.nu6 != 0) ? ((s.nu6 != 0) ? 3 : 2) : 1;
    for (int q = 0; q < nlap; q++) {
      const double* uu = q == 0 ? b.f[1] : b.L[2 * q - 2];
      const double* vv = q == 0 ? b.f[2] : b.L[2 * q - 1];
      // halos and wall fixes of ze, di and of the outputs are written by the passes
      LAUNCH("lapv_pass1", pdl_launch(k_lapv_pass1, dim3(dim3(g.x, (s.ny + LV_ROWS - 1) / LV_ROWS)), dim3(TX), st, s, uu, vv, b.ze, b.di));
      LAUNCH("lapv_pass2", pdl_launch(k_lapv_pass2, dim3(g), dim3(TX), st, s, b.ze, b.di, b.L[2 * q], b.L[2 * q + 1]));
    }
    if (k < 2) {
      LAUNCH("hyper_add", hyper_add(s, g, st, b.du[0], b.L[0], b.L[2], b.L[4]));
      LAUNCH("hyper_add", hyper_add(s, g, st, b.dv[0], b.L[1], b.L[3], b.L[5]));
    }
  }
  if (k >= 2) {
    // AB3 of u and v folded into the Coriolis updates (core.c:271-285); the v
    // tendency does not depend on the new u
    LAUNCH("coriolis_u", fused_tail(s, g, st, F(), b, 1, fbad));
    if (hk.u_out) cudaEventRecord(hk.u_out, st);  // u's interior is final
    LAUNCH("coriolis_v", fused_tail(s, g, st, F(), b, 2, fbad));
    rotate3(b.du);
    rotate3(b.dv);
  } else {
    LAUNCH("ab", pdl_launch(k_ab, dim3(g), dim3(TX), st, s, k, b.duAB, b.du[0], b.du[1], b.du[2]));
    LAUNCH("ab", pdl_launch(k_ab, dim3(g), dim3(TX), st, s, k, b.dvAB, b.dv[0], b.dv[1], b.dv[2]));
    rotate3(b.du);
    rotate3(b.dv);
    // Coriolis (core.c:282-285)
    LAUNCH("coriolis_u", pdl_launch(k_coriolis_u, dim3(g), dim3(TX), st, s, b.f[1], b.f[2], b.duAB));
    if (hk.u_out) cudaEventRecord(hk.u_out, st);
    LAUNCH("coriolis_v", pdl_launch(k_coriolis_v, dim3(g), dim3(TX), st, s, b.f[1], b.f[2], b.dvAB));
  }

  // halos (core.c:287-290)
  LAUNCH("halo", halo_wrap2(b.f[1], b.f[2], s.nx, s.ny, st));
  return nl;
}

// Tail of a step: the reference adds its time-dependent forcing before it
// (core.c:292-294); the halo refresh of tracer and eta that follows the
// forcing (core.c:296-300) is done by the forcing calls themselves, so the
// tail is do_channel and the range checks (core.c:303-312).
int step_tail(const DevState& s, Fp64Buffers& b, bool tracer, StepChecks chk, int slot, cudaStream_t st,
              Timers* tm, bool fused_checks) {
  const dim3 g((s.nx + TX - 1) / TX, s.ny);
  const int gw = (s.nx + 127) / 128;
  int nl = 0;
  if (s.polar == 0) LAUNCH("channel", pdl_launch(k_channel, dim3(gw), dim3(128), st, s.nx, s.ny, b.f[1], b.f[2], b.f[4], b.f[5]));

  // range checks of tracer, eta, u, v (core.c:309-312); an all-zero tracer
  // passes trivially
  RangeFields r{};
  if (tracer) r.f[r.n++] = b.f[3];
  r.f[r.n++] = b.f[0];
  r.f[r.n++] = b.f[1];
  r.f[r.n++] = b.f[2];
  if (!fused_checks) LAUNCH("range", pdl_launch(k_range, dim3(g), dim3(TX), st, s, r, chk.bad + slot));
  return nl;
}
#undef LAUNCH

}  // namespace

int fp64_step(const DevState& s, Fp64Buffers& b, int sch, int k, bool tracer, StepChecks chk, int slot,
              cudaStream_t st, Timers* tm, int parts, StepHooks hk) {
  int nl = 0;
  const bool fused_checks = (parts == STEP_FULL) && !tracer && k >= 2;
  if (parts & STEP_HEAD) nl += step_head(s, b, sch, k, tracer, chk, slot, st, tm, fused_checks, hk);
  if (parts & STEP_TAIL) nl += step_tail(s, b, tracer, chk, slot, st, tm, fused_checks);
  return nl;
}

// Compensated sums: each thread accumulates with Neumaier's method, then the
// (sum, error) pairs are combined along a tree with Knuth's TwoSum, so the
// result carries the rounding errors of every addition.
struct Pair {
  double hi, lo;
};
__device__ __forceinline__ Pair two_sum_add(Pair a, Pair b) {
  const double s = a.hi + b.hi;
  const double bb = s - a.hi;
  const double err = (a.hi - (s - bb)) + (b.hi - bb);
  return Pair{s, (a.lo + b.lo) + err};
}
__device__ __forceinline__ void neumaier(double& acc, double& cmp, double term) {
  const double t = acc + term;
  cmp += (fabs(acc) >= fabs(term)) ? ((acc - t) + term) : ((term - t) + acc);
  acc = t;
}
// Block-wide combine of three pairs per thread (blockDim a multiple of 32, <= 1024);
// thread 0 receives the totals.
__device__ __forceinline__ void block_combine3(Pair v[3]) {
  __shared__ double sh[3][2][32];
  for (int o = 16; o > 0; o >>= 1)
    for (int c = 0; c < 3; c++) {
      const Pair w{__shfl_down_sync(0xffffffffu, v[c].hi, o), __shfl_down_sync(0xffffffffu, v[c].lo, o)};
      v[c] = two_sum_add(v[c], w);
    }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (lane == 0)
    for (int c = 0; c < 3; c++) { sh[c][0][warp] = v[c].hi; sh[c][1][warp] = v[c].lo; }
  __syncthreads();
  if (warp == 0) {
    for (int c = 0; c < 3; c++) v[c] = (lane < nw) ? Pair{sh[c][0][lane], sh[c][1][lane]} : Pair{0.0, 0.0};
    for (int o = 16; o > 0; o >>= 1)
      for (int c = 0; c < 3; c++) {
        const Pair w{__shfl_down_sync(0xffffffffu, v[c].hi, o), __shfl_down_sync(0xffffffffu, v[c].lo, o)};
        v[c] = two_sum_add(v[c], w);
      }
  }
}

// Energy per interior row (energy.c:36-41), compensated over i.
__global__ void k_energy_rows(DevState s, F7 f, double* out) {
  const int W = s.W;
  const int j = blockIdx.x + 1;
  double acc[3] = {0, 0, 0}, cmp[3] = {0, 0, 0};
  const double surf = RW(s, R_SURF, j), gcrow = RW(s, R_GC, j), depth = s.depth;
  for (int i = threadIdx.x + 1; i <= s.nx; i += blockDim.x) {
    const double gc = s.polar ? PF(s, P_GC, IX(W, i, j)) : gcrow;
#define UW(i, j) (f.u[IX(W, i, j)] + f.wx[IX(W, i, j)])
#define VW(i, j) (f.v[IX(W, i, j)] + f.wy[IX(W, i, j)])
#define HH(i, j) (f.eta[IX(W, i, j)] + s.depth - f.hb[IX(W, i, j)])
    const double uc = 0.5 * (UW(i, j) + UW(i - 1, j));
    const double vc = 0.5 * (VW(i, j) + VW(i, j - 1));
    const double w0 = f.wx[IX(W, i, j)], w1 = f.wy[IX(W, i, j)];
    const double h = HH(i, j);
    const double term[3] = {0.5 * h * (uc * uc + vc * vc) * surf - 0.5 * ((w0 * w0) + (w1 * w1)) * surf,
                            0.5 * gc * (h * h) * surf - 0.5 * gc * (depth * depth) * surf, h * surf};
#undef UW
#undef VW
#undef HH
    for (int c = 0; c < 3; c++) neumaier(acc[c], cmp[c], term[c]);
  }
  Pair v[3] = {{acc[0], cmp[0]}, {acc[1], cmp[1]}, {acc[2], cmp[2]}};
  block_combine3(v);
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; c++) out[3 * (j - 1) + c] = v[c].hi + v[c].lo;
}

__global__ void k_energy_sum(const double* rows, int ny, double* out) {
  double acc[3] = {0, 0, 0}, cmp[3] = {0, 0, 0};
  for (int j = threadIdx.x; j < ny; j += blockDim.x)
    for (int c = 0; c < 3; c++) neumaier(acc[c], cmp[c], rows[3 * j + c]);
  Pair v[3] = {{acc[0], cmp[0]}, {acc[1], cmp[1]}, {acc[2], cmp[2]}};
  block_combine3(v);
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; c++) out[c] = v[c].hi + v[c].lo;
}

void energy_rows(const DevState& s, const double* const* f, double* row_out, cudaStream_t st) {
  k_energy_rows<<<s.ny, 256, 0, st>>>(s, F7{f[0], f[1], f[2], f[3], f[4], f[5], f[6]}, row_out);
}

void energy_sum(const double* row_in, int ny, double* out3, cudaStream_t st) {
  k_energy_sum<<<1, 1024, 0, st>>>(row_in, ny, out3);
}

}  // namespace sw2g
