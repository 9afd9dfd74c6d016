// FP32 precision form of the SW2 step: host side (tensor maps, member
// descriptors, the launch sequence of a step) and the limiter-independent
// kernels. The kernels themselves are in step_fp32.cuh.
#include <cudaTypedefs.h>

#include <cstring>
#include <vector>

#include "step_fp32.cuh"

namespace sw2g {
namespace f32 {


__global__ void kb_advance(int* counter) { *counter += 1; }

// FP32 shadow of an FP64 field over all padded cells (pitch W -> pitch P).
__global__ void k_shadow(float* dst, const double* src, int nx, int ny, int W, int P) {
  const int n = W * (ny + 4);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int r = t / W, c = t - r * W;
    dst[r * P + c + 2] = d2f(src[t]);
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
  *P = SW * ((nx + SW - 1) / SW) + 8;  // every strip's staged rows lie inside the row
  *R = ny + 4;
}

void fp32_tiles(int nx, int ny, int th, int* nbx, int* nby) {
  *nbx = (nx + SW - 1) / SW;
  *nby = (ny + th - 1) / th;
}

// ---------------------------------------------------------- tensor maps
namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) ==
            cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Rows of BOXW floats of a P x R FP32 array (pitch P floats).
bool encode_rows(CUtensorMap* m, const float* base, int P, int R) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)P, (cuuint64_t)R};
  const cuuint64_t strides[1] = {(cuuint64_t)P * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)BOXW, 1u};
  const cuuint32_t es[2] = {1u, 1u};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

size_t fp32_map_bytes() { return sizeof(CUtensorMap) * TM_NUM; }

bool fp32_write_maps(void* d_maps, const Fp32Ctx& c, const Fp32Engine& e, cudaStream_t st) {
  std::vector<CUtensorMap> m(TM_NUM);
  std::memset(m.data(), 0, sizeof(CUtensorMap) * TM_NUM);
  const float* src[TM_NUM] = {};
  src[TM_ES] = e.es[0]; src[TM_ES + 1] = e.es[1];
  src[TM_US] = e.us[0]; src[TM_US + 1] = e.us[1];
  src[TM_VS] = e.vs[0]; src[TM_VS + 1] = e.vs[1];
  src[TM_LU] = e.Lu; src[TM_LV] = e.Lv;
  src[TM_LLU] = e.LLu; src[TM_LLV] = e.LLv;
  src[TM_TS] = e.ts[0]; src[TM_TS + 1] = e.ts[1];
  src[TM_WX] = c.wx; src[TM_WY] = c.wy; src[TM_HB] = c.hb;
  for (int k = 0; k < TM_NUM; k++)
    if (src[k] && !encode_rows(&m[k], src[k], c.P, c.R)) return false;
  if (cudaMemcpyAsync(d_maps, m.data(), sizeof(CUtensorMap) * TM_NUM, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return false;
  return cudaStreamSynchronize(st) == cudaSuccess;
}

MemberDesc fp32_desc(const Fp32Ctx& c, const Fp32Engine& e, int k) {
  MemberDesc d;
  std::memset(&d, 0, sizeof d);  // padding included, so descriptors compare with memcmp
  d.nx = c.nx; d.ny = c.ny; d.P = c.P;
  d.extra = c.extra;
  d.sig2dt = c.sig2dt; d.sigdt = c.sigdt; d.nu2dt = c.nu2dt; d.nu4dt = c.nu4dt; d.nu6dt = c.nu6dt;
  d.q = c.q;
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
  d.tm = reinterpret_cast<const CUtensorMap*>(e.maps);
  d.cfl = e.cfl; d.bad = e.bad;
  d.cur0 = e.cur;
  d.w0 = e.w;
  d.k0 = k > 2 ? 2 : k;
  d.tile_test = c.tile_test;
  d.open_step = c.open_step;
  d.polar = c.polar;
  d.pf = c.pf;
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

template <int N>
int batch_step_n(int sch, int sr, const MemberDesc* desc, int nmem, const int4* tiles, int ntiles, int nbx, int nby,
                 int* counter, unsigned* queue, cudaStream_t st, Timers* tm) {
  static_assert(sizeof(DescSet<N>) + 64 <= 32760, "launch parameters are limited to 32 KB");
  std::vector<DescSet<N>> hold(1);  // heap: up to ~28 KB
  DescSet<N>& ds = hold[0];
  std::memset(&ds, 0, sizeof ds);
  for (int m = 0; m < nmem; m++) ds.m[m] = desc[m];
  const PhaseArgs<N> a{&ds, tiles, (N == 1) ? nbx * nby : ntiles, nbx, sr, desc[0].ny, counter, queue, st, tm};
  const bool polar = (N == 1) && desc[0].polar != 0;  // polar caps step alone
  bool extra = false, tracer = false, nu6 = false;
  for (int m = 0; m < nmem; m++) {
    extra = extra || desc[m].extra;
    tracer = tracer || (desc[m].trd != nullptr);
    nu6 = nu6 || (desc[m].nu6dt != 0.f);
  }
  int nl = 0;
  if (tracer) {  // reads the step's old u, v and tracer only (core.c:161-182)
    switch (sch) {
      case 0: sch_tracer<0, N>(extra, polar, a, nl); break;
      case 1: sch_tracer<1, N>(extra, polar, a, nl); break;
      case 2: sch_tracer<2, N>(extra, polar, a, nl); break;
      case 4: sch_tracer<4, N>(extra, polar, a, nl); break;
      case 5: sch_tracer<5, N>(extra, polar, a, nl); break;
      case 6: sch_tracer<6, N>(extra, polar, a, nl); break;
      case 7: sch_tracer<7, N>(extra, polar, a, nl); break;
      case 8: sch_tracer<8, N>(extra, polar, a, nl); break;
      case 9: sch_tracer<9, N>(extra, polar, a, nl); break;
      default: sch_tracer<kVanLeerSafe, N>(extra, polar, a, nl); break;
    }
  }
  if constexpr (N == 1) {
    if (polar) run_phase<kb_lap1<1, true>, 1>("f32_lap1", kSmemLap, a, nl);
    else run_phase<kb_lap1<1>, 1>("f32_lap1", kSmemLap, a, nl);
  } else {
    run_phase<kb_lap1<N>, N>("f32_lap1", kSmemLap, a, nl);
  }
  switch (sch) {  // the FP32 form runs Van Leer in its safe form (kVanLeerSafe)
    case 0: sch_main1<0, N>(extra, polar, a, nl); break;
    case 1: sch_main1<1, N>(extra, polar, a, nl); break;
    case 2: sch_main1<2, N>(extra, polar, a, nl); break;
    case 4: sch_main1<4, N>(extra, polar, a, nl); break;
    case 5: sch_main1<5, N>(extra, polar, a, nl); break;
    case 6: sch_main1<6, N>(extra, polar, a, nl); break;
    case 7: sch_main1<7, N>(extra, polar, a, nl); break;
    case 8: sch_main1<8, N>(extra, polar, a, nl); break;
    case 9: sch_main1<9, N>(extra, polar, a, nl); break;
    default: sch_main1<kVanLeerSafe, N>(extra, polar, a, nl); break;
  }
  if constexpr (N == 1) {
    if (nu6 && polar) run_phase<kb_lap3<1, true>, 1>("f32_lap3", kSmemLap, a, nl);
    else if (nu6) run_phase<kb_lap3<1>, 1>("f32_lap3", kSmemLap, a, nl);
    if (polar) run_phase<kb_main2<1, true>, 1>("f32_main2", kSmemMain2, a, nl);
    else run_phase<kb_main2<1>, 1>("f32_main2", kSmemMain2, a, nl);
  } else {
    if (nu6) run_phase<kb_lap3<N>, N>("f32_lap3", kSmemLap, a, nl);
    run_phase<kb_main2<N>, N>("f32_main2", kSmemMain2, a, nl);
  }
  kb_advance<<<1, 1, 0, st>>>(counter);
  nl++;
  return nl;
}

template <int N>
void prepare_n() {
  grid_cap<kb_lap1<N>>(kSmemLap);
  grid_cap<kb_lap3<N>>(kSmemLap);
  grid_cap<kb_main2<N>>(kSmemMain2);
  if constexpr (N == 1) {
    grid_cap<kb_lap1<1, true>>(kSmemLap);
    grid_cap<kb_lap3<1, true>>(kSmemLap);
    grid_cap<kb_main2<1, true>>(kSmemMain2);
  }
}

}  // namespace

void fp32_prepare() {
  prepare_n<1>();
  prepare_n<kMaxBatch>();
  sch_prepare<0>(); sch_prepare<1>(); sch_prepare<2>(); sch_prepare<4>(); sch_prepare<5>();
  sch_prepare<6>(); sch_prepare<7>(); sch_prepare<8>(); sch_prepare<9>(); sch_prepare<kVanLeerSafe>();
}

int fp32_batch_step(int sch, int sr, const MemberDesc* desc, int nmem, const int4* tiles, int ntiles, int nbx,
                    int nby, int* counter, unsigned* queue, cudaStream_t st, Timers* tm) {
  if (nmem == 1) return batch_step_n<1>(sch, sr, desc, nmem, tiles, ntiles, nbx, nby, counter, queue, st, tm);
  return batch_step_n<kMaxBatch>(sch, sr, desc, nmem, tiles, ntiles, nbx, nby, counter, queue, st, tm);
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
