// FP32 precision form: the limiter-dependent kernels (mass, momentum and
// tracer sweeps), instantiated for one group of limiters per compilation
// (SW2G_LIMITER_GROUP 0..3), so that the groups compile in parallel.
#include "step_fp32.cuh"

#ifndef SW2G_LIMITER_GROUP
#error "compile with -DSW2G_LIMITER_GROUP=0..3"
#endif

namespace sw2g {
namespace f32 {

template <int SCH, int N>
void sch_main1(bool extra, bool polar, const PhaseArgs<N>& a, int& nl) {
  if constexpr (N == 1) {
    if (polar) {
      run_phase<kb_main1<SCH, true, 1, true>, 1>("f32_main1", smem_main1<true>(), a, nl);
      return;
    }
  }
  if (extra) run_phase<kb_main1<SCH, true, N>, N>("f32_main1", smem_main1<true>(), a, nl);
  else run_phase<kb_main1<SCH, false, N>, N>("f32_main1", smem_main1<false>(), a, nl);
}

template <int SCH, int N>
void sch_tracer(bool extra, bool polar, const PhaseArgs<N>& a, int& nl) {
  if constexpr (N == 1) {
    if (polar) {
      run_phase<kb_tracer<SCH, true, 1, true>, 1>("f32_tracer", smem_tracer<true>(), a, nl);
      return;
    }
  }
  if (extra) run_phase<kb_tracer<SCH, true, N>, N>("f32_tracer", smem_tracer<true>(), a, nl);
  else run_phase<kb_tracer<SCH, false, N>, N>("f32_tracer", smem_tracer<false>(), a, nl);
}

template <int SCH>
void sch_prepare() {
  grid_cap<kb_main1<SCH, false, 1>>(smem_main1<false>());
  grid_cap<kb_main1<SCH, true, 1>>(smem_main1<true>());
  grid_cap<kb_main1<SCH, false, kMaxBatch>>(smem_main1<false>());
  grid_cap<kb_main1<SCH, true, kMaxBatch>>(smem_main1<true>());
  grid_cap<kb_tracer<SCH, false, 1>>(smem_tracer<false>());
  grid_cap<kb_tracer<SCH, true, 1>>(smem_tracer<true>());
  grid_cap<kb_tracer<SCH, false, kMaxBatch>>(smem_tracer<false>());
  grid_cap<kb_tracer<SCH, true, kMaxBatch>>(smem_tracer<true>());
  grid_cap<kb_main1<SCH, true, 1, true>>(smem_main1<true>());
  grid_cap<kb_tracer<SCH, true, 1, true>>(smem_tracer<true>());
}

#define SW2G_LIMITER(S)                                                      \
  template void sch_prepare<S>();                                            \
  template void sch_main1<S, 1>(bool, bool, const PhaseArgs<1>&, int&);      \
  template void sch_main1<S, kMaxBatch>(bool, bool, const PhaseArgs<kMaxBatch>&, int&); \
  template void sch_tracer<S, 1>(bool, bool, const PhaseArgs<1>&, int&);     \
  template void sch_tracer<S, kMaxBatch>(bool, bool, const PhaseArgs<kMaxBatch>&, int&);

#if SW2G_LIMITER_GROUP == 0
SW2G_LIMITER(2)
SW2G_LIMITER(1)
#elif SW2G_LIMITER_GROUP == 1
SW2G_LIMITER(kVanLeerSafe)
SW2G_LIMITER(0)
#elif SW2G_LIMITER_GROUP == 2
SW2G_LIMITER(4)
SW2G_LIMITER(5)
SW2G_LIMITER(6)
#else
SW2G_LIMITER(7)
SW2G_LIMITER(8)
SW2G_LIMITER(9)
#endif
#undef SW2G_LIMITER

}  // namespace f32
}  // namespace sw2g
