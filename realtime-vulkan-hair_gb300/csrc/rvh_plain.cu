// rvh_plain.cu — instantiations of the per-asset phase-A kernels.
//
// The build compiles this file once per (fixed point count, math mode) with
// -DRVH_NFIX=N -DRVH_EXACT=0|1 (N = 0: any point count), so the kernels
// compile in parallel; compiled without them it instantiates all of them.
#include <type_traits>

#include "rvh_kernels.cuh"
#include "rvh_registry.h"

namespace rvh {

namespace {
// Lanes per strand a phase-A kernel exists for: at most 10 points per lane and
// at most two lanes per point.
template <int NFIX, class M>
const void* pick_a(int lanes) {
    constexpr int NMAX = NFIX > 0 ? NFIX : RVH_MAX_POINTS;
    switch (lanes) {
#define RVH_CASE(LL)                                                                         \
    case LL:                                                                                 \
        if constexpr ((NMAX + LL - 1) / LL <= 10 && LL <= 2 * NMAX)                          \
            return reinterpret_cast<const void*>(&k_plain_a<NFIX, LL, M>);                   \
        return nullptr;
        RVH_CASE(1) RVH_CASE(2) RVH_CASE(4) RVH_CASE(8) RVH_CASE(16) RVH_CASE(32)
#undef RVH_CASE
        default: return nullptr;
    }
}
}  // namespace

#define RVH_PLAIN_INST(N, E)                                                                   \
    template <>                                                                                \
    const void* plain_a_inst<N, E>(int lanes) {                                                \
        return pick_a<N, std::conditional_t<E, ExactMath, FastMath>>(lanes);                   \
    }

#if defined(RVH_NFIX)
RVH_PLAIN_INST(RVH_NFIX, (RVH_EXACT != 0))
#else
RVH_PLAIN_INST(0, false) RVH_PLAIN_INST(0, true)
RVH_PLAIN_INST(8, false) RVH_PLAIN_INST(8, true)
RVH_PLAIN_INST(10, false) RVH_PLAIN_INST(10, true)
RVH_PLAIN_INST(16, false) RVH_PLAIN_INST(16, true)
RVH_PLAIN_INST(24, false) RVH_PLAIN_INST(24, true)
RVH_PLAIN_INST(32, false) RVH_PLAIN_INST(32, true)
#endif

}  // namespace rvh
