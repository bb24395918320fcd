// rvh_batch.cu — instantiations of the persistent batch kernel.
//
// The build compiles this file once per (lanes per strand, math mode) with
// -DRVH_LANES=L -DRVH_EXACT=0|1, so the kernels compile in parallel; compiled
// without them it instantiates all of them.  Lanes 1 is the one-thread-per-
// strand streaming kernel.
#include <type_traits>

#include "rvh_kernels.cuh"
#include "rvh_registry.h"

namespace rvh {

#define RVH_BATCH_INST(LL, E)                                                                  \
    template <>                                                                                \
    const void* batch_kernel_inst<LL, E>() {                                                   \
        using Math = std::conditional_t<E, ExactMath, FastMath>;                               \
        return reinterpret_cast<const void*>(&k_batch<LL, Math>);                              \
    }

#if defined(RVH_LANES)
RVH_BATCH_INST(RVH_LANES, (RVH_EXACT != 0))
#else
RVH_BATCH_INST(1, false) RVH_BATCH_INST(1, true)
RVH_BATCH_INST(4, false) RVH_BATCH_INST(4, true)
RVH_BATCH_INST(8, false) RVH_BATCH_INST(8, true)
RVH_BATCH_INST(16, false) RVH_BATCH_INST(16, true)
RVH_BATCH_INST(32, false) RVH_BATCH_INST(32, true)
#endif

}  // namespace rvh
