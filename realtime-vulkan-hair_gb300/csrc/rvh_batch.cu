// rvh_batch.cu — instantiations of the persistent batch kernel.
#include "rvh_kernels.cuh"
#include "rvh_registry.h"

namespace rvh {

const void* batch_kernel(int lanes, bool exact) {
    switch (lanes) {
#define RVH_CASE(LL)                                                                    \
    case LL:                                                                            \
        return exact ? reinterpret_cast<const void*>(&k_batch<LL, ExactMath>)           \
                     : reinterpret_cast<const void*>(&k_batch<LL, FastMath>);
        RVH_CASE(4) RVH_CASE(8) RVH_CASE(16) RVH_CASE(32)
#undef RVH_CASE
        default: return nullptr;
    }
}
bool batch_supported(int lanes) { return batch_kernel(lanes, false) != nullptr; }

}  // namespace rvh
