// rvh_plain.cu — instantiations of the per-asset phase-A / phase-B kernels.
#include <mutex>
#include <set>

#include "rvh_kernels.cuh"
#include "rvh_registry.h"

namespace rvh {

namespace {
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

template <class M>
const void* pick_n(int n, int lanes) {
    switch (n) {
        case 8: return pick_a<8, M>(lanes);
        case 10: return pick_a<10, M>(lanes);
        case 16: return pick_a<16, M>(lanes);
        case 24: return pick_a<24, M>(lanes);
        case 32: return pick_a<32, M>(lanes);
        default: return (n >= RVH_MIN_POINTS && n <= RVH_MAX_POINTS) ? pick_a<0, M>(lanes) : nullptr;
    }
}
}  // namespace

bool prepare_kernel(const void* fn) {
    static std::mutex mu;
    static std::set<const void*> done;
    std::lock_guard<std::mutex> g(mu);
    if (!fn) return false;
    if (done.count(fn)) return true;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes) != cudaSuccess)
        return false;
    done.insert(fn);
    return true;
}

const void* plain_a_kernel(int n, int lanes, bool exact) {
    return exact ? pick_n<ExactMath>(n, lanes) : pick_n<FastMath>(n, lanes);
}
bool plain_a_supported(int n, int lanes) { return plain_a_kernel(n, lanes, false) != nullptr; }
const void* plain_b_kernel(bool exact) {
    return exact ? reinterpret_cast<const void*>(&k_plain_b<ExactMath>)
                 : reinterpret_cast<const void*>(&k_plain_b<FastMath>);
}

}  // namespace rvh
