// rvh_registry.cu — lookup of the compiled step kernels by shape; the
// phase-B kernel's instantiations.
#include "rvh_kernels.cuh"
#include "rvh_optin.hpp"
#include "rvh_registry.h"

namespace rvh {

bool prepare_kernel(const void* fn) {
    static OptInRecord record;
    if (!fn) return false;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    return record.ensure(dev, fn, [&] {
        return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes) == cudaSuccess;
    });
}

namespace {
template <bool E>
const void* plain_a_of(int n, int lanes) {
    switch (n) {
        case 8: return plain_a_inst<8, E>(lanes);
        case 10: return plain_a_inst<10, E>(lanes);
        case 16: return plain_a_inst<16, E>(lanes);
        case 24: return plain_a_inst<24, E>(lanes);
        case 32: return plain_a_inst<32, E>(lanes);
        default: return (n >= RVH_MIN_POINTS && n <= RVH_MAX_POINTS) ? plain_a_inst<0, E>(lanes) : nullptr;
    }
}
}  // namespace

const void* plain_a_kernel(int n, int lanes, bool exact) {
    return exact ? plain_a_of<true>(n, lanes) : plain_a_of<false>(n, lanes);
}
bool plain_a_supported(int n, int lanes) { return plain_a_kernel(n, lanes, false) != nullptr; }
const void* plain_b_kernel(bool exact) {
    return exact ? reinterpret_cast<const void*>(&k_plain_b<ExactMath>)
                 : reinterpret_cast<const void*>(&k_plain_b<FastMath>);
}

const void* batch_kernel(int lanes, bool exact) {
    switch (lanes) {
        case 1: return exact ? batch_kernel_inst<1, true>() : batch_kernel_inst<1, false>();
        case 4: return exact ? batch_kernel_inst<4, true>() : batch_kernel_inst<4, false>();
        case 8: return exact ? batch_kernel_inst<8, true>() : batch_kernel_inst<8, false>();
        case 16: return exact ? batch_kernel_inst<16, true>() : batch_kernel_inst<16, false>();
        case 32: return exact ? batch_kernel_inst<32, true>() : batch_kernel_inst<32, false>();
        default: return nullptr;
    }
}
bool batch_supported(int lanes) { return batch_kernel(lanes, false) != nullptr; }

}  // namespace rvh
