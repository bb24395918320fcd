// rvh_registry.h — lookup of the compiled step kernels by shape.
#pragma once

namespace rvh {

// Lanes per strand the plain phase-A kernel is compiled for, given n points
// (strands per warp = 32 / lanes).  Returns false when (n, lanes) has no
// kernel; n values without a fixed-size kernel use the generic one.
bool plain_a_supported(int n, int lanes);
const void* plain_a_kernel(int n, int lanes, bool exact);
const void* plain_b_kernel(bool exact);
// Persistent batch kernel; lanes in {1, 4, 8, 16, 32} (1: one thread per strand).
const void* batch_kernel(int lanes, bool exact);
bool batch_supported(int lanes);
// One translation unit per instantiation (compiled in parallel): the
// persistent batch kernel for (lanes, math) and the phase-A kernels for a
// fixed point count (0: any count) and math, by lanes per strand.
template <int L, bool EXACT>
const void* batch_kernel_inst();
template <int NFIX, bool EXACT>
const void* plain_a_inst(int lanes);
// Opts a kernel into kSmemBytes of dynamic shared memory on the current
// device (once per device and kernel).
bool prepare_kernel(const void* fn);

}  // namespace rvh
