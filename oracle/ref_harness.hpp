/*
 * ref_harness.hpp — TEST INFRASTRUCTURE ONLY.
 *
 * Prelude that lets the reference's own GLSL compute shader
 * (src/shaders/compute.comp, read in place by oracle/build_ref.py) compile as
 * C++ against the reference's vendored glm 0.9.9.0, so the shader's own code
 * can run on the CPU and pin the oracle.
 *
 * It supplies what GLSL provides implicitly: gl_GlobalInvocationID,
 * barrier() and the int/uint atomicAdd.  Each invocation runs on its own
 * host thread.  barrier() waits for ALL invocations of the dispatch, which
 * gives the shader the global splat/gather phase split its barriers intend
 * (on a GPU they only order one 32-invocation workgroup).
 */
#pragma once
#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>

#include <atomic>

using namespace glm;

static thread_local uvec3 gl_GlobalInvocationID;
void barrier();
static inline int atomicAdd(int& x, int v) { return std::atomic_ref<int>(x).fetch_add(v); }
static inline uint atomicAdd(uint& x, uint v) { return std::atomic_ref<uint>(x).fetch_add(v); }
#define main shader_main
