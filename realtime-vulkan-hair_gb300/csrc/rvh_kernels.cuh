// rvh_kernels.cuh — kernel templates of the hair step.
//
//   k_plain_a / k_plain_b : one asset per launch sequence (the drop-in for one
//                           Renderer::Frame() compute submit, src/Renderer.cpp:
//                           2063-2071: clear grid, dispatch).
//   k_batch               : every asset of a batch in ONE persistent launch.
//                           CTAs pull work items (grid clears, phase-A strand
//                           tiles, phase-B point tiles) from a queue in order; a
//                           phase-B tile waits (bounded) on its asset's count of
//                           finished phase-A tiles.  Items are fetched in queue
//                           order and every wait is on items earlier in the
//                           queue, so the launch makes progress whatever the
//                           number of co-resident CTAs.
#pragma once

#include "rvh_device.cuh"

namespace rvh {

constexpr int kThreads = 256;          // CTA size of every step kernel
constexpr int kWarps = kThreads / 32;

enum : int32_t { ITEM_CLEAR = 0, ITEM_A = 1, ITEM_B = 2 };

struct WorkItem {
    int32_t kind;
    int32_t asset;
    int32_t begin;   // strands (A), points (B) or 16-B grid chunks (CLEAR)
    int32_t end;
};

struct BatchDev {
    const DevAsset* assets;
    const WorkItem* items;
    int32_t n_items;
    uint32_t spin_limit;        // bounded wait of a phase-B tile (iterations of ~256 ns)
    unsigned* head;             // next item (reset to 0 before every launch)
    unsigned* done_a;           // per asset: finished phase-A tiles (reset before every launch)
    const unsigned* need_a;     // per asset: phase-A tiles in this launch
    int* error;                 // nonzero: a wait gave up (RVH_ERR_TIMEOUT)
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Strands [begin, end) of one asset, S = 32/L strands per warp per round.
template <int NFIX, int L, class M>
__device__ __forceinline__ void tile_a(const DevAsset& A, int begin, int end) {
    constexpr int S = 32 / L;
    const int warp = threadIdx.x >> 5;
    const int g = (threadIdx.x & 31) / L;
    for (int s0 = begin + warp * S; s0 < end; s0 += kWarps * S) {
        const int strand = s0 + g;
        strand_phase_a<NFIX, L, M>(A, strand, g < S && strand < end);
    }
}

template <int L, class M>
__device__ __forceinline__ void tile_a_any(const DevAsset& A, int begin, int end) {
    switch (A.n_points) {
        case 8: tile_a<8, L, M>(A, begin, end); break;
        case 16: tile_a<16, L, M>(A, begin, end); break;
        case 24: tile_a<24, L, M>(A, begin, end); break;
        case 32: tile_a<32, L, M>(A, begin, end); break;
        default: tile_a<0, L, M>(A, begin, end); break;
    }
}

template <class M>
__device__ __forceinline__ void tile_b(const DevAsset& A, long long begin, long long end) {
    for (long long p = begin + threadIdx.x; p < end; p += kThreads) point_phase_b<M>(A, p);
}

__device__ __forceinline__ void write_draw(const DevAsset& A) {
    if (A.draw) {
        A.draw->vertex_count = (uint32_t)A.n_strands;  // compute.comp:302, one per strand
        A.draw->instance_count = 1u;
        A.draw->first_vertex = 0u;
        A.draw->first_instance = 0u;
    }
}

// ---- plain path -------------------------------------------------------------

template <int NFIX, int L, class M>
__global__ void __launch_bounds__(kThreads) k_plain_a(const __grid_constant__ DevAsset A) {
    constexpr int S = 32 / L;
    const int begin = blockIdx.x * kWarps * S;
    const int end = min(begin + kWarps * S, A.n_strands);
    tile_a<NFIX, L, M>(A, begin, end);
    if (!A.grid_enabled && blockIdx.x == 0 && threadIdx.x == 0) write_draw(A);
}

template <class M>
__global__ void __launch_bounds__(kThreads) k_plain_b(const __grid_constant__ DevAsset A) {
    const long long total = (long long)A.n_strands * A.n_points;
    for (long long p = (long long)blockIdx.x * kThreads + threadIdx.x; p < total;
         p += (long long)gridDim.x * kThreads)
        point_phase_b<M>(A, p);
    if (blockIdx.x == 0 && threadIdx.x == 0) write_draw(A);
}

// ---- batched persistent path -----------------------------------------------

template <int L, class M>
__global__ void __launch_bounds__(kThreads) k_batch(const __grid_constant__ BatchDev B) {
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(B.head, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= B.n_items) break;
        const WorkItem w = B.items[it];
        const DevAsset& A = B.assets[w.asset];
        if (w.kind == ITEM_A) {
            tile_a_any<L, M>(A, w.begin, w.end);
            if (!A.grid_enabled && w.begin == 0 && threadIdx.x == 0) write_draw(A);
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(B.done_a + w.asset, 1u);
            }
        } else if (w.kind == ITEM_B) {
            if (threadIdx.x == 0) {
                const unsigned need = B.need_a[w.asset];
                uint32_t spins = 0;
                while (ld_acquire_gpu(B.done_a + w.asset) < need) {
                    if (++spins > B.spin_limit) {
                        atomicExch(B.error, RVH_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(256);
                }
            }
            __syncthreads();
            tile_b<M>(A, (long long)w.begin * A.n_points, (long long)w.end * A.n_points);
            if (w.begin == 0 && threadIdx.x == 0) write_draw(A);
        } else {
            uint4* g = reinterpret_cast<uint4*>(A.grid_next);
            for (int c = w.begin + threadIdx.x; c < w.end; c += kThreads) g[c] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();  // s_item is rewritten only after every thread has read it
    }
}

}  // namespace rvh
