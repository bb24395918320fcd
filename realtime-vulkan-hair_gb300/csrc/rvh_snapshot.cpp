// rvh_snapshot.cpp — checkpoint / resume of an asset through host memory.
//
// The reference keeps its state only in VkBuffers (src/Strand.cpp:186-191,
// src/Scene.cpp:4-20); here an asset's whole simulation state can be written
// to a flat host buffer and restored into a new asset (another context, another
// GPU, a later process): the header rvh_snapshot_header, then 16-byte aligned
// sections
//   rest lengths            n_strands floats
//   strand wind  (flag 1)   n_strands float4
//   rest roots   (flag 2)   n_strands float4 (the roots a head motion carries)
//   Strand records          48 * n_points bytes per strand
// A pending friction (fused batched steps) is finished first, so a restored
// asset continues with the same bits as the original.
#include <cstring>
#include <new>
#include <vector>

#include "rvh_internal.hpp"

namespace rvh {
namespace {

constexpr char kMagic[8] = {'R', 'V', 'H', 'S', 'N', 'A', 'P', '\0'};
constexpr uint32_t kVersion = 1;

size_t pad16(size_t x) { return (x + 15u) & ~size_t(15); }

struct Layout {
    size_t rest = 0, wind = 0, roots = 0, records = 0, total = 0;
};

Layout layout_of(int n_strands, int n_points, uint32_t flags) {
    Layout L;
    size_t off = pad16(sizeof(rvh_snapshot_header));
    L.rest = off;
    off += pad16(size_t(n_strands) * 4u);
    if (flags & RVH_SNAPSHOT_WIND) {
        L.wind = off;
        off += size_t(n_strands) * 16u;
    }
    if (flags & RVH_SNAPSHOT_ROOTS) {
        L.roots = off;
        off += size_t(n_strands) * 16u;
    }
    L.records = off;
    off += size_t(n_strands) * 48u * size_t(n_points);
    L.total = off;
    return L;
}

uint32_t flags_of(const Asset* a) {
    uint32_t f = 0;
    if (a->has_wind && a->wind.ptr) f |= RVH_SNAPSHOT_WIND;
    if (a->root_rest.ptr) f |= RVH_SNAPSHOT_ROOTS;
    if (a->head_active) f |= RVH_SNAPSHOT_HEAD_ACTIVE;
    return f;
}

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_asset_snapshot_bytes(rvh_asset* a, uint64_t* bytes) {
    if (!a || !bytes) return fail(RVH_ERR_INVALID_ARG, "snapshot_bytes: NULL argument");
    *bytes = layout_of(a->n_strands, a->n_points, flags_of(a)).total;
    return RVH_OK;
}

rvh_status rvh_asset_snapshot(rvh_asset* a, void* host_dst, uint64_t bytes) {
    TraceRange trace("rvh_asset_snapshot");
    if (!a || !host_dst) return fail(RVH_ERR_INVALID_ARG, "snapshot: NULL argument");
    const uint32_t flags = flags_of(a);
    const Layout L = layout_of(a->n_strands, a->n_points, flags);
    if (bytes != L.total) return fail(RVH_ERR_INVALID_ARG, "snapshot: size must be rvh_asset_snapshot_bytes");
    if (a->colliders.size() > RVH_MAX_COLLIDERS) return fail(RVH_ERR_STATE, "snapshot: too many colliders");
    RVH_DEVICE(a->ctx->device);
    rvh_status st = finish_pending(a, a->ctx->stream);
    if (st != RVH_OK) return st;
    RVH_CUDA(cudaStreamSynchronize(a->ctx->stream));
    auto* base = static_cast<unsigned char*>(host_dst);
    std::memset(base, 0, L.records);
    rvh_snapshot_header h{};
    std::memcpy(h.magic, kMagic, sizeof kMagic);
    h.version = kVersion;
    h.header_bytes = uint32_t(sizeof(rvh_snapshot_header));
    h.total_bytes = L.total;
    h.n_strands = a->n_strands;
    h.n_points = a->n_points;
    h.flags = flags;
    h.n_colliders = int32_t(a->colliders.size());
    h.lanes_per_strand = a->lanes;
    h.params = a->params;
    for (size_t i = 0; i < a->colliders.size(); ++i) h.colliders[i] = a->colliders[i];
    std::memcpy(h.head, a->head, sizeof h.head);
    std::memcpy(base, &h, sizeof h);
    const size_t ns = size_t(a->n_strands);
    if (ns) {
        RVH_CUDA(cudaMemcpy(base + L.rest, a->rest.ptr, ns * 4u, cudaMemcpyDeviceToHost));
        if (flags & RVH_SNAPSHOT_WIND) RVH_CUDA(cudaMemcpy(base + L.wind, a->wind.ptr, ns * 16u, cudaMemcpyDeviceToHost));
        if (flags & RVH_SNAPSHOT_ROOTS)
            RVH_CUDA(cudaMemcpy(base + L.roots, a->root_rest.ptr, ns * 16u, cudaMemcpyDeviceToHost));
        RVH_CUDA(cudaMemcpy(base + L.records, a->strands.ptr, a->record_bytes(), cudaMemcpyDeviceToHost));
    }
    return RVH_OK;
}

rvh_status rvh_asset_restore(rvh_context* ctx, const void* host_src, uint64_t bytes, int32_t lanes_per_strand,
                             rvh_asset** out) {
    if (!ctx || !host_src || !out) return fail(RVH_ERR_INVALID_ARG, "restore: NULL argument");
    *out = nullptr;
    if (bytes < sizeof(rvh_snapshot_header)) return fail(RVH_ERR_INVALID_ARG, "restore: buffer shorter than a header");
    rvh_snapshot_header h;
    std::memcpy(&h, host_src, sizeof h);
    if (std::memcmp(h.magic, kMagic, sizeof kMagic) != 0) return fail(RVH_ERR_INVALID_ARG, "restore: not a snapshot");
    if (h.version != kVersion || h.header_bytes != sizeof(rvh_snapshot_header))
        return fail(RVH_ERR_UNSUPPORTED, "restore: unknown snapshot version");
    if (h.n_strands < 0 || h.n_points < RVH_MIN_POINTS || h.n_points > RVH_MAX_POINTS || h.n_colliders < 0 ||
        h.n_colliders > RVH_MAX_COLLIDERS ||
        (h.flags & ~uint32_t(RVH_SNAPSHOT_WIND | RVH_SNAPSHOT_ROOTS | RVH_SNAPSHOT_HEAD_ACTIVE)) != 0 ||
        ((h.flags & RVH_SNAPSHOT_HEAD_ACTIVE) && !(h.flags & RVH_SNAPSHOT_ROOTS)))
        return fail(RVH_ERR_INVALID_ARG, "restore: corrupt header");
    const Layout L = layout_of(h.n_strands, h.n_points, h.flags);
    if (h.total_bytes != L.total || bytes != L.total) return fail(RVH_ERR_INVALID_ARG, "restore: size mismatch");
    const auto* base = static_cast<const unsigned char*>(host_src);
    const size_t ns = size_t(h.n_strands);
    std::vector<float> rest(ns), wind3;
    if (ns) std::memcpy(rest.data(), base + L.rest, ns * 4u);
    if (h.flags & RVH_SNAPSHOT_WIND) {
        wind3.resize(ns * 3);
        for (size_t i = 0; i < ns; ++i) std::memcpy(&wind3[3 * i], base + L.wind + 16 * i, 12);
    }
    rvh_asset_desc d{};
    d.n_strands = h.n_strands;
    d.n_points = h.n_points;
    d.strands = base + L.records;
    d.strands_location = RVH_MEM_HOST;
    d.rest_lengths = ns ? rest.data() : nullptr;
    d.uniform_rest_length = 0.f;
    d.strand_wind = wind3.empty() ? nullptr : wind3.data();
    d.lanes_per_strand = lanes_per_strand ? lanes_per_strand : h.lanes_per_strand;
    rvh_asset* a = nullptr;
    rvh_status st = rvh_asset_create(ctx, &d, &a);
    if (st != RVH_OK) return st;
    auto bail = [&](rvh_status s) {
        rvh_asset_destroy(a);
        return s;
    };
    if ((st = rvh_asset_set_params(a, &h.params)) != RVH_OK) return bail(st);
    if ((st = rvh_asset_set_colliders(a, h.colliders, h.n_colliders)) != RVH_OK) return bail(st);
    if ((h.flags & RVH_SNAPSHOT_ROOTS) && ns) {
        if ((st = ctx->alloc(a->root_rest, ns * 16u)) != RVH_OK) return bail(st);
        cudaError_t e = cudaMemcpy(a->root_rest.ptr, base + L.roots, ns * 16u, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy rest roots"));
    }
    if (h.flags & RVH_SNAPSHOT_HEAD_ACTIVE) {
        std::memcpy(a->head, h.head, sizeof a->head);
        a->head_active = true;
    }
    *out = a;
    return RVH_OK;
}

}  // extern "C"
