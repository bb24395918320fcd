// rvh_capi.cpp — context, assets, parameter helpers and the plain per-asset
// step of the C ABI declared in include/rvh.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "rvh_internal.hpp"
#include "rvh_registry.h"

namespace rvh {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }
rvh_status fail(rvh_status s, const std::string& msg) {
    set_error(msg);
    return s;
}
rvh_status cuda_fail(cudaError_t e, const char* what) {
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return RVH_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) return RVH_ERR_NO_DEVICE;
    return RVH_ERR_CUDA;
}

rvh_status Context::alloc(DevBuf& b, size_t bytes) {
    b = DevBuf{};
    if (bytes == 0) return RVH_OK;
    const size_t rounded = (bytes + 255) & ~size_t(255);
    if (!budget.reserve(rounded))
        return fail(RVH_ERR_BUDGET, "HBM budget exceeded: requested " + std::to_string(rounded) + " B, used " +
                                        std::to_string(budget.used()) + " of " + std::to_string(budget.budget()));
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, rounded);
    if (e != cudaSuccess) {
        budget.release(rounded);
        return cuda_fail(e, "cudaMalloc");
    }
    b.ptr = p;
    b.bytes = rounded;
    b.owner = this;
    b.owned = true;
    return RVH_OK;
}

void Context::free(DevBuf& b) {
    if (b.ptr && b.owned) {
        cudaFree(b.ptr);
        budget.release(b.bytes);
    }
    b = DevBuf{};
}

rvh_status validate_params(const rvh_sim_params& p) {
    const float vals[] = {p.gravity[0], p.gravity[1], p.gravity[2], p.damping, p.dftl_damping, p.vmax,
                          p.k_penalty, p.friction, p.repulsion, p.grid_scale, p.grid_origin[0], p.grid_origin[1],
                          p.grid_origin[2], p.grid_h};
    for (float v : vals)
        if (!std::isfinite(v)) return fail(RVH_ERR_INVALID_ARG, "sim params: non-finite value");
    if (!(p.vmax > 0.f)) return fail(RVH_ERR_INVALID_ARG, "sim params: vmax must be > 0");
    if (p.grid_enabled) {
        if (!(p.grid_h > 0.f)) return fail(RVH_ERR_INVALID_ARG, "sim params: grid_h must be > 0");
        if (!(p.grid_scale > 0.f && p.grid_scale <= 1e30f))
            return fail(RVH_ERR_INVALID_ARG, "sim params: grid_scale must be in (0, 1e30]");
        for (int i = 0; i < 3; ++i)
            if (p.grid_dims[i] < 1 || p.grid_dims[i] > 512)
                return fail(RVH_ERR_INVALID_ARG, "sim params: grid_dims must be in [1, 512]");
        const uint64_t cells = uint64_t(p.grid_dims[0]) * p.grid_dims[1] * p.grid_dims[2];
        if (cells > (1ull << 26)) return fail(RVH_ERR_INVALID_ARG, "sim params: grid larger than 2^26 cells");
    }
    return RVH_OK;
}

rvh_status validate_frame(const rvh_frame& f) {
    if (!std::isfinite(f.dt) || !(f.dt > 0.f)) return fail(RVH_ERR_INVALID_ARG, "frame: dt must be finite and > 0");
    if (!std::isfinite(f.t) || !std::isfinite(f.wind[0]) || !std::isfinite(f.wind[1]) || !std::isfinite(f.wind[2]))
        return fail(RVH_ERR_INVALID_ARG, "frame: non-finite time or wind");
    return RVH_OK;
}

DevCollider pack_collider(const rvh_collider& c) {
    DevCollider d{};
    d.kind = c.kind;
    d.radius = c.radius;
    for (int r = 0; r < 3; ++r) d.c[r] = c.transform[12 + r];
    if (c.kind == RVH_COLLIDER_ELLIPSOID) {
        // local = inv * (p, 1) with |local| <= 1 means p = T * (local, 1): |p - centre| <= |M local| <=
        // max column norm of M times sqrt(3) in general; for T = translate * rotate * scale (Scene.h:35)
        // the columns are orthogonal and the largest column norm bounds it.  The margin covers the
        // FP32 inverse and a non-orthogonal M (Frobenius norm bound).
        double fro = 0.0, colmax = 0.0;
        for (int col = 0; col < 3; ++col) {
            double n2 = 0.0;
            for (int r = 0; r < 3; ++r) n2 += double(c.transform[col * 4 + r]) * double(c.transform[col * 4 + r]);
            fro += n2;
            colmax = std::max(colmax, std::sqrt(n2));
        }
        double dots = 0.0;  // orthogonality of the columns
        for (int i = 0; i < 3; ++i)
            for (int j = i + 1; j < 3; ++j) {
                double dd = 0.0;
                for (int r = 0; r < 3; ++r) dd += double(c.transform[i * 4 + r]) * double(c.transform[j * 4 + r]);
                dots = std::max(dots, std::fabs(dd));
            }
        const double bound = (dots <= 1e-5 * fro) ? colmax : std::sqrt(fro);
        d.radius = float(bound * 1.001 + 1e-6);
    }
    for (int col = 0; col < 4; ++col)
        for (int r = 0; r < 3; ++r) {
            d.inv[col * 3 + r] = c.inv[col * 4 + r];
            d.xf[col * 3 + r] = c.transform[col * 4 + r];
            if (col < 3) d.itr[col * 3 + r] = c.inv_trans[col * 4 + r];
        }
    return d;
}

// Fewest lanes per strand with a compiled phase-A kernel, starting from the
// preferred count for n (point counts without a fixed-size kernel use the
// generic one, which needs >= 4 lanes).  Longer strands prefer 8 lanes: the
// 100k-strand x 32-point head's plain step measured 0.41 / 0.28 / 0.30 / 0.37 ms
// with 4 / 8 / 16 / 32 lanes per strand.
int default_lanes(int n) {
    const int pref = n <= 10 ? 1 : n <= 16 ? 2 : 8;
    for (int l = pref; l <= 32; l *= 2)
        if (plain_a_supported(n, l)) return l;
    return pref;
}

int Asset::pick_grid(int avoid1, int avoid2) const {
    int fallback = -1;
    for (int i = 0; i < 3; ++i) {
        if (i == avoid1 || i == avoid2) continue;
        if (!grid_dirty[i]) return i;
        if (fallback < 0) fallback = i;
    }
    return fallback;
}

DevAsset Asset::device_view(const rvh_frame& f, int g, int prev, int next) const {
    DevAsset A{};
    A.strands = static_cast<float4*>(strands.ptr);
    A.rest = static_cast<const float*>(rest.ptr);
    A.strand_wind = has_wind ? static_cast<const float4*>(wind.ptr) : nullptr;
    auto gp = [&](int i) { return i >= 0 ? static_cast<unsigned long long*>(grid[i].ptr) : nullptr; };
    A.grid = gp(g);
    A.grid_next = gp(next);
    A.grid_prev = gp(prev);
    A.dt_prev = dt_prev;
    A.wait_entry = -1;
    A.draw = static_cast<rvh_draw_indirect*>(draw.ptr);
    A.n_strands = n_strands;
    A.n_points = n_points;
    for (int i = 0; i < 3; ++i) A.gravity[i] = params.gravity[i];
    A.damping = params.damping;
    A.dftl = params.dftl_damping;
    A.vmax = params.vmax;
    A.k_penalty = params.k_penalty;
    A.friction = params.friction;
    A.repulsion = params.repulsion;
    A.scale = params.grid_scale;
    A.grid_enabled = params.grid_enabled ? 1 : 0;
    A.wrap32 = params.grid_wrap32 ? 1 : 0;
    for (int i = 0; i < 3; ++i) A.origin[i] = params.grid_origin[i];
    A.h = params.grid_h;
    A.inv_h = 1.0f / params.grid_h;
    A.nx = params.grid_dims[0];
    A.ny = params.grid_dims[1];
    A.nz = params.grid_dims[2];
    A.dt = f.dt;
    A.t = f.t;
    for (int i = 0; i < 3; ++i) A.wind[i] = f.wind[i];
    A.n_colliders = int32_t(colliders.size());
    for (size_t j = 0; j < colliders.size(); ++j) {
        rvh_collider moved;
        if (head_active && colliders[j].attach_to_head && follow_collider(colliders[j], head, &moved))
            A.col[j] = pack_collider(moved);
        else
            A.col[j] = pack_collider(colliders[j]);
    }
    A.root_rest = head_active ? static_cast<const float4*>(root_rest.ptr) : nullptr;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) A.head[r * 4 + c] = head[c * 4 + r];   // row-major 3 x 4 of m
    return A;
}

rvh_status ensure_grid(Asset* a) {
    if (!a->params.grid_enabled || a->server_managed) return RVH_OK;
    const size_t cells = size_t(a->params.grid_dims[0]) * a->params.grid_dims[1] * a->params.grid_dims[2];
    if (cells == a->grid_cells && a->grid[0].ptr) return RVH_OK;
    for (int i = 0; i < 3; ++i) a->ctx->free(a->grid[i]);
    a->grid_cells = cells;
    for (int i = 0; i < 3; ++i) {
        rvh_status s = a->ctx->alloc(a->grid[i], a->grid_bytes());
        if (s != RVH_OK) {
            for (int j = 0; j < 3; ++j) a->ctx->free(a->grid[j]);
            a->grid_cells = 0;
            return s;
        }
        RVH_CUDA(cudaMemset(a->grid[i].ptr, 0, a->grid_bytes()));
        a->grid_dirty[i] = false;
    }
    a->pending = false;
    a->last_grid = -1;
    return RVH_OK;
}

static rvh_status launch_plain_b(Asset* a, const DevAsset& A, cudaStream_t s) {
    const void* kb = plain_b_kernel(a->ctx->math == RVH_MATH_EXACT);
    if (!prepare_kernel(kb)) return fail(RVH_ERR_CUDA, "cannot opt the step kernels into shared memory");
    const long long pts = (long long)a->n_strands * a->n_points;
    long long blocks = (pts + kTileB - 1) / kTileB;
    const long long cap = (long long)a->ctx->sm_count * 2 * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    void* args[] = {const_cast<DevAsset*>(&A)};
    RVH_CUDA(cudaLaunchKernel(kb, dim3(unsigned(blocks)), dim3(kThreads), args, kSmemBytes, s));
    return RVH_OK;
}

rvh_status finish_pending(Asset* a, cudaStream_t s) {
    if (!a->pending) return RVH_OK;
    if (!a->grid[a->pend].ptr) return fail(RVH_ERR_STATE, "finish: the pending grid is gone");
    rvh_frame f{};
    f.dt = a->dt_prev;
    const DevAsset A = a->device_view(f, a->pend);
    rvh_status st = launch_plain_b(a, A, s);
    if (st != RVH_OK) return st;
    a->pending = false;
    a->grid_dirty[a->pend] = true;
    return RVH_OK;
}

rvh_status launch_plain(Asset* a, const rvh_frame& f, cudaStream_t s) {
    if (a->params.grid_enabled && a->grid_grouped())
        return fail(RVH_ERR_STATE, "step: the asset shares its grid with other assets; step the group in one batch");
    if (a->params.grid_enabled && (!a->grid[0].ptr || !a->grid[1].ptr || !a->grid[2].ptr))
        return fail(RVH_ERR_STATE, "step: the asset's grid is held by a request server and no request is active");
    const bool exact = a->ctx->math == RVH_MATH_EXACT;
    const void* ka = plain_a_kernel(a->n_points, a->lanes, exact);
    if (!ka) return fail(RVH_ERR_UNSUPPORTED, "no phase-A kernel for this (n_points, lanes_per_strand)");
    if (!prepare_kernel(ka)) return fail(RVH_ERR_CUDA, "cannot opt the step kernels into shared memory");
    rvh_status fs = finish_pending(a, s);
    if (fs != RVH_OK) return fs;
    const int which = a->params.grid_enabled ? a->pick_grid(-1, -1) : -1;
    DevAsset A = a->device_view(f, which);
    if (a->params.grid_enabled) RVH_CUDA(cudaMemsetAsync(A.grid, 0, a->grid_bytes(), s));
    const int per_cta = kWarps * (32 / a->lanes);
    const unsigned blocks_a = unsigned((a->n_strands + per_cta - 1) / per_cta);
    void* args[] = {&A};
    if (blocks_a > 0) RVH_CUDA(cudaLaunchKernel(ka, dim3(blocks_a), dim3(kThreads), args, kSmemBytes, s));
    if (a->params.grid_enabled) {
        rvh_status st = launch_plain_b(a, A, s);
        if (st != RVH_OK) return st;
        a->grid_dirty[which] = true;
        a->last_grid = which;
    }
    return RVH_OK;
}

}  // namespace rvh

using namespace rvh;

namespace {
cudaStream_t pick_stream(rvh_asset* a, void* s) { return s ? static_cast<cudaStream_t>(s) : a->ctx->stream; }


// 4x4 column-major float matrices as used by the reference (glm).
struct M4 {
    double m[16];  // m[col*4 + row]
};
M4 mat_identity() {
    M4 r{};
    for (int i = 0; i < 4; ++i) r.m[i * 4 + i] = 1.0;
    return r;
}
M4 mat_mul(const M4& a, const M4& b) {
    M4 r{};
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a.m[k * 4 + rr] * b.m[c * 4 + k];
            r.m[c * 4 + rr] = s;
        }
    return r;
}
// Right-handed rotation by `ang` radians about principal axis `ax`.
M4 mat_rot(int ax, double ang) {
    M4 r = mat_identity();
    const double c = std::cos(ang), s = std::sin(ang);
    const int i = (ax + 1) % 3, j = (ax + 2) % 3;
    r.m[i * 4 + i] = c;
    r.m[j * 4 + j] = c;
    r.m[i * 4 + j] = s;   // column i, row j
    r.m[j * 4 + i] = -s;  // column j, row i
    return r;
}
// Inverse of an affine matrix [R t; 0 1] with general 3x3 R.
bool mat_inverse_affine(const M4& a, M4& out) {
    const double* m = a.m;
    const double a00 = m[0], a01 = m[4], a02 = m[8], a10 = m[1], a11 = m[5], a12 = m[9], a20 = m[2], a21 = m[6],
                 a22 = m[10];
    const double c00 = a11 * a22 - a12 * a21, c01 = a02 * a21 - a01 * a22, c02 = a01 * a12 - a02 * a11;
    const double c10 = a12 * a20 - a10 * a22, c11 = a00 * a22 - a02 * a20, c12 = a02 * a10 - a00 * a12;
    const double c20 = a10 * a21 - a11 * a20, c21 = a01 * a20 - a00 * a21, c22 = a00 * a11 - a01 * a10;
    const double det = a00 * c00 + a01 * c10 + a02 * c20;
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    const double inv[3][3] = {{c00 / det, c01 / det, c02 / det}, {c10 / det, c11 / det, c12 / det},
                              {c20 / det, c21 / det, c22 / det}};
    out = mat_identity();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out.m[c * 4 + r] = inv[r][c];
    for (int r = 0; r < 3; ++r)
        out.m[12 + r] = -(inv[r][0] * m[12] + inv[r][1] * m[13] + inv[r][2] * m[14]);
    return true;
}
bool fill_collider(const M4& T, int32_t kind, float radius, rvh_collider* out) {
    M4 I;
    if (!mat_inverse_affine(T, I)) return false;
    std::memset(out, 0, sizeof(*out));
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            out->transform[c * 4 + r] = float(T.m[c * 4 + r]);
            out->inv[c * 4 + r] = float(I.m[c * 4 + r]);
            out->inv_trans[c * 4 + r] = float(I.m[r * 4 + c]);
        }
    out->kind = kind;
    out->radius = radius;
    return true;
}
// m: finite, column-major, last row (0, 0, 0, 1)
bool affine_finite(const float* m) {
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(m[k])) return false;
    return m[3] == 0.f && m[7] == 0.f && m[11] == 0.f && m[15] == 1.f;
}
}  // namespace

// transform = m * rest.transform in double, inverse and inverse-transpose from it
bool rvh::follow_collider(const rvh_collider& rest, const float* m, rvh_collider* out) {
    M4 H{}, T{};
    for (int i = 0; i < 16; ++i) {
        H.m[i] = m[i];
        T.m[i] = rest.transform[i];
    }
    if (!fill_collider(mat_mul(H, T), rest.kind, rest.radius, out)) return false;
    out->attach_to_head = rest.attach_to_head;
    return true;
}

extern "C" {

int32_t rvh_abi_version(void) { return RVH_ABI_VERSION; }
const char* rvh_last_error(void) { return last_error_cstr(); }

const char* rvh_status_string(rvh_status s) {
    switch (s) {
        case RVH_OK: return "ok";
        case RVH_ERR_INVALID_ARG: return "invalid argument";
        case RVH_ERR_CUDA: return "CUDA error";
        case RVH_ERR_OUT_OF_MEMORY: return "out of device memory";
        case RVH_ERR_BUDGET: return "HBM budget exceeded";
        case RVH_ERR_TIMEOUT: return "device-side wait timed out";
        case RVH_ERR_STATE: return "invalid state";
        case RVH_ERR_UNSUPPORTED: return "unsupported";
        case RVH_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

rvh_status rvh_context_create(const rvh_context_desc* desc, rvh_context** out) {
    if (!out) return fail(RVH_ERR_INVALID_ARG, "rvh_context_create: out is NULL");
    *out = nullptr;
    rvh_context_desc d{};
    if (desc) d = *desc;
    if (d.math != RVH_MATH_FAST && d.math != RVH_MATH_EXACT)
        return fail(RVH_ERR_INVALID_ARG, "rvh_context_create: unknown math mode");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(RVH_ERR_NO_DEVICE, "no CUDA device");
    if (d.device < 0 || d.device >= count) return fail(RVH_ERR_NO_DEVICE, "device ordinal out of range");
    RVH_CUDA(cudaSetDevice(d.device));
    size_t free_b = 0, total_b = 0;
    RVH_CUDA(cudaMemGetInfo(&free_b, &total_b));
    rvh_context* c = new (std::nothrow) rvh_context();
    if (!c) return fail(RVH_ERR_OUT_OF_MEMORY, "host allocation failed");
    c->device = d.device;
    c->math = d.math;
    c->budget.init(d.hbm_budget_bytes ? d.hbm_budget_bytes : uint64_t(double(free_b) * 0.9));
    cudaDeviceProp prop{};
    e = cudaGetDeviceProperties(&prop, d.device);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaGetDeviceProperties");
    }
    c->sm_count = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    *out = c;
    return RVH_OK;
}

rvh_status rvh_context_destroy(rvh_context* ctx) {
    if (!ctx) return RVH_OK;
    DeviceGuard g(ctx->device);   // releases even if the switch fails
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return RVH_OK;
}

rvh_status rvh_context_synchronize(rvh_context* ctx) {
    if (!ctx) return fail(RVH_ERR_INVALID_ARG, "ctx is NULL");
    RVH_DEVICE(ctx->device);
    RVH_CUDA(cudaDeviceSynchronize());
    return RVH_OK;
}

rvh_status rvh_pinned_alloc(size_t bytes, void** out) {
    if (!out) return fail(RVH_ERR_INVALID_ARG, "pinned_alloc: NULL");
    *out = nullptr;
    if (!bytes) return RVH_OK;
    RVH_CUDA(cudaMallocHost(out, bytes));
    return RVH_OK;
}

rvh_status rvh_pinned_free(void* p) {
    if (p) RVH_CUDA(cudaFreeHost(p));
    return RVH_OK;
}

rvh_status rvh_context_memory(rvh_context* ctx, uint64_t* used, uint64_t* budget) {
    if (!ctx) return fail(RVH_ERR_INVALID_ARG, "ctx is NULL");
    if (used) *used = ctx->budget.used();
    if (budget) *budget = ctx->budget.budget();
    return RVH_OK;
}

rvh_status rvh_sim_params_reference(rvh_sim_params* p) {
    if (!p) return fail(RVH_ERR_INVALID_ARG, "params is NULL");
    std::memset(p, 0, sizeof(*p));
    p->gravity[0] = 0.0f;
    p->gravity[1] = -9.8f;
    p->gravity[2] = 0.0f;
    p->damping = 0.998f;
    p->dftl_damping = 0.998f;
    p->vmax = 10.0f;
    p->k_penalty = 1900.0f;
    p->friction = 0.08f;
    p->repulsion = 0.0f;
    p->grid_scale = 1000000.0f;
    p->grid_enabled = 1;
    p->grid_wrap32 = 1;
    p->grid_origin[0] = -3.0f;
    p->grid_origin[1] = -2.0f;
    p->grid_origin[2] = -5.0f;
    p->grid_h = 7.0f / 64.0f;
    p->grid_dims[0] = p->grid_dims[1] = p->grid_dims[2] = 64;
    return RVH_OK;
}

rvh_status rvh_collider_from_trs(const float trans[3], const float rot_deg[3], const float scale[3], int32_t kind,
                                 float radius, rvh_collider* out) {
    if (!trans || !rot_deg || !scale || !out) return fail(RVH_ERR_INVALID_ARG, "collider_from_trs: NULL argument");
    if (kind != RVH_COLLIDER_SPHERE && kind != RVH_COLLIDER_ELLIPSOID)
        return fail(RVH_ERR_INVALID_ARG, "collider_from_trs: unknown kind");
    const double deg = 0.01745329251;  // degrees to radians as the reference converts (float)
    M4 T = mat_identity();
    for (int i = 0; i < 3; ++i) T.m[12 + i] = trans[i];
    M4 S = mat_identity();
    for (int i = 0; i < 3; ++i) S.m[i * 4 + i] = scale[i];
    const M4 Rx = mat_rot(0, double(float(rot_deg[0] * float(deg))));
    const M4 Ry = mat_rot(1, double(float(rot_deg[1] * float(deg))));
    const M4 Rz = mat_rot(2, double(float(rot_deg[2] * float(deg))));
    const M4 M = mat_mul(mat_mul(mat_mul(mat_mul(T, Rz), Ry), Rx), S);
    if (!fill_collider(M, kind, radius, out)) return fail(RVH_ERR_INVALID_ARG, "collider_from_trs: singular scale");
    return RVH_OK;
}

rvh_status rvh_collider_translate(rvh_collider* c, const float delta[3]) {
    if (!c || !delta) return fail(RVH_ERR_INVALID_ARG, "collider_translate: NULL argument");
    M4 M{};
    for (int i = 0; i < 16; ++i) M.m[i] = c->transform[i];
    M4 D = mat_identity();
    for (int i = 0; i < 3; ++i) D.m[12 + i] = delta[i];
    const M4 N = mat_mul(M, D);
    const int32_t attach = c->attach_to_head;
    if (!fill_collider(N, c->kind, c->radius, c)) return fail(RVH_ERR_INVALID_ARG, "collider_translate: singular");
    c->attach_to_head = attach;
    return RVH_OK;
}

rvh_status rvh_collider_follow(const rvh_collider* rest, const float m[16], rvh_collider* out) {
    if (!rest || !m || !out) return fail(RVH_ERR_INVALID_ARG, "collider_follow: NULL argument");
    if (!affine_finite(m)) return fail(RVH_ERR_INVALID_ARG, "collider_follow: m must be a finite affine matrix");
    rvh_collider c;
    if (!follow_collider(*rest, m, &c)) return fail(RVH_ERR_INVALID_ARG, "collider_follow: singular transform");
    *out = c;
    return RVH_OK;
}

rvh_status rvh_init_strands_reference(const float* roots, const float* normals, int32_t ns, int32_t n, float seg,
                                      const float dir_offset[3], void* out_records) {
    if (!roots || !normals || !dir_offset || !out_records || ns < 0 || n < RVH_MIN_POINTS || n > RVH_MAX_POINTS)
        return fail(RVH_ERR_INVALID_ARG, "init_strands_reference: bad argument");
    float* rec = static_cast<float*>(out_records);
    for (int s = 0; s < ns; ++s) {
        float* r = rec + size_t(s) * 12 * n;
        float p[3] = {roots[3 * s], roots[3 * s + 1], roots[3 * s + 2]};
        float d[3] = {normals[3 * s] + dir_offset[0], normals[3 * s + 1] + dir_offset[1],
                      normals[3 * s + 2] + dir_offset[2]};
        for (int j = 0; j < n; ++j) {
            float* x = r + 4 * j;
            float* v = r + 4 * n + 4 * j;
            float* c = r + 8 * n + 4 * j;
            x[0] = p[0]; x[1] = p[1]; x[2] = p[2]; x[3] = 1.0f;
            v[0] = 0.0f; v[1] = 0.0f; v[2] = -1.0f; v[3] = 0.0f;
            c[0] = c[1] = c[2] = c[3] = 0.0f;
            for (int q = 0; q < 3; ++q) p[q] += seg * d[q];
        }
    }
    return RVH_OK;
}

rvh_status rvh_asset_create(rvh_context* ctx, const rvh_asset_desc* desc, rvh_asset** out) {
    if (!ctx || !desc || !out) return fail(RVH_ERR_INVALID_ARG, "asset_create: NULL argument");
    *out = nullptr;
    const rvh_asset_desc& d = *desc;
    if (d.n_strands < 0 || d.n_points < RVH_MIN_POINTS || d.n_points > RVH_MAX_POINTS)
        return fail(RVH_ERR_INVALID_ARG, "asset_create: n_points must be in [2, 32] and n_strands >= 0");
    if (d.n_strands > 0 && !d.strands) return fail(RVH_ERR_INVALID_ARG, "asset_create: strands is NULL");
    if (d.strands_location < RVH_MEM_HOST || d.strands_location > RVH_MEM_DEVICE_BORROWED)
        return fail(RVH_ERR_INVALID_ARG, "asset_create: unknown strands_location");
    if (!d.rest_lengths && !(std::isfinite(d.uniform_rest_length) && d.uniform_rest_length >= 0.f))
        return fail(RVH_ERR_INVALID_ARG, "asset_create: bad uniform_rest_length");
    const int lanes = d.lanes_per_strand ? d.lanes_per_strand : default_lanes(d.n_points);
    if (!plain_a_supported(d.n_points, lanes))
        return fail(RVH_ERR_UNSUPPORTED, "asset_create: lanes_per_strand not supported for this n_points");
    RVH_DEVICE(ctx->device);
    rvh_asset* a = new (std::nothrow) rvh_asset();
    if (!a) return fail(RVH_ERR_OUT_OF_MEMORY, "host allocation failed");
    a->ctx = ctx;
    a->n_strands = d.n_strands;
    a->n_points = d.n_points;
    a->lanes = lanes;
    rvh_sim_params_reference(&a->params);
    auto cleanup = [&](rvh_status s) {
        rvh_asset_destroy(a);
        return s;
    };
    const size_t rb = a->record_bytes();
    rvh_status s;
    if (d.strands_location == RVH_MEM_DEVICE_BORROWED) {
        if (reinterpret_cast<uintptr_t>(d.strands) % 16 != 0)
            return cleanup(fail(RVH_ERR_INVALID_ARG, "asset_create: borrowed buffer must be 16-byte aligned"));
        a->strands.ptr = const_cast<void*>(d.strands);
        a->strands.bytes = rb;
        a->strands.owned = false;
    } else if (rb) {
        if ((s = ctx->alloc(a->strands, rb)) != RVH_OK) return cleanup(s);
        cudaError_t e = cudaMemcpy(a->strands.ptr, d.strands, rb,
                                   d.strands_location == RVH_MEM_HOST ? cudaMemcpyHostToDevice
                                                                      : cudaMemcpyDeviceToDevice);
        if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMemcpy strands"));
    }
    std::vector<float> rest(size_t(d.n_strands), d.uniform_rest_length);
    if (d.rest_lengths)
        for (int i = 0; i < d.n_strands; ++i) {
            if (!std::isfinite(d.rest_lengths[i]) || d.rest_lengths[i] < 0.f)
                return cleanup(fail(RVH_ERR_INVALID_ARG, "asset_create: bad rest length"));
            rest[i] = d.rest_lengths[i];
        }
    if (d.n_strands) {
        if ((s = ctx->alloc(a->rest, rest.size() * 4)) != RVH_OK) return cleanup(s);
        cudaError_t e = cudaMemcpy(a->rest.ptr, rest.data(), rest.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMemcpy rest"));
    }
    if (d.strand_wind && d.n_strands) {
        std::vector<float> w(size_t(d.n_strands) * 4, 0.f);
        for (int i = 0; i < d.n_strands; ++i)
            for (int q = 0; q < 3; ++q) w[4 * i + q] = d.strand_wind[3 * i + q];
        if ((s = ctx->alloc(a->wind, w.size() * 4)) != RVH_OK) return cleanup(s);
        cudaError_t e = cudaMemcpy(a->wind.ptr, w.data(), w.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMemcpy wind"));
        a->has_wind = true;
    }
    if ((s = ctx->alloc(a->draw, sizeof(rvh_draw_indirect))) != RVH_OK) return cleanup(s);
    rvh_draw_indirect di{uint32_t(d.n_strands), 1u, 0u, 0u};
    cudaError_t e = cudaMemcpy(a->draw.ptr, &di, sizeof(di), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMemcpy draw"));
    if ((s = ensure_grid(a)) != RVH_OK) return cleanup(s);
    *out = a;
    return RVH_OK;
}

rvh_status rvh_asset_destroy(rvh_asset* a) {
    if (!a) return RVH_OK;
    DeviceGuard g(a->ctx->device);   // releases even if the switch fails
    cudaStreamSynchronize(a->ctx->stream);
    Context* c = a->ctx;
    // a grid group outlives neither side: a member leaves its owner; an owner's members get
    // grids of their own back (empty, and stepping then fails, if that allocation fails)
    if (a->grid_owner) {
        auto& m = a->grid_owner->grid_members;
        m.erase(std::remove(m.begin(), m.end(), static_cast<Asset*>(a)), m.end());
        for (int i = 0; i < 3; ++i) a->grid[i] = DevBuf{};
    }
    for (Asset* m : a->grid_members) {
        m->grid_owner = nullptr;
        for (int i = 0; i < 3; ++i) m->grid[i] = DevBuf{};
        m->grid_cells = 0;
        m->pending = false;
        m->box_layout = 0u;
        m->last_grid = -1;
        if (ensure_grid(m) != RVH_OK) set_error("");
    }
    a->grid_members.clear();
    c->free(a->strands);
    c->free(a->rest);
    c->free(a->wind);
    for (int i = 0; i < 3; ++i) c->free(a->grid[i]);
    c->free(a->draw);
    c->free(a->root_rest);
    c->free(a->group_boxes);
    c->free(a->tess_tables);
    c->free(a->tess_cache);
    c->free(a->raster_px);
    c->free(a->raster_frags);
    c->free(a->raster_clip);
    delete a;
    return RVH_OK;
}

// Same grid geometry (what a grid group shares).
static bool same_grid(const rvh_sim_params& x, const rvh_sim_params& y) {
    return x.grid_enabled == y.grid_enabled && x.grid_dims[0] == y.grid_dims[0] && x.grid_dims[1] == y.grid_dims[1] &&
           x.grid_dims[2] == y.grid_dims[2] && x.grid_h == y.grid_h && x.grid_origin[0] == y.grid_origin[0] &&
           x.grid_origin[1] == y.grid_origin[1] && x.grid_origin[2] == y.grid_origin[2] &&
           x.grid_scale == y.grid_scale && x.grid_wrap32 == y.grid_wrap32;
}

rvh_status rvh_asset_set_params(rvh_asset* a, const rvh_sim_params* p) {
    if (!a || !p) return fail(RVH_ERR_INVALID_ARG, "set_params: NULL argument");
    rvh_status s = validate_params(*p);
    if (s != RVH_OK) return s;
    if (a->grid_grouped() && !same_grid(a->params, *p))
        return fail(RVH_ERR_STATE, "set_params: the asset shares its grid; leave the group to change the grid");
    RVH_DEVICE(a->ctx->device);
    s = finish_pending(a, a->ctx->stream);  // the pending gather uses the old grid geometry
    if (s != RVH_OK) return s;
    a->params = *p;
    return ensure_grid(a);
}

rvh_status rvh_asset_share_grid(rvh_asset* a, rvh_asset* owner) {
    if (!a) return fail(RVH_ERR_INVALID_ARG, "share_grid: NULL asset");
    RVH_DEVICE(a->ctx->device);
    if (!owner) {   // leave the group: the pending friction first, then grids of its own
        if (!a->grid_owner) {
            if (!a->grid_members.empty()) return fail(RVH_ERR_STATE, "share_grid: other assets share this asset's grid");
            return RVH_OK;
        }
        rvh_status fs = finish_pending(a, a->ctx->stream);
        if (fs != RVH_OK) return fs;
        RVH_CUDA(cudaStreamSynchronize(a->ctx->stream));
        auto& m = a->grid_owner->grid_members;
        m.erase(std::remove(m.begin(), m.end(), static_cast<Asset*>(a)), m.end());
        a->grid_owner = nullptr;
        for (int i = 0; i < 3; ++i) a->grid[i] = DevBuf{};
        a->grid_cells = 0;
        a->pending = false;
        a->box_layout = 0u;
        a->last_grid = -1;
        return ensure_grid(a);
    }
    if (a == owner || a->ctx != owner->ctx) return fail(RVH_ERR_INVALID_ARG, "share_grid: another asset of the same context");
    if (!a->params.grid_enabled || !same_grid(a->params, owner->params))
        return fail(RVH_ERR_INVALID_ARG, "share_grid: both assets need the grid, with the same dims, origin, cell size, "
                                         "scale and wrap mode");
    if (a->grid_grouped()) return fail(RVH_ERR_STATE, "share_grid: the asset already shares a grid");
    if (owner->grid_owner) return fail(RVH_ERR_STATE, "share_grid: the owner shares another asset's grid");
    if (a->server_managed || owner->server_managed)
        return fail(RVH_ERR_STATE, "share_grid: an asset registered with a request server");
    if (!owner->grid[0].ptr || !owner->grid[1].ptr || !owner->grid[2].ptr)
        return fail(RVH_ERR_STATE, "share_grid: the owner has no grid");
    rvh_status fs = finish_pending(a, a->ctx->stream);   // gathers from a's own grid, which goes
    if (fs != RVH_OK) return fs;
    RVH_CUDA(cudaStreamSynchronize(a->ctx->stream));
    for (int i = 0; i < 3; ++i) {
        a->ctx->free(a->grid[i]);
        a->grid[i] = DevBuf{owner->grid[i].ptr, owner->grid[i].bytes, owner->ctx, false};
        a->grid_dirty[i] = owner->grid_dirty[i];
    }
    a->grid_cells = owner->grid_cells;
    a->grid_owner = owner;
    owner->grid_members.push_back(a);
    a->pending = false;
    a->box_layout = 0u;
    a->last_grid = -1;
    return RVH_OK;
}

rvh_status rvh_asset_set_colliders(rvh_asset* a, const rvh_collider* c, int32_t n) {
    if (!a || (n > 0 && !c)) return fail(RVH_ERR_INVALID_ARG, "set_colliders: NULL argument");
    if (n < 0 || n > RVH_MAX_COLLIDERS) return fail(RVH_ERR_INVALID_ARG, "set_colliders: at most 8 colliders");
    for (int i = 0; i < n; ++i) {
        if (c[i].kind != RVH_COLLIDER_SPHERE && c[i].kind != RVH_COLLIDER_ELLIPSOID)
            return fail(RVH_ERR_INVALID_ARG, "set_colliders: unknown collider kind");
        if (c[i].kind == RVH_COLLIDER_SPHERE && !(c[i].radius >= 0.f))
            return fail(RVH_ERR_INVALID_ARG, "set_colliders: sphere radius must be >= 0");
        for (int k = 0; k < 16; ++k)
            if (!std::isfinite(c[i].transform[k]) || !std::isfinite(c[i].inv[k]) || !std::isfinite(c[i].inv_trans[k]))
                return fail(RVH_ERR_INVALID_ARG, "set_colliders: non-finite matrix");
    }
    a->colliders.assign(c, c + n);
    return RVH_OK;
}

rvh_status rvh_asset_set_head_transform(rvh_asset* a, const float m[16]) {
    if (!a) return fail(RVH_ERR_INVALID_ARG, "set_head_transform: NULL asset");
    if (!m) {
        a->head_active = false;
        return RVH_OK;
    }
    if (!affine_finite(m)) return fail(RVH_ERR_INVALID_ARG, "set_head_transform: m must be a finite affine matrix");
    if (!a->root_rest.ptr && a->n_strands > 0) {
        // the roots now are the rest pose of m = identity (roots never move without a head motion)
        RVH_DEVICE(a->ctx->device);
        rvh_status s = a->ctx->alloc(a->root_rest, size_t(a->n_strands) * 16u);
        if (s != RVH_OK) return s;
        RVH_CUDA(cudaStreamSynchronize(a->ctx->stream));
        RVH_CUDA(cudaMemcpy2D(a->root_rest.ptr, 16, a->strands.ptr, size_t(48) * a->n_points, 16, size_t(a->n_strands),
                              cudaMemcpyDeviceToDevice));
    }
    std::memcpy(a->head, m, sizeof(a->head));
    a->head_active = true;
    return RVH_OK;
}

rvh_status rvh_asset_set_rest_lengths(rvh_asset* a, const float* rest) {
    if (!a || (!rest && a->n_strands)) return fail(RVH_ERR_INVALID_ARG, "set_rest_lengths: NULL argument");
    for (int i = 0; i < a->n_strands; ++i)
        if (!std::isfinite(rest[i]) || rest[i] < 0.f) return fail(RVH_ERR_INVALID_ARG, "set_rest_lengths: bad value");
    if (!a->n_strands) return RVH_OK;
    RVH_DEVICE(a->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(a->ctx->stream));
    RVH_CUDA(cudaMemcpy(a->rest.ptr, rest, sizeof(float) * a->n_strands, cudaMemcpyHostToDevice));
    return RVH_OK;
}

rvh_status rvh_asset_set_strand_wind(rvh_asset* a, const float* wind3) {
    if (!a) return fail(RVH_ERR_INVALID_ARG, "set_strand_wind: NULL asset");
    RVH_DEVICE(a->ctx->device);
    RVH_CUDA(cudaStreamSynchronize(a->ctx->stream));
    if (!wind3 || !a->n_strands) {
        a->has_wind = false;
        return RVH_OK;
    }
    std::vector<float> w(size_t(a->n_strands) * 4, 0.f);
    for (int i = 0; i < a->n_strands; ++i)
        for (int q = 0; q < 3; ++q) {
            if (!std::isfinite(wind3[3 * i + q])) return fail(RVH_ERR_INVALID_ARG, "set_strand_wind: non-finite");
            w[4 * i + q] = wind3[3 * i + q];
        }
    if (!a->wind.ptr) {
        rvh_status s = a->ctx->alloc(a->wind, w.size() * 4);
        if (s != RVH_OK) return s;
    }
    RVH_CUDA(cudaMemcpy(a->wind.ptr, w.data(), w.size() * 4, cudaMemcpyHostToDevice));
    a->has_wind = true;
    return RVH_OK;
}

rvh_status rvh_asset_device_ptr(rvh_asset* a, void** out) {
    if (!a || !out) return fail(RVH_ERR_INVALID_ARG, "device_ptr: NULL argument");
    *out = a->strands.ptr;
    return RVH_OK;
}

rvh_status rvh_asset_draw_indirect(rvh_asset* a, void** out) {
    if (!a || !out) return fail(RVH_ERR_INVALID_ARG, "draw_indirect: NULL argument");
    *out = a->draw.ptr;
    return RVH_OK;
}

rvh_status rvh_asset_strand_count(rvh_asset* a, int32_t* ns, int32_t* n) {
    if (!a) return fail(RVH_ERR_INVALID_ARG, "strand_count: NULL asset");
    if (ns) *ns = a->n_strands;
    if (n) *n = a->n_points;
    return RVH_OK;
}

rvh_status rvh_asset_read(rvh_asset* a, void* dst, size_t bytes) {
    if (!a || (!dst && bytes)) return fail(RVH_ERR_INVALID_ARG, "asset_read: NULL argument");
    if (bytes != a->record_bytes()) return fail(RVH_ERR_INVALID_ARG, "asset_read: size must be 48*n_points*n_strands");
    RVH_DEVICE(a->ctx->device);
    rvh_status fs = finish_pending(a, a->ctx->stream);
    if (fs != RVH_OK) return fs;
    RVH_CUDA(cudaDeviceSynchronize());
    if (bytes) RVH_CUDA(cudaMemcpy(dst, a->strands.ptr, bytes, cudaMemcpyDeviceToHost));
    return RVH_OK;
}

rvh_status rvh_asset_write(rvh_asset* a, const void* src, size_t bytes) {
    if (!a || (!src && bytes)) return fail(RVH_ERR_INVALID_ARG, "asset_write: NULL argument");
    if (bytes != a->record_bytes()) return fail(RVH_ERR_INVALID_ARG, "asset_write: size must be 48*n_points*n_strands");
    RVH_DEVICE(a->ctx->device);
    RVH_CUDA(cudaDeviceSynchronize());
    a->pending = false;  // the new state carries no pending friction
    if (bytes) RVH_CUDA(cudaMemcpy(a->strands.ptr, src, bytes, cudaMemcpyHostToDevice));
    return RVH_OK;
}

rvh_status rvh_asset_read_positions_async(rvh_asset* a, void* dst, size_t bytes, void* stream) {
    if (!a || (!dst && bytes)) return fail(RVH_ERR_INVALID_ARG, "read_positions: NULL argument");
    const size_t need = size_t(a->n_strands) * a->n_points * 16u;
    if (bytes != need) return fail(RVH_ERR_INVALID_ARG, "read_positions: size must be 16*n_points*n_strands");
    if (!need) return RVH_OK;
    RVH_DEVICE(a->ctx->device);
    cudaStream_t s = pick_stream(a, stream);
    // curvePoints[n] is the first 16*n bytes of each 48*n-byte record: one strided 2-D copy.
    RVH_CUDA(cudaMemcpy2DAsync(dst, 16u * a->n_points, a->strands.ptr, 48u * a->n_points, 16u * a->n_points,
                               size_t(a->n_strands), cudaMemcpyDeviceToHost, s));
    return RVH_OK;
}

rvh_status rvh_asset_read_draw(rvh_asset* a, rvh_draw_indirect* out) {
    if (!a || !out) return fail(RVH_ERR_INVALID_ARG, "read_draw: NULL argument");
    RVH_DEVICE(a->ctx->device);
    RVH_CUDA(cudaDeviceSynchronize());
    RVH_CUDA(cudaMemcpy(out, a->draw.ptr, sizeof(*out), cudaMemcpyDeviceToHost));
    return RVH_OK;
}

rvh_status rvh_asset_read_grid(rvh_asset* a, int64_t* dst, size_t bytes) {
    if (!a || !dst) return fail(RVH_ERR_INVALID_ARG, "read_grid: NULL argument");
    if (!a->params.grid_enabled) return fail(RVH_ERR_STATE, "read_grid: the grid is disabled");
    if (bytes != a->grid_bytes()) return fail(RVH_ERR_INVALID_ARG, "read_grid: size must be 32*cells");
    RVH_DEVICE(a->ctx->device);
    RVH_CUDA(cudaDeviceSynchronize());
    if (a->last_grid < 0) return fail(RVH_ERR_STATE, "read_grid: no step has splatted yet");
    RVH_CUDA(cudaMemcpy(dst, a->grid[a->last_grid].ptr, bytes, cudaMemcpyDeviceToHost));
    return RVH_OK;
}

rvh_status rvh_step(rvh_asset* a, const rvh_frame* frame, void* stream) {
    TraceRange trace("rvh_step");
    if (!a || !frame) return fail(RVH_ERR_INVALID_ARG, "step: NULL argument");
    rvh_status s = validate_frame(*frame);
    if (s != RVH_OK) return s;
    if (a->n_strands == 0) return RVH_OK;
    RVH_DEVICE(a->ctx->device);
    return launch_plain(a, *frame, pick_stream(a, stream));
}

}  // extern "C"
