/*
 * scene_oracle.hpp — TEST INFRASTRUCTURE ONLY.
 *
 * A second, independent statement of the seeded synthetic inputs that the
 * benchmarks and tests step (include/rvh_scene.h: rvh_generate_head,
 * rvh_wind_at, with rvh_collider_from_trs and rvh_sim_params_reference from
 * include/rvh.h).  The CPU timing arm of bench.py builds its workload sample
 * with it, so that process never maps the CUDA library; tests/test_host.py
 * checks that it gives the library's bytes for the workloads it stands in for.
 *
 * The inputs stand in for the reference's asset set-up: straight strands along
 * the root normal (src/Strand.cpp:157-175 builds them from OBJ roots), the
 * reference constants (src/shaders/compute.comp:7-11,150,163,187,205-206,296)
 * and colliders built as T * Rz * Ry * Rx * S (src/Scene.h:29-39).
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../include/rvh_scene.h"
#include "../include/rvh_types.h"

namespace oracle {
namespace scene {

constexpr double kPi = 3.14159265358979323846;
constexpr uint64_t kGolden = 0x9e3779b97f4a7c15ull;

/* SplitMix64's output function (Steele, Lea and Flood, OOPSLA 2014). */
inline uint64_t splitmix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

/* Draw `counter` of the stream of `seed` (counters start at 0). */
inline uint64_t draw_u64(uint64_t seed, uint64_t counter) {
    return splitmix(splitmix(seed + kGolden) + (counter + 1) * kGolden);
}
inline double draw_uniform(uint64_t seed, uint64_t counter) {
    return double(draw_u64(seed, counter) >> 11) * (1.0 / 9007199254740992.0);
}
/* Box-Muller on draws 2c and 2c+1. */
inline double draw_normal(uint64_t seed, uint64_t counter) {
    const double a = draw_uniform(seed, 2 * counter), b = draw_uniform(seed, 2 * counter + 1);
    return std::sqrt(-2.0 * std::log(1.0 - a)) * std::cos(2.0 * kPi * b);
}

/* A sequential stream: the k-th call returns draw k of the seed. */
struct Stream {
    uint64_t seed;
    uint64_t next = 0;
    explicit Stream(uint64_t s) : seed(s) {}
    double uniform() { return draw_uniform(seed, next++); }
    double between(double lo, double hi) { return lo + (hi - lo) * uniform(); }
};

struct d3 {
    double x, y, z;
};

/* Upper-hemisphere direction, uniform in area: the height is uniform in [0, 1). */
inline d3 hemisphere(Stream& s) {
    const double h = s.uniform();
    const double az = 2.0 * kPi * s.uniform();
    const double ring = std::sqrt(std::max(0.0, 1.0 - h * h));
    return {ring * std::cos(az), h, ring * std::sin(az)};
}

/* Dart throwing on the unit upper hemisphere: a candidate is kept when no
 * kept point is closer than the current radius (chord distance); the radius
 * shrinks by 10% whenever 200 n + 1000 candidates in a row were rejected. */
inline std::vector<d3> darts(Stream& s, int n) {
    const double r0 = 0.8 * std::sqrt(4.376 / std::max(1, n));
    const double cw = r0;   // bucket width: the starting radius
    const int nb = int(std::ceil(2.0 / cw)) + 2;
    auto bucket = [&](double v) { return int(std::floor((v + 1.0) / cw)); };
    auto id = [&](int i, int j, int k) { return (int64_t(i) * nb + j) * nb + k; };
    std::unordered_map<int64_t, std::vector<int>> buckets;
    std::vector<d3> kept;
    kept.reserve(size_t(std::max(n, 0)));
    double r = r0;
    int64_t misses = 0;
    const int64_t patience = int64_t(n) * 200 + 1000;
    while (int(kept.size()) < n) {
        if (++misses > patience) {
            r *= 0.9;
            misses = 0;
        }
        const d3 p = hemisphere(s);
        const int bi = bucket(p.x), bj = bucket(p.y), bk = bucket(p.z);
        bool far = true;
        for (int i = bi - 1; i <= bi + 1 && far; ++i)
            for (int j = bj - 1; j <= bj + 1 && far; ++j)
                for (int k = bk - 1; k <= bk + 1 && far; ++k) {
                    const auto it = buckets.find(id(i, j, k));
                    if (it == buckets.end()) continue;
                    for (int q : it->second) {
                        const double dx = kept[q].x - p.x, dy = kept[q].y - p.y, dz = kept[q].z - p.z;
                        if (dx * dx + dy * dy + dz * dz < r * r) {
                            far = false;
                            break;
                        }
                    }
                }
        if (!far) continue;
        buckets[id(bi, bj, bk)].push_back(int(kept.size()));
        kept.push_back(p);
    }
    return kept;
}

/* Interleaves the low 10 bits of x, y, z (x in bit 0). */
inline uint64_t interleave3(uint32_t x, uint32_t y, uint32_t z) {
    uint64_t key = 0;
    for (int b = 0; b < 10; ++b) {
        key |= uint64_t((x >> b) & 1u) << (3 * b);
        key |= uint64_t((y >> b) & 1u) << (3 * b + 1);
        key |= uint64_t((z >> b) & 1u) << (3 * b + 2);
    }
    return key;
}

/* Column-major 4x4 in double: a[col * 4 + row]. */
struct Mat {
    double a[16];
};
inline Mat eye() {
    Mat m{};
    m.a[0] = m.a[5] = m.a[10] = m.a[15] = 1.0;
    return m;
}
inline Mat mul(const Mat& p, const Mat& q) {
    Mat m{};
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            double acc = 0;
            for (int k = 0; k < 4; ++k) acc += p.a[k * 4 + row] * q.a[col * 4 + k];
            m.a[col * 4 + row] = acc;
        }
    return m;
}
/* Rotation by `rad` about axis `axis` (0 x, 1 y, 2 z), right-handed. */
inline Mat rotation(int axis, double rad) {
    Mat m = eye();
    const int u = (axis + 1) % 3, w = (axis + 2) % 3;
    const double c = std::cos(rad), s = std::sin(rad);
    m.a[u * 4 + u] = c;
    m.a[w * 4 + w] = c;
    m.a[u * 4 + w] = s;
    m.a[w * 4 + u] = -s;
    return m;
}
/* Inverse of [A t; 0 1] by the adjugate of A; false when A is singular. */
inline bool affine_inverse(const Mat& m, Mat& out) {
    const double* a = m.a;
    // cofactor matrix entries, cof[r][c], of the 3x3 block A(r, c) = a[c*4 + r]
    const double A00 = a[0], A01 = a[4], A02 = a[8], A10 = a[1], A11 = a[5], A12 = a[9], A20 = a[2], A21 = a[6],
                 A22 = a[10];
    const double adj[3][3] = {{A11 * A22 - A12 * A21, A02 * A21 - A01 * A22, A01 * A12 - A02 * A11},
                              {A12 * A20 - A10 * A22, A00 * A22 - A02 * A20, A02 * A10 - A00 * A12},
                              {A10 * A21 - A11 * A20, A01 * A20 - A00 * A21, A00 * A11 - A01 * A10}};
    const double det = A00 * adj[0][0] + A01 * adj[1][0] + A02 * adj[2][0];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    double inv[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) inv[r][c] = adj[r][c] / det;
    out = eye();
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out.a[c * 4 + r] = inv[r][c];
    for (int r = 0; r < 3; ++r) out.a[12 + r] = -(inv[r][0] * a[12] + inv[r][1] * a[13] + inv[r][2] * a[14]);
    return true;
}

/* Collider = {T * Rz * Ry * Rx * S, its inverse, the inverse's transpose}
 * rounded to float (src/Scene.h:29-39; degrees to radians in float with the
 * reference's constant). */
inline bool collider_trs(const float t[3], const float deg[3], const float s[3], int32_t kind, float radius,
                         rvh_collider* out) {
    const double to_rad = 0.01745329251;
    Mat T = eye(), S = eye();
    for (int i = 0; i < 3; ++i) {
        T.a[12 + i] = t[i];
        S.a[i * 5] = s[i];
    }
    Mat R[3];
    for (int ax = 0; ax < 3; ++ax) R[ax] = rotation(ax, double(float(deg[ax] * float(to_rad))));
    const Mat M = mul(mul(mul(mul(T, R[2]), R[1]), R[0]), S);
    Mat I;
    if (!affine_inverse(M, I)) return false;
    std::memset(out, 0, sizeof(*out));
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            out->transform[c * 4 + r] = float(M.a[c * 4 + r]);
            out->inv[c * 4 + r] = float(I.a[c * 4 + r]);
            out->inv_trans[c * 4 + r] = float(I.a[r * 4 + c]);
        }
    out->kind = kind;
    out->radius = radius;
    return true;
}

/* The reference's constants (compute.comp:7-11,150,163,187,205-206,296). */
inline void reference_params(rvh_sim_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->gravity[1] = -9.8f;
    p->damping = 0.998f;
    p->dftl_damping = 0.998f;
    p->vmax = 10.0f;
    p->k_penalty = 1900.0f;
    p->friction = 0.08f;
    p->grid_scale = 1000000.0f;
    p->grid_enabled = 1;
    p->grid_wrap32 = 1;
    p->grid_origin[0] = -3.0f;
    p->grid_origin[1] = -2.0f;
    p->grid_origin[2] = -5.0f;
    p->grid_h = 7.0f / 64.0f;
    p->grid_dims[0] = p->grid_dims[1] = p->grid_dims[2] = 64;
}

/* A synthetic head: draws roots (uniform or dart throwing), then lengths, in
 * one stream of the seed; optionally orders the strands along a Morton curve
 * of the root direction; colliders from a second stream (seed ^ 0x5deece66d). */
inline int head(const rvh_head_desc* d, float* rec, float* rest, rvh_sim_params* params, rvh_collider* cols,
                int32_t* n_cols) {
    if (!d || d->n_strands < 0 || d->n_points < RVH_MIN_POINTS || d->n_points > RVH_MAX_POINTS) return 1;
    if ((!rec || !rest) && d->n_strands > 0) return 1;
    const int want = (d->head_collider ? 1 : 0) + std::max(0, int(d->n_ellipsoids));
    if (want > RVH_MAX_COLLIDERS) return 1;
    const int ns = d->n_strands, n = d->n_points;
    Stream s(d->seed);
    std::vector<d3> dir;
    if (d->root_sampling == RVH_ROOTS_POISSON) {
        dir = darts(s, ns);
    } else {
        for (int i = 0; i < ns; ++i) dir.push_back(hemisphere(s));
    }
    const size_t count = size_t(ns);
    std::vector<double> len(count);
    for (int i = 0; i < ns; ++i) len[i] = s.between(d->length_min, d->length_max);
    std::vector<int> order(count);
    for (int i = 0; i < ns; ++i) order[i] = i;
    if (d->sort_roots) {
        auto q10 = [](double v) { return uint32_t(std::min(1023.0, std::max(0.0, (v + 1.0) * 511.5))); };
        std::vector<std::pair<uint64_t, int>> key(count);
        for (int i = 0; i < ns; ++i) key[i] = {interleave3(q10(dir[i].x), q10(dir[i].y), q10(dir[i].z)), i};
        std::stable_sort(key.begin(), key.end());
        for (int i = 0; i < ns; ++i) order[i] = key[i].second;
    }
    const double R = d->head_radius;
    for (int i = 0; i < ns; ++i) {
        const d3 u = dir[order[i]];
        const float seg = float(len[order[i]] / double(n - 1));
        rest[i] = seg;
        const float root[3] = {float(d->head_center[0] + R * u.x), float(d->head_center[1] + R * u.y),
                               float(d->head_center[2] + R * u.z)};
        const float nrm[3] = {float(u.x), float(u.y), float(u.z)};
        float* x = rec + size_t(i) * 12 * n;
        std::memset(x, 0, sizeof(float) * 12 * n);
        for (int j = 0; j < n; ++j) {
            for (int q = 0; q < 3; ++q) x[4 * j + q] = root[q] + float(j) * seg * nrm[q];
            x[4 * j + 3] = 1.0f;
        }
    }
    if (params) {
        reference_params(params);
        if (d->dftl_damping > 0.f) params->dftl_damping = d->dftl_damping;
        params->friction = d->friction;
        params->repulsion = d->repulsion;
        params->grid_wrap32 = 0;
        params->grid_enabled = d->grid_res > 0 ? 1 : 0;
        if (d->grid_res > 0) {
            const double half = R + d->length_max + 0.05;
            params->grid_dims[0] = params->grid_dims[1] = params->grid_dims[2] = d->grid_res;
            params->grid_h = float(2.0 * half / d->grid_res);
            for (int q = 0; q < 3; ++q) params->grid_origin[q] = float(d->head_center[q] - half);
        }
    }
    int k = 0;
    if (cols) {
        const float zero[3] = {0.f, 0.f, 0.f}, one[3] = {1.f, 1.f, 1.f};
        if (d->head_collider) {
            const float c[3] = {float(d->head_center[0]), float(d->head_center[1]), float(d->head_center[2])};
            collider_trs(c, zero, one, RVH_COLLIDER_SPHERE, float(R), &cols[k++]);
        }
        Stream e(d->seed ^ 0x5deece66dull);
        for (int q = 0; q < d->n_ellipsoids; ++q) {
            const double phi = 2.0 * kPi * e.uniform();
            const double el = e.between(-0.9, 0.2);
            const double dist = R * e.between(1.0, 1.5);
            const float c[3] = {float(d->head_center[0] + dist * std::cos(el) * std::cos(phi)),
                                float(d->head_center[1] + dist * std::sin(el)),
                                float(d->head_center[2] + dist * std::cos(el) * std::sin(phi))};
            float deg[3], ax[3];
            for (int a = 0; a < 3; ++a) deg[a] = float(e.between(0.0, 360.0));
            for (int a = 0; a < 3; ++a) ax[a] = float(e.between(d->axis_min, d->axis_max));
            if (!collider_trs(c, deg, ax, RVH_COLLIDER_ELLIPSOID, 1.0f, &cols[k++])) return 1;
        }
    }
    if (n_cols) *n_cols = cols ? k : 0;
    return 0;
}

/* Wind of frame `step` at time t: amplitude sin(omega t) dir + a Gaussian gust
 * per component (draws 3 step + q of the seed's normal stream). */
inline void wind(const rvh_wind_desc* w, int64_t step, float t, float out[3]) {
    const double base = double(w->amplitude) * std::sin(double(w->omega) * double(t));
    for (int q = 0; q < 3; ++q) {
        const double gust = w->gust_sigma > 0.f ? double(w->gust_sigma) * draw_normal(w->seed, uint64_t(step) * 3 + q)
                                                : 0.0;
        out[q] = float(base * double(w->dir[q]) + gust);
    }
}

}  // namespace scene
}  // namespace oracle
