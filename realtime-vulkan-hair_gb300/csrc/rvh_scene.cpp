// rvh_scene.cpp — seeded synthetic heads, wind and orbiting colliders
// (include/rvh_scene.h).  Host-only C++.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/rvh.h"
#include "../../include/rvh_scene.h"
#include "rvh_internal.hpp"

namespace {

// SplitMix64 finaliser (Steele, Lea, Flood 2014); counter-based use: the
// stream of a seed is mix(mix(seed) + (counter + 1) * golden).
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
constexpr uint64_t kGolden = 0x9e3779b97f4a7c15ull;
constexpr double kPi = 3.14159265358979323846;

struct Rng {
    uint64_t key;
    uint64_t ctr = 0;
    explicit Rng(uint64_t seed) : key(mix64(seed + kGolden)) {}
    uint64_t u64() { return mix64(key + (++ctr) * kGolden); }
    double uniform() { return double(u64() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * uniform(); }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(2.0 * kPi * u2);
    }
};

struct V3 {
    double x, y, z;
};

// Uniform direction on the upper hemisphere (y >= 0): y ~ U(0,1) (Archimedes).
V3 hemi_dir(Rng& r) {
    const double y = r.uniform();
    const double phi = 2.0 * kPi * r.uniform();
    const double s = std::sqrt(std::max(0.0, 1.0 - y * y));
    return {s * std::cos(phi), y, s * std::sin(phi)};
}

// Dart throwing on the unit upper hemisphere with a minimum chord distance.
std::vector<V3> poisson_hemi(Rng& r, int n) {
    const double rmin = 0.8 * std::sqrt(4.376 / std::max(1, n));
    const double cell = rmin;
    const int dim = int(std::ceil(2.0 / cell)) + 2;
    std::unordered_map<int64_t, std::vector<int>> hash;
    auto key = [&](int i, int j, int k) { return (int64_t(i) * dim + j) * dim + k; };
    auto cidx = [&](double v) { return int(std::floor((v + 1.0) / cell)); };
    std::vector<V3> pts;
    pts.reserve(n);
    int64_t attempts = 0;
    const int64_t max_attempts = int64_t(n) * 200 + 1000;
    double rr = rmin;
    while (int(pts.size()) < n) {
        if (++attempts > max_attempts) {  // saturated: shrink the radius and continue
            rr *= 0.9;
            attempts = 0;
        }
        const V3 p = hemi_dir(r);
        const int ci = cidx(p.x), cj = cidx(p.y), ck = cidx(p.z);
        bool ok = true;
        for (int di = -1; di <= 1 && ok; ++di)
            for (int dj = -1; dj <= 1 && ok; ++dj)
                for (int dk = -1; dk <= 1 && ok; ++dk) {
                    auto it = hash.find(key(ci + di, cj + dj, ck + dk));
                    if (it == hash.end()) continue;
                    for (int q : it->second) {
                        const double dx = pts[q].x - p.x, dy = pts[q].y - p.y, dz = pts[q].z - p.z;
                        if (dx * dx + dy * dy + dz * dz < rr * rr) {
                            ok = false;
                            break;
                        }
                    }
                }
        if (!ok) continue;
        hash[key(ci, cj, ck)].push_back(int(pts.size()));
        pts.push_back(p);
    }
    return pts;
}

uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    auto spread = [](uint64_t v) {
        v &= 0x3ff;
        v = (v | (v << 16)) & 0x30000ff;
        v = (v | (v << 8)) & 0x300f00f;
        v = (v | (v << 4)) & 0x30c30c3;
        v = (v | (v << 2)) & 0x9249249;
        return v;
    };
    return spread(x) | (spread(y) << 1) | (spread(z) << 2);
}

}  // namespace

extern "C" {

uint64_t rvh_rng_u64(uint64_t seed, uint64_t counter) { return mix64(mix64(seed + kGolden) + (counter + 1) * kGolden); }
double rvh_rng_uniform(uint64_t seed, uint64_t counter) {
    return double(rvh_rng_u64(seed, counter) >> 11) * (1.0 / 9007199254740992.0);
}
double rvh_rng_normal(uint64_t seed, uint64_t counter) {
    const double u1 = rvh_rng_uniform(seed, 2 * counter), u2 = rvh_rng_uniform(seed, 2 * counter + 1);
    return std::sqrt(-2.0 * std::log(1.0 - u1)) * std::cos(2.0 * kPi * u2);
}

rvh_status rvh_wind_at(const rvh_wind_desc* w, int64_t step, float t, float out[3]) {
    if (!w || !out) return rvh::fail(RVH_ERR_INVALID_ARG, "wind_at: NULL argument");
    const double base = double(w->amplitude) * std::sin(double(w->omega) * double(t));
    for (int q = 0; q < 3; ++q) {
        double g = 0.0;
        if (w->gust_sigma > 0.f) g = double(w->gust_sigma) * rvh_rng_normal(w->seed, uint64_t(step) * 3 + q);
        out[q] = float(base * double(w->dir[q]) + g);
    }
    return RVH_OK;
}

rvh_status rvh_sphere_on_orbit(const rvh_orbit* o, float t, rvh_collider* out) {
    if (!o || !out) return rvh::fail(RVH_ERR_INVALID_ARG, "sphere_on_orbit: NULL argument");
    const double a = double(o->omega) * double(t) + double(o->phase);
    const float c[3] = {float(o->center[0] + o->orbit_radius * std::cos(a)), o->center[1],
                        float(o->center[2] + o->orbit_radius * std::sin(a))};
    const float rot[3] = {0.f, 0.f, 0.f}, one[3] = {1.f, 1.f, 1.f};
    return rvh_collider_from_trs(c, rot, one, RVH_COLLIDER_SPHERE, o->sphere_radius, out);
}

rvh_status rvh_generate_head(const rvh_head_desc* d, void* records, float* rest, rvh_sim_params* params,
                             rvh_collider* colliders, int32_t* n_colliders) {
    if (!d || (!records && d->n_strands > 0) || (!rest && d->n_strands > 0))
        return rvh::fail(RVH_ERR_INVALID_ARG, "generate_head: NULL argument");
    if (d->n_strands < 0 || d->n_points < RVH_MIN_POINTS || d->n_points > RVH_MAX_POINTS)
        return rvh::fail(RVH_ERR_INVALID_ARG, "generate_head: bad sizes");
    if (!(d->head_radius > 0.f) || d->length_min < 0.f || d->length_max < d->length_min)
        return rvh::fail(RVH_ERR_INVALID_ARG, "generate_head: bad radius or lengths");
    const int ncol = (d->head_collider ? 1 : 0) + std::max(0, int(d->n_ellipsoids));
    if (ncol > RVH_MAX_COLLIDERS) return rvh::fail(RVH_ERR_INVALID_ARG, "generate_head: too many colliders");
    const int ns = d->n_strands, n = d->n_points;
    const double R = d->head_radius;
    const V3 c = {d->head_center[0], d->head_center[1], d->head_center[2]};
    Rng rng(d->seed);
    std::vector<V3> dirs;
    if (d->root_sampling == RVH_ROOTS_POISSON) {
        dirs = poisson_hemi(rng, ns);
    } else {
        dirs.resize(ns);
        for (int s = 0; s < ns; ++s) dirs[s] = hemi_dir(rng);
    }
    std::vector<double> len(ns);
    for (int s = 0; s < ns; ++s) len[s] = rng.range(d->length_min, d->length_max);
    if (d->sort_roots) {
        std::vector<std::pair<uint64_t, int>> key(ns);
        for (int s = 0; s < ns; ++s) {
            auto q = [](double v) { return uint32_t(std::min(1023.0, std::max(0.0, (v + 1.0) * 511.5))); };
            key[s] = {morton3(q(dirs[s].x), q(dirs[s].y), q(dirs[s].z)), s};
        }
        std::stable_sort(key.begin(), key.end());
        std::vector<V3> d2(ns);
        std::vector<double> l2(ns);
        for (int s = 0; s < ns; ++s) {
            d2[s] = dirs[key[s].second];
            l2[s] = len[key[s].second];
        }
        dirs.swap(d2);
        len.swap(l2);
    }
    float* rec = static_cast<float*>(records);
    for (int s = 0; s < ns; ++s) {
        const float seg = float(len[s] / double(n - 1));
        rest[s] = seg;
        const float root[3] = {float(c.x + R * dirs[s].x), float(c.y + R * dirs[s].y), float(c.z + R * dirs[s].z)};
        const float nrm[3] = {float(dirs[s].x), float(dirs[s].y), float(dirs[s].z)};
        float* r = rec + size_t(s) * 12 * n;
        for (int j = 0; j < n; ++j) {
            float* x = r + 4 * j;
            float* v = r + 4 * n + 4 * j;
            float* cc = r + 8 * n + 4 * j;
            for (int q = 0; q < 3; ++q) x[q] = root[q] + float(j) * seg * nrm[q];
            x[3] = 1.0f;
            v[0] = v[1] = v[2] = v[3] = 0.0f;
            cc[0] = cc[1] = cc[2] = cc[3] = 0.0f;
        }
    }
    if (params) {
        rvh_sim_params_reference(params);
        params->dftl_damping = d->dftl_damping > 0.f ? d->dftl_damping : params->dftl_damping;
        params->friction = d->friction;
        params->repulsion = d->repulsion;
        params->grid_wrap32 = 0;
        if (d->grid_res > 0) {
            const double half = R + d->length_max + 0.05;
            params->grid_enabled = 1;
            params->grid_dims[0] = params->grid_dims[1] = params->grid_dims[2] = d->grid_res;
            params->grid_h = float(2.0 * half / d->grid_res);
            params->grid_origin[0] = float(c.x - half);
            params->grid_origin[1] = float(c.y - half);
            params->grid_origin[2] = float(c.z - half);
        } else {
            params->grid_enabled = 0;
        }
    }
    int k = 0;
    if (colliders) {
        if (d->head_collider) {
            const float ctr[3] = {float(c.x), float(c.y), float(c.z)};
            const float rot[3] = {0.f, 0.f, 0.f}, one[3] = {1.f, 1.f, 1.f};
            rvh_collider_from_trs(ctr, rot, one, RVH_COLLIDER_SPHERE, float(R), &colliders[k++]);
        }
        Rng er(d->seed ^ 0x5deece66dull);
        for (int e = 0; e < d->n_ellipsoids; ++e) {
            // around the head, from the equator down to the shoulders
            const double phi = 2.0 * kPi * er.uniform();
            const double el = er.range(-0.9, 0.2);
            const double dist = R * er.range(1.0, 1.5);
            const double ce = std::cos(el);
            const float ctr[3] = {float(c.x + dist * ce * std::cos(phi)), float(c.y + dist * std::sin(el)),
                                  float(c.z + dist * ce * std::sin(phi))};
            const float rot[3] = {float(er.range(0.0, 360.0)), float(er.range(0.0, 360.0)), float(er.range(0.0, 360.0))};
            const float ax[3] = {float(er.range(d->axis_min, d->axis_max)), float(er.range(d->axis_min, d->axis_max)),
                                 float(er.range(d->axis_min, d->axis_max))};
            rvh_status st = rvh_collider_from_trs(ctr, rot, ax, RVH_COLLIDER_ELLIPSOID, 1.0f, &colliders[k++]);
            if (st != RVH_OK) return st;
        }
    }
    if (n_colliders) *n_colliders = colliders ? k : 0;
    return RVH_OK;
}

}  // extern "C"
