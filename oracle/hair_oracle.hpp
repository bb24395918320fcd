/*
 * hair_oracle.hpp — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference hair-physics compute shader
 * (clach/Realtime-Vulkan-Hair, src/shaders/compute.comp:124-303), templated on the
 * scalar type: T = double is the FP64 oracle every GPU result is checked against,
 * T = float is its FP32 twin (same operation order) that separates FP32 rounding
 * from bugs.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use it.
 *
 * Semantics follow the shader line by line, with the deliberate definitions below
 * where the reference is ill-defined or hard-coded:
 *   - one grid per asset and a GLOBAL phase split: every strand runs loops 1+2
 *     (predict/collide/FTL, then DFTL + splat) before any strand runs loop 3
 *     (gather + friction).  The shader's barrier() is workgroup-only
 *     (compute.comp:209,255), so its cross-workgroup order is undefined;
 *   - exactly n_strands strands (the dispatch at src/Renderer.cpp:2070 runs
 *     out-of-range invocations; they are dropped);
 *   - constants become rvh_sim_params fields (reference values in rvh_types.h);
 *     n_points and the per-strand rest length are runtime values
 *     (compute.comp:5,139-140 hard-code 10 points and length 2.5);
 *   - colliders carry a kind: compute.comp:160-169 treats colliders[0] as a
 *     sphere of radius 1.0 and the rest as ellipsoids (:170-178);
 *   - grid sums are exact int64; with grid_wrap32 they are read back as wrapped
 *     int32, which equals the shader's wrapping int32 atomicAdd (:245-248);
 *   - extensions that are zero in reference mode: wind (force += wind, before
 *     the collider term; the shader's wind is commented out at :151-152), a
 *     per-strand wind, and repulsion (density-gradient push in loop 3).
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/rvh_types.h"

namespace oracle {

template <class T>
struct v3 {
    T x, y, z;
};
template <class T> inline v3<T> mk(T x, T y, T z) { return {x, y, z}; }
template <class T> inline v3<T> operator+(v3<T> a, v3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline v3<T> operator-(v3<T> a, v3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline v3<T> operator*(T s, v3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline v3<T> operator*(v3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline v3<T> operator/(v3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot(v3<T> a, v3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(v3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline T distance(v3<T> a, v3<T> b) { return length(a - b); }
/* GLSL normalize(x) = x * inversesqrt(dot(x, x)). */
template <class T> inline v3<T> normalize(v3<T> a) { return a * (T(1) / std::sqrt(dot(a, a))); }

/* xyz of (m * vec4(p, w)) for a column-major float mat4 (GLSL convention),
 * summed as (c0*x + c1*y) + (c2*z + c3*w). */
template <class T>
inline v3<T> mat_xyz(const float* m, v3<T> p, T w) {
    return {(T(m[0]) * p.x + T(m[4]) * p.y) + (T(m[8]) * p.z + T(m[12]) * w),
            (T(m[1]) * p.x + T(m[5]) * p.y) + (T(m[9]) * p.z + T(m[13]) * w),
            (T(m[2]) * p.x + T(m[6]) * p.y) + (T(m[10]) * p.z + T(m[14]) * w)};
}

/* A 4-component slot of the Strand record. */
template <class T> inline v3<T> ld(const T* q) { return {q[0], q[1], q[2]}; }
template <class T> inline void st(T* q, v3<T> a, T w) { q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = w; }

/* Grid: 4 int64 per cell {vx, vy, vz, density}, cell index a + b*nx + c*nx*ny
 * (compute.comp:234 with GRID_DIM generalised per axis). */
struct Grid {
    int nx = 0, ny = 0, nz = 0;
    std::vector<int64_t> cells;
    void reset(const rvh_sim_params& p) {
        nx = p.grid_dims[0]; ny = p.grid_dims[1]; nz = p.grid_dims[2];
        cells.assign(size_t(nx) * ny * nz * 4, 0);
    }
};

/* Corner range of one axis (compute.comp:224-229).  floor() is clamped to
 * [-2, dim] before the int conversion; that keeps the conversion defined and
 * leaves the (possibly empty) range unchanged. */
template <class T>
inline void corner_range(T g, int dim, int& lo, int& hi) {
    T f = std::floor(g);
    f = std::min(std::max(f, T(-2)), T(dim));
    const int fi = int(f);
    lo = std::max(fi, 0);
    hi = std::min(fi + 1, dim - 1);
}

template <class T>
inline T tri_weight(T g, int a) {  /* clamp(1 - abs(g - a), 0, 1)  compute.comp:237-239 */
    return std::min(std::max(T(1) - std::abs(g - T(a)), T(0)), T(1));
}

/* Truncating float->int conversion of one contribution, int(SCALE * x) (compute.comp:245-248). */
template <class T>
inline int64_t fixed(T scale, T x) {
    const T y = scale * x;
    return int64_t(int32_t(y));
}

inline int64_t grid_read(const int64_t* c, int k, bool wrap32) {
    return wrap32 ? int64_t(int32_t(uint32_t(uint64_t(c[k])))) : c[k];
}

/*
 * Loops 1 and 2 for one strand (compute.comp:144-202 and :211-216).
 * rec = 12*n scalars: curvePoints[n], curveVels[n], correctionVecs[n] (Strand.h:11-15).
 * force0 = gravity + frame wind + per-strand wind.
 */
template <class T>
void strand_predict(T* rec, int n, T radius, v3<T> force0, const rvh_collider* cols, int ncol,
                    const rvh_sim_params& P, T dt) {
    T* X = rec;
    T* V = rec + 4 * n;
    T* C = rec + 8 * n;
    const T k = T(P.k_penalty);
    const T damping = T(P.damping), dftl = T(P.dftl_damping), vmax = T(P.vmax);
    for (int i = 1; i < n; i++) {                      /* :144 */
        const v3<T> currentPos = ld(X + 4 * i);        /* :145 */
        const v3<T> currentVel = ld(V + 4 * i);        /* :146 */
        const v3<T> parentPos = ld(X + 4 * (i - 1));   /* :147, parent already moved this step */
        v3<T> force = force0;                          /* :150 (+ wind extension) */
        int numColliders = 0;                          /* :155 */
        v3<T> addedForce = mk<T>(0, 0, 0);
        for (int j = 0; j < ncol; j++) {               /* :158 */
            const rvh_collider& c = cols[j];
            if (c.kind == RVH_COLLIDER_SPHERE) {       /* :160-169 */
                const T r = T(c.radius);
                const v3<T> centre = mk(T(c.transform[12]), T(c.transform[13]), T(c.transform[14]));
                if (distance(currentPos, centre) < r) {
                    const T d = r - distance(currentPos, centre);
                    const v3<T> normal = normalize(currentPos - centre);
                    addedForce = addedForce + (k * d) * normal;
                    numColliders++;
                }
            } else {                                   /* :170-178 */
                const v3<T> local = mat_xyz(c.inv, currentPos, T(1));        /* EllipsoidCollision :64-67 */
                if (length(local) <= T(1)) {
                    const v3<T> onSurf = mat_xyz(c.transform, normalize(local), T(1)); /* :76-79 */
                    const T d = distance(onSurf, currentPos);
                    const v3<T> nrm = normalize(mat_xyz(c.inv_trans, local, T(0))); /* :70-73 */
                    const v3<T> normal = normalize(nrm);                            /* :175 */
                    addedForce = addedForce + (k * d) * normal;
                    numColliders++;
                }
            }
        }
        if (numColliders > 0) force = force + addedForce / T(numColliders);   /* :182-184 */
        const v3<T> predictedPos = currentPos + dt * currentVel + (dt * dt) * force;  /* :187 */
        const v3<T> direction = normalize(predictedPos - parentPos);                  /* :191 */
        const v3<T> newPos = parentPos + radius * direction;                          /* :192 */
        const v3<T> newVel = (newPos - currentPos) / dt;                              /* :195 */
        st(X + 4 * i, newPos, T(1));                                                  /* :196 */
        v3<T> vel = damping * newVel;                                                 /* :197 */
        if (length(vel) > vmax) vel = normalize(vel) * vmax;                          /* :198-200 */
        st(V + 4 * i, vel, T(0));
        st(C + 4 * i, dftl * (newPos - predictedPos), T(0));                          /* :201 */
    }
    for (int i = 1; i < n; ++i) {                                                     /* :211 */
        if (i != n - 1) {                                                             /* :213-215 */
            const v3<T> v = ld(V + 4 * i) - ld(C + 4 * (i + 1)) / dt;
            st(V + 4 * i, v, V[4 * i + 3]);
        }
    }
}

/* Trilinear splat of one point into the grid (compute.comp:217-252). */
template <class T, bool ATOMIC>
void splat_point(Grid& G, const rvh_sim_params& P, v3<T> pos, v3<T> vel) {
    const T h = T(P.grid_h);
    const v3<T> origin = mk(T(P.grid_origin[0]), T(P.grid_origin[1]), T(P.grid_origin[2]));
    const T x = (pos.x - origin.x) / h, y = (pos.y - origin.y) / h, z = (pos.z - origin.z) / h;
    int xmin, xmax, ymin, ymax, zmin, zmax;
    corner_range(x, G.nx, xmin, xmax);
    corner_range(y, G.ny, ymin, ymax);
    corner_range(z, G.nz, zmin, zmax);
    const T scale = T(P.grid_scale);
    for (int a = xmin; a <= xmax; ++a)
        for (int b = ymin; b <= ymax; ++b)
            for (int c = zmin; c <= zmax; ++c) {
                const size_t index = size_t(a) + size_t(b) * G.nx + size_t(c) * G.nx * G.ny;
                const T totalWeight = tri_weight(x, a) * tri_weight(y, b) * tri_weight(z, c);
                const v3<T> wv = totalWeight * vel;
                const int64_t add[4] = {fixed(scale, wv.x), fixed(scale, wv.y), fixed(scale, wv.z),
                                        fixed(scale, totalWeight)};
                int64_t* cell = &G.cells[index * 4];
                for (int q = 0; q < 4; ++q) {
                    if (ATOMIC) __atomic_fetch_add(cell + q, add[q], __ATOMIC_RELAXED);
                    else cell[q] += add[q];
                }
            }
}

/* Loop 3 for one point: gather + friction (compute.comp:258-297), plus the
 * repulsion extension when P.repulsion != 0:
 *   rho  = sum_c w_c * dens_c/scale,  grad = sum_c grad(w_c) * dens_c/scale
 *   v   += -repulsion * (h/dt) * grad / max(rho, 1)
 * over the same corners and the same density > 0 test; grad(w_c) is the
 * derivative of the trilinear weight in grid units, d/dg clamp(1-|g-a|,0,1) =
 * -1 for g >= a, +1 for g < a, inside |g-a| < 1. */
template <class T>
v3<T> gather_point(const Grid& G, const rvh_sim_params& P, v3<T> pos, v3<T> vel, T dt) {
    const T h = T(P.grid_h);
    const v3<T> origin = mk(T(P.grid_origin[0]), T(P.grid_origin[1]), T(P.grid_origin[2]));
    const T x = (pos.x - origin.x) / h, y = (pos.y - origin.y) / h, z = (pos.z - origin.z) / h;
    int xmin, xmax, ymin, ymax, zmin, zmax;
    corner_range(x, G.nx, xmin, xmax);
    corner_range(y, G.ny, ymin, ymax);
    corner_range(z, G.nz, zmin, zmax);
    const bool wrap = P.grid_wrap32 != 0;
    const bool rep = P.repulsion != 0.0f;
    const T scale = T(P.grid_scale);
    v3<T> gridVelocity = mk<T>(0, 0, 0);
    T rho = 0;
    v3<T> grad = mk<T>(0, 0, 0);
    for (int a = xmin; a <= xmax; ++a)
        for (int b = ymin; b <= ymax; ++b)
            for (int c = zmin; c <= zmax; ++c) {
                const size_t index = size_t(a) + size_t(b) * G.nx + size_t(c) * G.nx * G.ny;
                const int64_t* cell = &G.cells[index * 4];
                const int64_t density = grid_read(cell, 3, wrap);
                if (density > 0) {
                    const T wx = tri_weight(x, a), wy = tri_weight(y, b), wz = tri_weight(z, c);
                    const T totalWeight = wx * wy * wz;
                    const v3<T> gv = mk(T(grid_read(cell, 0, wrap)), T(grid_read(cell, 1, wrap)),
                                        T(grid_read(cell, 2, wrap)));
                    gridVelocity = gridVelocity + (totalWeight * (T(1) / T(density))) * gv;
                    if (rep) {
                        const T rc = T(density) / scale;
                        const T dx = (std::abs(x - T(a)) < T(1)) ? (x >= T(a) ? T(-1) : T(1)) : T(0);
                        const T dy = (std::abs(y - T(b)) < T(1)) ? (y >= T(b) ? T(-1) : T(1)) : T(0);
                        const T dz = (std::abs(z - T(c)) < T(1)) ? (z >= T(c) ? T(-1) : T(1)) : T(0);
                        rho += totalWeight * rc;
                        grad = grad + rc * mk(dx * wy * wz, wx * dy * wz, wx * wy * dz);
                    }
                }
            }
    const T friction = T(P.friction);
    v3<T> out = (T(1) - friction) * vel + friction * gridVelocity;            /* :296-297 */
    if (rep) out = out - (T(P.repulsion) * (h / dt) / std::max(rho, T(1))) * grad;
    return out;
}

/* The effective constant force of one strand: gravity + frame wind + strand wind. */
template <class T>
inline v3<T> base_force(const rvh_sim_params& P, const rvh_frame& F, const float* strand_wind, int s) {
    v3<T> f = mk(T(P.gravity[0]), T(P.gravity[1]), T(P.gravity[2]));
    f = f + mk(T(F.wind[0]), T(F.wind[1]), T(F.wind[2]));
    if (strand_wind) f = f + mk(T(strand_wind[3 * s]), T(strand_wind[3 * s + 1]), T(strand_wind[3 * s + 2]));
    return f;
}

/*
 * One full step of one asset (the per-frame clear + dispatch of
 * src/Renderer.cpp:2063-2071, with a global splat/gather split).
 * state: n_strands * 12 * n scalars.  threads > 1 runs strands in parallel with
 * OpenMP; int64 sums make the result independent of the thread count.
 */
/* Kinematic head (no counterpart in the reference, whose roots stay where
 * Hair::Hair put them): root = head * (root_rest, 1) for a column-major 4x4
 * affine head, each row summed as ((m0 x + m1 y) + m2 z) + m3. */
template <class T>
inline v3<T> head_point(const float* m, const float* r) {
    const T x = T(r[0]), y = T(r[1]), z = T(r[2]);
    v3<T> o;
    o.x = ((T(m[0]) * x + T(m[4]) * y) + T(m[8]) * z) + T(m[12]);
    o.y = ((T(m[1]) * x + T(m[5]) * y) + T(m[9]) * z) + T(m[13]);
    o.z = ((T(m[2]) * x + T(m[6]) * y) + T(m[10]) * z) + T(m[14]);
    return o;
}

template <class T>
void step_asset(T* state, int ns, int n, const float* rest, const float* strand_wind,
                const rvh_sim_params& P, const rvh_frame& F, const rvh_collider* cols, int ncol,
                Grid& G, int threads, const float* head = nullptr, const float* root_rest = nullptr) {
    const T dt = T(F.dt);
    const bool grid = P.grid_enabled != 0;
    if (grid) G.reset(P);
    const size_t stride = size_t(12) * n;
    (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (int s = 0; s < ns; ++s) {
        T* rec = state + stride * s;
        if (head) st(rec, head_point<T>(head, root_rest + 3 * size_t(s)), T(1));
        strand_predict<T>(rec, n, T(rest[s]), base_force<T>(P, F, strand_wind, s), cols, ncol, P, dt);
        if (grid) {
            for (int i = 1; i < n; ++i) {
                if (threads > 1) splat_point<T, true>(G, P, ld(rec + 4 * i), ld(rec + 4 * n + 4 * i));
                else splat_point<T, false>(G, P, ld(rec + 4 * i), ld(rec + 4 * n + 4 * i));
            }
        }
    }
    if (!grid) return;
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
    for (int s = 0; s < ns; ++s) {
        T* rec = state + stride * s;
        for (int i = 1; i < n; ++i) {                                          /* :257 */
            const v3<T> v = gather_point<T>(G, P, ld(rec + 4 * i), ld(rec + 4 * n + 4 * i), dt);
            st(rec + 4 * n + 4 * i, v, T(0));
        }
    }
}

/*
 * One step of a group of assets sharing one grid (the reference clears one
 * Scene-owned grid and dispatches every hair into it, src/Renderer.cpp:2063-2071,
 * src/Scene.h:75-77).  The reference orders nothing between the dispatches; here
 * every member's loops 1-2 and splat come before any member's loop 3, as within
 * one asset (step_asset).  The grid geometry is the first member's (the members
 * share it); each member gathers with its own friction and repulsion.
 */
template <class T>
struct GroupMember {
    T* state;
    int ns, n;
    const float* rest;
    const rvh_sim_params* P;
};

template <class T>
void step_group(GroupMember<T>* m, int nm, const rvh_frame& F, const rvh_collider* cols, int ncol, Grid& G) {
    if (nm < 1) return;
    const T dt = T(F.dt);
    G.reset(*m[0].P);
    for (int k = 0; k < nm; ++k) {
        const size_t stride = size_t(12) * m[k].n;
        for (int s = 0; s < m[k].ns; ++s) {
            T* rec = m[k].state + stride * s;
            strand_predict<T>(rec, m[k].n, T(m[k].rest[s]), base_force<T>(*m[k].P, F, nullptr, s), cols, ncol,
                              *m[k].P, dt);
            for (int i = 1; i < m[k].n; ++i) splat_point<T, false>(G, *m[k].P, ld(rec + 4 * i), ld(rec + 4 * m[k].n + 4 * i));
        }
    }
    for (int k = 0; k < nm; ++k) {
        const size_t stride = size_t(12) * m[k].n;
        for (int s = 0; s < m[k].ns; ++s) {
            T* rec = m[k].state + stride * s;
            for (int i = 1; i < m[k].n; ++i) {
                const v3<T> v = gather_point<T>(G, *m[k].P, ld(rec + 4 * i), ld(rec + 4 * m[k].n + 4 * i), dt);
                st(rec + 4 * m[k].n + 4 * i, v, T(0));
            }
        }
    }
}

}  // namespace oracle
