/*
 * rvh_scene.h — seeded synthetic heads and per-frame scene inputs.
 *
 * The reference builds one asset from an OBJ scalp (src/Strand.cpp:26-146,
 * srand(8) at :88) and animates one sphere collider from the keyboard
 * (src/main.cpp:133-157, Scene::translateSphere src/Scene.cpp:110-135).  These
 * helpers build the synthetic stand-ins the benchmarks and tests use, with a
 * counter-based RNG (SplitMix64) so every host produces the same bytes.
 */
#ifndef RVH_SCENE_H
#define RVH_SCENE_H

#include "rvh_types.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { RVH_ROOTS_UNIFORM = 0, RVH_ROOTS_POISSON = 1 };

typedef struct rvh_head_desc {
    uint64_t seed;
    int32_t n_strands;
    int32_t n_points;
    float head_radius;          /* the head is a sphere; roots lie on its upper hemisphere */
    float head_center[3];
    int32_t root_sampling;      /* RVH_ROOTS_UNIFORM or RVH_ROOTS_POISSON (dart throwing) */
    int32_t sort_roots;         /* 1 = order strands along a Morton curve of the root (locality) */
    float length_min;           /* strand length ~ U(length_min, length_max); rest = length/(n-1) */
    float length_max;
    int32_t head_collider;      /* 1 = the head sphere is collider 0 */
    int32_t n_ellipsoids;       /* random ellipsoid colliders near the head */
    float axis_min;             /* ellipsoid semi-axes ~ U(axis_min, axis_max) */
    float axis_max;
    int32_t grid_res;           /* hair-hair grid resolution per axis over the hair AABB; 0 = no grid */
    float friction;
    float repulsion;
    float dftl_damping;
} rvh_head_desc;

/* Fills Strand records (straight strands along the root normal, v = 0,
 * correction = 0), per-strand rest lengths, simulation params (reference
 * constants overridden by the desc) and up to RVH_MAX_COLLIDERS colliders. */
rvh_status rvh_generate_head(const rvh_head_desc* d, void* records, float* rest, rvh_sim_params* params,
                             rvh_collider* colliders, int32_t* n_colliders);

/* Wind acceleration of one frame: amp*sin(omega*t)*dir + gust, gust ~ N(0, sigma^2 I)
 * drawn from (seed, step). */
typedef struct rvh_wind_desc {
    float amplitude;
    float omega;
    float dir[3];
    float gust_sigma;
    uint64_t seed;
} rvh_wind_desc;
rvh_status rvh_wind_at(const rvh_wind_desc* w, int64_t step, float t, float out[3]);

/* A sphere collider whose centre moves on a horizontal circle:
 * centre(t) = (cx + R cos(omega t + phase), y, cz + R sin(omega t + phase)). */
typedef struct rvh_orbit {
    float center[3];
    float orbit_radius;
    float omega;
    float phase;
    float sphere_radius;
} rvh_orbit;
rvh_status rvh_sphere_on_orbit(const rvh_orbit* o, float t, rvh_collider* out);

/* ---- scalp meshes and root sampling (src/Strand.cpp:26-146) ------------------
 * A mesh is a list of triangles in the reference's flattened face-vertex form
 * (triangle t: corners 3t..3t+2, each a position and a normal; Strand.cpp:55-84). */
typedef struct rvh_mesh rvh_mesh;

/* Reads an OBJ file (v, vn, f; other statements are ignored) and triangulates
 * every polygon with the ear-clipping rule of the reference's loader
 * (tiny_obj_loader 2.0, src/tiny_obj_loader.h:1328-1560), so triangle t is the
 * reference's triangle t.  Replaces tinyobj::LoadObj + the flattening loop of
 * GeneratePointsOnMesh (src/Strand.cpp:35-84).  A corner without a normal gets
 * the triangle's geometric normal (the reference reads out of bounds there).
 * A bad index is RVH_ERR_INVALID_ARG (the reference exits, Strand.cpp:45-47). */
rvh_status rvh_mesh_load_obj(const char* path, rvh_mesh** out);
/* A mesh from face-vertex arrays: 9 floats of positions and 9 of normals per triangle. */
rvh_status rvh_mesh_from_triangles(const float* positions, const float* normals, int32_t n_triangles, rvh_mesh** out);
void rvh_mesh_destroy(rvh_mesh* m);
/* Triangle count and total area (either pointer may be NULL). */
rvh_status rvh_mesh_info(const rvh_mesh* m, int32_t* n_triangles, double* area);
/* Copies the face-vertex arrays out (9 floats per triangle each; either may be NULL). */
rvh_status rvh_mesh_triangles(const rvh_mesh* m, float* positions, float* normals);

enum {
    RVH_MESH_ROOTS_REFERENCE = 0,   /* triangle-uniform on glibc rand() seeded with `seed` (the reference: srand(8)) */
    RVH_MESH_ROOTS_AREA = 1         /* area-uniform, SplitMix64 stream of `seed` */
};
enum {
    RVH_ROOT_NORMAL_FIRST_CORNER = 0,   /* the triangle's first corner normal (the reference, Strand.cpp:97) */
    RVH_ROOT_NORMAL_INTERPOLATED = 1    /* barycentric blend of the corner normals, normalized */
};
typedef struct rvh_mesh_roots_desc {
    int32_t mode;          /* RVH_MESH_ROOTS_* */
    int32_t n_roots;
    uint64_t seed;
    int32_t normal_mode;   /* RVH_ROOT_NORMAL_* */
    int32_t reserved;
} rvh_mesh_roots_desc;

/* Samples n_roots hair roots (3 floats each) and their normals on the mesh.
 * RVH_MESH_ROOTS_REFERENCE with seed 8 and RVH_ROOT_NORMAL_FIRST_CORNER gives
 * the bits of GeneratePointsOnMesh (src/Strand.cpp:88-110): triangle =
 * rand() % n_triangles, u, v = rand() / (float)RAND_MAX folded when
 * u + v >= 1, root = p1*u + p2*v + p3*(1-u-v).  Feed the result to
 * rvh_init_strands_reference to get Hair::Hair's strands. */
rvh_status rvh_mesh_sample_roots(const rvh_mesh* m, const rvh_mesh_roots_desc* d, float* roots, float* normals);

/* The first n values of glibc's rand() after srand(seed), from this library's
 * own restatement of that generator (the reference-mode sampler uses it). */
rvh_status rvh_libc_rand_sequence(uint32_t seed, int32_t n, int32_t* out);

/* Deterministic stream helpers (SplitMix64), exposed so tests draw the same numbers. */
uint64_t rvh_rng_u64(uint64_t seed, uint64_t counter);
double rvh_rng_uniform(uint64_t seed, uint64_t counter);   /* [0, 1) */
double rvh_rng_normal(uint64_t seed, uint64_t counter);    /* N(0, 1), Box-Muller on two draws */

#ifdef __cplusplus
}
#endif
#endif /* RVH_SCENE_H */
