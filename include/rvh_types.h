/*
 * rvh_types.h — plain-C data types shared by the hair-step C ABI (rvh.h).
 *
 * Every struct here restates a layout that the reference binds to its compute
 * shader (clach/Realtime-Vulkan-Hair, src/shaders/compute.comp) so a caller that
 * already fills those Vulkan buffers can fill these with the same bytes.
 */
#ifndef RVH_TYPES_H
#define RVH_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RVH_ABI_VERSION 1
#define RVH_MAX_COLLIDERS 8   /* reference NUM_COLLIDERS = 6 (compute.comp:8) */
#define RVH_MAX_POINTS 32     /* reference NUM_CURVE_POINTS = 10 (compute.comp:5, Strand.h:9) */
#define RVH_MIN_POINTS 2

typedef int32_t rvh_status;
enum {
    RVH_OK = 0,
    RVH_ERR_INVALID_ARG = 1,
    RVH_ERR_CUDA = 2,
    RVH_ERR_OUT_OF_MEMORY = 3,
    RVH_ERR_BUDGET = 4,       /* HBM admission budget would be exceeded */
    RVH_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    RVH_ERR_STATE = 6,        /* call not valid in the object's current state */
    RVH_ERR_UNSUPPORTED = 7,
    RVH_ERR_NO_DEVICE = 8
};

enum { RVH_COLLIDER_SPHERE = 0, RVH_COLLIDER_ELLIPSOID = 1 };

enum {
    RVH_MEM_HOST = 0,            /* records are copied from host memory */
    RVH_MEM_DEVICE = 1,          /* records are copied from a device pointer */
    RVH_MEM_DEVICE_BORROWED = 2  /* the caller's device buffer is used in place (zero copy) */
};

/*
 * One collider: the three column-major mat4 of `struct Collider`
 * (src/Scene.h:23-27, GLSL compute.comp:25-29), plus its kind.
 *   sphere    — centre = transform[12..14] (transform[3].xyz), `radius`
 *               (compute.comp:160-169 hard-codes radius 1.0 for colliders[0]);
 *   ellipsoid — inside test / surface point / normal of compute.comp:64-79.
 */
typedef struct rvh_collider {
    float transform[16];
    float inv[16];
    float inv_trans[16];
    int32_t kind;
    float radius;
    int32_t attach_to_head;   /* 1: moves with the asset's head (rvh_asset_set_head_transform) */
    int32_t reserved;
} rvh_collider;

/*
 * Simulation constants. The reference hard-codes each one in the shader; the
 * citation gives the value rvh_sim_params_reference() fills in.
 */
typedef struct rvh_sim_params {
    float gravity[3];       /* (0,-9.8,0)   compute.comp:150 */
    float damping;          /* 0.998        compute.comp:7,197 (velocity damping) */
    float dftl_damping;     /* 0.998        compute.comp:7,201 (correction-vector factor) */
    float vmax;             /* 10           compute.comp:198-200 */
    float k_penalty;        /* 1900         compute.comp:163,173 */
    float friction;         /* 0.08         compute.comp:296 */
    float repulsion;        /* 0            extension: density-gradient push (absent in the reference) */
    float grid_scale;       /* 1e6          compute.comp:11 (fixed-point SCALE) */
    int32_t grid_enabled;   /* 1            the reference always splats and gathers */
    int32_t grid_wrap32;    /* 1            sums wrap as int32, like GridCell's ivec3/int (Scene.h:42-50) */
    float grid_origin[3];   /* (-3,-2,-5)   compute.comp:206 */
    float grid_h;           /* 7/64         compute.comp:205 */
    int32_t grid_dims[3];   /* 64,64,64     compute.comp:9 */
    int32_t reserved;
} rvh_sim_params;

/* Per-frame inputs: `struct Time` (src/Scene.h:16-19) plus a wind acceleration. */
typedef struct rvh_frame {
    float dt;        /* Time.deltaTime */
    float t;         /* Time.totalTime */
    float wind[3];   /* added to gravity before the collider term (extension; 0 = reference) */
    int32_t reserved;
} rvh_frame;

/* `struct StrandDrawIndirect` (src/Strand.h:53-58); the step writes vertexCount. */
typedef struct rvh_draw_indirect {
    uint32_t vertex_count;
    uint32_t instance_count;
    uint32_t first_vertex;
    uint32_t first_instance;
} rvh_draw_indirect;

#ifdef __cplusplus
}
#endif
#endif /* RVH_TYPES_H */
