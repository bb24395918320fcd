/*
 * rvh.h — C ABI of the GB300 hair-physics step.
 *
 * A drop-in for the hair simulation of clach/Realtime-Vulkan-Hair: the
 * reference runs it as one Vulkan compute shader (src/shaders/compute.comp)
 * over a `Strand[]` storage buffer, recorded once and submitted every frame.
 * Here the same buffer layout (float4 curvePoints[n], curveVels[n],
 * correctionVecs[n] per strand, src/Strand.h:11-15) lives in HBM and each
 * call below replaces one piece of that Vulkan plumbing (cited per entry).
 *
 * Conventions: every call returns rvh_status (RVH_OK = 0); no C++ exception
 * crosses the ABI; rvh_last_error() gives a message for the calling thread.
 * Stream arguments are cudaStream_t passed as void* (NULL = the context's own
 * stream).  Work is asynchronous on its stream unless stated otherwise.
 * One GPU per context.
 */
#ifndef RVH_H
#define RVH_H

#include "rvh_scene.h"
#include "rvh_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rvh_context rvh_context;
typedef struct rvh_asset rvh_asset;
typedef struct rvh_batch rvh_batch;
typedef struct rvh_server rvh_server;

enum { RVH_MATH_FAST = 0, RVH_MATH_EXACT = 1 };

typedef struct rvh_context_desc {
    int32_t device;               /* CUDA device ordinal */
    int32_t math;                 /* RVH_MATH_FAST, or RVH_MATH_EXACT: separately rounded IEEE ops in
                                     the oracle's order (bit-identical to the FP32 restatement) */
    uint64_t hbm_budget_bytes;    /* admission budget for everything the context allocates; 0 = 90% of free */
} rvh_context_desc;

typedef struct rvh_asset_desc {
    int32_t n_strands;
    int32_t n_points;             /* curve points per strand, 2..32 (reference NUM_CURVE_POINTS = 10) */
    const void* strands;          /* n_strands Strand records, 48*n_points bytes each */
    int32_t strands_location;     /* RVH_MEM_HOST / RVH_MEM_DEVICE / RVH_MEM_DEVICE_BORROWED */
    float uniform_rest_length;    /* used when rest_lengths is NULL (reference 2.5/(n-1), compute.comp:139-140) */
    const float* rest_lengths;    /* optional host array: rest segment length per strand */
    const float* strand_wind;     /* optional host array: wind acceleration per strand (3 floats) */
    int32_t lanes_per_strand;     /* 0 = by point count: 1 up to 10 points, 2 up to 16, 8 above (or the next
                                     compiled count); else 1,2,4,8,16,32 (strands per warp = 32/lanes) */
    int32_t reserved;
} rvh_asset_desc;

/* ---- context --------------------------------------------------------------
 * Replaces the Instance / Device / queue set-up (src/main.cpp:164-184,
 * src/Device.h:13-17) for the compute half. */
rvh_status rvh_context_create(const rvh_context_desc* desc, rvh_context** out);
rvh_status rvh_context_destroy(rvh_context* ctx);
rvh_status rvh_context_synchronize(rvh_context* ctx);
/* bytes the context has admitted against its budget, and the budget */
rvh_status rvh_context_memory(rvh_context* ctx, uint64_t* used, uint64_t* budget);
const char* rvh_last_error(void);
/* Page-locked host memory (for asynchronous copies). */
rvh_status rvh_pinned_alloc(size_t bytes, void** out);
rvh_status rvh_pinned_free(void* p);
const char* rvh_status_string(rvh_status s);
int32_t rvh_abi_version(void);

/* ---- parameter helpers ------------------------------------------------------ */
/* The constants compute.comp hard-codes (lines cited in rvh_types.h). */
rvh_status rvh_sim_params_reference(rvh_sim_params* out);
/* Collider(trans, rot, scale) of src/Scene.h:28-39: transform = T*Rz*Ry*Rx*S
 * (rotation in degrees), inv, invTrans; kind/radius as given. */
rvh_status rvh_collider_from_trs(const float trans[3], const float rot_deg[3], const float scale[3],
                                 int32_t kind, float radius, rvh_collider* out);
/* Scene::translateSphere (src/Scene.cpp:110-120): transform = transform *
 * translate(delta); inv and invTrans recomputed. */
rvh_status rvh_collider_translate(rvh_collider* c, const float delta[3]);
/* A collider carried by a rigid head motion m (column-major 4x4 affine, glm
 * layout): transform = m * rest.transform, inv = inverse(transform), inv_trans =
 * transpose(inv), computed in double and rounded once.  Scene::translateSphere
 * (src/Scene.cpp:110-120) is the special case m = translate(delta) applied on
 * the right; this is the head-follows-motion form the asset uses for colliders
 * with attach_to_head set. */
rvh_status rvh_collider_follow(const rvh_collider* rest, const float m[16], rvh_collider* out);
/* Initial straight strands as Hair::Hair builds them (src/Strand.cpp:157-175):
 * point j = root + j*seg*(normal + dir_offset), velocity (0,0,-1), correction 0.
 * The reference uses seg = 2.5/9 and dir_offset = (0.05, 5, -2). */
rvh_status rvh_init_strands_reference(const float* roots, const float* normals, int32_t n_strands,
                                      int32_t n_points, float seg, const float dir_offset[3], void* out_records);

/* ---- assets -----------------------------------------------------------------
 * Replaces Hair::Hair's buffer creation (src/Strand.cpp:186-191,
 * BufferUtils::CreateBufferFromData, src/BufferUtils.cpp:68-94) and the
 * per-asset descriptor set 4 (src/Renderer.cpp:836-997). */
rvh_status rvh_asset_create(rvh_context* ctx, const rvh_asset_desc* desc, rvh_asset** out);
rvh_status rvh_asset_destroy(rvh_asset* a);
/* Time/Collider/Grid uniforms of sets 1-3 (compute.comp:20-42, Scene.cpp:4-20). */
rvh_status rvh_asset_set_params(rvh_asset* a, const rvh_sim_params* p);
rvh_status rvh_asset_set_colliders(rvh_asset* a, const rvh_collider* c, int32_t n);
/* Grid groups: the reference clears ONE Scene-owned grid and dispatches every
 * hair into it (src/Renderer.cpp:2063-2071, src/Scene.h:75-77), so hair-hair
 * friction couples the hairs of a frame.  rvh_asset_share_grid(a, owner) makes
 * `a` splat into and gather from owner's grid: both need the grid enabled with
 * the same dims, origin, cell size, scale and wrap mode; `a` must share no grid
 * yet and `owner` must not share another asset's.  `a`'s pending friction is
 * applied and its own grids are released.  A group is stepped by a batch that
 * holds all of its assets, in fused steps: every member's loops 1-2 and splat
 * come before any member's loop 3 (the reference orders nothing between its
 * dispatches).  rvh_step, full-step batches and request servers refuse group
 * members (RVH_ERR_STATE / RVH_ERR_UNSUPPORTED), and set_params may not change
 * a member's grid geometry.  owner = NULL takes `a` out of its group (friction
 * applied, grids of its own again); an owner leaves only after its members.
 * Destroying an owner gives its members grids of their own. */
rvh_status rvh_asset_share_grid(rvh_asset* a, rvh_asset* owner);
/* Kinematic head: the pose m (column-major 4x4 affine) of the asset's head for
 * the following steps, relative to its pose when head motion was first set.
 * Each step then places every strand's root at m * root_rest (root_rest = the
 * roots at that first call; the reference pins them where Hair::Hair put them,
 * compute.comp:144 starts at point 1) before the FTL chain, and uses
 * rvh_collider_follow(c, m) for each collider with attach_to_head set.  In the
 * reference only collider 0 and the head model move, by keyboard translations
 * (Scene::translateSphere, src/Scene.cpp:110-135; src/main.cpp:133-157); here
 * the roots and the attached colliders move together, so hair follows its
 * head.  m = NULL stops the motion (roots stay where the last step put them). */
rvh_status rvh_asset_set_head_transform(rvh_asset* a, const float m[16]);
/* Per-strand rest segment lengths (host array, n_strands floats; the
 * reference's strandLength/(n-1), compute.comp:139-140) and per-strand wind
 * (host array, 3 floats per strand, or NULL to remove it). */
rvh_status rvh_asset_set_rest_lengths(rvh_asset* a, const float* rest);
rvh_status rvh_asset_set_strand_wind(rvh_asset* a, const float* wind3);
/* Device pointer of the Strand records (the VkBuffer Hair::GetStrandsBuffer(), Strand.cpp:195). */
rvh_status rvh_asset_device_ptr(rvh_asset* a, void** out);
/* Device pointer of the StrandDrawIndirect record the step writes (Strand.cpp:199, compute.comp:302). */
rvh_status rvh_asset_draw_indirect(rvh_asset* a, void** out);
rvh_status rvh_asset_strand_count(rvh_asset* a, int32_t* n_strands, int32_t* n_points);
/* Copy records to / from host memory (synchronous). */
rvh_status rvh_asset_read(rvh_asset* a, void* host_dst, size_t bytes);
rvh_status rvh_asset_write(rvh_asset* a, const void* host_src, size_t bytes);
/* Positions only (float4 per point, the curvePoints the renderer reads, hair.vert:9,15),
 * gathered on the device and copied to host memory asynchronously on `stream`. */
rvh_status rvh_asset_read_positions_async(rvh_asset* a, void* host_dst, size_t bytes, void* stream);
/* Copy of the StrandDrawIndirect record (synchronous). */
rvh_status rvh_asset_read_draw(rvh_asset* a, rvh_draw_indirect* out);
/* Last grid sums (4 int64 per cell {vx,vy,vz,density}); synchronous; for tests. */
rvh_status rvh_asset_read_grid(rvh_asset* a, int64_t* host_dst, size_t bytes);

/* ---- the step ---------------------------------------------------------------
 * One Renderer::Frame() compute submit (src/Renderer.cpp:2309-2319) for one
 * asset: clear its grid (vkCmdFillBuffer, Renderer.cpp:2063), phase A
 * (compute.comp:144-253), phase B (:257-298); writes vertexCount (:302).
 * Plain path: one launch sequence per call, no graph. */
rvh_status rvh_step(rvh_asset* a, const rvh_frame* frame, void* stream);

/* ---- the plain step without device allocations ------------------------------
 * No counterpart in the reference.  For callers that cannot let the library
 * allocate device memory (a frame loop where a cudaMalloc could stall the
 * device, or a host application whose own allocator owns all GPU memory):
 * the caller passes every buffer, and the step's only scratch, the hair-hair
 * grid, lives in a static device array of RVH_NOALLOC_MAX_GRID_CELLS cells
 * (8 MiB per GPU that loads the library, held until exit).  Larger grids are
 * rejected with RVH_ERR_INVALID_ARG.  Each call clears the grid cells it
 * uses; calls on one device whose work overlaps on the GPU race on the shared
 * array.  The first call on a device (and the first after its context was
 * torn down, e.g. by cudaDeviceReset) looks up the array's address and should
 * come before any stream capture.  Same results as rvh_step on an asset with
 * the same state, params, colliders and math mode; with n_strands = 0 it only
 * writes the draw record (vertex_count 0). */
#define RVH_NOALLOC_MAX_GRID_CELLS (64 * 64 * 64)
typedef struct rvh_noalloc_step_desc {
    void* strands;                /* device: n_strands Strand records, updated in place */
    const float* rest_lengths;    /* device: n_strands floats */
    const float* strand_wind;     /* device: 4 floats per strand (xyz used), or NULL */
    void* draw_indirect;          /* device: one rvh_draw_indirect to write, or NULL */
    int32_t n_strands;
    int32_t n_points;
    int32_t lanes_per_strand;     /* 0 = default */
    int32_t math;                 /* RVH_MATH_FAST or RVH_MATH_EXACT */
    const rvh_sim_params* params; /* host */
    const rvh_collider* colliders;/* host, n_colliders entries */
    int32_t n_colliders;
    int32_t reserved;
} rvh_noalloc_step_desc;
rvh_status rvh_step_noalloc(const rvh_noalloc_step_desc* desc, const rvh_frame* frame, void* stream);

/* ---- strand tessellation (src/shaders/hair.tesc:19-20, src/shaders/hair.tese) ----
 * The reference's tessellation stages turn each guide strand into isolines of
 * a Bezier curve offset by a clump width (single-strand clumping,
 * hair.tese:153-330).  Without a graphics pipeline the same vertices are
 * written to a device buffer: per strand n_lines isolines of n_segments + 1
 * vertices, each a float4 {position xyz, strand width}, strand-major then
 * isoline-major.  The per-strand hash uses a correctly rounded sin (the
 * shader uses the platform's).  At v = 1 the curve ends at the tip (the shader
 * reads past the strand there). */
typedef struct rvh_tess_desc {
    int32_t n_lines;        /* isolines per strand, 1..64 (gl_TessLevelOuter[0] = 12, hair.tesc:19) */
    int32_t n_segments;     /* segments per isoline, 1..256 (gl_TessLevelOuter[1] = 42, hair.tesc:20) */
    float clump_radius;     /* hair.tese:239: 0.5 */
    float root_width;       /* hair.tese:324: 0.02 */
    float tip_width;        /* hair.tese:325: 0.01 */
    int32_t reserved;
} rvh_tess_desc;
/* The reference's constants. */
rvh_status rvh_tess_desc_reference(rvh_tess_desc* d);
/* Tessellates the asset's current positions on `stream` (NULL: the context's).
 * vertices: device, n_strands * n_lines * (n_segments + 1) float4.
 * frames: device or NULL, n_strands * (n_points - 1) * 3 float4 {tangent, b1,
 * b2} per segment (hair.tese:289-297: normalized segment direction and its
 * Frisvad orthonormal basis).  Both 16-byte aligned. */
rvh_status rvh_asset_tessellate(rvh_asset* a, const rvh_tess_desc* d, void* vertices, void* frames, void* stream);

/* ---- hair shading (src/Renderer.cpp's shadow, opacity and hair passes;
 * src/shaders/hairOpacity.frag, src/shaders/hair.frag) ----------------------
 * The reference draws the tessellated hair three times: into a light-space
 * depth map, into a deep opacity map (three layers of +0.3 per fragment
 * behind the first surface, d = 0.3, 8-bit unorm target with additive
 * blending) and into the framebuffer with hair.frag.  Here each tessellated
 * vertex is a fragment covering one texel (the ribbons are about a texel wide
 * and their vertices about a texel apart at the reference's sizes); the maps
 * and colours go to device buffers.  Matrices are column-major (glm's layout). */
typedef struct rvh_shade_desc {
    float camera_view[16];  /* Camera.cpp:13: lookAt((0, 1, 10), (0, 1, 0), (0, 1, 0)) */
    float camera_proj[16];  /* Camera.cpp:14-15: perspective(45 deg, 1.5, 0.1, 50), y flipped */
    float light_view[16];   /* Camera.cpp:28-30: lookAt(6.5 normalize((2, 0, 1) - (0, 1, 0)), (0, 1, 0), up) */
    float light_proj[16];   /* Camera.cpp:31-32: perspective(60 deg, 1.5, 1, 10), y flipped */
    int32_t map_width;      /* SHADOWMAP_WIDTH = 1080 (Renderer.cpp:9) */
    int32_t map_height;     /* SHADOWMAP_HEIGHT = 720 (Renderer.cpp:10) */
    int32_t map_mode;       /* RVH_SHADE_MAPS_QUADS (reference): the light passes rasterise hair.geom's
                               quads in the light's view; RVH_SHADE_MAPS_VERTICES: each tessellated
                               vertex covers one texel (cheaper) */
    int32_t image_mode;     /* rvh_asset_render_hair: RVH_IMAGE_BLEND (reference): the hair pipeline's
                               in-order alpha blending (Renderer.cpp:1657-1679); RVH_IMAGE_NEAREST: each
                               pixel takes its nearest fragment's colour (cheaper) */
} rvh_shade_desc;
enum { RVH_SHADE_MAPS_VERTICES = 0, RVH_SHADE_MAPS_QUADS = 1 };
enum { RVH_IMAGE_NEAREST = 0, RVH_IMAGE_BLEND = 1 };
/* The reference's cameras and map size (glm's float arithmetic, bit for bit). */
rvh_status rvh_shade_desc_reference(rvh_shade_desc* d);
/* hair.frag for n caller-given fragments (replaces the fragment stage of the
 * reference's hair pipeline, Renderer.cpp:1554-1746, whose fragment shader is
 * hair.frag).
 * inputs: device, n x 24 floats per fragment: in_uv (2), in_u, in_v, in_w (3
 * each), in_viewDir (3), in_lightDir (3), in_fragPosLightSpace (4), 3 unused
 * (hair.frag:14-20).  depth_map: map_width x map_height floats; opacity_map:
 * the same count of float4 (layers r, g, b).  colors: n float4 (outColor).
 * inputs, opacity_map and colors 16-byte aligned. */
rvh_status rvh_shade_fragments(rvh_context* ctx, int64_t n, const void* inputs, const void* depth_map,
                               const void* opacity_map, int32_t map_width, int32_t map_height, void* colors,
                               void* stream);
/* The three passes over an asset's tessellation (vertices and frames as
 * rvh_asset_tessellate wrote them with the same tessellation descriptor).  The
 * light passes draw what sd->map_mode says: hair.geom's quads expanded and
 * rasterised in the light's view (the reference's shadow and opacity passes:
 * src/Renderer.cpp:2107-2223, the light camera bound as the geometry shader's
 * camera), or one texel per vertex.
 * depth_map: map_width x map_height floats (4-byte aligned), opacity_map: the
 * same count of float4, colors: one float4 per tessellated vertex, or NULL to
 * skip the per-vertex hair.frag (the maps alone feed rvh_asset_render_hair).  The shadow pass's light depth map, the opacity pass's layers
 * (min(255, 77 n) / 255 for n fragments in a layer: 0.3 as unorm8, saturating
 * sum; alpha 0) and hair.frag's colour per vertex. */
rvh_status rvh_asset_shade(rvh_asset* a, const rvh_tess_desc* td, const rvh_shade_desc* sd, const void* vertices,
                           const void* frames, void* depth_map, void* opacity_map, void* colors, void* stream);
/* A headless stand-in for the framebuffer: every vertex inside the camera's
 * clip volume covers one pixel of a width x height float4 image; the nearest
 * (then the lowest vertex index) wins and the pixel takes its colour; empty
 * pixels are 0.  n_vertices < 2^32. */
/* The camera image with hair.geom's geometry (src/shaders/hair.geom:41-108 and
 * the hair pipeline, src/Renderer.cpp:1554-1746): each isoline segment of the
 * tessellation (vertices and frames from rvh_asset_tessellate with td) becomes
 * the geometry shader's camera-facing quad of width (|random(3.242551 u, u u)| +
 * 0.5) * 0.075 * distance * strandWidth, rasterised with a LESS depth test and
 * shaded by hair.frag with perspective-correct inputs and the maps of
 * rvh_asset_shade (sd's light and map size).
 * sd->image_mode RVH_IMAGE_BLEND (the reference pipeline): quads in segment
 * order, each quad's triangles (V0, V1, V2) then (V2, V1, V3); a fragment that
 * passes the depth test against the earlier fragments (depth cleared to 1.0)
 * writes its depth and blends SRC_ALPHA / ONE_MINUS_SRC_ALPHA into the colour and
 * ONE / ONE into the alpha (clamped to 1); the image starts at the reference's
 * clear colour (101, 129, 140, 255) / 255 (the head mesh the reference draws
 * first is not drawn) and is kept in float (the reference's 8-bit swapchain
 * rounds each write).  Fewer than 2^31 segments.  Uses device scratch of 12 B
 * per pixel and 8 B per fragment, admitted against the context's budget.
 * RVH_IMAGE_NEAREST: each pixel takes its nearest fragment's colour (empty
 * pixels 0).
 * image: width x height float4; fragment_ids (device, nullable): width x height
 * uint32, the nearest fragment's segment (s * n_lines + j) * n_segments + k (in
 * blend mode the last one written, which is the same), or 0xffffffff.  A quad
 * with a corner behind the camera has each triangle clipped at the near plane
 * (z = 0 in clip space) and the kept part drawn, as Vulkan clips; the light
 * passes of rvh_asset_shade clip the same way.  Such quads and quads covering
 * more than 65,536 pixels are drawn from a list of up to 2^20 per pass.  Scratch:
 * 4 B per segment up to 2^20 segments and 4 B per pixel for those quads. */
rvh_status rvh_asset_render_hair(rvh_asset* a, const rvh_tess_desc* td, const rvh_shade_desc* sd, const void* vertices,
                                 const void* frames, const void* depth_map, const void* opacity_map, int32_t width,
                                 int32_t height, void* image, void* fragment_ids, void* stream);
rvh_status rvh_render_image(rvh_context* ctx, int64_t n_vertices, const void* vertices, const void* colors,
                            const rvh_shade_desc* sd, int32_t width, int32_t height, void* image, void* stream);

/* ---- failure detection ------------------------------------------------------
 * The reference has none.  A scan of the asset's records (after finishing a
 * pending friction; synchronous): non-finite position or velocity components
 * (the root's velocity included), the largest |v| (clamped to vmax before the
 * DFTL correction and the friction blend, compute.comp:198-215, so it can exceed
 * vmax), and the largest |segment - rest| / (rest * (n - 1))
 * with its strand (FTL keeps it near rounding, compute.comp:191-192). */
typedef struct rvh_health {
    uint64_t nonfinite;
    float max_speed;
    float max_length_error;
    int32_t worst_strand;     /* strand of max_length_error, -1 for an empty asset */
    int32_t reserved;
} rvh_health;
rvh_status rvh_asset_health(rvh_asset* a, rvh_health* out);

/* ---- checkpoint / resume ---------------------------------------------------
 * The reference's state lives only in its VkBuffers (Strand.cpp:186-191,
 * Scene.cpp:4-20).  A snapshot is the whole simulation state of one asset in
 * a flat host buffer: this header, then 16-byte aligned sections: rest lengths
 * (n_strands floats), strand wind (n_strands float4, flag RVH_SNAPSHOT_WIND),
 * the rest roots of a head motion (n_strands float4, flag RVH_SNAPSHOT_ROOTS),
 * the Strand records (48 * n_points bytes per strand).  A pending friction is
 * finished first, so a restored asset continues with the same bits. */
enum { RVH_SNAPSHOT_WIND = 1, RVH_SNAPSHOT_ROOTS = 2, RVH_SNAPSHOT_HEAD_ACTIVE = 4 };
typedef struct rvh_snapshot_header {
    char magic[8];                /* "RVHSNAP" */
    uint32_t version;             /* 1 */
    uint32_t header_bytes;        /* sizeof(rvh_snapshot_header) */
    uint64_t total_bytes;
    int32_t n_strands;
    int32_t n_points;
    uint32_t flags;
    int32_t n_colliders;
    int32_t lanes_per_strand;
    int32_t reserved;
    rvh_sim_params params;
    rvh_collider colliders[RVH_MAX_COLLIDERS];
    float head[16];               /* head pose (column-major) when RVH_SNAPSHOT_HEAD_ACTIVE */
} rvh_snapshot_header;
rvh_status rvh_asset_snapshot_bytes(rvh_asset* a, uint64_t* bytes);
/* Synchronous; bytes must equal rvh_asset_snapshot_bytes. */
rvh_status rvh_asset_snapshot(rvh_asset* a, void* host_dst, uint64_t bytes);
/* A new asset in ctx from a snapshot (lanes_per_strand 0: the snapshot's). */
rvh_status rvh_asset_restore(rvh_context* ctx, const void* host_src, uint64_t bytes, int32_t lanes_per_strand,
                             rvh_asset** out);

/* ---- batching: many assets, one persistent launch in a CUDA graph ---------- */
typedef struct rvh_batch_desc {
    int32_t lanes_per_strand;     /* 0 = tuner's choice (8 without a tuned record); else 1 (one thread walks
                                     each strand), 4, 8, 16, 32 */
    int32_t strands_per_tile;     /* phase-A tile size in strands; 0 = the tuner's choice with lanes_per_strand 0,
                                     else whole groups of rounds (the kernel's box span) near 4,096 points */
    int32_t ctas_per_sm;          /* 0 = occupancy limit */
    int32_t use_graph;            /* 1 = capture the launch in a CUDA graph (default) */
    int32_t full_steps;           /* 0 (default): fused steps - each launch first applies the previous
                                     step's gather + friction (loop 3), then runs loops 1-2, so a step is
                                     one pass over the records with no wait inside the launch; positions
                                     are final after every step, velocities after rvh_batch_finish (and
                                     every read).  1: every launch completes its step (phase B waits on
                                     its asset's phase A inside the launch). */
    int32_t reserved;
} rvh_batch_desc;
rvh_status rvh_batch_create(rvh_context* ctx, rvh_asset* const* assets, int32_t n, const rvh_batch_desc* desc,
                            rvh_batch** out);
rvh_status rvh_batch_destroy(rvh_batch* b);
/* One step of every asset; frames[i] belongs to assets[i]. */
rvh_status rvh_batch_step(rvh_batch* b, const rvh_frame* frames, void* stream);
/* Applies the last step's pending gather + friction of every asset (fused
 * steps only); afterwards the records hold the exact step result.  Reads,
 * plain steps and parameter changes of an asset do this for it implicitly. */
rvh_status rvh_batch_finish(rvh_batch* b, void* stream);
/* Nonzero device-side status of the last finished batch launch (RVH_ERR_TIMEOUT if a bounded wait gave up). */
rvh_status rvh_batch_check(rvh_batch* b);
rvh_status rvh_batch_info(rvh_batch* b, int32_t* lanes, int32_t* n_items, int32_t* n_ctas, int64_t* n_points);
/* Kernel timing: while enabled, every rvh_batch_step records CUDA events on
 * its stream around the persistent launch.  rvh_batch_timing_read waits for
 * them and returns the summed device time and the launch count since the
 * last read (then resets). */
/* Counters since the last call (then reset): phase-A rounds splatted through
 * the shared-memory box, rounds splatted with direct global atomics, phase-B
 * tiles gathered from the box, tiles gathered from the global grid. */
rvh_status rvh_batch_box_stats(rvh_batch* b, uint32_t out[4]);
/* Every asset's curvePoints (asset after asset in batch order) copied to host
 * memory: bytes = 16 * points gives the float4 records (w = 1), bytes = 12 *
 * points the xyz triples only (the w = 1 the reference stores carries no
 * information; a quarter fewer bytes over the host link).  A packing kernel on
 * `stream` writes a device staging buffer, then a copy stream moves it while
 * later steps run.  Two staging slots alternate; host_dst should be pinned
 * (rvh_pinned_alloc) for the copy to overlap.  rvh_batch_positions_wait blocks
 * until every copy is done. */
rvh_status rvh_batch_read_positions_async(rvh_batch* b, void* host_dst, size_t bytes, void* stream);
/* rvh_batch_step, then that step's curvePoints to host memory as xyz triples
 * (bytes = 12 * points, the layout of rvh_batch_read_positions_async): the
 * step kernel itself writes each new position into a staging slot beside the
 * Strand record it stores, so no separate pass reads the records again.  The
 * copy runs on the copy stream; rvh_batch_positions_wait blocks until it is
 * done. */
rvh_status rvh_batch_step_read_positions(rvh_batch* b, const rvh_frame* frames, void* host_dst, size_t bytes,
                                         void* stream);
rvh_status rvh_batch_positions_wait(rvh_batch* b);
/* Bytes rvh_batch_step copies host->device per step (per-asset frame and collider tables). */
rvh_status rvh_batch_h2d_bytes(rvh_batch* b, uint64_t* bytes);
rvh_status rvh_batch_timing_enable(rvh_batch* b, int32_t on);
rvh_status rvh_batch_timing_read(rvh_batch* b, double* total_ms, int32_t* launches);

/* ---- autotuning -------------------------------------------------------------
 * Times real batched steps of `assets` for every candidate: lanes per strand
 * {1, 4, 8, 16, 32} (strands per warp 32, 8, 4, 2, 1) x phase-A tile {whole
 * groups near 4,096 points, 1, 2, 4 rounds}, and with tune_grid also each listed grid resolution (every
 * grid-enabled asset re-gridded over the same bounds).  The strand records
 * are restored after every trial.  The winner is cached per workload
 * signature; rvh_batch_create with lanes_per_strand = 0 uses it. */
typedef struct rvh_tune_desc {
    int32_t steps;                /* timed steps per candidate (default 3) */
    int32_t tune_grid;            /* 1 = sweep grid_res[] too and leave the assets on the winner */
    int32_t use_cache;            /* 1 = return a cached result for this workload when there is one */
    int32_t n_grid_res;
    int32_t grid_res[8];
} rvh_tune_desc;
typedef struct rvh_tune_result {
    int32_t lanes_per_strand, strands_per_tile, grid_res, n_tried;
    float best_ms;
    int32_t tried_lanes[96], tried_tile[96], tried_res[96];
    float tried_ms[96];
} rvh_tune_result;
rvh_status rvh_tune_batch(rvh_context* ctx, rvh_asset* const* assets, int32_t n, const rvh_frame* frames,
                          const rvh_tune_desc* desc, rvh_tune_result* out);
rvh_status rvh_tune_lookup(rvh_asset* const* assets, int32_t n, int32_t tuned_grid, rvh_tune_result* out);

/* ---- serving: continuous batching of step requests for resident characters ----
 * The server replays the reference's per-frame loop (src/main.cpp:257-285)
 * for many characters at once: each launch advances every admitted request
 * by up to steps_per_launch steps (one persistent launch; a request's later
 * steps wait on the device for its earlier ones).  Requests are admitted in
 * arrival order as slots free up (a slot frees when a request's last step is
 * enqueued), their character has no request in flight, and their grid scratch
 * fits the server's HBM budget; their work shares launches on the device.  Every step is a fused step (the friction of a step is applied
 * at the start of the next), so a character keeps its grids between requests
 * with its last step's friction pending; when an admission waits for space,
 * the least recently stepped idle characters have that friction applied and
 * give their grids back, and the end of a run does the same for every
 * character, so each asset leaves a run fully stepped. */
typedef struct rvh_server_desc {
    int32_t max_active;           /* requests co-scheduled per launch (default 16): a request holds a
                                     slot from admission until its last step is enqueued */
    int32_t lanes_per_strand;     /* batch kernel shape: 1, 4, 8, 16, 32 (0: 8) */
    int32_t pipeline_depth;       /* launches in flight (default 2) */
    int32_t steps_per_launch;     /* consecutive steps of a request per launch (0: 1; at most 16):
                                     later steps wait on the device for the earlier one */
    uint64_t scratch_budget_bytes;/* HBM for the grids of admitted requests; charged to the context */
} rvh_server_desc;
typedef struct rvh_request {
    int32_t character;            /* id from rvh_server_add_character */
    int32_t n_steps;
    double arrival_s;             /* seconds after rvh_server_run starts */
} rvh_request;
typedef struct rvh_request_result {
    double admit_s;
    double done_s;
    float max_step_ms;            /* device time of the slowest launch that carried one of its steps */
    int32_t steps_done;
    int32_t status;
    int32_t reserved;
} rvh_request_result;
typedef struct rvh_server_stats {
    int64_t requests, steps, point_steps;
    int32_t launches, max_active;
    double wall_s, point_steps_per_s;
    double step_ms_p50, step_ms_p99, step_ms_p999;   /* device time of the launch carrying each step */
    double request_ms_p50, request_ms_p99;           /* arrival -> last step observed complete */
    double queue_ms_p50, queue_ms_p99;               /* arrival -> admission */
    double mean_batch;                               /* requests per launch */
    int64_t admission_waits;                         /* admissions deferred for lack of scratch memory */
    uint64_t scratch_used_bytes;                     /* at the end of the run (0 unless the run failed) */
    double gpu_busy_frac;                            /* sum of the launches' device times / wall time */
    double host_ms_per_launch;                       /* mean host time to plan, upload and enqueue a launch */
} rvh_server_stats;
rvh_status rvh_server_create(rvh_context* ctx, const rvh_server_desc* desc, rvh_server** out);
rvh_status rvh_server_destroy(rvh_server* s);
/* Registers a resident character; its grids become per-request scratch from
 * the server's pool.  Frames: dt fixed, t = (steps+1)*dt, wind from `wind`
 * (NULL = none) evaluated at the character's own step count. */
rvh_status rvh_server_add_character(rvh_server* s, rvh_asset* a, const rvh_wind_desc* wind, float dt, int32_t* id);
rvh_status rvh_server_character_steps(rvh_server* s, int32_t id, int64_t* steps);
/* Runs a request trace to completion (requests arrive at their arrival_s on the wall clock). */
rvh_status rvh_server_run(rvh_server* s, const rvh_request* reqs, int32_t n, rvh_request_result* results,
                          rvh_server_stats* stats);

/* ---- differentiation --------------------------------------------------------
 * Reverse-mode derivative of n_steps steps from the asset's current state,
 * through penalty collisions, PBD predict, FTL, the velocity clamp and the
 * DFTL correction (compute.comp:144-216); the hair-hair grid must be off.
 * Loss = 1/ns * sum_s |x_tip,s - target_s|^2 after the last step.  Gradients
 * with respect to the per-strand wind (3 floats per strand), the rest segment
 * lengths (1 per strand) and the initial velocities (3 per point); any output
 * may be NULL.  Checkpoints every `checkpoint_every` steps (0 = 10) and
 * recomputes each segment.  The asset's state is not modified.  Synchronous. */
rvh_status rvh_adjoint(rvh_asset* a, const rvh_frame* frames, int32_t n_steps, int32_t checkpoint_every,
                       const float* targets, double* loss, float* d_wind, float* d_rest, float* d_v0);

#ifdef __cplusplus
}
#endif
#endif /* RVH_H */
