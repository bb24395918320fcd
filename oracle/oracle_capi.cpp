/*
 * oracle_capi.cpp — TEST INFRASTRUCTURE ONLY.
 *
 * extern "C" entry points over hair_oracle.hpp for the Python tests (ctypes),
 * __graft_entry__.smoke() and bench.py's CPU legs.  Built by oracle/build.py
 * into oracle/_build/liboracle.so.  Nothing in the product links this.
 */
#include <omp.h>

#include <cstdio>
#include <vector>

#include "hair_adjoint.hpp"
#include "hair_oracle.hpp"
#include "scene_oracle.hpp"
#include "shade_oracle.hpp"
#include "tess_oracle.hpp"

namespace {

template <class T>
int run(T* state, int ns, int n, const float* rest, const float* strand_wind, const rvh_sim_params* P,
        const rvh_frame* frames, const rvh_collider* cols, int ncol, int n_steps, int threads,
        int64_t* grid_out, const float* heads = nullptr, const float* root_rest = nullptr) {
    if (!state || !rest || !P || !frames || ns < 0 || n < RVH_MIN_POINTS || n > RVH_MAX_POINTS ||
        ncol < 0 || ncol > RVH_MAX_COLLIDERS || n_steps < 0 || (ncol > 0 && !cols))
        return 1;
    if (threads < 1) threads = 1;
    oracle::Grid G;
    for (int s = 0; s < n_steps; ++s)
        oracle::step_asset<T>(state, ns, n, rest, strand_wind, *P, frames[s], cols + size_t(s) * ncol, ncol,
                              G, threads, heads ? heads + 16 * size_t(s) : nullptr, root_rest);
    if (grid_out && P->grid_enabled && !G.cells.empty())
        std::copy(G.cells.begin(), G.cells.end(), grid_out);
    return 0;
}

template <class T>
int run_group(int nm, T** states, const int* ns, const int* n, const float** rest, const rvh_sim_params* P,
              const rvh_frame* frames, const rvh_collider* cols, int ncol, int n_steps) {
    if (nm < 1 || !states || !ns || !n || !rest || !P || !frames || ncol < 0 || ncol > RVH_MAX_COLLIDERS ||
        n_steps < 0 || (ncol > 0 && !cols))
        return 1;
    std::vector<oracle::GroupMember<T>> m(nm);
    for (int k = 0; k < nm; ++k) {
        if (!states[k] || !rest[k] || ns[k] < 0 || n[k] < RVH_MIN_POINTS || n[k] > RVH_MAX_POINTS ||
            !P[k].grid_enabled || P[k].grid_dims[0] != P[0].grid_dims[0] || P[k].grid_dims[1] != P[0].grid_dims[1] ||
            P[k].grid_dims[2] != P[0].grid_dims[2] || P[k].grid_h != P[0].grid_h ||
            P[k].grid_scale != P[0].grid_scale || P[k].grid_wrap32 != P[0].grid_wrap32 ||
            P[k].grid_origin[0] != P[0].grid_origin[0] || P[k].grid_origin[1] != P[0].grid_origin[1] ||
            P[k].grid_origin[2] != P[0].grid_origin[2])
            return 1;
        m[k] = oracle::GroupMember<T>{states[k], ns[k], n[k], rest[k], &P[k]};
    }
    oracle::Grid G;
    for (int s = 0; s < n_steps; ++s)
        oracle::step_group<T>(m.data(), nm, frames[s], cols + size_t(s) * ncol, ncol, G);
    return 0;
}

}  // namespace

extern "C" {

/* Steps of a group of nm assets sharing one grid (hair_oracle.hpp step_group):
 * per member a state (ns[k] * 12 * n[k] scalars), rest lengths and params (the
 * same grid geometry); frames and colliders (n_steps * ncol) shared. */
int oracle_run_group_f64(int nm, double** states, const int* ns, const int* n, const float** rest,
                         const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                         int n_steps) {
    return run_group<double>(nm, states, ns, n, rest, P, frames, cols, ncol, n_steps);
}
int oracle_run_group_f32(int nm, float** states, const int* ns, const int* n, const float** rest,
                         const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                         int n_steps) {
    return run_group<float>(nm, states, ns, n, rest, P, frames, cols, ncol, n_steps);
}

/* Advance n_steps steps in FP64.  state = ns*12*n doubles (Strand records);
 * cols = n_steps*ncol colliders (one set per step); grid_out (nullable) gets the
 * last step's 4*nx*ny*nz int64 sums. */
int oracle_run_f64(double* state, int ns, int n, const float* rest, const float* strand_wind,
                   const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                   int n_steps, int threads, int64_t* grid_out) {
    return run<double>(state, ns, n, rest, strand_wind, P, frames, cols, ncol, n_steps, threads, grid_out);
}

/* The FP32 twin: same operation order, float state. */
int oracle_run_f32(float* state, int ns, int n, const float* rest, const float* strand_wind,
                   const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                   int n_steps, int threads, int64_t* grid_out) {
    return run<float>(state, ns, n, rest, strand_wind, P, frames, cols, ncol, n_steps, threads, grid_out);
}

/* As oracle_run_f64/f32 with a kinematic head: heads = n_steps column-major
 * 4x4 affine poses, root_rest = ns*3 rest roots; each step first places the
 * roots at heads[s] * root_rest. */
int oracle_run_head_f64(double* state, int ns, int n, const float* rest, const float* strand_wind,
                        const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                        int n_steps, int threads, int64_t* grid_out, const float* heads, const float* root_rest) {
    if (!heads || !root_rest) return 1;
    return run<double>(state, ns, n, rest, strand_wind, P, frames, cols, ncol, n_steps, threads, grid_out, heads,
                       root_rest);
}
int oracle_run_head_f32(float* state, int ns, int n, const float* rest, const float* strand_wind,
                        const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                        int n_steps, int threads, int64_t* grid_out, const float* heads, const float* root_rest) {
    if (!heads || !root_rest) return 1;
    return run<float>(state, ns, n, rest, strand_wind, P, frames, cols, ncol, n_steps, threads, grid_out, heads,
                      root_rest);
}
/* Strand tessellation (tess_oracle.hpp): out = ns * n_lines * (n_segments+1)
 * float4; frames (nullable) = ns * (n-1) * 3 float4.  sin_mode 0: the C
 * library's float sin in the hash (as the reference compiled here), 1: the
 * double sin rounded once (the library's definition). */
int oracle_tess(const float* records, int ns, int n, int n_lines, int n_segments, float clump_radius,
                float root_width, float tip_width, int sin_mode, float* out, float* frames) {
    if (!records || !out || ns < 0 || n < 2 || n > RVH_MAX_POINTS || n_lines < 1 || n_segments < 1) return 1;
    oracle::tess::TessParams P;
    P.n_lines = n_lines;
    P.n_segments = n_segments;
    P.clump_radius = clump_radius;
    P.root_width = root_width;
    P.tip_width = tip_width;
    oracle::tess::tessellate(records, ns, n, P,
                             sin_mode == 0 ? oracle::tess::RefSin::kFloat : oracle::tess::RefSin::kDouble, out,
                       frames);
    return 0;
}
/* Hair shading (shade_oracle.hpp).  Fragments: in = n x 24 floats, depth =
 * w*h floats, opacity = w*h float4, out = n float4.  sin_mode as for
 * oracle_tess. */
int oracle_shade_fragments(long long n, const float* in, const float* depth, const float* opacity, int w, int h,
                           int sin_mode, float* out) {
    if (n < 0 || (n > 0 && (!in || !depth || !opacity || !out)) || w < 1 || h < 1) return 1;
    const oracle::shade::Maps M{depth, opacity, w, h};
    const auto mode = sin_mode == 0 ? oracle::shade::RefSin::kFloat : oracle::shade::RefSin::kDouble;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) oracle::shade::shade_fragment(in + 24 * i, M, mode, out + 4 * i);
    return 0;
}
/* hairOpacity.frag's outColor for n fragments (layers 1-3, z0). */
int oracle_opacity_fragments(long long n, const float* in, const float* depth, int w, int h, float* out) {
    if (n < 0 || (n > 0 && (!in || !depth || !out)) || w < 1 || h < 1) return 1;
    for (long long i = 0; i < n; ++i) oracle::shade::opacity_fragment(in + 24 * i, depth, w, h, out + 4 * i);
    return 0;
}
/* Light-space projection and the eyes of the camera and light views (matrices
 * column-major): lvp[16], cam_pos[3], light_pos[3]. */
int oracle_shade_camera(const float* camera_view, const float* light_view, const float* light_proj, float* lvp,
                        float* cam_pos, float* light_pos) {
    if (!camera_view || !light_view || !light_proj || !lvp || !cam_pos || !light_pos) return 1;
    const oracle::shade::Camera K = oracle::shade::make_camera(camera_view, light_view, light_proj);
    for (int k = 0; k < 16; ++k) lvp[k] = K.lvp[k];
    for (int k = 0; k < 3; ++k) {
        cam_pos[k] = K.cam_pos[k];
        light_pos[k] = K.light_pos[k];
    }
    return 0;
}
/* Light depth and deep opacity maps of nv vertices (float4 each). */
int oracle_shade_maps(const float* verts, long long nv, const float* lvp, int w, int h, float* depth,
                      float* opacity) {
    if (nv < 0 || (nv > 0 && !verts) || !lvp || !depth || !opacity || w < 1 || h < 1) return 1;
    oracle::shade::light_maps(verts, nv, lvp, w, h, depth, opacity);
    return 0;
}
/* Fragment inputs (n_vertices x 24) of tessellated vertices and their frames. */
int oracle_shade_vertex_inputs(const float* verts, const float* frames, int ns, int n, int n_lines, int n_segments,
                               const float* camera_view, const float* light_view, const float* light_proj,
                               float* in) {
    if (!verts || !frames || !in || ns < 0 || n < 2 || n_lines < 1 || n_segments < 1) return 1;
    const oracle::shade::Camera K = oracle::shade::make_camera(camera_view, light_view, light_proj);
    const long long nv = (long long)ns * n_lines * (n_segments + 1);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nv; ++i)
        oracle::shade::vertex_inputs(verts, frames, n, n_lines, n_segments, K, i, in + 24 * i);
    return 0;
}
/* Camera image (w x h float4) of nv vertices with the given colours. */
int oracle_render_image(const float* verts, const float* colors, long long nv, const float* view, const float* proj,
                        int w, int h, float* image) {
    if (nv < 0 || (nv > 0 && (!verts || !colors)) || !view || !proj || !image || w < 1 || h < 1) return 1;
    oracle::shade::render_image(verts, colors, nv, view, proj, w, h, image);
    return 0;
}
/* Camera image of hair.geom's quads over a tessellation (shade_oracle.hpp
 * render_hair): image w x h float4, ids (nullable) w x h uint32. */
int oracle_render_hair(const float* verts, const float* frames, int ns, int n, int n_lines, int n_segments,
                       const float* camera_view, const float* camera_proj, const float* light_view,
                       const float* light_proj, const float* depth, const float* opacity, int mw, int mh, int w, int h,
                       int sin_mode, float* image, uint32_t* ids) {
    if (!verts || !frames || !image || !depth || !opacity || ns < 0 || n < 2 || n_lines < 1 || n_segments < 1 ||
        w < 1 || h < 1 || mw < 1 || mh < 1)
        return 1;
    oracle::shade::Raster R;
    if (!oracle::shade::make_raster(camera_view, camera_proj, light_view, light_proj, w, h, R)) return 2;
    const oracle::shade::Maps M{depth, opacity, mw, mh};
    oracle::shade::render_hair(verts, frames, ns, n, n_lines, n_segments, R, M,
                               sin_mode == 0 ? oracle::shade::RefSin::kFloat : oracle::shade::RefSin::kDouble, image,
                               ids);
    return 0;
}
/* The hair pass with the pipeline's in-order blending (shade_oracle.hpp
 * render_hair_blend), from clear colour clear_rgba. */
int oracle_render_hair_blend(const float* verts, const float* frames, int ns, int n, int n_lines, int n_segments,
                             const float* camera_view, const float* camera_proj, const float* light_view,
                             const float* light_proj, const float* depth, const float* opacity, int mw, int mh, int w,
                             int h, int sin_mode, const float* clear_rgba, float* image, uint32_t* ids) {
    if (!verts || !frames || !image || !depth || !opacity || !clear_rgba || ns < 0 || n < 2 || n_lines < 1 ||
        n_segments < 1 || w < 1 || h < 1 || mw < 1 || mh < 1)
        return 1;
    oracle::shade::Raster R;
    if (!oracle::shade::make_raster(camera_view, camera_proj, light_view, light_proj, w, h, R)) return 2;
    const oracle::shade::Maps M{depth, opacity, mw, mh};
    oracle::shade::render_hair_blend(verts, frames, ns, n, n_lines, n_segments, R, M,
                                     sin_mode == 0 ? oracle::shade::RefSin::kFloat : oracle::shade::RefSin::kDouble,
                                     clear_rgba, image, ids);
    return 0;
}
/* Light depth and deep opacity maps rasterised from hair.geom's quads in the
 * light's view (shade_oracle.hpp light_maps_quads). */
int oracle_shade_maps_quads(const float* verts, int ns, int n_lines, int n_segments, const float* light_view,
                            const float* light_proj, int w, int h, int sin_mode, float* depth, float* opacity) {
    if (!verts || !light_view || !light_proj || !depth || !opacity || ns < 0 || n_lines < 1 || n_segments < 1 ||
        w < 1 || h < 1)
        return 1;
    oracle::shade::Raster R;
    oracle::shade::make_light_raster(light_view, light_proj, w, h, R);
    oracle::shade::light_maps_quads(verts, ns, n_lines, n_segments, R,
                                    sin_mode == 0 ? oracle::shade::RefSin::kFloat : oracle::shade::RefSin::kDouble,
                                    depth, opacity);
    return 0;
}
/* FP64 adjoint of the no-grid step (FTL + DFTL + collisions); see hair_adjoint.hpp. */
int oracle_adjoint_f64(const double* state0, int ns, int n, const double* rest, const double* strand_wind,
                       const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                       int n_steps, const double* targets, int threads, double* loss, double* d_wind,
                       double* d_rest, double* d_v0) {
    if (!state0 || !rest || !P || !frames || !targets || !loss || ns < 1 || n < RVH_MIN_POINTS ||
        n > RVH_MAX_POINTS || ncol < 0 || ncol > RVH_MAX_COLLIDERS || n_steps < 1 || (ncol > 0 && !cols))
        return 1;
    if (P->grid_enabled) return 7;
    if (threads < 1) threads = 1;
    oracle::adjoint_asset(state0, ns, n, rest, strand_wind, *P, frames, cols, ncol, n_steps, targets,
                          threads, loss, d_wind, d_rest, d_v0);
    return 0;
}

/* Loss alone (forward only), for central finite differences in FP64. */
int oracle_loss_f64(const double* state0, int ns, int n, const double* rest, const double* strand_wind,
                    const rvh_sim_params* P, const rvh_frame* frames, const rvh_collider* cols, int ncol,
                    int n_steps, const double* targets, int threads, double* loss) {
    if (!state0 || !rest || !P || !frames || !targets || !loss || ns < 1 || n < RVH_MIN_POINTS ||
        n > RVH_MAX_POINTS || n_steps < 1 || (ncol > 0 && !cols))
        return 1;
    if (P->grid_enabled) return 7;
    if (threads < 1) threads = 1;
    *loss = oracle::forward_loss(state0, ns, n, rest, strand_wind, *P, frames, cols, ncol, n_steps, targets,
                                 threads);
    return 0;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

/* The seeded synthetic head of include/rvh_scene.h, from scene_oracle.hpp:
 * records = ns*12*n floats, rest = ns floats, params and up to
 * RVH_MAX_COLLIDERS colliders (either may be NULL). */
int oracle_generate_head(const rvh_head_desc* d, float* records, float* rest, rvh_sim_params* params,
                         rvh_collider* colliders, int32_t* n_colliders) {
    return oracle::scene::head(d, records, rest, params, colliders, n_colliders);
}

/* Wind of frame `step` at time t (scene_oracle.hpp). */
int oracle_wind_at(const rvh_wind_desc* w, int64_t step, float t, float* out) {
    if (!w || !out) return 1;
    oracle::scene::wind(w, step, t, out);
    return 0;
}

}  // extern "C"
