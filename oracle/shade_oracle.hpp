/*
 * shade_oracle.hpp — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's hair shading, the three graphics passes
 * of src/Renderer.cpp that follow the tessellation:
 *
 *  1. light depth map (shadow-map pass): the hair drawn from the shadow
 *     camera into a 1080 x 720 depth target cleared to 1.0 (Renderer.cpp:9-10,
 *     the clear in the command buffer), nearest depth kept;
 *  2. deep opacity map (opacity pass, src/shaders/hairOpacity.frag): every
 *     fragment compares its light depth z with z0 = the depth map sampled at
 *     its position and adds val = 0.3 to layer 1, 2 and 3 when z is in
 *     [z0, z0 + d), to layers 2 and 3 in [z0 + d, z0 + 2d), to layer 3 beyond
 *     (d = 0.3, hairOpacity.frag:42-59).  The target is the swapchain's
 *     B8G8R8A8_UNORM (Renderer.cpp:1939-1951) with ONE + ONE additive blending
 *     (Renderer.cpp:1471-1480): 0.3 is stored as 77/255 and the sum saturates,
 *     so a layer that received c fragments reads min(255, 77 c) / 255;
 *  3. camera pass (src/shaders/hair.frag): per fragment a Marschner-style
 *     single-scattering lobe, a multiple-scattering term damped by the opacity
 *     layer the fragment falls in, a 7x7 PCF shadow test, an ambient term and
 *     a per-isoline brightness hash.
 *
 * Without a rasteriser the passes take the tessellated vertices as their
 * fragments: a vertex covers the one texel its light-space position falls in
 * (strands are about one texel wide and their vertices about one texel apart
 * at the reference's sizes), and the fragment inputs of a vertex are the ones
 * the tessellation and geometry stages hand the fragment shader at the ribbon's
 * centre line (hair.tese:289-330, hair.geom:43-61): uv = (isoline u, v), the
 * segment frame {tangent, Frisvad b1, b2}, normalize(cameraPos - pos),
 * normalize(lightPos - pos), lightProj * lightView * pos.
 *
 * Samplers are bilinear, clamp to edge, texel centres at (i + 0.5) / size,
 * weights in full float precision (the reference's VK_FILTER_LINEAR +
 * CLAMP_TO_EDGE samplers, Renderer.cpp:14,1899-1902,1956-1962).  The opacity
 * map's clear value is uninitialised in the reference (the command buffer
 * fills the shadow map's clear value twice); here it is 0.
 *
 * hair.frag's hash random(st) = fract(sin(dot(st, (12.9898, 78.233))) *
 * 43758.5453123) (:129-131) multiplies sin's rounding by 43758:
 * RefSin::kFloat calls the C library's float sin (the reference compiled on
 * this host), RefSin::kDouble rounds the double sin once (a correctly rounded
 * sin, what the library computes on the GPU).  All other float operations are
 * separately rounded in the shader's order (build with -ffp-contract=off) and
 * call the C library's float acos, sin, cos, exp, pow.
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace oracle {
namespace shade {

enum class RefSin { kFloat, kDouble };

struct V3 {
    float x, y, z;
};
inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(float s, V3 a) { return mk(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator/(V3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline V3 cross(V3 a, V3 b) { return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
// GLSL clamp(x, 0, 1) as min(max(x, 0), 1) with max(a, b) = a < b ? b : a, min(a, b) = b < a ? b : a
inline float clamp01(float x) {
    const float m = x < 0.f ? 0.f : x;
    return 1.f < m ? 1.f : m;
}

constexpr float kPi = 3.14159265359f;        // hair.frag:4-8
constexpr float kPiOver2 = 1.57079632679f;
constexpr float kRadToDeg = 57.2957795131f;
constexpr float kDegToRad = 0.01745329251f;
constexpr float kEps = 0.001f;
constexpr int kLayerUnit = 77;               // 0.3 as an 8-bit unorm: round(0.3f * 255) = round(76.500003)

struct Maps {
    const float* depth;     // w x h
    const float* opacity;   // w x h x 4 (layers r, g, b; a unused)
    int w, h;
};

inline float texel(const float* img, int w, int h, int ch, int x, int y, int c) {
    x = std::min(std::max(x, 0), w - 1);
    y = std::min(std::max(y, 0), h - 1);
    return img[(size_t(y) * w + x) * ch + c];
}
inline float sample(const float* img, int w, int h, int ch, float u, float v, int c) {
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float fx = x - x0, fy = y - y0;
    // texel indices clamped before the conversion (only the clamp to edge reads them);
    // keeps an infinite or NaN coordinate defined
    const int ix = (int)std::fmin(std::fmax(x0, -1.f), (float)w), iy = (int)std::fmin(std::fmax(y0, -1.f), (float)h);
    const float t00 = texel(img, w, h, ch, ix, iy, c), t10 = texel(img, w, h, ch, ix + 1, iy, c);
    const float t01 = texel(img, w, h, ch, ix, iy + 1, c), t11 = texel(img, w, h, ch, ix + 1, iy + 1, c);
    const float a = t00 + fx * (t10 - t00);
    const float b = t01 + fx * (t11 - t01);
    return a + fy * (b - a);
}

inline float frag_random(float x, float y, RefSin mode) {   // hair.frag:129-131
    const float d = x * 12.9898f + y * 78.233f;
    const float s = mode == RefSin::kFloat ? std::sin(d) : (float)std::sin((double)d);
    const float m = s * 43758.5453123f;
    return m - std::floor(m);
}

// hair.frag:24-28
inline bool vec3_compare(V3 a, V3 b) {
    return std::fabs(a.x - b.x) < kEps && std::fabs(a.y - b.y) < kEps && std::fabs(a.z - b.z) < kEps;
}
// hair.frag:31-39
inline float angle_vector_plane(V3 v, V3 n) {
    float angle = std::acos(dot(v, n) / (length(v) * length(n)));
    if (angle < kPiOver2) angle = kPiOver2 - angle;
    else angle = -(angle - kPiOver2);
    return angle;
}
// hair.frag:41-43
inline V3 project_onto_plane(V3 v, V3 n) { return v - dot(v, n) * n; }
// hair.frag:45-55
inline float directional_angle(V3 v1, V3 v2, V3 n) {
    const float angle = std::acos(dot(v1, v2) / (length(v1) * length(v2)));
    if (vec3_compare(normalize(cross(v2, v1)), n)) return angle;
    return (2.0f * kPi) - angle;
}
// hair.frag:80-82
inline float gaussian(float alpha, float beta, float ti, float to) {
    const float e = std::sin(ti * kDegToRad) + std::sin(to * kDegToRad) - alpha;
    return (1.f / (beta * std::sqrt(2.f * kPi))) * std::exp(-std::pow(e, 2.0f) / (2.f * beta * beta));
}
// hair.frag:88-92
inline float schlicks(float n, float x) {
    const float R0 = ((1.f - n) * (1.f - n)) / ((1.f + n) * (1.f + n));
    return R0 + (1.f - R0) * std::pow(1.f - x, 5.0f);
}

// hair.frag:99-124; the texel size is the shader's constant 1 / (1080, 720)
inline float pcf_shadow(const Maps& M, float px, float py, float pz, float pw) {
    const float x = px / pw, y = py / pw, z = pz / pw;
    if (std::fabs(x) > 1.f || std::fabs(y) > 1.f || std::fabs(z) > 1.f) return 0.f;
    const float u = x * 0.5f + 0.5f, v = y * 0.5f + 0.5f;
    const float tsx = 1.f / 1080.0f, tsy = 1.f / 720.0f;
    float lighted = 0.f;
    for (int dx = -3; dx <= 3; ++dx)
        for (int dy = -3; dy <= 3; ++dy) {
            const float cu = u + (float)dx * tsx, cv = v + (float)dy * tsy;
            if (z > sample(M.depth, M.w, M.h, 1, cu, cv, 0)) lighted += 1.f;
        }
    const float kernel = 2.f * 3 + 1.f;
    return lighted / (kernel * kernel);
}

/* hair.frag main (:133-261) for one fragment.  in[24]: uv (2), u, v, w (3
 * each), viewDir (3), lightDir (3), fragPosLightSpace (4), 3 unused.  The
 * shader's unused values (the transformed directions, theta_h, phi_h, the
 * colour gradient, gamma_t, the TRT lobe it computes and then replaces by the
 * TT lobe at :222) do not reach the output and are not computed. */
inline void shade_fragment_bright(const float* in, const Maps& M, float bright, float out[4]);
inline void shade_fragment(const float* in, const Maps& M, RefSin mode, float out[4]) {
    shade_fragment_bright(in, M, 0.8f * std::fabs(frag_random(in[0], in[0], mode)) + 0.6f, out);
}
/* hair.frag with the brightness factor 0.8 |random(uv.x, uv.x)| + 0.6 given. */
inline void shade_fragment_bright(const float* in, const Maps& M, float bright, float out[4]) {
    const V3 fu = mk(in[2], in[3], in[4]), fv = mk(in[5], in[6], in[7]);
    const V3 view = mk(in[11], in[12], in[13]), light = mk(in[14], in[15], in[16]);
    const float px = in[17], py = in[18], pz = in[19], pw = in[20];
    const float over255 = 1.0f / 255.0f;
    const V3 w_i = normalize(light);
    const V3 w_o = normalize(view);
    const float n = 1.55f;
    const V3 C = mk(101.0f, 67.0f, 33.0f) * over255;
    const float roughness = 0.2f, shift = 0.01f;
    const float theta_i = angle_vector_plane(w_i, fu) * kRadToDeg;
    const float theta_o = angle_vector_plane(w_o, fu) * kRadToDeg;
    const float phi_i = directional_angle(normalize(project_onto_plane(w_i, fu)), fv, fu) * kRadToDeg;
    const float phi_o = directional_angle(normalize(project_onto_plane(w_o, fu)), fv, fu) * kRadToDeg;
    const float theta_d = (theta_o - theta_i) / 2.f;
    const float phi_d = phi_o - phi_i;
    const float alpha_R = -2.f * shift, alpha_TT = shift, alpha_TRT = 4.f * shift;
    const float beta_R = roughness * roughness, beta_TT = 0.5f * beta_R, beta_TRT = 2.f * beta_R;
    const float M_R = gaussian(alpha_R, beta_R, theta_i, theta_o);
    const float M_TT = gaussian(alpha_TT, beta_TT, theta_i, theta_o);
    const float M_TRT = gaussian(alpha_TRT, beta_TRT, theta_i, theta_o);
    const float cosTheta_d = std::cos(theta_d * kDegToRad);
    const float cosPhi_d = std::cos(phi_d * kDegToRad);
    const float cosPhi_dOver2 = std::cos((phi_d / 2.f) * kDegToRad);
    const float nR = schlicks(n, std::sqrt(0.5f + 0.5f * dot(w_i, w_o))) * (0.25f * std::sqrt(0.5f + 0.5f * cosPhi_d));
    const V3 N_R = mk(nR, nR, nR);
    const float n_prime = (1.19f / cosTheta_d) + 0.36f * cosTheta_d;
    const float a = 1.f / n_prime;
    const float h_TT = (1.f + a * (0.6f - 0.8f * cosPhi_d)) * cosPhi_dOver2;
    const float f_TT = schlicks(n, cosTheta_d * std::sqrt(1.f - h_TT * h_TT));
    const float Cpower_TT = std::sqrt(1.f - h_TT * h_TT * a * a) / (2.f * cosTheta_d);
    const V3 T_TT = mk(std::pow(C.x, Cpower_TT), std::pow(C.y, Cpower_TT), std::pow(C.z, Cpower_TT));
    const V3 A_TT = (1.f - f_TT) * (1.f - f_TT) * T_TT;
    const float D_TT = std::exp(-3.65f * cosPhi_d - 3.98f);
    const V3 N_TT = A_TT * D_TT;
    const V3 N_TRT = A_TT * D_TT;
    const V3 S_single = (1.3f * N_R * M_R + 0.5f * N_TT * M_TT + N_TRT * M_TRT) / (cosTheta_d * cosTheta_d);
    const float shadow = pcf_shadow(M, px, py, pz, pw);
    const float x = px / pw, y = py / pw, currentDepth = pz / pw;
    const float u = x * 0.5f + 0.5f, v = y * 0.5f + 0.5f;
    const float z0 = sample(M.depth, M.w, M.h, 1, u, v, 0);
    const float d = 0.3f;
    float opacity = 0.f;
    if (currentDepth >= z0 && currentDepth < z0 + d) opacity = sample(M.opacity, M.w, M.h, 4, u, v, 0);
    else if (currentDepth >= z0 + d && currentDepth < z0 + 2.f * d) opacity = sample(M.opacity, M.w, M.h, 4, u, v, 1);
    else if (currentDepth >= z0 + 2.f * d) opacity = sample(M.opacity, M.w, M.h, 4, u, v, 2);
    const V3 fakeNormal = normalize(w_o - fu * dot(fu, w_o));
    const float luma = 0.3f;
    const V3 Cexp = mk(std::pow(C.x / luma, 1.f - opacity), std::pow(C.y / luma, 1.f - opacity),
                       std::pow(C.z / luma, 1.f - opacity));
    const V3 sqrtC = mk(std::sqrt(C.x), std::sqrt(C.y), std::sqrt(C.z));
    const V3 S_multi = sqrtC * ((dot(fakeNormal, w_i) + 1.f) / (4.f * kPi)) * Cexp;
    const V3 col = ((S_single + S_multi) * (1.f - shadow) + 0.3f * C) * bright;
    out[0] = clamp01(col.x);
    out[1] = clamp01(col.y);
    out[2] = clamp01(col.z);
    out[3] = 0.75f;
}

// ---- cameras ---------------------------------------------------------------------------
struct Camera {
    float lvp[16];       // light proj * light view, column-major, product in double rounded once
    float cam_pos[3];    // eye of the camera view: -R^T t
    float light_pos[3];  // eye of the light view
};

inline void eye_of(const float* view, float out[3]) {
    for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc -= double(view[i * 4 + k]) * double(view[12 + k]);
        out[i] = float(acc);
    }
}

inline Camera make_camera(const float* camera_view, const float* light_view, const float* light_proj) {
    Camera K;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += double(light_proj[k * 4 + r]) * double(light_view[c * 4 + k]);
            K.lvp[c * 4 + r] = float(acc);
        }
    eye_of(camera_view, K.cam_pos);
    eye_of(light_view, K.light_pos);
    return K;
}

inline void mul_point(const float* m, V3 p, float& x, float& y, float& z, float& w) {
    x = ((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12];
    y = ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13];
    z = ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14];
    w = ((m[3] * p.x + m[7] * p.y) + m[11] * p.z) + m[15];
}

/* The texel a vertex covers in a (w x h) map of projection m, and its depth and
 * map coordinates; false outside the clip volume (x, y in [-1, 1], depth in
 * [0, 1], w > 0), where the rasteriser would clip it. */
inline bool project_texel(const float* m, V3 p, int w, int h, int& tx, int& ty, float& depth, float& u, float& v) {
    float x, y, z, ww;
    mul_point(m, p, x, y, z, ww);
    if (!(ww > 0.f)) return false;
    x = x / ww;
    y = y / ww;
    z = z / ww;
    if (std::fabs(x) > 1.f || std::fabs(y) > 1.f || z < 0.f || z > 1.f) return false;
    u = x * 0.5f + 0.5f;
    v = y * 0.5f + 0.5f;
    tx = std::min((int)(u * (float)w), w - 1);
    ty = std::min((int)(v * (float)h), h - 1);
    depth = z;
    return true;
}

// ---- passes ------------------------------------------------------------------------------
/* The opacity layer a fragment at light depth z adds to, given z0
 * (hairOpacity.frag:50-59): 1 = layers 1-3, 2 = layers 2-3, 3 = layer 3, 0 = none. */
inline int opacity_layer(float z, float z0) {
    const float d = 0.3f;
    if (z >= z0 && z < z0 + d) return 1;
    if (z >= z0 + d && z < z0 + 2.f * d) return 2;
    if (z >= z0 + 2.f * d) return 3;
    return 0;
}

/* hairOpacity.frag's outColor for one fragment (in as for shade_fragment):
 * (layer1, layer2, layer3, z0). */
inline void opacity_fragment(const float* in, const float* depth, int w, int h, float out[4]) {
    const float x = in[17] / in[20], y = in[18] / in[20], z = in[19] / in[20];
    const float u = x * 0.5f + 0.5f, v = y * 0.5f + 0.5f;
    const float z0 = sample(depth, w, h, 1, u, v, 0);
    const int l = opacity_layer(z, z0);
    const float val = 0.3f;
    out[0] = l == 1 ? 0.f + val : 0.f;
    out[1] = (l == 1 || l == 2) ? 0.f + val : 0.f;
    out[2] = l != 0 ? 0.f + val : 0.f;
    out[3] = z0;
}

/* Passes 1 and 2 over nv tessellated vertices (float4 {pos, width}). */
inline void light_maps(const float* verts, long long nv, const float* lvp, int w, int h, float* depth, float* opacity) {
    const size_t texels = size_t(w) * h;
    std::fill(depth, depth + texels, 1.0f);
    for (long long i = 0; i < nv; ++i) {
        const float* q = verts + 4 * i;
        int tx, ty;
        float z, u, v;
        if (project_texel(lvp, mk(q[0], q[1], q[2]), w, h, tx, ty, z, u, v)) {
            float& t = depth[size_t(ty) * w + tx];
            if (z < t) t = z;
        }
    }
    std::vector<uint32_t> count(texels * 3, 0);
    for (long long i = 0; i < nv; ++i) {
        const float* q = verts + 4 * i;
        int tx, ty;
        float z, u, v;
        if (!project_texel(lvp, mk(q[0], q[1], q[2]), w, h, tx, ty, z, u, v)) continue;
        const int l = opacity_layer(z, sample(depth, w, h, 1, u, v, 0));
        uint32_t* c = count.data() + (size_t(ty) * w + tx) * 3;
        if (l == 1) c[0]++;
        if (l == 1 || l == 2) c[1]++;
        if (l != 0) c[2]++;
    }
    for (size_t t = 0; t < texels; ++t) {
        for (int l = 0; l < 3; ++l) {
            const uint32_t c = count[t * 3 + l];
            const uint32_t k = c >= 4 ? 255u : std::min<uint32_t>(255u, (uint32_t)kLayerUnit * c);
            opacity[t * 4 + l] = (float)k / 255.0f;
        }
        opacity[t * 4 + 3] = 0.f;
    }
}

/* The fragment inputs of tessellated vertex (strand s, isoline j, vertex k). */
inline void vertex_inputs(const float* verts, const float* frames, int n_points, int n_lines, int n_segments,
                          const Camera& K, long long i, float in[24]) {
    const int S1 = n_segments + 1;
    const long long per = (long long)n_lines * S1;
    const long long s = i / per;
    const int r = (int)(i - s * per);
    const int j = r / S1, k = r - j * S1;
    const float u = (float)j / (float)n_lines, v = (float)k / (float)n_segments;
    const float x = v * (float)(n_points - 1);
    const int sf = std::min((int)std::floor(x), n_points - 2);
    const float* fr = frames + (size_t(s) * (n_points - 1) + sf) * 12;
    const float* q = verts + 4 * i;
    const V3 p = mk(q[0], q[1], q[2]);
    in[0] = u;
    in[1] = v;
    for (int c = 0; c < 3; ++c)
        for (int e = 0; e < 3; ++e) in[2 + 3 * c + e] = fr[4 * c + e];
    const V3 vd = normalize(mk(K.cam_pos[0], K.cam_pos[1], K.cam_pos[2]) - p);
    const V3 ld = normalize(mk(K.light_pos[0], K.light_pos[1], K.light_pos[2]) - p);
    in[11] = vd.x;
    in[12] = vd.y;
    in[13] = vd.z;
    in[14] = ld.x;
    in[15] = ld.y;
    in[16] = ld.z;
    mul_point(K.lvp, p, in[17], in[18], in[19], in[20]);
    in[21] = in[22] = in[23] = 0.f;
}

/* Camera image: every vertex inside the camera's clip volume covers one pixel;
 * the nearest (smallest depth, then smallest vertex index) wins and the pixel
 * takes its colour; empty pixels stay 0. */
inline void render_image(const float* verts, const float* colors, long long nv, const float* view, const float* proj,
                         int w, int h, float* image) {
    float vp[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += double(proj[k * 4 + r]) * double(view[c * 4 + k]);
            vp[c * 4 + r] = float(acc);
        }
    const size_t px = size_t(w) * h;
    std::vector<uint64_t> key(px, ~0ull);
    for (long long i = 0; i < nv; ++i) {
        const float* q = verts + 4 * i;
        int tx, ty;
        float z, u, v;
        if (!project_texel(vp, mk(q[0], q[1], q[2]), w, h, tx, ty, z, u, v)) continue;
        uint32_t zb;
        std::memcpy(&zb, &z, 4);
        const uint64_t kk = (uint64_t(zb) << 32) | uint64_t(uint32_t(i));
        uint64_t& t = key[size_t(ty) * w + tx];
        if (kk < t) t = kk;
    }
    for (size_t p = 0; p < px; ++p) {
        if (key[p] == ~0ull) {
            for (int c = 0; c < 4; ++c) image[p * 4 + c] = 0.f;
        } else {
            const size_t i = size_t(key[p] & 0xffffffffu);
            for (int c = 0; c < 4; ++c) image[p * 4 + c] = colors[i * 4 + c];
        }
    }
}


// ---- rasterising hair.geom's quads into a camera image ------------------------------------
/*
 * hair.geom (:41-108) turns each isoline segment (tessellated vertices k, k+1 of
 * isoline j of strand s) into a camera-facing quad: with P = camera proj * view,
 * c1 = P [pos_k, 1], c2 = P [pos_k+1, 1] and the width
 *   width1 = (|random(3.242551 u, u u)| + 0.5) * 0.075 * |cameraPos - pos_k| * strandWidth_k
 * (width2 is computed and unused; every corner uses width1) it emits the strip
 *   V0 = c1 - (width1, 0, 0, 0), V1 = c1 + (width1, 0, 0, 0), V2 = c2 - ..., V3 = c2 + ...
 * with vertex k's attributes on V0, V1 and vertex k+1's on V2, V3; the light-space
 * position of a corner is lightProj * lightView * inverse(view) * inverse(proj) * V.
 * The hair pipeline rasterises with no culling and a LESS depth test
 * (src/Renderer.cpp:1640-1664); its alpha blending is order dependent, so the
 * headless image keeps, per pixel, the nearest fragment's outColor.
 *
 * Rasterisation (this restatement's definition of Vulkan's rules):
 *   screen x = (x/w * 0.5 + 0.5) W, y = (y/w * 0.5 + 0.5) H, depth = z/w; pixel
 *   centres at (px + 0.5, py + 0.5); triangles (V0, V1, V2) and (V2, V1, V3),
 *   each reordered to positive area; a centre is covered when every edge
 *   function is > 0, or = 0 on a top-left edge (dy < 0, or dy = 0 and dx > 0);
 *   depth interpolated linearly in screen space and kept in [0, 1]; attributes
 *   interpolated perspective-correctly (barycentrics over w).  A quad with a
 *   corner at w <= 0 is clipped at the near plane (clip_quad); one with a
 *   non-finite corner is dropped.  The nearest fragment wins; ties go to
 *   the smaller segment id = (s * n_lines + j) * n_segments + k, then to the
 *   first triangle.  uv.x is constant along an isoline, so the brightness hash
 *   takes the isoline's own u.
 */
struct Raster {
    float vp[16];      // camera proj * view
    float lmap[16];    // light proj * light view * inverse(view) * inverse(proj)
    float cam_pos[3], light_pos[3];
    int width, height;
};

inline bool invert4(const double* m, double* inv) {   // column-major, Gauss-Jordan with partial pivoting
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][4 + c] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0) return false;
        for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        const double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[c * 4 + r] = a[r][4 + c];
    return true;
}

inline void mul4d(const double* a, const double* b, double* o) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += a[k * 4 + r] * b[c * 4 + k];
            o[c * 4 + r] = acc;
        }
}

inline bool make_raster(const float* cam_view, const float* cam_proj, const float* light_view, const float* light_proj,
                        int w, int h, Raster& R) {
    double cv[16], cp[16], lv[16], lp[16], t[16], u[16], icv[16], icp[16], vp[16];
    for (int k = 0; k < 16; ++k) {
        cv[k] = cam_view[k];
        cp[k] = cam_proj[k];
        lv[k] = light_view[k];
        lp[k] = light_proj[k];
    }
    if (!invert4(cv, icv) || !invert4(cp, icp)) return false;
    mul4d(cp, cv, vp);
    mul4d(lp, lv, t);
    mul4d(t, icv, u);
    mul4d(u, icp, t);
    for (int k = 0; k < 16; ++k) {
        R.vp[k] = float(vp[k]);
        R.lmap[k] = float(t[k]);
    }
    eye_of(cam_view, R.cam_pos);
    eye_of(light_view, R.light_pos);
    R.width = w;
    R.height = h;
    return true;
}

inline void mul_vec4(const float* m, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r) o[r] = ((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * v[3];
}

struct Quad {
    float clip[4][4];   // V0..V3 clip positions
    float sx[4], sy[4], sz[4];
    int x0, x1, y0, y1; // covered pixel range (inclusive)
    bool ok;
    bool near_clip;     // a corner has w <= 0: rasterised through clip_quad instead (ok is false)
};

inline Quad make_quad(const Raster& R, const float* p_k, const float* p_k1, float width_k, float rand_u) {
    Quad Q;
    Q.ok = false;
    const V3 a = mk(p_k[0], p_k[1], p_k[2]), b = mk(p_k1[0], p_k1[1], p_k1[2]);
    const float dist = length(mk(R.cam_pos[0], R.cam_pos[1], R.cam_pos[2]) - a);
    const float scale = rand_u * 0.075f * dist;
    const float w1 = scale * width_k;
    float c1[4], c2[4];
    const float pa[4] = {a.x, a.y, a.z, 1.f}, pb[4] = {b.x, b.y, b.z, 1.f};
    mul_vec4(R.vp, pa, c1);
    mul_vec4(R.vp, pb, c2);
    const float* src[4] = {c1, c1, c2, c2};
    const float off[4] = {-w1, w1, -w1, w1};
    Q.near_clip = false;
    bool behind = false, finite = true;
    for (int v = 0; v < 4; ++v) {
        Q.clip[v][0] = src[v][0] + off[v];
        Q.clip[v][1] = src[v][1];
        Q.clip[v][2] = src[v][2];
        Q.clip[v][3] = src[v][3];
        for (int e = 0; e < 4; ++e) finite = finite && std::isfinite(Q.clip[v][e]);
        behind = behind || !(Q.clip[v][3] > 0.f);
    }
    if (!finite) return Q;
    if (behind) {   // the triangles are clipped at the near plane (clip_quad)
        Q.near_clip = true;
        return Q;
    }
    float xmin = 3e38f, xmax = -3e38f, ymin = 3e38f, ymax = -3e38f;
    for (int v = 0; v < 4; ++v) {
        const float cw = Q.clip[v][3];
        Q.sx[v] = (Q.clip[v][0] / cw * 0.5f + 0.5f) * (float)R.width;
        Q.sy[v] = (Q.clip[v][1] / cw * 0.5f + 0.5f) * (float)R.height;
        Q.sz[v] = Q.clip[v][2] / cw;
        if (!std::isfinite(Q.sx[v]) || !std::isfinite(Q.sy[v]) || !std::isfinite(Q.sz[v])) return Q;
        xmin = std::fmin(xmin, Q.sx[v]);
        xmax = std::fmax(xmax, Q.sx[v]);
        ymin = std::fmin(ymin, Q.sy[v]);
        ymax = std::fmax(ymax, Q.sy[v]);
    }
    // pixel centres px + 0.5 in [xmin, xmax]
    const float fx0 = std::ceil(xmin - 0.5f), fx1 = std::floor(xmax - 0.5f);
    const float fy0 = std::ceil(ymin - 0.5f), fy1 = std::floor(ymax - 0.5f);
    const float cx0 = std::fmax(fx0, 0.f), cx1 = std::fmin(fx1, (float)(R.width - 1));
    const float cy0 = std::fmax(fy0, 0.f), cy1 = std::fmin(fy1, (float)(R.height - 1));
    if (cx0 > cx1 || cy0 > cy1) return Q;
    Q.x0 = (int)cx0;
    Q.x1 = (int)cx1;
    Q.y0 = (int)cy0;
    Q.y1 = (int)cy1;
    Q.ok = true;
    return Q;
}

inline float edge_fn(float ax, float ay, float bx, float by, float px, float py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
inline bool top_left(float ax, float ay, float bx, float by) {
    const float dy = by - ay, dx = bx - ax;
    return dy < 0.f || (dy == 0.f && dx > 0.f);
}

/* Coverage of pixel centre (px, py) by triangle (i0, i1, i2) of quad Q: the
 * barycentrics l[3] (in i0, i1, i2 order) and depth z; false when not covered. */
inline bool cover_tri(const Quad& Q, int i0, int i1, int i2, float px, float py, int idx[3], float l[3], float& z) {
    float area = edge_fn(Q.sx[i0], Q.sy[i0], Q.sx[i1], Q.sy[i1], Q.sx[i2], Q.sy[i2]);
    if (area == 0.f) return false;
    if (area < 0.f) {
        std::swap(i1, i2);
        area = -area;
    }
    const int v[3] = {i0, i1, i2};
    float e[3];
    for (int t = 0; t < 3; ++t) {   // edge t opposite vertex t: from v[t+1] to v[t+2]
        const int a = v[(t + 1) % 3], b = v[(t + 2) % 3];
        e[t] = edge_fn(Q.sx[a], Q.sy[a], Q.sx[b], Q.sy[b], px, py);
        if (e[t] < 0.f || (e[t] == 0.f && !top_left(Q.sx[a], Q.sy[a], Q.sx[b], Q.sy[b]))) return false;
    }
    for (int t = 0; t < 3; ++t) {
        l[t] = e[t] / area;
        idx[t] = v[t];
    }
    z = (l[0] * Q.sz[v[0]] + l[1] * Q.sz[v[1]]) + l[2] * Q.sz[v[2]];
    return z >= 0.f && z <= 1.f;
}

/* The nearest covering triangle of the quad at a pixel: 0 (none), 1 or 2. */
inline int cover_quad(const Quad& Q, int px, int py, int idx[3], float l[3], float& z) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    int ia[3], ib[3];
    float la[3], lb[3], za = 0.f, zb = 0.f;
    const bool a = cover_tri(Q, 0, 1, 2, cx, cy, ia, la, za);
    const bool b = cover_tri(Q, 2, 1, 3, cx, cy, ib, lb, zb);
    if (a && (!b || za <= zb)) {
        for (int t = 0; t < 3; ++t) idx[t] = ia[t], l[t] = la[t];
        z = za;
        return 1;
    }
    if (b) {
        for (int t = 0; t < 3; ++t) idx[t] = ib[t], l[t] = lb[t];
        z = zb;
        return 2;
    }
    return 0;
}

/* Near-plane clipping of a quad with a corner at w <= 0 (one behind the eye).
 * Each triangle, (V0, V1, V2) and (V2, V1, V3), is clipped in clip space to the
 * half-space z >= 0 (the near plane of a depth-zero-to-one projection, as Vulkan
 * clips: 0 <= z <= w) by Sutherland-Hodgman, corners in triangle order: a corner
 * with z >= 0 is kept, and an edge whose ends lie on opposite sides adds the
 * point at s = z_a / (z_a - z_b) from its first end, its z set to 0.  The 3 or 4
 * vertices are fanned into sub-triangles (v0, v1, v2), (v0, v2, v3), each covering
 * pixels with the same rules as an unclipped triangle; a vertex with w <= 0 after
 * the clip (possible only with a projection whose near plane is not z = 0) or
 * a non-finite screen position drops its triangle.  Vertex attributes are the
 * corners' lerped by s, interpolated perspective-correctly with the vertices' w.
 * The pixel box is that of every kept vertex, clamped to the target.  The depth
 * test and the [0, 1] depth range apply per fragment as before. */
struct ClipVert {
    float c[4];          // clip position
    float sx, sy, sz;    // screen position and depth
    int a, b;            // corners lerped: corner a + s (corner b - corner a)
    float s;
};
struct ClipQuad {
    ClipVert v[2][4];
    int nv[2];           // vertices of triangle 0 and 1 after the clip (0: dropped)
    int x0, x1, y0, y1;
    bool ok;
};

inline int clip_triangle(const Raster& R, const Quad& Q, const int tri[3], ClipVert out[4]) {
    int n = 0;
    for (int e = 0; e < 3; ++e) {
        const int a = tri[e], b = tri[(e + 1) % 3];
        const float za = Q.clip[a][2], zb = Q.clip[b][2];
        if (za >= 0.f) {
            ClipVert& o = out[n++];
            for (int q = 0; q < 4; ++q) o.c[q] = Q.clip[a][q];
            o.a = o.b = a;
            o.s = 0.f;
        }
        if ((za >= 0.f) != (zb >= 0.f)) {
            ClipVert& o = out[n++];
            const float t = za / (za - zb);
            for (int q = 0; q < 4; ++q) o.c[q] = Q.clip[a][q] + t * (Q.clip[b][q] - Q.clip[a][q]);
            o.c[2] = 0.f;
            o.a = a;
            o.b = b;
            o.s = t;
        }
    }
    if (n < 3) return 0;
    for (int v = 0; v < n; ++v) {
        ClipVert& o = out[v];
        const float cw = o.c[3];
        if (!(cw > 0.f)) return 0;
        o.sx = (o.c[0] / cw * 0.5f + 0.5f) * (float)R.width;
        o.sy = (o.c[1] / cw * 0.5f + 0.5f) * (float)R.height;
        o.sz = o.c[2] / cw;
        if (!std::isfinite(o.sx) || !std::isfinite(o.sy) || !std::isfinite(o.sz)) return 0;
    }
    return n;
}

inline ClipQuad clip_quad(const Raster& R, const Quad& Q) {
    ClipQuad C;
    C.ok = false;
    const int tris[2][3] = {{0, 1, 2}, {2, 1, 3}};
    float xmin = 3e38f, xmax = -3e38f, ymin = 3e38f, ymax = -3e38f;
    for (int t = 0; t < 2; ++t) {
        C.nv[t] = clip_triangle(R, Q, tris[t], C.v[t]);
        for (int v = 0; v < C.nv[t]; ++v) {
            xmin = std::fmin(xmin, C.v[t][v].sx);
            xmax = std::fmax(xmax, C.v[t][v].sx);
            ymin = std::fmin(ymin, C.v[t][v].sy);
            ymax = std::fmax(ymax, C.v[t][v].sy);
        }
    }
    if (C.nv[0] == 0 && C.nv[1] == 0) return C;
    const float fx0 = std::ceil(xmin - 0.5f), fx1 = std::floor(xmax - 0.5f);
    const float fy0 = std::ceil(ymin - 0.5f), fy1 = std::floor(ymax - 0.5f);
    const float cx0 = std::fmax(fx0, 0.f), cx1 = std::fmin(fx1, (float)(R.width - 1));
    const float cy0 = std::fmax(fy0, 0.f), cy1 = std::fmin(fy1, (float)(R.height - 1));
    if (cx0 > cx1 || cy0 > cy1) return C;
    C.x0 = (int)cx0;
    C.x1 = (int)cx1;
    C.y0 = (int)cy0;
    C.y1 = (int)cy1;
    C.ok = true;
    return C;
}

/* Coverage of pixel centre (px, py) by sub-triangle (i0, i1, i2) of a clipped
 * triangle's vertices: cover_tri's arithmetic on the vertices' screen positions. */
inline bool cover_sub(const ClipVert* V, int i0, int i1, int i2, float px, float py, int idx[3], float l[3], float& z) {
    float area = edge_fn(V[i0].sx, V[i0].sy, V[i1].sx, V[i1].sy, V[i2].sx, V[i2].sy);
    if (area == 0.f) return false;
    if (area < 0.f) {
        std::swap(i1, i2);
        area = -area;
    }
    const int v[3] = {i0, i1, i2};
    float e[3];
    for (int t = 0; t < 3; ++t) {
        const int a = v[(t + 1) % 3], b = v[(t + 2) % 3];
        e[t] = edge_fn(V[a].sx, V[a].sy, V[b].sx, V[b].sy, px, py);
        if (e[t] < 0.f || (e[t] == 0.f && !top_left(V[a].sx, V[a].sy, V[b].sx, V[b].sy))) return false;
    }
    for (int t = 0; t < 3; ++t) {
        l[t] = e[t] / area;
        idx[t] = v[t];
    }
    z = (l[0] * V[v[0]].sz + l[1] * V[v[1]].sz) + l[2] * V[v[2]].sz;
    return z >= 0.f && z <= 1.f;
}

/* Coverage by clipped triangle t of C: the first of its sub-triangles that covers. */
inline bool cover_clip_tri(const ClipQuad& C, int t, int px, int py, int idx[3], float l[3], float& z) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    if (C.nv[t] >= 3 && cover_sub(C.v[t], 0, 1, 2, cx, cy, idx, l, z)) return true;
    return C.nv[t] == 4 && cover_sub(C.v[t], 0, 2, 3, cx, cy, idx, l, z);
}

/* cover_quad for a clipped quad: 0 (none), 1 or 2, the nearer triangle (ties: the first). */
inline int cover_clip_quad(const ClipQuad& C, int px, int py, int idx[3], float l[3], float& z) {
    int ia[3], ib[3];
    float la[3], lb[3], za = 0.f, zb = 0.f;
    const bool a = cover_clip_tri(C, 0, px, py, ia, la, za);
    const bool b = cover_clip_tri(C, 1, px, py, ib, lb, zb);
    if (a && (!b || za <= zb)) {
        for (int t = 0; t < 3; ++t) idx[t] = ia[t], l[t] = la[t];
        z = za;
        return 1;
    }
    if (b) {
        for (int t = 0; t < 3; ++t) idx[t] = ib[t], l[t] = lb[t];
        z = zb;
        return 2;
    }
    return 0;
}

/* hair.geom's per-isoline width factor |random(3.242551 u, u u)| + 0.5 (:46). */
inline float geom_rand(float u, RefSin mode) { return std::fabs(frag_random(3.242551f * u, u * u, mode)) + 0.5f; }

/* hair.frag's inputs at corner c of segment (s, j, k)'s quad Q (V0, V1 take
 * vertex k's, V2, V3 vertex k + 1's). */
inline void corner_inputs(const float* verts, const float* frames, int n, int L, int S, const Raster& R, int s, int j,
                          int k, const Quad& Q, int c, float a[24]) {
    const int S1 = S + 1;
    const int kk = c < 2 ? k : k + 1;
    const float* p = verts + 4 * ((size_t(s) * L + j) * S1 + kk);
    const V3 pos = mk(p[0], p[1], p[2]);
    const float u = (float)j / (float)L, v = (float)kk / (float)S;
    const float x = v * (float)(n - 1);
    const int sf = std::min((int)std::floor(x), n - 2);
    const float* fr = frames + (size_t(s) * (n - 1) + sf) * 12;
    a[0] = u;
    a[1] = v;
    for (int q = 0; q < 3; ++q)
        for (int e = 0; e < 3; ++e) a[2 + 3 * q + e] = fr[4 * q + e];
    const V3 vd = normalize(mk(R.cam_pos[0], R.cam_pos[1], R.cam_pos[2]) - pos);
    const V3 ld = normalize(mk(R.light_pos[0], R.light_pos[1], R.light_pos[2]) - pos);
    a[11] = vd.x;
    a[12] = vd.y;
    a[13] = vd.z;
    a[14] = ld.x;
    a[15] = ld.y;
    a[16] = ld.z;
    mul_vec4(R.lmap, Q.clip[c], a + 17);
    a[21] = a[22] = a[23] = 0.f;
}

/* hair.frag's outColor for the fragment of segment (s, j, k)'s quad Q at a
 * pixel, covered by the quad's triangle with corners idx[] and barycentrics
 * l[]: the corners' inputs interpolated perspective-correctly. */
inline void segment_fragment(const float* verts, const float* frames, int n, int L, int S, const Raster& R,
                             const Maps& M, float bright, int s, int j, int k, const Quad& Q, const int idx[3],
                             const float l[3], float o[4]) {
    float attr[4][24];
    for (int c = 0; c < 4; ++c) corner_inputs(verts, frames, n, L, S, R, s, j, k, Q, c, attr[c]);
    const float q0 = l[0] / Q.clip[idx[0]][3], q1 = l[1] / Q.clip[idx[1]][3], q2 = l[2] / Q.clip[idx[2]][3];
    const float qs = (q0 + q1) + q2;
    float in[24];
    for (int e = 0; e < 24; ++e) in[e] = ((q0 * attr[idx[0]][e] + q1 * attr[idx[1]][e]) + q2 * attr[idx[2]][e]) / qs;
    in[0] = (float)j / (float)L;
    shade_fragment_bright(in, M, bright, o);
}

/* segment_fragment for a fragment of clipped triangle t of C (vertices idx[] of
 * C.v[t], barycentrics l[]).  A clipped vertex stands for corners a and b lerped
 * by s, so the perspective-correct interpolation is a weighted sum of the four
 * corners' inputs: w_c = the sum over the vertices of q_i = l_i / w_i times 1
 * (c = a = b), 1 - s (c = a) or s (c = b), accumulated vertex by vertex; the
 * inputs are (sum over c = 0..3 in order of w_c inputs_c) / (q_0 + q_1 + q_2). */
inline void segment_fragment_clip(const float* verts, const float* frames, int n, int L, int S, const Raster& R,
                                  const Maps& M, float bright, int s, int j, int k, const Quad& Q, const ClipQuad& C,
                                  int t, const int idx[3], const float l[3], float o[4]) {
    float attr[4][24];
    for (int c = 0; c < 4; ++c) corner_inputs(verts, frames, n, L, S, R, s, j, k, Q, c, attr[c]);
    float w[4] = {0.f, 0.f, 0.f, 0.f}, q[3];
    for (int i = 0; i < 3; ++i) {
        const ClipVert& V = C.v[t][idx[i]];
        q[i] = l[i] / V.c[3];
        if (V.a == V.b) {
            w[V.a] = w[V.a] + q[i];
        } else {
            w[V.a] = w[V.a] + q[i] * (1.0f - V.s);
            w[V.b] = w[V.b] + q[i] * V.s;
        }
    }
    const float qs = (q[0] + q[1]) + q[2];
    float in[24];
    for (int e = 0; e < 24; ++e) {
        float acc = w[0] * attr[0][e];
        for (int c = 1; c < 4; ++c) acc = acc + w[c] * attr[c][e];
        in[e] = acc / qs;
    }
    in[0] = (float)j / (float)L;
    shade_fragment_bright(in, M, bright, o);
}

/* Per-isoline factors: hair.geom's width factor and hair.frag's brightness. */
inline void isoline_factors(int L, RefSin mode, std::vector<float>& rnd, std::vector<float>& bright) {
    rnd.resize(L);
    bright.resize(L);
    for (int j = 0; j < L; ++j) {
        const float u = (float)j / (float)L;
        rnd[j] = geom_rand(u, mode);
        bright[j] = 0.8f * std::fabs(frag_random(u, u, mode)) + 0.6f;
    }
}

/* The camera image of a tessellation (vertices ns x L x (S+1) float4, frames
 * ns x (n-1) x 3 float4) shaded with hair.frag over the given maps; ids (nullable)
 * receives the winning segment id per pixel, 0xffffffff where none. */
inline void render_hair(const float* verts, const float* frames, int ns, int n, int L, int S, const Raster& R,
                        const Maps& M, RefSin mode, float* image, uint32_t* ids) {
    const int W = R.width, H = R.height;
    std::vector<uint64_t> key(size_t(W) * H, ~0ull);
    std::vector<float> rnd, bright;
    isoline_factors(L, mode, rnd, bright);
    const int S1 = S + 1;
    auto vert = [&](int s, int j, int k) { return verts + 4 * ((size_t(s) * L + j) * S1 + k); };
    const long long nseg = (long long)ns * L * S;
    for (long long id = 0; id < nseg; ++id) {
        const int k = int(id % S);
        const long long line = id / S;
        const int j = int(line % L), s = int(line / L);
        const float* pk = vert(s, j, k);
        const Quad Q = make_quad(R, pk, vert(s, j, k + 1), pk[3], rnd[j]);
        const ClipQuad C = Q.near_clip ? clip_quad(R, Q) : ClipQuad{};
        if (!Q.ok && !(Q.near_clip && C.ok)) continue;
        const int x0 = Q.ok ? Q.x0 : C.x0, x1 = Q.ok ? Q.x1 : C.x1, y0 = Q.ok ? Q.y0 : C.y0, y1 = Q.ok ? Q.y1 : C.y1;
        for (int py = y0; py <= y1; ++py)
            for (int px = x0; px <= x1; ++px) {
                int idx[3];
                float l[3], z;
                if (!(Q.ok ? cover_quad(Q, px, py, idx, l, z) : cover_clip_quad(C, px, py, idx, l, z))) continue;
                uint32_t zb;
                std::memcpy(&zb, &z, 4);
                const uint64_t kk = (uint64_t(zb) << 32) | uint64_t(uint32_t(id));
                uint64_t& t = key[size_t(py) * W + px];
                if (kk < t) t = kk;
            }
    }
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const size_t p = size_t(py) * W + px;
            float* out = image + 4 * p;
            if (key[p] == ~0ull) {
                out[0] = out[1] = out[2] = out[3] = 0.f;
                if (ids) ids[p] = 0xffffffffu;
                continue;
            }
            const uint32_t id = uint32_t(key[p] & 0xffffffffu);
            if (ids) ids[p] = id;
            const int k = int(id % S);
            const long long line = id / S;
            const int j = int(line % L), s = int(line / L);
            const float* pk = vert(s, j, k);
            const Quad Q = make_quad(R, pk, vert(s, j, k + 1), pk[3], rnd[j]);
            int idx[3];
            float l[3], z;
            if (Q.ok) {
                cover_quad(Q, px, py, idx, l, z);
                segment_fragment(verts, frames, n, L, S, R, M, bright[j], s, j, k, Q, idx, l, out);
            } else {
                const ClipQuad C = clip_quad(R, Q);
                const int t = cover_clip_quad(C, px, py, idx, l, z) - 1;
                segment_fragment_clip(verts, frames, n, L, S, R, M, bright[j], s, j, k, Q, C, t, idx, l, out);
            }
        }
}

/* The hair pass as the reference's pipeline draws it (src/Renderer.cpp:1657-1679):
 * segments in order, each quad's triangles (V0, V1, V2) then (V2, V1, V3); a
 * fragment passes the LESS depth test against the depth the fragments before it
 * wrote (cleared to 1.0, Renderer.cpp:2236), writes its depth and blends
 * SRC_ALPHA / ONE_MINUS_SRC_ALPHA into the colour, ONE / ONE into the alpha
 * (clamped to 1, as the unorm target clamps), hair.frag's alpha being 0.75.
 * The colour starts at clear_rgba (the reference clears to (101, 129, 140,
 * 255) / 255 and draws the head mesh first; here the hair alone is drawn) and
 * is kept in float (the reference's 8-bit swapchain rounds every write).
 * ids (nullable): the last fragment written per pixel (its nearest), or
 * 0xffffffff. */
inline void render_hair_blend(const float* verts, const float* frames, int ns, int n, int L, int S, const Raster& R,
                              const Maps& M, RefSin mode, const float clear_rgba[4], float* image, uint32_t* ids) {
    const int W = R.width, H = R.height;
    std::vector<float> depth(size_t(W) * H, 1.0f);
    for (size_t p = 0; p < size_t(W) * H; ++p) {
        for (int c = 0; c < 4; ++c) image[4 * p + c] = clear_rgba[c];
        if (ids) ids[p] = 0xffffffffu;
    }
    std::vector<float> rnd, bright;
    isoline_factors(L, mode, rnd, bright);
    const int S1 = S + 1;
    auto vert = [&](int s, int j, int k) { return verts + 4 * ((size_t(s) * L + j) * S1 + k); };
    const long long nseg = (long long)ns * L * S;
    for (long long id = 0; id < nseg; ++id) {
        const int k = int(id % S);
        const long long line = id / S;
        const int j = int(line % L), s = int(line / L);
        const float* pk = vert(s, j, k);
        const Quad Q = make_quad(R, pk, vert(s, j, k + 1), pk[3], rnd[j]);
        const ClipQuad C = Q.near_clip ? clip_quad(R, Q) : ClipQuad{};
        if (!Q.ok && !(Q.near_clip && C.ok)) continue;
        const int x0 = Q.ok ? Q.x0 : C.x0, x1 = Q.ok ? Q.x1 : C.x1, y0 = Q.ok ? Q.y0 : C.y0, y1 = Q.ok ? Q.y1 : C.y1;
        for (int tri = 0; tri < 2; ++tri)
            for (int py = y0; py <= y1; ++py)
                for (int px = x0; px <= x1; ++px) {
                    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
                    int idx[3];
                    float l[3], z;
                    const bool cov = !Q.ok ? cover_clip_tri(C, tri, px, py, idx, l, z)
                                     : tri == 0 ? cover_tri(Q, 0, 1, 2, cx, cy, idx, l, z)
                                                : cover_tri(Q, 2, 1, 3, cx, cy, idx, l, z);
                    const size_t p = size_t(py) * W + px;
                    if (!cov || !(z < depth[p])) continue;
                    depth[p] = z;
                    float c[4];
                    if (Q.ok) segment_fragment(verts, frames, n, L, S, R, M, bright[j], s, j, k, Q, idx, l, c);
                    else segment_fragment_clip(verts, frames, n, L, S, R, M, bright[j], s, j, k, Q, C, tri, idx, l, c);
                    float* out = image + 4 * p;
                    const float ia = 1.0f - c[3];
                    for (int e = 0; e < 3; ++e) out[e] = c[e] * c[3] + out[e] * ia;
                    out[3] = std::min(1.0f, c[3] + out[3]);
                    if (ids) ids[p] = uint32_t(id);
                }
    }
}


/* The light camera as the geometry shader's camera: the shadow and opacity passes
 * bind it at set 0 (src/Renderer.cpp:2147-2160, 2203-2216), so quads are expanded
 * with the light's projection and the distance to the light, and a fragment's
 * light-space position lightProj * lightView * inverse(lightView) *
 * inverse(lightProj) * V is V itself (taken exactly). */
inline bool make_light_raster(const float* light_view, const float* light_proj, int w, int h, Raster& R) {
    double lv[16], lp[16], vp[16];
    for (int k = 0; k < 16; ++k) {
        lv[k] = light_view[k];
        lp[k] = light_proj[k];
    }
    mul4d(lp, lv, vp);
    for (int k = 0; k < 16; ++k) {
        R.vp[k] = float(vp[k]);
        R.lmap[k] = (k % 5 == 0) ? 1.f : 0.f;
    }
    eye_of(light_view, R.cam_pos);
    eye_of(light_view, R.light_pos);
    R.width = w;
    R.height = h;
    return true;
}

/* Light depth and deep opacity maps from hair.geom's quads rasterised in the
 * light's view: the depth pass keeps each texel's nearest fragment
 * (LESS_OR_EQUAL, cleared to 1.0); the opacity pass has no depth attachment, so
 * every fragment adds to the layer its depth falls in relative to the depth map
 * sampled at its light-space position (hairOpacity.frag:36-59), saturating as in
 * light_maps.  That position is the fragment's own (the light camera is the
 * geometry shader's camera here): its pixel centre and its rasterised depth. */
inline void light_maps_quads(const float* verts, int ns, int L, int S, const Raster& R, RefSin mode, float* depth,
                             float* opacity) {
    const int W = R.width, H = R.height;
    const size_t texels = size_t(W) * H;
    std::fill(depth, depth + texels, 1.0f);
    std::vector<float> rnd(L);
    for (int j = 0; j < L; ++j) rnd[j] = geom_rand((float)j / (float)L, mode);
    const int S1 = S + 1;
    auto vert = [&](int s, int j, int k) { return verts + 4 * ((size_t(s) * L + j) * S1 + k); };
    const long long nseg = (long long)ns * L * S;
    for (int pass = 0; pass < 2; ++pass) {
        std::vector<uint32_t> count(pass == 1 ? texels * 3 : 0, 0);
        for (long long id = 0; id < nseg; ++id) {
            const int k = int(id % S);
            const long long line = id / S;
            const int j = int(line % L), s = int(line / L);
            const float* pk = vert(s, j, k);
            const Quad Q = make_quad(R, pk, vert(s, j, k + 1), pk[3], rnd[j]);
            const ClipQuad C = Q.near_clip ? clip_quad(R, Q) : ClipQuad{};
            if (!Q.ok && !(Q.near_clip && C.ok)) continue;
            const int x0 = Q.ok ? Q.x0 : C.x0, x1 = Q.ok ? Q.x1 : C.x1, y0 = Q.ok ? Q.y0 : C.y0, y1 = Q.ok ? Q.y1 : C.y1;
            for (int py = y0; py <= y1; ++py)
                for (int px = x0; px <= x1; ++px) {
                    int idx[3];
                    float l[3], z;
                    if (!(Q.ok ? cover_quad(Q, px, py, idx, l, z) : cover_clip_quad(C, px, py, idx, l, z))) continue;
                    const size_t t = size_t(py) * W + px;
                    if (pass == 0) {
                        if (z < depth[t]) depth[t] = z;
                        continue;
                    }
                    // the fragment's light-space position is its own: texture coordinates at the
                    // pixel centre, depth the rasterised one (what the perspective-correct
                    // interpolation of V and the divide by w give in exact arithmetic)
                    const float u = ((float)px + 0.5f) / (float)W, v = ((float)py + 0.5f) / (float)H;
                    const int layer = opacity_layer(z, sample(depth, W, H, 1, u, v, 0));
                    uint32_t* cnt = count.data() + t * 3;
                    if (layer == 1) cnt[0]++;
                    if (layer == 1 || layer == 2) cnt[1]++;
                    if (layer != 0) cnt[2]++;
                }
        }
        if (pass == 1)
            for (size_t t = 0; t < texels; ++t) {
                for (int l = 0; l < 3; ++l) {
                    const uint32_t c = count[t * 3 + l];
                    opacity[t * 4 + l] = (float)(c >= 4 ? 255u : (uint32_t)kLayerUnit * c) / 255.0f;
                }
                opacity[t * 4 + 3] = 0.f;
            }
    }
}

}  // namespace shade
}  // namespace oracle
