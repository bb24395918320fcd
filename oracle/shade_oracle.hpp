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
inline void shade_fragment(const float* in, const Maps& M, RefSin mode, float out[4]) {
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
    const float bright = 0.8f * std::fabs(frag_random(in[0], in[0], mode)) + 0.6f;
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

}  // namespace shade
}  // namespace oracle
