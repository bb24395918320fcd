// rvh_shade.cu — hair shading of tessellated strands into headless buffers.
//
// The reference shades hair in three graphics passes (src/Renderer.cpp): the
// hair drawn from the shadow camera into a depth map cleared to 1.0; an
// opacity pass (hairOpacity.frag) adding 0.3 per fragment to three layers
// behind the first surface z0, at z0 + [0, d), [d, 2d), [2d, ...) with d =
// 0.3, into the swapchain's 8-bit unorm format with additive blending; then
// the camera pass, hair.frag per fragment: a Marschner-style R / TT / TRT
// single-scattering lobe in the strand's frame, a multiple-scattering term
// damped by the opacity layer the fragment falls in, a 7x7 PCF shadow test,
// an ambient term and a per-isoline brightness hash.  Without a graphics
// pipeline these are CUDA kernels over the tessellated vertices
// (rvh_asset_tessellate), each vertex one fragment covering one texel:
//
//   k_clear_maps      depth = 1.0, layer counts = 0
//   k_light_depth     nearest light-space depth per texel (atomic min of the bits)
//   k_light_opacity   each vertex counted into the layer its depth falls in,
//                     relative to the bilinear z0 at its position
//   k_opacity_finish  layer value = min(255, 77 count) / 255 (0.3 as unorm8,
//                     saturating sum), in place over the counts
//   k_shade_vertices  hair.frag's colour per vertex (k_shade_fragments: per
//                     caller-given fragment inputs)
//   k_image_*         optional camera image: nearest vertex per pixel
//
// The maps live in L2 (the reference's 1080 x 720: 3.1 MB of depth, 12.4 MB
// of layers); the vertex passes stream the tessellated vertices from HBM.
// Samplers are clamp-to-edge bilinear with texel centres at (i + 0.5) / size
// (the reference's VK_FILTER_LINEAR + CLAMP_TO_EDGE samplers,
// src/Renderer.cpp:14,1899-1902).  The brightness hash uses a correctly
// rounded sin, as the tessellation does.  Float arithmetic is separately
// rounded in the shader's order; acos, sin, cos, exp and pow are CUDA's, so
// colours agree with a host evaluation to a few float ulps of those functions
// while the maps, every comparison against them and the camera image's
// depth test agree bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "rvh_internal.hpp"
#include "rvh_registry.h"

namespace rvh {
namespace {

constexpr int kShadeThreads = 256;
constexpr float kPi = 3.14159265359f;
constexpr float kPiOver2 = 1.57079632679f;
constexpr float kRadToDeg = 57.2957795131f;
constexpr float kDegToRad = 0.01745329251f;
constexpr float kEps = 0.001f;

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float len3(V3 a) { return sqrtf(dot3(a, a)); }
// glm normalize: v * inversesqrt(dot(v, v)), inversesqrt = 1 / sqrt
__device__ __forceinline__ V3 nrm3(V3 a) { return a * (1.0f / sqrtf(dot3(a, a))); }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ---- hair.frag's helper functions (src/shaders/hair.frag:24-124) ----------------------
__device__ __forceinline__ bool vec3_compare(V3 a, V3 b) {
    return fabsf(a.x - b.x) < kEps && fabsf(a.y - b.y) < kEps && fabsf(a.z - b.z) < kEps;
}
__device__ __forceinline__ float angle_vector_plane(V3 v, V3 n) {
    float angle = acosf(dot3(v, n) / (len3(v) * len3(n)));
    if (angle < kPiOver2) angle = kPiOver2 - angle;
    else angle = -(angle - kPiOver2);
    return angle;
}
__device__ __forceinline__ V3 project_onto_plane(V3 v, V3 n) { return v - dot3(v, n) * n; }
__device__ __forceinline__ float directional_angle(V3 v1, V3 v2, V3 n) {
    const float angle = acosf(dot3(v1, v2) / (len3(v1) * len3(v2)));
    if (vec3_compare(nrm3(cross3(v2, v1)), n)) return angle;
    return (2.0f * kPi) - angle;
}
// gaussian(alpha, beta, theta_i, theta_o) with sin_i = sin(theta_i DEG_TO_RAD),
// sin_o = sin(theta_o DEG_TO_RAD) computed once for the three lobes;
// pow(e, 2) is e * e (the correctly rounded square)
__device__ __forceinline__ float gaussian(float alpha, float beta, float sin_i, float sin_o) {
    const float e = sin_i + sin_o - alpha;
    return (1.f / (beta * sqrtf(2.f * kPi))) * expf(-(e * e) / (2.f * beta * beta));
}
// pow(1 - x, 5) as ((y^2)^2) y
__device__ __forceinline__ float schlicks(float n, float x) {
    const float R0 = ((1.f - n) * (1.f - n)) / ((1.f + n) * (1.f + n));
    const float y = 1.f - x, y2 = y * y;
    return R0 + (1.f - R0) * ((y2 * y2) * y);
}
// GLSL's pow(x, y) = exp2(y log2(x)) for the constant bases of the hair colour:
// log2 of midBrown / 255 and of midBrown / 255 / luma, each computed in double
// from the float base and rounded once.
constexpr float kLog2C[3] = {-0x1.560d64p+0f, -0x1.eda2b8p+0f, -0x1.799844p+1f};
constexpr float kLog2CLuma[3] = {0x1.9a7186p-2f, -0x1.87c794p-3f, -0x1.3686c2p+0f};
// GLSL clamp(x, 0, 1) = min(max(x, 0), 1) with max(a, b) = a < b ? b : a and
// min(a, b) = b < a ? b : a: a NaN passes through, as in the shader.
__device__ __forceinline__ float clamp01(float x) {
    const float m = x < 0.f ? 0.f : x;
    return 1.f < m ? 1.f : m;
}
__device__ __forceinline__ float shade_hash(float x, float y) {   // random(), correctly rounded sin
    const float d = x * 12.9898f + y * 78.233f;
    const float m = (float)sin((double)d) * 43758.5453123f;
    return m - floorf(m);
}

// Clamp-to-edge bilinear sample of channel c of a (w x h x ch) float image.
__device__ __forceinline__ float tex_texel(const float* img, int w, int h, int ch, int x, int y, int c) {
    x = min(max(x, 0), w - 1);
    y = min(max(y, 0), h - 1);
    return __ldg(img + ((size_t)y * w + x) * ch + c);
}
__device__ __forceinline__ float tex_sample(const float* img, int w, int h, int ch, float u, float v, int c) {
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    // texel indices clamped before the conversion (only the clamp to edge reads them);
    // keeps an infinite or NaN coordinate defined
    const int ix = (int)fminf(fmaxf(x0, -1.f), (float)w), iy = (int)fminf(fmaxf(y0, -1.f), (float)h);
    const float t00 = tex_texel(img, w, h, ch, ix, iy, c), t10 = tex_texel(img, w, h, ch, ix + 1, iy, c);
    const float t01 = tex_texel(img, w, h, ch, ix, iy + 1, c), t11 = tex_texel(img, w, h, ch, ix + 1, iy + 1, c);
    const float a = t00 + fx * (t10 - t00);
    const float b = t01 + fx * (t11 - t01);
    return a + fy * (b - a);
}

struct Maps {
    const float* depth;     // w x h
    const float* opacity;   // w x h x 4 (layers r, g, b)
    int w, h;
};

// PCFshadowCalculation (hair.frag:99-125): the shader's texel size is fixed at
// 1/1080 x 1/720.  Each of the 7 x 7 taps is a bilinear sample at (u + dx ts_x,
// v + dy ts_y); when the taps' texel columns are 7 consecutive integers and so
// are their rows (the usual case: a tap step is one texel of a 1080 x 720 map),
// the taps share one 8 x 8 window of texels, loaded once (64 loads instead of
// 196) and walked two rows at a time; every tap's arithmetic is unchanged.
// center receives the (0, 0) tap (= the shader's z0 sample) when computed.
__device__ __forceinline__ float tap_coord(float c, int size, int& i) {
    const float x = c * (float)size - 0.5f;
    const float x0 = floorf(x);
    i = (int)fminf(fmaxf(x0, -1.f), (float)size);
    return x - x0;
}

__device__ float pcf_shadow(const Maps& M, float px, float py, float pz, float pw, float& center, bool& has_center) {
    has_center = false;
    const float x = px / pw, y = py / pw, z = pz / pw;
    if (fabsf(x) > 1.f || fabsf(y) > 1.f || fabsf(z) > 1.f) return 0.f;
    const float u = x * 0.5f + 0.5f, v = y * 0.5f + 0.5f;
    const float tsx = 1.f / 1080.0f, tsy = 1.f / 720.0f;
    // the taps' texel columns and rows: consecutive from the first?
    float fx[7];
    int ix0, iy0;
    fx[0] = tap_coord(u + (float)(-3) * tsx, M.w, ix0);
    (void)tap_coord(v + (float)(-3) * tsy, M.h, iy0);
    bool window = true;
#pragma unroll
    for (int d = 1; d < 7; ++d) {
        int i, j;
        fx[d] = tap_coord(u + (float)(d - 3) * tsx, M.w, i);
        (void)tap_coord(v + (float)(d - 3) * tsy, M.h, j);
        window = window && i == ix0 + d && j == iy0 + d;
    }
    float lighted = 0.f;
    if (window) {
        // h[dx] = the horizontal lerp a = t00 + fx (t10 - t00) of row r for tap
        // column dx; tap (dx, dy) is hprev[dx] + fy (hcur[dx] - hprev[dx]) with
        // rows iy0 + dy and iy0 + dy + 1, the same operands as the shader's
        // sample, so each row's lerps serve two rows of taps
        int col[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) col[c] = min(max(ix0 + c, 0), M.w - 1);
        float hprev[7];
        {
            const float* row = M.depth + (size_t)min(max(iy0, 0), M.h - 1) * M.w;
            float t[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) t[c] = __ldg(row + col[c]);
#pragma unroll
            for (int dx = 0; dx < 7; ++dx) hprev[dx] = t[dx] + fx[dx] * (t[dx + 1] - t[dx]);
        }
#pragma unroll 1
        for (int dy = 0; dy < 7; ++dy) {
            int iy;
            const float fy = tap_coord(v + (float)(dy - 3) * tsy, M.h, iy);
            const float* row = M.depth + (size_t)min(max(iy0 + dy + 1, 0), M.h - 1) * M.w;
            float t[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) t[c] = __ldg(row + col[c]);
#pragma unroll
            for (int dx = 0; dx < 7; ++dx) {
                const float hcur = t[dx] + fx[dx] * (t[dx + 1] - t[dx]);
                const float tap = hprev[dx] + fy * (hcur - hprev[dx]);
                if (z > tap) lighted += 1.f;
                if (dx == 3 && dy == 3) center = tap;
                hprev[dx] = hcur;
            }
        }
        has_center = true;
    } else {
        for (int dx = -3; dx <= 3; ++dx)
            for (int dy = -3; dy <= 3; ++dy) {
                const float cu = u + (float)dx * tsx, cv = v + (float)dy * tsy;
                if (z > tex_sample(M.depth, M.w, M.h, 1, cu, cv, 0)) lighted += 1.f;
            }
    }
    const float kernel = 2.f * 3 + 1.f;
    return lighted / (kernel * kernel);
}

// hair.frag main (:133-262) for one fragment.  in: uv (2), u, v, w (3 each),
// viewDir (3), lightDir (3), fragPosLightSpace (4).
// bright: the brightness factor 0.8 |random(uv.x, uv.x)| + 0.6 when the caller
// has it (a per-isoline table), else negative and computed here.
__device__ float4 shade_fragment(const float* in, const Maps& M, float bright) {
    const float uv_x = in[0];   // in_uv.y only feeds hair.frag's unused colour gradient (:228-232)
    const V3 fu = mk(in[2], in[3], in[4]), fv = mk(in[5], in[6], in[7]);
    const V3 view = mk(in[11], in[12], in[13]), light = mk(in[14], in[15], in[16]);
    const float px = in[17], py = in[18], pz = in[19], pw = in[20];
    const float over255 = 1.0f / 255.0f;
    const V3 w_i = nrm3(light);
    const V3 w_o = nrm3(view);
    const float n = 1.55f;
    const V3 C = mk(101.0f, 67.0f, 33.0f) * over255;   // midBrown
    const float roughness = 0.2f, shift = 0.01f;
    const float theta_i = angle_vector_plane(w_i, fu) * kRadToDeg;
    const float theta_o = angle_vector_plane(w_o, fu) * kRadToDeg;
    const float phi_i = directional_angle(nrm3(project_onto_plane(w_i, fu)), fv, fu) * kRadToDeg;
    const float phi_o = directional_angle(nrm3(project_onto_plane(w_o, fu)), fv, fu) * kRadToDeg;
    const float theta_d = (theta_o - theta_i) / 2.f;
    const float phi_d = phi_o - phi_i;
    const float alpha_R = -2.f * shift, alpha_TT = shift, alpha_TRT = 4.f * shift;
    const float beta_R = roughness * roughness, beta_TT = 0.5f * beta_R, beta_TRT = 2.f * beta_R;
    const float sin_i = sinf(theta_i * kDegToRad), sin_o = sinf(theta_o * kDegToRad);
    const float M_R = gaussian(alpha_R, beta_R, sin_i, sin_o);
    const float M_TT = gaussian(alpha_TT, beta_TT, sin_i, sin_o);
    const float M_TRT = gaussian(alpha_TRT, beta_TRT, sin_i, sin_o);
    const float cosTheta_d = cosf(theta_d * kDegToRad);
    const float cosPhi_d = cosf(phi_d * kDegToRad);
    const float cosPhi_dOver2 = cosf((phi_d / 2.f) * kDegToRad);
    const float nR = schlicks(n, sqrtf(0.5f + 0.5f * dot3(w_i, w_o))) * (0.25f * sqrtf(0.5f + 0.5f * cosPhi_d));
    const V3 N_R = mk(nR, nR, nR);
    const float n_prime = (1.19f / cosTheta_d) + 0.36f * cosTheta_d;
    const float a = 1.f / n_prime;
    const float h_TT = (1.f + a * (0.6f - 0.8f * cosPhi_d)) * cosPhi_dOver2;
    const float f_TT = schlicks(n, cosTheta_d * sqrtf(1.f - h_TT * h_TT));
    const float Cpower_TT = sqrtf(1.f - h_TT * h_TT * a * a) / (2.f * cosTheta_d);
    const V3 T_TT = mk(exp2f(Cpower_TT * kLog2C[0]), exp2f(Cpower_TT * kLog2C[1]), exp2f(Cpower_TT * kLog2C[2]));
    const V3 A_TT = (1.f - f_TT) * (1.f - f_TT) * T_TT;
    const float D_TT = expf(-3.65f * cosPhi_d - 3.98f);
    const V3 N_TT = A_TT * D_TT;
    const V3 N_TRT = A_TT * D_TT;   // the shader reuses the TT lobe here (hair.frag:236)
    const V3 S_single = (1.3f * N_R * M_R + 0.5f * N_TT * M_TT + N_TRT * M_TRT) / (cosTheta_d * cosTheta_d);
    float z0;
    bool has_z0;
    const float shadow = pcf_shadow(M, px, py, pz, pw, z0, has_z0);
    const float x = px / pw, y = py / pw, currentDepth = pz / pw;
    const float u = x * 0.5f + 0.5f, v = y * 0.5f + 0.5f;
    if (!has_z0) z0 = tex_sample(M.depth, M.w, M.h, 1, u, v, 0);
    const float d = 0.3f;
    float opacity = 0.f;
    if (currentDepth >= z0 && currentDepth < z0 + d) opacity = tex_sample(M.opacity, M.w, M.h, 4, u, v, 0);
    else if (currentDepth >= z0 + d && currentDepth < z0 + 2.f * d) opacity = tex_sample(M.opacity, M.w, M.h, 4, u, v, 1);
    else if (currentDepth >= z0 + 2.f * d) opacity = tex_sample(M.opacity, M.w, M.h, 4, u, v, 2);
    const V3 fakeNormal = nrm3(w_o - fu * dot3(fu, w_o));
    const float oe = 1.f - opacity;
    const V3 Cexp = mk(exp2f(oe * kLog2CLuma[0]), exp2f(oe * kLog2CLuma[1]), exp2f(oe * kLog2CLuma[2]));
    const V3 sqrtC = mk(sqrtf(C.x), sqrtf(C.y), sqrtf(C.z));
    const V3 S_multi = sqrtC * ((dot3(fakeNormal, w_i) + 1.f) / (4.f * kPi)) * Cexp;
    if (bright < 0.f) bright = 0.8f * fabsf(shade_hash(uv_x, uv_x)) + 0.6f;
    const V3 col = ((S_single + S_multi) * (1.f - shadow) + 0.3f * C) * bright;
    return make_float4(clamp01(col.x), clamp01(col.y), clamp01(col.z), 0.75f);
}

__global__ void __launch_bounds__(kShadeThreads) k_shade_fragments(long long n, const float* __restrict__ in, Maps M,
                                                                   float4* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * kShadeThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kShadeThreads)
        out[i] = shade_fragment(in + (size_t)i * 24, M, -1.f);
}

// ---- the maps and per-vertex shading from tessellated strands ---------------------------
struct Proj {
    float m[16];        // column-major projection * view
};
constexpr int kMaxLines = 64;
struct Lines {
    float bright[kMaxLines];   // 0.8 |random(u, u)| + 0.6 of isoline u = j / n_lines
};
struct Cam {
    float lvp[16];      // light proj * light view (column-major)
    float cam_pos[3];   // eye of the camera view
    float light_pos[3]; // eye of the light view
};

__device__ __forceinline__ void mul_point(const float* m, V3 p, float& x, float& y, float& z, float& w) {
    x = ((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12];
    y = ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13];
    z = ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14];
    w = ((m[3] * p.x + m[7] * p.y) + m[11] * p.z) + m[15];
}

// The texel a vertex covers in a (w x h) target of projection m, its depth and
// map coordinates; false outside the clip volume, where a rasteriser clips it.
__device__ __forceinline__ bool project_texel(const float* m, V3 p, int w, int h, int& tx, int& ty, float& depth,
                                              float& u, float& v) {
    float x, y, z, ww;
    mul_point(m, p, x, y, z, ww);
    if (!(ww > 0.f)) return false;
    x = x / ww;
    y = y / ww;
    z = z / ww;
    if (fabsf(x) > 1.f || fabsf(y) > 1.f || z < 0.f || z > 1.f) return false;
    u = x * 0.5f + 0.5f;
    v = y * 0.5f + 0.5f;
    tx = min((int)(u * (float)w), w - 1);
    ty = min((int)(v * (float)h), h - 1);
    depth = z;
    return true;
}

// Passes 1 and 2 walk the vertices by (strand s, vertex k) over the isolines
// j: a lane's vertices (s, j, k) for consecutive j are often in one texel (the
// isolines of a strand clump together near its root), so a lane folds runs of
// equal texels before its atomic; lanes of a warp read consecutive k of one
// isoline at a time (coalesced).
struct VertexWalk {
    const float4* verts;
    long long n_columns;   // n_strands * (n_segments + 1)
    int n_lines, s1;
};
__device__ __forceinline__ const float4* column_base(const VertexWalk& W, long long q) {
    const long long s = q / W.s1;
    const int k = (int)(q - s * W.s1);
    return W.verts + s * W.n_lines * W.s1 + k;
}

constexpr int kChunk = 4;   // vertices of a column loaded together

// Pass 1: nearest light depth per texel (z in [0, 1]: the bits order like the
// values).  A texel's value only decreases, so a flush whose minimum is not
// below the value it reads has nothing to do and skips the atomic.
__device__ __forceinline__ void flush_min(unsigned* texel, unsigned best) {
    if (best < *reinterpret_cast<volatile unsigned*>(texel)) atomicMin(texel, best);
}

__global__ void __launch_bounds__(kShadeThreads) k_light_depth(VertexWalk W, Cam K, int w, int h,
                                                               unsigned* __restrict__ depth_bits) {
    for (long long q = (long long)blockIdx.x * kShadeThreads + threadIdx.x; q < W.n_columns;
         q += (long long)gridDim.x * kShadeThreads) {
        const float4* v = column_base(W, q);
        long long cur = -1;
        unsigned best = 0u;
        for (int j0 = 0; j0 < W.n_lines; j0 += kChunk) {
            float4 p[kChunk];
#pragma unroll
            for (int c = 0; c < kChunk; ++c)
                if (j0 + c < W.n_lines) p[c] = __ldg(v + (size_t)(j0 + c) * W.s1);
#pragma unroll
            for (int c = 0; c < kChunk; ++c) {
                if (j0 + c >= W.n_lines) break;
                int tx, ty;
                float z, u, vv;
                if (!project_texel(K.lvp, mk(p[c].x, p[c].y, p[c].z), w, h, tx, ty, z, u, vv)) continue;
                const long long t = (long long)ty * w + tx;
                const unsigned bits = __float_as_uint(z);
                if (t == cur) {
                    best = min(best, bits);
                } else {
                    if (cur >= 0) flush_min(depth_bits + cur, best);
                    cur = t;
                    best = bits;
                }
            }
        }
        if (cur >= 0) flush_min(depth_bits + cur, best);
    }
}

// Pass 2: fragments per opacity layer (hairOpacity.frag:36-59), counted per
// texel in one 64-bit word: n1, n2, n3 = fragments in [z0, z0 + d), [z0 + d,
// z0 + 2d), [z0 + 2d, ...) in 21-bit fields.  A layer value saturates at 4
// fragments (4 x 77 > 255), so a field only needs to reach 4: a flush adds
// at most 4 per field and skips fields already at 4 or more, which bounds a
// field by 4 + 4 x (flushes in flight) < 2^21.
constexpr int kFieldBits = 21;
constexpr unsigned long long kFieldMask = (1ull << kFieldBits) - 1ull;

__device__ __forceinline__ void add_counts(unsigned long long* word, unsigned n1, unsigned n2, unsigned n3) {
    const unsigned long long seen = *reinterpret_cast<volatile unsigned long long*>(word);
    if ((seen & kFieldMask) >= 4u) n1 = 0u;
    if (((seen >> kFieldBits) & kFieldMask) >= 4u) n2 = 0u;
    if (((seen >> (2 * kFieldBits)) & kFieldMask) >= 4u) n3 = 0u;
    const unsigned long long add = (unsigned long long)min(n1, 4u) |
                                   ((unsigned long long)min(n2, 4u) << kFieldBits) |
                                   ((unsigned long long)min(n3, 4u) << (2 * kFieldBits));
    if (add) atomicAdd(word, add);
}

__global__ void __launch_bounds__(kShadeThreads) k_light_opacity(VertexWalk W, Cam K, int w, int h,
                                                                 const float* __restrict__ depth,
                                                                 uint4* __restrict__ counts) {
    auto* words = reinterpret_cast<unsigned long long*>(counts);   // texel t: words[2 t]
    for (long long q = (long long)blockIdx.x * kShadeThreads + threadIdx.x; q < W.n_columns;
         q += (long long)gridDim.x * kShadeThreads) {
        const float4* v = column_base(W, q);
        long long cur = -1;
        unsigned n1 = 0u, n2 = 0u, n3 = 0u;
        for (int j0 = 0; j0 < W.n_lines; j0 += kChunk) {
            float4 p[kChunk];
#pragma unroll
            for (int c = 0; c < kChunk; ++c)
                if (j0 + c < W.n_lines) p[c] = __ldg(v + (size_t)(j0 + c) * W.s1);
            long long t[kChunk];
            float z[kChunk], z0[kChunk];
#pragma unroll
            for (int c = 0; c < kChunk; ++c) {
                t[c] = -1;
                int tx, ty;
                float u, vv;
                if (j0 + c < W.n_lines && project_texel(K.lvp, mk(p[c].x, p[c].y, p[c].z), w, h, tx, ty, z[c], u, vv)) {
                    t[c] = (long long)ty * w + tx;
                    z0[c] = tex_sample(depth, w, h, 1, u, vv, 0);
                }
            }
#pragma unroll
            for (int c = 0; c < kChunk; ++c) {
                if (t[c] < 0) continue;
                const float d = 0.3f;
                const int layer = (z[c] >= z0[c] && z[c] < z0[c] + d) ? 1
                                  : (z[c] >= z0[c] + d && z[c] < z0[c] + 2.f * d) ? 2
                                  : (z[c] >= z0[c] + 2.f * d) ? 3 : 0;
                if (layer == 0) continue;
                if (t[c] != cur) {
                    if (cur >= 0) add_counts(words + 2 * cur, n1, n2, n3);
                    cur = t[c];
                    n1 = n2 = n3 = 0u;
                }
                n1 += layer == 1;
                n2 += layer == 2;
                n3 += layer == 3;
            }
        }
        if (cur >= 0) add_counts(words + 2 * cur, n1, n2, n3);
    }
}

// Layer counts -> the 8-bit unorm target's additive sum: 0.3 is stored as 77/255
// and the sum saturates, min(255, 77 c) / 255 with c = n1, n1 + n2, n1 + n2 + n3
// for layers 1, 2, 3.  In place: each texel's count word becomes its float4.
__device__ __forceinline__ float layer_value(unsigned c) {
    return (float)(c >= 4u ? 255u : 77u * c) / 255.0f;
}
__global__ void __launch_bounds__(kShadeThreads) k_opacity_finish(long long texels, uint4* map) {
    for (long long t = (long long)blockIdx.x * kShadeThreads + threadIdx.x; t < texels; t += (long long)gridDim.x * kShadeThreads) {
        const unsigned long long word = reinterpret_cast<const unsigned long long*>(map)[2 * t];
        const unsigned n1 = (unsigned)(word & kFieldMask), n2 = (unsigned)((word >> kFieldBits) & kFieldMask);
        const unsigned n3 = (unsigned)((word >> (2 * kFieldBits)) & kFieldMask);
        reinterpret_cast<float4*>(map)[t] =
            make_float4(layer_value(n1), layer_value(n1 + n2), layer_value(n1 + n2 + n3), 0.f);
    }
}

// Pass 3: hair.frag's colour of every tessellated vertex, from the fragment
// inputs the tessellation and geometry stages hand it on the ribbon's centre
// line (hair.tese:286-330, hair.geom:43-61): uv = (isoline u, v), the frame
// of the vertex's segment, normalize(cameraPos - pos), normalize(lightPos -
// pos), lightProj * lightView * pos.
__global__ void __launch_bounds__(kShadeThreads) k_shade_vertices(const float4* __restrict__ verts,
                                                                  const float4* __restrict__ frames, int n_strands,
                                                                  int n_points, int n_lines, int n_segments, Cam K,
                                                                  Maps M, Lines B, float4* __restrict__ out) {
    const int S1 = n_segments + 1;
    const long long nv = (long long)n_lines * S1 * n_strands;   // < 2^32, checked by the caller
    for (unsigned i = blockIdx.x * kShadeThreads + threadIdx.x; i < (unsigned)nv; i += gridDim.x * kShadeThreads) {
        const unsigned line = i / (unsigned)S1;                 // s * n_lines + j
        const int k = (int)(i - line * (unsigned)S1);
        const unsigned s = line / (unsigned)n_lines;
        const int j = (int)(line - s * (unsigned)n_lines);
        const float u = (float)j / (float)n_lines, v = (float)k / (float)n_segments;
        const float x = v * (float)(n_points - 1);
        const int sf = min((int)floorf(x), n_points - 2);
        const float4* fr = frames + ((size_t)s * (n_points - 1) + sf) * 3;
        const float4 q = verts[i];
        const V3 p = mk(q.x, q.y, q.z);
        float in[24];
        in[0] = u;
        in[1] = v;
        for (int c = 0; c < 3; ++c) {
            const float4 f = __ldg(fr + c);
            in[2 + 3 * c] = f.x;
            in[3 + 3 * c] = f.y;
            in[4 + 3 * c] = f.z;
        }
        const V3 vd = nrm3(mk(K.cam_pos[0], K.cam_pos[1], K.cam_pos[2]) - p);
        const V3 ld = nrm3(mk(K.light_pos[0], K.light_pos[1], K.light_pos[2]) - p);
        in[11] = vd.x;
        in[12] = vd.y;
        in[13] = vd.z;
        in[14] = ld.x;
        in[15] = ld.y;
        in[16] = ld.z;
        mul_point(K.lvp, p, in[17], in[18], in[19], in[20]);
        in[21] = in[22] = in[23] = 0.f;
        out[i] = shade_fragment(in, M, B.bright[j]);
    }
}

// ---- maps and image -----------------------------------------------------------------
__global__ void __launch_bounds__(kShadeThreads) k_clear_maps(long long texels, unsigned* __restrict__ depth_bits,
                                                              uint4* __restrict__ counts) {
    for (long long t = (long long)blockIdx.x * kShadeThreads + threadIdx.x; t < texels; t += (long long)gridDim.x * kShadeThreads) {
        depth_bits[t] = 0x3f800000u;   // 1.0f, the shadow pass's clear depth
        counts[t] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// Camera image with a depth test: while splatting, the first 8 bytes of each
// float4 pixel hold the key (depth bits << 32 | vertex index) of the nearest
// vertex so far; the resolve pass replaces it by that vertex's colour.
constexpr unsigned long long kNoVertex = ~0ull;

__global__ void __launch_bounds__(kShadeThreads) k_image_clear(long long px, float4* __restrict__ image) {
    for (long long t = (long long)blockIdx.x * kShadeThreads + threadIdx.x; t < px; t += (long long)gridDim.x * kShadeThreads)
        reinterpret_cast<unsigned long long*>(image)[2 * t] = kNoVertex;
}

__global__ void __launch_bounds__(kShadeThreads) k_image_depth(const float4* __restrict__ verts, long long nv, Proj P,
                                                               int w, int h, float4* __restrict__ image) {
    for (long long i = (long long)blockIdx.x * kShadeThreads + threadIdx.x; i < nv; i += (long long)gridDim.x * kShadeThreads) {
        const float4 q = verts[i];
        int tx, ty;
        float z, u, v;
        if (!project_texel(P.m, mk(q.x, q.y, q.z), w, h, tx, ty, z, u, v)) continue;
        const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | (unsigned long long)(unsigned)i;
        unsigned long long* px = reinterpret_cast<unsigned long long*>(image) + 2 * ((size_t)ty * w + tx);
        if (key < *reinterpret_cast<volatile unsigned long long*>(px)) atomicMin(px, key);   // keys only decrease
    }
}

__global__ void __launch_bounds__(kShadeThreads) k_image_resolve(long long px, const float4* __restrict__ colors,
                                                                 float4* __restrict__ image) {
    for (long long t = (long long)blockIdx.x * kShadeThreads + threadIdx.x; t < px; t += (long long)gridDim.x * kShadeThreads) {
        const unsigned long long key = reinterpret_cast<const unsigned long long*>(image)[2 * t];
        image[t] = key == kNoVertex ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(colors + (key & 0xffffffffull));
    }
}

// ---- rasterised camera image: hair.geom's quads ------------------------------------
// hair.geom (:41-108) turns each isoline segment (vertices k, k+1 of isoline j of
// strand s) into a camera-facing quad: with P = camera proj * view, c1 = P
// [pos_k, 1], c2 = P [pos_k+1, 1] and width1 = (|random(3.242551 u, u u)| + 0.5)
// * 0.075 * |cameraPos - pos_k| * strandWidth_k (every corner uses width1), the
// strip V0 = c1 - (width1, 0, 0, 0), V1 = c1 + ..., V2 = c2 - ..., V3 = c2 + ...;
// V0, V1 carry vertex k's attributes, V2, V3 vertex k+1's, and a corner's
// light-space position is lightProj * lightView * inverse(view) * inverse(proj) * V.
// Rasterisation rules (a definition of Vulkan's; the oracle restates the same
// arithmetic): screen x = (x/w * 0.5 + 0.5) W, y likewise with H, depth z/w;
// pixel centres at +0.5; triangles (V0, V1, V2), (V2, V1, V3) reordered to
// positive area; covered when every edge function is > 0, or = 0 on a top-left
// edge; depth linear in screen space, kept in [0, 1]; attributes perspective-
// correct.  A quad with a corner at w <= 0 (behind the eye) has each triangle
// clipped at the near plane z = 0 in clip space (clip_quad); a quad with a
// non-finite corner is dropped.  The
// nearest fragment wins (ties: the smaller segment id, then the first triangle)
// and the pixel takes its hair.frag colour (RVH_IMAGE_NEAREST; RVH_IMAGE_BLEND
// blends every passing fragment in primitive order, below).
//   k_hair_raster   one thread per segment: the quad's pixels, depth-tested by an
//                   atomic min of (depth bits << 32 | segment id) in the image
//   k_hair_resolve  one thread per pixel: the winner's quad again, perspective-
//                   correct inputs, hair.frag
struct RasterDev {
    float vp[16];      // camera proj * view
    float lmap[16];    // light proj * light view * inverse(view) * inverse(proj)
    float cam_pos[3], light_pos[3];
    int width, height;
    float rnd[kMaxLines];      // hair.geom's |random(3.242551 u, u u)| + 0.5 per isoline
    float bright[kMaxLines];   // hair.frag's 0.8 |random(u, u)| + 0.6 per isoline
};

struct TessView {
    const float4* verts;   // ns x L x (S + 1)
    const float4* frames;  // ns x (n - 1) x 3
    int n, L, S;
};

__device__ __forceinline__ void mul_vec4(const float* m, const float v[4], float o[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = ((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * v[3];
}

struct Quad {
    float clip[4][4];
    float sx[4], sy[4], sz[4];
    int x0, x1, y0, y1;
    bool ok;          // drawn by the warp-cooperative passes
    bool near_clip;   // a corner has w <= 0: drawn through clip_quad from the list (ok is false)
    bool big;         // a box over 65,536 pixels: drawn from the list (ok is false, the box is set)
};

__device__ __forceinline__ Quad make_quad(const RasterDev& R, float4 pk, float4 pk1, float rand_u) {
    Quad Q{};   // every field defined, also for a dropped quad (its box is shuffled but never used)
    Q.ok = false;
    const V3 a = mk(pk.x, pk.y, pk.z), b = mk(pk1.x, pk1.y, pk1.z);
    const float dist = len3(mk(R.cam_pos[0], R.cam_pos[1], R.cam_pos[2]) - a);
    const float scale = rand_u * 0.075f * dist;
    const float w1 = scale * pk.w;
    float c1[4], c2[4];
    const float pa[4] = {a.x, a.y, a.z, 1.f}, pb[4] = {b.x, b.y, b.z, 1.f};
    mul_vec4(R.vp, pa, c1);
    mul_vec4(R.vp, pb, c2);
    bool behind = false, finite = true;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const float* src = v < 2 ? c1 : c2;
        Q.clip[v][0] = src[0] + ((v & 1) ? w1 : -w1);
        Q.clip[v][1] = src[1];
        Q.clip[v][2] = src[2];
        Q.clip[v][3] = src[3];
#pragma unroll
        for (int e = 0; e < 4; ++e) finite = finite && isfinite(Q.clip[v][e]);
        behind = behind || !(Q.clip[v][3] > 0.f);
    }
    if (!finite) return Q;
    if (behind) {   // the triangles are clipped at the near plane (clip_quad)
        Q.near_clip = true;
        return Q;
    }
    float xmin = 3e38f, xmax = -3e38f, ymin = 3e38f, ymax = -3e38f;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const float cw = Q.clip[v][3];
        Q.sx[v] = (Q.clip[v][0] / cw * 0.5f + 0.5f) * (float)R.width;
        Q.sy[v] = (Q.clip[v][1] / cw * 0.5f + 0.5f) * (float)R.height;
        Q.sz[v] = Q.clip[v][2] / cw;
        if (!isfinite(Q.sx[v]) || !isfinite(Q.sy[v]) || !isfinite(Q.sz[v])) return Q;
        xmin = fminf(xmin, Q.sx[v]);
        xmax = fmaxf(xmax, Q.sx[v]);
        ymin = fminf(ymin, Q.sy[v]);
        ymax = fmaxf(ymax, Q.sy[v]);
    }
    const float fx0 = ceilf(xmin - 0.5f), fx1 = floorf(xmax - 0.5f);
    const float fy0 = ceilf(ymin - 0.5f), fy1 = floorf(ymax - 0.5f);
    const float cx0 = fmaxf(fx0, 0.f), cx1 = fminf(fx1, (float)(R.width - 1));
    const float cy0 = fmaxf(fy0, 0.f), cy1 = fminf(fy1, (float)(R.height - 1));
    if (cx0 > cx1 || cy0 > cy1) return Q;
    Q.x0 = (int)cx0;
    Q.x1 = (int)cx1;
    Q.y0 = (int)cy0;
    Q.y1 = (int)cy1;
    // the cooperative passes' per-warp pixel counts stay below 2^21; larger quads are listed
    if ((cx1 - cx0 + 1.f) * (cy1 - cy0 + 1.f) > 65536.f) Q.big = true;
    else Q.ok = true;
    return Q;
}

__device__ __forceinline__ float edge_fn(float ax, float ay, float bx, float by, float px, float py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
__device__ __forceinline__ bool top_left(float ax, float ay, float bx, float by) {
    const float dy = by - ay, dx = bx - ax;
    return dy < 0.f || (dy == 0.f && dx > 0.f);
}

// Triangle (i0, i1, i2) of quad Q at centre (px, py): the corners' values are
// taken into registers (no indexed local arrays) and swapped when the area is
// negative; idx[] reports the corners in the order of l[].
__device__ __forceinline__ bool cover_tri(const Quad& Q, int i0, int i1, int i2, float px, float py, int idx[3],
                                          float l[3], float& z) {
    float x0 = Q.sx[i0], y0 = Q.sy[i0], z0 = Q.sz[i0];
    float x1 = Q.sx[i1], y1 = Q.sy[i1], z1 = Q.sz[i1];
    float x2 = Q.sx[i2], y2 = Q.sy[i2], z2 = Q.sz[i2];
    float area = edge_fn(x0, y0, x1, y1, x2, y2);
    if (area == 0.f) return false;
    if (area < 0.f) {
        float t = x1;
        x1 = x2;
        x2 = t;
        t = y1;
        y1 = y2;
        y2 = t;
        t = z1;
        z1 = z2;
        z2 = t;
        const int ti = i1;
        i1 = i2;
        i2 = ti;
        area = -area;
    }
    // edge t is opposite vertex t: from vertex t+1 to vertex t+2
    const float e0 = edge_fn(x1, y1, x2, y2, px, py);
    if (e0 < 0.f || (e0 == 0.f && !top_left(x1, y1, x2, y2))) return false;
    const float e1 = edge_fn(x2, y2, x0, y0, px, py);
    if (e1 < 0.f || (e1 == 0.f && !top_left(x2, y2, x0, y0))) return false;
    const float e2 = edge_fn(x0, y0, x1, y1, px, py);
    if (e2 < 0.f || (e2 == 0.f && !top_left(x0, y0, x1, y1))) return false;
    l[0] = e0 / area;
    l[1] = e1 / area;
    l[2] = e2 / area;
    idx[0] = i0;
    idx[1] = i1;
    idx[2] = i2;
    z = (l[0] * z0 + l[1] * z1) + l[2] * z2;
    return z >= 0.f && z <= 1.f;
}

__device__ __forceinline__ int cover_quad(const Quad& Q, int px, int py, int idx[3], float l[3], float& z) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    int ia[3], ib[3];
    float la[3], lb[3], za = 0.f, zb = 0.f;
    const bool a = cover_tri(Q, 0, 1, 2, cx, cy, ia, la, za);
    const bool b = cover_tri(Q, 2, 1, 3, cx, cy, ib, lb, zb);
    if (a && (!b || za <= zb)) {
#pragma unroll
        for (int t = 0; t < 3; ++t) idx[t] = ia[t], l[t] = la[t];
        z = za;
        return 1;
    }
    if (b) {
#pragma unroll
        for (int t = 0; t < 3; ++t) idx[t] = ib[t], l[t] = lb[t];
        z = zb;
        return 2;
    }
    return 0;
}

// Near-plane clipping of a quad with a corner at w <= 0.  Each triangle,
// (V0, V1, V2) and (V2, V1, V3), is clipped in clip space to z >= 0 (Vulkan's
// near plane for a depth-zero-to-one projection) by Sutherland-Hodgman in
// triangle order: a corner with z >= 0 is kept, and an edge whose ends lie on
// opposite sides adds the point at s = z_a / (z_a - z_b) from its first end, its
// z set to 0.  The 3 or 4 vertices fan into sub-triangles (v0, v1, v2), (v0, v2,
// v3) that cover pixels by the unclipped rules; a vertex left at w <= 0 or at a
// non-finite screen position drops its triangle.  A vertex's attributes are its
// corners' lerped by s, interpolated perspective-correctly with the vertices' w.
// The box is every kept vertex's, clamped.  Such quads are rare (the eye inside
// the hair) and are drawn from a list.
struct ClipVert {
    float c[4];
    float sx, sy, sz;
    int a, b;   // corners lerped: corner a + s (corner b - corner a)
    float s;
};
struct ClipQuad {
    ClipVert v[2][4];
    int nv[2];
    int x0, x1, y0, y1;
    bool ok;
};

__device__ __forceinline__ int clip_triangle(const RasterDev& R, const Quad& Q, int i0, int i1, int i2, ClipVert* out) {
    const int tri[3] = {i0, i1, i2};
    int n = 0;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int a = tri[e], b = tri[(e + 1) % 3];
        const float za = Q.clip[a][2], zb = Q.clip[b][2];
        if (za >= 0.f) {
            ClipVert& o = out[n++];
#pragma unroll
            for (int q = 0; q < 4; ++q) o.c[q] = Q.clip[a][q];
            o.a = o.b = a;
            o.s = 0.f;
        }
        if ((za >= 0.f) != (zb >= 0.f)) {
            ClipVert& o = out[n++];
            const float t = __fdiv_rn(za, za - zb);
#pragma unroll
            for (int q = 0; q < 4; ++q) o.c[q] = __fadd_rn(Q.clip[a][q], __fmul_rn(t, __fsub_rn(Q.clip[b][q], Q.clip[a][q])));
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
        if (!isfinite(o.sx) || !isfinite(o.sy) || !isfinite(o.sz)) return 0;
    }
    return n;
}

__device__ __noinline__ ClipQuad clip_quad(const RasterDev& R, const Quad& Q) {
    ClipQuad C{};
    C.ok = false;
    C.nv[0] = clip_triangle(R, Q, 0, 1, 2, C.v[0]);
    C.nv[1] = clip_triangle(R, Q, 2, 1, 3, C.v[1]);
    float xmin = 3e38f, xmax = -3e38f, ymin = 3e38f, ymax = -3e38f;
    for (int t = 0; t < 2; ++t)
        for (int v = 0; v < C.nv[t]; ++v) {
            xmin = fminf(xmin, C.v[t][v].sx);
            xmax = fmaxf(xmax, C.v[t][v].sx);
            ymin = fminf(ymin, C.v[t][v].sy);
            ymax = fmaxf(ymax, C.v[t][v].sy);
        }
    if (C.nv[0] == 0 && C.nv[1] == 0) return C;
    const float fx0 = ceilf(xmin - 0.5f), fx1 = floorf(xmax - 0.5f);
    const float fy0 = ceilf(ymin - 0.5f), fy1 = floorf(ymax - 0.5f);
    const float cx0 = fmaxf(fx0, 0.f), cx1 = fminf(fx1, (float)(R.width - 1));
    const float cy0 = fmaxf(fy0, 0.f), cy1 = fminf(fy1, (float)(R.height - 1));
    if (cx0 > cx1 || cy0 > cy1) return C;
    C.x0 = (int)cx0;
    C.x1 = (int)cx1;
    C.y0 = (int)cy0;
    C.y1 = (int)cy1;
    C.ok = true;
    return C;
}

// cover_tri's arithmetic on sub-triangle (i0, i1, i2) of a clipped triangle's vertices.
__device__ __forceinline__ bool cover_sub(const ClipVert* V, int i0, int i1, int i2, float px, float py, int idx[3],
                                          float l[3], float& z) {
    float area = edge_fn(V[i0].sx, V[i0].sy, V[i1].sx, V[i1].sy, V[i2].sx, V[i2].sy);
    if (area == 0.f) return false;
    if (area < 0.f) {
        const int t = i1;
        i1 = i2;
        i2 = t;
        area = -area;
    }
    const ClipVert &A = V[i0], &B = V[i1], &Cv = V[i2];
    const float e0 = edge_fn(B.sx, B.sy, Cv.sx, Cv.sy, px, py);
    if (e0 < 0.f || (e0 == 0.f && !top_left(B.sx, B.sy, Cv.sx, Cv.sy))) return false;
    const float e1 = edge_fn(Cv.sx, Cv.sy, A.sx, A.sy, px, py);
    if (e1 < 0.f || (e1 == 0.f && !top_left(Cv.sx, Cv.sy, A.sx, A.sy))) return false;
    const float e2 = edge_fn(A.sx, A.sy, B.sx, B.sy, px, py);
    if (e2 < 0.f || (e2 == 0.f && !top_left(A.sx, A.sy, B.sx, B.sy))) return false;
    l[0] = e0 / area;
    l[1] = e1 / area;
    l[2] = e2 / area;
    idx[0] = i0;
    idx[1] = i1;
    idx[2] = i2;
    z = (l[0] * A.sz + l[1] * B.sz) + l[2] * Cv.sz;
    return z >= 0.f && z <= 1.f;
}

// Coverage by clipped triangle t: the first of its sub-triangles that covers.
__device__ __forceinline__ bool cover_clip_tri(const ClipQuad& C, int t, int px, int py, int idx[3], float l[3],
                                               float& z) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    const ClipVert* V = C.v[t];
    if (C.nv[t] >= 3 && cover_sub(V, 0, 1, 2, cx, cy, idx, l, z)) return true;
    return C.nv[t] == 4 && cover_sub(V, 0, 2, 3, cx, cy, idx, l, z);
}

// cover_quad of a clipped quad: 0 (none), 1 or 2, the nearer triangle (ties: the first).
__device__ __forceinline__ int cover_quad(const ClipQuad& C, int px, int py, int idx[3], float l[3], float& z) {
    int ia[3], ib[3];
    float la[3], lb[3], za = 0.f, zb = 0.f;
    const bool a = cover_clip_tri(C, 0, px, py, ia, la, za);
    const bool b = cover_clip_tri(C, 1, px, py, ib, lb, zb);
    if (a && (!b || za <= zb)) {
#pragma unroll
        for (int t = 0; t < 3; ++t) idx[t] = ia[t], l[t] = la[t];
        z = za;
        return 1;
    }
    if (b) {
#pragma unroll
        for (int t = 0; t < 3; ++t) idx[t] = ib[t], l[t] = lb[t];
        z = zb;
        return 2;
    }
    return 0;
}

__device__ __forceinline__ void segment_of(const TessView& T, unsigned id, int& s, int& j, int& k) {
    const unsigned line = id / (unsigned)T.S;
    k = (int)(id - line * (unsigned)T.S);
    s = (int)(line / (unsigned)T.L);
    j = (int)(line - (unsigned)s * (unsigned)T.L);
}

__device__ __forceinline__ const float4* vert_at(const TessView& T, int s, int j, int k) {
    return T.verts + ((size_t)s * T.L + j) * (T.S + 1) + k;
}

// Warp-cooperative rasterisation: a lane per quad leaves most lanes idle while
// one walks a larger pixel box (about 8 of 32 lanes active per instruction).  A
// warp instead takes 32 consecutive segments, prefix-sums their boxes' pixel
// counts and hands the (segment, pixel) jobs out 32 at a time: a lane finds the
// job's quad by a shuffle search over the prefix sums and fetches its corners by
// shuffles.  Each (segment, pixel) test is the same function on the same values
// as before, so the results do not change.
// The screen-space corners of lane `lane`'s quad (all the coverage test reads).
__device__ __forceinline__ void shfl_quad(const Quad& src, Quad& dst, int lane) {
    const unsigned FULL = 0xffffffffu;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        dst.sx[v] = __shfl_sync(FULL, src.sx[v], lane);
        dst.sy[v] = __shfl_sync(FULL, src.sy[v], lane);
        dst.sz[v] = __shfl_sync(FULL, src.sz[v], lane);
    }
}

// Near-clipped quads and quads over 65,536 pixels found by a rasterising pass:
// the pass appends their segment ids (append != 0), and k_listed_quads then
// rasterises each with one warp, so their state stays out of the common path's
// registers.  A later pass over the same quads reuses the list (append == 0).
struct ClipList {
    unsigned* count;
    unsigned* ids;
    unsigned cap;
    int append;
};

// frag(Q, id, j, px, py) for every pixel of every quad of segments [0, n_seg)
// (near-clipped quads: appended to CL); called by all threads of the grid
// (whole warps).
template <class Frag>
__device__ __forceinline__ void raster_warp(const TessView& T, const RasterDev& R, unsigned n_seg, const ClipList& CL,
                                            Frag frag) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned warp0 = (blockIdx.x * kShadeThreads + (threadIdx.x & ~31u));
    for (unsigned base = warp0; base < n_seg; base += gridDim.x * kShadeThreads) {   // warp-uniform
        const unsigned id = base + lane;
        Quad Q{};
        int j = 0;
        if (id < n_seg) {
            int s, k;
            segment_of(T, id, s, j, k);
            const float4* pv = vert_at(T, s, j, k);
            Q = make_quad(R, __ldg(pv), __ldg(pv + 1), R.rnd[j]);
            if ((Q.near_clip || Q.big) && CL.append) {
                const unsigned slot = atomicAdd(CL.count, 1u);
                if (slot < CL.cap) CL.ids[slot] = id;
            }
        }
        const int bw = Q.ok ? Q.x1 - Q.x0 + 1 : 0;
        const int cnt = Q.ok ? bw * (Q.y1 - Q.y0 + 1) : 0;   // <= 65,536 per quad
        int incl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, off);
            if (lane >= off) incl += v;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        for (int t0 = 0; t0 < total; t0 += 32) {
            const int t = t0 + lane;
            int o = 0;   // the job's quad: the number of lanes whose prefix ends at or before t
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int v = __shfl_sync(FULL, incl, o + step - 1);
                if (v <= t) o += step;
            }
            o = min(o, 31);
            Quad Qo{};
            shfl_quad(Q, Qo, o);
            const int o_incl = __shfl_sync(FULL, incl, o), o_cnt = __shfl_sync(FULL, cnt, o);
            const int o_bw = __shfl_sync(FULL, bw, o), o_x0 = __shfl_sync(FULL, Q.x0, o);
            const int o_y0 = __shfl_sync(FULL, Q.y0, o), o_j = __shfl_sync(FULL, j, o);
            if (t >= total) continue;
            const int local = t - (o_incl - o_cnt);
            const int ry = local / o_bw;
            frag(Qo, base + (unsigned)o, o_j, o_x0 + (local - ry * o_bw), o_y0 + ry);
        }
    }
}

// frag(Q or C, id, j, px, py) for every pixel of every listed quad's box (the
// clipped quad C of a near-clipped one), a warp per quad, its lanes striding
// over the box (the list is almost always empty).
template <class Frag>
__global__ void __launch_bounds__(kShadeThreads) k_listed_quads(TessView T, RasterDev R, ClipList CL, Frag frag) {
    const unsigned n = min(*CL.count, CL.cap);
    const int lane = threadIdx.x & 31;
    const unsigned warps = gridDim.x * (kShadeThreads / 32);
    for (unsigned q = (blockIdx.x * kShadeThreads + threadIdx.x) >> 5; q < n; q += warps) {
        const unsigned id = CL.ids[q];
        int s, j, k;
        segment_of(T, id, s, j, k);
        const float4* pv = vert_at(T, s, j, k);
        const Quad Q = make_quad(R, __ldg(pv), __ldg(pv + 1), R.rnd[j]);
        if (Q.big) {
            const int bw = Q.x1 - Q.x0 + 1, area = bw * (Q.y1 - Q.y0 + 1);   // <= 16384^2
            for (int t = lane; t < area; t += 32) frag(Q, id, j, Q.x0 + t % bw, Q.y0 + t / bw);
        } else if (Q.near_clip) {
            const ClipQuad C = clip_quad(R, Q);
            if (!C.ok) continue;
            const int bw = C.x1 - C.x0 + 1, area = bw * (C.y1 - C.y0 + 1);
            for (int t = lane; t < area; t += 32) frag(C, id, j, C.x0 + t % bw, C.y0 + t / bw);
        }
    }
}

// Nearest fragment per pixel: an atomic min of (depth bits << 32 | segment id).
struct NearestFrag {
    unsigned long long* keys;   // 2 words per float4 pixel
    int width;
    template <class Q>
    __device__ __forceinline__ void operator()(const Q& q, unsigned id, int, int px, int py) const {
        int idx[3];
        float l[3], z;
        if (!cover_quad(q, px, py, idx, l, z)) return;
        const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | id;
        unsigned long long* slot = keys + 2 * ((size_t)py * width + px);
        if (key < *reinterpret_cast<volatile unsigned long long*>(slot)) atomicMin(slot, key);
    }
};

__global__ void __launch_bounds__(kShadeThreads) k_hair_raster(TessView T, RasterDev R, unsigned n_seg, ClipList CL,
                                                               float4* __restrict__ image) {
    raster_warp(T, R, n_seg, CL, NearestFrag{reinterpret_cast<unsigned long long*>(image), R.width});
}

// Light maps from hair.geom's quads, the light camera bound as the geometry
// shader's camera (the reference's shadow and opacity passes): the depth pass
// keeps each texel's nearest fragment (LESS_OR_EQUAL, cleared to 1.0); the
// opacity pass has no depth test, so every fragment adds to the layer its depth
// falls in relative to the depth map at its light-space position, which is the
// fragment's own (lightProj * lightView * inverse(lightView) * inverse(lightProj)
// is the identity): its pixel centre and its rasterised depth.
struct LightDepthFrag {
    unsigned* depth_bits;
    int width;
    template <class Q>
    __device__ __forceinline__ void operator()(const Q& q, unsigned, int, int px, int py) const {
        int idx[3];
        float l[3], z;
        if (!cover_quad(q, px, py, idx, l, z)) return;
        flush_min(depth_bits + (size_t)py * width + px, __float_as_uint(z));
    }
};

struct LightOpacityFrag {
    const float* depth;
    unsigned long long* words;
    int width, height;
    template <class Q>
    __device__ __forceinline__ void operator()(const Q& q, unsigned, int, int px, int py) const {
        int idx[3];
        float l[3], cz;
        if (!cover_quad(q, px, py, idx, l, cz)) return;
        // the fragment's light-space position: its pixel centre and rasterised depth
        const float u = ((float)px + 0.5f) / (float)width, v = ((float)py + 0.5f) / (float)height;
        const float z0 = tex_sample(depth, width, height, 1, u, v, 0);
        const float d = 0.3f;
        const int layer = (cz >= z0 && cz < z0 + d) ? 1 : (cz >= z0 + d && cz < z0 + 2.f * d) ? 2
                                                          : (cz >= z0 + 2.f * d) ? 3 : 0;
        if (layer == 0) return;
        add_counts(words + 2 * ((size_t)py * width + px), layer == 1, layer == 2, layer == 3);
    }
};

__global__ void __launch_bounds__(kShadeThreads) k_light_quads_depth(TessView T, RasterDev R, unsigned n_seg,
                                                                     ClipList CL, unsigned* __restrict__ depth_bits) {
    raster_warp(T, R, n_seg, CL, LightDepthFrag{depth_bits, R.width});
}

__global__ void __launch_bounds__(kShadeThreads) k_light_quads_opacity(TessView T, RasterDev R, unsigned n_seg,
                                                                       ClipList CL, const float* __restrict__ depth,
                                                                       uint4* __restrict__ counts) {
    raster_warp(T, R, n_seg, CL,
                LightOpacityFrag{depth, reinterpret_cast<unsigned long long*>(counts), R.width, R.height});
}

// hair.frag's inputs at corner c of segment (s, j, k)'s quad Q (V0, V1 take
// vertex k's, V2, V3 vertex k + 1's).
__device__ __forceinline__ void corner_inputs(const TessView& T, const RasterDev& R, int s, int j, int k, const Quad& Q,
                                              int c, float a[24]) {
    const int kk = c < 2 ? k : k + 1;
    const float4 P4 = __ldg(vert_at(T, s, j, kk));
    const V3 pos = mk(P4.x, P4.y, P4.z);
    const float u = (float)j / (float)T.L, v = (float)kk / (float)T.S;
    const float x = v * (float)(T.n - 1);
    const int sf = min((int)floorf(x), T.n - 2);
    const float4* fr = T.frames + ((size_t)s * (T.n - 1) + sf) * 3;
    a[0] = u;
    a[1] = v;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float4 f = __ldg(fr + q);
        a[2 + 3 * q] = f.x;
        a[3 + 3 * q] = f.y;
        a[4 + 3 * q] = f.z;
    }
    const V3 vd = nrm3(mk(R.cam_pos[0], R.cam_pos[1], R.cam_pos[2]) - pos);
    const V3 ld = nrm3(mk(R.light_pos[0], R.light_pos[1], R.light_pos[2]) - pos);
    a[11] = vd.x;
    a[12] = vd.y;
    a[13] = vd.z;
    a[14] = ld.x;
    a[15] = ld.y;
    a[16] = ld.z;
    float cl[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) cl[e] = Q.clip[c][e];
    mul_vec4(R.lmap, cl, a + 17);
    a[21] = a[22] = a[23] = 0.f;
}

// hair.frag's inputs for the fragment of segment (s, j, k)'s quad Q at pixel
// (px, py), covered by the triangle with corners idx[] and barycentrics l[]:
// the corners' inputs interpolated perspective-correctly.
__device__ __forceinline__ void segment_inputs(const TessView& T, const RasterDev& R, int s, int j, int k,
                                               const Quad& Q, const int idx[3], const float l[3], float in[24]) {
    const float q0 = l[0] / Q.clip[idx[0]][3], q1 = l[1] / Q.clip[idx[1]][3], q2 = l[2] / Q.clip[idx[2]][3];
    const float qs = (q0 + q1) + q2;
    const float qc[3] = {q0, q1, q2};
    float acc[24];
#pragma unroll
    for (int e = 0; e < 24; ++e) acc[e] = 0.f;
    // the corners' hair.frag inputs, accumulated in the oracle's order (q0 a0 + q1 a1) + q2 a2
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        float a[24];
        corner_inputs(T, R, s, j, k, Q, idx[t], a);
#pragma unroll
        for (int e = 0; e < 24; ++e) acc[e] = t == 0 ? qc[0] * a[e] : acc[e] + qc[t] * a[e];
    }
#pragma unroll
    for (int e = 0; e < 24; ++e) in[e] = acc[e] / qs;
    in[0] = (float)j / (float)T.L;
}

// hair.frag's inputs for the fragment of near-clipped quad Q at pixel (px, py):
// that of triangle t (0 or 1), or with t < 0 the nearer covering triangle's.  A
// clipped vertex stands for corners a and b lerped by s, so the perspective-
// correct interpolation is a weighted sum of the four corners' inputs: weight
// w_c = sum over the vertices of q_i = l_i / w_i times 1 (c = a = b), 1 - s
// (c = a) or s (c = b), accumulated vertex by vertex; in = (sum over c in order
// of w_c inputs_c) / (q_0 + q_1 + q_2).
__device__ __forceinline__ void segment_inputs_clip(const TessView& T, const RasterDev& R, int s, int j, int k, int px,
                                                 int py, int t, float* in) {
    const float4* pv = vert_at(T, s, j, k);
    const Quad Q = make_quad(R, __ldg(pv), __ldg(pv + 1), R.rnd[j]);
    const ClipQuad C = clip_quad(R, Q);
    int idx[3];
    float l[3], z;
    if (t < 0) t = cover_quad(C, px, py, idx, l, z) - 1;
    else cover_clip_tri(C, t, px, py, idx, l, z);
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
    float acc[24];
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        float a[24];
        corner_inputs(T, R, s, j, k, Q, c, a);
#pragma unroll
        for (int e = 0; e < 24; ++e) acc[e] = c == 0 ? w[0] * a[e] : acc[e] + w[c] * a[e];
    }
#pragma unroll
    for (int e = 0; e < 24; ++e) in[e] = acc[e] / qs;
    in[0] = (float)j / (float)T.L;
}

// Pixels whose fragment comes from a near-clipped quad: the common resolve pass
// lists them (a pixel at most once, cap = the pixel count) and leaves them to a
// second pass compiled with the clipped path, so that path's registers stay out
// of the common one.
struct DeferList {
    unsigned* count;
    unsigned* ids;
    unsigned cap;
};

__device__ __forceinline__ void defer_pixel(const DeferList& D, long long p) {
    const unsigned slot = atomicAdd(D.count, 1u);
    if (slot < D.cap) D.ids[slot] = (unsigned)p;
}

// kClipped: the listed pixels only (their winners are near-clipped quads).
template <bool kClipped>
__global__ void __launch_bounds__(kShadeThreads) k_hair_resolve(TessView T, RasterDev R, Maps M, long long px_count,
                                                                float4* __restrict__ image, unsigned* __restrict__ ids,
                                                                DeferList D) {
    const long long n = kClipped ? (long long)min(*D.count, D.cap) : px_count;
    for (long long i = (long long)blockIdx.x * kShadeThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kShadeThreads) {
        const long long p = kClipped ? (long long)D.ids[i] : i;
        const unsigned long long key = reinterpret_cast<const unsigned long long*>(image)[2 * p];
        if (key == kNoVertex) {
            image[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ids) ids[p] = 0xffffffffu;
            continue;
        }
        const unsigned id = (unsigned)(key & 0xffffffffull);
        if (ids) ids[p] = id;
        int s, j, k;
        segment_of(T, id, s, j, k);
        const float4* pv = vert_at(T, s, j, k);
        const Quad Q = make_quad(R, __ldg(pv), __ldg(pv + 1), R.rnd[j]);
        const int py = (int)(p / R.width), px = (int)(p - (long long)py * R.width);
        float in[24];
        if constexpr (kClipped) {
            segment_inputs_clip(T, R, s, j, k, px, py, -1, in);
        } else {
            if (Q.near_clip) {   // the second pass shades it
                defer_pixel(D, p);
                continue;
            }
            int idx[3];
            float l[3], z;
            cover_quad(Q, px, py, idx, l, z);
            segment_inputs(T, R, s, j, k, Q, idx, l, in);
        }
        image[p] = shade_fragment(in, M, R.bright[j]);
    }
}

// ---- the hair pass with the pipeline's in-order blending (RVH_IMAGE_BLEND) -----------
// The reference's hair pipeline (src/Renderer.cpp:1657-1679) draws the quads in
// segment order, each quad's triangles (V0, V1, V2) then (V2, V1, V3); a
// fragment passes a LESS depth test against the depth the earlier fragments
// wrote (cleared to 1.0), writes its depth and blends SRC_ALPHA /
// ONE_MINUS_SRC_ALPHA into the colour, ONE / ONE into the alpha (clamped to 1).
// So a pixel's colour is the fold, in primitive order, over the fragments whose
// depth is below every earlier fragment's.  Here every fragment is listed per
// pixel (count, scan, scatter) as (primitive key << 32 | depth bits), primitive
// key = 2 * segment + triangle + 1; a warp per pixel then walks the passing
// fragments in primitive order (each the smallest key above the last one with a
// depth below the last one's), shades up to 32 of them in parallel and folds.

// Calls f(t, idx, l, z) for each of quad Q's triangles t (0, 1) covering pixel (px, py).
template <class F>
__device__ __forceinline__ void for_covering_triangles(const Quad& Q, int px, int py, F f) {
    const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
    int idx[3];
    float l[3], z;
    if (cover_tri(Q, 0, 1, 2, cx, cy, idx, l, z)) f(0, idx, l, z);
    if (cover_tri(Q, 2, 1, 3, cx, cy, idx, l, z)) f(1, idx, l, z);
}
template <class F>
__device__ __forceinline__ void for_covering_triangles(const ClipQuad& C, int px, int py, F f) {
    int idx[3];
    float l[3], z;
    if (cover_clip_tri(C, 0, px, py, idx, l, z)) f(0, idx, l, z);
    if (cover_clip_tri(C, 1, px, py, idx, l, z)) f(1, idx, l, z);
}

struct BlendCountFrag {
    unsigned* counts;
    int width;
    template <class Q>
    __device__ __forceinline__ void operator()(const Q& q, unsigned, int, int px, int py) const {
        for_covering_triangles(q, px, py, [&](int, const int*, const float*, float) {
            atomicAdd(counts + (size_t)py * width + px, 1u);
        });
    }
};

__global__ void __launch_bounds__(kShadeThreads) k_blend_count(TessView T, RasterDev R, unsigned n_seg, ClipList CL,
                                                               unsigned* __restrict__ counts) {
    raster_warp(T, R, n_seg, CL, BlendCountFrag{counts, R.width});
}

// Exclusive scan of counts[0, n) into offs[0, n] (offs[n] = the total) and
// cursor[0, n), in tiles of kScanTile: local scans, a scan of the tile totals,
// then the tile offsets added.
constexpr int kScanTile = 4 * kShadeThreads;
__global__ void __launch_bounds__(kShadeThreads) k_scan_tiles(const unsigned* __restrict__ counts, long long n,
                                                              unsigned* __restrict__ offs, unsigned* __restrict__ sums) {
    __shared__ unsigned warp_tot[kShadeThreads / 32];
    const long long base = (long long)blockIdx.x * kScanTile + 4 * threadIdx.x;
    unsigned v[4], run = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        v[q] = base + q < n ? counts[base + q] : 0u;
        run += v[q];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned before = 0;
    for (int w = 0; w < warp; ++w) before += warp_tot[w];
    unsigned acc = before + incl - run;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (base + q < n) offs[base + q] = acc;
        acc += v[q];
    }
    if (threadIdx.x == kShadeThreads - 1) sums[blockIdx.x] = before + incl;
}

__global__ void __launch_bounds__(kShadeThreads) k_scan_sums(unsigned* __restrict__ sums, int n_tiles) {
    // one CTA: each thread scans a contiguous run of tiles, then the runs are offset
    __shared__ unsigned part[kShadeThreads];
    const int per = (n_tiles + kShadeThreads - 1) / kShadeThreads;
    const int t0 = threadIdx.x * per, t1 = min(n_tiles, t0 + per);
    unsigned run = 0;
    for (int t = t0; t < t1; ++t) run += sums[t];
    part[threadIdx.x] = run;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned acc = 0;
        for (int i = 0; i < kShadeThreads; ++i) {
            const unsigned x = part[i];
            part[i] = acc;
            acc += x;
        }
    }
    __syncthreads();
    unsigned acc = part[threadIdx.x];
    for (int t = t0; t < t1; ++t) {
        const unsigned x = sums[t];
        sums[t] = acc;
        acc += x;
    }
}

// ... and lists the pixels with fragments in active (their number in *n_active,
// one atomic per warp), then zeroes counts (it becomes the per-pixel count of
// passing fragments).
__global__ void __launch_bounds__(kShadeThreads) k_scan_add(unsigned* __restrict__ counts, long long n,
                                                            const unsigned* __restrict__ sums, unsigned* __restrict__ offs,
                                                            unsigned* __restrict__ cursor, unsigned* __restrict__ active,
                                                            unsigned* __restrict__ n_active) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * kShadeThreads; base < n; base += (long long)gridDim.x * kShadeThreads) {
        const long long i = base + threadIdx.x;   // the loop is uniform across each warp
        const unsigned c = i < n ? counts[i] : 0u;
        if (i < n) {
            const unsigned o = offs[i] + sums[i / kScanTile];
            offs[i] = o;
            cursor[i] = o;
            counts[i] = 0u;
            if (i == n - 1) offs[n] = o + c;
        }
        const unsigned m = __ballot_sync(FULL, c > 0u);
        unsigned slot = 0;
        if (lane == 0 && m) slot = atomicAdd(n_active, (unsigned)__popc(m));
        slot = __shfl_sync(FULL, slot, 0);
        if (c > 0u) active[slot + __popc(m & ((1u << lane) - 1u))] = (unsigned)i;
    }
}

// A listed fragment: (2 * segment + triangle + 1) << 32 | depth bits, the depth's
// sign bit (depths are in [0, 1]; -0 is stored as +0) set for a fragment of a
// listed quad (near-clipped or over 65,536 pixels).
constexpr unsigned kListedFrag = 0x80000000u;
__device__ __forceinline__ float frag_depth(unsigned long long v) { return __uint_as_float((unsigned)v & 0x7fffffffu); }

struct BlendScatterFrag {
    unsigned* cursor;
    unsigned long long* frags;
    unsigned long long capacity;
    int width;
    unsigned flag;   // kListedFrag from the listed quads' pass, else 0
    template <class Q>
    __device__ __forceinline__ void operator()(const Q& q, unsigned id, int, int px, int py) const {
        for_covering_triangles(q, px, py, [&](int t, const int*, const float*, float z) {
            const unsigned slot = atomicAdd(cursor + (size_t)py * width + px, 1u);
            if (slot < capacity)   // the count pass sized the list; this never fails
                frags[slot] = ((unsigned long long)(2u * id + (unsigned)t + 1u) << 32) |
                              ((__float_as_uint(z) & 0x7fffffffu) | flag);
        });
    }
};

__global__ void __launch_bounds__(kShadeThreads) k_blend_scatter(TessView T, RasterDev R, unsigned n_seg, ClipList CL,
                                                                 unsigned* __restrict__ cursor,
                                                                 unsigned long long* __restrict__ frags,
                                                                 unsigned long long capacity) {
    raster_warp(T, R, n_seg, CL, BlendScatterFrag{cursor, frags, capacity, R.width, 0u});
}

constexpr int kOrderCap = 8192;                 // most fragments of one pixel sorted in shared memory (68 KB)
constexpr int kOrderCapSmall = 2048;            // the first pass's cap (17 KB, 5 CTAs per SM; 9 in 10 pixels)
constexpr unsigned kDeferredPx = 0xffffffffu;   // pass_count of a pixel left to k_blend_resolve

// Shared-memory slot of sorted-list element e: one 8-byte pad after every 16
// elements, so that a warp's 64-bit accesses at any power-of-two stride of the
// sort passes spread over the banks (two wavefronts per instruction, the least
// for 32 x 8 bytes) instead of piling onto two of them.
__device__ __forceinline__ unsigned sx(unsigned e) { return e + (e >> 4); }
constexpr int order_smem_bytes(int cap) { return (cap + cap / 16) * 8; }

// NST consecutive bitonic stages (strides low << (NST - 1) down to low) of the
// ascending/descending network for merge size k over sk[0, N): the elements of a
// group differ only in the NST index bits from position p0 up, so all of a
// group's compare-exchanges of these stages stay in registers.
template <int NST>
__device__ __forceinline__ void sort_group(unsigned long long* sk, unsigned N, unsigned k, unsigned low, int p0,
                                           int tid) {
    constexpr int G = 1 << NST;
    const unsigned below = (1u << p0) - 1u;
    for (unsigned g = tid; g < (N >> NST); g += kShadeThreads) {
        const unsigned base = ((g & ~below) << NST) | (g & below);
        const bool up = (base & k) == 0u;   // every member shares the bits above p0 + NST - 1
        unsigned long long v[G];
#pragma unroll
        for (int m = 0; m < G; ++m) v[m] = sk[sx(base + m * low)];
#pragma unroll
        for (int st = NST - 1; st >= 0; --st)   // stride low << st: member bit st
#pragma unroll
            for (int m = 0; m < G; ++m)
                if (!(m & (1 << st))) {
                    const unsigned long long a = v[m], b = v[m | (1 << st)];
                    const bool swap = (a > b) == up;
                    v[m] = swap ? b : a;
                    v[m | (1 << st)] = swap ? a : b;
                }
#pragma unroll
        for (int m = 0; m < G; ++m) sk[sx(base + m * low)] = v[m];
    }
}

// One block per pixel (grid-stride).  A fragment passes the LESS test in
// primitive order exactly when its depth is below 1.0 and below every
// earlier fragment's: a failing fragment is never below the depth buffer, so
// the buffer is the running minimum of all earlier depths.  The pixel's
// fragments are sorted by primitive key in shared memory (bitonic; keys are
// unique within a pixel), each warp takes a segment of the sorted list (the
// minimum of the segments before it from the warps' minima) and finds its
// passing fragments 32 at a time with warp min-scans, and the passing
// fragments are written in order to the start of the pixel's list, their
// number to pass_count[p].  A first pass with a small cap (more CTAs per SM, so
// more pixels in flight) lists the larger pixels in Over for a second pass with
// the full cap.  A pixel with more than kOrderCap fragments, or with one of a
// listed quad, is listed in D instead (pass_count = kDeferredPx) and its list
// left as it is for k_blend_resolve.  Only the pixels with fragments (active)
// are visited; the others keep pass_count 0.
template <int kCap>
__global__ void __launch_bounds__(kShadeThreads) k_blend_order(const unsigned* __restrict__ active,
                                                               const unsigned* __restrict__ n_active,
                                                               const unsigned* __restrict__ offs,
                                                               unsigned long long* __restrict__ frags,
                                                               unsigned* __restrict__ pass_count, DeferList D,
                                                               DeferList Over) {
    extern __shared__ unsigned long long sk[];   // order_smem_bytes(kCap)
    __shared__ float s_wmin[kShadeThreads / 32];
    __shared__ unsigned s_wcnt[kShadeThreads / 32];
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned n = *n_active;
    for (unsigned a = blockIdx.x; a < n; a += gridDim.x) {
        const long long p = active[a];
        const unsigned lo = offs[p], F = offs[p + 1] - lo;   // block-uniform, > 0
        if (F > (unsigned)kCap) {
            if (tid == 0) {
                if (Over.count) {   // to the pass with the larger cap
                    defer_pixel(Over, p);
                } else {
                    pass_count[p] = kDeferredPx;
                    defer_pixel(D, p);
                }
            }
            continue;
        }
        unsigned N = 1;
        while (N < F) N <<= 1;
        bool listed = false;
        for (unsigned i = tid; i < N; i += kShadeThreads) {
            const unsigned long long v = i < F ? frags[lo + i] : ~0ull;
            listed = listed || (i < F && ((unsigned)v & kListedFrag) != 0u);
            sk[sx(i)] = v;
        }
        if (__syncthreads_or(listed)) {
            if (tid == 0) {
                pass_count[p] = kDeferredPx;
                defer_pixel(D, p);
            }
            continue;
        }
        // bitonic sort, up to three stages (j, j/2, j/4) per pass over shared memory: each
        // thread takes groups of 2^nst elements whose indices differ only in those bits,
        // runs the stages in registers and stores the group back (a third of the passes,
        // barriers and shared-memory traffic of one stage per pass)
        for (unsigned k = 2; k <= N; k <<= 1)
            for (unsigned j = k >> 1; j > 0;) {
                const int lj = 31 - __clz(j);
                const int nst = lj >= 2 ? 3 : lj + 1;   // stages in this pass
                const unsigned low = j >> (nst - 1);     // the smallest stride of the group
                const int p0 = lj - nst + 1;             // its bit position
                if (nst == 3) sort_group<3>(sk, N, k, low, p0, tid);
                else if (nst == 2) sort_group<2>(sk, N, k, low, p0, tid);
                else sort_group<1>(sk, N, k, low, p0, tid);
                __syncthreads();
                j >>= nst;
            }
        // each warp takes a segment of the sorted list and walks it 32 fragments at a time
        // (lane i reads element i of the chunk: no bank conflicts), with warp min-scans
        constexpr unsigned kW = kShadeThreads / 32;
        const unsigned seg = (F + 32 * kW - 1) / (32 * kW) * 32;
        const unsigned w0 = min(F, warp * seg), w1 = min(F, w0 + seg);
        float m = 1.0f;
        for (unsigned i = w0 + lane; i < w1; i += 32) m = fminf(m, frag_depth(sk[sx(i)]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(FULL, m, o));
        if (lane == 0) s_wmin[warp] = m;
        __syncthreads();
        float before = 1.0f;   // the minimum depth of every fragment before this segment
        for (unsigned w = 0; w < (unsigned)warp; ++w) before = fminf(before, s_wmin[w]);
        // one chunk: which of its fragments pass, given the running minimum r before it
        auto chunk = [&](unsigned c, float& r, float& d, bool& pass) {
            const unsigned i = c + lane;
            d = i < w1 ? frag_depth(sk[sx(i)]) : 2.0f;   // 2.0 never passes
            float incl = d;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl = fminf(incl, t);
            }
            float ex = __shfl_up_sync(FULL, incl, 1);
            ex = lane == 0 ? r : fminf(ex, r);
            pass = d < ex;
            r = fminf(r, __shfl_sync(FULL, incl, 31));
        };
        unsigned cnt = 0;
        float r = before;
        for (unsigned c = w0; c < w1; c += 32) {   // warp-uniform
            float d;
            bool pass;
            chunk(c, r, d, pass);
            cnt += __popc(__ballot_sync(FULL, pass));
        }
        if (lane == 0) s_wcnt[warp] = cnt;
        __syncthreads();
        unsigned q = 0, total = 0;
        for (unsigned w = 0; w < kW; ++w) {
            if (w < (unsigned)warp) q += s_wcnt[w];
            total += s_wcnt[w];
        }
        r = before;
        for (unsigned c = w0; c < w1; c += 32) {
            float d;
            bool pass;
            chunk(c, r, d, pass);
            const unsigned mask = __ballot_sync(FULL, pass);
            if (pass) frags[lo + q + __popc(mask & ((1u << lane) - 1u))] = sk[sx(c + lane)];
            q += __popc(mask);
        }
        if (tid == 0) pass_count[p] = total;
        __syncthreads();   // sk and the scan scratch are free for the next pixel
    }
}

// One warp per pixel: the pass_count[p] passing fragments at the start of its
// list, shaded 32 at a time in parallel and folded in order with
// SRC_ALPHA / ONE_MINUS_SRC_ALPHA (alpha ONE / ONE, clamped to 1) from clear.
__global__ void __launch_bounds__(kShadeThreads) k_blend_shade(TessView T, RasterDev R, Maps M, long long px_count,
                                                               const unsigned* __restrict__ offs,
                                                               const unsigned long long* __restrict__ frags,
                                                               const unsigned* __restrict__ pass_count, float4 clear,
                                                               float4* __restrict__ image, unsigned* __restrict__ ids) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (kShadeThreads / 32);
    for (long long p = ((long long)blockIdx.x * kShadeThreads + threadIdx.x) >> 5; p < px_count; p += warps) {
        const unsigned P = pass_count[p];
        if (P == kDeferredPx) continue;
        const unsigned lo = offs[p];
        const int py = (int)(p / R.width), px = (int)(p - (long long)py * R.width);
        float3 rgb = make_float3(clear.x, clear.y, clear.z);
        float alpha = clear.w;
        unsigned last = 0xffffffffu;
        for (unsigned base = 0; base < P; base += 32) {
            const unsigned q = base + lane;
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            unsigned id = 0u;
            if (q < P) {
                const unsigned key = (unsigned)(__ldg(frags + lo + q) >> 32) - 1u;
                id = key >> 1;
                int s, j, k;
                segment_of(T, id, s, j, k);
                const float4* pv = vert_at(T, s, j, k);
                const Quad Q = make_quad(R, __ldg(pv), __ldg(pv + 1), R.rnd[j]);
                const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
                int idx[3];
                float l[3], z;
                if (key & 1u) cover_tri(Q, 2, 1, 3, cx, cy, idx, l, z);
                else cover_tri(Q, 0, 1, 2, cx, cy, idx, l, z);
                float in[24];
                segment_inputs(T, R, s, j, k, Q, idx, l, in);
                c = shade_fragment(in, M, R.bright[j]);
            }
            const int np = (int)min(32u, P - base);
            for (int t = 0; t < np; ++t) {
                const float cr = __shfl_sync(FULL, c.x, t), cg = __shfl_sync(FULL, c.y, t);
                const float cb = __shfl_sync(FULL, c.z, t), ca = __shfl_sync(FULL, c.w, t);
                const float ia = 1.0f - ca;
                rgb = make_float3(cr * ca + rgb.x * ia, cg * ca + rgb.y * ia, cb * ca + rgb.z * ia);
                alpha = fminf(1.0f, ca + alpha);
            }
            last = __shfl_sync(FULL, id, np - 1);
        }
        if (lane == 0) {
            image[p] = make_float4(rgb.x, rgb.y, rgb.z, alpha);
            if (ids) ids[p] = last;
        }
    }
}

// The listed pixels of k_blend_order (a fragment of a listed quad, or too many
// to sort), one warp per pixel over the untouched list: each pass over the
// candidates finds the next passing fragment, the smallest key above the last
// passing one's with a depth below it (a warp-wide min); up to 32 are shaded
// in parallel (through the clipped path for a near-clipped quad), then folded.
__global__ void __launch_bounds__(kShadeThreads) k_blend_resolve(TessView T, RasterDev R, Maps M,
                                                                 const unsigned* __restrict__ offs,
                                                                 const unsigned long long* __restrict__ frags,
                                                                 float4 clear, float4* __restrict__ image,
                                                                 unsigned* __restrict__ ids, DeferList D) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (kShadeThreads / 32);
    const long long n = (long long)min(*D.count, D.cap);
    for (long long i = ((long long)blockIdx.x * kShadeThreads + threadIdx.x) >> 5; i < n; i += warps) {
        const long long p = (long long)D.ids[i];
        const unsigned lo = offs[p], hi = offs[p + 1];
        const int py = (int)(p / R.width), px = (int)(p - (long long)py * R.width);
        float3 rgb = make_float3(clear.x, clear.y, clear.z);
        float alpha = clear.w;
        unsigned last = 0xffffffffu;
        unsigned cur_key = 0u;
        float cur_z = 1.0f;
        for (;;) {
            // the next (up to) 32 passing fragments, in primitive order: lane i holds the i-th
            unsigned long long mine = ~0ull;
            int npass = 0;
            while (npass < 32) {
                unsigned long long best = ~0ull;
                for (unsigned f = lo + lane; f < hi; f += 32) {
                    const unsigned long long v = __ldg(frags + f);
                    if ((unsigned)(v >> 32) > cur_key && frag_depth(v) < cur_z && v < best) best = v;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const unsigned long long t = __shfl_xor_sync(FULL, best, o);
                    best = t < best ? t : best;
                }
                if (best == ~0ull) break;
                if (lane == npass) mine = best;
                cur_key = (unsigned)(best >> 32);
                cur_z = frag_depth(best);
                ++npass;
            }
            if (npass == 0) break;
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < npass) {
                const unsigned key = (unsigned)(mine >> 32) - 1u;
                const unsigned id = key >> 1;
                int s, j, k;
                segment_of(T, id, s, j, k);
                const float4* pv = vert_at(T, s, j, k);
                const Quad Q = make_quad(R, __ldg(pv), __ldg(pv + 1), R.rnd[j]);
                const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
                float in[24];
                if (Q.near_clip) {
                    segment_inputs_clip(T, R, s, j, k, px, py, (int)(key & 1u), in);
                } else {
                    int idx[3];
                    float l[3], z;
                    if (key & 1u) cover_tri(Q, 2, 1, 3, cx, cy, idx, l, z);
                    else cover_tri(Q, 0, 1, 2, cx, cy, idx, l, z);
                    segment_inputs(T, R, s, j, k, Q, idx, l, in);
                }
                c = shade_fragment(in, M, R.bright[j]);
            }
            for (int t = 0; t < npass; ++t) {   // SRC_ALPHA / ONE_MINUS_SRC_ALPHA, alpha ONE / ONE
                const float cr = __shfl_sync(FULL, c.x, t), cg = __shfl_sync(FULL, c.y, t);
                const float cb = __shfl_sync(FULL, c.z, t), ca = __shfl_sync(FULL, c.w, t);
                const float ia = 1.0f - ca;
                rgb = make_float3(cr * ca + rgb.x * ia, cg * ca + rgb.y * ia, cb * ca + rgb.z * ia);
                alpha = fminf(1.0f, ca + alpha);
            }
            last = ((unsigned)(__shfl_sync(FULL, mine, npass - 1) >> 32) - 1u) >> 1;
            if (npass < 32) break;
        }
        if (lane == 0) {
            image[p] = make_float4(rgb.x, rgb.y, rgb.z, alpha);
            if (ids) ids[p] = last;
        }
    }
}

// ---- host ---------------------------------------------------------------------------
// glm's normalize, cross, lookAtRH and perspectiveRH_ZO in float, in glm's
// operation order (glm 0.9.9 gtc/matrix_transform.inl), so the reference's
// matrices come out bit for bit; the y flip of src/Camera.cpp:15,32.
struct H3 {
    float x, y, z;
};
H3 h_norm(H3 a) {
    const float inv = 1.0f / std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z);
    return H3{a.x * inv, a.y * inv, a.z * inv};
}
H3 h_cross(H3 a, H3 b) { return H3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
float h_dot(H3 a, H3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

void look_at(H3 eye, H3 ctr, H3 up, float* m) {
    const H3 f = h_norm(H3{ctr.x - eye.x, ctr.y - eye.y, ctr.z - eye.z});
    const H3 s = h_norm(h_cross(f, up));
    const H3 u = h_cross(s, f);
    const float cols[4][4] = {{s.x, u.x, -f.x, 0.f},
                              {s.y, u.y, -f.y, 0.f},
                              {s.z, u.z, -f.z, 0.f},
                              {-h_dot(s, eye), -h_dot(u, eye), h_dot(f, eye), 1.f}};
    std::memcpy(m, cols, sizeof cols);
}

void perspective_flipped(float fovy_deg, float aspect, float znear, float zfar, float* m) {
    const float fovy = fovy_deg * 0.01745329251994329576923690768489f;   // glm::radians
    const float t = std::tan(fovy / 2.0f);
    std::memset(m, 0, 16 * sizeof(float));
    m[0] = 1.0f / (aspect * t);
    m[5] = -(1.0f / t);
    m[10] = zfar / (znear - zfar);
    m[11] = -1.0f;
    m[14] = -(zfar * znear) / (zfar - znear);
}

// Eye of a rigid view matrix, -R^T t, in double rounded once.
void eye_of(const float* view, float out[3]) {
    for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc -= double(view[i * 4 + k]) * double(view[12 + k]);
        out[i] = float(acc);
    }
}

// Column-major a * b in double, rounded once.
void mat_mul(const float* a, const float* b, float* o) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += double(a[k * 4 + r]) * double(b[c * 4 + k]);
            o[c * 4 + r] = float(acc);
        }
}

bool finite16(const float* m) {
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(m[k])) return false;
    return true;
}

rvh_status check_desc(const rvh_shade_desc& d) {
    if (d.map_width < 1 || d.map_height < 1 || d.map_width > 16384 || d.map_height > 16384)
        return fail(RVH_ERR_INVALID_ARG, "shade: map size must be in [1, 16384]");
    if (d.map_mode != RVH_SHADE_MAPS_VERTICES && d.map_mode != RVH_SHADE_MAPS_QUADS)
        return fail(RVH_ERR_INVALID_ARG, "shade: map_mode must be RVH_SHADE_MAPS_VERTICES or RVH_SHADE_MAPS_QUADS");
    if (d.image_mode != RVH_IMAGE_NEAREST && d.image_mode != RVH_IMAGE_BLEND)
        return fail(RVH_ERR_INVALID_ARG, "shade: image_mode must be RVH_IMAGE_NEAREST or RVH_IMAGE_BLEND");
    if (!finite16(d.camera_view) || !finite16(d.camera_proj) || !finite16(d.light_view) || !finite16(d.light_proj))
        return fail(RVH_ERR_INVALID_ARG, "shade: non-finite matrix");
    return RVH_OK;
}

Cam make_cam(const rvh_shade_desc& d) {
    Cam K;
    mat_mul(d.light_proj, d.light_view, K.lvp);
    eye_of(d.camera_view, K.cam_pos);
    eye_of(d.light_view, K.light_pos);
    return K;
}

int grid_for(long long n, int sms) {
    const long long b = (n + kShadeThreads - 1) / kShadeThreads;
    return (int)std::max(1LL, std::min(b, (long long)sms * 8));
}

constexpr long long kMaxClipped = 1LL << 20;   // near-clipped quads drawn per rasterising pass

// The asset's lists for one rasterising call over n_seg quads into px pixels
// (grown as needed, counters zeroed): near-clipped quads (up to kMaxClipped),
// the pixels deferred to the search resolve (up to px) and the pixels the first
// ordering pass leaves to the second (up to px).
rvh_status raster_lists(Asset* a, long long n_seg, long long px, cudaStream_t s, ClipList* CL, DeferList* D,
                        DeferList* Over = nullptr) {
    const long long cap = std::max(1LL, std::min(n_seg, kMaxClipped));
    const long long npx = std::max(1LL, px);
    const size_t need = size_t(3 + cap + 2 * npx) * 4;
    if (a->raster_clip.bytes < need) {
        a->ctx->free(a->raster_clip);
        rvh_status st = a->ctx->alloc(a->raster_clip, need);
        if (st != RVH_OK) return st;
    }
    auto* p = static_cast<unsigned*>(a->raster_clip.ptr);
    RVH_CUDA(cudaMemsetAsync(p, 0, 12, s));
    *CL = ClipList{p, p + 3, unsigned(cap), 1};
    if (D) *D = DeferList{p + 1, p + 3 + cap, unsigned(npx)};
    if (Over) *Over = DeferList{p + 2, p + 3 + cap + npx, unsigned(npx)};
    return RVH_OK;
}

// The same list, read by a later pass over the same quads.
ClipList reuse(ClipList CL) {
    CL.append = 0;
    return CL;
}

// The hair pass with in-order blending: count the fragments per pixel, scan,
// list them, resolve per pixel.  Scratch (counts, offsets, cursors, tile sums,
// fragment list) lives in the asset, grown as needed; the fragment total is
// read back once to size the list.
rvh_status render_blend(Asset* a, const TessView& T, const RasterDev& R, const Maps& M, long long n_seg, long long px,
                        float4* img, unsigned* ids, cudaStream_t s) {
    if (n_seg >= (1LL << 31)) return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: blending needs fewer than 2^31 segments");
    const int sms = a->ctx->sm_count;
    const long long tiles = (px + kScanTile - 1) / kScanTile;
    // counts, offs (+1), cursor, tile sums, the active pixels and their number
    const size_t need_px = size_t(px) * 4 * 4 + 8 + size_t(tiles) * 4;
    if (a->raster_px.bytes < need_px) {
        a->ctx->free(a->raster_px);
        rvh_status st = a->ctx->alloc(a->raster_px, need_px);
        if (st != RVH_OK) return st;
    }
    unsigned* counts = static_cast<unsigned*>(a->raster_px.ptr);
    unsigned* offs = counts + px;
    unsigned* cursor = offs + px + 1;
    unsigned* sums = cursor + px;
    unsigned* active = sums + tiles;
    unsigned* n_active = active + px;
    RVH_CUDA(cudaMemsetAsync(counts, 0, size_t(px) * 4, s));
    RVH_CUDA(cudaMemsetAsync(n_active, 0, 4, s));
    ClipList CL{};
    DeferList D{}, Over{};
    rvh_status lst = raster_lists(a, n_seg, px, s, &CL, &D, &Over);
    if (lst != RVH_OK) return lst;
    if (n_seg > 0) {
        k_blend_count<<<grid_for(n_seg, sms), kShadeThreads, 0, s>>>(T, R, (unsigned)n_seg, CL, counts);
        k_listed_quads<<<sms, kShadeThreads, 0, s>>>(T, R, CL, BlendCountFrag{counts, R.width});
    }
    k_scan_tiles<<<unsigned(tiles), kShadeThreads, 0, s>>>(counts, px, offs, sums);
    k_scan_sums<<<1, kShadeThreads, 0, s>>>(sums, int(tiles));
    k_scan_add<<<grid_for(px, sms), kShadeThreads, 0, s>>>(counts, px, sums, offs, cursor, active, n_active);
    RVH_CUDA(cudaGetLastError());
    unsigned total = 0;
    RVH_CUDA(cudaMemcpyAsync(&total, offs + px, 4, cudaMemcpyDeviceToHost, s));
    RVH_CUDA(cudaStreamSynchronize(s));
    const size_t need_f = size_t(std::max(total, 1u)) * 8;
    if (a->raster_frags.bytes < need_f) {
        a->ctx->free(a->raster_frags);
        rvh_status st = a->ctx->alloc(a->raster_frags, need_f + need_f / 4);   // room to grow
        if (st != RVH_OK) return st;
    }
    auto* frags = static_cast<unsigned long long*>(a->raster_frags.ptr);
    if (n_seg > 0) {
        const BlendScatterFrag F{cursor, frags, (unsigned long long)total, R.width, kListedFrag};
        k_blend_scatter<<<grid_for(n_seg, sms), kShadeThreads, 0, s>>>(T, R, (unsigned)n_seg, reuse(CL), cursor, frags,
                                                                        (unsigned long long)total);
        k_listed_quads<<<sms, kShadeThreads, 0, s>>>(T, R, CL, F);
    }
    const float4 clear = make_float4(101.f / 255.f, 129.f / 255.f, 140.f / 255.f, 1.0f);   // Renderer.cpp:2235
    unsigned* pass_count = counts;   // zeroed by k_scan_add (the counts are in offs)
    if (!prepare_kernel(reinterpret_cast<const void*>(k_blend_order<kOrderCap>)))
        return fail(RVH_ERR_CUDA, "asset_render_hair: shared memory opt-in of the ordering kernel");
    k_blend_order<kOrderCapSmall><<<sms * 5, kShadeThreads, order_smem_bytes(kOrderCapSmall), s>>>(
        active, n_active, offs, frags, pass_count, D, Over);
    k_blend_order<kOrderCap><<<sms * 3, kShadeThreads, order_smem_bytes(kOrderCap), s>>>(Over.ids, Over.count, offs,
                                                                                        frags, pass_count, D, DeferList{});
    k_blend_shade<<<grid_for(px * 32, sms), kShadeThreads, 0, s>>>(T, R, M, px, offs, frags, pass_count, clear, img, ids);
    k_blend_resolve<<<sms, kShadeThreads, 0, s>>>(T, R, M, offs, frags, clear, img, ids, D);
    RVH_CUDA(cudaGetLastError());
    return RVH_OK;
}


bool aligned16(const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; }

// Column-major 4x4 inverse by Gauss-Jordan with partial pivoting, in double (the
// oracle's restatement uses the same steps, so both round to the same floats).
bool invert4(const double* m, double* inv) {
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

void mul4d(const double* a, const double* b, double* o) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc += a[k * 4 + r] * b[c * 4 + k];
            o[c * 4 + r] = acc;
        }
}

// hair.frag:260's brightness factor per isoline, with the kernel's hash
// (a correctly rounded sin: the double sin rounded once).
Lines line_table(int n_lines) {
    Lines B{};
    for (int j = 0; j < n_lines; ++j) {
        const float u = (float)j / (float)n_lines;
        const float d = u * 12.9898f + u * 78.233f;
        const float m = (float)std::sin((double)d) * 43758.5453123f;
        B.bright[j] = 0.8f * std::fabs(m - std::floor(m)) + 0.6f;
    }
    return B;
}

float hash01(float x, float y) {   // random(x, y) with the double sin rounded once
    const float d = x * 12.9898f + y * 78.233f;
    const float m = (float)std::sin((double)d) * 43758.5453123f;
    return m - std::floor(m);
}

void set_line_tables(RasterDev& R, int n_lines) {
    for (int j = 0; j < kMaxLines; ++j) R.rnd[j] = R.bright[j] = 0.f;
    for (int j = 0; j < n_lines; ++j) {
        const float uu = (float)j / (float)n_lines;
        R.rnd[j] = std::fabs(hash01(3.242551f * uu, uu * uu)) + 0.5f;   // hair.geom:46
        R.bright[j] = 0.8f * std::fabs(hash01(uu, uu)) + 0.6f;         // hair.frag:260
    }
}

bool raster_setup(const rvh_shade_desc& d, int n_lines, int w, int h, RasterDev& R) {
    double cv[16], cp[16], lv[16], lp[16], t[16], u[16], icv[16], icp[16], vp[16];
    for (int k = 0; k < 16; ++k) {
        cv[k] = d.camera_view[k];
        cp[k] = d.camera_proj[k];
        lv[k] = d.light_view[k];
        lp[k] = d.light_proj[k];
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
    eye_of(d.camera_view, R.cam_pos);
    eye_of(d.light_view, R.light_pos);
    R.width = w;
    R.height = h;
    set_line_tables(R, n_lines);
    return true;
}

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_shade_desc_reference(rvh_shade_desc* d) {
    if (!d) return fail(RVH_ERR_INVALID_ARG, "shade_desc_reference: NULL");
    std::memset(d, 0, sizeof(*d));
    const float aspect = 1080.f / 720.f;                          // src/main.cpp:162-163,188-189
    const H3 up{0.0f, 1.0f, 0.0f}, ctr{0.0f, 1.0f, 0.0f};
    look_at(H3{0.0f, 1.f, 10.f}, ctr, up, d->camera_view);        // src/Camera.cpp:9-15
    perspective_flipped(45.0f, aspect, 0.1f, 50.0f, d->camera_proj);
    const H3 nrm = h_norm(H3{2.f - 0.f, 0.f - 1.f, 1.f - 0.f});  // src/Camera.cpp:28-32
    look_at(H3{6.5f * nrm.x, 6.5f * nrm.y, 6.5f * nrm.z}, ctr, up, d->light_view);
    perspective_flipped(60.0f, aspect, 1.f, 10.f, d->light_proj);
    d->map_width = 1080;                                          // SHADOWMAP_WIDTH x HEIGHT, src/Renderer.cpp:9-10
    d->map_height = 720;
    d->map_mode = RVH_SHADE_MAPS_QUADS;                           // the passes draw hair.geom's quads
    d->image_mode = RVH_IMAGE_BLEND;                              // the hair pipeline blends (Renderer.cpp:1672-1677)
    return RVH_OK;
}

rvh_status rvh_shade_fragments(rvh_context* ctx, int64_t n, const void* inputs, const void* depth_map,
                               const void* opacity_map, int32_t map_width, int32_t map_height, void* colors,
                               void* stream) {
    if (!ctx || n < 0) return fail(RVH_ERR_INVALID_ARG, "shade_fragments: NULL context or negative count");
    if (map_width < 1 || map_height < 1) return fail(RVH_ERR_INVALID_ARG, "shade_fragments: bad map size");
    if (n == 0) return RVH_OK;
    if (!inputs || !depth_map || !opacity_map || !colors)
        return fail(RVH_ERR_INVALID_ARG, "shade_fragments: NULL buffer");
    if (!aligned16(opacity_map) || !aligned16(colors) || !aligned16(inputs))
        return fail(RVH_ERR_INVALID_ARG, "shade_fragments: inputs, opacity map and colors must be 16-byte aligned");
    RVH_DEVICE(ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const Maps M{static_cast<const float*>(depth_map), static_cast<const float*>(opacity_map), map_width, map_height};
    k_shade_fragments<<<grid_for(n, ctx->sm_count), kShadeThreads, 0, s>>>((long long)n, static_cast<const float*>(inputs), M,
                                                                              static_cast<float4*>(colors));
    RVH_CUDA(cudaGetLastError());
    return RVH_OK;
}

rvh_status rvh_asset_shade(rvh_asset* a, const rvh_tess_desc* td, const rvh_shade_desc* sd, const void* vertices,
                           const void* frames, void* depth_map, void* opacity_map, void* colors, void* stream) {
    TraceRange trace("rvh_asset_shade");
    if (!a || !td || !sd) return fail(RVH_ERR_INVALID_ARG, "asset_shade: NULL argument");
    rvh_status st = check_desc(*sd);
    if (st != RVH_OK) return st;
    if (td->n_lines < 1 || td->n_lines > kMaxLines || td->n_segments < 1 || td->n_segments > 256)
        return fail(RVH_ERR_INVALID_ARG, "asset_shade: n_lines must be in [1, 64], n_segments in [1, 256]");
    if (!depth_map || !opacity_map) return fail(RVH_ERR_INVALID_ARG, "asset_shade: NULL map");
    if (a->n_strands > 0 && (!vertices || !frames)) return fail(RVH_ERR_INVALID_ARG, "asset_shade: NULL buffer");
    if (!aligned16(vertices) || !aligned16(frames) || !aligned16(opacity_map) || !aligned16(colors) ||
        reinterpret_cast<uintptr_t>(depth_map) % 4)
        return fail(RVH_ERR_INVALID_ARG, "asset_shade: float4 buffers 16-byte aligned, the depth map 4-byte");
    RVH_DEVICE(a->ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : a->ctx->stream;
    const Cam K = make_cam(*sd);
    const int w = sd->map_width, h = sd->map_height;
    const long long texels = (long long)w * h;
    const long long nv = (long long)a->n_strands * td->n_lines * (td->n_segments + 1);
    if (nv >= (1LL << 32) - (long long)a->ctx->sm_count * 8 * kShadeThreads)
        return fail(RVH_ERR_INVALID_ARG, "asset_shade: fewer than 2^32 tessellated vertices per asset");
    const int sms = a->ctx->sm_count;
    auto* depth_bits = static_cast<unsigned*>(depth_map);
    auto* counts = static_cast<uint4*>(opacity_map);   // layer counts in place until the finish pass
    k_clear_maps<<<grid_for(texels, sms), kShadeThreads, 0, s>>>(texels, depth_bits, counts);
    if (nv > 0 && sd->map_mode == RVH_SHADE_MAPS_QUADS) {
        RasterDev R;   // the light camera as the geometry shader's camera
        std::memcpy(R.vp, K.lvp, sizeof R.vp);
        for (int q = 0; q < 16; ++q) R.lmap[q] = (q % 5 == 0) ? 1.f : 0.f;
        for (int q = 0; q < 3; ++q) R.cam_pos[q] = R.light_pos[q] = K.light_pos[q];
        R.width = w;
        R.height = h;
        set_line_tables(R, td->n_lines);
        const TessView T{static_cast<const float4*>(vertices), static_cast<const float4*>(frames), a->n_points,
                         td->n_lines, td->n_segments};
        const long long n_seg = (long long)a->n_strands * td->n_lines * td->n_segments;
        ClipList CL{};
        st = raster_lists(a, n_seg, 0, s, &CL, nullptr);
        if (st != RVH_OK) return st;
        k_light_quads_depth<<<grid_for(n_seg, sms), kShadeThreads, 0, s>>>(T, R, (unsigned)n_seg, CL, depth_bits);
        k_listed_quads<<<sms, kShadeThreads, 0, s>>>(T, R, CL, LightDepthFrag{depth_bits, R.width});
        const LightOpacityFrag F{static_cast<const float*>(depth_map), reinterpret_cast<unsigned long long*>(counts),
                                 R.width, R.height};
        k_light_quads_opacity<<<grid_for(n_seg, sms), kShadeThreads, 0, s>>>(T, R, (unsigned)n_seg, reuse(CL),
                                                                            static_cast<const float*>(depth_map), counts);
        k_listed_quads<<<sms, kShadeThreads, 0, s>>>(T, R, CL, F);
    } else if (nv > 0) {
        const VertexWalk W{static_cast<const float4*>(vertices), (long long)a->n_strands * (td->n_segments + 1),
                           td->n_lines, td->n_segments + 1};
        k_light_depth<<<grid_for(W.n_columns, sms), kShadeThreads, 0, s>>>(W, K, w, h, depth_bits);
        k_light_opacity<<<grid_for(W.n_columns, sms), kShadeThreads, 0, s>>>(W, K, w, h,
                                                                             static_cast<const float*>(depth_map), counts);
    }
    k_opacity_finish<<<grid_for(texels, sms), kShadeThreads, 0, s>>>(texels, counts);
    if (nv > 0 && colors) {   // colours are optional: the maps alone feed rvh_asset_render_hair
        const Maps M{static_cast<const float*>(depth_map), static_cast<const float*>(opacity_map), w, h};
        k_shade_vertices<<<grid_for(nv, sms), kShadeThreads, 0, s>>>(
            static_cast<const float4*>(vertices), static_cast<const float4*>(frames), a->n_strands, a->n_points,
            td->n_lines, td->n_segments, K, M, line_table(td->n_lines), static_cast<float4*>(colors));
    }
    RVH_CUDA(cudaGetLastError());
    return RVH_OK;
}

rvh_status rvh_asset_render_hair(rvh_asset* a, const rvh_tess_desc* td, const rvh_shade_desc* sd, const void* vertices,
                                 const void* frames, const void* depth_map, const void* opacity_map, int32_t width,
                                 int32_t height, void* image, void* fragment_ids, void* stream) {
    TraceRange trace("rvh_asset_render_hair");
    if (!a || !td || !sd) return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: NULL argument");
    rvh_status st = check_desc(*sd);
    if (st != RVH_OK) return st;
    if (td->n_lines < 1 || td->n_lines > kMaxLines || td->n_segments < 1 || td->n_segments > 256)
        return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: n_lines must be in [1, 64], n_segments in [1, 256]");
    if (width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: image size must be in [1, 16384]");
    if (!image || !depth_map || !opacity_map || (a->n_strands > 0 && (!vertices || !frames)))
        return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: NULL buffer");
    if (!aligned16(image) || !aligned16(vertices) || !aligned16(frames) || !aligned16(opacity_map) ||
        reinterpret_cast<uintptr_t>(depth_map) % 4 || reinterpret_cast<uintptr_t>(fragment_ids) % 4)
        return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: float4 buffers 16-byte aligned, others 4-byte");
    const long long n_seg = (long long)a->n_strands * td->n_lines * td->n_segments;
    if (n_seg >= (1LL << 32) - (long long)a->ctx->sm_count * 8 * kShadeThreads)
        return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: fewer than 2^32 segments per asset");
    RasterDev R;
    if (!raster_setup(*sd, td->n_lines, width, height, R))
        return fail(RVH_ERR_INVALID_ARG, "asset_render_hair: a camera matrix is singular");
    RVH_DEVICE(a->ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : a->ctx->stream;
    const TessView T{static_cast<const float4*>(vertices), static_cast<const float4*>(frames), a->n_points, td->n_lines,
                     td->n_segments};
    const Maps M{static_cast<const float*>(depth_map), static_cast<const float*>(opacity_map), sd->map_width,
                 sd->map_height};
    const long long px = (long long)width * height;
    const int sms = a->ctx->sm_count;
    auto* img = static_cast<float4*>(image);
    if (sd->image_mode == RVH_IMAGE_BLEND) return render_blend(a, T, R, M, n_seg, px, img, static_cast<unsigned*>(fragment_ids), s);
    k_image_clear<<<grid_for(px, sms), kShadeThreads, 0, s>>>(px, img);
    ClipList CL{};
    DeferList D{};
    st = raster_lists(a, n_seg, px, s, &CL, &D);
    if (st != RVH_OK) return st;
    if (n_seg > 0) {
        k_hair_raster<<<grid_for(n_seg, sms), kShadeThreads, 0, s>>>(T, R, (unsigned)n_seg, CL, img);
        k_listed_quads<<<sms, kShadeThreads, 0, s>>>(T, R, CL,
                                                      NearestFrag{reinterpret_cast<unsigned long long*>(img), R.width});
    }
    auto* fid = static_cast<unsigned*>(fragment_ids);
    k_hair_resolve<false><<<grid_for(px, sms), kShadeThreads, 0, s>>>(T, R, M, px, img, fid, D);
    k_hair_resolve<true><<<sms, kShadeThreads, 0, s>>>(T, R, M, px, img, fid, D);
    RVH_CUDA(cudaGetLastError());
    return RVH_OK;
}

rvh_status rvh_render_image(rvh_context* ctx, int64_t n_vertices, const void* vertices, const void* colors,
                            const rvh_shade_desc* sd, int32_t width, int32_t height, void* image, void* stream) {
    if (!ctx || !sd || n_vertices < 0) return fail(RVH_ERR_INVALID_ARG, "render_image: NULL argument");
    if (width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(RVH_ERR_INVALID_ARG, "render_image: size must be in [1, 16384]");
    if (!finite16(sd->camera_view) || !finite16(sd->camera_proj))
        return fail(RVH_ERR_INVALID_ARG, "render_image: non-finite matrix");
    if (!image || (n_vertices > 0 && (!vertices || !colors))) return fail(RVH_ERR_INVALID_ARG, "render_image: NULL buffer");
    if (!aligned16(image) || !aligned16(vertices) || !aligned16(colors))
        return fail(RVH_ERR_INVALID_ARG, "render_image: buffers must be 16-byte aligned");
    if (n_vertices > 0xffffffffLL) return fail(RVH_ERR_INVALID_ARG, "render_image: at most 2^32 - 1 vertices");
    RVH_DEVICE(ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    float vp[16];
    mat_mul(sd->camera_proj, sd->camera_view, vp);
    Proj P;
    std::memcpy(P.m, vp, sizeof vp);
    const long long px = (long long)width * height;
    auto* img = static_cast<float4*>(image);
    k_image_clear<<<grid_for(px, ctx->sm_count), kShadeThreads, 0, s>>>(px, img);
    if (n_vertices > 0)
        k_image_depth<<<grid_for(n_vertices, ctx->sm_count), kShadeThreads, 0, s>>>(
            static_cast<const float4*>(vertices), n_vertices, P, width, height, img);
    k_image_resolve<<<grid_for(px, ctx->sm_count), kShadeThreads, 0, s>>>(px, static_cast<const float4*>(colors), img);
    RVH_CUDA(cudaGetLastError());
    return RVH_OK;
}

}  // extern "C"
