/*
 * tess_oracle.hpp — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's strand tessellation, the
 * single-strand-clumping path of src/shaders/hair.tese (what the shader
 * finally emits: pos = singleStrandPos, :305-311), with the tessellation
 * levels of src/shaders/hair.tesc:19-20 (12 isolines x 42 segments) as
 * parameters.  Per output vertex (isoline j, vertex k of strand s):
 *
 *   u = j / n_lines, v = k / n_segments                  (gl_TessCoord.y, .x)
 *   segment sf = floor(v * (n-1)), t = v * (n-1) - sf     (:166-167, :219)
 *   Bezier control points from the 4 surrounding points, the end neighbours
 *   mirrored (:45-66), evaluated by de Casteljau with glm's
 *   mix(a, b, t) = a + t * (b - a) (:69-77)
 *   width = clumpRadius * mix(mix(0.05, 0.3, v), mix(0.3, 0.1, v), v)
 *           * (|random(u, u*u)| + 0.5)                   (:237-241)
 *   dir = normalize(cos(2 pi u), 0, sin(2 pi u)) * sd    (:245-246, :284)
 *   sd from randomChoice = random(u, root.x) * random(root.y, root.z)
 *   (five profiles of v above 0.5, 1 otherwise, 1 at v = 0; :253-283)
 *   pos = c + width * dir,  w = mix(rootWidth, tipWidth, v)   (:308, :326)
 *   frame = tangent normalize(P[sf+1] - P[sf]) and its Frisvad basis (:289-297)
 *
 * random(st) = fract(sin(dot(st, (12.9898, 78.233))) * 43758.5453123)
 * (:29-31).  The hash multiplies sin's rounding by 43758, so its value
 * depends on the sin implementation: RefSin::kFloat calls the C library's
 * float sin (what the reference compiled on this host does), RefSin::kDouble
 * rounds the double sin once (a correctly rounded sin, the library's
 * definition, reproducible on the GPU).
 *
 * Two deliberate definitions where the shader is undefined:
 *   - at v = 1 the shader indexes point n (out of bounds); here the last
 *     segment is used with t = 1, which ends the curve at the tip;
 *   - n is a runtime value (the shader fixes NUM_CURVE_POINTS = 10).
 *
 * Operation order follows the shader (separately rounded float operations;
 * build with -ffp-contract=off).  Per-line and per-vertex constants are
 * tables, computed once per (n_lines, n_segments, constants).
 */
#pragma once

#include <cmath>
#include <vector>

namespace oracle {
namespace tess {

enum class RefSin { kFloat, kDouble };

struct TessParams {
    int n_lines = 12;          // hair.tesc:19, gl_TessLevelOuter[0]
    int n_segments = 42;       // hair.tesc:20, gl_TessLevelOuter[1]
    float clump_radius = 0.5f; // hair.tese:239
    float root_width = 0.02f;  // hair.tese:324
    float tip_width = 0.01f;   // hair.tese:325
};

inline float t_fract(float x) { return x - std::floor(x); }
inline float t_mix(float a, float b, float t) { return a + t * (b - a); }

inline float tess_random(float x, float y, RefSin mode) {
    const float d = x * 12.9898f + y * 78.233f;   // dot: (x * a) + (y * b)
    const float s = mode == RefSin::kFloat ? std::sin(d) : (float)std::sin((double)d);
    return t_fract(s * 43758.5453123f);
}

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
inline V3 vmix(V3 a, V3 b, float t) { return a + t * (b - a); }
inline float vdot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// glm normalize: v * inversesqrt(dot(v, v)), inversesqrt = 1 / sqrt
inline V3 vnormalize(V3 a) { return a * (1.0f / std::sqrt(vdot(a, a))); }

// Profile index of randomChoice (0: sd = 1)
inline int sd_profile(float choice) {
    if (!(choice > 0.5f)) return 0;
    if (choice > 0.9f) return 1;
    if (choice > 0.8f) return 2;
    if (choice > 0.7f) return 3;
    if (choice > 0.6f) return 4;
    return 5;
}

struct TessTables {
    std::vector<float> u, v;           // per line, per vertex
    std::vector<float> width;          // [line][vertex]
    std::vector<V3> dir;               // per line
    std::vector<float> sd;             // [profile 0..5][vertex]
    std::vector<float> strand_width;   // per vertex
};

inline TessTables tess_tables(const TessParams& P, RefSin mode) {
    TessTables T;
    const int L = P.n_lines, S = P.n_segments;
    for (int j = 0; j < L; ++j) T.u.push_back((float)j / (float)L);
    for (int k = 0; k <= S; ++k) T.v.push_back((float)k / (float)S);
    const float PI = 3.141592653f;
    for (int j = 0; j < L; ++j) {
        const float u = T.u[j];
        const float rand2 = std::fabs(tess_random(u, u * u, mode));
        for (int k = 0; k <= S; ++k) {
            const float v = T.v[k];
            T.width.push_back(P.clump_radius * t_mix(t_mix(0.05f, 0.3f, v), t_mix(0.3f, 0.1f, v), v) * (rand2 + 0.5f));
        }
        const float uRad = 2.f * PI * u;
        T.dir.push_back(vnormalize(v3(std::cos(uRad), 0.f, std::sin(uRad))));
    }
    const float den = 2.0f * std::pow(0.2f, 2.0f);
    for (int p = 0; p < 6; ++p)
        for (int k = 0; k <= S; ++k) {
            const float v = T.v[k];
            float sd = 1.0f;
            switch (p) {
                case 1: sd = 1.8f * std::exp(-std::pow(v - 0.25f, 2.0f) / den); break;
                case 2: sd = 4.5f * std::pow(v, 10.0f); break;
                case 3: sd = 2.5f * std::exp(-std::pow(v - 0.7f, 2.0f) / den); break;
                case 4: sd = 4.f * std::pow(v, 1.3f); break;
                case 5: sd = 1.8f * std::exp(-std::pow(v - 0.8f, 2.0f) / den); break;
                default: break;
            }
            if (v == 0.0f) sd = 1.0f;
            T.sd.push_back(sd);
        }
    for (int k = 0; k <= S; ++k) T.strand_width.push_back(t_mix(P.root_width, P.tip_width, T.v[k]));
    return T;
}

// Frisvad's orthonormal basis of unit n (hair.tese:140-151)
inline void frisvad(V3 n, V3& b1, V3& b2) {
    if (n.z < -0.9999999f) {
        b1 = v3(0.0f, -1.0f, 0.0f);
        b2 = v3(-1.0f, 0.0f, 0.0f);
        return;
    }
    const float a = 1.0f / (1.0f + n.z);
    const float b = -n.x * n.y * a;
    b1 = vnormalize(v3(1.0f - n.x * n.x * a, b, -n.x));
    b2 = vnormalize(v3(b, 1.0f - n.y * n.y * a, -n.y));
}

/*
 * Tessellates ns strands of n points (Strand records, float4 curvePoints
 * first).  out: ns * n_lines * (n_segments + 1) float4 {pos, width};
 * frames (nullable): ns * (n - 1) * 3 float4 {tangent, b1, b2} (w = 0).
 */
inline void tessellate(const float* records, int ns, int n, const TessParams& P, RefSin mode, float* out,
                       float* frames) {
    const TessTables T = tess_tables(P, mode);
    const int L = P.n_lines, S = P.n_segments;
    std::vector<V3> pts(n), b1s(n > 1 ? n - 1 : 0), b2s(n > 1 ? n - 1 : 0);
    for (int s = 0; s < ns; ++s) {
        const float* rec = records + size_t(s) * 12 * n;
        for (int i = 0; i < n; ++i) pts[i] = v3(rec[4 * i], rec[4 * i + 1], rec[4 * i + 2]);
        for (int sf = 0; sf + 1 < n; ++sf) {   // control points of each segment (:45-66)
            const V3 p1 = pts[sf], p2 = pts[sf + 1];
            const V3 p0 = sf == 0 ? p1 + (p1 - p2) : pts[sf - 1];
            const V3 p3 = sf + 1 == n - 1 ? p2 + (p2 - p1) : pts[sf + 2];
            b1s[sf] = p1 + ((1.0f / 3.0f) * ((p2 - p0) / 2.0f));
            b2s[sf] = p2 - ((1.0f / 3.0f) * ((p3 - p1) / 2.0f));
            if (frames) {
                const V3 tg = vnormalize(pts[sf + 1] - pts[sf]);
                V3 f1, f2;
                frisvad(tg, f1, f2);
                float* fr = frames + (size_t(s) * (n - 1) + sf) * 12;
                const V3 fs[3] = {tg, f1, f2};
                for (int q = 0; q < 3; ++q) {
                    fr[4 * q] = fs[q].x;
                    fr[4 * q + 1] = fs[q].y;
                    fr[4 * q + 2] = fs[q].z;
                    fr[4 * q + 3] = 0.f;
                }
            }
        }
        const V3 root = pts[0];
        const float ryz = tess_random(root.y, root.z, mode);
        for (int j = 0; j < L; ++j) {
            const float choice = tess_random(T.u[j], root.x, mode) * ryz;
            const float* sdt = &T.sd[size_t(sd_profile(choice)) * (S + 1)];
            for (int k = 0; k <= S; ++k) {
                const float v = T.v[k];
                const float x = v * (float)(n - 1);
                int sf = (int)std::floor(x);
                if (sf > n - 2) sf = n - 2;
                const float t = x - (float)sf;
                const V3 b0 = pts[sf], b1 = b1s[sf], b2 = b2s[sf], b3 = pts[sf + 1];
                const V3 b01 = vmix(b0, b1, t), b11 = vmix(b1, b2, t), b21 = vmix(b2, b3, t);
                const V3 b02 = vmix(b01, b11, t), b12 = vmix(b11, b21, t);
                const V3 c = vmix(b02, b12, t);
                const V3 dir = T.dir[j] * sdt[k];
                const V3 pos = c + T.width[size_t(j) * (S + 1) + k] * dir;
                float* o = out + ((size_t(s) * L + j) * (S + 1) + k) * 4;
                o[0] = pos.x;
                o[1] = pos.y;
                o[2] = pos.z;
                o[3] = T.strand_width[k];
            }
        }
    }
}

}  // namespace tess
}  // namespace oracle
