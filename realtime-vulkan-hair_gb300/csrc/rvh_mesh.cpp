// rvh_mesh.cpp — scalp meshes and hair-root sampling on them.
//
// The reference builds its hair asset from an OBJ scalp
// (GeneratePointsOnMesh, src/Strand.cpp:26-146): the OBJ is read with
// polygons triangulated, flattened into face-vertex arrays (triangle t has
// corners 3t, 3t+1, 3t+2, each with a position and a normal,
// src/Strand.cpp:55-84), and each root picks a triangle uniformly with
// rand() % n_triangles after srand(8), then a point u*p1 + v*p2 + (1-u-v)*p3
// with u, v = rand()/RAND_MAX folded into the triangle, and the triangle's
// first normal (src/Strand.cpp:88-110).
//
// This file reads OBJ text itself (v, vn, f; 1-based and negative indices),
// triangulates polygons with the same ear-clipping rule as the loader the
// reference vendors (tiny_obj_loader 2.0, src/tiny_obj_loader.h:1328-1560: a
// projection plane from the first non-degenerate corner, the polygon's signed
// area, an ear is a corner turning with the polygon whose triangle contains no
// other remaining vertex, the ear's middle vertex is removed, the last three
// vertices form the last triangle), so triangle indices — and so the sampled
// roots — match the reference's.  Its rand() is the glibc generator (additive
// feedback, r[i] = r[i-3] + r[i-31], seeded by the 16807 multiplicative
// congruence, 310 outputs discarded), restated here so every host gives the
// same sequence.  A second sampler is area-uniform (the reference's own TODO,
// src/Strand.cpp:92), on SplitMix64.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "rvh_internal.hpp"
#include "../../include/rvh_scene.h"

struct rvh_mesh {
    std::vector<float> pos;   // 9 floats per triangle (3 corners)
    std::vector<float> nrm;   // 9 floats per triangle
    double area = 0.0;
};

namespace rvh {
namespace {

// ---- glibc-compatible rand() --------------------------------------------------
struct LibcRand {
    uint32_t ring[31];   // the last 31 values of the feedback sequence
    int head = 0;
    explicit LibcRand(uint32_t seed) {
        int32_t s[344];
        s[0] = seed == 0 ? 1 : (int32_t)seed;
        for (int k = 1; k < 31; ++k) {
            // s[k] = 16807 * s[k-1] mod (2^31 - 1), kept in signed range
            const int64_t t = (16807LL * s[k - 1]) % 2147483647LL;
            s[k] = (int32_t)(t < 0 ? t + 2147483647LL : t);
        }
        for (int k = 31; k < 34; ++k) s[k] = s[k - 31];
        std::vector<uint32_t> all(344);
        for (int k = 0; k < 34; ++k) all[k] = (uint32_t)s[k];
        for (int k = 34; k < 344; ++k) all[k] = all[k - 31] + all[k - 3];
        for (int k = 0; k < 31; ++k) ring[k] = all[344 - 31 + k];
        head = 0;
    }
    // next rand(): o = (r[k-31] + r[k-3]) >> 1 over the last 31 values
    int32_t next() {
        const uint32_t a = ring[head];             // r[k-31]
        const uint32_t b = ring[(head + 28) % 31]; // r[k-3]
        const uint32_t v = a + b;
        ring[head] = v;
        head = (head + 1) % 31;
        return (int32_t)(v >> 1);
    }
};

// ---- OBJ reading ------------------------------------------------------------------
struct FaceVert {
    int v = -1, vn = -1;
};

bool fix_index(long idx, size_t n, int* out) {
    if (idx > 0) {
        *out = (int)(idx - 1);
        return true;
    }
    if (idx == 0) return false;   // zero is not a valid OBJ index
    *out = (int)((long)n + idx);  // negative: relative to the last element so far
    return true;
}

// ---- in_triangle and triangulate: derived from tiny_obj_loader 2.0 ----------
// They restate the polygon triangulation of tiny_obj_loader 2.0 (the loader
// the reference vendors, src/tiny_obj_loader.h:1314-1326 and :1380-1500), so
// that triangle t of a mesh is the reference's triangle t.  That code is
// distributed under the MIT License:
//
//   The MIT License (MIT)
//
//   Copyright (c) 2012-2018 Syoyo Fujita and many contributors.
//
//   Permission is hereby granted, free of charge, to any person obtaining a copy
//   of this software and associated documentation files (the "Software"), to deal
//   in the Software without restriction, including without limitation the rights
//   to use, copy, modify, merge, publish, distribute, sublicense, and/or sell
//   copies of the Software, and to permit persons to whom the Software is
//   furnished to do so, subject to the following conditions:
//
//   The above copyright notice and this permission notice shall be included in
//   all copies or substantial portions of the Software.
//
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS OR
//   IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF MERCHANTABILITY,
//   FITNESS FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT. IN NO EVENT SHALL THE
//   AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR ANY CLAIM, DAMAGES OR OTHER
//   LIABILITY, WHETHER IN AN ACTION OF CONTRACT, TORT OR OTHERWISE, ARISING FROM,
//   OUT OF OR IN CONNECTION WITH THE SOFTWARE OR THE USE OR OTHER DEALINGS IN
//   THE SOFTWARE.

// tiny_obj_loader's pnpoly (W. R. Franklin's crossing test) on three vertices.
bool in_triangle(const float* vx, const float* vy, float tx, float ty) {
    bool c = false;
    for (int a = 0, b = 2; a < 3; b = a++)
        if (((vy[a] > ty) != (vy[b] > ty)) && (tx < (vx[b] - vx[a]) * (ty - vy[a]) / (vy[b] - vy[a]) + vx[a])) c = !c;
    return c;
}

// Triangulates one polygon (corner list) into `out` (3 corners per triangle)
// with the ear-clipping rule described at the top of the file.
void triangulate(const std::vector<FaceVert>& face, const std::vector<float>& v, std::vector<FaceVert>& out) {
    const size_t np0 = face.size();
    if (np0 < 3) return;
    int ax0 = 1, ax1 = 2;
    for (size_t k = 0; k < np0; ++k) {
        const FaceVert &i0 = face[k % np0], &i1 = face[(k + 1) % np0], &i2 = face[(k + 2) % np0];
        const float* p0 = &v[3 * i0.v];
        const float* p1 = &v[3 * i1.v];
        const float* p2 = &v[3 * i2.v];
        const float e0x = p1[0] - p0[0], e0y = p1[1] - p0[1], e0z = p1[2] - p0[2];
        const float e1x = p2[0] - p1[0], e1y = p2[1] - p1[1], e1z = p2[2] - p1[2];
        const float cx = std::fabs(e0y * e1z - e0z * e1y);
        const float cy = std::fabs(e0z * e1x - e0x * e1z);
        const float cz = std::fabs(e0x * e1y - e0y * e1x);
        const float eps = std::numeric_limits<float>::epsilon();
        if (cx > eps || cy > eps || cz > eps) {
            if (!(cx > cy && cx > cz)) {
                ax0 = 0;
                if (cz > cx && cz > cy) ax1 = 1;
            }
            break;
        }
    }
    float area = 0.f;
    for (size_t k = 0; k < np0; ++k) {
        const float* p0 = &v[3 * face[k].v];
        const float* p1 = &v[3 * face[(k + 1) % np0].v];
        area += (p0[ax0] * p1[ax1] - p0[ax1] * p1[ax0]) * 0.5f;
    }
    std::vector<FaceVert> rem = face;
    size_t guess = 0;
    size_t iters_left = rem.size(), prev_size = rem.size();
    while (rem.size() > 3 && iters_left > 0) {
        const size_t np = rem.size();
        if (guess >= np) guess -= np;
        if (prev_size != np) {
            prev_size = np;
            iters_left = np;
        } else {
            --iters_left;
        }
        FaceVert ind[3];
        float vx[3], vy[3];
        for (int k = 0; k < 3; ++k) {
            ind[k] = rem[(guess + k) % np];
            vx[k] = v[3 * ind[k].v + ax0];
            vy[k] = v[3 * ind[k].v + ax1];
        }
        const float e0x = vx[1] - vx[0], e0y = vy[1] - vy[0];
        const float e1x = vx[2] - vx[1], e1y = vy[2] - vy[1];
        const float cross = e0x * e1y - e0y * e1x;
        if (cross * area < 0.f) {  // reflex corner
            guess += 1;
            continue;
        }
        bool overlap = false;
        for (size_t o = 3; o < np; ++o) {
            const size_t idx = (guess + o) % np;
            const float* q = &v[3 * rem[idx].v];
            if (in_triangle(vx, vy, q[ax0], q[ax1])) {
                overlap = true;
                break;
            }
        }
        if (overlap) {
            guess += 1;
            continue;
        }
        out.push_back(ind[0]);
        out.push_back(ind[1]);
        out.push_back(ind[2]);
        rem.erase(rem.begin() + (long)((guess + 1) % np));   // drop the ear's middle vertex
    }
    if (rem.size() == 3) {
        out.push_back(rem[0]);
        out.push_back(rem[1]);
        out.push_back(rem[2]);
    }
}

rvh_status parse_obj(FILE* f, rvh_mesh& m) {
    std::vector<float> v, vn;
    std::vector<FaceVert> tris, face;
    std::string line, cur;
    char buf[4096];
    int lineno = 0;
    auto handle = [&](const std::string& ln) -> rvh_status {
        const char* p = ln.c_str();
        while (*p == ' ' || *p == '\t') ++p;
        if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
            float a[3] = {0.f, 0.f, 0.f};
            char* e = const_cast<char*>(p + 2);
            for (int k = 0; k < 3; ++k) a[k] = (float)std::strtod(e, &e);
            v.insert(v.end(), a, a + 3);
        } else if (p[0] == 'v' && p[1] == 'n' && (p[2] == ' ' || p[2] == '\t')) {
            float a[3] = {0.f, 0.f, 0.f};
            char* e = const_cast<char*>(p + 3);
            for (int k = 0; k < 3; ++k) a[k] = (float)std::strtod(e, &e);
            vn.insert(vn.end(), a, a + 3);
        } else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
            face.clear();
            const char* q = p + 2;
            const size_t nv = v.size() / 3, nn = vn.size() / 3;
            for (;;) {
                while (*q == ' ' || *q == '\t') ++q;
                if (*q == '\0' || *q == '\r' || *q == '\n') break;
                FaceVert fv;
                char* e = nullptr;
                long iv = std::strtol(q, &e, 10);
                if (!fix_index(iv, nv, &fv.v)) return fail(RVH_ERR_INVALID_ARG, "obj: bad vertex index on line " + std::to_string(lineno));
                q = e;
                if (*q == '/') {
                    ++q;
                    if (*q != '/') {  // texture coordinate: read and ignore
                        std::strtol(q, &e, 10);
                        q = e;
                    }
                    if (*q == '/') {
                        ++q;
                        long in = std::strtol(q, &e, 10);
                        if (!fix_index(in, nn, &fv.vn)) return fail(RVH_ERR_INVALID_ARG, "obj: bad normal index on line " + std::to_string(lineno));
                        q = e;
                    }
                }
                while (*q && *q != ' ' && *q != '\t' && *q != '\r' && *q != '\n') ++q;
                if (fv.v < 0 || size_t(fv.v) >= nv) return fail(RVH_ERR_INVALID_ARG, "obj: vertex index out of range on line " + std::to_string(lineno));
                if (fv.vn >= 0 && size_t(fv.vn) >= nn) return fail(RVH_ERR_INVALID_ARG, "obj: normal index out of range on line " + std::to_string(lineno));
                face.push_back(fv);
            }
            triangulate(face, v, tris);
        }
        return RVH_OK;
    };
    while (std::fgets(buf, sizeof buf, f)) {
        line = buf;
        const bool full = !line.empty() && line.back() == '\n';
        if (!full && !std::feof(f)) {   // a line longer than the buffer: keep reading it
            cur += line;
            continue;
        }
        cur += line;
        while (!cur.empty() && (cur.back() == '\n' || cur.back() == '\r')) cur.pop_back();
        ++lineno;
        const rvh_status s = handle(cur);
        cur.clear();
        if (s != RVH_OK) return s;
    }
    if (!cur.empty()) {
        const rvh_status s = handle(cur);
        if (s != RVH_OK) return s;
    }
    const size_t nt = tris.size() / 3;
    m.pos.resize(9 * nt);
    m.nrm.resize(9 * nt);
    for (size_t t = 0; t < nt; ++t) {
        const float* c[3] = {&v[3 * tris[3 * t].v], &v[3 * tris[3 * t + 1].v], &v[3 * tris[3 * t + 2].v]};
        // corners without a normal get the triangle's geometric normal
        float gn[3];
        {
            const float e0[3] = {c[1][0] - c[0][0], c[1][1] - c[0][1], c[1][2] - c[0][2]};
            const float e1[3] = {c[2][0] - c[0][0], c[2][1] - c[0][1], c[2][2] - c[0][2]};
            gn[0] = e0[1] * e1[2] - e0[2] * e1[1];
            gn[1] = e0[2] * e1[0] - e0[0] * e1[2];
            gn[2] = e0[0] * e1[1] - e0[1] * e1[0];
            const float l = std::sqrt(gn[0] * gn[0] + gn[1] * gn[1] + gn[2] * gn[2]);
            for (int a = 0; a < 3; ++a) gn[a] = l > 0.f ? gn[a] / l : 0.f;
        }
        for (int k = 0; k < 3; ++k) {
            const FaceVert& fv = tris[3 * t + k];
            for (int a = 0; a < 3; ++a) {
                m.pos[9 * t + 3 * k + a] = c[k][a];
                m.nrm[9 * t + 3 * k + a] = fv.vn >= 0 ? vn[3 * fv.vn + a] : gn[a];
            }
        }
    }
    return RVH_OK;
}

double tri_area(const float* p) {
    const double e0[3] = {double(p[3]) - p[0], double(p[4]) - p[1], double(p[5]) - p[2]};
    const double e1[3] = {double(p[6]) - p[0], double(p[7]) - p[1], double(p[8]) - p[2]};
    const double c[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
    return 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
}

void finish_mesh(rvh_mesh& m) {
    m.area = 0.0;
    for (size_t t = 0; t < m.pos.size() / 9; ++t) m.area += tri_area(&m.pos[9 * t]);
}

}  // namespace
}  // namespace rvh

using namespace rvh;

extern "C" {

rvh_status rvh_mesh_load_obj(const char* path, rvh_mesh** out) {
    if (!path || !out) return fail(RVH_ERR_INVALID_ARG, "mesh_load_obj: NULL argument");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(RVH_ERR_INVALID_ARG, std::string("mesh_load_obj: cannot open ") + path);
    rvh_mesh* m = new (std::nothrow) rvh_mesh();
    if (!m) {
        std::fclose(f);
        return fail(RVH_ERR_OUT_OF_MEMORY, "mesh_load_obj: out of host memory");
    }
    const rvh_status s = parse_obj(f, *m);
    std::fclose(f);
    if (s != RVH_OK) {
        delete m;
        return s;
    }
    finish_mesh(*m);
    *out = m;
    return RVH_OK;
}

rvh_status rvh_mesh_from_triangles(const float* positions, const float* normals, int32_t n_triangles, rvh_mesh** out) {
    if (!out || n_triangles < 0 || (n_triangles > 0 && (!positions || !normals)))
        return fail(RVH_ERR_INVALID_ARG, "mesh_from_triangles: bad arguments");
    rvh_mesh* m = new (std::nothrow) rvh_mesh();
    if (!m) return fail(RVH_ERR_OUT_OF_MEMORY, "mesh_from_triangles: out of host memory");
    m->pos.assign(positions, positions + 9 * size_t(n_triangles));
    m->nrm.assign(normals, normals + 9 * size_t(n_triangles));
    finish_mesh(*m);
    *out = m;
    return RVH_OK;
}

void rvh_mesh_destroy(rvh_mesh* m) { delete m; }

rvh_status rvh_mesh_info(const rvh_mesh* m, int32_t* n_triangles, double* area) {
    if (!m) return fail(RVH_ERR_INVALID_ARG, "mesh_info: NULL mesh");
    if (n_triangles) *n_triangles = (int32_t)(m->pos.size() / 9);
    if (area) *area = m->area;
    return RVH_OK;
}

rvh_status rvh_mesh_triangles(const rvh_mesh* m, float* positions, float* normals) {
    if (!m) return fail(RVH_ERR_INVALID_ARG, "mesh_triangles: NULL mesh");
    if (positions) std::memcpy(positions, m->pos.data(), m->pos.size() * sizeof(float));
    if (normals) std::memcpy(normals, m->nrm.data(), m->nrm.size() * sizeof(float));
    return RVH_OK;
}

rvh_status rvh_libc_rand_sequence(uint32_t seed, int32_t n, int32_t* out) {
    if (n < 0 || (n > 0 && !out)) return fail(RVH_ERR_INVALID_ARG, "libc_rand_sequence: bad arguments");
    LibcRand r(seed);
    for (int32_t k = 0; k < n; ++k) out[k] = r.next();
    return RVH_OK;
}

rvh_status rvh_mesh_sample_roots(const rvh_mesh* m, const rvh_mesh_roots_desc* d, float* roots, float* normals) {
    if (!m || !d) return fail(RVH_ERR_INVALID_ARG, "mesh_sample_roots: NULL argument");
    if (d->n_roots < 0 || (d->n_roots > 0 && (!roots || !normals)))
        return fail(RVH_ERR_INVALID_ARG, "mesh_sample_roots: bad output arrays");
    const int32_t nt = (int32_t)(m->pos.size() / 9);
    if (d->n_roots > 0 && nt == 0) return fail(RVH_ERR_INVALID_ARG, "mesh_sample_roots: the mesh has no triangles");
    if (d->normal_mode != RVH_ROOT_NORMAL_FIRST_CORNER && d->normal_mode != RVH_ROOT_NORMAL_INTERPOLATED)
        return fail(RVH_ERR_INVALID_ARG, "mesh_sample_roots: unknown normal mode");
    auto put_normal = [&](int32_t i, int32_t t, float b0, float b1, float b2) {
        const float* n = &m->nrm[9 * size_t(t)];
        if (d->normal_mode == RVH_ROOT_NORMAL_FIRST_CORNER) {
            for (int a = 0; a < 3; ++a) normals[3 * i + a] = n[a];
            return;
        }
        float v[3];
        for (int a = 0; a < 3; ++a) v[a] = b0 * n[a] + b1 * n[3 + a] + b2 * n[6 + a];
        const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int a = 0; a < 3; ++a) normals[3 * i + a] = l > 0.f ? v[a] / l : n[a];
    };
    if (d->mode == RVH_MESH_ROOTS_REFERENCE) {
        // src/Strand.cpp:88-110: triangle = rand() % nt; u, v = rand() / (float)RAND_MAX,
        // folded when u + v >= 1; pos = p1*u + p2*v + p3*(1 - u - v); the first corner's normal
        LibcRand r((uint32_t)d->seed);
        const float rand_max = 2147483647.0f;   // (float)RAND_MAX rounds to 2^31
        for (int32_t i = 0; i < d->n_roots; ++i) {
            const int32_t t = r.next() % nt;
            float u = (float)r.next() / rand_max;
            float v = (float)r.next() / rand_max;
            if (u + v >= 1.f) {
                u = 1.f - u;
                v = 1.f - v;
            }
            const float* p = &m->pos[9 * size_t(t)];
            const float w = (1.f - u) - v;
            for (int a = 0; a < 3; ++a) roots[3 * i + a] = (p[a] * u + p[3 + a] * v) + p[6 + a] * w;
            put_normal(i, t, u, v, w);
        }
        return RVH_OK;
    }
    if (d->mode == RVH_MESH_ROOTS_AREA) {
        if (!(m->area > 0.0)) return fail(RVH_ERR_INVALID_ARG, "mesh_sample_roots: the mesh has zero area");
        std::vector<double> cum(size_t(nt) + 1, 0.0);
        for (int32_t t = 0; t < nt; ++t) cum[t + 1] = cum[t] + tri_area(&m->pos[9 * size_t(t)]);
        for (int32_t i = 0; i < d->n_roots; ++i) {
            const double x = rvh_rng_uniform(d->seed, 3ull * (uint64_t)i) * cum[nt];
            int32_t lo = 0, hi = nt - 1;   // first t with cum[t+1] > x
            while (lo < hi) {
                const int32_t mid = (lo + hi) / 2;
                if (cum[mid + 1] > x) hi = mid;
                else lo = mid + 1;
            }
            const double s = std::sqrt(rvh_rng_uniform(d->seed, 3ull * (uint64_t)i + 1));
            const double r2 = rvh_rng_uniform(d->seed, 3ull * (uint64_t)i + 2);
            const double b0 = 1.0 - s, b1 = s * (1.0 - r2), b2 = s * r2;   // uniform on the triangle
            const float* p = &m->pos[9 * size_t(lo)];
            for (int a = 0; a < 3; ++a) roots[3 * i + a] = (float)(b0 * p[a] + b1 * p[3 + a] + b2 * p[6 + a]);
            put_normal(i, lo, (float)b0, (float)b1, (float)b2);
        }
        return RVH_OK;
    }
    return fail(RVH_ERR_INVALID_ARG, "mesh_sample_roots: unknown mode");
}

}  // extern "C"
