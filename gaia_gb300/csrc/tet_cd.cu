// Contact detection of the tet VBD step (see tet_cd.hpp). Compiled with --fmad=false:
// every FP32 operation of the predicates rounds on its own, in the order written, as
// in the CPU oracle, so that contact sets match it bit for bit.
//
// Order of one pass (VBD/VBDPhysics.cpp:1958-2035 dcd, 2037-2076 intermediateDCD,
// 2078-2116 ccd, 2118-2156 intermediateCCD, 1812-1894 prepareCollisionDataGPU):
//   substep start: DCD on the positions at the start of the substep for the surface
//     vertices below collisionOffHeight (a vertex strictly inside a tet is "penetrated"
//     and gets the nearest feasible surface face of that tet's mesh); without DCD all
//     results are cleared; CCD for the vertices below the height (current positions)
//     that DCD did not mark;
//   intermediate: DCD on the current positions for the penetrated vertices (for all
//     when CCD is off); CCD as above;
//   then the records: every hit becomes its vertex's own contact and a relation of each
//   face vertex that has fewer than four, in (mesh, surface vertex) order.
// Results of vertices a pass does not revisit are kept, as in the reference.
//
// The cubic root finder below (cubic_roots, find_closed, quadratic_roots) follows, branch
// for branch, the one in Cem Yuksel's cyCodeBase (cyPolynomial.h, the method of "High-
// Performance Polynomial Root Finding for Graphics", HPG 2022), specialised to float and
// degree 3; the CCD result must equal the reference's bit for bit, so the structure is
// kept. cyCodeBase is distributed under the MIT license:
//   Copyright (c) 2022, Cem Yuksel <cem@cemyuksel.com>. All rights reserved.
//   Permission is hereby granted, free of charge, to any person obtaining a copy of this
//   software and associated documentation files (the "Software"), to deal in the Software
//   without restriction, including without limitation the rights to use, copy, modify,
//   merge, publish, distribute, sublicense, and/or sell copies of the Software, and to
//   permit persons to whom the Software is furnished to do so, subject to the following
//   conditions: The above copyright notice and this permission notice shall be included in
//   all copies or substantial portions of the Software. THE SOFTWARE IS PROVIDED "AS IS",
//   WITHOUT WARRANTY OF ANY KIND, EXPRESS OR IMPLIED, INCLUDING BUT NOT LIMITED TO THE
//   WARRANTIES OF MERCHANTABILITY, FITNESS FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT. IN
//   NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR ANY CLAIM, DAMAGES OR
//   OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT, TORT OR OTHERWISE, ARISING FROM, OUT
//   OF OR IN CONNECTION WITH THE SOFTWARE OR THE USE OR OTHER DEALINGS IN THE SOFTWARE.
#include "tet_cd.hpp"

#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <stdexcept>
#include <string>

#include "lbvh.cuh"

namespace gaia {
namespace tetcd {
namespace {

using cloth::add;
using cloth::closest_point_triangle;
using cloth::cross;
using cloth::dot;
using cloth::ld3;
using cloth::mul;
using cloth::sub;
using cloth::v3;

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
#define TCD_CUDA(x) check((x), #x)

template <typename T>
T* dalloc(size_t n, size_t& bytes) {
    T* p = nullptr;
    if (n == 0) n = 1;
    TCD_CUDA(cudaMalloc(&p, n * sizeof(T)));
    bytes += n * sizeof(T);
    return p;
}
inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

constexpr float kCmpEps = 1e-5f;       // CMP_EPSILON (Types/Types.h:20)
constexpr float kRootError = 6e-4f;    // PolynomialDefaultError<float> (cyPolynomial.h:168)
constexpr int kMaxBracketSteps = 256;  // bound of the safeguarded root iteration
constexpr int kStack = 64;

struct Dev {
    int32_t nslots, nsv, nf;
    const int4* faces;
    const int4* face_nbr;
    const int2* sv;
    const int32_t* ring_ofs;
    const int32_t* ring;
    const int4* tets;
    const int32_t* tet_mesh;
    const int4* tet_nbr;   // per tet: tet across the face omitting vertex x/y/z/w (-1: none)
    const int2* face_tet;  // per face: the tet it bounds, the local vertex it omits
    int32_t* hit;        // per surface vertex: global face or -1
    float* hit_tt;       // CCD time of impact, -1 for a DCD hit
    uint8_t* pen;        // per surface vertex: DCD found it inside a tet (substep start)
    unsigned long long* counters;
};

// ---- FP32 geometry in the oracle's operation order ------------------------------
__device__ __forceinline__ float3 neg(float3 a) { return v3(a.x * -1.f, a.y * -1.f, a.z * -1.f); }
__device__ __forceinline__ float3 normalized(float3 v) {
    const float l = sqrtf(dot(v, v));
    return v3(v.x / l, v.y / l, v.z / l);
}

// pointInTet (CollisionDetector/CollisionGeometry.h:56-82)
__device__ __forceinline__ float tet_vol6(float3 a, float3 b, float3 c, float3 d) {
    return dot(sub(b, a), cross(sub(c, a), sub(d, a)));
}
__device__ bool point_in_tet(float3 p, float3 a, float3 b, float3 c, float3 d) {
    const float vol = tet_vol6(a, b, c, d);
    if (fabsf(vol) < kCmpEps) return false;
    const float3 vs[4] = {a, b, c, d};
    const int order[4][3] = {{1, 2, 3}, {2, 0, 3}, {0, 1, 3}, {1, 0, 2}};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float3 v1 = vs[order[i][0]], v2 = vs[order[i][1]], v3_ = vs[order[i][2]];
        if (dot(sub(p, v1), cross(sub(v2, v1), sub(v3_, v2))) * vol >= 0.f) return false;
    }
    return true;
}

// ---- CCD of a moving point against a moving triangle (CCDSolver.h:97-196 with the
// cubic root finder of cyPolynomial.h: CubicRoots 800-903, FindClosed 382-450) ----------
__device__ __forceinline__ float fmin_ref(float a, float b) { return a <= b ? a : b; }
__device__ __forceinline__ float fmax_ref(float a, float b) { return a >= b ? a : b; }
__device__ __forceinline__ bool diff_sign(float a, float b) { return (a < 0.f) != (b < 0.f); }
__device__ __forceinline__ float mult_sign(float v, float s) { return v * (s < 0.f ? -1.0f : 1.0f); }
__device__ __forceinline__ float eval3(const float* c, float x) {
    float r = c[3];
    r = r * x + c[2];
    r = r * x + c[1];
    return r * x + c[0];
}
__device__ __forceinline__ float eval2(const float* c, float x) {
    float r = c[2];
    r = r * x + c[1];
    return r * x + c[0];
}

__device__ int quadratic_roots(float* roots, const float* c, float x0, float x1) {
    const float cc = c[0], b = c[1], a = c[2];
    const float delta = b * b - 4.0f * a * cc;
    if (delta > 0.f) {
        const float d = sqrtf(delta);
        const float q = -0.5f * (b + mult_sign(d, b));
        const float rv0 = q / a, rv1 = cc / q;
        const float r0 = fmin_ref(rv0, rv1), r1 = fmax_ref(rv0, rv1);
        const int r0i = (r0 >= x0) & (r0 <= x1);
        const int r1i = (r1 >= x0) & (r1 <= x1);
        roots[0] = r0;
        roots[r0i] = r1;
        return r0i + r1i;
    }
    if (delta < 0.f) return 0;
    const float r0 = -0.5f * b / a;
    roots[0] = r0;
    return (r0 >= x0) & (r0 <= x1);
}

// The single root in [x0, x1] of a cubic that changes sign there: up to 16 clamped
// Newton steps from the midpoint, then Newton steps safeguarded by bisection of the
// sign-change bracket (Yuksel, "High-Performance Polynomial Root Finding for
// Graphics", HPG 2022).
__device__ float find_closed(const float* coef, const float* deriv, float x0, float x1, float y0) {
    const float xError = kRootError;
    const float ep2 = 2.0f * xError;
    float xr = (x0 + x1) / 2.0f;
    if (x1 - x0 <= ep2) return xr;
    const float xr0 = xr;
    for (int k = 0; k < 16; ++k) {
        float xn = xr - eval3(coef, xr) / eval2(deriv, xr);
        xn = fmin_ref(x1, fmax_ref(x0, xn));
        if (fabsf(xr - xn) <= xError) return xn;
        xr = xn;
    }
    if (!isfinite(xr)) xr = xr0;
    float yr = eval3(coef, xr);
    float xb0 = x0, xb1 = x1;
    for (int k = 0; k < kMaxBracketSteps; ++k) {
        const bool side = diff_sign(y0, yr);
        if (side) xb1 = xr;
        else xb0 = xr;
        const float dy = eval2(deriv, xr);
        const float xn = xr - yr / dy;
        if (xn > xb0 && xn < xb1) {
            const float step = fabsf(xr - xn);
            xr = xn;
            if (step > xError) yr = eval3(coef, xr);
            else break;
        } else {
            xr = (xb0 + xb1) / 2.0f;
            if (xr == xb0 || xr == xb1 || xb1 - xb0 <= ep2) break;
            yr = eval3(coef, xr);
        }
    }
    return xr;
}

__device__ int deflate_rest(float* roots, const float* coef, float lo, float x1) {
    float def[3];
    def[2] = coef[3];
    def[1] = coef[2] + roots[0] * def[2];
    def[0] = coef[1] + roots[0] * def[1];
    return quadratic_roots(roots + 1, def, lo, x1) + 1;
}

__device__ int cubic_roots(float* roots, const float* coef, float x0, float x1) {
    const float y0 = eval3(coef, x0), y1 = eval3(coef, x1);
    const float a = coef[3] * 3.0f, b_2 = coef[2], c = coef[1];
    const float deriv[3] = {c, 2.0f * b_2, a};
    const float delta_4 = b_2 * b_2 - a * c;
    if (delta_4 > 0.f) {
        const float d_2 = sqrtf(delta_4);
        const float q = -(b_2 + mult_sign(d_2, b_2));
        const float rv0 = q / a, rv1 = c / q;
        const float xa = fmin_ref(rv0, rv1), xb = fmax_ref(rv0, rv1);
        if (diff_sign(y0, y1)) {
            if (xa >= x1 || xb <= x0 || (xa <= x0 && xb >= x1)) {
                roots[0] = find_closed(coef, deriv, x0, x1, y0);
                return 1;
            }
        } else {
            if ((xa >= x1 || xb <= x0) || (xa <= x0 && xb >= x1)) return 0;
        }
        if (xa > x0) {
            const float ya = eval3(coef, xa);
            if (diff_sign(y0, ya)) {
                roots[0] = find_closed(coef, deriv, x0, xa, y0);
                if (diff_sign(ya, y1) || (xb < x1 && diff_sign(ya, eval3(coef, xb))))
                    return deflate_rest(roots, coef, xa, x1);
                return 1;
            }
            if (xb < x1) {
                const float yb = eval3(coef, xb);
                if (diff_sign(ya, yb)) {
                    roots[0] = find_closed(coef, deriv, xa, xb, ya);
                    if (diff_sign(yb, y1)) return deflate_rest(roots, coef, xb, x1);
                    return 1;
                }
                if (diff_sign(yb, y1)) {
                    roots[0] = find_closed(coef, deriv, xb, x1, yb);
                    return 1;
                }
            } else if (diff_sign(ya, y1)) {
                roots[0] = find_closed(coef, deriv, xa, x1, ya);
                return 1;
            }
        } else {
            const float yb = eval3(coef, xb);
            if (diff_sign(y0, yb)) {
                roots[0] = find_closed(coef, deriv, x0, xb, y0);
                if (diff_sign(yb, y1)) return deflate_rest(roots, coef, xb, x1);
                return 1;
            }
            if (diff_sign(yb, y1)) {
                roots[0] = find_closed(coef, deriv, xb, x1, yb);
                return 1;
            }
        }
        return 0;
    }
    if (diff_sign(y0, y1)) {
        roots[0] = find_closed(coef, deriv, x0, x1, y0);
        return 1;
    }
    return 0;
}

__device__ __forceinline__ float3 lerp(float3 a, float3 b, float t) { return add(a, mul(t, sub(b, a))); }
__device__ __forceinline__ float cross2(float ax, float ay, float bx, float by) { return -ay * bx + ax * by; }

// Returns 1 with the time of impact tt if the point p0 -> p1 passes through the moving
// triangle a[k] -> b[k] during [0, 1].
__device__ int ccd_tri_point(const float3* a, const float3* b, float3 p0, float3 p1, float& tt) {
    const float3 A[4] = {a[0], a[1], a[2], p0};
    const float3 B[4] = {b[0], b[1], b[2], p1};
    const float3 dx0 = sub(B[0], A[0]), dx1 = sub(B[1], A[1]), dx2 = sub(B[2], A[2]), dx3 = sub(B[3], A[3]);
    const float3 e1 = sub(A[1], A[0]), e2 = sub(A[2], A[0]), e3 = sub(A[3], A[0]);
    const float3 de0 = sub(dx3, dx0), de1 = sub(dx1, dx0), de2 = sub(dx2, dx0);
    const float3 e1xe2 = cross(e1, e2);
    const float3 de1xde2 = cross(de1, de2);
    const float3 mixed = add(cross(e1, de2), cross(de1, e2));
    float poly[4];
    poly[0] = dot(e3, e1xe2);
    poly[1] = dot(de0, e1xe2) + dot(e3, mixed);
    poly[2] = dot(e3, de1xde2) + dot(de0, mixed);
    poly[3] = dot(de0, de1xde2);
    float t[3];
    const int nt = cubic_roots(t, poly, 0.0f, 1.0f);
    for (int i = 0; i < nt; ++i) {
        const float3 q0 = lerp(A[0], B[0], t[i]), q1 = lerp(A[1], B[1], t[i]);
        const float3 q2 = lerp(A[2], B[2], t[i]), q3 = lerp(A[3], B[3], t[i]);
        const float3 n = cross(sub(q1, q0), sub(q2, q0));
        const float nx = fabsf(n.x), ny = fabsf(n.y), nz = fabsf(n.z);
        const int xy = nx < ny, xz = nx < nz, yz = ny < nz;
        const int axis = (xy | xz) + (xz & yz);
        float w[4][2];
        const float3 q[4] = {q0, q1, q2, q3};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            w[k][0] = axis == 0 ? q[k].y : q[k].x;
            w[k][1] = axis == 2 ? q[k].y : q[k].z;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            w[k][0] = w[k][0] - w[3][0];
            w[k][1] = w[k][1] - w[3][1];
        }
        const bool s01 = signbit(cross2(w[0][0], w[0][1], w[1][0], w[1][1]));
        const bool s12 = signbit(cross2(w[1][0], w[1][1], w[2][0], w[2][1]));
        const bool s20 = signbit(cross2(w[2][0], w[2][1], w[0][0], w[0][1]));
        if (s01 == s12 && s01 == s20) {
            tt = t[i];
            return 1;
        }
    }
    return 0;
}

// checkEdgeFeasibleRegion / checkVertexFeasibleRegion (DiscreteCollisionDetector.cpp:
// 703-815) for the closest point of type `type` on global face g.
__device__ bool feasible(const Dev& D, const float4* P, float3 p, int32_t g, int type, float eps) {
    if (type == cloth::AtInterior) return true;
    const int4 fv = D.faces[g];
    if (type >= cloth::AtAB) {
        const int k = type == cloth::AtAB ? 0 : (type == cloth::AtBC ? 1 : 2);
        const int32_t e1 = k == 0 ? fv.x : (k == 1 ? fv.y : fv.z);
        const int32_t e2 = k == 0 ? fv.y : (k == 1 ? fv.z : fv.x);
        const int4 nbs = D.face_nbr[g];
        const int32_t nb = k == 0 ? nbs.x : (k == 1 ? nbs.y : nbs.z);
        if (nb < 0) return true;
        const int4 gv = D.faces[nb];
        const float3 n1 = neg(normalized(cross(sub(ld3(P, fv.y), ld3(P, fv.x)), sub(ld3(P, fv.z), ld3(P, fv.x)))));
        const float3 n2 = neg(normalized(cross(sub(ld3(P, gv.y), ld3(P, gv.x)), sub(ld3(P, gv.z), ld3(P, gv.x)))));
        const float3 v1 = ld3(P, e1), v2 = ld3(P, e2);
        const float3 AP = sub(p, v1), BP = sub(p, v2), AB = sub(v2, v1), BA = neg(AB);
        const float relaxed = -dot(AB, AB) * eps;
        if (dot(AP, AB) < relaxed) return false;
        if (dot(BP, BA) < relaxed) return false;
        if (dot(AP, cross(n1, AB)) < relaxed) return false;
        if (dot(AP, cross(n2, BA)) < relaxed) return false;
        return true;
    }
    const int32_t va = type == cloth::AtA ? fv.x : (type == cloth::AtB ? fv.y : fv.z);
    const float3 A = ld3(P, va), AP = sub(p, A);
    for (int32_t r = D.ring_ofs[va]; r < D.ring_ofs[va + 1]; ++r) {
        const float3 BA = sub(A, ld3(P, D.ring[r]));
        if (dot(AP, BA) < -dot(BA, BA) * eps) return false;
    }
    return true;
}

// ---- tetrahedral traversal (TetMesh/TetMeshFEM.cpp:503-740 static, 908-1100 dynamic) ----
// The walk from a surface face along a ray through the tets of its mesh that the DCD
// closest-point query requires to reach the tet containing the query point
// (CollisionDetector/DiscreteCollisionDetector.cpp:189-300). One thread walks; the
// candidate exit faces form a stack of (tet << 2 | local face) entries.
__constant__ int kTet4Faces[4][3] = {{1, 2, 3}, {2, 0, 3}, {0, 1, 3}, {1, 0, 2}};  // TetMeshFEM::tet4Faces
__constant__ int kExit3[3][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}};                 // posibleExit3Faces
constexpr int kStaticStack = 32;      // SIZE_CANDIDATE_FACE_STACK
constexpr int kLoopRing = 32;         // SIZE_TRAVERSED_CIRCULAR_ARRAY
constexpr int kPassThroughSteps = 5;  // TetMeshFEM::passThroughCheckSteps
constexpr int kDynamicStack = 256;    // bound of the dynamic walk (a std::vector in the reference)
constexpr int kMaxWalkSteps = 1 << 16;

struct TraverseCfg {
    int check, non_self, stop_after, shift_center, use_static;
    float shift, eps, max_mult;
};

TraverseCfg traverse_cfg(const Params& p) {
    return TraverseCfg{p.check_traverse, p.traverse_non_self, p.stop_after_passing, p.shift_to_center, p.static_traverse,
                       p.center_shift, p.ray_eps, p.max_search_mult};
}

__device__ __forceinline__ int tv_of(int4 q, int k) { return k == 0 ? q.x : (k == 1 ? q.y : (k == 2 ? q.z : q.w)); }

struct Walk {
    const float4* P;
    const int4* tets;
    const int4* nbr;
    float3 o, ax0, ax1;
    float max_dis, eps;
    int32_t target;

    // projectTo2DCoordinates: the incoming face's vertices in tet4Faces order, then the apex
    __device__ void project(int4 q, int inc, float2* p, float3* X) const {
        for (int i = 0; i < 4; ++i) {
            X[i] = ld3(P, tv_of(q, i < 3 ? kTet4Faces[inc][i] : inc));
            const float3 d = sub(X[i], o);
            p[i] = make_float2(dot(ax0, d), dot(ax1, d));
        }
    }
    // exitFaceSelection (TetMesh/TetMeshFEM.h:423-483)
    __device__ void exits(const float2* p, bool* out) const {
        const float v1x = p[1].x - p[0].x, v1y = p[1].y - p[0].y, v2x = p[2].x - p[0].x, v2y = p[2].y - p[0].y;
        const float area = v1x * v2y - v1y * v2x;
        const float sg = copysignf(1.0f, area);
        const float d0 = p[3].x * p[0].y - p[3].y * p[0].x;
        const float d1 = p[3].x * p[1].y - p[3].y * p[1].x;
        const float d2 = p[3].x * p[2].y - p[3].y * p[2].x;
        out[0] = d1 * sg >= -eps && d2 * sg <= eps;
        out[1] = d2 * sg >= -eps && d0 * sg <= eps;
        out[2] = d0 * sg >= -eps && d1 * sg <= eps;
    }
    // the ray's crossing of exit face i lies beyond max_dis (originBarycentric2DTriangle)
    __device__ bool passed(const float2* p, const float3* X, int i) const {
        const float2 a = p[kExit3[i][0]], b = p[kExit3[i][1]], c = p[kExit3[i][2]];
        const float v0x = b.x - a.x, v0y = b.y - a.y, v1x = c.x - a.x, v1y = c.y - a.y, v2x = -a.x, v2y = -a.y;
        const float den = v0x * v1y - v1x * v0y;
        const float w1 = (v2x * v1y - v1x * v2y) / den;
        const float w2 = (v0x * v2y - v2x * v0y) / den;
        const float w0 = 1.0f - w1 - w2;
        const float3 A = X[kExit3[i][0]], B = X[kExit3[i][1]], C = X[kExit3[i][2]];
        const float3 x = v3((w0 * A.x + w1 * B.x) + w2 * C.x, (w0 * A.y + w1 * B.y) + w2 * C.y,
                            (w0 * A.z + w1 * B.z) + w2 * C.z);
        const float3 d = sub(x, o);
        return dot(d, d) > max_dis * max_dis;
    }
};

// 1 reached, 0 not reached, -1 gave up on a bound
__device__ __noinline__ int walk(const Walk& w, int32_t start, int start_face, bool dynamic, int32_t* stack) {
    const int cap = dynamic ? kDynamicStack : kStaticStack;
    int32_t ring[kLoopRing];
    int nring = 0;
    ring[nring++ % kLoopRing] = start;
    float2 p[4];
    float3 X[4];
    bool ex[3];
    int4 q = w.tets[start];
    w.project(q, start_face, p, X);
    w.exits(p, ex);
    int sp = 0;
    for (int i = 0; i < 3; ++i)
        if (ex[i]) stack[sp++] = (start << 2) | kTet4Faces[start_face][i];
    int n = 0;
    for (int steps = 0; sp > 0; ++steps) {
        if (steps >= kMaxWalkSteps) return -1;
        const int32_t e = stack[--sp];
        const int32_t prev = e >> 2;
        const int f = e & 3;
        const int4 qp = w.tets[prev];
        const int32_t fv0 = tv_of(qp, kTet4Faces[f][0]), fv1 = tv_of(qp, kTet4Faces[f][1]), fv2 = tv_of(qp, kTet4Faces[f][2]);
        const int32_t cur = tv_of(w.nbr[prev], f);
        if (cur == w.target) return 1;
        if (cur < 0) return 0;  // reached the boundary
        bool seen = false;
        const int m = nring < kLoopRing ? nring : kLoopRing;
        for (int i = 0; i < m; ++i) seen |= ring[i] == cur;
        if (seen) continue;
        ring[nring++ % kLoopRing] = cur;
        q = w.tets[cur];
        const int32_t apex = q.x ^ q.y ^ q.z ^ q.w ^ fv0 ^ fv1 ^ fv2;
        const int inc = apex == q.x ? 0 : (apex == q.y ? 1 : (apex == q.z ? 2 : 3));
        w.project(q, inc, p, X);
        w.exits(p, ex);
        const int4 nb = w.nbr[cur];
        for (int i = 0; i < 3; ++i) {
            if (!ex[i]) continue;
            const int ef = kTet4Faces[inc][i];
            const int32_t next = tv_of(nb, ef);
            if (!dynamic && next == w.target) return 1;
            if (sp >= cap) return -1;
            stack[sp++] = (cur << 2) | ef;
            if (dynamic && next == w.target) return 1;
            const bool check = dynamic ? (!(n % kPassThroughSteps) || n == 2) : !(n % kPassThroughSteps);
            if (check && w.max_dis > 0.f && w.passed(p, X, i)) return 0;
        }
        ++n;
    }
    return 0;  // empty stack
}

// Orthonormal basis of the plane normal to unit n (CuMatrix::buildOrthonormalBasis, whose
// source is not in the reference tree): Duff et al., "Building an Orthonormal Basis,
// Revisited", JCGT 6(1), 2017.
__device__ __forceinline__ void ortho_basis(float3 n, float3& b1, float3& b2) {
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float b = n.x * n.y * a;
    b1 = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    b2 = v3(b, sign + n.y * n.y * a, -n.y);
}

// The traversal check for surface face g with closest point cp (type 6 = interior) of
// the query point moved toward the containing tet (target_pt).
__device__ __noinline__ bool traverse_ok(const Dev& D, const float4* P, const TraverseCfg& c, int32_t g, int type,
                                         float3 cp, float3 target_pt, int32_t target_tet) {
    const int2 ft = D.face_tet[g];
    if (ft.x == target_tet) return true;
    const int4 fv = D.faces[g];
    float3 o = cp;
    if (type != 6) {
        const float3 sum = add(add(ld3(P, fv.x), ld3(P, fv.y)), ld3(P, fv.z));
        const float3 a = mul(1.f - c.shift, cp), b = mul(c.shift / 3.0f, sum);
        o = add(a, b);
    }
    const float3 ray = sub(target_pt, o);
    const float len = sqrtf(dot(ray, ray));
    Walk w;
    w.P = P;
    w.tets = D.tets;
    w.nbr = D.tet_nbr;
    w.o = o;
    ortho_basis(v3(ray.x / len, ray.y / len, ray.z / len), w.ax0, w.ax1);
    w.max_dis = c.stop_after ? c.max_mult * len : -1.f;
    w.eps = c.eps;
    w.target = target_tet;
    int32_t stack[kDynamicStack];
    int r = c.use_static ? walk(w, ft.x, ft.y, false, stack) : -1;
    if (r < 0) r = walk(w, ft.x, ft.y, true, stack);  // the static stack overflowed
    if (r < 0) atomicAdd(&D.counters[cloth::CC_TRUNCATIONS], 1ull);  // the walk gave up on a bound
    return r == 1;
}

__device__ __forceinline__ float box_dist2(float3 p, float4 lo, float4 hi) {
    const float dx = fmaxf(fmaxf(lo.x - p.x, 0.f), p.x - hi.x);
    const float dy = fmaxf(fmaxf(lo.y - p.y, 0.f), p.y - hi.y);
    const float dz = fmaxf(fmaxf(lo.z - p.z, 0.f), p.z - hi.z);
    return dx * dx + dy * dy + dz * dz;
}
__device__ __forceinline__ bool box_overlap(float3 lo, float3 hi, float4 blo, float4 bhi) {
    return !(hi.x < blo.x || lo.x > bhi.x || hi.y < blo.y || lo.y > bhi.y || hi.z < blo.z || lo.z > bhi.z);
}

// ---- kernels ---------------------------------------------------------------------

// Whether any tet has |6 V| >= CMP_EPSILON at positions P (else no point-in-tet test
// can succeed and DCD finds nothing).
__global__ void k_tet_volume_flag(Dev D, const int4* tets, int32_t ntet, const float4* P, int* flag) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    bool big = false;
    if (t < ntet) {
        const int4 q = tets[t];
        big = fabsf(tet_vol6(ld3(P, q.x), ld3(P, q.y), ld3(P, q.z), ld3(P, q.w))) >= kCmpEps;
    }
    if (__syncthreads_or(big) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void k_clear_hits(Dev D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < D.nsv) D.hit[i] = -1;
}

// DCD of one surface vertex per thread.
template <bool INTERMEDIATE>
__global__ void k_dcd(Dev D, bvh::LbvhDev tb, bvh::LbvhDev fb, const float4* xf, const int* vol_flag, int ccd_on,
                      int handle_self, int check_feasible, float eps, float off, TraverseCfg tc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.nsv) return;
    const int2 q = D.sv[i];
    const int slot = q.x, m = q.y;
    const float4* P = INTERMEDIATE ? xf : xf + D.nslots;
    bool query;
    if (INTERMEDIATE) {
        query = D.pen[i] || !ccd_on;
    } else {
        query = xf[D.nslots + slot].y < off;
        D.pen[i] = 0;
    }
    if (!query) return;
    D.hit[i] = -1;
    if (!*vol_flag) return;
    const float3 p = ld3(P, slot);
    // vertexCollisionDetection: the lowest (mesh, tet) that strictly contains p
    int32_t best_t = 0x7fffffff;
    bvh::traverse(tb, p, 0.f, D.counters, [&](int t) {
        if (t >= best_t) return;
        const int tm = D.tet_mesh[t];
        if (!handle_self && tm == m) return;
        const int4 tv = D.tets[t];
        if (tm == m && (tv.x == slot || tv.y == slot || tv.z == slot || tv.w == slot)) return;
        if (point_in_tet(p, ld3(P, tv.x), ld3(P, tv.y), ld3(P, tv.z), ld3(P, tv.w))) best_t = t;
    });
    if (best_t == 0x7fffffff) return;
    if (!INTERMEDIATE) D.pen[i] = 1;
    const int im = D.tet_mesh[best_t];
    // closestPointQuery: nearest feasible surface face of mesh im from which the
    // tetrahedral traversal reaches best_t, ties to the lower face
    const bool traverse = tc.check && (im == m || tc.non_self);
    float3 target = p;
    if (traverse && tc.shift_center) {
        const int4 tv = D.tets[best_t];
        const float3 cen = mul(0.25f, add(add(add(ld3(P, tv.x), ld3(P, tv.y)), ld3(P, tv.z)), ld3(P, tv.w)));
        target = add(mul(1.f - tc.shift, p), mul(tc.shift, cen));
    }
    float best = __int_as_float(0x7f800000);
    int32_t bestg = -1;
    int stack[kStack];
    int sp = 0;
    if (fb.n > 0) stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        if (box_dist2(p, fb.bmin[node], fb.bmax[node]) > best * best * 1.0001f) continue;
        if (node >= fb.n - 1) {
            const int g = int(fb.keys[node - (fb.n - 1)] & 0xffffffffull);
            const int4 fv = D.faces[g];
            if (fv.w != im) continue;
            float3 bary, cp;
            const int type = closest_point_triangle<float3, float>(p, ld3(P, fv.x), ld3(P, fv.y), ld3(P, fv.z), bary, cp);
            if (im == m && type <= cloth::AtC && (type == 0 ? fv.x : (type == 1 ? fv.y : fv.z)) == slot) continue;
            const float3 dd = sub(p, cp);
            const float d = sqrtf(dot(dd, dd));
            if (!(d < best || (d == best && g < bestg))) continue;
            if (check_feasible && !feasible(D, P, p, g, type, eps)) continue;
            if (traverse && !traverse_ok(D, P, tc, g, type, cp, target, best_t)) continue;
            best = d;
            bestg = g;
        } else {
            if (sp + 2 > kStack) {
                atomicAdd(&D.counters[cloth::CC_STACK_OVERFLOW], 1ull);
                continue;
            }
            const int2 c = fb.child[node];
            stack[sp++] = c.y;
            stack[sp++] = c.x;
        }
    }
    D.hit[i] = bestg;
    D.hit_tt[i] = -1.f;
}

// CCD of one surface vertex per thread: the first face its trajectory crosses.
__global__ void k_ccd(Dev D, bvh::LbvhDev fb, const float4* xf, float off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.nsv) return;
    const int slot = D.sv[i].x;
    const float3 p1 = ld3(xf, slot);
    if (!(p1.y < off) || D.pen[i]) return;
    const float3 p0 = ld3(xf, D.nslots + slot);
    const float dx = p1.x - p0.x, dy = p1.y - p0.y, dz = p1.z - p0.z;
    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
    const float3 lo = v3(fminf(p0.x, p1.x), fminf(p0.y, p1.y), fminf(p0.z, p1.z));
    const float3 hi = v3(fmaxf(p0.x, p1.x), fmaxf(p0.y, p1.y), fmaxf(p0.z, p1.z));
    float bestd = 0.f, besttt = 0.f;
    int32_t bestg = -1;
    int stack[kStack];
    int sp = 0;
    if (fb.n > 0) stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        if (!box_overlap(lo, hi, fb.bmin[node], fb.bmax[node])) continue;
        if (node >= fb.n - 1) {
            const int g = int(fb.keys[node - (fb.n - 1)] & 0xffffffffull);
            const int4 fv = D.faces[g];
            if (fv.x == slot || fv.y == slot || fv.z == slot) continue;
            const float3 a[3] = {ld3(xf, D.nslots + fv.x), ld3(xf, D.nslots + fv.y), ld3(xf, D.nslots + fv.z)};
            const float3 b[3] = {ld3(xf, fv.x), ld3(xf, fv.y), ld3(xf, fv.z)};
            float tt;
            if (!ccd_tri_point(a, b, p0, p1, tt)) continue;
            const float depth = tt * len;
            if (bestg < 0 || depth < bestd || (depth == bestd && g < bestg)) {
                bestd = depth;
                besttt = tt;
                bestg = g;
            }
        } else {
            if (sp + 2 > kStack) {
                atomicAdd(&D.counters[cloth::CC_STACK_OVERFLOW], 1ull);
                continue;
            }
            const int2 c = fb.child[node];
            stack[sp++] = c.y;
            stack[sp++] = c.x;
        }
    }
    D.hit[i] = bestg;
    D.hit_tt[i] = besttt;
}

// Own contacts and relation keys (face vertex slot, surface vertex, order).
__global__ void k_own(Dev D, uint8_t* info, int4* own, unsigned long long* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) atomicAdd(&D.counters[cloth::CC_DETECTIONS], 1ull);  // one per detection pass
    if (i >= D.nsv) return;
    const int g = D.hit[i];
    if (g < 0) {
        keys[3 * size_t(i)] = keys[3 * size_t(i) + 1] = keys[3 * size_t(i) + 2] = ~0ull;
        return;
    }
    const int slot = D.sv[i].x;
    const int4 fv = D.faces[g];
    own[slot] = fv;
    info[slot] = 8;
    const int f[3] = {fv.x, fv.y, fv.z};
#pragma unroll
    for (int j = 0; j < 3; ++j)
        keys[3 * size_t(i) + j] = (static_cast<unsigned long long>(f[j]) << 32) | (static_cast<unsigned>(i) << 2) | j;
}

// The first four relations of each face vertex in (surface vertex) order.
__global__ void k_rel(Dev D, const unsigned long long* keys, int32_t n, uint8_t* info, int32_t* rel) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const unsigned long long k = keys[e];
    if (k == ~0ull) return;
    const int s = int(k >> 32);
    int rank = 0;
    while (rank < 4 && e - rank - 1 >= 0 && int(keys[e - rank - 1] >> 32) == s) ++rank;
    if (rank >= 4) return;
    const int i = int((k & 0xffffffffull) >> 2);
    const int order = int(k & 3ull);
    rel[4 * size_t(s) + rank] = (D.sv[i].x << 2) | order;
    const bool last = e + 1 == n || int(keys[e + 1] >> 32) != s;
    if (rank == 3 || last) info[s] = uint8_t(info[s] | (rank + 1));
}

}  // namespace

struct Detector::Impl {
    Dev D{};
    int4* faces = nullptr;
    int4* face_nbr = nullptr;
    int2* sv = nullptr;
    int32_t *ring_ofs = nullptr, *ring = nullptr, *tet_mesh = nullptr;
    int4* tets = nullptr;
    int4* tet_nbr = nullptr;
    int2* face_tet = nullptr;
    int32_t* hit = nullptr;
    float* hit_tt = nullptr;
    uint8_t* pen = nullptr;
    uint8_t* info = nullptr;
    int4* own = nullptr;
    int32_t* rel = nullptr;
    int32_t* list = nullptr;
    int32_t* nlist = nullptr;
    int* vol_flag = nullptr;
    unsigned long long *keys = nullptr, *keys_sorted = nullptr, *counters = nullptr;
    void* sort_tmp = nullptr;
    size_t sort_tmp_bytes = 0;
    void* select_tmp = nullptr;
    size_t select_tmp_bytes = 0;
    bvh::Lbvh face_bvh, tet_bvh;
};

Detector::~Detector() { release(); }

void Detector::release() {
    if (!d_) return;
    d_->face_bvh.release();
    d_->tet_bvh.release();
    for (void* p : {(void*)d_->faces, (void*)d_->face_nbr, (void*)d_->sv, (void*)d_->ring_ofs, (void*)d_->ring,
                    (void*)d_->tet_mesh, (void*)d_->tets, (void*)d_->tet_nbr, (void*)d_->face_tet, (void*)d_->hit, (void*)d_->hit_tt, (void*)d_->pen,
                    (void*)d_->info, (void*)d_->own, (void*)d_->rel, (void*)d_->list, (void*)d_->nlist,
                    (void*)d_->vol_flag, (void*)d_->keys, (void*)d_->keys_sorted, (void*)d_->counters, d_->sort_tmp,
                    d_->select_tmp})
        if (p) cudaFree(p);
    delete d_;
    d_ = nullptr;
}

template <typename T>
static T* upload(const std::vector<T>& h, size_t& bytes) {
    T* p = dalloc<T>(h.size(), bytes);
    if (!h.empty()) TCD_CUDA(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

void Detector::init(const Topo& t, const Params& prm, size_t& bytes) {
    release();
    prm_ = prm;
    d_ = new Impl;
    nslots_ = t.nslots;
    nf_ = int32_t(t.faces.size());
    nsv_ = int32_t(t.verts.size());
    ntet_ = int32_t(t.tets.size());
    if (!enabled()) return;
    Impl& I = *d_;
    I.faces = upload(t.faces, bytes);
    I.face_nbr = upload(t.face_nbr, bytes);
    I.sv = upload(t.verts, bytes);
    I.ring_ofs = upload(t.ring_ofs, bytes);
    I.ring = upload(t.ring, bytes);
    I.tets = upload(t.tets, bytes);
    I.tet_mesh = upload(t.tet_mesh, bytes);
    I.tet_nbr = upload(t.tet_nbr, bytes);
    I.face_tet = upload(t.face_tet, bytes);
    I.hit = dalloc<int32_t>(nsv_, bytes);
    I.hit_tt = dalloc<float>(nsv_, bytes);
    I.pen = dalloc<uint8_t>(nsv_, bytes);
    I.info = dalloc<uint8_t>(nslots_, bytes);
    I.own = dalloc<int4>(nslots_, bytes);
    I.rel = dalloc<int32_t>(4 * size_t(nslots_), bytes);
    I.list = dalloc<int32_t>(nslots_, bytes);
    I.nlist = dalloc<int32_t>(1, bytes);
    I.vol_flag = dalloc<int>(1, bytes);
    I.keys = dalloc<unsigned long long>(3 * size_t(nsv_), bytes);
    I.keys_sorted = dalloc<unsigned long long>(3 * size_t(nsv_), bytes);
    I.counters = dalloc<unsigned long long>(cloth::CC_N, bytes);
    TCD_CUDA(cudaMemset(I.hit, 0xff, sizeof(int32_t) * std::max(nsv_, 1)));
    TCD_CUDA(cudaMemset(I.pen, 0, std::max(nsv_, 1)));
    TCD_CUDA(cudaMemset(I.info, 0, std::max(nslots_, 1)));
    TCD_CUDA(cudaMemset(I.nlist, 0, sizeof(int32_t)));
    TCD_CUDA(cudaMemset(I.counters, 0, sizeof(unsigned long long) * cloth::CC_N));
    TCD_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, I.sort_tmp_bytes, I.keys, I.keys_sorted, 3 * nsv_));
    I.sort_tmp = dalloc<char>(I.sort_tmp_bytes, bytes);
    TCD_CUDA(cub::DeviceSelect::Flagged(nullptr, I.select_tmp_bytes, thrust::counting_iterator<int32_t>(0), I.info,
                                        I.list, I.nlist, nslots_));
    I.select_tmp = dalloc<char>(I.select_tmp_bytes, bytes);
    I.face_bvh.alloc(nf_, bvh::Prims{I.faces, 3, nslots_}, bytes);
    if (prm.dcd) I.tet_bvh.alloc(ntet_, bvh::Prims{I.tets, 4, 0}, bytes);
    Dev& D = I.D;
    D.nslots = nslots_;
    D.nsv = nsv_;
    D.nf = nf_;
    D.faces = I.faces;
    D.face_nbr = I.face_nbr;
    D.sv = I.sv;
    D.ring_ofs = I.ring_ofs;
    D.ring = I.ring;
    D.tets = I.tets;
    D.tet_mesh = I.tet_mesh;
    D.tet_nbr = I.tet_nbr;
    D.face_tet = I.face_tet;
    D.hit = I.hit;
    D.hit_tt = I.hit_tt;
    D.pen = I.pen;
    D.counters = I.counters;
}

void Detector::enqueue(const float4* xf, bool intermediate, bool rebuild, cudaStream_t st) {
    if (!enabled() || nsv_ == 0) return;
    Impl& I = *d_;
    const Dev& D = I.D;
    // the face hierarchy covers each face at both positions (current, substep start)
    if (nf_ > 0) {
        if (rebuild) I.face_bvh.build(xf, st);
        else I.face_bvh.refit(xf, nullptr, st);
    }
    if (prm_.dcd) {
        const float4* P = intermediate ? xf : xf + nslots_;
        TCD_CUDA(cudaMemsetAsync(I.vol_flag, 0, sizeof(int), st));
        if (ntet_ > 0) k_tet_volume_flag<<<blocks(ntet_, 256), 256, 0, st>>>(D, I.tets, ntet_, P, I.vol_flag);
        if (ntet_ > 0) I.tet_bvh.refit(P, I.vol_flag, st);
        if (intermediate)
            k_dcd<true><<<blocks(nsv_, 128), 128, 0, st>>>(D, I.tet_bvh.dev(), I.face_bvh.dev(), xf, I.vol_flag, prm_.ccd,
                                                           prm_.handle_self, prm_.check_feasible, prm_.feasible_eps,
                                                           prm_.off_height, traverse_cfg(prm_));
        else
            k_dcd<false><<<blocks(nsv_, 128), 128, 0, st>>>(D, I.tet_bvh.dev(), I.face_bvh.dev(), xf, I.vol_flag, prm_.ccd,
                                                            prm_.handle_self, prm_.check_feasible, prm_.feasible_eps,
                                                            prm_.off_height, traverse_cfg(prm_));
    } else if (!intermediate) {
        k_clear_hits<<<blocks(nsv_, 256), 256, 0, st>>>(D);
    }
    if (prm_.ccd) k_ccd<<<blocks(nsv_, 128), 128, 0, st>>>(D, I.face_bvh.dev(), xf, prm_.off_height);
    // records, and the ascending list of slots that have any
    TCD_CUDA(cudaMemsetAsync(I.info, 0, size_t(nslots_), st));
    k_own<<<blocks(nsv_, 256), 256, 0, st>>>(D, I.info, I.own, I.keys);
    size_t tb = I.sort_tmp_bytes;
    TCD_CUDA(cub::DeviceRadixSort::SortKeys(I.sort_tmp, tb, I.keys, I.keys_sorted, 3 * nsv_, 0, 64, st));
    k_rel<<<blocks(3 * int64_t(nsv_), 256), 256, 0, st>>>(D, I.keys_sorted, 3 * nsv_, I.info, I.rel);
    size_t sb = I.select_tmp_bytes;
    TCD_CUDA(cub::DeviceSelect::Flagged(I.select_tmp, sb, thrust::counting_iterator<int32_t>(0), I.info, I.list,
                                        I.nlist, nslots_, st));
    TCD_CUDA(cudaGetLastError());
}

void Detector::build(const float4* xf, cudaStream_t st) {
    if (!enabled() || nsv_ == 0) return;
    if (nf_ > 0) d_->face_bvh.build(xf, st);
    if (prm_.dcd && ntet_ > 0) d_->tet_bvh.build(xf + nslots_, st);
    TCD_CUDA(cudaGetLastError());
}

void Detector::reset(cudaStream_t st) {
    if (!enabled() || !d_) return;
    Impl& I = *d_;
    TCD_CUDA(cudaMemsetAsync(I.hit, 0xff, sizeof(int32_t) * std::max(nsv_, 1), st));
    TCD_CUDA(cudaMemsetAsync(I.pen, 0, std::max(nsv_, 1), st));
    TCD_CUDA(cudaMemsetAsync(I.info, 0, std::max(nslots_, 1), st));
    TCD_CUDA(cudaMemsetAsync(I.nlist, 0, sizeof(int32_t), st));
}

Records Detector::records() const {
    Records r;
    if (!d_ || !enabled()) return r;
    r.info = d_->info;
    r.own = d_->own;
    r.rel = d_->rel;
    r.list = d_->list;
    r.nlist = d_->nlist;
    return r;
}

void Detector::contacts(std::vector<int32_t>& rows, cudaStream_t st) const {
    rows.clear();
    if (!d_ || !enabled() || nsv_ == 0) return;
    std::vector<int32_t> hit(nsv_);
    std::vector<float> tt(nsv_);
    std::vector<int2> sv(nsv_);
    TCD_CUDA(cudaMemcpyAsync(hit.data(), d_->hit, sizeof(int32_t) * nsv_, cudaMemcpyDeviceToHost, st));
    TCD_CUDA(cudaMemcpyAsync(tt.data(), d_->hit_tt, sizeof(float) * nsv_, cudaMemcpyDeviceToHost, st));
    TCD_CUDA(cudaMemcpyAsync(sv.data(), d_->sv, sizeof(int2) * nsv_, cudaMemcpyDeviceToHost, st));
    TCD_CUDA(cudaStreamSynchronize(st));
    for (int32_t i = 0; i < nsv_; ++i)
        if (hit[i] >= 0) {
            rows.push_back(sv[i].x);
            rows.push_back(hit[i]);
            rows.push_back(tt[i] < 0.f ? 2 : 1);
        }
}

void Detector::counters(unsigned long long* out, cudaStream_t st) const {
    for (int i = 0; i < cloth::CC_N; ++i) out[i] = 0;
    if (!d_ || !enabled()) return;
    TCD_CUDA(cudaMemcpyAsync(out, d_->counters, sizeof(unsigned long long) * cloth::CC_N, cudaMemcpyDeviceToHost, st));
    TCD_CUDA(cudaStreamSynchronize(st));
}

}  // namespace tetcd
}  // namespace gaia
