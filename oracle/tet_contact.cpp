// Tet-mesh contact for the CPU oracle — TEST INFRASTRUCTURE ONLY (see tet_contact.h).
//
// Paths are relative to the reference project's Simulator/Modules directory unless
// they start with Simulator/. Compiled with -ffp-contract=off: every FP32 operation
// of the CCD test rounds on its own, as in the reference's SSE build.
//
// The cubic root finder of the CCD test restates the one in Cem Yuksel's cyCodeBase
// (cyPolynomial.h; "High-Performance Polynomial Root Finding for Graphics", HPG 2022),
// which is MIT-licensed: Copyright (c) 2022, Cem Yuksel <cem@cemyuksel.com>; the
// permission notice and warranty disclaimer are reproduced in the header of the GPU
// detector, gaia_gb300/csrc/tet_cd.cu.
#include "tet_contact.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <unordered_map>

namespace oracle_tc {

void build_surface_topology(int nv, Surface& s);

// ---------------------------------------------------------------------------
// Surface extraction
// ---------------------------------------------------------------------------
Surface extract_surface(int nv, int ntet, const int32_t* tets, const double* X) {
    static const int kFace[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
    std::map<std::array<int32_t, 3>, std::vector<int32_t>> owners;  // sorted face -> 4 * tet + k
    for (int t = 0; t < ntet; ++t)
        for (int k = 0; k < 4; ++k) {
            std::array<int32_t, 3> key = {tets[4 * t + kFace[k][0]], tets[4 * t + kFace[k][1]],
                                          tets[4 * t + kFace[k][2]]};
            std::sort(key.begin(), key.end());
            owners[key].push_back(4 * t + k);
        }
    Surface s;
    // neighbour across each face: the other tet of a face shared by exactly two
    s.tet_nbr.assign(4 * size_t(ntet), -1);
    for (const auto& kv : owners)
        if (kv.second.size() == 2) {
            s.tet_nbr[size_t(kv.second[0])] = kv.second[1] / 4;
            s.tet_nbr[size_t(kv.second[1])] = kv.second[0] / 4;
        }
    std::vector<char> on(size_t(nv), 0);
    for (int t = 0; t < ntet; ++t) {
        const int32_t* v = tets + 4 * t;
        double e[3][3];
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) e[i][d] = X[3 * size_t(v[i + 1]) + d] - X[3 * size_t(v[0]) + d];
        const double vol = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                           e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
        for (int k = 0; k < 4; ++k) {
            std::array<int32_t, 3> f = {v[kFace[k][0]], v[kFace[k][1]], v[kFace[k][2]]};
            std::array<int32_t, 3> key = f;
            std::sort(key.begin(), key.end());
            if (owners[key].size() != 1) continue;
            if (vol < 0) std::swap(f[1], f[2]);
            s.face_tet.push_back(t);
            s.face_tet.push_back(k);
            for (int i = 0; i < 3; ++i) {
                s.faces.push_back(f[i]);
                on[size_t(f[i])] = 1;
            }
        }
    }
    for (int i = 0; i < nv; ++i)
        if (on[size_t(i)]) s.verts.push_back(i);
    build_surface_topology(nv, s);
    return s;
}

// ---------------------------------------------------------------------------
// FP32 CCD (moving point vs moving triangle)
// ---------------------------------------------------------------------------
namespace {

struct F3 {
    float x, y, z;
};
struct F2 {
    float x, y;
};

inline F3 sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 add(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 scale(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 cross(F3 a, F3 b) { return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// 2D cross product as (-a.y, a.x) . b (cyVector.h Vec2::Cross)
inline float cross2(F2 a, F2 b) { return -a.y * b.x + a.x * b.y; }
// a + (b - a) * t, per component
inline F3 lerp(F3 a, F3 b, float t) { return add(a, scale(sub(b, a), t)); }

inline float fmin_ref(float a, float b) { return a <= b ? a : b; }  // cyCore.h Min
inline float fmax_ref(float a, float b) { return a >= b ? a : b; }  // cyCore.h Max
inline bool diff_sign(float a, float b) { return (a < 0) != (b < 0); }
inline float mult_sign(float v, float s) { return v * (s < 0 ? -1.0f : 1.0f); }

// Horner evaluation, highest coefficient first (cyPolynomial.h PolynomialEval).
inline float eval3(const float c[4], float x) {
    float r = c[3];
    r = r * x + c[2];
    r = r * x + c[1];
    return r * x + c[0];
}
inline float eval2(const float c[3], float x) {
    float r = c[2];
    r = r * x + c[1];
    return r * x + c[0];
}

// Real roots of c0 + c1 x + c2 x^2 within [x0, x1], ascending.
int quadratic_roots(float roots[2], const float c[3], float x0, float x1) {
    const float cc = c[0], b = c[1], a = c[2];
    const float delta = b * b - 4 * a * cc;
    if (delta > 0) {
        const float d = std::sqrt(delta);
        const float q = -0.5f * (b + mult_sign(d, b));
        const float rv0 = q / a, rv1 = cc / q;
        const float r0 = fmin_ref(rv0, rv1), r1 = fmax_ref(rv0, rv1);
        const int r0i = (r0 >= x0) & (r0 <= x1);
        const int r1i = (r1 >= x0) & (r1 <= x1);
        roots[0] = r0;
        roots[r0i] = r1;
        return r0i + r1i;
    }
    if (delta < 0) return 0;
    const float r0 = -0.5f * b / a;
    roots[0] = r0;
    return (r0 >= x0) & (r0 <= x1);
}

constexpr float kRootError = 6e-4f;  // PolynomialDefaultError<float>
constexpr int kMaxBracketSteps = 256;

// The single root of a cubic in [x0, x1] with f(x0), f(x1) of different signs:
// up to 16 clamped Newton steps from the midpoint, then Newton steps safeguarded
// by bisection of the sign-change bracket (Yuksel, "High-Performance Polynomial
// Root Finding for Graphics", HPG 2022; RootFinderNewton::FindClosed without the
// error bound option).
float find_closed(const float coef[4], const float deriv[3], float x0, float x1, float y0, float xError) {
    const float ep2 = 2 * xError;
    float xr = (x0 + x1) / 2;
    if (x1 - x0 <= ep2) return xr;
    const float xr0 = xr;
    for (int k = 0; k < 16; ++k) {
        float xn = xr - eval3(coef, xr) / eval2(deriv, xr);
        xn = fmin_ref(x1, fmax_ref(x0, xn));
        if (std::fabs(xr - xn) <= xError) return xn;
        xr = xn;
    }
    if (!std::isfinite(xr)) xr = xr0;
    float yr = eval3(coef, xr);
    float xb0 = x0, xb1 = x1;
    for (int k = 0; k < kMaxBracketSteps; ++k) {
        const bool side = diff_sign(y0, yr);
        if (side) xb1 = xr;
        else xb0 = xr;
        const float dy = eval2(deriv, xr);
        const float xn = xr - yr / dy;
        if (xn > xb0 && xn < xb1) {
            const float step = std::fabs(xr - xn);
            xr = xn;
            if (step > xError) yr = eval3(coef, xr);
            else break;
        } else {
            xr = (xb0 + xb1) / 2;
            if (xr == xb0 || xr == xb1 || xb1 - xb0 <= ep2) break;
            yr = eval3(coef, xr);
        }
    }
    return xr;
}

// Roots of a cubic in [x0, x1] (cyPolynomial.h CubicRoots, boundError = false):
// the derivative's roots split [x0, x1] into monotonic pieces; the first piece with
// a sign change gives the first root, the rest come from the deflated quadratic.
int cubic_roots(float roots[3], const float coef[4], float x0, float x1) {
    const float xError = kRootError;
    const float y0 = eval3(coef, x0), y1 = eval3(coef, x1);
    const float a = coef[3] * 3, b_2 = coef[2], c = coef[1];
    const float deriv[3] = {c, 2 * b_2, a};
    const float delta_4 = b_2 * b_2 - a * c;
    auto deflate_rest = [&](float lo) {
        float def[3];
        def[2] = coef[3];
        def[1] = coef[2] + roots[0] * def[2];
        def[0] = coef[1] + roots[0] * def[1];
        return quadratic_roots(roots + 1, def, lo, x1) + 1;
    };
    if (delta_4 > 0) {
        const float d_2 = std::sqrt(delta_4);
        const float q = -(b_2 + mult_sign(d_2, b_2));
        const float rv0 = q / a, rv1 = c / q;
        const float xa = fmin_ref(rv0, rv1), xb = fmax_ref(rv0, rv1);
        if (diff_sign(y0, y1)) {
            if (xa >= x1 || xb <= x0 || (xa <= x0 && xb >= x1)) {
                roots[0] = find_closed(coef, deriv, x0, x1, y0, xError);
                return 1;
            }
        } else {
            if ((xa >= x1 || xb <= x0) || (xa <= x0 && xb >= x1)) return 0;
        }
        if (xa > x0) {
            const float ya = eval3(coef, xa);
            if (diff_sign(y0, ya)) {
                roots[0] = find_closed(coef, deriv, x0, xa, y0, xError);
                if (diff_sign(ya, y1) || (xb < x1 && diff_sign(ya, eval3(coef, xb)))) return deflate_rest(xa);
                return 1;
            }
            if (xb < x1) {
                const float yb = eval3(coef, xb);
                if (diff_sign(ya, yb)) {
                    roots[0] = find_closed(coef, deriv, xa, xb, ya, xError);
                    if (diff_sign(yb, y1)) return deflate_rest(xb);
                    return 1;
                }
                if (diff_sign(yb, y1)) {
                    roots[0] = find_closed(coef, deriv, xb, x1, yb, xError);
                    return 1;
                }
            } else if (diff_sign(ya, y1)) {
                roots[0] = find_closed(coef, deriv, xa, x1, ya, xError);
                return 1;
            }
        } else {
            const float yb = eval3(coef, xb);
            if (diff_sign(y0, yb)) {
                roots[0] = find_closed(coef, deriv, x0, xb, y0, xError);
                if (diff_sign(yb, y1)) return deflate_rest(xb);
                return 1;
            }
            if (diff_sign(yb, y1)) {
                roots[0] = find_closed(coef, deriv, xb, x1, yb, xError);
                return 1;
            }
        }
        return 0;
    }
    if (diff_sign(y0, y1)) {
        roots[0] = find_closed(coef, deriv, x0, x1, y0, xError);
        return 1;
    }
    return 0;
}

// Times in [0, 1] at which four linearly moving points are coplanar
// (CCDSolver.h:97-127): the cubic det[x1-x0, x2-x0, x3-x0](t).
int coplanar_times(float t[3], const F3 a[4], const F3 b[4]) {
    const F3 dx0 = sub(b[0], a[0]), dx1 = sub(b[1], a[1]), dx2 = sub(b[2], a[2]), dx3 = sub(b[3], a[3]);
    const F3 e1 = sub(a[1], a[0]), e2 = sub(a[2], a[0]), e3 = sub(a[3], a[0]);
    const F3 de0 = sub(dx3, dx0), de1 = sub(dx1, dx0), de2 = sub(dx2, dx0);
    const F3 e1xe2 = cross(e1, e2);
    const F3 de1xde2 = cross(de1, de2);
    const F3 mixed = add(cross(e1, de2), cross(de1, e2));
    float poly[4];
    poly[0] = dot(e3, e1xe2);
    poly[1] = dot(de0, e1xe2) + dot(e3, mixed);
    poly[2] = dot(e3, de1xde2) + dot(de0, mixed);
    poly[3] = dot(de0, de1xde2);
    return cubic_roots(t, poly, 0.0f, 1.0f);
}

// Index of the largest component (cyVector.h Vec3::MaxComp, same tie rule).
inline int max_comp(F3 v) {
    const int xy = v.x < v.y, xz = v.x < v.z, yz = v.y < v.z;
    return (xy | xz) + (xz & yz);
}

inline F2 drop_axis(F3 v, int axis) {
    if (axis == 0) return F2{v.y, v.z};
    if (axis == 1) return F2{v.x, v.z};
    return F2{v.x, v.y};
}

}  // namespace

// CCDSolver.h:155-196 (IntersectContinuousTriPoint): for each coplanarity time, project
// the four interpolated points on the plane that drops the triangle normal's largest
// axis and test whether the point lies inside the triangle (equal signs of the three
// 2D cross products, sign bits as std::signbit reads them).
int ccd_tri_point(const float x0[9], const float x1[9], const float p0[3], const float p1[3], float* tt,
                  float bary[3]) {
    const F3 a[4] = {{x0[0], x0[1], x0[2]}, {x0[3], x0[4], x0[5]}, {x0[6], x0[7], x0[8]}, {p0[0], p0[1], p0[2]}};
    const F3 b[4] = {{x1[0], x1[1], x1[2]}, {x1[3], x1[4], x1[5]}, {x1[6], x1[7], x1[8]}, {p1[0], p1[1], p1[2]}};
    float t[3];
    const int nt = coplanar_times(t, a, b);
    for (int i = 0; i < nt; ++i) {
        const F3 q0 = lerp(a[0], b[0], t[i]), q1 = lerp(a[1], b[1], t[i]);
        const F3 q2 = lerp(a[2], b[2], t[i]), q3 = lerp(a[3], b[3], t[i]);
        const F3 n = cross(sub(q1, q0), sub(q2, q0));
        const int axis = max_comp(F3{std::fabs(n.x), std::fabs(n.y), std::fabs(n.z)});
        const F2 w3 = drop_axis(q3, axis);
        F2 w0 = drop_axis(q0, axis), w1 = drop_axis(q1, axis), w2 = drop_axis(q2, axis);
        w0 = F2{w0.x - w3.x, w0.y - w3.y};
        w1 = F2{w1.x - w3.x, w1.y - w3.y};
        w2 = F2{w2.x - w3.x, w2.y - w3.y};
        const bool s01 = std::signbit(cross2(w0, w1));
        const bool s12 = std::signbit(cross2(w1, w2));
        const bool s20 = std::signbit(cross2(w2, w0));
        if (s01 == s12 && s01 == s20) {
            const float tc = t[i];
            *tt = tc;
            // CCDSolver.h:140-152 (Barycentric) at the time of impact
            const F3 p = lerp(a[3], b[3], tc);
            const F3 A = lerp(a[0], b[0], tc), B = lerp(a[1], b[1], tc), C = lerp(a[2], b[2], tc);
            const F3 v0 = sub(B, A), v1 = sub(C, A), v2 = sub(p, A);
            const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
            const float d20 = dot(v2, v0), d21 = dot(v2, v1);
            const float denom = d00 * d11 - d01 * d01;
            bary[1] = (d11 * d20 - d01 * d21) / denom;
            bary[2] = (d00 * d21 - d01 * d20) / denom;
            bary[0] = 1.0f - bary[1] - bary[2];
            return 1;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Broad phase: a uniform hash grid of boxes. Every query below re-tests candidates
// exactly, so the grid only has to be conservative.
// ---------------------------------------------------------------------------
namespace {

struct Box {
    float lo[3], hi[3];
};

class HashGrid {
public:
    void build(const std::vector<Box>& boxes) {
        cells_.clear();
        big_.clear();
        double ext = 0;
        for (const Box& b : boxes)
            ext += double(b.hi[0] - b.lo[0]) + double(b.hi[1] - b.lo[1]) + double(b.hi[2] - b.lo[2]);
        h_ = boxes.empty() ? 1.0 : std::max(1e-6, 1.5 * ext / (3.0 * double(boxes.size())));
        for (size_t i = 0; i < boxes.size(); ++i) {
            int64_t r[6];
            range(boxes[i], r);
            if ((r[1] - r[0] + 1) * (r[3] - r[2] + 1) * (r[5] - r[4] + 1) > 4096) {
                big_.push_back(int32_t(i));
                continue;
            }
            for (int64_t a = r[0]; a <= r[1]; ++a)
                for (int64_t b = r[2]; b <= r[3]; ++b)
                    for (int64_t c = r[4]; c <= r[5]; ++c) cells_[key(a, b, c)].push_back(int32_t(i));
        }
        stamp_.assign(boxes.size(), -1);
    }
    // Ascending ids of the boxes in cells that the query box touches.
    std::vector<int32_t> query(const Box& q) {
        std::vector<int32_t> out;
        ++gen_;
        auto take = [&](int32_t i) {
            if (stamp_[size_t(i)] != gen_) {
                stamp_[size_t(i)] = gen_;
                out.push_back(i);
            }
        };
        for (int32_t i : big_) take(i);
        int64_t r[6];
        range(q, r);
        for (int64_t a = r[0]; a <= r[1]; ++a)
            for (int64_t b = r[2]; b <= r[3]; ++b)
                for (int64_t c = r[4]; c <= r[5]; ++c) {
                    auto it = cells_.find(key(a, b, c));
                    if (it != cells_.end())
                        for (int32_t i : it->second) take(i);
                }
        std::sort(out.begin(), out.end());
        return out;
    }

private:
    int64_t cell(float c) const { return int64_t(std::floor(double(c) / h_)); }
    void range(const Box& b, int64_t r[6]) const {
        for (int d = 0; d < 3; ++d) {
            r[2 * d] = cell(b.lo[d]);
            r[2 * d + 1] = cell(b.hi[d]);
        }
    }
    static uint64_t key(int64_t i, int64_t j, int64_t k) {
        return uint64_t(i * 73856093) ^ uint64_t(j * 19349663) ^ uint64_t(k * 83492791);
    }
    double h_ = 1.0;
    std::unordered_map<uint64_t, std::vector<int32_t>> cells_;
    std::vector<int32_t> big_;
    std::vector<int32_t> stamp_;
    int32_t gen_ = 0;
};

inline Box empty_box() {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = 3.4e38f;
        b.hi[d] = -3.4e38f;
    }
    return b;
}
inline void extend(Box& b, const float* p) {
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = std::min(b.lo[d], p[d]);
        b.hi[d] = std::max(b.hi[d], p[d]);
    }
}
inline F3 ld(const float* x, int32_t v) { return F3{x[3 * size_t(v)], x[3 * size_t(v) + 1], x[3 * size_t(v) + 2]}; }
inline F3 normalized(F3 v) {
    const float l = std::sqrt(dot(v, v));
    return F3{v.x / l, v.y / l, v.z / l};
}

// pointInTet (CollisionDetector/CollisionGeometry.h:56-82): tets with |6 V| below
// CMP_EPSILON = 1e-5 (Types/Types.h:20) never contain a point; otherwise p must be
// strictly inside all four face planes.
bool point_in_tet(F3 p, F3 a, F3 b, F3 c, F3 d) {
    const float vol = dot(sub(b, a), cross(sub(c, a), sub(d, a)));
    if (std::fabs(vol) < 1e-5f) return false;
    const F3 vs[4] = {a, b, c, d};
    static const int order[4][3] = {{1, 2, 3}, {2, 0, 3}, {0, 1, 3}, {1, 0, 2}};
    for (int i = 0; i < 4; ++i) {
        const F3 v1 = vs[order[i][0]], v2 = vs[order[i][1]], v3 = vs[order[i][2]];
        if (dot(sub(p, v1), cross(sub(v2, v1), sub(v3, v2))) * vol >= 0) return false;
    }
    return true;
}

// Closest point on triangle abc (CollisionDetector/CollisionGeometry.h:84-145); returns
// 0..2 at a vertex, 3 = AB, 4 = BC, 5 = AC, 6 = interior.
int closest_point(F3 p, F3 a, F3 b, F3 c, float bary[3], F3& cp) {
    const F3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) { bary[0] = 1; bary[1] = 0; bary[2] = 0; cp = a; return 0; }
    const F3 bp = sub(p, b);
    const float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) { bary[0] = 0; bary[1] = 1; bary[2] = 0; cp = b; return 1; }
    const F3 cpv = sub(p, c);
    const float d5 = dot(ab, cpv), d6 = dot(ac, cpv);
    if (d6 >= 0.f && d5 <= d6) { bary[0] = 0; bary[1] = 0; bary[2] = 1; cp = c; return 2; }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
        const float v = d1 / (d1 - d3);
        bary[0] = 1.f - v; bary[1] = v; bary[2] = 0;
        cp = add(a, scale(ab, v));
        return 3;
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
        const float v = d2 / (d2 - d6);
        bary[0] = 1.f - v; bary[1] = 0; bary[2] = v;
        cp = add(a, scale(ac, v));
        return 5;
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
        const float v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary[0] = 0; bary[1] = 1.f - v; bary[2] = v;
        cp = add(b, scale(sub(c, b), v));
        return 4;
    }
    const float denom = 1.f / (va + vb + vc);
    const float v = vb * denom, w = vc * denom;
    bary[0] = 1.f - v - w; bary[1] = v; bary[2] = w;
    cp = add(add(a, scale(ab, v)), scale(ac, w));
    return 6;
}

}  // namespace

// ---------------------------------------------------------------------------
// Tetrahedral traversal (TetMesh/TetMeshFEM.cpp:503-740 static, 908-1100 dynamic)
// ---------------------------------------------------------------------------
namespace {

// TetMeshFEM::tet4Faces: the face omitting local vertex k, in the order the walk
// projects it; posibleExit3Faces: the exit face across incoming-face vertex i, as
// indices into (incoming face vertices 0..2, apex 3).
const int kTet4Faces[4][3] = {{1, 2, 3}, {2, 0, 3}, {0, 1, 3}, {1, 0, 2}};
const int kExit3[3][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}};
constexpr int kStaticStack = 32;      // SIZE_CANDIDATE_FACE_STACK
constexpr int kLoopRing = 32;         // SIZE_TRAVERSED_CIRCULAR_ARRAY
constexpr int kPassThroughSteps = 5;  // TetMeshFEM::passThroughCheckSteps
// Bounds of the dynamic walk (unbounded in the reference); shared with the GPU.
constexpr int kDynamicStack = 1024;
constexpr int kMaxWalkSteps = 1 << 16;

// Orthonormal basis of the plane normal to unit n (CuMatrix::buildOrthonormalBasis;
// its source is not in the reference tree): Duff et al., "Building an Orthonormal
// Basis, Revisited", JCGT 6(1), 2017.
void ortho_basis(F3 n, F3& b1, F3& b2) {
    const float sign = std::copysign(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float b = n.x * n.y * a;
    b1 = F3{1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x};
    b2 = F3{b, sign + n.y * n.y * a, -n.y};
}

struct Walk {
    const float* X;
    const int32_t* tets;
    const int32_t* nbr;
    F3 o, ax0, ax1;
    float max_dis, eps;
    int32_t target;

    int32_t tv(int32_t t, int k) const { return tets[4 * size_t(t) + size_t(k)]; }
    F3 vert(int32_t t, int k) const { return ld(X, tv(t, k)); }
    // projectTo2DCoordinates: incoming face's vertices in tet4Faces order, then the apex
    void project(int32_t t, int inc, F2 p[4], F3 P[4]) const {
        for (int i = 0; i < 4; ++i) {
            P[i] = vert(t, i < 3 ? kTet4Faces[inc][i] : inc);
            const F3 d = sub(P[i], o);
            p[i] = F2{dot(ax0, d), dot(ax1, d)};
        }
    }
    // exitFaceSelection (TetMesh/TetMeshFEM.h:423-483): the faces whose 2D wedge at the
    // apex holds the ray (the origin), with the sign of the incoming triangle
    static void exits(const F2 p[4], float eps, bool out[3]) {
        const F2 v1{p[1].x - p[0].x, p[1].y - p[0].y}, v2{p[2].x - p[0].x, p[2].y - p[0].y};
        const float area = v1.x * v2.y - v1.y * v2.x;
        const float sg = std::copysign(1.0f, area);
        const float d0 = p[3].x * p[0].y - p[3].y * p[0].x;
        const float d1 = p[3].x * p[1].y - p[3].y * p[1].x;
        const float d2 = p[3].x * p[2].y - p[3].y * p[2].x;
        out[0] = d1 * sg >= -eps && d2 * sg <= eps;
        out[1] = d2 * sg >= -eps && d0 * sg <= eps;
        out[2] = d0 * sg >= -eps && d1 * sg <= eps;
    }
    // the ray's crossing of exit face i beyond max_dis from the origin
    // (originBarycentric2DTriangle, TetMesh/TetMeshFEM.h:625-633)
    bool passed(const F2 p[4], const F3 P[4], int i) const {
        const F2 a = p[kExit3[i][0]], b = p[kExit3[i][1]], c = p[kExit3[i][2]];
        const F2 v0{b.x - a.x, b.y - a.y}, v1{c.x - a.x, c.y - a.y}, v2{-a.x, -a.y};
        const float den = v0.x * v1.y - v1.x * v0.y;
        const float w1 = (v2.x * v1.y - v1.x * v2.y) / den;
        const float w2 = (v0.x * v2.y - v2.x * v0.y) / den;
        const float w0 = 1.0f - w1 - w2;
        const F3 A = P[kExit3[i][0]], B = P[kExit3[i][1]], C = P[kExit3[i][2]];
        const F3 x{(w0 * A.x + w1 * B.x) + w2 * C.x, (w0 * A.y + w1 * B.y) + w2 * C.y, (w0 * A.z + w1 * B.z) + w2 * C.z};
        const F3 d = sub(x, o);
        return dot(d, d) > max_dis * max_dis;
    }
};

// Last kLoopRing tets entered (CircularArray::hasBackward of the traversed set).
struct LoopRing {
    int32_t v[kLoopRing];
    int n = 0;
    bool has(int32_t t) const {
        const int m = n < kLoopRing ? n : kLoopRing;
        for (int i = 0; i < m; ++i)
            if (v[i] == t) return true;
        return false;
    }
    void push(int32_t t) { v[n++ % kLoopRing] = t; }
};

// result: 1 reached, 0 not reached, -1 gave up on a bound
int walk(const Walk& w, int32_t start, int start_face, bool dynamic) {
    const int cap = dynamic ? kDynamicStack : kStaticStack;
    std::vector<int32_t> sf(static_cast<size_t>(cap)), st(static_cast<size_t>(cap));
    int sp = 0;
    LoopRing ring;
    ring.push(start);
    F2 p[4];
    F3 P[4];
    bool ex[3];
    w.project(start, start_face, p, P);
    Walk::exits(p, w.eps, ex);
    for (int i = 0; i < 3; ++i)
        if (ex[i]) {
            sf[size_t(sp)] = kTet4Faces[start_face][i];
            st[size_t(sp++)] = start;
        }
    int n = 0;
    for (int steps = 0; sp > 0; ++steps) {
        if (steps >= kMaxWalkSteps) return -1;
        --sp;
        const int f = sf[size_t(sp)];
        const int32_t prev = st[size_t(sp)];
        const int32_t fv0 = w.tv(prev, kTet4Faces[f][0]), fv1 = w.tv(prev, kTet4Faces[f][1]),
                      fv2 = w.tv(prev, kTet4Faces[f][2]);
        const int32_t cur = w.nbr[4 * size_t(prev) + size_t(f)];
        if (cur == w.target) return 1;
        if (cur < 0) return 0;  // reached the boundary
        if (ring.has(cur)) continue;
        ring.push(cur);
        const int32_t apex = w.tv(cur, 0) ^ w.tv(cur, 1) ^ w.tv(cur, 2) ^ w.tv(cur, 3) ^ fv0 ^ fv1 ^ fv2;
        int inc = 3;
        for (int k = 0; k < 3; ++k)
            if (apex == w.tv(cur, k)) {
                inc = k;
                break;
            }
        w.project(cur, inc, p, P);
        Walk::exits(p, w.eps, ex);
        for (int i = 0; i < 3; ++i) {
            if (!ex[i]) continue;
            const int ef = kTet4Faces[inc][i];
            const int32_t next = w.nbr[4 * size_t(cur) + size_t(ef)];
            if (!dynamic && next == w.target) return 1;
            if (sp >= cap) return -1;
            sf[size_t(sp)] = ef;
            st[size_t(sp++)] = cur;
            if (dynamic && next == w.target) return 1;
            const bool check = dynamic ? (!(n % kPassThroughSteps) || n == 2) : !(n % kPassThroughSteps);
            if (check && w.max_dis > 0.f && w.passed(p, P, i)) return 0;
        }
        ++n;
    }
    return 0;  // empty stack
}

}  // namespace

bool tet_traverse(const float* X, const int32_t* tets, const Surface& s, const float origin[3], const float dir[3],
                  float max_dis, int32_t face, int32_t target, float ray_eps, bool use_static, int* status) {
    *status = 0;
    const int32_t start = s.face_tet[2 * size_t(face)];
    const int start_face = s.face_tet[2 * size_t(face) + 1];
    if (start == target) return true;
    Walk w;
    w.X = X;
    w.tets = tets;
    w.nbr = s.tet_nbr.data();
    w.o = F3{origin[0], origin[1], origin[2]};
    ortho_basis(F3{dir[0], dir[1], dir[2]}, w.ax0, w.ax1);
    w.max_dis = max_dis;
    w.eps = ray_eps;
    w.target = target;
    int r = use_static ? walk(w, start, start_face, false) : -1;
    if (r < 0) r = walk(w, start, start_face, true);  // the static stack overflowed
    if (r < 0) *status = 1;
    return r == 1;
}

// ---------------------------------------------------------------------------
// Surface topology for the feasible-region tests.
// ---------------------------------------------------------------------------
void build_surface_topology(int nv, Surface& s) {
    const size_t nf = s.faces.size() / 3;
    std::map<std::pair<int32_t, int32_t>, std::vector<int32_t>> edge_faces;
    for (size_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) {
            int32_t a = s.faces[3 * f + k], b = s.faces[3 * f + (k + 1) % 3];
            edge_faces[{std::min(a, b), std::max(a, b)}].push_back(int32_t(f));
        }
    s.face_nbr.assign(3 * nf, -1);
    std::vector<std::vector<int32_t>> ring(static_cast<size_t>(nv));
    for (size_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) {
            int32_t a = s.faces[3 * f + k], b = s.faces[3 * f + (k + 1) % 3];
            for (int32_t g : edge_faces[{std::min(a, b), std::max(a, b)}])
                if (g != int32_t(f)) {
                    s.face_nbr[3 * f + k] = g;
                    break;
                }
            ring[size_t(a)].push_back(b);
            ring[size_t(b)].push_back(a);
        }
    s.ring_ofs.assign(size_t(nv) + 1, 0);
    s.ring.clear();
    for (int v = 0; v < nv; ++v) {
        auto& r = ring[size_t(v)];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        s.ring.insert(s.ring.end(), r.begin(), r.end());
        s.ring_ofs[size_t(v) + 1] = int32_t(s.ring.size());
    }
}

// ---------------------------------------------------------------------------
// Detection
// ---------------------------------------------------------------------------
struct Detector::Impl {
    std::vector<CcdMesh> meshes;
    std::vector<int32_t> fofs, tofs;  // global face / tet offsets per mesh
    HashGrid swept, tets;
    bool use_prev_tets = false;

    std::pair<int, int32_t> face_of(int32_t g) const {
        const size_t m = size_t(std::upper_bound(fofs.begin(), fofs.end(), g) - fofs.begin()) - 1;
        return {int(m), g - fofs[m]};
    }
    std::pair<int, int32_t> tet_of(int32_t g) const {
        const size_t m = size_t(std::upper_bound(tofs.begin(), tofs.end(), g) - tofs.begin()) - 1;
        return {int(m), g - tofs[m]};
    }
};

Detector::Detector(const std::vector<CcdMesh>& meshes) : d_(new Impl) {
    d_->meshes = meshes;
    d_->fofs.assign(meshes.size() + 1, 0);
    d_->tofs.assign(meshes.size() + 1, 0);
    for (size_t m = 0; m < meshes.size(); ++m) {
        d_->fofs[m + 1] = d_->fofs[m] + int32_t(meshes[m].surf->faces.size() / 3);
        d_->tofs[m + 1] = d_->tofs[m] + meshes[m].ntet;
    }
}
Detector::~Detector() { delete d_; }

void Detector::build_swept() {
    std::vector<Box> boxes;
    boxes.reserve(size_t(d_->fofs.back()));
    for (const CcdMesh& M : d_->meshes) {
        const auto& F = M.surf->faces;
        for (size_t f = 0; f < F.size() / 3; ++f) {
            Box b = empty_box();
            for (int k = 0; k < 3; ++k) {
                extend(b, M.x + 3 * size_t(F[3 * f + k]));
                extend(b, M.xprev + 3 * size_t(F[3 * f + k]));
            }
            boxes.push_back(b);
        }
    }
    d_->swept.build(boxes);
}

void Detector::build_tets(bool prev) {
    std::vector<Box> boxes;
    boxes.reserve(size_t(d_->tofs.back()));
    for (const CcdMesh& M : d_->meshes) {
        const float* P = prev ? M.xprev : M.x;
        for (int t = 0; t < M.ntet; ++t) {
            Box b = empty_box();
            for (int k = 0; k < 4; ++k) extend(b, P + 3 * size_t(M.tets[4 * size_t(t) + k]));
            boxes.push_back(b);
        }
    }
    d_->tets.build(boxes);
    d_->use_prev_tets = prev;
}

CcdHit Detector::ccd(int m, int i) const {
    const CcdMesh& M = d_->meshes[size_t(m)];
    const int32_t v = M.surf->verts[size_t(i)];
    const float* p1 = M.x + 3 * size_t(v);
    const float* p0 = M.xprev + 3 * size_t(v);
    Box q = empty_box();
    extend(q, p0);
    extend(q, p1);
    CcdHit best;
    // the trajectory length as cyVector's Length: sqrt((x*x + y*y) + z*z)
    const float dx = p1[0] - p0[0], dy = p1[1] - p0[1], dz = p1[2] - p0[2];
    const float len = std::sqrt(dx * dx + dy * dy + dz * dz);
    for (int32_t g : d_->swept.query(q)) {
        const auto [fm, f] = d_->face_of(g);
        const CcdMesh& FM = d_->meshes[size_t(fm)];
        const int32_t* fv = &FM.surf->faces[3 * size_t(f)];
        if (fm == m && (fv[0] == v || fv[1] == v || fv[2] == v)) continue;
        float a0[9], a1[9];
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) {
                a0[3 * k + c] = FM.xprev[3 * size_t(fv[k]) + c];
                a1[3 * k + c] = FM.x[3 * size_t(fv[k]) + c];
            }
        float tt, bary[3];
        if (!ccd_tri_point(a0, a1, p0, p1, &tt, bary)) continue;
        const float depth = tt * len;
        if (best.face < 0 || depth < best.depth) {
            best.fmesh = fm;
            best.face = f;
            best.tt = tt;
            best.depth = depth;
            for (int k = 0; k < 3; ++k) best.bary[k] = bary[k];
        }
    }
    return best;
}

// checkEdgeFeasibleRegion / checkVertexFeasibleRegion (DiscreteCollisionDetector.cpp:
// 703-815), looking from inside the mesh (face normals negated).
static bool feasible(const CcdMesh& M, const float* P, F3 p, int32_t f, int type, float eps) {
    const int32_t* fv = &M.surf->faces[3 * size_t(f)];
    if (type == 6) return true;
    auto fnormal = [&](int32_t g) {
        const int32_t* gv = &M.surf->faces[3 * size_t(g)];
        const F3 a = ld(P, gv[0]), b = ld(P, gv[1]), c = ld(P, gv[2]);
        return normalized(cross(sub(b, a), sub(c, a)));
    };
    if (type >= 3) {
        // edge k: AB = 0, BC = 1, AC = 2 (from C to A)
        const int k = type == 3 ? 0 : (type == 4 ? 1 : 2);
        const int32_t e1 = k == 2 ? fv[2] : fv[k], e2 = k == 2 ? fv[0] : fv[k + 1];
        const int32_t nb = M.surf->face_nbr[3 * size_t(f) + size_t(k)];
        if (nb < 0) return true;
        const F3 n1 = scale(fnormal(f), -1.f), n2 = scale(fnormal(nb), -1.f);
        const F3 v1 = ld(P, e1), v2 = ld(P, e2);
        const F3 AP = sub(p, v1), BP = sub(p, v2), AB = sub(v2, v1), BA = scale(AB, -1.f);
        const float relaxed = -dot(AB, AB) * eps;
        if (dot(AP, AB) < relaxed) return false;
        if (dot(BP, BA) < relaxed) return false;
        if (dot(AP, cross(n1, AB)) < relaxed) return false;
        if (dot(AP, cross(n2, BA)) < relaxed) return false;
        return true;
    }
    const int32_t va = fv[type];
    const F3 A = ld(P, va), AP = sub(p, A);
    for (int32_t r = M.surf->ring_ofs[size_t(va)]; r < M.surf->ring_ofs[size_t(va) + 1]; ++r) {
        const F3 BA = sub(A, ld(P, M.surf->ring[size_t(r)]));
        if (dot(AP, BA) < -dot(BA, BA) * eps) return false;
    }
    return true;
}

bool Detector::dcd(int m, int i, const DcdParams& prm, CcdHit& hit) const {
    hit = CcdHit{};
    const CcdMesh& M = d_->meshes[size_t(m)];
    const bool prev = d_->use_prev_tets;
    const int32_t v = M.surf->verts[size_t(i)];
    const F3 p = ld(prev ? M.xprev : M.x, v);
    Box q = empty_box();
    const float pp[3] = {p.x, p.y, p.z};
    extend(q, pp);
    // vertexCollisionDetection (DiscreteCollisionDetector.cpp:517-536, callback 12-95):
    // the first tet (lowest mesh, tet) that strictly contains the vertex
    int im = -1;
    int32_t it = -1;
    for (int32_t g : d_->tets.query(q)) {
        const auto [tm, t] = d_->tet_of(g);
        if (!prm.handle_self && tm == m) continue;
        const CcdMesh& T = d_->meshes[size_t(tm)];
        const int32_t* tv = &T.tets[4 * size_t(t)];
        if (tm == m && (tv[0] == v || tv[1] == v || tv[2] == v || tv[3] == v)) continue;
        const float* P = prev ? T.xprev : T.x;
        if (point_in_tet(p, ld(P, tv[0]), ld(P, tv[1]), ld(P, tv[2]), ld(P, tv[3]))) {
            im = tm;
            it = t;
            break;
        }
    }
    if (im < 0) return false;
    // closestPointQuery (:538-660, callback 97-329): the nearest surface face of the
    // intersected mesh whose closest point is not the vertex itself, lies in the face's
    // feasible region and from which the tetrahedral traversal reaches the containing
    // tet (:189-300); equal distances keep the lower face
    const CcdMesh& S = d_->meshes[size_t(im)];
    const float* P = prev ? S.xprev : S.x;
    const bool traverse = prm.check_traverse && (im == m || prm.traverse_non_self);
    // the query point moved a little toward the containing tet's centroid (:215-224)
    F3 target = p;
    if (traverse && prm.shift_to_center) {
        const int32_t* tv = &S.tets[4 * size_t(it)];
        const F3 cen = scale(add(add(add(ld(P, tv[0]), ld(P, tv[1])), ld(P, tv[2])), ld(P, tv[3])), 0.25f);
        target = add(scale(p, 1.f - prm.center_shift), scale(cen, prm.center_shift));
    }
    float best = 3.4e38f;
    for (size_t f = 0; f < S.surf->faces.size() / 3; ++f) {
        const int32_t* fv = &S.surf->faces[3 * f];
        float bary[3];
        F3 cp;
        const int type = closest_point(p, ld(P, fv[0]), ld(P, fv[1]), ld(P, fv[2]), bary, cp);
        const F3 dd = sub(p, cp);
        const float d = std::sqrt(dot(dd, dd));
        if (im == m && type <= 2 && fv[type] == v) continue;
        if (!(d < best)) continue;
        if (prm.check_feasible && !feasible(S, P, p, int32_t(f), type, prm.feasible_eps)) continue;
        if (traverse) {
            // from the closest point (moved a little toward the face's centroid unless it is
            // interior) toward the query point (:206-247)
            F3 o = cp;
            if (type != 6) {
                const F3 sum = add(add(ld(P, fv[0]), ld(P, fv[1])), ld(P, fv[2]));
                o = add(scale(cp, 1.f - prm.center_shift), scale(sum, prm.center_shift / 3.0f));
            }
            const F3 ray = sub(target, o);
            const float len = std::sqrt(dot(ray, ray));
            const float dir[3] = {ray.x / len, ray.y / len, ray.z / len};
            const float org[3] = {o.x, o.y, o.z};
            const float max_dis = prm.stop_after_passing ? prm.max_search_mult * len : -1.f;
            int status = 0;
            const bool ok =
                tet_traverse(P, S.tets, *S.surf, org, dir, max_dis, int32_t(f), it, prm.ray_eps, prm.static_traverse,
                             &status);
            if (!ok) continue;
        }
        best = d;
        hit.fmesh = im;
        hit.face = int32_t(f);
        hit.depth = d;
        hit.tt = -1.f;
        for (int k = 0; k < 3; ++k) hit.bary[k] = bary[k];
    }
    return true;
}

}  // namespace oracle_tc

extern "C" {

int32_t oracle_ccd_tri_point(const float* x0, const float* x1, const float* p0, const float* p1, float* tt,
                             float* bary) {
    return oracle_tc::ccd_tri_point(x0, x1, p0, p1, tt, bary);
}

int32_t oracle_tet_walk(int32_t nv, int32_t ntet, const int32_t* tets, const double* X, int32_t face, int32_t target,
                        const float* origin, const float* dir, float max_dis, float ray_eps, int32_t use_static,
                        int32_t* status) {
    const oracle_tc::Surface s = oracle_tc::extract_surface(nv, ntet, tets, X);
    if (face < 0 || size_t(face) >= s.faces.size() / 3 || target < 0 || target >= ntet) return -1;
    std::vector<float> xf(3 * size_t(nv));
    for (size_t i = 0; i < xf.size(); ++i) xf[i] = float(X[i]);
    int st = 0;
    const bool ok = oracle_tc::tet_traverse(xf.data(), tets, s, origin, dir, max_dis, face, target, ray_eps, use_static != 0,
                                            &st);
    if (status) *status = st;
    return ok ? 1 : 0;
}

void oracle_tet_surface(int32_t nv, int32_t ntet, const int32_t* tets, const double* X, int32_t* nfaces,
                        int32_t* nverts, int32_t* faces, int32_t* verts) {
    oracle_tc::Surface s = oracle_tc::extract_surface(nv, ntet, tets, X);
    *nfaces = int32_t(s.faces.size() / 3);
    *nverts = int32_t(s.verts.size());
    if (faces) std::copy(s.faces.begin(), s.faces.end(), faces);
    if (verts) std::copy(s.verts.begin(), s.verts.end(), verts);
}

}  // extern "C"
