// Device-side geometry and contact model of the cloth VBD step, shared by the
// contact detector (cloth_cd.cu) and the per-color solve (cloth_engine.cu).
//
// The geometric predicates (closest point on a triangle, closest points of two
// segments, feasible regions) are evaluated in FP32 in a fixed operation order;
// the detector's translation unit is compiled without FMA contraction so that
// its results are bit-identical to the CPU restatement of the same formulas.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gaia {
namespace cloth {

constexpr int VF_CAP = 32;   // VF contacts kept per query vertex
constexpr int EE_CAP = 64;   // EE contacts kept per query edge
constexpr int FV_CAP = 32;   // contacting vertices linked per face (FV_CONTACT_PREALLOCATE)
constexpr int CAND_CAP = 128; // narrow-phase candidates per query before ordering
constexpr float CMP_EPS = 1e-5f;                  // CMP_EPSILON (Types/Types.h:20)
constexpr float CMP_EPS2 = CMP_EPS * CMP_EPS;     // CMP_EPSILON2
constexpr float FEASIBLE_EPS = 1e-3f;             // feasible-region epsilon of the VF query
constexpr float ABS_RELAX = 1e-6f;                // ABSOLUTE_RELAXIATION (TriMeshCollisionGeometry.cpp:4)

// ClosestPointOnTriangleType (CollisionDetector/CollisionDetertionParameters.h:141-151)
enum PointType : int { AtA = 0, AtB, AtC, AtAB, AtBC, AtAC, AtInterior, NotFound };
// ClosestPointOnPrimitiveType (:153-160)
enum PrimType : int { PrimVertex = 0, PrimEdge = 1, PrimFace = 2, PrimNone = 4 };

// overflow / event counters
enum { CC_VF_OVERFLOW = 0, CC_EE_OVERFLOW, CC_FV_OVERFLOW, CC_CAND_OVERFLOW, CC_STACK_OVERFLOW, CC_TRUNCATIONS,
       CC_DETECTIONS, CC_FP64_SOLVES, CC_FAILED, CC_NONFINITE, CC_N };

// ---- vector helpers (float3 / double3, fixed operation order) --------------------
__host__ __device__ __forceinline__ float3 v3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 sub(float3 a, float3 b) { return float3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ float3 add(float3 a, float3 b) { return float3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ float3 mul(float s, float3 a) { return float3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return float3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ __forceinline__ double3 sub(double3 a, double3 b) { return double3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ double3 add(double3 a, double3 b) { return double3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ double3 mul(double s, double3 a) { return double3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ double dot(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ double3 cross(double3 a, double3 b) {
    return double3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float3 ld3(const float4* x, int i) {
    float4 p = x[i];
    return v3(p.x, p.y, p.z);
}

// Closest point on triangle abc to p (CollisionGeometry.h:84-145, the
// Voronoi-region walk of Ericson's "Real-Time Collision Detection" 5.1.5).
template <typename V, typename S>
__host__ __device__ __forceinline__ int closest_point_triangle(V p, V a, V b, V c, V& bary, V& cp) {
    const V ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    const S d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= S(0) && d2 <= S(0)) {
        bary = V{S(1), S(0), S(0)};
        cp = a;
        return AtA;
    }
    const V bp = sub(p, b);
    const S d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= S(0) && d4 <= d3) {
        bary = V{S(0), S(1), S(0)};
        cp = b;
        return AtB;
    }
    const V cpv = sub(p, c);
    const S d5 = dot(ab, cpv), d6 = dot(ac, cpv);
    if (d6 >= S(0) && d5 <= d6) {
        bary = V{S(0), S(0), S(1)};
        cp = c;
        return AtC;
    }
    const S vc = d1 * d4 - d3 * d2;
    if (vc <= S(0) && d1 >= S(0) && d3 <= S(0)) {
        const S v = d1 / (d1 - d3);
        bary = V{S(1) - v, v, S(0)};
        cp = add(a, mul(v, ab));
        return AtAB;
    }
    const S vb = d5 * d2 - d1 * d6;
    if (vb <= S(0) && d2 >= S(0) && d6 <= S(0)) {
        const S v = d2 / (d2 - d6);
        bary = V{S(1) - v, S(0), v};
        cp = add(a, mul(v, ac));
        return AtAC;
    }
    const S va = d3 * d6 - d5 * d4;
    if (va <= S(0) && (d4 - d3) >= S(0) && (d5 - d6) >= S(0)) {
        const S v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary = V{S(0), S(1) - v, v};
        cp = add(b, mul(v, sub(c, b)));
        return AtBC;
    }
    const S denom = S(1) / (va + vb + vc);
    const S v = vb * denom, w = vc * denom;
    bary = V{S(1) - v - w, v, w};
    cp = add(add(a, mul(v, ab)), mul(w, ac));
    return AtInterior;
}

__host__ __device__ __forceinline__ int prim_type(int t) {
    return t <= AtC ? PrimVertex : (t <= AtAC ? PrimEdge : (t == AtInterior ? PrimFace : PrimNone));
}

// Closest points of segments p0p1 and q0q1 with parameters s, t
// (CollisionGeometry.h:147-255, Eberly's segment-segment distance).
template <typename V, typename S>
__host__ __device__ __forceinline__ void closest_points_segments(V p0, V p1, V q0, V q1, V& cps, V& cqt, S& s, S& t) {
    const V p = sub(p1, p0), q = sub(q1, q0), r = sub(p0, q0);
    const S a = dot(p, p), b = dot(p, q), c = dot(q, q), d = dot(p, r), e = dot(q, r);
    s = S(0);
    t = S(0);
    const S det = a * c - b * b;
    if (det > S(CMP_EPS)) {
        const S bte = b * e, ctd = c * d;
        if (bte <= ctd) {
            if (e <= S(0)) {
                s = (-d >= a ? S(1) : (-d > S(0) ? -d / a : S(0)));
                t = S(0);
            } else if (e < c) {
                s = S(0);
                t = e / c;
            } else {
                s = (b - d >= a ? S(1) : (b - d > S(0) ? (b - d) / a : S(0)));
                t = S(1);
            }
        } else {
            s = bte - ctd;
            if (s >= det) {
                if (b + e <= S(0)) {
                    s = (-d <= S(0) ? S(0) : (-d < a ? -d / a : S(1)));
                    t = S(0);
                } else if (b + e < c) {
                    s = S(1);
                    t = (b + e) / c;
                } else {
                    s = (b - d <= S(0) ? S(0) : (b - d < a ? (b - d) / a : S(1)));
                    t = S(1);
                }
            } else {
                const S ate = a * e, btd = b * d;
                if (ate <= btd) {
                    s = (-d <= S(0) ? S(0) : (-d >= a ? S(1) : -d / a));
                    t = S(0);
                } else {
                    t = ate - btd;
                    if (t >= det) {
                        s = (b - d <= S(0) ? S(0) : (b - d >= a ? S(1) : (b - d) / a));
                        t = S(1);
                    } else {
                        s /= det;
                        t /= det;
                    }
                }
            }
        }
    } else {
        if (e <= S(0)) {
            s = (-d <= S(0) ? S(0) : (-d >= a ? S(1) : -d / a));
            t = S(0);
        } else if (e >= c) {
            s = (b - d <= S(0) ? S(0) : (b - d >= a ? S(1) : (b - d) / a));
            t = S(1);
        } else {
            s = S(0);
            t = e / c;
        }
    }
    cps = add(mul(S(1) - s, p0), mul(s, p1));
    cqt = add(mul(S(1) - t, q0), mul(t, q1));
}

// ---- contact model (templated on the solve precision) ---------------------------

// computeContactRepulsiveForce (VBDCloth/VBDClothPhysics.cpp:1533-1579), energy type 1
// (quadratic-logarithmic, two stages; C2 at tau = r / 2).
template <typename R>
__host__ __device__ __forceinline__ void contact_repulsion(R dis, R thickness, R r, R k, R& dEdD, R& d2E) {
    const R dadj = dis - thickness;
    const R tau = r * R(0.5);
    if (dadj < tau && dadj > R(CMP_EPS)) {
        const R k2 = R(0.5) * tau * tau * k;
        dEdD = -k2 / dadj;
        d2E = k2 / (dadj * dadj);
    } else {
        dEdD = -k * (r - dadj);
        d2E = k;
    }
}

// computeFriction (VBDClothPhysics.cpp:1500-1531): lagged IPC friction in the tangent
// frame T = [t0 t1] (unit columns); adds b * force and b^2 * the (PSD, n-frozen) Hessian.
template <typename R>
__host__ __device__ __forceinline__ void friction(R mu, R lambda, const R* t0, const R* t1, R u0, R u1, R epsU, R b,
                                                  R* f, R* H) {
    const R un = sqrt(u0 * u0 + u1 * u1);
    if (!(un > R(0))) return;
    const R f1 = un > epsU ? R(1) / un : (-un / epsU + R(2)) / epsU;
    const R s = -mu * lambda * f1 * b;
    const R hs = mu * lambda * f1 * b * b;
#pragma unroll
    for (int i = 0; i < 3; ++i) f[i] += s * (t0[i] * u0 + t1[i] * u1);
    // H (sym: 00 01 02 11 12 22) += hs (t0 t0^T + t1 t1^T)
    H[0] += hs * (t0[0] * t0[0] + t1[0] * t1[0]);
    H[1] += hs * (t0[0] * t0[1] + t1[0] * t1[1]);
    H[2] += hs * (t0[0] * t0[2] + t1[0] * t1[2]);
    H[3] += hs * (t0[1] * t0[1] + t1[1] * t1[1]);
    H[4] += hs * (t0[1] * t0[2] + t1[1] * t1[2]);
    H[5] += hs * (t0[2] * t0[2] + t1[2] * t1[2]);
}

}  // namespace cloth
}  // namespace gaia
