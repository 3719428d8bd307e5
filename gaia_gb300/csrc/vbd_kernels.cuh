// Device code of the GB300 VBD step.
//
// Precision modes (template parameters ST = state trait, R = compute type; see vbd_state.cuh):
//   fp32  <StF32, float>  : everything FP32
//   mixed <StDF,  float>  : displacements / inertia targets stored as double-float
//                           pairs; every per-incidence force and Hessian term, their
//                           accumulation and the 3x3 solve in FP32 (FP64 retry for
//                           ill-conditioned blocks). No FP64 instruction runs per
//                           incidence.
//   fp64  <StF64, double> : everything FP64 (the plain FP64 baseline)
//
// The state is the displacement u = x - X from the FP32 rest positions X, and
// the elastic terms are written in the displacement gradient G = F - I. Near
// rest, the reference's P = mu F + lambda (J - a) cof F is a difference of
// O(mu) terms (lambda (1 - a) = -mu), which costs FP32 three digits at strains
// of 1e-3; in G the same stress is mu (G - Cg) + lambda dJ (I + Cg) with
// Cg = cof(F) - I and dJ = det F - 1, built from small quantities only.
//
// Data layout in HBM (built once on the host, see vbd_engine.cu):
//   * vertices are renumbered into "slots": the solvable vertices of merged
//     color 0, then color 1, ..., then all fixed vertices. Per-slot arrays are
//     therefore contiguous per color and every per-vertex access of a color
//     sweep is coalesced.
//   * u[s]     = displacement and mass (ST::U: 16 B FP32, 32 B double-float or FP64)
//     rest[s]  = (X, Y, Z, unused)  float4, rest position
//     y[s]     = inertia target, as a displacement (ST::U)
//     xprev[s] = displacement at the start of the substep (ST::U)
//     vel[s]   = velocity (ST::V: FP32, or FP64 in the fp64 mode)
//   * incidence records, one per (solvable vertex, incident tet), stored in
//     slot order (CSR offsets inc_ofs): the slots of the tet's three other
//     vertices and their rows of dF/dx ("m vectors", from the FP64 DmInv):
//       FP32: rec_n = int4{n0, n1, n2, bits(m2.z)}, rec_a = {m0.xyz, m1.x},
//             rec_b = {m1.yz, m2.xy}                          -> 48 B
//       FP64: rec_n = int4{n0, n1, n2, 0}, rec_a, rec_b (double4), rec_c = m2.z -> 88 B
//     The own vertex's row is -(m0+m1+m2), and the rest volume is
//     1 / (6 det[m0;m1;m2]) (the rows are stored in an order that makes the
//     determinant equal det(DmInv)), so neither is stored.
//
// Per incidence the Neo-Hookean block is evaluated in closed form. With
// G = sum_j (u_j - u_o) m_j^T (so F = I + G), J = det F, g = cof(F) m_o (= dJ/dx_o):
//   force  -= A [ mu F m_o + lambda (J - a) g ]      (evaluated in G, see above)
//   H      += A [ lambda g g^T ] + A mu |m_o|^2 I
// which equals the reference's contraction of its 9x9 d2E/dF2 with the vertex
// row of dF/dx (VBDPhysicsCompute.cu:2035-2232, VBD_NeoHookean.cpp:379-581):
// det F is affine in x_o, so the (J - a) d2J/dF2 term contracts to zero.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cloth_dev.cuh"
#include "vbd_state.cuh"

namespace gaia {
namespace dev {

template <typename R>
struct MeshMat {
    R mu, lmbd, a, kh, kd, exp_damp, const_damp, pad;
    int32_t init_type, pad2, pad3, pad4;
};

template <typename R>
struct Consts {
    R dt, inv_dt, dt2inv;
    R kb, fr_mu, fr_epsU;
    R kc;  // collisionStiffness of the tet-mesh v-f contact
    R step, step_gd;
    double dt_d;
    double g[3];
    double lo[3], hi[3];
    float dt_f, g_f[3], lo_f[3], hi_f[3];  // the same constants for FP32 state arithmetic
    int32_t plane, assoc_grav;
    int32_t spin_limit;  // polls of a bounded wait before it gives up (kMbarSpinLimit unless a test lowers it)
};

// The FP64 or FP32 copy of a constant, matching the state scalar type.
template <typename Sc>
__device__ __forceinline__ Sc pick(double d, float f);
template <>
__device__ __forceinline__ float pick<float>(double, float f) { return f; }
template <>
__device__ __forceinline__ double pick<double>(double d, float) { return d; }

// Programmatic dependent launch: let the next grid in the stream start its
// prologue now, and wait for the previous grid's results (no-ops when the
// kernel was not launched as a programmatic dependent).
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Counter slots in device memory. CNT_TIMEOUT: blocks whose bounded wait on staged
// records (or on a grid barrier) ran out and that skipped their vertices; CNT_DRAIN: of
// those, blocks whose final drain wait ran out too.
enum { CNT_FP64_SOLVES = 0, CNT_FAILED_SOLVES = 1, CNT_NONFINITE = 2, CNT_TIMEOUT = 3, CNT_DRAIN = 4, CNT_N = 8 };

template <typename ST, typename R>
struct Ptrs {
    typename ST::U* u;
    const float4* rest;
    typename ST::U* y;
    typename ST::U* xprev;
    typename ST::V* vel;
    typename ST::V* vprev;
    const int32_t* inc_ofs;
    const int4* rec_n;
    const R4<R>* rec_a;
    const R4<R>* rec_b;
    const R* rec_c;            // FP64 only
    const int32_t* slot_mesh;
    const MeshMat<R>* mats;
    unsigned long long* counters;
    int32_t nactive, nslots;
    // tet-mesh contact records (tet_cd.hpp; null when contact detection is off)
    const uint8_t* col_info;
    const int4* col_own;
    const int32_t* col_rel;
    const double2* mesh_fric;      // per mesh: frictionDynamic, frictionEpsV
    R* col_scratch;                // 9 per slot: contact force (3) and Hessian (6) of the solve
    // mesh frames (null when off): per mesh the shift that the substep's initial step takes
    // out of every state of the mesh and the frame offset F (FP64); per slot the reference
    // position X + F as a float pair, which the world-box test uses in place of X
    const float4* frame_shift;
    const double4* frame_F;
    float4* rest_fh;
    float4* rest_fl;
};


struct DeformerDev {
    int32_t type;              // 0 rotator, 1 translator
    double axis[3], omega, end_time, speed[3];
};

struct DeformVerts {
    const int32_t* slot;
    const int32_t* def;        // deformer index
    const double* a;           // root (rotator) or original position (translator), 3 per vertex
    const double* b;           // root-relative point (rotator), 3 per vertex
    const DeformerDev* defs;
    int32_t n;
};

// ---------------------------------------------------------------------------
// small math
// ---------------------------------------------------------------------------
__device__ __forceinline__ float f_bits(int v) { return __int_as_float(v); }

// Symmetric 3x3 solve by LDL^T (the same algorithm as the oracle's
// solve3x3_ldlt). H = {h00, h01, h02, h11, h12, h22}.
template <typename R>
__device__ __forceinline__ bool ldlt3(const R* H, const R* b, R* x, R rel_tol) {
    R scale = fmax(fabs(H[0]), fmax(fabs(H[3]), fabs(H[5])));
    if (!(scale > R(0))) return false;
    R tol = rel_tol * scale;
    R d0 = H[0];
    if (!(d0 > tol)) return false;
    R l10 = H[1] / d0, l20 = H[2] / d0;
    R d1 = H[3] - l10 * H[1];
    if (!(d1 > tol)) return false;
    R l21 = (H[4] - l20 * H[1]) / d1;
    R d2 = H[5] - l20 * H[2] - l21 * l21 * d1;
    if (!(d2 > tol)) return false;
    R z0 = b[0];
    R z1 = b[1] - l10 * z0;
    R z2 = b[2] - l20 * z0 - l21 * z1;
    z0 /= d0;
    z1 /= d1;
    z2 /= d2;
    x[2] = z2;
    x[1] = z1 - l21 * x[2];
    x[0] = z0 - l10 * x[1] - l20 * x[2];
    return isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]);
}

// FP32: one reciprocal per pivot instead of two divisions per pivot (three IEEE divisions
// instead of six on the vertex's serial path); the FP64 factorisation divides.
template <>
__device__ __forceinline__ bool ldlt3<float>(const float* H, const float* b, float* x, float rel_tol) {
    const float scale = fmaxf(fabsf(H[0]), fmaxf(fabsf(H[3]), fabsf(H[5])));
    if (!(scale > 0.f)) return false;
    const float tol = rel_tol * scale;
    const float d0 = H[0];
    if (!(d0 > tol)) return false;
    const float r0 = 1.f / d0;
    const float l10 = H[1] * r0, l20 = H[2] * r0;
    const float d1 = H[3] - l10 * H[1];
    if (!(d1 > tol)) return false;
    const float r1 = 1.f / d1;
    const float l21 = (H[4] - l20 * H[1]) * r1;
    const float d2 = H[5] - l20 * H[2] - l21 * l21 * d1;
    if (!(d2 > tol)) return false;
    const float r2 = 1.f / d2;
    const float z0 = b[0];
    const float z1 = b[1] - l10 * z0;
    const float z2 = b[2] - l20 * z0 - l21 * z1;
    x[2] = z2 * r2;
    x[1] = z1 * r1 - l21 * x[2];
    x[0] = z0 * r0 - l10 * x[1] - l20 * x[2];
    return isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]);
}

// Relative pivot thresholds of the 3x3 LDL^T: an FP32 factorisation, the FP64 retry of an
// FP32-accumulated block, and an FP64 block. The retry's entries carry the rounding of
// their FP32 accumulation (a few 1e-7 of the largest diagonal after 10-30 incidences), so
// a pivot below kRetryPivot of it is rounding noise, not information: such a block is
// treated as singular (the gradient step) instead of being solved into a wild step.
constexpr float kFp32Pivot = 1e-5f;
constexpr double kRetryPivot = 2e-6;
constexpr double kFp64Pivot = 1e-12;

// FP32 solve with FP64 retry for ill-conditioned blocks; FP64 solve directly.
template <typename R>
__device__ __forceinline__ bool solve3(const R* H, const R* b, R* x, unsigned long long* counters);
template <>
__device__ __forceinline__ bool solve3<float>(const float* H, const float* b, float* x, unsigned long long* counters) {
    if (ldlt3<float>(H, b, x, kFp32Pivot)) return true;
    double Hd[6], bd[3], xd[3];
#pragma unroll
    for (int i = 0; i < 6; ++i) Hd[i] = H[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) bd[i] = b[i];
    atomicAdd(&counters[CNT_FP64_SOLVES], 1ull);
    if (!ldlt3<double>(Hd, bd, xd, kRetryPivot)) return false;
#pragma unroll
    for (int i = 0; i < 3; ++i) x[i] = float(xd[i]);
    return true;
}
template <>
__device__ __forceinline__ bool solve3<double>(const double* H, const double* b, double* x, unsigned long long*) {
    return ldlt3<double>(H, b, x, kFp64Pivot);
}

// One incidence record as loaded from HBM (streaming loads: each record is
// read once per iteration). load() issues the loads; the fields are decoded
// where they are used, so a record can be in flight while the previous one
// is being computed.
template <typename R>
struct RecRaw;
template <>
struct RecRaw<float> {
    int4 n;
    float4 a, b;
    __device__ __forceinline__ void load(const int4* rec_n, const R4<float>* rec_a, const R4<float>* rec_b,
                                         const float*, int r) {
        n = __ldcs(rec_n + r);
        a = __ldcs(reinterpret_cast<const float4*>(rec_a) + r);
        b = __ldcs(reinterpret_cast<const float4*>(rec_b) + r);
    }
    // cached (not streaming): for a kernel that reads the same records every iteration
    __device__ __forceinline__ void load_kept(const int4* rec_n, const R4<float>* rec_a, const R4<float>* rec_b,
                                              const float*, int r) {
        n = __ldg(rec_n + r);
        a = __ldg(reinterpret_cast<const float4*>(rec_a) + r);
        b = __ldg(reinterpret_cast<const float4*>(rec_b) + r);
    }
    __device__ __forceinline__ void rows(float* m0, float* m1, float* m2) const {
        m0[0] = a.x; m0[1] = a.y; m0[2] = a.z;
        m1[0] = a.w; m1[1] = b.x; m1[2] = b.y;
        m2[0] = b.z; m2[1] = b.w; m2[2] = f_bits(n.w);
    }
};
template <>
struct RecRaw<double> {
    int4 n;
    double2 a0, a1, b0, b1;
    double c;
    __device__ __forceinline__ void load(const int4* rec_n, const R4<double>* rec_a, const R4<double>* rec_b,
                                         const double* rec_c, int r) {
        n = __ldcs(rec_n + r);
        const double2* pa = reinterpret_cast<const double2*>(rec_a + r);
        const double2* pb = reinterpret_cast<const double2*>(rec_b + r);
        a0 = __ldcs(pa); a1 = __ldcs(pa + 1); b0 = __ldcs(pb); b1 = __ldcs(pb + 1);
        c = __ldcs(rec_c + r);
    }
    __device__ __forceinline__ void load_kept(const int4* rec_n, const R4<double>* rec_a, const R4<double>* rec_b,
                                              const double* rec_c, int r) {
        n = __ldg(rec_n + r);
        const double2* pa = reinterpret_cast<const double2*>(rec_a + r);
        const double2* pb = reinterpret_cast<const double2*>(rec_b + r);
        a0 = __ldg(pa); a1 = __ldg(pa + 1); b0 = __ldg(pb); b1 = __ldg(pb + 1);
        c = __ldg(rec_c + r);
    }
    __device__ __forceinline__ void rows(double* m0, double* m1, double* m2) const {
        m0[0] = a0.x; m0[1] = a0.y; m0[2] = a1.x;
        m1[0] = a1.y; m1[1] = b0.x; m1[2] = b0.y;
        m2[0] = b1.x; m2[1] = b1.y; m2[2] = c;
    }
};

// Accumulator of one vertex: force (3), lambda-part of the Hessian (6, upper
// triangle), and S = sum A mu |m_o|^2 (the isotropic part).
template <typename R>
struct Acc {
    R f0, f1, f2, h00, h01, h02, h11, h12, h22, S;
};

// e0, e1, e2 = u_j - u_o (relative displacements) of the three other vertices.
template <typename R>
__device__ __forceinline__ void incidence(const R* e0, const R* e1, const R* e2, const R* m0, const R* m1,
                                          const R* m2, R mu, R lmbd, Acc<R>& acc) {
    R G[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) G[r][c] = e0[r] * m0[c] + e1[r] * m1[c] + e2[r] * m2[c];
    // rest volume from the stored rows: A = 1 / (6 det[m0; m1; m2])
    R detM = m0[0] * (m1[1] * m2[2] - m1[2] * m2[1]) - m0[1] * (m1[0] * m2[2] - m1[2] * m2[0]) +
             m0[2] * (m1[0] * m2[1] - m1[1] * m2[0]);
    R A = R(1) / (R(6) * detM);
    R mo[3] = {-(m0[0] + m1[0] + m2[0]), -(m0[1] + m1[1] + m2[1]), -(m0[2] + m1[2] + m2[2])};
    // Cg = cof(I + G) - I, entrywise
    R C00 = G[1][1] + G[2][2] + (G[1][1] * G[2][2] - G[1][2] * G[2][1]);
    R C11 = G[0][0] + G[2][2] + (G[0][0] * G[2][2] - G[0][2] * G[2][0]);
    R C22 = G[0][0] + G[1][1] + (G[0][0] * G[1][1] - G[0][1] * G[1][0]);
    R C01 = G[1][2] * G[2][0] - G[1][0] * (R(1) + G[2][2]);
    R C02 = G[1][0] * G[2][1] - (R(1) + G[1][1]) * G[2][0];
    R C10 = G[0][2] * G[2][1] - G[0][1] * (R(1) + G[2][2]);
    R C12 = G[0][1] * G[2][0] - (R(1) + G[0][0]) * G[2][1];
    R C20 = G[0][1] * G[1][2] - G[0][2] * (R(1) + G[1][1]);
    R C21 = G[0][2] * G[1][0] - (R(1) + G[0][0]) * G[1][2];
    // dJ = det(I + G) - 1 = G00 (1 + Cg00) + G01 C01 + G02 C02 + Cg00
    R dJ = G[0][0] * (R(1) + C00) + G[0][1] * C01 + G[0][2] * C02 + C00;
    // g = cof(F) m_o = m_o + Cg m_o
    R cm0 = C00 * mo[0] + C01 * mo[1] + C02 * mo[2];
    R cm1 = C10 * mo[0] + C11 * mo[1] + C12 * mo[2];
    R cm2 = C20 * mo[0] + C21 * mo[1] + C22 * mo[2];
    R g0 = mo[0] + cm0, g1 = mo[1] + cm1, g2 = mo[2] + cm2;
    R Gm0 = G[0][0] * mo[0] + G[0][1] * mo[1] + G[0][2] * mo[2];
    R Gm1 = G[1][0] * mo[0] + G[1][1] * mo[1] + G[1][2] * mo[2];
    R Gm2 = G[2][0] * mo[0] + G[2][1] * mo[1] + G[2][2] * mo[2];
    // P m_o = mu (G - Cg) m_o + lambda dJ g
    R Am = A * mu;
    R Ald = A * lmbd * dJ;
    acc.f0 -= Am * (Gm0 - cm0) + Ald * g0;
    acc.f1 -= Am * (Gm1 - cm1) + Ald * g1;
    acc.f2 -= Am * (Gm2 - cm2) + Ald * g2;
    R Al = A * lmbd;
    R lg0 = Al * g0, lg1 = Al * g1, lg2 = Al * g2;
    acc.h00 += lg0 * g0;
    acc.h01 += lg0 * g1;
    acc.h02 += lg0 * g2;
    acc.h11 += lg1 * g1;
    acc.h12 += lg1 * g2;
    acc.h22 += lg2 * g2;
    acc.S += Am * (mo[0] * mo[0] + mo[1] * mo[1] + mo[2] * mo[2]);
}

template <int L, typename R>
__device__ __forceinline__ void reduce_group(Acc<R>& a) {
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1) {
        a.f0 += __shfl_xor_sync(0xffffffffu, a.f0, off);
        a.f1 += __shfl_xor_sync(0xffffffffu, a.f1, off);
        a.f2 += __shfl_xor_sync(0xffffffffu, a.f2, off);
        a.h00 += __shfl_xor_sync(0xffffffffu, a.h00, off);
        a.h01 += __shfl_xor_sync(0xffffffffu, a.h01, off);
        a.h02 += __shfl_xor_sync(0xffffffffu, a.h02, off);
        a.h11 += __shfl_xor_sync(0xffffffffu, a.h11, off);
        a.h12 += __shfl_xor_sync(0xffffffffu, a.h12, off);
        a.h22 += __shfl_xor_sync(0xffffffffu, a.h22, off);
        a.S += __shfl_xor_sync(0xffffffffu, a.S, off);
    }
}

// IPC-style lagged friction (VBD_GeneralCompute.h:10-66; VBDPhysics.cpp:2563-2592)
// for an axis-aligned contact normal along `d`: tangents e_{d+1}, e_{d+2}.
template <typename R>
__device__ __forceinline__ void axis_friction(int d, const R* dx, R mu, R lambda, R epsU, R* f, R* H) {
    int t0 = (d + 1) % 3, t1 = (d + 2) % 3;
    R u0 = dx[t0], u1 = dx[t1];
    R un = sqrt(u0 * u0 + u1 * u1);
    if (!(un > R(0))) return;
    R f1 = un > epsU ? R(1) / un : (-un / epsU + R(2)) / epsU;
    R s = mu * lambda * f1;
    f[t0] -= s * u0;
    f[t1] -= s * u1;
    // H += s * (e_t0 e_t0^T + e_t1 e_t1^T): diagonal entries of the two tangents
    H[t0 == 0 ? 0 : (t0 == 1 ? 3 : 5)] += s;
    H[t1 == 0 ? 0 : (t1 == 1 ? 3 : 5)] += s;
}

// ---------------------------------------------------------------------------
// Per-color block solve. One group of L lanes per vertex of the color range
// [beg, end). PROBE = write force/Hessian of the single vertex `beg` to
// probe_out instead of moving it.
// ---------------------------------------------------------------------------
template <typename ST, typename R, bool PROBE>
__device__ __forceinline__ bool vertex_tail(const Ptrs<ST, R>& P, const Consts<R>& c, int v, const typename ST::U& uo,
                                            const MeshMat<R>& mat, const Acc<R>& acc, int friction,
                                            double* probe_out, int beg, int end, typename ST::U* unew = nullptr);

// ---------------------------------------------------------------------------
// Tet-mesh vertex-face contact (VBDPhysicsCompute.cu:1731-1773, 1812-1930)
// ---------------------------------------------------------------------------
template <typename R>
struct V3T;
template <>
struct V3T<float> {
    using type = float3;
};
template <>
struct V3T<double> {
    using type = double3;
};

// accumlateCollisionForceAndHessianPerCollision_v2: the contact of vertex sp with its
// recorded face, at the current positions, on the contact vertex of index `order`
// (3 = sp itself, 0..2 = a face vertex). Positions are taken relative to sp's: q - p =
// (X_q - X_p) + (u_q - u_p). Penalty k * depth along the face normal (interior closest
// point) or the closest-point direction oriented like the face normal, lagged IPC
// friction in the frame (edge AB, AB x n); scaled by b = 1 (sp) or -barycentric.
template <typename ST, typename R>
__device__ __forceinline__ void contact_term(const Ptrs<ST, R>& P, const Consts<R>& c, int sp, int order, R* f,
                                             R* H) {
    using U = typename ST::U;
    using V = typename V3T<R>::type;
    const int4 fo = P.col_own[sp];
    const int fs[3] = {fo.x, fo.y, fo.z};
    const U up = P.u[sp];
    const float4 Xp = P.rest[sp];
    V q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 Xq = P.rest[fs[k]];
        R d[3];
        ST::diff(P.u[fs[k]], up, d);
        q[k] = V{R(Xq.x) - R(Xp.x) + d[0], R(Xq.y) - R(Xp.y) + d[1], R(Xq.z) - R(Xp.z) + d[2]};
    }
    const V o{R(0), R(0), R(0)};
    V bary, cp;
    const int type = cloth::closest_point_triangle<V, R>(o, q[0], q[1], q[2], bary, cp);
    V fn = cloth::cross(cloth::sub(q[1], q[0]), cloth::sub(q[2], q[0]));
    const R fl = sqrt(cloth::dot(fn, fn));
    fn = V{fn.x / fl, fn.y / fl, fn.z / fl};
    const V diff = cp;
    V n;
    if (type == cloth::AtInterior) {
        n = fn;
    } else {
        const R inv = R(1) / sqrt(cloth::dot(diff, diff));
        n = cloth::mul(inv, diff);
        if (cloth::dot(n, fn) < R(0)) n = V{-n.x, -n.y, -n.z};
    }
    const R depth = cloth::dot(diff, n);
    if (!(depth > R(0))) return;
    const R bw[4] = {-bary.x, -bary.y, -bary.z, R(1)};
    const R b = bw[order];
    const R lambda = depth * c.kc;
    const R nn[3] = {n.x, n.y, n.z};
    const R s1 = b * lambda, s2 = b * b * c.kc;
    f[0] += s1 * nn[0]; f[1] += s1 * nn[1]; f[2] += s1 * nn[2];
    H[0] += s2 * nn[0] * nn[0]; H[1] += s2 * nn[0] * nn[1]; H[2] += s2 * nn[0] * nn[2];
    H[3] += s2 * nn[1] * nn[1]; H[4] += s2 * nn[1] * nn[2]; H[5] += s2 * nn[2] * nn[2];
    // relative tangential displacement over the substep: dx_p - sum_k bary_k dx_k
    R dx[3];
    ST::diff(up, P.xprev[sp], dx);
    const R bk[3] = {bary.x, bary.y, bary.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R dk[3];
        ST::diff(P.u[fs[k]], P.xprev[fs[k]], dk);
        dx[0] -= bk[k] * dk[0];
        dx[1] -= bk[k] * dk[1];
        dx[2] -= bk[k] * dk[2];
    }
    V t0 = cloth::sub(q[1], q[0]);
    const R l0 = sqrt(cloth::dot(t0, t0));
    t0 = V{t0.x / l0, t0.y / l0, t0.z / l0};
    V t1 = cloth::cross(t0, n);
    const R l1 = sqrt(cloth::dot(t1, t1));
    t1 = V{t1.x / l1, t1.y / l1, t1.z / l1};
    const R ta[3] = {t0.x, t0.y, t0.z}, tb[3] = {t1.x, t1.y, t1.z};
    const R u0 = ta[0] * dx[0] + ta[1] * dx[1] + ta[2] * dx[2];
    const R u1 = tb[0] * dx[0] + tb[1] * dx[1] + tb[2] * dx[2];
    const double2 fp = P.mesh_fric[P.slot_mesh[sp]], ff = P.mesh_fric[fo.w];
    const R mu = (R(fp.x) + R(ff.x)) * R(0.5);
    const R epsU = (R(fp.y) + R(ff.y)) * R(0.5) * c.dt;
    cloth::friction<R>(mu, lambda, ta, tb, u0, u1, epsU, b, f, H);
}

// accumulateCollisionForceAndHessian (VBDPhysicsCompute.cu:1731-1773) for the vertices
// with contact records in the slot range [beg, end) of one color, evaluated just before
// that color's solve kernel: the vertex's own contact, then its relations, summed into
// its 9 scratch values, which the solve adds between inertia and boundary. Running
// before the color's solve, every read sees the positions of earlier colors updated and
// those of this color not yet, which is the reference's Jacobi-within-color update
// (positionsNew, VBDPhysicsCompute.cu:803-908). `list` holds the slots with records,
// ascending, so a color's vertices are one sub-range.
template <typename ST, typename R>
__global__ void __launch_bounds__(128) k_contact_color(Ptrs<ST, R> P, Consts<R> c, int beg, int end,
                                                       const int32_t* list, const int32_t* nlist) {
    pdl_launch_dependents();
    pdl_wait();
    const int n = *nlist;
    auto lower = [&](int key) {
        int lo = 0, hi = n;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (list[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    const int i0 = lower(beg), i1 = lower(end);
    for (int i = i0 + int(blockIdx.x * blockDim.x + threadIdx.x); i < i1; i += int(gridDim.x * blockDim.x)) {
        const int v = list[i];
        const int info = P.col_info[v];
        R f[3] = {R(0), R(0), R(0)}, H[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
        if (info & 8) contact_term<ST, R>(P, c, v, 3, f, H);
        const int nrel = info & 7;
        for (int j = 0; j < nrel; ++j) {
            const int e = P.col_rel[4 * v + j];
            contact_term<ST, R>(P, c, e >> 2, e & 3, f, H);
        }
        R* o = P.col_scratch + 9 * size_t(v);
        o[0] = f[0]; o[1] = f[1]; o[2] = f[2];
#pragma unroll
        for (int k = 0; k < 6; ++k) o[3 + k] = H[k];
    }
}

// The vertex tail's own inputs (inertia target, start-of-substep state, rest position) into
// L1 while the incidence loop runs: they do not change during a sweep, and loaded only in
// the tail their latency would follow the lane reduction on the critical path.
template <typename ST, typename R>
__device__ __forceinline__ void prefetch_tail(const Ptrs<ST, R>& P, int v) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(P.y + v));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(P.xprev + v));
    asm volatile("prefetch.global.L1 [%0];" ::"l"(P.rest + v));
    if (P.rest_fh) {
        asm volatile("prefetch.global.L1 [%0];" ::"l"(P.rest_fh + v));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(P.rest_fl + v));
    }
}

// How the incidence loop reads neighbour states and records:
//  kStateStream  states through the read-only cache (written by earlier launches only),
//                records streamed (read once per launch);
//  kStateBlock   states with plain loads (written earlier in the same kernel by the same
//                block, ordered by a block barrier), records kept in the caches (read
//                every iteration by the persistent sweeps);
//  kStateGrid    states through L2 only (written earlier in the same kernel by other
//                blocks, ordered by a grid barrier), records kept.
enum StateRead { kStateStream = 0, kStateBlock = 1, kStateGrid = 2 };

// The incidence loop of one lane: records r, r + L, ... below e, the first (`cur`) already
// loaded; two-stage pipeline (the next record is in flight during this incidence).
template <int L, typename ST, typename R, int COHERENT>
__device__ __forceinline__ void accumulate_records(const Ptrs<ST, R>& P, int r, int e, RecRaw<R> cur,
                                                   const typename ST::U& uo_full, R mu, R lmbd, Acc<R>& acc) {
    using U = typename ST::U;
    const U uo = ST::nb(uo_full);
    while (r < e) {
        const int rn = r + L;
        RecRaw<R> nxt;
        if (rn < e) {
            if constexpr (COHERENT != kStateStream) nxt.load_kept(P.rec_n, P.rec_a, P.rec_b, P.rec_c, rn);
            else nxt.load(P.rec_n, P.rec_a, P.rec_b, P.rec_c, rn);
        }
        U q0, q1, q2;
        if constexpr (COHERENT == kStateGrid) {
            q0 = ST::ldcg(P.u, cur.n.x);
            q1 = ST::ldcg(P.u, cur.n.y);
            q2 = ST::ldcg(P.u, cur.n.z);
        } else if constexpr (COHERENT == kStateBlock) {
            q0 = ST::ld(P.u, cur.n.x);
            q1 = ST::ld(P.u, cur.n.y);
            q2 = ST::ld(P.u, cur.n.z);
        } else {
            q0 = ST::ldg(P.u, cur.n.x);
            q1 = ST::ldg(P.u, cur.n.y);
            q2 = ST::ldg(P.u, cur.n.z);
        }
        R m0[3], m1[3], m2[3];
        cur.rows(m0, m1, m2);
        R e0[3], e1[3], e2[3];
        ST::diff(q0, uo, e0);
        ST::diff(q1, uo, e1);
        ST::diff(q2, uo, e2);
        incidence<R>(e0, e1, e2, m0, m1, m2, mu, lmbd, acc);
        cur = nxt;
        r = rn;
    }
}

// Bulk prefetch into L2 (no shared memory, no completion to wait for): addr and bytes
// 16-byte aligned.
__device__ __forceinline__ void bulk_prefetch_l2(const void* addr, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(addr), "r"(bytes) : "memory");
}

// The FP32 records (three 16-byte arrays) of block b of a color launch with blockDim / L
// vertices per block, prefetched into L2: the block that runs one resident wave later then
// finds its record stream in L2, and the DRAM reads run ahead of the warps that consume
// them (a latency-bound sweep keeps more bytes in flight than its warps' registers hold).
template <int L, typename ST, typename R>
__device__ __forceinline__ void prefetch_block_records(const Ptrs<ST, R>& P, int beg, int end, int b) {
    const int vpb = int(blockDim.x) / L;
    const long long v0l = (long long)beg + (long long)b * vpb;
    if (v0l >= end) return;
    const int v0 = int(v0l), v1 = min(end, v0 + vpb);
    const int r0 = P.inc_ofs[v0], r1 = P.inc_ofs[v1];
    if (r1 <= r0) return;
    const uint32_t bytes = uint32_t(r1 - r0) * 16u;
    bulk_prefetch_l2(P.rec_n + r0, bytes);
    bulk_prefetch_l2(P.rec_a + r0, bytes);
    bulk_prefetch_l2(P.rec_b + r0, bytes);
}

// Minimum resident blocks of 256 threads: caps FP32-compute kernels at 64
// registers (32 warps per SM, no spills); the FP64 kernel keeps its registers.
template <typename R>
struct SolveOcc {
    static constexpr int kMinBlocks = sizeof(R) == 8 ? 2 : 4;
};

template <int L, typename ST, typename R, bool PROBE>
__global__ void __launch_bounds__(256, SolveOcc<R>::kMinBlocks)
    k_solve(Ptrs<ST, R> P, Consts<R> c, int beg, int end, int friction, double* probe_out, int pf) {
    using U = typename ST::U;
    using Sc = typename ST::Sc;
    pdl_launch_dependents();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = tid & (L - 1);
    const int v = beg + tid / L;
    const bool valid = v < end;
    Acc<R> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    U uo{};
    MeshMat<R> mat;
    int r = 0, e = 0;
    RecRaw<R> cur;
    // the records of the block pf blocks ahead (one resident wave later) into L2
    if constexpr (sizeof(R) == 4 && !PROBE)
        if (pf > 0 && threadIdx.x == 0) prefetch_block_records<L>(P, beg, end, int(blockIdx.x) + pf);
    // prologue on static data (records, CSR offsets, materials): overlaps the
    // previous color's tail when launched as a programmatic dependent
    if (valid) {
        mat = P.mats[P.slot_mesh[v]];
        r = P.inc_ofs[v] + lane;
        e = P.inc_ofs[v + 1];
        if (r < e) cur.load(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r);
        if (lane == 0 && !PROBE) prefetch_tail(P, v);
    }
    pdl_wait();
    if (valid) {
        uo = P.u[v];
        accumulate_records<L, ST, R, kStateStream>(P, r, e, cur, uo, mat.mu, mat.lmbd, acc);
    }
    reduce_group<L, R>(acc);
    if (!valid || lane != 0) return;
    vertex_tail<ST, R, PROBE>(P, c, v, uo, mat, acc, friction, probe_out, beg, end);
}

// The same incidence loop with two records in flight beyond the one being computed
// (`cur` and `nx1` already loaded): more loads outstanding per lane, for colors whose
// record stream is long enough to need the memory-level parallelism (HBM-bound sweeps).
template <int L, typename ST, typename R>
__device__ __forceinline__ void accumulate_records3(const Ptrs<ST, R>& P, int r, int e, RecRaw<R> cur,
                                                    RecRaw<R> nx1, const typename ST::U& uo_full, R mu, R lmbd,
                                                    Acc<R>& acc) {
    using U = typename ST::U;
    const U uo = ST::nb(uo_full);
    while (r < e) {
        const int r2 = r + 2 * L;
        RecRaw<R> nx2;
        if (r2 < e) nx2.load(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r2);
        const U q0 = ST::ldg(P.u, cur.n.x), q1 = ST::ldg(P.u, cur.n.y), q2 = ST::ldg(P.u, cur.n.z);
        R m0[3], m1[3], m2[3];
        cur.rows(m0, m1, m2);
        R e0[3], e1[3], e2[3];
        ST::diff(q0, uo, e0);
        ST::diff(q1, uo, e1);
        ST::diff(q2, uo, e2);
        incidence<R>(e0, e1, e2, m0, m1, m2, mu, lmbd, acc);
        cur = nx1;
        nx1 = nx2;
        r += L;
    }
}

// k_solve with the deeper record pipeline (variant 4): the prologue loads the first two
// records of each lane before the programmatic-dependency wait. Three resident blocks of
// 256 threads leave it the registers the second record in flight needs (no spills).
template <int L, typename ST, typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 8 ? 2 : 3)
    k_solve_deep(Ptrs<ST, R> P, Consts<R> c, int beg, int end, int friction) {
    using U = typename ST::U;
    pdl_launch_dependents();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = tid & (L - 1);
    const int v = beg + tid / L;
    const bool valid = v < end;
    Acc<R> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    U uo{};
    MeshMat<R> mat;
    int r = 0, e = 0;
    RecRaw<R> cur, nx1;
    if (valid) {
        mat = P.mats[P.slot_mesh[v]];
        r = P.inc_ofs[v] + lane;
        e = P.inc_ofs[v + 1];
        if (r < e) cur.load(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r);
        if (r + L < e) nx1.load(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r + L);
        if (lane == 0) prefetch_tail(P, v);
    }
    pdl_wait();
    if (valid) {
        uo = P.u[v];
        accumulate_records3<L, ST, R>(P, r, e, cur, nx1, uo, mat.mu, mat.lmbd, acc);
    }
    reduce_group<L, R>(acc);
    if (!valid || lane != 0) return;
    vertex_tail<ST, R, false>(P, c, v, uo, mat, acc, friction, nullptr, beg, end);
}

// ---- per-vertex tail (lane 0 of a vertex group): damping, inertia, ground and
// friction, 3x3 solve, update ------------------------------------------------------
// The new state goes to P.u[v], or to *unew when given; returns whether the vertex moved.
template <typename ST, typename R, bool PROBE>
__device__ __forceinline__ bool vertex_tail(const Ptrs<ST, R>& P, const Consts<R>& c, int v, const typename ST::U& uo,
                                            const MeshMat<R>& mat, const Acc<R>& acc, int friction,
                                            double* probe_out, int beg, int end, typename ST::U* unew) {
    using U = typename ST::U;
    using Sc = typename ST::Sc;
    R f[3] = {acc.f0, acc.f1, acc.f2};
    R H[6] = {acc.h00 + acc.S, acc.h01, acc.h02, acc.h11 + acc.S, acc.h12, acc.h22 + acc.S};
    const U xp = P.xprev[v];
    R dx[3];
    ST::diff(uo, xp, dx);
    if (mat.kh > R(0) || mat.kd > R(0)) {
        // damping Hessian (k_h H_lambda + k_d S I) / dt (VBD_NeoHookean.cpp:562-574)
        R D[6] = {mat.kh * acc.h00 + mat.kd * acc.S, mat.kh * acc.h01, mat.kh * acc.h02,
                  mat.kh * acc.h11 + mat.kd * acc.S, mat.kh * acc.h12, mat.kh * acc.h22 + mat.kd * acc.S};
#pragma unroll
        for (int i = 0; i < 6; ++i) D[i] *= c.inv_dt;
        f[0] -= D[0] * dx[0] + D[1] * dx[1] + D[2] * dx[2];
        f[1] -= D[1] * dx[0] + D[3] * dx[1] + D[4] * dx[2];
        f[2] -= D[2] * dx[0] + D[4] * dx[1] + D[5] * dx[2];
#pragma unroll
        for (int i = 0; i < 6; ++i) H[i] += D[i];
    }
    // inertia (VBD_GeneralCompute.h:68-85)
    {
        const U yv = P.y[v];
        R dy[3];
        ST::diff(yv, uo, dy);
        R w = R(ST::mass(uo)) * c.dt2inv;
        f[0] += w * dy[0];
        f[1] += w * dy[1];
        f[2] += w * dy[2];
        H[0] += w; H[3] += w; H[5] += w;
    }
    // tet-mesh contact (between inertia and boundary, VBDPhysicsCompute.cu:893-895),
    // evaluated by k_contact_color just before this color
    if (P.col_info && P.col_info[v]) {
        const R* cs = P.col_scratch + 9 * size_t(v);
        f[0] += cs[0]; f[1] += cs[1]; f[2] += cs[2];
#pragma unroll
        for (int i = 0; i < 6; ++i) H[i] += cs[3 + i];
    }
    // plane ground / world box with friction on each violated axis (VBDPhysics.cpp:2858-2953)
    if (c.plane) {
        // x = X + u, or (X + F) + u in a mesh frame F, X + F held as a float pair per slot
        const bool framed = P.rest_fh != nullptr;
        const float4 X = framed ? P.rest_fh[v] : P.rest[v];
        const float4 Xl = framed ? P.rest_fl[v] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float Xc[3] = {X.x, X.y, X.z}, Xlc[3] = {Xl.x, Xl.y, Xl.z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            // below = lo - x, above = x - hi
            R below = framed ? ST::template sub_plane<R>(pick<Sc>(c.lo[d], c.lo_f[d]), Xc[d], Xlc[d], uo, d)
                             : ST::template sub_from<R>(pick<Sc>(c.lo[d], c.lo_f[d]), Xc[d], uo, d);
            R depth;
            if (below > R(0)) {
                depth = below;
                f[d] += depth * c.kb;
            } else {
                R above = framed ? -ST::template sub_plane<R>(pick<Sc>(c.hi[d], c.hi_f[d]), Xc[d], Xlc[d], uo, d)
                                 : -ST::template sub_from<R>(pick<Sc>(c.hi[d], c.hi_f[d]), Xc[d], uo, d);
                if (!(above > R(0))) continue;
                depth = above;
                f[d] -= depth * c.kb;
            }
            H[d == 0 ? 0 : (d == 1 ? 3 : 5)] += c.kb;
            if (friction) axis_friction<R>(d, dx, c.fr_mu, depth * c.kb, c.fr_epsU, f, H);
        }
    }
    if (PROBE) {
        probe_out[0] = f[0]; probe_out[1] = f[1]; probe_out[2] = f[2];
        probe_out[3] = H[0]; probe_out[4] = H[1]; probe_out[5] = H[2];
        probe_out[6] = H[1]; probe_out[7] = H[3]; probe_out[8] = H[4];
        probe_out[9] = H[2]; probe_out[10] = H[4]; probe_out[11] = H[5];
        return false;
    }
    // CMP_EPSILON2 gate (Types/Types.h:20-21; VBDPhysics.cpp:2432); a non-finite force (a
    // NaN or Inf position among the vertex's neighbours) is counted, as the reference's
    // CPU path stops on a NaN descent direction (VBDPhysics.cpp:2460-2464)
    const R fn2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    if (!(fn2 > R(1e-5f * 1e-5f))) {
        if (!(fn2 <= R(1e-5f * 1e-5f))) atomicAdd(&P.counters[CNT_NONFINITE], 1ull);
        return false;
    }
    R d3[3];
    R step = c.step;
    if (!solve3<R>(H, f, d3, P.counters)) {
        // VBDPhysics.cpp:2452-2458: gradient step along the force
        atomicAdd(&P.counters[CNT_FAILED_SOLVES], 1ull);
        step = c.step_gd;
        d3[0] = f[0]; d3[1] = f[1]; d3[2] = f[2];
    }
    const Sc s0 = Sc(step * d3[0]), s1 = Sc(step * d3[1]), s2 = Sc(step * d3[2]);
    if (!(isfinite(s0) && isfinite(s1) && isfinite(s2))) {
        atomicAdd(&P.counters[CNT_NONFINITE], 1ull);
        return false;
    }
    if (unew) *unew = ST::add(uo, s0, s1, s2);
    else P.u[v] = ST::add(uo, s0, s1, s2);
    return true;
}

// ---------------------------------------------------------------------------
// TMA-staged solve (FP32 compute). Each block owns vpb = blockDim / L
// consecutive vertices of the color; their incidence records are one
// contiguous range [inc_ofs[v0], inc_ofs[v0 + vpb]). Thread 0 stages the range
// into shared memory with three bulk copies (cp.async.bulk, one per record
// array) completing on an mbarrier, issued before the programmatic-dependency
// wait: a block's whole record range is in flight at once, overlapping the
// previous color's tail, at no register cost. Neighbour positions are gathered
// as in k_solve. max_rec bounds the records of any block of this launch (the
// host sizes the dynamic shared memory from it).
// ---------------------------------------------------------------------------
constexpr int kMbarSpinLimit = 1 << 20;
// Polls of the final drain wait of a block whose first wait ran out, each after a 1 us
// sleep: about two seconds in all, far beyond the time any issued copy takes to land.
constexpr int kDrainPolls = 1 << 21;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait on an mbarrier phase: at most `limit` polls; false if the phase did not
// complete within them.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit) {
    for (int i = 0; i < limit; ++i)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// The wait of a block that gave up: the phase completes when every byte its copies
// declared (expect_tx = exactly the bytes issued) has landed, so this waits, bounded and
// with sleeps, until no copy of the block is left writing into its shared memory.
__device__ __forceinline__ bool mbar_drain(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < kDrainPolls; ++i) {
        if (mbar_test(bar, parity)) return true;
        __nanosleep(1000);
    }
    return false;
}

template <int L, typename ST>
__global__ void __launch_bounds__(256, 4)
    k_solve_tma(Ptrs<ST, float> P, Consts<float> c, int beg, int end, int friction, int max_rec) {
    using U = typename ST::U;
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t bar = smem_u32(smem);
    int4* s_n = reinterpret_cast<int4*>(smem + 16);
    float4* s_a = reinterpret_cast<float4*>(smem + 16 + 16 * size_t(max_rec));
    float4* s_b = reinterpret_cast<float4*>(smem + 16 + 32 * size_t(max_rec));
    pdl_launch_dependents();
    const int vpb = blockDim.x / L;
    const int v0 = beg + blockIdx.x * vpb;
    const int v1 = min(end, v0 + vpb);
    const int r0 = P.inc_ofs[v0];
    const int nrec = min(P.inc_ofs[v1] - r0, max_rec);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = uint32_t(nrec) * 16u;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(3u * bytes) : "memory");
        if (bytes) {
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(s_n)),
                "l"(P.rec_n + r0), "r"(bytes), "r"(bar)
                : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(s_a)),
                "l"(P.rec_a + r0), "r"(bytes), "r"(bar)
                : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(s_b)),
                "l"(P.rec_b + r0), "r"(bytes), "r"(bar)
                : "memory");
        }
    }
    const int lane = threadIdx.x & (L - 1);
    const int v = v0 + int(threadIdx.x) / L;
    const bool valid = v < v1;
    MeshMat<float> mat;
    int rb = 0, re = 0;
    if (valid) {
        mat = P.mats[P.slot_mesh[v]];
        rb = P.inc_ofs[v] - r0 + lane;
        re = min(P.inc_ofs[v + 1] - r0, nrec);
        if (lane == 0) prefetch_tail(P, v);
    }
    pdl_wait();
    U uo{};
    if (valid) uo = P.u[v];
    // the block goes on only if every thread saw the records land within the limit
    const bool ok = __syncthreads_and(mbar_wait(bar, 0, c.spin_limit)) != 0;
    Acc<float> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (valid && ok) {
        const U uon = ST::nb(uo);
        for (int r = rb; r < re; r += L) {
            const int4 n = s_n[r];
            const float4 a = s_a[r], b = s_b[r];
            const U q0 = ST::ldg(P.u, n.x), q1 = ST::ldg(P.u, n.y), q2 = ST::ldg(P.u, n.z);
            const float m0[3] = {a.x, a.y, a.z}, m1[3] = {a.w, b.x, b.y}, m2[3] = {b.z, b.w, f_bits(n.w)};
            float e0[3], e1[3], e2[3];
            ST::diff(q0, uon, e0);
            ST::diff(q1, uon, e1);
            ST::diff(q2, uon, e2);
            incidence<float>(e0, e1, e2, m0, m1, m2, mat.mu, mat.lmbd, acc);
        }
    }
    if (!ok) {
        // the records did not land within the limit: the block skips its vertices (none
        // moves) and records it, which the host reports as a device-timeout status; thread
        // 0 then drains the copies so that none is left writing into this block's shared
        // memory after it exits
        if (threadIdx.x == 0) {
            atomicAdd(&P.counters[CNT_TIMEOUT], 1ull);
            if (!mbar_drain(bar, 0)) atomicAdd(&P.counters[CNT_DRAIN], 1ull);
        }
        return;
    }
    reduce_group<L, float>(acc);
    if (!valid || lane != 0) return;
    vertex_tail<ST, float, false>(P, c, v, uo, mat, acc, friction, nullptr, beg, end);
}

// ---------------------------------------------------------------------------
// Persistent scene-major sweep: every iteration of a substep in one launch. Each block
// takes whole scenes (meshes) from a work counter, in the order `scene_order` (largest
// first), and runs all `iterations` of that scene: per iteration its colors in sequence,
// each color's vertices over the block's vertex groups, a block barrier between colors.
// Meshes do not interact (no contact records in this mode), so per mesh the sequence
// of color updates, and every vertex's arithmetic, equal the merged color-major sweep's;
// a scene's records and states stay in the block's L1 / the L2 across its iterations,
// and no launch or device-wide barrier separates colors. Layout: the slots of a mesh
// are contiguous and color-major within it; colors[scene_ofs[m] .. scene_ofs[m + 1])
// are mesh m's color slot ranges in sweep order. MAXB bounds the block size (and so the
// registers a thread may use: 256 leaves the compiler all it needs, 1024 caps it at 64).
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Double-buffered TMA pipeline (FP32 compute). A persistent grid walks the color's tiles
// of vpt = blockDim / L consecutive vertices (tile t of block b: t = b, b + grid, ...). The
// records of a tile are one contiguous range; thread 0 stages the next tile's range into
// the other shared-memory buffer (three cp.async.bulk copies on that buffer's mbarrier)
// while the block computes the current one, so the record stream of the whole color is in
// flight ahead of the warps without occupying their registers. Each lane then prefetches
// the neighbour states of its next incidence (ids from shared memory) before evaluating the
// current one: two incidences' gathers in flight per lane. Bounded waits as in k_solve_tma:
// a block whose wait runs out counts a timeout, drains every copy it issued and returns.
// max_rec bounds the records of any tile (the host sizes the buffers from it).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

template <int L, typename ST>
__global__ void __launch_bounds__(256)
    k_solve_pipe(Ptrs<ST, float> P, Consts<float> c, int beg, int end, int friction, int max_rec) {
    using U = typename ST::U;
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t bar0 = smem_u32(smem);
    const size_t buf_bytes = 48 * size_t(max_rec);
    auto s_n = [&](int b) { return reinterpret_cast<int4*>(smem + 16 + size_t(b) * buf_bytes); };
    auto s_a = [&](int b) { return reinterpret_cast<float4*>(smem + 16 + size_t(b) * buf_bytes + 16 * size_t(max_rec)); };
    auto s_b = [&](int b) { return reinterpret_cast<float4*>(smem + 16 + size_t(b) * buf_bytes + 32 * size_t(max_rec)); };
    const int vpt = int(blockDim.x) / L;
    const int ntiles = (end - beg + vpt - 1) / vpt;
    pdl_launch_dependents();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // thread 0: the records of tile t into buffer b (records are static: no ordering with
    // the previous color needed)
    auto issue = [&](int t, int b) {
        const int v0 = beg + t * vpt, v1 = min(end, v0 + vpt);
        const int r0 = P.inc_ofs[v0];
        const uint32_t bytes = uint32_t(min(P.inc_ofs[v1] - r0, max_rec)) * 16u;
        const uint32_t bar = bar0 + 8u * uint32_t(b);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(3u * bytes) : "memory");
        if (bytes) {
            bulk_g2s(s_n(b), P.rec_n + r0, bytes, bar);
            bulk_g2s(s_a(b), P.rec_a + r0, bytes, bar);
            bulk_g2s(s_b(b), P.rec_b + r0, bytes, bar);
        }
    };
    if (threadIdx.x == 0 && int(blockIdx.x) < ntiles) issue(int(blockIdx.x), 0);
    pdl_wait();
    const int lane = int(threadIdx.x) & (L - 1);
    int k = 0;
    for (int t = int(blockIdx.x); t < ntiles; t += int(gridDim.x), ++k) {
        const int b = k & 1;
        const uint32_t parity = uint32_t(k >> 1) & 1u;
        const int tn = t + int(gridDim.x);
        // the next tile into the other buffer (released by the barrier that ended the last tile)
        if (threadIdx.x == 0 && tn < ntiles) issue(tn, b ^ 1);
        const int v0 = beg + t * vpt, v1 = min(end, v0 + vpt);
        const int r0 = P.inc_ofs[v0];
        const int nrec = min(P.inc_ofs[v1] - r0, max_rec);
        const int v = v0 + int(threadIdx.x) / L;
        const bool valid = v < v1;
        MeshMat<float> mat;
        int rb = 0, re = 0;
        U uo{};
        if (valid) {
            mat = P.mats[P.slot_mesh[v]];
            rb = P.inc_ofs[v] - r0 + lane;
            re = min(P.inc_ofs[v + 1] - r0, nrec);
            if (lane == 0) prefetch_tail(P, v);
            uo = P.u[v];
        }
        const bool ok = __syncthreads_and(mbar_wait(bar0 + 8u * uint32_t(b), parity, c.spin_limit)) != 0;
        if (!ok) {
            // this tile's records did not land within the limit: skip the block's remaining
            // tiles (their vertices do not move), count it, and drain every copy issued (this
            // tile's and, if issued, the next one's) before the block exits
            if (threadIdx.x == 0) {
                atomicAdd(&P.counters[CNT_TIMEOUT], 1ull);
                bool drained = mbar_drain(bar0 + 8u * uint32_t(b), parity);
                if (tn < ntiles) drained = mbar_drain(bar0 + 8u * uint32_t(b ^ 1), uint32_t((k + 1) >> 1) & 1u) && drained;
                if (!drained) atomicAdd(&P.counters[CNT_DRAIN], 1ull);
            }
            return;
        }
        Acc<float> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (valid && rb < re) {
            const int4* sn = s_n(b);
            const float4* sa = s_a(b);
            const float4* sb = s_b(b);
            const U uon = ST::nb(uo);
            int4 n = sn[rb];
            U q0 = ST::ldg(P.u, n.x), q1 = ST::ldg(P.u, n.y), q2 = ST::ldg(P.u, n.z);
            for (int r = rb; r < re; r += L) {
                const int rn = r + L;
                int4 nn = n;
                U p0 = q0, p1 = q1, p2 = q2;
                if (rn < re) {  // the next incidence's gathers in flight during this one
                    nn = sn[rn];
                    p0 = ST::ldg(P.u, nn.x);
                    p1 = ST::ldg(P.u, nn.y);
                    p2 = ST::ldg(P.u, nn.z);
                }
                const float4 a = sa[r], bb = sb[r];
                const float m0[3] = {a.x, a.y, a.z}, m1[3] = {a.w, bb.x, bb.y}, m2[3] = {bb.z, bb.w, f_bits(n.w)};
                float e0[3], e1[3], e2[3];
                ST::diff(q0, uon, e0);
                ST::diff(q1, uon, e1);
                ST::diff(q2, uon, e2);
                incidence<float>(e0, e1, e2, m0, m1, m2, mat.mu, mat.lmbd, acc);
                n = nn;
                q0 = p0;
                q1 = p1;
                q2 = p2;
            }
        }
        reduce_group<L, float>(acc);
        if (valid && lane == 0) vertex_tail<ST, float, false>(P, c, v, uo, mat, acc, friction, nullptr, beg, end);
        __syncthreads();  // every read of buffer b done before the next iteration refills it
    }
}

template <int L, typename ST, typename R, int MAXB>
__global__ void __launch_bounds__(MAXB) k_sweep_scenes(Ptrs<ST, R> P, Consts<R> c, const int2* colors,
                                                       const int32_t* scene_ofs, const int32_t* scene_order,
                                                       int32_t nscenes, int32_t iterations, int32_t friction_start,
                                                       int32_t* work) {
    using U = typename ST::U;
    __shared__ int s_scene;
    const int groups = int(blockDim.x) / L;
    const int g = int(threadIdx.x) / L;
    const int lane = int(threadIdx.x) & (L - 1);
    for (;;) {
        if (threadIdx.x == 0) s_scene = atomicAdd(work, 1);
        __syncthreads();
        const int k = s_scene;
        __syncthreads();  // every thread has read s_scene before it is written again
        if (k >= nscenes) return;
        const int sc = scene_order[k];
        const int c0 = scene_ofs[sc], c1 = scene_ofs[sc + 1];
        for (int it = 0; it < iterations; ++it) {
            const int friction = it >= friction_start ? 1 : 0;
            for (int ci = c0; ci < c1; ++ci) {
                const int2 rg = colors[ci];
                for (int base = rg.x; base < rg.y; base += groups) {
                    const int v = base + g;
                    const bool valid = v < rg.y;
                    Acc<R> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                    U uo{};
                    MeshMat<R> mat;
                    if (valid) {
                        mat = P.mats[P.slot_mesh[v]];
                        const int r = P.inc_ofs[v] + lane, e = P.inc_ofs[v + 1];
                        RecRaw<R> cur;
                        if (r < e) cur.load_kept(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r);
                        if (lane == 0) prefetch_tail(P, v);
                        uo = ST::ld_own(P.u, v);
                        accumulate_records<L, ST, R, kStateBlock>(P, r, e, cur, uo, mat.mu, mat.lmbd, acc);
                    }
                    reduce_group<L, R>(acc);
                    if (valid && lane == 0) vertex_tail<ST, R, false>(P, c, v, uo, mat, acc, friction, nullptr, rg.x, rg.y);
                }
                __syncthreads();  // this color's updates before the next color reads them
            }
        }
    }
}

// Mesh frames, at the start of every substep: per mesh, the FP32 head of its reference
// vertex's state becomes the shift that k_initial_step takes out of every state of the mesh
// (exactly in the double-float modes; the FP32 mode rounds u - s, which is small where the
// mesh moves as a whole), and the frame offset F accumulates it in FP64. A mesh that falls
// or slides as a body then keeps states of the size of its deformation and of one substep's
// motion, and every FP32 difference and update of the solve rounds at that scale instead of
// at the scale of the distance travelled.
template <typename ST>
__global__ void k_frame_update(const typename ST::U* u, const int32_t* ref, double4* F, float4* shift,
                               int32_t nmesh) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmesh) return;
    const int r = ref[m];
    const float4 sh = r >= 0 ? ST::head(u[r]) : make_float4(0.f, 0.f, 0.f, 0.f);
    double4 f = F[m];
    f.x += double(sh.x);
    f.y += double(sh.y);
    f.z += double(sh.z);
    F[m] = f;
    shift[m] = sh;
}

// Initial step of a substep over all slots: VBD_BaseMaterial.h:201-259 and
// VBD_BaseMaterial.cpp:7-31 (initialization types 0..4). Displacements: every
// update is linear in x, so it reads as in positions.
template <typename ST, typename R>
__global__ void k_initial_step(Ptrs<ST, R> P, Consts<R> c) {
    using U = typename ST::U;
    using V = typename ST::V;
    using Sc = typename ST::Sc;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.nslots) return;
    const Sc dt = pick<Sc>(c.dt_d, c.dt_f);
    const int mesh = P.slot_mesh[s];
    U x = P.u[s];
    // mesh frames: the substep starts in the frame moved by this substep's shift (x, and the
    // start-of-substep state, inertia target and initial guess derived from it)
    if (P.frame_shift) {
        const float4 sh = P.frame_shift[mesh];
        x = ST::shift(x, sh.x, sh.y, sh.z);
        // X + F of this slot for the world-box test, as a float pair
        const float4 X = P.rest[s];
        const double4 F = P.frame_F[mesh];
        const double xf[3] = {double(X.x) + F.x, double(X.y) + F.y, double(X.z) + F.z};
        float4 h, l;
        h.x = float(xf[0]); l.x = float(xf[0] - double(h.x));
        h.y = float(xf[1]); l.y = float(xf[1] - double(h.y));
        h.z = float(xf[2]); l.z = float(xf[2] - double(h.z));
        h.w = 0.f; l.w = 0.f;
        P.rest_fh[s] = h;
        P.rest_fl[s] = l;
    }
    V v = P.vel[s];
    P.xprev[s] = x;
    const bool fixed = s >= P.nactive;
    const int init_type = P.mats[mesh].init_type;
    if (init_type == 2 || init_type == 4) P.vprev[s] = v;
    const V vp = v;
    if (c.assoc_grav) {
        v.x += dt * pick<Sc>(c.g[0], c.g_f[0]);
        v.y += dt * pick<Sc>(c.g[1], c.g_f[1]);
        v.z += dt * pick<Sc>(c.g[2], c.g_f[2]);
    }
    if (fixed) { v.x = 0; v.y = 0; v.z = 0; }
    const U yv = ST::add(x, dt * v.x, dt * v.y, dt * v.z);
    P.vel[s] = v;
    P.y[s] = yv;
    U xn;
    switch (init_type) {
        case 1: xn = x; break;
        case 2: xn = ST::add(x, dt * vp.x, dt * vp.y, dt * vp.z); break;
        case 3: xn = ST::add(x, Sc(0.5) * dt * v.x, Sc(0.5) * dt * v.y, Sc(0.5) * dt * v.z); break;
        case 4: {
            const Sc h = Sc(0.5) * dt * dt;
            xn = ST::add(x, dt * vp.x + h * pick<Sc>(c.g[0], c.g_f[0]), dt * vp.y + h * pick<Sc>(c.g[1], c.g_f[1]), dt * vp.z + h * pick<Sc>(c.g[2], c.g_f[2]));
            break;
        }
        default: xn = yv; break;
    }
    P.u[s] = xn;
}

// Deformers (VBD/VBDDeformer.h:45-172). Rotator: p = root + R(theta) rootP with
// theta = omega * t; Translator: p = orig + speed * t. t = time after this substep's
// advance, clamped to the end time. Per selected vertex, in FP64 (a few thousand
// boundary vertices per substep).
template <typename ST>
__global__ void k_deformers(typename ST::U* u, const float4* rest, DeformVerts D, const double* time, double dt) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= D.n) return;
    const DeformerDev d = D.defs[D.def[k]];
    double t = time[0] + dt;
    if (t >= d.end_time && d.end_time > 0) t = d.end_time;
    int s = D.slot[k];
    const float4 X = rest[s];
    const double* a = D.a + 3 * size_t(k);
    double p[3];
    if (d.type == 0) {
        const double* b = D.b + 3 * size_t(k);
        double th = t * d.omega, co = cos(th), si = sin(th), C = 1 - co;
        double ux = d.axis[0], uy = d.axis[1], uz = d.axis[2];
        double Rm[9] = {co + ux * ux * C, ux * uy * C - uz * si, ux * uz * C + uy * si,
                        uy * ux * C + uz * si, co + uy * uy * C, uy * uz * C - ux * si,
                        uz * ux * C - uy * si, uz * uy * C + ux * si, co + uz * uz * C};
        p[0] = a[0] + (Rm[0] * b[0] + Rm[1] * b[1] + Rm[2] * b[2]);
        p[1] = a[1] + (Rm[3] * b[0] + Rm[4] * b[1] + Rm[5] * b[2]);
        p[2] = a[2] + (Rm[6] * b[0] + Rm[7] * b[1] + Rm[8] * b[2]);
    } else {
        p[0] = d.speed[0] * t + a[0];
        p[1] = d.speed[1] * t + a[1];
        p[2] = d.speed[2] * t + a[2];
    }
    double du[3] = {p[0] - double(X.x), p[1] - double(X.y), p[2] - double(X.z)};
    u[s] = ST::from_d(du, ST::mass(u[s]));
}

// Velocity update with the CPU path's damping (VBDPhysics.cpp:2486-2561);
// fixed vertices get zero velocity. Thread 0 advances the substep clock.
template <typename ST, typename R>
__global__ void k_velocity(Ptrs<ST, R> P, Consts<R> c, double* time) {
    using V = typename ST::V;
    using Sc = typename ST::Sc;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) time[0] += c.dt_d;
    if (s >= P.nslots) return;
    V v{0, 0, 0, 0};
    if (s < P.nactive) {
        const Sc dt = pick<Sc>(c.dt_d, c.dt_f);
        Sc d[3];
        ST::diff(P.u[s], P.xprev[s], d);
        v.x = d[0] / dt;
        v.y = d[1] / dt;
        v.z = d[2] / dt;
        const MeshMat<R> mat = P.mats[P.slot_mesh[s]];
        Sc vm = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        if (vm > Sc(1e-6f)) {
            Sc vn = vm * Sc(mat.exp_damp) - Sc(mat.const_damp);
            vn = vn > Sc(1e-6f) ? vn : Sc(0);
            Sc sc = vn / vm;
            v.x *= sc; v.y *= sc; v.z *= sc;
        } else {
            v.x *= Sc(0); v.y *= Sc(0); v.z *= Sc(0);
        }
    }
    P.vel[s] = v;
}

// Chebyshev over-relaxation of the iterate (VBDPhysicsCompute.cu:910-944):
// x = pp + omega (x - pp), then pp = the iterate before this iteration's sweep.
template <typename ST>
__global__ void k_accel_apply(typename ST::U* u, typename ST::U* prevprev, const typename ST::U* prev_iter,
                              int32_t nactive, double omega, const uint8_t* col_info) {
    using Sc = typename ST::Sc;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nactive) return;
    // vertices in contact are not extrapolated (VBDPhysicsCompute.cu:928, activeCollisionMask)
    if (col_info && col_info[s]) {
        prevprev[s] = prev_iter[s];
        return;
    }
    const typename ST::U x = u[s], pp = prevprev[s];
    Sc d[3];
    ST::diff(x, pp, d);
    const Sc om = Sc(omega);
    typename ST::U r = ST::add(pp, om * d[0], om * d[1], om * d[2]);
    r.w = x.w;
    u[s] = r;
    prevprev[s] = prev_iter[s];
}

// FP32 positions for contact detection: xf[s] = X + u (now), xf[nslots + s] = X + xprev
// (start of the substep), each rounded once from FP64.
template <typename ST>
__global__ void k_gather_xf(const typename ST::U* u, const typename ST::U* xprev, const float4* rest, float4* xf,
                            int32_t nslots) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    const float4 X = rest[s];
    double a[3], b[3];
    ST::to_d(u[s], a);
    ST::to_d(xprev[s], b);
    xf[s] = make_float4(float(double(X.x) + a[0]), float(double(X.y) + a[1]), float(double(X.z) + a[2]), 0.f);
    xf[nslots + s] = make_float4(float(double(X.x) + b[0]), float(double(X.y) + b[1]), float(double(X.z) + b[2]), 0.f);
}

// ---------------------------------------------------------------------------
// Host-order state <-> slots (positions = X + u).
// ---------------------------------------------------------------------------
// Mesh frames (frame non-null): positions = X + F[mesh] + u, F per mesh in FP64.
__device__ __forceinline__ double4 frame_of(const double4* frame, const int32_t* slot_mesh, int s) {
    return frame ? frame[slot_mesh[s]] : make_double4(0.0, 0.0, 0.0, 0.0);
}

template <typename ST>
__global__ void k_scatter_state(typename ST::U* u, const float4* rest, typename ST::V* vel, const float* x,
                                const float* v, const int32_t* slot_of, int32_t n, const double4* frame,
                                const int32_t* slot_mesh) {
    using Sc = typename ST::Sc;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = slot_of[i];
    if (x) {
        const float4 X = rest[s];
        const double4 F = frame_of(frame, slot_mesh, s);
        double du[3] = {double(x[3 * size_t(i)]) - double(X.x) - F.x,
                        double(x[3 * size_t(i) + 1]) - double(X.y) - F.y,
                        double(x[3 * size_t(i) + 2]) - double(X.z) - F.z};
        u[s] = ST::from_d(du, ST::mass(u[s]));
    }
    if (v) {
        typename ST::V w{Sc(v[3 * size_t(i)]), Sc(v[3 * size_t(i) + 1]), Sc(v[3 * size_t(i) + 2]), Sc(0)};
        vel[s] = w;
    }
}

template <typename ST>
__global__ void k_gather_positions(const typename ST::U* u, const float4* rest, float* out32, double* out64,
                                   const int32_t* slot_of, int32_t n, const double4* frame,
                                   const int32_t* slot_mesh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = slot_of[i];
    double p[3];
    ST::to_d(u[s], p);
    const float4 X = rest[s];
    const double4 F = frame_of(frame, slot_mesh, s);
    p[0] += double(X.x) + F.x;
    p[1] += double(X.y) + F.y;
    p[2] += double(X.z) + F.z;
    if (out32) {
        out32[3 * size_t(i)] = float(p[0]);
        out32[3 * size_t(i) + 1] = float(p[1]);
        out32[3 * size_t(i) + 2] = float(p[2]);
    } else {
        out64[3 * size_t(i)] = p[0];
        out64[3 * size_t(i) + 1] = p[1];
        out64[3 * size_t(i) + 2] = p[2];
    }
}

template <typename V>
__global__ void k_gather_velocities(const V* vel, float* out32, double* out64, const int32_t* slot_of, int32_t n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V v = vel[slot_of[i]];
    if (out32) {
        out32[3 * size_t(i)] = float(v.x);
        out32[3 * size_t(i) + 1] = float(v.y);
        out32[3 * size_t(i) + 2] = float(v.z);
    } else {
        out64[3 * size_t(i)] = double(v.x);
        out64[3 * size_t(i) + 1] = double(v.y);
        out64[3 * size_t(i) + 2] = double(v.z);
    }
}

template <typename ST>
__global__ void k_scatter_positions_f64(typename ST::U* u, const float4* rest, const double* in,
                                        const int32_t* slot_of, int32_t n, const double4* frame,
                                        const int32_t* slot_mesh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = slot_of[i];
    const float4 X = rest[s];
    const double4 F = frame_of(frame, slot_mesh, s);
    double du[3] = {in[3 * size_t(i)] - double(X.x) - F.x, in[3 * size_t(i) + 1] - double(X.y) - F.y,
                    in[3 * size_t(i) + 2] - double(X.z) - F.z};
    u[s] = ST::from_d(du, ST::mass(u[s]));
}

template <typename ST>
__global__ void k_scatter_velocities_f64(typename ST::V* vel, const double* in, const int32_t* slot_of, int32_t n) {
    using Sc = typename ST::Sc;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vel[slot_of[i]] = typename ST::V{Sc(in[3 * size_t(i)]), Sc(in[3 * size_t(i) + 1]), Sc(in[3 * size_t(i) + 2]), Sc(0)};
}

}  // namespace dev
}  // namespace gaia
