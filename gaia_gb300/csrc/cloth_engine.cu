// GB300 cloth VBD step: per-color block solve of the StVK membrane, quadratic
// bending, inertia, world-box contact and the vertex-face / edge-edge contact
// energies with lagged friction; conservative-bound step truncation; GPU
// contact detection (cloth_cd.cu) re-run inside the iteration loop whenever a
// vertex left its bound; the whole substep captured in one CUDA graph.
//
// Step semantics follow VBDClothSimulationFramework::runStep_CDEveryIter
// (VBDCloth/VBDClothPhysics.cpp:389-518):
//   per iteration: [detection if required or first iteration] -> [initial
//   guess on the first iteration] -> per merged color: solve every vertex of the
//   color into x_next from the current positions, then commit (the reference's
//   vertexPositionNext copy, VBDClothPhysics.cpp:480-492) -> [Chebyshev step];
//   then the velocity update.
// The per-vertex solve is VBDStepWithExistingCollisions (VBDClothPhysics.cpp:1026-1154).
//
// Layout in HBM: all meshes' vertices concatenated (simulated meshes first,
// then colliders), positions as 4-component vectors (FP32 or FP64), incidence
// lists per simulated vertex (faces with the vertex's order, edges, bending
// stencils) as CSR int2 arrays, per-face DmInv (2x2) and area, per-edge 4x4
// bending form. The detector reads a float4 copy of the positions taken at the
// last detection (the reference's positionsAtPrevCollisionDetection).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "cloth_cd.hpp"
#include "cloth_dev.cuh"
#include "cloth_scene.hpp"
#include "gaia_cloth.h"
#include "scene.hpp"
#include "state_io.hpp"
#include "vbd_kernels.cuh"

namespace gaia {
void set_last_global_error(const std::string& msg);

namespace cloth {
namespace {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define CL_CUDA(call)                                                                                    \
    do {                                                                                                 \
        cudaError_t e__ = (call);                                                                        \
        if (e__ != cudaSuccess)                                                                          \
            throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e__) + " (" + __FILE__ + ":" + \
                            std::to_string(__LINE__) + ")");                                             \
    } while (0)

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    Buf() = default;
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    ~Buf() {
        if (p) cudaFree(p);
    }
    void alloc(size_t count, size_t* total) {
        if (p) cudaFree(p);
        p = nullptr;
        n = count;
        CL_CUDA(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
        if (total) *total += std::max<size_t>(count, 1) * sizeof(T);
    }
    void upload(const std::vector<T>& h, size_t* total, cudaStream_t st) {
        alloc(h.size(), total);
        if (!h.empty()) CL_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    }
};

inline int nblk(int64_t n, int b) { return int((n + b - 1) / b); }

}  // namespace

template <typename R>
struct alignas(4 * sizeof(R)) P4 {
    R x, y, z, w;
};
template <typename R>
struct Vec;
template <>
struct Vec<float> {
    using T = float3;
};
template <>
struct Vec<double> {
    using T = double3;
};

template <typename R>
struct ClothMat {
    R miu, lambda, dampStVK, dampBend, kBend, fricMu, fricEps, expDamp, constDamp, maxVel, noGravThr;
    int hasNoGrav, initType, pad;
};

template <typename R>
struct Consts {
    R dt, dtSqrRecip, stepSize, g[3], lo[3], hi[3], kb, muB, epsUB, kc, rc, thick, degThr2, relax, maxQ;
    int nSimV, nV, assocGrav, handleCollision;
};

template <typename R>
struct Args {
    P4<R>* x;
    P4<R>* xprev;
    P4<R>* y;
    P4<R>* xnext;
    // low halves of the double-float state (position = x + xlo, ...): null unless the
    // FP32 engine keeps double-float positions
    P4<float>* xlo;
    P4<float>* xprevlo;
    P4<float>* ylo;
    P4<float>* xnextlo;
    P4<R>* xcd;
    P4<R>* v;
    P4<R>* vprev;
    P4<R>* accel;
    P4<R>* xPrevIter;
    const P4<R>* xrest;      // rest positions (the loaded, transformed mesh)
    R* bound;
    const R* mass;
    const uint8_t* fixed;
    uint8_t* active;
    const int2* vInfo;
    const ClothMat<R>* mats;
    const int4* faces;
    const int4* edges;
    const int* vfOfs;
    const int2* vfList;
    const int* veOfs;
    const int2* veList;
    const int* vbOfs;
    const int2* vbList;
    const P4<R>* faceDmInv;  // (m00, m10, m01, m11) column-major
    const R* faceArea;
    const R* bendQ;          // 16 per edge, row-major
    float4* xf;
    CDOut cd;
    int* req;
    int* state;              // [0] = completed initial steps
    unsigned long long* counters;
};

namespace kern {

template <typename R>
__device__ __forceinline__ typename Vec<R>::T ld(const P4<R>* p, int i) {
    const P4<R> q = p[i];
    return typename Vec<R>::T{q.x, q.y, q.z};
}
template <typename R>
__device__ __forceinline__ void st(P4<R>* p, int i, typename Vec<R>::T v) {
    p[i] = P4<R>{v.x, v.y, v.z, R(0)};
}

// Where a solving vertex's terms take positions from. OrgAbs: the stored coordinates as they
// are (the FP32 and FP64 engines). OrgRel (the double-float state): every position relative
// to the vertex's own, (hi_i - hi_o) + (lo_i - lo_o), so the FP32 arithmetic works on the
// distances between nearby vertices with the digits of the double-float positions (all
// terms are translation invariant; the world box takes the absolute position from the
// origin).
template <typename R>
struct OrgAbs {
    static constexpr bool kRel = false;
};
template <typename R>
struct OrgRel {
    static constexpr bool kRel = true;
    typename Vec<R>::T h;  // the vertex's position: high half
    float lx, ly, lz;      // and low half
};
template <typename O, typename R>
__device__ __forceinline__ O origin(const Args<R>& a, int v) {
    O o{};
    if constexpr (O::kRel) {
        o.h = ld(a.x, v);
        const P4<float> q = a.xlo[v];
        o.lx = q.x;
        o.ly = q.y;
        o.lz = q.z;
    }
    return o;
}
// position i of the array (hi, lo) as the terms take it; an array without a low half (the
// detection snapshot) is taken as exact in its high half
template <typename R>
__device__ __forceinline__ typename Vec<R>::T rel(const P4<R>* hi, const P4<float>*, int i, const OrgAbs<R>&) {
    return ld(hi, i);
}
template <typename R>
__device__ __forceinline__ typename Vec<R>::T rel(const P4<R>* hi, const P4<float>* lo, int i, const OrgRel<R>& o) {
    const P4<R> p = hi[i];
    typename Vec<R>::T d{p.x - o.h.x, p.y - o.h.y, p.z - o.h.z};
    const float qx = lo ? lo[i].x : 0.f, qy = lo ? lo[i].y : 0.f, qz = lo ? lo[i].z : 0.f;
    d.x += R(qx - o.lx);
    d.y += R(qy - o.ly);
    d.z += R(qz - o.lz);
    return d;
}
template <typename V, typename R>
__device__ __forceinline__ V normalized(V a) {
    const R nn = dot(a, a);
    return nn > R(0) ? mul(R(1) / sqrt(nn), a) : a;
}
template <typename R>
__device__ __forceinline__ void add_outer(R* H, R s, R nx, R ny, R nz) {
    H[0] += s * nx * nx;
    H[1] += s * nx * ny;
    H[2] += s * nx * nz;
    H[3] += s * ny * ny;
    H[4] += s * ny * nz;
    H[5] += s * nz * nz;
}

// One vertex-face contact seen from vertex order `order` (3 = the vertex side, 0..2 =
// a face vertex): accumulateVFContactForceAndHessian (VBDClothPhysics.cpp:1248-1321) with
// the closest point recomputed from the current positions (updateVFContactPointInfo).
// The face's vertex ids and positions come in already loaded (the face-side loop loads them
// once per face).
template <typename R, typename O>
__device__ void vf_term_at(const Args<R>& a, const Consts<R>& c, const O& o, int u, int4 fv,
                           typename Vec<R>::T A, typename Vec<R>::T B, typename Vec<R>::T C, int order, R* f, R* H) {
    using V = typename Vec<R>::T;
    const V xu = rel(a.x, a.xlo, u, o);
    V bary, cp;
    closest_point_triangle<V, R>(xu, A, B, C, bary, cp);
    const V diff = sub(xu, cp);
    const V n = normalized<V, R>(diff);
    const R dis = dot(diff, n);
    if (!(dis < c.rc + c.thick)) return;
    const R b = order == 3 ? R(1) : -(order == 0 ? bary.x : (order == 1 ? bary.y : bary.z));
    R dEdD, d2E;
    contact_repulsion<R>(dis, c.thick, c.rc, c.kc, dEdD, d2E);
    const R lambda = -dEdD;
    f[0] += b * lambda * n.x;
    f[1] += b * lambda * n.y;
    f[2] += b * lambda * n.z;
    add_outer(H, d2E * b * b, n.x, n.y, n.z);
    const V dx3 = sub(xu, rel(a.xprev, a.xprevlo, u, o));
    const V cprev = add(add(mul(bary.x, rel(a.xprev, a.xprevlo, fv.x, o)), mul(bary.y, rel(a.xprev, a.xprevlo, fv.y, o))),
                        mul(bary.z, rel(a.xprev, a.xprevlo, fv.z, o)));
    const V dx = sub(dx3, sub(cp, cprev));
    const V e0 = normalized<V, R>(sub(B, A));
    const V e1 = normalized<V, R>(cross(e0, n));
    const ClothMat<R>& mf = a.mats[a.vInfo[fv.x].x];
    const ClothMat<R>& mu_ = a.mats[a.vInfo[u].x];
    const R mu = (mf.fricMu + mu_.fricMu) * R(0.5);
    const R epsU = (mf.fricEps + mu_.fricEps) * R(0.5) * c.dt;
    const R t0[3] = {e0.x, e0.y, e0.z}, t1[3] = {e1.x, e1.y, e1.z};
    friction<R>(mu, lambda, t0, t1, dot(e0, dx), dot(e1, dx), epsU, b, f, H);
}

template <typename R, typename O>
__device__ __forceinline__ void vf_term(const Args<R>& a, const Consts<R>& c, const O& o, int u, int face, int order,
                                        R* f, R* H) {
    const int4 fv = a.faces[face];
    vf_term_at(a, c, o, u, fv, rel(a.x, a.xlo, fv.x, o), rel(a.x, a.xlo, fv.y, o), rel(a.x, a.xlo, fv.z, o), order, f,
               H);
}

// One edge-edge contact of edge e (this vertex has order 0/1 on it) with edge e2:
// accumulateEEContactForceAndHessian (VBDClothPhysics.cpp:1323-1399). Edge e's vertex ids
// and positions come in already loaded (the edge loop loads them once per edge).
template <typename R, typename O>
__device__ void ee_term_at(const Args<R>& a, const Consts<R>& c, const O& o, int4 E, typename Vec<R>::T p1,
                           typename Vec<R>::T p2, int e2, int order, R* f, R* H) {
    using V = typename Vec<R>::T;
    const int4 F = a.edges[e2];
    const V q1 = rel(a.x, a.xlo, F.x, o), q2 = rel(a.x, a.xlo, F.y, o);
    V c1, c2;
    R s, t;
    closest_points_segments(p1, p2, q1, q2, c1, c2, s, t);
    const V diff = sub(c1, c2);
    const R dis = sqrt(dot(diff, diff));
    const V v1 = sub(p2, p1), v2 = sub(q2, q1);
    const V cr = cross(v1, v2);
    const R par = dot(cr, cr) / (sqrt(dot(v1, v1)) * sqrt(dot(v2, v2)));
    if (!(dis < c.rc + c.thick && par > R(CMP_EPS))) return;
    const V n = mul(R(1) / dis, diff);
    const R b = order == 0 ? R(1) - s : (order == 1 ? s : (order == 2 ? R(-1) + t : -t));
    R dEdD, d2E;
    contact_repulsion<R>(dis, c.thick, c.rc, c.kc, dEdD, d2E);
    const R lambda = -dEdD;
    f[0] += b * lambda * n.x;
    f[1] += b * lambda * n.y;
    f[2] += b * lambda * n.z;
    add_outer(H, d2E * b * b, n.x, n.y, n.z);
    const V c1p = add(mul(R(1) - s, rel(a.xprev, a.xprevlo, E.x, o)), mul(s, rel(a.xprev, a.xprevlo, E.y, o)));
    const V c2p = add(mul(R(1) - t, rel(a.xprev, a.xprevlo, F.x, o)), mul(t, rel(a.xprev, a.xprevlo, F.y, o)));
    const V dx = sub(sub(c1, c1p), sub(c2, c2p));
    const V e0 = normalized<V, R>(v1);
    const V e1 = normalized<V, R>(cross(e0, n));
    const ClothMat<R>& m1 = a.mats[a.vInfo[E.x].x];
    const ClothMat<R>& m2 = a.mats[a.vInfo[F.x].x];
    const R mu = (m1.fricMu + m2.fricMu) * R(0.5);
    const R epsU = (m1.fricEps + m2.fricEps) * R(0.5) * c.dt;
    const R t0[3] = {e0.x, e0.y, e0.z}, t1[3] = {e1.x, e1.y, e1.z};
    friction<R>(mu, lambda, t0, t1, dot(e0, dx), dot(e1, dx), epsU, b, f, H);
}

template <typename R>
__device__ __forceinline__ bool solve_block(const R* H, const R* b, R* x, unsigned long long* counters);
template <>
__device__ __forceinline__ bool solve_block<float>(const float* H, const float* b, float* x,
                                                   unsigned long long* counters) {
    if (gaia::dev::ldlt3<float>(H, b, x, gaia::dev::kFp32Pivot)) return true;
    double Hd[6], bd[3], xd[3];
    for (int i = 0; i < 6; ++i) Hd[i] = H[i];
    for (int i = 0; i < 3; ++i) bd[i] = b[i];
    atomicAdd(&counters[CC_FP64_SOLVES], 1ull);
    if (!gaia::dev::ldlt3<double>(Hd, bd, xd, gaia::dev::kRetryPivot)) return false;
    for (int i = 0; i < 3; ++i) x[i] = float(xd[i]);
    return true;
}
template <>
__device__ __forceinline__ bool solve_block<double>(const double* H, const double* b, double* x,
                                                    unsigned long long*) {
    return gaia::dev::ldlt3<double>(H, b, x, gaia::dev::kFp64Pivot);
}

// StVK membrane of one incident face: with F = [f0 f1] = Ds DmInv, G = (F^T F - I) / 2,
// S = 2 mu G + lambda tr(G) I and m the vertex's row of dF/dx:
//   force -= A F S m,  H += A [ (m^T S m) I + mu |m|^2 F F^T + (mu + lambda) (F m)(F m)^T ]
// which equals the reference's 6x6 d2W/dF2 contracted with m (accumlateStVKForceAndHessian,
// VBDTriMeshStVK.cpp:721-911, and assembleMembraneHessian, VBDBaseTriMesh.h:149-160).
// The strain is formed from displacements u = x - X: with Ds = Dr + dU (Dr the rest edges,
// Dr^T Dr = Dm^T Dm), G = DmInv^T (Dr^T dU + dU^T Dr + dU^T dU) DmInv / 2, so FP32 keeps
// the strain's own digits instead of those of F^T F - I.
template <typename R, typename O>
__device__ __forceinline__ void membrane(const Args<R>& a, const O& o, const ClothMat<R>& mat, int2 fo, R* f,
                                         R* Hm) {
    using V = typename Vec<R>::T;
    const int4 fv = a.faces[fo.x];
    const V x0 = rel(a.x, a.xlo, fv.x, o), x1 = rel(a.x, a.xlo, fv.y, o), x2 = rel(a.x, a.xlo, fv.z, o);
    const V X0 = ld(a.xrest, fv.x), X1 = ld(a.xrest, fv.y), X2 = ld(a.xrest, fv.z);
    const V e1 = sub(X1, X0), e2 = sub(X2, X0);  // rest edges
    V w1, w2;                                      // edge displacements
    if constexpr (O::kRel) {  // positions relative to the solving vertex: edge vectors minus rest edges
        w1 = sub(sub(x1, x0), e1);
        w2 = sub(sub(x2, x0), e2);
    } else {  // coordinates: displacements from the rest positions
        const V u0 = sub(x0, X0);
        w1 = sub(sub(x1, X1), u0);
        w2 = sub(sub(x2, X2), u0);
    }
    const P4<R> D = a.faceDmInv[fo.x];  // m00 m10 m01 m11
    const V d1 = add(e1, w1), d2 = add(e2, w2);
    const V f0 = add(mul(D.x, d1), mul(D.y, d2));
    const V f1 = add(mul(D.z, d1), mul(D.w, d2));
    // M = Dr^T dU + dU^T Dr + dU^T dU (2x2 symmetric)
    const R M00 = R(2) * dot(e1, w1) + dot(w1, w1);
    const R M11 = R(2) * dot(e2, w2) + dot(w2, w2);
    const R M01 = dot(e1, w2) + dot(w1, e2) + dot(w1, w2);
    // G = DmInv^T M DmInv / 2
    const R a0 = M00 * D.x + M01 * D.y, a1 = M01 * D.x + M11 * D.y;  // M * col0(DmInv)
    const R b0 = M00 * D.z + M01 * D.w, b1 = M01 * D.z + M11 * D.w;  // M * col1(DmInv)
    const R G00 = R(0.5) * (D.x * a0 + D.y * a1), G11 = R(0.5) * (D.z * b0 + D.w * b1);
    const R G01 = R(0.5) * (D.x * b0 + D.y * b1);
    const R tr = G00 + G11;
    const R S00 = R(2) * mat.miu * G00 + mat.lambda * tr, S11 = R(2) * mat.miu * G11 + mat.lambda * tr;
    const R S01 = R(2) * mat.miu * G01;
    R m1, m2;
    if (fo.y == 0) {
        m1 = -D.x - D.y;
        m2 = -D.z - D.w;
    } else if (fo.y == 1) {
        m1 = D.x;
        m2 = D.z;
    } else {
        m1 = D.y;
        m2 = D.w;
    }
    const R A = a.faceArea[fo.x];
    const R Sm0 = S00 * m1 + S01 * m2, Sm1 = S01 * m1 + S11 * m2;
    const V P = add(mul(Sm0, f0), mul(Sm1, f1));
    f[0] -= A * P.x;
    f[1] -= A * P.y;
    f[2] -= A * P.z;
    const R mSm = m1 * Sm0 + m2 * Sm1;
    const R mm = m1 * m1 + m2 * m2;
    const V g = add(mul(m1, f0), mul(m2, f1));
    const R kF = A * mat.miu * mm, kg = A * (mat.miu + mat.lambda);
    Hm[0] += A * mSm + kF * (f0.x * f0.x + f1.x * f1.x) + kg * g.x * g.x;
    Hm[1] += kF * (f0.x * f0.y + f1.x * f1.y) + kg * g.x * g.y;
    Hm[2] += kF * (f0.x * f0.z + f1.x * f1.z) + kg * g.x * g.z;
    Hm[3] += A * mSm + kF * (f0.y * f0.y + f1.y * f1.y) + kg * g.y * g.y;
    Hm[4] += kF * (f0.y * f0.z + f1.y * f1.z) + kg * g.y * g.z;
    Hm[5] += A * mSm + kF * (f0.z * f0.z + f1.z * f1.z) + kg * g.z * g.z;
}

// Quadratic bending of one stencil (accumlateBendingForceAndHessian,
// VBDTriMeshStVK.cpp:913-982): E = k/2 X^T Q X over its 4 vertices, Rayleigh damping.
template <typename R, typename O>
__device__ __forceinline__ void bending(const Args<R>& a, const Consts<R>& c, const O& o, const ClothMat<R>& mat,
                                        typename Vec<R>::T x, typename Vec<R>::T xp, int2 eo, R* f, R* H) {
    using V = typename Vec<R>::T;
    const int4 E = a.edges[eo.x];
    const V X0 = rel(a.x, a.xlo, E.x, o), X1 = rel(a.x, a.xlo, E.y, o), X2 = rel(a.x, a.xlo, E.z, o),
            X3 = rel(a.x, a.xlo, E.w, o);
    const V n1 = cross(sub(X1, X0), sub(X2, X0));
    const V n2 = cross(sub(X2, X3), sub(X1, X3));
    if (dot(n1, n1) < c.degThr2 || dot(n2, n2) < c.degThr2) return;
    const R db = mat.dampBend / c.dt;
    const R* Q = a.bendQ + size_t(eo.x) * 16 + 4 * eo.y;
    const V gr = add(add(mul(Q[0], X0), mul(Q[1], X1)), add(mul(Q[2], X2), mul(Q[3], X3)));
    const R hq = mat.kBend * Q[eo.y];
    f[0] -= mat.kBend * gr.x + hq * (x.x - xp.x) * db;
    f[1] -= mat.kBend * gr.y + hq * (x.y - xp.y) * db;
    f[2] -= mat.kBend * gr.z + hq * (x.z - xp.z) * db;
    const R hb = hq * (R(1) + db);
    H[0] += hb;
    H[3] += hb;
    H[5] += hb;
}

// The flattened face-side (faces = 1: items of the incident faces' FV links) or edge
// (faces = 0: items of the incident edges' EE contacts) contact terms of one lane: items
// lane, lane + L, ... of the concatenation, in order.
template <int L, typename R, int CAP, typename O>
__device__ __forceinline__ void flat_items(const Args<R>& a, const Consts<R>& c, const O& org, int lane,
                                           const int2* list, int n, const int* counts, int faces, R* f, R* H) {
    using V = typename Vec<R>::T;
    int i = -1, first = 0, cnt = 0;  // current primitive, its first flattened item, its item count
    int4 ids = make_int4(0, 0, 0, 0);
    V A{}, B{}, C{};
    int2 o = make_int2(0, 0);
    for (int k = lane;; k += L) {
        while (k >= first + cnt) {  // advance to the primitive holding item k
            first += cnt;
            if (++i >= n) return;
            o = list[i];
            cnt = min(counts[o.x], CAP);
            if (k < first + cnt) {
                if (faces) {
                    ids = a.faces[o.x];
                    A = rel(a.x, a.xlo, ids.x, org);
                    B = rel(a.x, a.xlo, ids.y, org);
                    C = rel(a.x, a.xlo, ids.z, org);
                } else {
                    ids = a.edges[o.x];
                    A = rel(a.x, a.xlo, ids.x, org);
                    B = rel(a.x, a.xlo, ids.y, org);
                }
            }
        }
        const int j = k - first;
        if (faces) vf_term_at(a, c, org, a.cd.fvVert[size_t(o.x) * CAP + j], ids, A, B, C, o.y, f, H);
        else ee_term_at(a, c, org, ids, A, B, a.cd.eeOther[size_t(o.x) * CAP + j], o.y, f, H);
    }
}

// Lane `lane` of an L-lane group's share of vertex v's incident terms: membrane (into Hm,
// for the Rayleigh term), bending, vertex-side VF contacts, face-side VF contacts (the
// vertices linked to each incident face, flattened over faces) and EE contacts (flattened
// over the incident edges). Within each kind, lane k takes items k, k + L, ...
template <int L, typename R, typename O>
__device__ __forceinline__ void partial(const Args<R>& a, const Consts<R>& c, const O& o, const ClothMat<R>& mat,
                                        int v, int lane, typename Vec<R>::T x, typename Vec<R>::T xp, R* f, R* H,
                                        R* Hm) {
    const int fa = a.vfOfs[v], nF = a.vfOfs[v + 1] - fa;
    const int ba = a.vbOfs[v], nB = mat.kBend != R(0) ? a.vbOfs[v + 1] - ba : 0;
    const int nVF = min(a.cd.vfCount[v], VF_CAP);
    // one loop per kind of item, so that the lanes of a warp run the same code together
    for (int k = lane; k < nF; k += L) membrane(a, o, mat, a.vfList[fa + k], f, Hm);
    for (int k = lane; k < nB; k += L) bending(a, c, o, mat, x, xp, a.vbList[ba + k], f, H);
    for (int k = lane; k < nVF; k += L) vf_term(a, c, o, v, a.cd.vfFace[size_t(v) * VF_CAP + k], 3, f, H);
    // Face side: items (incident face i, link j) in face order; edges: items (incident edge
    // i, contact j) in edge order. Lane `lane` takes the items whose flattened index is
    // lane, lane + L, ..., so every lane of the group has work until the last L items
    // (a face or an edge holds fewer items than a wide group has lanes, and a loop over the
    // faces would leave the other lanes idle). The face (edge) of each item follows from the
    // prefix of the item counts, which a lane walks forward as its index grows; the face's
    // (edge's) ids and positions are loaded again only when the lane's face (edge) changes.
    flat_items<L, R, FV_CAP>(a, c, o, lane, a.vfList + fa, nF, a.cd.fvCount, 1, f, H);
    flat_items<L, R, EE_CAP>(a, c, o, lane, a.veList + a.veOfs[v], a.veOfs[v + 1] - a.veOfs[v], a.cd.eeCount, 0, f,
                             H);
}

// Per-vertex terms: the membrane's Rayleigh damping on its own Hessian, inertia
// (VBDBaseTriMesh.cpp:316-323) and the world box (accumlateBoundaryForceAndHessian,
// VBDClothPhysics.cpp:1401-1463).
template <typename R, typename O>
__device__ __forceinline__ void vertex_terms(const Args<R>& a, const Consts<R>& c, const O& o,
                                             const ClothMat<R>& mat, int v, typename Vec<R>::T x, typename Vec<R>::T xp,
                                             R* f, R* H, const R* Hm) {
    using V = typename Vec<R>::T;
    const R dmp = mat.dampStVK / c.dt;
    const V du = sub(x, xp);
    f[0] -= dmp * (Hm[0] * du.x + Hm[1] * du.y + Hm[2] * du.z);
    f[1] -= dmp * (Hm[1] * du.x + Hm[3] * du.y + Hm[4] * du.z);
    f[2] -= dmp * (Hm[2] * du.x + Hm[4] * du.y + Hm[5] * du.z);
    for (int k = 0; k < 6; ++k) H[k] += Hm[k] * (R(1) + dmp);
    const R mh = a.mass[v] * c.dtSqrRecip;
    const V yv = rel(a.y, a.ylo, v, o);
    f[0] += mh * (yv.x - x.x);
    f[1] += mh * (yv.y - x.y);
    f[2] += mh * (yv.z - x.z);
    H[0] += mh;
    H[3] += mh;
    H[5] += mh;
    // the world box on the absolute position (relative terms: the origin, high and low half,
    // plus x)
    R xs[3] = {x.x, x.y, x.z}, xl[3] = {R(0), R(0), R(0)};
    if constexpr (O::kRel) {
        xs[0] = o.h.x + x.x;
        xs[1] = o.h.y + x.y;
        xs[2] = o.h.z + x.z;
        xl[0] = R(o.lx);
        xl[1] = R(o.ly);
        xl[2] = R(o.lz);
    }
    const R dxs[3] = {x.x - xp.x, x.y - xp.y, x.z - xp.z};
    const int diag[3] = {0, 3, 5};
    for (int d = 0; d < 3; ++d) {
        R pen;
        const R below = (c.lo[d] - xs[d]) - xl[d], above = (xs[d] - c.hi[d]) + xl[d];
        if (below > R(0)) {
            pen = below;
            f[d] += pen * c.kb;
        } else if (above > R(0)) {
            pen = above;
            f[d] -= pen * c.kb;
        } else {
            continue;
        }
        H[diag[d]] += c.kb;
        R t0[3] = {0, 0, 0}, t1[3] = {0, 0, 0};
        const int a1 = (d + 1) % 3, a2 = (d + 2) % 3;
        t0[a1] = R(1);
        t1[a2] = R(1);
        friction<R>(c.muB, pen * c.kb, t0, t1, dxs[a1], dxs[a2], c.epsUB, R(1), f, H);
    }
}

// Sum over the L lanes of a group (L divides 32; groups are aligned in the warp).
template <int L, typename R>
__device__ __forceinline__ void group_sum(R* v, int n, unsigned mask) {
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1)
        for (int k = 0; k < n; ++k) v[k] += __shfl_xor_sync(mask, v[k], off, L);
}

// Force and Hessian (sym 00 01 02 11 12 22) of vertex v at the current positions
// (one thread): VBDStepWithExistingCollisions up to its solve.
template <typename R, typename O>
__device__ void accumulate(const Args<R>& a, const Consts<R>& c, int v, R* f, R* H) {
    using V = typename Vec<R>::T;
    const O o = origin<O>(a, v);
    const V x = rel(a.x, a.xlo, v, o), xp = rel(a.xprev, a.xprevlo, v, o);
    const ClothMat<R> mat = a.mats[a.vInfo[v].x];
    R Hm[6] = {0, 0, 0, 0, 0, 0};
    partial<1, R, O>(a, c, o, mat, v, 0, x, xp, f, H, Hm);
    vertex_terms(a, c, o, mat, v, x, xp, f, H, Hm);
}

// The block solve of the vertices of one color, L lanes per vertex:
// VBDStepWithExistingCollisions (VBDClothPhysics.cpp:1026-1154) with the conservative
// bound truncation (applyConservativeBoundTruncation, :1223-1246). Writes x_next.
template <int L, typename R, typename O>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 6 : 1) k_solve(Args<R> a, Consts<R> c, const int* verts, int n) {
    using V = typename Vec<R>::T;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gid / L, lane = gid % L;
    if (i >= n) return;
    const int v = verts[i];
    if (a.fixed[v]) return;
    const unsigned mask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
    const O o = origin<O>(a, v);
    const V x = rel(a.x, a.xlo, v, o), xp = rel(a.xprev, a.xprevlo, v, o);  // relative terms: x is zero
    const ClothMat<R> mat = a.mats[a.vInfo[v].x];
    R acc[15];  // f[3], H[6], Hm[6]
#pragma unroll
    for (int k = 0; k < 15; ++k) acc[k] = R(0);
    partial<L, R, O>(a, c, o, mat, v, lane, x, xp, acc, acc + 3, acc + 9);
    if (L > 1) group_sum<L, R>(acc, 15, mask);
    if (lane != 0) return;
    R* f = acc;
    R* H = acc + 3;
    vertex_terms(a, c, o, mat, v, x, xp, f, H, acc + 9);
    R dx[3];
    V xn = x;  // relative to the origin
    if (solve_block<R>(H, f, dx, a.counters)) {
        xn = V{x.x + c.stepSize * dx[0], x.y + c.stepSize * dx[1], x.z + c.stepSize * dx[2]};
        const V xc = rel(a.xcd, static_cast<const P4<float>*>(nullptr), v, o);
        const V disp = sub(xn, xc);
        const R s = sqrt(dot(disp, disp));
        const R bnd = a.bound[v];
        if (s > bnd) {
            xn = add(xc, mul(bnd / s, disp));
            *a.req = 1;
            atomicAdd(&a.counters[CC_TRUNCATIONS], 1ull);
        }
        if (!(isfinite(xn.x) && isfinite(xn.y) && isfinite(xn.z))) {
            atomicAdd(&a.counters[CC_NONFINITE], 1ull);
            xn = x;
        }
    } else {
        atomicAdd(&a.counters[CC_FAILED], 1ull);
    }
    if constexpr (O::kRel) {
        // back to absolute: the origin plus the step (double-float add with the low halves)
        float hx = float(o.h.x), hy = float(o.h.y), hz = float(o.h.z), lx = o.lx, ly = o.ly, lz = o.lz;
        gaia::dev::df_add(hx, lx, float(xn.x));
        gaia::dev::df_add(hy, ly, float(xn.y));
        gaia::dev::df_add(hz, lz, float(xn.z));
        a.xnext[v] = P4<R>{R(hx), R(hy), R(hz), R(0)};
        a.xnextlo[v] = P4<float>{lx, ly, lz, 0.f};
    } else {
        st(a.xnext, v, xn);
    }
}

// One vertex's force and Hessian, for parity tests of the accumulation.
template <typename R, typename O>
__global__ void k_probe(Args<R> a, Consts<R> c, int v, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    R f[3] = {0, 0, 0}, H[6] = {0, 0, 0, 0, 0, 0};
    accumulate<R, O>(a, c, v, f, H);
    for (int k = 0; k < 3; ++k) out[k] = double(f[k]);
    for (int k = 0; k < 6; ++k) out[3 + k] = double(H[k]);
}

template <typename R>
__global__ void k_commit(Args<R> a, const int* verts, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int v = verts[i];
    if (!a.fixed[v]) {
        a.x[v] = a.xnext[v];
        if (a.xlo) a.xlo[v] = a.xnextlo[v];
    }
}

// (hi, lo) + d per component, d an increment in the working precision (the double-float
// state's update; without low halves a plain add)
template <typename R>
__device__ __forceinline__ void add_state(P4<R>* hi, P4<float>* lo, int v, typename Vec<R>::T base,
                                          const P4<float>& base_lo, typename Vec<R>::T d) {
    if (lo) {
        float hx = float(base.x), hy = float(base.y), hz = float(base.z);
        float lx = base_lo.x, ly = base_lo.y, lz = base_lo.z;
        gaia::dev::df_add(hx, lx, float(d.x));
        gaia::dev::df_add(hy, ly, float(d.y));
        gaia::dev::df_add(hz, lz, float(d.z));
        hi[v] = P4<R>{R(hx), R(hy), R(hz), R(0)};
        lo[v] = P4<float>{lx, ly, lz, 0.f};
    } else {
        st(hi, v, add(base, d));
    }
}

// applyInitialStep + forwardStep_intertia (VBDCloth/VBDBaseTriMesh.cpp:55-178, 180-196).
template <typename R>
__global__ void k_init_step(Args<R> a, Consts<R> c) {
    using V = typename Vec<R>::T;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= c.nSimV) return;
    const bool hasPrev = a.state[0] > 0;
    const V x = ld(a.x, v);
    const P4<float> xl = a.xlo ? a.xlo[v] : P4<float>{0.f, 0.f, 0.f, 0.f};
    st(a.xprev, v, x);
    if (a.xprevlo) a.xprevlo[v] = xl;
    V vel = ld(a.v, v);
    if (hasPrev) st(a.accel, v, mul(R(1) / c.dt, sub(vel, ld(a.vprev, v))));
    const V vp = vel;
    st(a.vprev, v, vel);
    if (c.assocGrav) vel = V{vel.x + c.dt * c.g[0], vel.y + c.dt * c.g[1], vel.z + c.dt * c.g[2]};
    if (a.fixed[v]) vel = V{0, 0, 0};
    st(a.v, v, vel);
    // the inertia target and the initial guess as increments of x (added to the double-float
    // state exactly where there is one)
    const V dy = mul(c.dt, vel);
    add_state(a.y, a.ylo, v, x, xl, dy);
    const int type = a.mats[a.vInfo[v].x].initType;
    V inc{R(0), R(0), R(0)};
    if (type == 0) {
        inc = dy;
    } else if (type == 1) {
        if (hasPrev) {
            const R gn = sqrt(c.g[0] * c.g[0] + c.g[1] * c.g[1] + c.g[2] * c.g[2]);
            const V gd = V{c.g[0] / gn, c.g[1] / gn, c.g[2] / gn};
            R ac = dot(ld(a.accel, v), gd);
            ac = ac < gn ? ac : gn;
            ac = ac > R(1e-5) ? ac : R(0);
            inc = add(mul(c.dt, vp), mul(c.dt * c.dt * ac, gd));
        } else {
            inc = dy;
        }
    } else if (type == 3) {
        V step = dy;
        const R s = sqrt(dot(step, step));
        const R bnd = a.bound[v];
        if (c.handleCollision && s > bnd && s != R(0)) step = mul(bnd / s, step);
        inc = step;
    }
    add_state(a.x, a.xlo, v, x, xl, inc);
}

// updateVelocity (VBDClothPhysics.cpp:2318-2360).
template <typename R>
__global__ void k_velocity(Args<R> a, Consts<R> c) {
    using V = typename Vec<R>::T;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v == 0) a.state[0] += 1;
    if (v >= c.nSimV) return;
    V dxv = sub(ld(a.x, v), ld(a.xprev, v));
    if (a.xlo) {  // the low halves' difference
        const P4<float> l = a.xlo[v], lp = a.xprevlo[v];
        dxv = V{dxv.x + R(l.x - lp.x), dxv.y + R(l.y - lp.y), dxv.z + R(l.z - lp.z)};
    }
    V vel = mul(R(1) / c.dt, dxv);
    const ClothMat<R> m = a.mats[a.vInfo[v].x];
    const R vm = sqrt(dot(vel, vel));
    if (m.hasNoGrav && m.maxVel > R(0) && vel.y > m.noGravThr) {
        if (vm > m.maxVel) vel = mul(m.maxVel / vm, vel);
    } else if (vm > R(1e-6)) {
        R vn = vm * m.expDamp - m.constDamp;
        vn = vn > R(1e-6) ? vn : R(0);
        vel = mul(vn / vm, vel);
    } else {
        vel = V{0, 0, 0};
    }
    if (a.fixed[v]) vel = V{0, 0, 0};
    st(a.v, v, vel);
}

// applyAcceleration (VBDClothPhysics.cpp:893-915): Chebyshev step outside active contacts.
template <typename R>
__global__ void k_accel(Args<R> a, Consts<R> c, R omega) {
    using V = typename Vec<R>::T;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= c.nSimV || a.active[v]) return;
    const V pi = ld(a.xPrevIter, v);
    V xn = add(mul(omega, sub(ld(a.x, v), pi)), pi);
    const V xc = ld(a.xcd, v);
    const V disp = sub(xn, xc);
    const R s = sqrt(dot(disp, disp));
    if (s > a.bound[v]) {
        xn = add(xc, mul(a.bound[v] / s, disp));
        *a.req = 1;
    }
    st(a.x, v, xn);
}

template <typename R>
__global__ void k_copy_positions(P4<R>* dst, const P4<R>* src, int n) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) dst[v] = src[v];
}

__global__ void k_set_int(int* p, int val) { *p = val; }

template <typename R>
__global__ void k_reset_active(Args<R> a, int n) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) a.active[v] = 0;
}

// positions of the simulated vertices at this detection: float copy for the
// detector, working-precision copy for the bound truncation
template <typename R>
__global__ void k_snapshot(Args<R> a, int n, const int* req) {
    if (req && *req == 0) return;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const P4<R> p = a.x[v];
    a.xcd[v] = p;
    a.xf[v] = make_float4(float(p.x), float(p.y), float(p.z), 0.f);
}

// conservative bounds and active-contact mask (VBDClothPhysics.cpp:780-814)
template <typename R>
__global__ void k_bounds(Args<R> a, Consts<R> c, const int* req) {
    if (*req == 0) return;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= c.nSimV) return;
    float dMin = float(c.maxQ);
    dMin = fminf(dMin, a.cd.vfMinDis[v]);
    bool act = a.cd.vfCount[v] > 0;
    for (int k = a.vfOfs[v]; k < a.vfOfs[v + 1]; ++k) {
        const int f = a.vfList[k].x;
        dMin = fminf(dMin, __int_as_float(a.cd.fMinDisBits[f]));
        act = act || a.cd.fvCount[f] > 0;
    }
    for (int k = a.veOfs[v]; k < a.veOfs[v + 1]; ++k) {
        const int e = a.veList[k].x;
        dMin = fminf(dMin, a.cd.eeMinDis[e]);
        act = act || a.cd.eeCount[e] > 0;
    }
    dMin = fmaxf(0.f, dMin - float(c.thick));
    a.bound[v] = R(dMin * float(c.relax));
    if (act) a.active[v] = 1;
}

template <typename R>
__global__ void k_bounds_inf(Args<R> a, int n) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) a.bound[v] = R(std::numeric_limits<float>::max());
}

}  // namespace kern

class ClothEngineBase {
public:
    virtual ~ClothEngineBase() {}
    virtual void run_steps(int n) = 0;
    virtual float run_steps_timed(int n) = 0;
    virtual void sync() = 0;
    virtual void get_positions(int mesh, double* out) = 0;
    virtual void set_positions(int mesh, const double* in) = 0;
    virtual void get_velocities(int mesh, double* out) = 0;
    virtual void set_velocities(int mesh, const double* in) = 0;
    virtual void detect() = 0;
    virtual void vf_contacts(std::vector<int32_t>& rows) = 0;
    virtual void ee_contacts(std::vector<int32_t>& rows) = 0;
    virtual void bounds(int mesh, double* out) = 0;
    virtual void min_distances(int mesh, float* vf, float* fv, float* ee) = 0;
    virtual void stats(gaia_cloth_stats* s) = 0;
    virtual void vertex_force_hessian(int mesh, int v, double* f3, double* h9) = 0;
    virtual float time_solve(int reps) = 0;
    virtual void autotune() = 0;
    virtual void lanes(std::vector<int>& out) const = 0;
};

template <typename R>
class ClothEngine : public ClothEngineBase {
public:
    // df: FP32 arithmetic on double-float positions (x, xprev, y, xnext as high + low halves)
    explicit ClothEngine(const Scene& s, bool df = false) : sc_(s), df_(df && sizeof(R) == 4) {
        if (df_ && sc_.p.applyAcceleration)
            throw std::runtime_error("gpuPrecision \"mixed\" is not supported with applyAcceleration");
        CL_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        CL_CUDA(cudaEventCreate(&ev0_));
        CL_CUDA(cudaEventCreate(&ev1_));
        build();
        tune_lanes();
        capture();
    }
    ~ClothEngine() override {
        if (graph_) cudaGraphExecDestroy(graph_);
        cudaEventDestroy(ev0_);
        cudaEventDestroy(ev1_);
        cudaStreamDestroy(st_);
    }

    void run_steps(int n) override {
        for (int i = 0; i < n; ++i) {
            if (sc_.p.handleCollision &&
                (!bvh_built_ || (sc_.p.contactBVHReconstructionSteps > 0 &&
                                 frame_ % sc_.p.contactBVHReconstructionSteps == 0)))
                rebuild_bvh();
            for (int s = 0; s < sc_.p.numSubsteps; ++s) CL_CUDA(cudaGraphLaunch(graph_, st_));
            ++frame_;
        }
    }
    float run_steps_timed(int n) override {
        CL_CUDA(cudaEventRecord(ev0_, st_));
        run_steps(n);
        CL_CUDA(cudaEventRecord(ev1_, st_));
        CL_CUDA(cudaEventSynchronize(ev1_));
        float ms = 0.f;
        CL_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
        check_nonfinite();
        return ms;
    }
    void sync() override {
        CL_CUDA(cudaStreamSynchronize(st_));
        check_nonfinite();
    }

    void get_positions(int mesh, double* out) override {
        copy_out(x_.p, mesh, out);
        if (df_) add_lo(xlo_.p, mesh, out);
    }
    void get_velocities(int mesh, double* out) override {
        if (mesh >= sc_.numSim) {
            std::fill(out, out + 3 * size_t(sc_.meshes[mesh].nv), 0.0);
            return;
        }
        copy_out(v_.p, mesh, out);
    }
    void set_positions(int mesh, const double* in) override {
        copy_in(x_.p, mesh, in);
        if (df_) copy_in_lo(xlo_.p, mesh, in);
        if (mesh >= sc_.numSim) {  // colliders: their previous positions and the detector copy too
            copy_in(xprev_.p, mesh, in);
            if (df_) copy_in_lo(xprevlo_.p, mesh, in);
            std::vector<float4> h(sc_.meshes[mesh].nv);
            for (size_t i = 0; i < h.size(); ++i)
                h[i] = make_float4(float(in[3 * i]), float(in[3 * i + 1]), float(in[3 * i + 2]), 0.f);
            CL_CUDA(cudaMemcpyAsync(xf_.p + vbase_[mesh], h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice, st_));
            CL_CUDA(cudaStreamSynchronize(st_));
        }
    }
    void set_velocities(int mesh, const double* in) override {
        if (mesh >= sc_.numSim) throw std::invalid_argument("colliders have no velocities");
        copy_in(v_.p, mesh, in);
    }

    void detect() override {
        if (sc_.numSim == 0) return;
        rebuild_bvh();
        kern::k_set_int<<<1, 1, 0, st_>>>(req_.p, 1);
        enqueue_detection();
        CL_CUDA(cudaStreamSynchronize(st_));
        CL_CUDA(cudaGetLastError());
    }
    void vf_contacts(std::vector<int32_t>& rows) override {
        const CDOut& o = cd_.out();
        const int nV = cdt_.nV;
        std::vector<int> cnt(nV), face(size_t(nV) * VF_CAP);
        CL_CUDA(cudaMemcpyAsync(cnt.data(), o.vfCount, nV * sizeof(int), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaMemcpyAsync(face.data(), o.vfFace, face.size() * sizeof(int), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        rows.clear();
        for (int v = 0; v < nV; ++v)
            for (int k = 0; k < std::min(cnt[v], VF_CAP); ++k) {
                const int f = face[size_t(v) * VF_CAP + k];
                rows.insert(rows.end(), {vmesh_[v], vlocal_[v], fmesh_[f], f - fbase_[fmesh_[f]]});
            }
    }
    void ee_contacts(std::vector<int32_t>& rows) override {
        const CDOut& o = cd_.out();
        const int nE = cdt_.nSimE;
        std::vector<int> cnt(nE), other(size_t(nE) * EE_CAP);
        CL_CUDA(cudaMemcpyAsync(cnt.data(), o.eeCount, nE * sizeof(int), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaMemcpyAsync(other.data(), o.eeOther, other.size() * sizeof(int), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        rows.clear();
        for (int e = 0; e < nE; ++e)
            for (int k = 0; k < std::min(cnt[e], EE_CAP); ++k) {
                const int e2 = other[size_t(e) * EE_CAP + k];
                rows.insert(rows.end(), {emesh_[e], e - ebase_[emesh_[e]], emesh_[e2], e2 - ebase_[emesh_[e2]]});
            }
    }
    void bounds(int mesh, double* out) override {
        if (mesh < 0 || mesh >= sc_.numSim) throw std::invalid_argument("bounds exist for simulated meshes only");
        const int nv = sc_.meshes[mesh].nv;
        std::vector<R> h(nv);
        CL_CUDA(cudaMemcpyAsync(h.data(), bound_.p + vbase_[mesh], nv * sizeof(R), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        for (int i = 0; i < nv; ++i) out[i] = double(h[i]);
    }
    void min_distances(int mesh, float* vf, float* fv, float* ee) override {
        const CDOut& o = cd_.out();
        const TriMesh& m = sc_.meshes[mesh];
        if (vf) CL_CUDA(cudaMemcpyAsync(vf, o.vfMinDis + vbase_[mesh], m.nv * sizeof(float), cudaMemcpyDeviceToHost, st_));
        if (fv) CL_CUDA(cudaMemcpyAsync(fv, o.fMinDisBits + fbase_[mesh], m.nf * sizeof(float), cudaMemcpyDeviceToHost, st_));
        if (ee) {
            if (mesh >= sc_.numSim) throw std::invalid_argument("edge-edge distances exist for simulated meshes only");
            CL_CUDA(cudaMemcpyAsync(ee, o.eeMinDis + ebase_[mesh], m.ne * sizeof(float), cudaMemcpyDeviceToHost, st_));
        }
        CL_CUDA(cudaStreamSynchronize(st_));
    }
    // Re-time the lanes per vertex of every color on the current state (its contacts
    // detected afresh) and capture the substep graph again.
    void autotune() override {
        tune_lanes(true);
        if (graph_) cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
        capture();
    }
    void lanes(std::vector<int>& out) const override { out = groupL_; }

    // Milliseconds of one sweep of the per-color solve and commit kernels over all
    // colors (CUDA events around `reps` sweeps on the current state); positions,
    // the detection flag and the counters are restored afterwards.
    float time_solve(int reps) override {
        if (reps <= 0) throw std::invalid_argument("reps must be positive");
        Buf<P4<R>> save;
        save.alloc(x_.n, nullptr);
        Buf<unsigned long long> csave;
        csave.alloc(CC_N, nullptr);
        Buf<int> rsave;
        rsave.alloc(1, nullptr);
        CL_CUDA(cudaMemcpyAsync(save.p, x_.p, x_.n * sizeof(P4<R>), cudaMemcpyDeviceToDevice, st_));
        Buf<P4<float>> save_lo;
        if (df_) {
            save_lo.alloc(xlo_.n, nullptr);
            CL_CUDA(cudaMemcpyAsync(save_lo.p, xlo_.p, xlo_.n * sizeof(P4<float>), cudaMemcpyDeviceToDevice, st_));
        }
        CL_CUDA(cudaMemcpyAsync(csave.p, counters_.p, CC_N * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st_));
        CL_CUDA(cudaMemcpyAsync(rsave.p, req_.p, sizeof(int), cudaMemcpyDeviceToDevice, st_));
        auto sweep = [&] {
            for (size_t gi = 0; gi < groups_.size(); ++gi) {
                const int n = int(groups_[gi]->n);
                if (n == 0) continue;
                launch_solve(groupL_[gi], groups_[gi]->p, n);
                kern::k_commit<R><<<nblk(n, 256), 256, 0, st_>>>(a_, groups_[gi]->p, n);
            }
        };
        sweep();  // warm-up
        CL_CUDA(cudaEventRecord(ev0_, st_));
        for (int r = 0; r < reps; ++r) sweep();
        CL_CUDA(cudaEventRecord(ev1_, st_));
        CL_CUDA(cudaEventSynchronize(ev1_));
        float ms = 0.f;
        CL_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
        CL_CUDA(cudaMemcpyAsync(x_.p, save.p, x_.n * sizeof(P4<R>), cudaMemcpyDeviceToDevice, st_));
        if (df_)
            CL_CUDA(cudaMemcpyAsync(xlo_.p, save_lo.p, xlo_.n * sizeof(P4<float>), cudaMemcpyDeviceToDevice, st_));
        CL_CUDA(cudaMemcpyAsync(counters_.p, csave.p, CC_N * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st_));
        CL_CUDA(cudaMemcpyAsync(req_.p, rsave.p, sizeof(int), cudaMemcpyDeviceToDevice, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        CL_CUDA(cudaGetLastError());
        return ms / reps;
    }
    void vertex_force_hessian(int mesh, int v, double* f3, double* h9) override {
        if (mesh < 0 || mesh >= sc_.numSim || v < 0 || v >= sc_.meshes[mesh].nv)
            throw std::invalid_argument("vertex out of range");
        Buf<double> out;
        out.alloc(9, nullptr);
        if (df_) kern::k_probe<R, kern::OrgRel<R>><<<1, 32, 0, st_>>>(a_, c_, vbase_[mesh] + v, out.p);
        else kern::k_probe<R, kern::OrgAbs<R>><<<1, 32, 0, st_>>>(a_, c_, vbase_[mesh] + v, out.p);
        double h[9];
        CL_CUDA(cudaMemcpyAsync(h, out.p, sizeof(h), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        for (int k = 0; k < 3; ++k) f3[k] = h[k];
        const int idx[9] = {3, 4, 5, 4, 6, 7, 5, 7, 8};
        for (int k = 0; k < 9; ++k) h9[k] = h[idx[k]];
    }
    void stats(gaia_cloth_stats* s) override {
        unsigned long long h[CC_N];
        CL_CUDA(cudaMemcpyAsync(h, counters_.p, sizeof(h), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        std::memset(s, 0, sizeof(*s));
        s->precision = sizeof(R) == 4 ? (df_ ? 48 : 32) : 64;
        s->num_groups = int32_t(groups_.size());
        s->num_vertices = cdt_.nV;
        s->num_sim_vertices = cdt_.nSimV;
        s->num_faces = cdt_.nF;
        s->num_edges = cdt_.nE;
        s->kernel_launches_per_step = launches_per_substep_ * sc_.p.numSubsteps;
        s->detections = int64_t(h[CC_DETECTIONS]);
        s->truncations = int64_t(h[CC_TRUNCATIONS]);
        s->vf_overflow = int64_t(h[CC_VF_OVERFLOW]);
        s->ee_overflow = int64_t(h[CC_EE_OVERFLOW]);
        s->fv_overflow = int64_t(h[CC_FV_OVERFLOW]);
        s->candidate_overflow = int64_t(h[CC_CAND_OVERFLOW]);
        s->stack_overflow = int64_t(h[CC_STACK_OVERFLOW]);
        s->fp64_fallback_solves = int64_t(h[CC_FP64_SOLVES]);
        s->failed_solves = int64_t(h[CC_FAILED]);
        s->device_bytes = int64_t(bytes_ + cd_.device_bytes());
    }

private:
    void check_nonfinite() {
        unsigned long long h = 0;
        CL_CUDA(cudaMemcpyAsync(&h, counters_.p + CC_NONFINITE, sizeof(h), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        if (h) throw std::domain_error("a cloth vertex solve produced a non-finite position");
    }
    void copy_out(const P4<R>* src, int mesh, double* out) {
        const int nv = sc_.meshes.at(mesh).nv;
        std::vector<P4<R>> h(nv);
        CL_CUDA(cudaMemcpyAsync(h.data(), src + vbase_[mesh], nv * sizeof(P4<R>), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        for (int i = 0; i < nv; ++i) {
            out[3 * i] = double(h[i].x);
            out[3 * i + 1] = double(h[i].y);
            out[3 * i + 2] = double(h[i].z);
        }
    }
    void copy_in(P4<R>* dst, int mesh, const double* in) {
        const int nv = sc_.meshes.at(mesh).nv;
        std::vector<P4<R>> h(nv);
        for (int i = 0; i < nv; ++i) h[i] = P4<R>{R(in[3 * i]), R(in[3 * i + 1]), R(in[3 * i + 2]), R(0)};
        CL_CUDA(cudaMemcpyAsync(dst + vbase_[mesh], h.data(), nv * sizeof(P4<R>), cudaMemcpyHostToDevice, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
    }
    // the low halves of the double-float positions: in - float(in), and their sum back
    void copy_in_lo(P4<float>* dst, int mesh, const double* in) {
        const int nv = sc_.meshes.at(mesh).nv;
        std::vector<P4<float>> h(nv);
        for (int i = 0; i < nv; ++i) {
            float l[3];
            for (int k = 0; k < 3; ++k) l[k] = float(in[3 * i + k] - double(float(in[3 * i + k])));
            h[i] = P4<float>{l[0], l[1], l[2], 0.f};
        }
        CL_CUDA(cudaMemcpyAsync(dst + vbase_[mesh], h.data(), nv * sizeof(P4<float>), cudaMemcpyHostToDevice, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
    }
    void add_lo(const P4<float>* src, int mesh, double* out) {
        const int nv = sc_.meshes.at(mesh).nv;
        std::vector<P4<float>> h(nv);
        CL_CUDA(cudaMemcpyAsync(h.data(), src + vbase_[mesh], nv * sizeof(P4<float>), cudaMemcpyDeviceToHost, st_));
        CL_CUDA(cudaStreamSynchronize(st_));
        for (int i = 0; i < nv; ++i) {
            out[3 * i] += double(h[i].x);
            out[3 * i + 1] += double(h[i].y);
            out[3 * i + 2] += double(h[i].z);
        }
    }

    void build() {
        const int nm = int(sc_.meshes.size());
        vbase_.assign(nm + 1, 0);
        fbase_.assign(nm + 1, 0);
        ebase_.assign(nm + 1, 0);
        for (int m = 0; m < nm; ++m) {
            vbase_[m + 1] = vbase_[m] + sc_.meshes[m].nv;
            fbase_[m + 1] = fbase_[m] + sc_.meshes[m].nf;
            ebase_[m + 1] = ebase_[m] + sc_.meshes[m].ne;
        }
        const int nV = vbase_[nm], nF = fbase_[nm], nE = ebase_[nm];
        const int ns = sc_.numSim;
        const int nSimV = vbase_[ns], nSimF = fbase_[ns], nSimE = ebase_[ns];
        if (int64_t(nV) * std::max(VF_CAP, 1) > (int64_t(1) << 31) || int64_t(nF) * FV_CAP > (int64_t(1) << 31))
            throw std::runtime_error("scene too large for 32-bit contact indexing");

        std::vector<P4<R>> hx(nV);
        std::vector<int2> vInfo(nV);
        std::vector<uint8_t> fixed(nV, 1);
        std::vector<R> mass(std::max(nSimV, 1), R(0));
        std::vector<int4> faces(nF), faceEdges(nF), edges(nE), edgeInfo(nE);
        std::vector<int> nbrVOfs(nV + 1, 0), nbrV;
        std::vector<int> vfOfs(nSimV + 1, 0), veOfs(nSimV + 1, 0), vbOfs(nSimV + 1, 0);
        std::vector<int2> vfList, veList, vbList;
        std::vector<P4<R>> dminv(std::max(nSimF, 1));
        std::vector<R> area(std::max(nSimF, 1)), bendQ(16 * size_t(std::max(nSimE, 1)), R(0));
        vmesh_.assign(nV, 0);
        vlocal_.assign(nV, 0);
        fmesh_.assign(nF, 0);
        emesh_.assign(nE, 0);
        for (int m = 0; m < nm; ++m) {
            const TriMesh& M = sc_.meshes[m];
            const int vb = vbase_[m], fb = fbase_[m], eb = ebase_[m];
            for (int i = 0; i < M.nv; ++i) {
                hx[vb + i] = P4<R>{R(M.X[3 * i]), R(M.X[3 * i + 1]), R(M.X[3 * i + 2]), R(0)};
                vInfo[vb + i] = make_int2(m, i);
                vmesh_[vb + i] = m;
                vlocal_[vb + i] = i;
                if (m < ns) {
                    fixed[vb + i] = M.fixed[i];
                    mass[vb + i] = R(M.mass[i]);
                }
                for (int k = M.nbrVOfs[i]; k < M.nbrVOfs[i + 1]; ++k) nbrV.push_back(vb + M.nbrV[k]);
                nbrVOfs[vb + i + 1] = int(nbrV.size());
            }
            for (int f = 0; f < M.nf; ++f) {
                faces[fb + f] = make_int4(vb + M.faces[3 * f], vb + M.faces[3 * f + 1], vb + M.faces[3 * f + 2], m);
                faceEdges[fb + f] = make_int4(eb + M.faceEdges[3 * f], eb + M.faceEdges[3 * f + 1], eb + M.faceEdges[3 * f + 2], f);
                fmesh_[fb + f] = m;
                if (m < ns) {
                    const double* d = &M.dminv[4 * f];
                    dminv[fb + f] = P4<R>{R(d[0]), R(d[1]), R(d[2]), R(d[3])};
                    area[fb + f] = R(M.area[f]);
                }
            }
            for (int e = 0; e < M.ne; ++e) {
                const Edge& E = M.edges[e];
                edges[eb + e] = make_int4(vb + E.v1, vb + E.v2, vb + E.v12next, E.v21next < 0 ? -1 : vb + E.v21next);
                edgeInfo[eb + e] = make_int4(fb + E.f1, E.f2 < 0 ? -1 : fb + E.f2, m, e);
                emesh_[eb + e] = m;
                if (m < ns)
                    for (int k = 0; k < 16; ++k) bendQ[16 * size_t(eb + e) + k] = R(M.bendQ[16 * size_t(e) + k]);
            }
            if (m < ns) {
                for (int i = 0; i < M.nv; ++i) {
                    for (int k = M.nbrFOfs[i]; k < M.nbrFOfs[i + 1]; ++k) vfList.push_back(make_int2(fb + M.nbrF[k], M.nbrFOrder[k]));
                    vfOfs[vb + i + 1] = int(vfList.size());
                    for (int k = M.nbrEOfs[i]; k < M.nbrEOfs[i + 1]; ++k) veList.push_back(make_int2(eb + M.nbrE[k], M.nbrEOrder[k]));
                    veOfs[vb + i + 1] = int(veList.size());
                    for (int k = M.bendOfs[i]; k < M.bendOfs[i + 1]; ++k) vbList.push_back(make_int2(eb + M.bendE[k], M.bendOrder[k]));
                    vbOfs[vb + i + 1] = int(vbList.size());
                }
            }
        }
        std::vector<ClothMat<R>> mats(nm);
        for (int m = 0; m < nm; ++m) {
            ClothMat<R> M{};
            if (m < ns) {
                const ObjectParams& o = sc_.objs[m];
                M.miu = R(o.miu);
                M.lambda = R(o.lambda);
                M.dampStVK = R(o.dampingStVK);
                M.dampBend = R(o.dampingBending);
                M.kBend = R(o.bendingStiffness);
                M.fricMu = R(o.frictionDynamic);
                M.fricEps = R(o.frictionEpsV);
                M.expDamp = R(o.exponentialVelDamping);
                M.constDamp = R(o.constantVelDamping);
                M.maxVel = R(o.maxVelocityMagnitude);
                M.noGravThr = R(o.noGravZoneThreshold);
                M.hasNoGrav = o.hasNoGravZone ? 1 : 0;
                M.initType = o.initializationType;
            } else {
                const int c = m - ns;
                M.fricMu = R(sc_.colliderFriction[2 * c]);
                M.fricEps = R(sc_.colliderFriction[2 * c + 1]);
            }
            mats[m] = M;
        }

        const PhysicsParams& p = sc_.p;
        Consts<R>& c = c_;
        c.dt = R(p.dt);
        c.dtSqrRecip = R(p.dtSqrReciprocal);
        c.stepSize = R(p.stepSize);
        for (int k = 0; k < 3; ++k) {
            c.g[k] = R(p.gravity[k]);
            c.lo[k] = R(p.worldLo[k]);
            c.hi[k] = R(p.worldHi[k]);
        }
        c.kb = R(p.boundaryContactStiffness);
        c.muB = R(p.boundaryFrictionDynamic);
        c.epsUB = R(p.boundaryFrictionEpsValue * p.dt);
        c.kc = R(p.contactStiffness);
        c.rc = R(p.contactRadius);
        c.thick = R(p.thickness);
        c.degThr2 = R(p.degenerateTriangleThres * p.degenerateTriangleThres);
        c.relax = R(p.conservativeStepRelaxation);
        c.maxQ = R(float(p.maxQueryDis));
        c.nSimV = nSimV;
        c.nV = nV;
        c.assocGrav = p.associateGravityWithInertia ? 1 : 0;
        c.handleCollision = p.handleCollision ? 1 : 0;

        size_t* tb = &bytes_;
        x_.upload(hx, tb, st_);
        xprev_.upload(hx, tb, st_);
        y_.upload(hx, tb, st_);
        xnext_.upload(hx, tb, st_);
        if (df_) {
            // low halves: the remainder of each FP64 input position after its FP32 rounding
            std::vector<P4<float>> hl(nV, P4<float>{0.f, 0.f, 0.f, 0.f});
            for (int m = 0; m < nm; ++m) {
                const TriMesh& M = sc_.meshes[m];
                for (int i = 0; i < M.nv; ++i) {
                    float l[3];
                    for (int k = 0; k < 3; ++k) l[k] = float(M.X[3 * i + k] - double(float(M.X[3 * i + k])));
                    hl[vbase_[m] + i] = P4<float>{l[0], l[1], l[2], 0.f};
                }
            }
            xlo_.upload(hl, tb, st_);
            xprevlo_.upload(hl, tb, st_);
            ylo_.upload(hl, tb, st_);
            xnextlo_.upload(hl, tb, st_);
        }
        xcd_.upload(hx, tb, st_);
        xPrevIter_.upload(hx, tb, st_);
        xrest_.upload(hx, tb, st_);
        std::vector<P4<R>> zeros(nV, P4<R>{0, 0, 0, 0});
        v_.upload(zeros, tb, st_);
        vprev_.upload(zeros, tb, st_);
        accel_.upload(zeros, tb, st_);
        bound_.upload(std::vector<R>(std::max(nSimV, 1), R(std::numeric_limits<float>::max())), tb, st_);
        mass_.upload(mass, tb, st_);
        fixed_.upload(fixed, tb, st_);
        active_.upload(std::vector<uint8_t>(std::max(nSimV, 1), 0), tb, st_);
        vInfo_.upload(vInfo, tb, st_);
        mats_.upload(mats, tb, st_);
        faces_.upload(faces, tb, st_);
        faceEdges_.upload(faceEdges, tb, st_);
        edges_.upload(edges, tb, st_);
        edgeInfo_.upload(edgeInfo, tb, st_);
        nbrVOfs_.upload(nbrVOfs, tb, st_);
        nbrV_.upload(nbrV, tb, st_);
        vfOfs_.upload(vfOfs, tb, st_);
        vfList_.upload(vfList, tb, st_);
        veOfs_.upload(veOfs, tb, st_);
        veList_.upload(veList, tb, st_);
        vbOfs_.upload(vbOfs, tb, st_);
        vbList_.upload(vbList, tb, st_);
        dminv_.upload(dminv, tb, st_);
        area_.upload(area, tb, st_);
        bendQ_.upload(bendQ, tb, st_);
        std::vector<float4> hf(nV);
        for (int i = 0; i < nV; ++i) hf[i] = make_float4(float(hx[i].x), float(hx[i].y), float(hx[i].z), 0.f);
        xf_.upload(hf, tb, st_);
        req_.upload(std::vector<int>{0}, tb, st_);
        state_.upload(std::vector<int>{0, 0}, tb, st_);
        counters_.upload(std::vector<unsigned long long>(CC_N, 0ull), tb, st_);

        groups_.clear();
        for (const auto& g : sc_.groups) {
            std::vector<int> gv;
            for (size_t k = 0; k + 1 < g.size(); k += 2) gv.push_back(vbase_[g[k]] + g[k + 1]);
            groups_.emplace_back(new Buf<int>());
            groups_.back()->upload(gv, tb, st_);
        }

        cdt_.nV = nV;
        cdt_.nF = nF;
        cdt_.nE = nE;
        cdt_.nSimV = nSimV;
        cdt_.nSimF = nSimF;
        cdt_.nSimE = nSimE;
        cdt_.numSimMeshes = ns;
        cdt_.faces = faces_.p;
        cdt_.faceEdges = faceEdges_.p;
        cdt_.edges = edges_.p;
        cdt_.edgeInfo = edgeInfo_.p;
        cdt_.vInfo = vInfo_.p;
        cdt_.nbrVOfs = nbrVOfs_.p;
        cdt_.nbrV = nbrV_.p;
        cd_.init(cdt_, counters_.p, st_);
        CL_CUDA(cudaStreamSynchronize(st_));

        Args<R>& a = a_;
        a.x = x_.p;
        a.xprev = xprev_.p;
        a.y = y_.p;
        a.xnext = xnext_.p;
        a.xlo = df_ ? xlo_.p : nullptr;
        a.xprevlo = df_ ? xprevlo_.p : nullptr;
        a.ylo = df_ ? ylo_.p : nullptr;
        a.xnextlo = df_ ? xnextlo_.p : nullptr;
        a.xcd = xcd_.p;
        a.v = v_.p;
        a.vprev = vprev_.p;
        a.accel = accel_.p;
        a.xPrevIter = xPrevIter_.p;
        a.xrest = xrest_.p;
        a.bound = bound_.p;
        a.mass = mass_.p;
        a.fixed = fixed_.p;
        a.active = active_.p;
        a.vInfo = vInfo_.p;
        a.mats = mats_.p;
        a.faces = faces_.p;
        a.edges = edges_.p;
        a.vfOfs = vfOfs_.p;
        a.vfList = vfList_.p;
        a.veOfs = veOfs_.p;
        a.veList = veList_.p;
        a.vbOfs = vbOfs_.p;
        a.vbList = vbList_.p;
        a.faceDmInv = dminv_.p;
        a.faceArea = area_.p;
        a.bendQ = bendQ_.p;
        a.xf = xf_.p;
        a.cd = cd_.out();
        a.req = req_.p;
        a.state = state_.p;
        a.counters = counters_.p;
    }

    template <typename O>
    void launch_solve_o(int L, const int* verts, int n) {
        const int B = sc_.p.blockSize;
        const int64_t threads = int64_t(n) * L;
        switch (L) {
            case 1: kern::k_solve<1, R, O><<<nblk(threads, B), B, 0, st_>>>(a_, c_, verts, n); break;
            case 2: kern::k_solve<2, R, O><<<nblk(threads, B), B, 0, st_>>>(a_, c_, verts, n); break;
            case 4: kern::k_solve<4, R, O><<<nblk(threads, B), B, 0, st_>>>(a_, c_, verts, n); break;
            case 8: kern::k_solve<8, R, O><<<nblk(threads, B), B, 0, st_>>>(a_, c_, verts, n); break;
            case 16: kern::k_solve<16, R, O><<<nblk(threads, B), B, 0, st_>>>(a_, c_, verts, n); break;
            case 32: kern::k_solve<32, R, O><<<nblk(threads, B), B, 0, st_>>>(a_, c_, verts, n); break;
            default: throw std::invalid_argument("lanesPerVertex must be 1, 2, 4, 8, 16 or 32");
        }
    }
    // the double-float state's terms relative to each vertex; the others on the coordinates
    void launch_solve(int L, const int* verts, int n) {
        if constexpr (sizeof(R) == 4) {
            if (df_) {
                launch_solve_o<kern::OrgRel<R>>(L, verts, n);
                return;
            }
        }
        launch_solve_o<kern::OrgAbs<R>>(L, verts, n);
    }

    // Lanes per vertex of each color's solve: fixed by lanesPerVertex, or the fastest of
    // 1..32 timed on the color's kernel alone (CUDA events over repeated launches on the
    // initial state with its contacts detected; positions and counters restored).
    void tune_lanes(bool force = false) {
        groupL_.assign(groups_.size(), sc_.p.lanesPerVertex > 0 ? sc_.p.lanesPerVertex : 16);
        if ((sc_.p.lanesPerVertex > 0 && !force) || cdt_.nSimV == 0) return;
        Buf<P4<R>> save;
        save.alloc(x_.n, nullptr);
        Buf<unsigned long long> csave;
        csave.alloc(CC_N, nullptr);
        CL_CUDA(cudaMemcpyAsync(save.p, x_.p, x_.n * sizeof(P4<R>), cudaMemcpyDeviceToDevice, st_));
        Buf<P4<float>> save_lo;
        if (df_) {
            save_lo.alloc(xlo_.n, nullptr);
            CL_CUDA(cudaMemcpyAsync(save_lo.p, xlo_.p, xlo_.n * sizeof(P4<float>), cudaMemcpyDeviceToDevice, st_));
        }
        CL_CUDA(cudaMemcpyAsync(csave.p, counters_.p, CC_N * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st_));
        if (sc_.p.handleCollision) {
            rebuild_bvh();
            kern::k_set_int<<<1, 1, 0, st_>>>(req_.p, 1);
            enqueue_detection();
        }
        const int Ls[] = {1, 2, 4, 8, 16, 32};
        for (size_t gi = 0; gi < groups_.size(); ++gi) {
            const int n = int(groups_[gi]->n);
            if (n == 0) continue;
            float best = 1e30f;
            for (int round = 0; round < 2; ++round)  // two interleaved rounds, best of both
                for (int L : Ls) {
                    launch_solve(L, groups_[gi]->p, n);  // warm-up
                    CL_CUDA(cudaEventRecord(ev0_, st_));
                    for (int r = 0; r < 4; ++r) launch_solve(L, groups_[gi]->p, n);
                    CL_CUDA(cudaEventRecord(ev1_, st_));
                    CL_CUDA(cudaEventSynchronize(ev1_));
                    float ms = 0.f;
                    CL_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
                    if (ms < best) {
                        best = ms;
                        groupL_[gi] = L;
                    }
                }
        }
        // back to the state before tuning (positions, counters, the detection flag); the
        // contact sets and bounds are recomputed by the detection that opens the next step
        CL_CUDA(cudaMemcpyAsync(x_.p, save.p, x_.n * sizeof(P4<R>), cudaMemcpyDeviceToDevice, st_));
        if (df_)
            CL_CUDA(cudaMemcpyAsync(xlo_.p, save_lo.p, xlo_.n * sizeof(P4<float>), cudaMemcpyDeviceToDevice, st_));
        CL_CUDA(cudaMemcpyAsync(counters_.p, csave.p, CC_N * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st_));
        CL_CUDA(cudaMemsetAsync(req_.p, 0, sizeof(int), st_));
        CL_CUDA(cudaStreamSynchronize(st_));
    }

    void rebuild_bvh() {
        if (cdt_.nSimV > 0) kern::k_snapshot<R><<<nblk(cdt_.nSimV, 256), 256, 0, st_>>>(a_, cdt_.nSimV, nullptr);
        cd_.rebuild(xf_.p, st_);
        bvh_built_ = true;
    }

    // snapshot -> refit + queries -> bounds, each gated on the device flag
    int enqueue_detection() {
        const int ns = cdt_.nSimV;
        kern::k_snapshot<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, ns, req_.p);
        cd_.enqueue_detect(xf_.p, float(sc_.p.maxQueryDis), req_.p, st_);
        kern::k_bounds<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, c_, req_.p);
        return 9;
    }

    // One substep: the iteration loop of runStep_CDEveryIter, captured once.
    void capture() {
        const PhysicsParams& p = sc_.p;
        const int ns = cdt_.nSimV;
        const int B = p.blockSize;
        CL_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        int launches = 0;
        R omega = R(1);
        for (int it = 0; it < p.iterations; ++it) {
            if (it == 0) {
                kern::k_reset_active<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, ns);
                ++launches;
            }
            if (p.handleCollision) {
                if (it == 0 || p.contactDetectionEveryIteration) {
                    kern::k_set_int<<<1, 1, 0, st_>>>(req_.p, 1);
                    ++launches;
                }
                launches += enqueue_detection();
                kern::k_set_int<<<1, 1, 0, st_>>>(req_.p, 0);
                ++launches;
            } else if (it == 0) {
                kern::k_bounds_inf<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, ns);
                ++launches;
            }
            if (p.applyAcceleration) {
                kern::k_copy_positions<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(xPrevIter_.p, x_.p, ns);
                ++launches;
            }
            if (it == 0) {
                kern::k_init_step<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, c_);
                ++launches;
            }
            for (size_t gi = 0; gi < groups_.size(); ++gi) {
                const int n = int(groups_[gi]->n);
                if (n == 0) continue;
                launch_solve(groupL_[gi], groups_[gi]->p, n);
                kern::k_commit<R><<<nblk(n, 256), 256, 0, st_>>>(a_, groups_[gi]->p, n);
                launches += 2;
            }
            if (p.applyAcceleration) {
                // ChebysevAccelerator::getAcceleratorOmega (SolverUtils/ChebysevAccelerator.h:15-35)
                const R rho = R(float(p.acceleratorRho));
                const int order = it + 1;
                if (rho == R(0)) omega = R(1);
                else if (order == 1) omega = R(1);
                else if (order == 2) omega = R(2) / (R(2) - rho * rho);
                else omega = R(4) / (R(4) - rho * rho * omega);
                if (omega > R(1)) {
                    kern::k_accel<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, c_, omega);
                    ++launches;
                }
            }
        }
        kern::k_velocity<R><<<nblk(std::max(ns, 1), 256), 256, 0, st_>>>(a_, c_);
        ++launches;
        cudaGraph_t g = nullptr;
        CL_CUDA(cudaStreamEndCapture(st_, &g));
        CL_CUDA(cudaGraphInstantiate(&graph_, g, 0));
        cudaGraphDestroy(g);
        launches_per_substep_ = launches;
    }

    Scene sc_;
    cudaStream_t st_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    int64_t frame_ = 0;
    bool bvh_built_ = false;  // the contact hierarchies exist (built at least once)
    int launches_per_substep_ = 0;
    size_t bytes_ = 0;
    std::vector<int> vbase_, fbase_, ebase_, vmesh_, vlocal_, fmesh_, emesh_;
    Buf<P4<R>> x_, xprev_, y_, xnext_, xcd_, xPrevIter_, xrest_, v_, vprev_, accel_;
    bool df_ = false;                                    // double-float positions (FP32 engine)
    Buf<P4<float>> xlo_, xprevlo_, ylo_, xnextlo_;       // their low halves
    Buf<R> bound_, mass_, area_, bendQ_;
    Buf<uint8_t> fixed_, active_;
    Buf<int2> vInfo_, vfList_, veList_, vbList_;
    Buf<ClothMat<R>> mats_;
    Buf<int4> faces_, faceEdges_, edges_, edgeInfo_;
    Buf<int> nbrVOfs_, nbrV_, vfOfs_, veOfs_, vbOfs_, req_, state_;
    Buf<P4<R>> dminv_;
    Buf<float4> xf_;
    Buf<unsigned long long> counters_;
    std::vector<std::unique_ptr<Buf<int>>> groups_;
    std::vector<int> groupL_;
    CDTopo cdt_;
    ContactDetector cd_;
    Args<R> a_{};
    Consts<R> c_{};
};

}  // namespace cloth
}  // namespace gaia

// ---- C ABI ---------------------------------------------------------------------

struct gaia_cloth {
    gaia::cloth::Scene scene;
    std::unique_ptr<gaia::cloth::ClothEngineBase> eng;
    std::string err;
    int64_t frame = 0;     // runStep calls since initialize / the last loaded state
    double time = 0.0;     // simulated time (timeStep per runStep)
};

namespace {

template <typename Fn>
int cguard(gaia_cloth* h, Fn&& fn) {
    try {
        fn();
        if (h) h->err.clear();
        return GAIA_VBD_OK;
    } catch (const gaia::cloth::CudaError& e) {
        if (h) h->err = e.what();
        gaia::set_last_global_error(e.what());
        return GAIA_VBD_E_CUDA;
    } catch (const std::invalid_argument& e) {
        if (h) h->err = e.what();
        gaia::set_last_global_error(e.what());
        return GAIA_VBD_E_INVALID_ARG;
    } catch (const std::domain_error& e) {
        if (h) h->err = e.what();
        gaia::set_last_global_error(e.what());
        return GAIA_VBD_E_NONFINITE;
    } catch (const std::exception& e) {
        if (h) h->err = e.what();
        gaia::set_last_global_error(e.what());
        std::string m = e.what();
        if (m.find("coloring") != std::string::npos) return GAIA_VBD_E_COLORING;
        if (m.find("degenerate") != std::string::npos || m.find("out of range") != std::string::npos ||
            m.find("manifold") != std::string::npos || m.find("oriented") != std::string::npos)
            return GAIA_VBD_E_MESH;
        if (m.find("not supported") != std::string::npos || m.find("only static") != std::string::npos ||
            m.find("not part of") != std::string::npos)
            return GAIA_VBD_E_UNSUPPORTED;
        return GAIA_VBD_E_INPUT;
    }
}

bool mesh_ok(gaia_cloth* h, int32_t mesh) {
    return h && h->eng && mesh >= 0 && size_t(mesh) < h->scene.meshes.size();
}

}  // namespace

extern "C" {

int gaia_cloth_load(const char* models_json, const char* params_json, const char* repo_root, gaia_cloth** out) {
    if (!out || !models_json || !params_json) return GAIA_VBD_E_INVALID_ARG;
    *out = nullptr;
    std::unique_ptr<gaia_cloth> h(new gaia_cloth());
    int rc = cguard(nullptr, [&] {
        gaia::cloth::load_scene(models_json, params_json, repo_root ? repo_root : "", h->scene);
    });
    if (rc) return rc;
    *out = h.release();
    return GAIA_VBD_OK;
}

int gaia_cloth_initialize(gaia_cloth* h) {
    if (!h) return GAIA_VBD_E_INVALID_ARG;
    if (h->eng) return GAIA_VBD_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        h->err = "no CUDA device is visible";
        gaia::set_last_global_error(h->err);
        return GAIA_VBD_E_NO_DEVICE;
    }
    return cguard(h, [&] {
        if (h->scene.p.gpuPrecision == "fp64") h->eng.reset(new gaia::cloth::ClothEngine<double>(h->scene));
        else h->eng.reset(new gaia::cloth::ClothEngine<float>(h->scene, h->scene.p.gpuPrecision == "mixed"));
    });
}

int gaia_cloth_create(const char* models_json, const char* params_json, const char* repo_root, gaia_cloth** out) {
    gaia_cloth* h = nullptr;
    int rc = gaia_cloth_load(models_json, params_json, repo_root, &h);
    if (rc) return rc;
    rc = gaia_cloth_initialize(h);
    if (rc) {
        gaia::set_last_global_error(h->err);
        delete h;
        return rc;
    }
    *out = h;
    return GAIA_VBD_OK;
}

void gaia_cloth_destroy(gaia_cloth* h) { delete h; }

const char* gaia_cloth_last_error(gaia_cloth* h) { return h ? h->err.c_str() : ""; }

int gaia_cloth_run_step(gaia_cloth* h, int32_t n) {
    if (!h || !h->eng || n < 0) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        h->eng->run_steps(n);
        h->frame += n;
        h->time += n * h->scene.p.timeStep;
    });
}

namespace {
// All vertices and faces of every simulated mesh (TriMeshFEM::saveAsPLY, writeAllToBinary).
std::vector<gaia::FrameMesh> cloth_frame(gaia_cloth* h) {
    std::vector<gaia::FrameMesh> out;
    for (int m = 0; m < h->scene.numSim; ++m) {
        const gaia::cloth::TriMesh& M = h->scene.meshes[m];
        std::vector<double> x(3 * size_t(M.nv));
        h->eng->get_positions(m, x.data());
        gaia::FrameMesh fm;
        fm.X.assign(x.begin(), x.end());
        fm.faces = M.faces;
        fm.model_path = h->scene.objs[m].path;
        out.push_back(std::move(fm));
    }
    return out;
}
}  // namespace

int gaia_cloth_write_ply(gaia_cloth* h, const char* path, int32_t all_in_one, int32_t add_model_name) {
    if (!h || !h->eng || !path) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { gaia::write_frame_ply(path, cloth_frame(h), all_in_one != 0, add_model_name != 0, true); });
}

int gaia_cloth_write_binary(gaia_cloth* h, const char* path) {
    if (!h || !h->eng || !path) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { gaia::write_frame_binary(path, cloth_frame(h)); });
}

int gaia_cloth_save_state(gaia_cloth* h, const char* path, int32_t binary) {
    if (!h || !h->eng || !path) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        gaia::PhysicsStateFile st;
        st.frameId = int(h->frame);
        st.curTime = h->time;
        for (int m = 0; m < h->scene.numSim; ++m) {
            const size_t nv = size_t(h->scene.meshes[m].nv);
            std::vector<double> x(3 * nv), v(3 * nv);
            h->eng->get_positions(m, x.data());
            h->eng->get_velocities(m, v.data());
            st.position.emplace_back(x.begin(), x.end());
            st.velocity.emplace_back(v.begin(), v.end());
        }
        gaia::write_physics_state(path, st, binary != 0);
    });
}

int gaia_cloth_load_state(gaia_cloth* h, const char* path) {
    if (!h || !h->eng || !path) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        gaia::PhysicsStateFile st = gaia::read_physics_state(path);
        for (int m = 0; m < h->scene.numSim && size_t(m) < st.position.size(); ++m) {
            const size_t nv = size_t(h->scene.meshes[m].nv);
            if (st.position[m].size() != 3 * nv)
                throw std::invalid_argument("state file mesh " + std::to_string(m) + " has " +
                                            std::to_string(st.position[m].size() / 3) + " vertices, the scene " +
                                            std::to_string(nv));
            std::vector<double> x(st.position[m].begin(), st.position[m].end());
            std::vector<double> v(st.velocity[m].begin(), st.velocity[m].end());
            h->eng->set_positions(m, x.data());
            h->eng->set_velocities(m, v.data());
        }
        h->frame = st.frameId;
        h->time = st.curTime;
    });
}

int gaia_cloth_run_step_timed(gaia_cloth* h, int32_t n, float* total_ms) {
    if (!h || !h->eng || n < 0) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        float ms = h->eng->run_steps_timed(n);
        if (total_ms) *total_ms = ms;
    });
}

int gaia_cloth_synchronize(gaia_cloth* h) {
    if (!h || !h->eng) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->sync(); });
}

int gaia_cloth_num_meshes(gaia_cloth* h, int32_t* num_sim, int32_t* num_colliders) {
    if (!h) return GAIA_VBD_E_INVALID_ARG;
    if (num_sim) *num_sim = h->scene.numSim;
    if (num_colliders) *num_colliders = int32_t(h->scene.meshes.size()) - h->scene.numSim;
    return GAIA_VBD_OK;
}

int64_t gaia_cloth_num_vertices(gaia_cloth* h, int32_t mesh) {
    return (h && mesh >= 0 && size_t(mesh) < h->scene.meshes.size()) ? h->scene.meshes[mesh].nv : -1;
}
int64_t gaia_cloth_num_faces(gaia_cloth* h, int32_t mesh) {
    return (h && mesh >= 0 && size_t(mesh) < h->scene.meshes.size()) ? h->scene.meshes[mesh].nf : -1;
}
int64_t gaia_cloth_num_edges(gaia_cloth* h, int32_t mesh) {
    return (h && mesh >= 0 && size_t(mesh) < h->scene.meshes.size()) ? h->scene.meshes[mesh].ne : -1;
}

int gaia_cloth_get_positions(gaia_cloth* h, int32_t mesh, double* xyz) {
    if (!mesh_ok(h, mesh) || !xyz) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->get_positions(mesh, xyz); });
}
int gaia_cloth_set_positions(gaia_cloth* h, int32_t mesh, const double* xyz) {
    if (!mesh_ok(h, mesh) || !xyz) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->set_positions(mesh, xyz); });
}
int gaia_cloth_get_velocities(gaia_cloth* h, int32_t mesh, double* xyz) {
    if (!mesh_ok(h, mesh) || !xyz) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->get_velocities(mesh, xyz); });
}
int gaia_cloth_set_velocities(gaia_cloth* h, int32_t mesh, const double* xyz) {
    if (!mesh_ok(h, mesh) || !xyz) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->set_velocities(mesh, xyz); });
}

int gaia_cloth_get_topology(gaia_cloth* h, int32_t mesh, int32_t* edges6, int32_t* face_edges3) {
    if (!h || mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) return GAIA_VBD_E_INVALID_ARG;
    const gaia::cloth::TriMesh& m = h->scene.meshes[mesh];
    if (edges6)
        for (int e = 0; e < m.ne; ++e) {
            const gaia::cloth::Edge& E = m.edges[e];
            int32_t* r = edges6 + 6 * size_t(e);
            r[0] = E.v1;
            r[1] = E.v2;
            r[2] = E.v12next;
            r[3] = E.v21next;
            r[4] = E.f1;
            r[5] = E.f2;
        }
    if (face_edges3) std::memcpy(face_edges3, m.faceEdges.data(), m.faceEdges.size() * sizeof(int32_t));
    return GAIA_VBD_OK;
}

int gaia_cloth_get_rest_shape(gaia_cloth* h, int32_t mesh, double* dminv4, double* area, double* mass) {
    if (!h || mesh < 0 || mesh >= h->scene.numSim) return GAIA_VBD_E_INVALID_ARG;
    const gaia::cloth::TriMesh& m = h->scene.meshes[mesh];
    if (dminv4) std::memcpy(dminv4, m.dminv.data(), m.dminv.size() * sizeof(double));
    if (area) std::memcpy(area, m.area.data(), m.area.size() * sizeof(double));
    if (mass) std::memcpy(mass, m.mass.data(), m.mass.size() * sizeof(double));
    return GAIA_VBD_OK;
}

int gaia_cloth_num_groups(gaia_cloth* h) { return h ? int(h->scene.groups.size()) : -1; }

int64_t gaia_cloth_group_size(gaia_cloth* h, int32_t g) {
    if (!h || g < 0 || size_t(g) >= h->scene.groups.size()) return -1;
    return int64_t(h->scene.groups[g].size() / 2);
}

int gaia_cloth_get_group(gaia_cloth* h, int32_t g, int32_t* pairs) {
    if (!h || !pairs || g < 0 || size_t(g) >= h->scene.groups.size()) return GAIA_VBD_E_INVALID_ARG;
    std::memcpy(pairs, h->scene.groups[g].data(), h->scene.groups[g].size() * sizeof(int32_t));
    return GAIA_VBD_OK;
}

int gaia_cloth_detect(gaia_cloth* h) {
    if (!h || !h->eng) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->detect(); });
}

int gaia_cloth_get_vf_contacts(gaia_cloth* h, int32_t* rows4, int64_t cap, int64_t* n) {
    if (!h || !h->eng || !n || cap < 0 || (cap > 0 && !rows4)) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        std::vector<int32_t> r;
        h->eng->vf_contacts(r);
        *n = int64_t(r.size() / 4);
        std::memcpy(rows4, r.data(), size_t(std::min<int64_t>(cap, *n)) * 4 * sizeof(int32_t));
    });
}

int gaia_cloth_get_ee_contacts(gaia_cloth* h, int32_t* rows4, int64_t cap, int64_t* n) {
    if (!h || !h->eng || !n || cap < 0 || (cap > 0 && !rows4)) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        std::vector<int32_t> r;
        h->eng->ee_contacts(r);
        *n = int64_t(r.size() / 4);
        std::memcpy(rows4, r.data(), size_t(std::min<int64_t>(cap, *n)) * 4 * sizeof(int32_t));
    });
}

int gaia_cloth_get_bounds(gaia_cloth* h, int32_t mesh, double* bounds) {
    if (!mesh_ok(h, mesh) || !bounds) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->bounds(mesh, bounds); });
}

int gaia_cloth_get_min_distances(gaia_cloth* h, int32_t mesh, float* vertex_face, float* face_vertex, float* edge_edge) {
    if (!mesh_ok(h, mesh)) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->min_distances(mesh, vertex_face, face_vertex, edge_edge); });
}

int gaia_cloth_vertex_force_hessian(gaia_cloth* h, int32_t mesh, int32_t v, double* f3, double* h9) {
    if (!h || !h->eng || !f3 || !h9) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->vertex_force_hessian(mesh, v, f3, h9); });
}

int gaia_cloth_autotune(gaia_cloth* h) {
    if (!h || !h->eng) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->autotune(); });
}

int gaia_cloth_get_group_lanes(gaia_cloth* h, int32_t* lanes) {
    if (!h || !h->eng || !lanes) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] {
        std::vector<int> L;
        h->eng->lanes(L);
        std::memcpy(lanes, L.data(), L.size() * sizeof(int32_t));
    });
}

int gaia_cloth_time_solve(gaia_cloth* h, int32_t reps, float* ms_per_sweep) {
    if (!h || !h->eng || !ms_per_sweep || reps <= 0) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { *ms_per_sweep = h->eng->time_solve(reps); });
}

int gaia_cloth_get_stats(gaia_cloth* h, gaia_cloth_stats* out) {
    if (!h || !h->eng || !out) return GAIA_VBD_E_INVALID_ARG;
    return cguard(h, [&] { h->eng->stats(out); });
}

static int32_t color_tri(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t* colors, bool mcs) {
    if (nv <= 0 || nf < 0 || !faces || !colors) return -1;
    try {
        gaia::cloth::TriMesh m;
        m.X.assign(3 * size_t(nv), 0.f);
        m.faces.assign(faces, faces + 3 * size_t(nf));
        for (int32_t v : m.faces)
            if (v < 0 || v >= nv) return -1;
        gaia::cloth::build_topology(m);
        std::vector<int64_t> ofs;
        std::vector<int32_t> adj;
        gaia::cloth::tri_vertex_graph(m, bending != 0, ofs, adj);
        return mcs ? gaia::color_mcs_graph(nv, ofs, adj, colors) : gaia::color_greedy_graph(nv, ofs, adj, colors);
    } catch (const std::exception& e) {
        gaia::set_last_global_error(e.what());
        return -1;
    }
}

int32_t gaia_cloth_color_greedy(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t* colors) {
    return color_tri(nv, nf, faces, bending, colors, false);
}

int32_t gaia_cloth_color_mcs(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t* colors) {
    return color_tri(nv, nf, faces, bending, colors, true);
}

int32_t gaia_cloth_color_tool(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t algorithm,
                              int32_t balance, float goal_ratio, int32_t* colors, int32_t* order) {
    if (nv <= 0 || nf < 0 || !faces || !colors || (algorithm != 0 && algorithm != 1)) return -1;
    try {
        gaia::cloth::TriMesh m;
        m.X.assign(3 * size_t(nv), 0.f);
        m.faces.assign(faces, faces + 3 * size_t(nf));
        for (int32_t v : m.faces)
            if (v < 0 || v >= nv) return -1;
        gaia::cloth::build_topology(m);
        std::vector<int64_t> ofs;
        std::vector<int32_t> adj;
        gaia::cloth::tri_vertex_graph(m, bending != 0, ofs, adj);
        const int32_t n = algorithm == 0 ? gaia::color_mcs_graph(nv, ofs, adj, colors)
                                         : gaia::color_greedy_graph(nv, ofs, adj, colors);
        auto cats = gaia::colors_to_categories(nv, colors);
        if (balance) gaia::balance_categories(nv, ofs, adj, colors, cats, goal_ratio);
        if (order) {
            size_t k = 0;
            for (auto& c : cats)
                for (int32_t v : c) order[k++] = v;
        }
        return n;
    } catch (const std::exception& e) {
        gaia::set_last_global_error(e.what());
        return -1;
    }
}

}  // extern "C"
