// GPU contact detection of the cloth VBD step. See cloth_cd.hpp.
//
// This translation unit is compiled with --fmad=false: every predicate of the
// narrow phase rounds exactly like the CPU restatement of the same formulas.
#include <cub/cub.cuh>

#include <stdexcept>
#include <string>

#include "cloth_cd.hpp"
#include "cloth_dev.cuh"
#include "lbvh.cuh"

namespace gaia {
namespace cloth {

namespace {

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
#define CD_CUDA(x) check((x), #x)

template <typename T>
T* dalloc(size_t n, size_t& bytes) {
    T* p = nullptr;
    if (n == 0) n = 1;
    CD_CUDA(cudaMalloc(&p, n * sizeof(T)));
    bytes += n * sizeof(T);
    return p;
}

// checkVertexFeasibleRegion (CollisionDetector/TriMeshCollisionGeometry.cpp:162-195)
__device__ bool vertex_feasible(const CDTopo& t, const float4* xf, float3 p, int a) {
    const float3 A = ld3(xf, a);
    const float3 AP = sub(p, A);
    const float relaxed = -FEASIBLE_EPS - ABS_RELAX;
    for (int k = t.nbrVOfs[a]; k < t.nbrVOfs[a + 1]; ++k) {
        const float3 BA = sub(A, ld3(xf, t.nbrV[k]));
        if (dot(AP, BA) < relaxed) return false;
    }
    return true;
}

// checkEdgeFeasibleRegion (TriMeshCollisionGeometry.cpp:104-160)
__device__ bool edge_feasible(const CDTopo& t, const float4* xf, float3 p, int e) {
    const int4 E = t.edges[e];
    const float3 v1 = ld3(xf, E.x), v2 = ld3(xf, E.y);
    const float3 AP = sub(p, v1), BP = sub(p, v2), AB = sub(v2, v1);
    const float relaxed = FEASIBLE_EPS + ABS_RELAX;
    if (dot(AP, AB) < -relaxed) return false;
    if (dot(BP, AB) > relaxed) return false;
    const float ABsq = dot(AB, AB);
    if (ABsq < CMP_EPS2) return false;
    const int opp[2] = {E.z, E.w};
    for (int k = 0; k < 2; ++k) {
        if (opp[k] == -1) continue;
        const float3 vo = ld3(xf, opp[k]);
        const float tt = dot(AB, sub(vo, v1)) / ABsq;
        const float3 foot = add(v1, mul(tt, AB));
        if (dot(sub(vo, foot), sub(p, foot)) > relaxed) return false;
    }
    return true;
}

// checkFeasibleRegion (TriMeshCollisionGeometry.cpp:7-44)
__device__ bool feasible(const CDTopo& t, const float4* xf, float3 p, int f, int type) {
    const int4 fv = t.faces[f];
    const int4 fe = t.faceEdges[f];
    switch (type) {
        case AtInterior: return true;
        case AtAB: return edge_feasible(t, xf, p, fe.x);
        case AtBC: return edge_feasible(t, xf, p, fe.y);
        case AtAC: return edge_feasible(t, xf, p, fe.z);
        case AtA: return vertex_feasible(t, xf, p, fv.x);
        case AtB: return vertex_feasible(t, xf, p, fv.y);
        case AtC: return vertex_feasible(t, xf, p, fv.z);
        default: return false;
    }
}

__global__ void k_cd_reset(CDTopo t, CDOut o, float maxQueryDis, const int* req) {
    if (*req == 0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < t.nF) o.fMinDisBits[i] = __float_as_int(maxQueryDis);
    if (i < t.nSimF) o.fvCount[i] = 0;
    if (i == 0) atomicAdd(&o.counters[CC_DETECTIONS], 1ull);
}

// Vertex-face radius query of one vertex (all meshes' vertices):
// triMeshVFRadiusQueryWithTopologyFilteringAndFaceMinDisCaculatingFunc and its collider
// variant (ClothContactDetector.cpp:144-288, 440-560). Candidates within the query radius
// update the vertex's and the face's minimum distance; they are then taken in ascending
// face order, de-duplicated on (closest-point primitive type, mesh-local primitive id),
// checked for the feasible region and recorded; contacts on simulated faces are linked
// back to the face. Thread v takes vertex v (grid order: a warp's vertices are neighbours in
// space), and the warp walks the face hierarchy once for all of them (traverse_warp).
__global__ void __launch_bounds__(128) k_vf_query(CDTopo t, bvh::LbvhDev fb, const float4* xf, float r, CDOut o,
                                                  const int* req) {
    if (*req == 0) return;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = v < t.nV;  // every lane walks with the warp; lanes past the end without a query
    const float3 p = valid ? ld3(xf, v) : v3(0.f, 0.f, 0.f);
    const int2 vi = valid ? t.vInfo[v] : make_int2(0, 0);
    const bool vSim = vi.x < t.numSimMeshes;
    float minDis = r;
    int cf[CAND_CAP];
    unsigned char ct[CAND_CAP];
    int nc = 0;
    const float rq = r * 1.0001f;
    bvh::traverse_warp(fb, p, rq * rq, valid, o.counters, [&](int f) {
        const int4 fv = t.faces[f];
        const bool fSim = fv.w < t.numSimMeshes;
        if (!fSim && !vSim) return;
        if (fv.w == vi.x && (fv.x == v || fv.y == v || fv.z == v)) return;
        float3 bary, cp;
        const int type = closest_point_triangle<float3, float>(p, ld3(xf, fv.x), ld3(xf, fv.y), ld3(xf, fv.z), bary, cp);
        const float3 df = sub(p, cp);
        const float d = sqrtf(dot(df, df));
        if (!(d < r)) return;
        minDis = fminf(minDis, d);
        atomicMin(&o.fMinDisBits[f], __float_as_int(d));
        if (nc < CAND_CAP) {
            cf[nc] = f;
            ct[nc] = (unsigned char)type;
            ++nc;
        } else {
            atomicAdd(&o.counters[CC_CAND_OVERFLOW], 1ull);
        }
    });
    if (!valid) return;
    // ascending face order
    for (int a = 1; a < nc; ++a) {
        const int kf = cf[a];
        const unsigned char kt = ct[a];
        int b = a - 1;
        while (b >= 0 && cf[b] > kf) {
            cf[b + 1] = cf[b];
            ct[b + 1] = ct[b];
            --b;
        }
        cf[b + 1] = kf;
        ct[b + 1] = kt;
    }
    int accType[VF_CAP], accId[VF_CAP];
    int na = 0;
    for (int a = 0; a < nc; ++a) {
        const int f = cf[a], type = ct[a];
        const int4 fv = t.faces[f];
        const int4 fe = t.faceEdges[f];
        int pid = -1;
        switch (type) {
            case AtA: pid = t.vInfo[fv.x].y; break;
            case AtB: pid = t.vInfo[fv.y].y; break;
            case AtC: pid = t.vInfo[fv.z].y; break;
            case AtAB: pid = t.edgeInfo[fe.x].w; break;
            case AtBC: pid = t.edgeInfo[fe.y].w; break;
            case AtAC: pid = t.edgeInfo[fe.z].w; break;
            case AtInterior: pid = fe.w; break;
            default: break;
        }
        const int pt = prim_type(type);
        bool dup = false;
        for (int k = 0; k < na; ++k)
            if (accType[k] == pt && accId[k] == pid) dup = true;
        if (dup) continue;
        if (!feasible(t, xf, p, f, type)) continue;
        if (na >= VF_CAP) {
            atomicAdd(&o.counters[CC_VF_OVERFLOW], 1ull);
            break;
        }
        accType[na] = pt;
        accId[na] = pid;
        o.vfFace[size_t(v) * VF_CAP + na] = f;
        ++na;
        if (f < t.nSimF) {
            const int slot = atomicAdd(&o.fvCount[f], 1);
            if (slot < FV_CAP) o.fvVert[size_t(f) * FV_CAP + slot] = v;
            else atomicAdd(&o.counters[CC_FV_OVERFLOW], 1ull);
        }
    }
    o.vfCount[v] = na;
    o.vfMinDis[v] = minDis;
}

// The vertices linked to each face in ascending order (the links arrive in any order).
__global__ void k_fv_sort(CDTopo t, CDOut o, const int* req) {
    if (*req == 0) return;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= t.nSimF) return;
    const int n = min(o.fvCount[f], FV_CAP);
    int* a = o.fvVert + size_t(f) * FV_CAP;
    for (int i = 1; i < n; ++i) {
        const int k = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > k) {
            a[j + 1] = a[j];
            --j;
        }
        a[j + 1] = k;
    }
}

// Edge-edge query of one simulated edge: triMeshEdgeContactQueryFunc
// (ClothContactDetector.cpp:731-813) with the query sphere of contactQueryEE
// (:1106-1135): centre at the edge midpoint, radius maxQueryDis + half the edge length.
// Thread i takes the edge of leaf i of the edge hierarchy (Morton order of the last build),
// so the queries of a warp are neighbours in space, and the warp walks the hierarchy once
// for all of them (traverse_warp); leaves of collider edges have no query.
__global__ void __launch_bounds__(128) k_ee_query(CDTopo t, bvh::LbvhDev eb, const float4* xf, float r, CDOut o,
                                                  const int* req) {
    if (*req == 0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int e = i < eb.n ? int(eb.keys[i] & 0xffffffffull) : -1;
    const bool valid = e >= 0 && e < t.nSimE;  // lanes past the end or on collider edges walk without a query
    if (!valid) e = 0;
    const int4 E = valid ? t.edges[e] : make_int4(0, 0, 0, 0);
    const int m1 = valid ? t.edgeInfo[e].z : -1;
    const float3 p1 = valid ? ld3(xf, E.x) : v3(0.f, 0.f, 0.f), p2 = valid ? ld3(xf, E.y) : p1;
    const float3 dd = sub(p1, p2);
    const float eLen = sqrtf(dot(dd, dd));
    const float3 c = mul(0.5f, add(p1, p2));
    const float rq = (r + eLen * 0.5f) * 1.0001f;
    float minDis = r;
    int cand[CAND_CAP];
    int nc = 0;
    bvh::traverse_warp(eb, c, rq * rq, valid, o.counters, [&](int e2) {
        const int4 F = t.edges[e2];
        const int m2 = t.edgeInfo[e2].z;
        if (m1 == m2) {
            if (e2 == e) return;
            if (E.x == F.x || E.x == F.y || E.y == F.x || E.y == F.y) return;
        }
        const float3 q1 = ld3(xf, F.x), q2 = ld3(xf, F.y);
        float3 c1, c2;
        float s, tt;
        closest_points_segments(p1, p2, q1, q2, c1, c2, s, tt);
        const float3 df = sub(c1, c2);
        const float d = sqrtf(dot(df, df));
        minDis = fminf(minDis, d);
        if (!(d < r)) return;
        const float3 ev1 = sub(p2, p1), ev2 = sub(q2, q1);
        const bool ok = (dot(sub(c2, p1), ev1) >= 0.f && dot(sub(p2, c2), ev1) >= 0.f) ||
                        (dot(sub(c1, q1), ev2) >= 0.f && dot(sub(q2, c1), ev2) >= 0.f);
        if (!ok) return;
        if (nc < CAND_CAP) cand[nc++] = e2;
        else atomicAdd(&o.counters[CC_CAND_OVERFLOW], 1ull);
    });
    if (!valid) return;
    for (int a = 1; a < nc; ++a) {
        const int k = cand[a];
        int b = a - 1;
        while (b >= 0 && cand[b] > k) {
            cand[b + 1] = cand[b];
            --b;
        }
        cand[b + 1] = k;
    }
    if (nc > EE_CAP) {
        atomicAdd(&o.counters[CC_EE_OVERFLOW], 1ull);
        nc = EE_CAP;
    }
    for (int a = 0; a < nc; ++a) o.eeOther[size_t(e) * EE_CAP + a] = cand[a];
    o.eeCount[e] = nc;
    o.eeMinDis[e] = minDis;
}

inline int blocks(int n, int b) { return (n + b - 1) / b; }

}  // namespace

// The detector's hierarchies (the header names the type without the BVH code).
class Lbvh : public bvh::Lbvh {};

ContactDetector::~ContactDetector() {
    if (faceBvh_) {
        faceBvh_->release();
        delete faceBvh_;
    }
    if (edgeBvh_) {
        edgeBvh_->release();
        delete edgeBvh_;
    }

    for (void* p : {(void*)out_.vfFace, (void*)out_.vfCount, (void*)out_.vfMinDis, (void*)out_.fMinDisBits,
                    (void*)out_.fvVert, (void*)out_.fvCount, (void*)out_.eeOther, (void*)out_.eeCount,
                    (void*)out_.eeMinDis})
        if (p) cudaFree(p);
}

void ContactDetector::init(const CDTopo& t, unsigned long long* counters, cudaStream_t st) {
    t_ = t;
    out_.counters = counters;
    out_.vfFace = dalloc<int>(size_t(t.nV) * VF_CAP, bytes_);
    out_.vfCount = dalloc<int>(t.nV, bytes_);
    out_.vfMinDis = dalloc<float>(t.nV, bytes_);
    out_.fMinDisBits = dalloc<int>(t.nF, bytes_);
    out_.fvVert = dalloc<int>(size_t(t.nSimF) * FV_CAP, bytes_);
    out_.fvCount = dalloc<int>(t.nSimF, bytes_);
    out_.eeOther = dalloc<int>(size_t(t.nSimE) * EE_CAP, bytes_);
    out_.eeCount = dalloc<int>(t.nSimE, bytes_);
    out_.eeMinDis = dalloc<float>(t.nSimE, bytes_);
    CD_CUDA(cudaMemsetAsync(out_.vfCount, 0, sizeof(int) * std::max(t.nV, 1), st));
    CD_CUDA(cudaMemsetAsync(out_.fvCount, 0, sizeof(int) * std::max(t.nSimF, 1), st));
    CD_CUDA(cudaMemsetAsync(out_.eeCount, 0, sizeof(int) * std::max(t.nSimE, 1), st));
    faceBvh_ = new Lbvh();
    edgeBvh_ = new Lbvh();
    faceBvh_->alloc(t.nF, bvh::Prims{t.faces, 3}, bytes_);
    edgeBvh_->alloc(t.nE, bvh::Prims{t.edges, 2}, bytes_);
}

void ContactDetector::rebuild(const float4* xf, cudaStream_t st) {
    faceBvh_->build(xf, st);
    edgeBvh_->build(xf, st);
}

void ContactDetector::enqueue_detect(const float4* xf, float maxQueryDis, const int* d_req, cudaStream_t st) {
    faceBvh_->refit(xf, d_req, st);
    edgeBvh_->refit(xf, d_req, st);
    const int nr = std::max(t_.nF, 1);
    k_cd_reset<<<blocks(nr, 256), 256, 0, st>>>(t_, out_, maxQueryDis, d_req);
    if (t_.nV > 0) k_vf_query<<<blocks(t_.nV, 128), 128, 0, st>>>(t_, faceBvh_->dev(), xf, maxQueryDis, out_, d_req);
    if (t_.nSimF > 0) k_fv_sort<<<blocks(t_.nSimF, 128), 128, 0, st>>>(t_, out_, d_req);
    if (t_.nSimE > 0) k_ee_query<<<blocks(t_.nE, 128), 128, 0, st>>>(t_, edgeBvh_->dev(), xf, maxQueryDis, out_, d_req);
    CD_CUDA(cudaGetLastError());
}

}  // namespace cloth
}  // namespace gaia
