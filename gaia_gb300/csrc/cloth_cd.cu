// GPU contact detection of the cloth VBD step. See cloth_cd.hpp.
//
// This translation unit is compiled with --fmad=false: every predicate of the
// narrow phase rounds exactly like the CPU restatement of the same formulas.
#include <cub/cub.cuh>

#include <stdexcept>
#include <string>

#include "cloth_cd.hpp"
#include "cloth_dev.cuh"

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

// Order-preserving int encoding of a float (for atomicMin / atomicMax on floats).
__device__ __forceinline__ int ford(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fdec(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ unsigned int expand_bits(unsigned int v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Primitive kinds: 0 = face (3 vertices), 1 = edge (2 vertices).
template <int KIND>
__device__ __forceinline__ void prim_box(const CDTopo& t, const float4* xf, int p, float3& lo, float3& hi) {
    if (KIND == 0) {
        const int4 f = t.faces[p];
        const float3 a = ld3(xf, f.x), b = ld3(xf, f.y), c = ld3(xf, f.z);
        lo = v3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
        hi = v3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
    } else {
        const int4 e = t.edges[p];
        const float3 a = ld3(xf, e.x), b = ld3(xf, e.y);
        lo = v3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z));
        hi = v3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z));
    }
}

struct MinOp {
    __device__ __forceinline__ float operator()(float a, float b) const { return fminf(a, b); }
};

template <int KIND>
__global__ void k_centroid_bounds(CDTopo t, const float4* xf, int n, int* bounds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float3 lo = v3(3.4e38f, 3.4e38f, 3.4e38f), hi = v3(-3.4e38f, -3.4e38f, -3.4e38f);
    if (i < n) {
        float3 a, b;
        prim_box<KIND>(t, xf, i, a, b);
        lo = v3(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z));
        hi = lo;
    }
    using BR = cub::BlockReduce<float, 256>;
    __shared__ typename BR::TempStorage tmp;
    float vals[6] = {lo.x, lo.y, lo.z, -hi.x, -hi.y, -hi.z};
    for (int k = 0; k < 6; ++k) {
        float m = BR(tmp).Reduce(vals[k], MinOp());
        __syncthreads();
        if (threadIdx.x == 0) atomicMin(&bounds[k], ford(m));
    }
}

__global__ void k_bounds_init(int* bounds) {
    if (threadIdx.x < 6) bounds[threadIdx.x] = ford(3.4e38f);
}

template <int KIND>
__global__ void k_morton(CDTopo t, const float4* xf, int n, const int* bounds, unsigned long long* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 a, b;
    prim_box<KIND>(t, xf, i, a, b);
    const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned int code = 0;
    for (int k = 0; k < 3; ++k) {
        const float lo = fdec(bounds[k]), hi = -fdec(bounds[3 + k]);
        const float ext = hi - lo;
        float u = ext > 0.f ? (c[k] - lo) / ext : 0.f;
        u = fminf(fmaxf(u * 1024.f, 0.f), 1023.f);
        code |= expand_bits((unsigned int)u) << (2 - k);
    }
    keys[i] = (static_cast<unsigned long long>(code) << 32) | static_cast<unsigned int>(i);
}

__device__ __forceinline__ int delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    return __clzll(k[i] ^ k[j]);
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and k-d
// trees": internal node i spans a key range found by binary search; keys are unique.
__global__ void k_karras(const unsigned long long* keys, int n, int2* child, int* parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int s = lmax / 2; s >= 1; s /= 2)
        if (delta(keys, n, i, i + (l + s) * d) > dmin) l += s;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0, tt = l;
    do {
        tt = (tt + 1) >> 1;
        if (delta(keys, n, i, i + (s + tt) * d) > dnode) s += tt;
    } while (tt > 1);
    const int gamma = i + s * d + min(d, 0);
    const int left = (min(i, j) == gamma) ? (n - 1) + gamma : gamma;
    const int right = (max(i, j) == gamma + 1) ? (n - 1) + gamma + 1 : gamma + 1;
    child[i] = make_int2(left, right);
    parent[left] = i;
    parent[right] = i;
    if (i == 0) parent[0] = -1;
}

// Leaf boxes from the current positions, then bottom-up unions: the second thread to
// reach an internal node computes its box (the first returns) and resets its flag.
template <int KIND>
__global__ void k_refit(CDTopo t, const float4* xf, int n, const unsigned long long* keys, const int2* child,
                        const int* parent, float4* bmin, float4* bmax, int* flags, const int* req) {
    if (req && *req == 0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int node = (n - 1) + i;
    float3 lo, hi;
    prim_box<KIND>(t, xf, int(keys[i] & 0xffffffffull), lo, hi);
    bmin[node] = make_float4(lo.x, lo.y, lo.z, 0.f);
    bmax[node] = make_float4(hi.x, hi.y, hi.z, 0.f);
    if (n == 1) return;
    __threadfence();
    int p = parent[node];
    while (p >= 0) {
        if (atomicAdd(&flags[p], 1) == 0) return;
        flags[p] = 0;
        __threadfence();
        const int2 c = child[p];
        const float4 l0 = __ldcg(&bmin[c.x]), l1 = __ldcg(&bmax[c.x]);
        const float4 r0 = __ldcg(&bmin[c.y]), r1 = __ldcg(&bmax[c.y]);
        bmin[p] = make_float4(fminf(l0.x, r0.x), fminf(l0.y, r0.y), fminf(l0.z, r0.z), 0.f);
        bmax[p] = make_float4(fmaxf(l1.x, r1.x), fmaxf(l1.y, r1.y), fmaxf(l1.z, r1.z), 0.f);
        __threadfence();
        p = parent[p];
    }
}

struct LbvhDev {
    int n;
    const unsigned long long* keys;
    const int2* child;
    const float4* bmin;
    const float4* bmax;
};

__device__ __forceinline__ bool sphere_box(float3 p, float r2, float4 lo, float4 hi) {
    const float dx = fmaxf(fmaxf(lo.x - p.x, 0.f), p.x - hi.x);
    const float dy = fmaxf(fmaxf(lo.y - p.y, 0.f), p.y - hi.y);
    const float dz = fmaxf(fmaxf(lo.z - p.z, 0.f), p.z - hi.z);
    return dx * dx + dy * dy + dz * dz <= r2;
}

// Visits every primitive whose box is within sqrt(r2) of p (stack traversal).
template <typename F>
__device__ __forceinline__ void traverse(const LbvhDev& b, float3 p, float r2, unsigned long long* counters, F&& leaf) {
    if (b.n <= 0) return;
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        if (!sphere_box(p, r2, b.bmin[node], b.bmax[node])) continue;
        if (node >= b.n - 1) {
            leaf(int(b.keys[node - (b.n - 1)] & 0xffffffffull));
        } else {
            if (sp + 2 > 64) {
                atomicAdd(&counters[CC_STACK_OVERFLOW], 1ull);
                continue;
            }
            const int2 c = b.child[node];
            stack[sp++] = c.y;
            stack[sp++] = c.x;
        }
    }
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
// back to the face.
__global__ void __launch_bounds__(128) k_vf_query(CDTopo t, LbvhDev fb, const float4* xf, float r, CDOut o,
                                                  const int* req) {
    if (*req == 0) return;
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= t.nV) return;
    const float3 p = ld3(xf, v);
    const int2 vi = t.vInfo[v];
    const bool vSim = vi.x < t.numSimMeshes;
    float minDis = r;
    int cf[CAND_CAP];
    unsigned char ct[CAND_CAP];
    int nc = 0;
    const float rq = r * 1.0001f;
    traverse(fb, p, rq * rq, o.counters, [&](int f) {
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
__global__ void __launch_bounds__(128) k_ee_query(CDTopo t, LbvhDev eb, const float4* xf, float r, CDOut o,
                                                  const int* req) {
    if (*req == 0) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= t.nSimE) return;
    const int4 E = t.edges[e];
    const int m1 = t.edgeInfo[e].z;
    const float3 p1 = ld3(xf, E.x), p2 = ld3(xf, E.y);
    const float3 dd = sub(p1, p2);
    const float eLen = sqrtf(dot(dd, dd));
    const float3 c = mul(0.5f, add(p1, p2));
    const float rq = (r + eLen * 0.5f) * 1.0001f;
    float minDis = r;
    int cand[CAND_CAP];
    int nc = 0;
    traverse(eb, c, rq * rq, o.counters, [&](int e2) {
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

class Lbvh {
public:
    int n = 0;
    int kind = 0;
    unsigned long long* keys = nullptr;
    unsigned long long* keysTmp = nullptr;
    int2* child = nullptr;
    int* parent = nullptr;
    float4* bmin = nullptr;
    float4* bmax = nullptr;
    int* flags = nullptr;
    int* bounds = nullptr;
    void* temp = nullptr;
    size_t tempBytes = 0;

    void alloc(int n_, int kind_, size_t& bytes) {
        n = n_;
        kind = kind_;
        if (n == 0) return;
        keys = dalloc<unsigned long long>(n, bytes);
        keysTmp = dalloc<unsigned long long>(n, bytes);
        child = dalloc<int2>(std::max(n - 1, 1), bytes);
        parent = dalloc<int>(2 * n - 1, bytes);
        bmin = dalloc<float4>(2 * n - 1, bytes);
        bmax = dalloc<float4>(2 * n - 1, bytes);
        flags = dalloc<int>(std::max(n - 1, 1), bytes);
        bounds = dalloc<int>(6, bytes);
        CD_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tempBytes, keysTmp, keys, n, 0, 62));
        temp = dalloc<char>(tempBytes, bytes);
        CD_CUDA(cudaMemset(flags, 0, sizeof(int) * std::max(n - 1, 1)));
        CD_CUDA(cudaMemset(parent, 0xff, sizeof(int) * (2 * n - 1)));
    }
    void release() {
        for (void* p : {(void*)keys, (void*)keysTmp, (void*)child, (void*)parent, (void*)bmin, (void*)bmax,
                        (void*)flags, (void*)bounds, temp})
            if (p) cudaFree(p);
        keys = keysTmp = nullptr;
        child = nullptr;
        parent = flags = bounds = nullptr;
        bmin = bmax = nullptr;
        temp = nullptr;
    }
    void build(const CDTopo& t, const float4* xf, cudaStream_t st) {
        if (n == 0) return;
        k_bounds_init<<<1, 32, 0, st>>>(bounds);
        if (kind == 0) {
            k_centroid_bounds<0><<<blocks(n, 256), 256, 0, st>>>(t, xf, n, bounds);
            k_morton<0><<<blocks(n, 256), 256, 0, st>>>(t, xf, n, bounds, keysTmp);
        } else {
            k_centroid_bounds<1><<<blocks(n, 256), 256, 0, st>>>(t, xf, n, bounds);
            k_morton<1><<<blocks(n, 256), 256, 0, st>>>(t, xf, n, bounds, keysTmp);
        }
        size_t tb = tempBytes;
        CD_CUDA(cub::DeviceRadixSort::SortKeys(temp, tb, keysTmp, keys, n, 0, 62, st));
        if (n > 1) k_karras<<<blocks(n - 1, 256), 256, 0, st>>>(keys, n, child, parent);
        refit(t, xf, nullptr, st);
        CD_CUDA(cudaGetLastError());
    }
    void refit(const CDTopo& t, const float4* xf, const int* req, cudaStream_t st) {
        if (n == 0) return;
        if (kind == 0)
            k_refit<0><<<blocks(n, 256), 256, 0, st>>>(t, xf, n, keys, child, parent, bmin, bmax, flags, req);
        else
            k_refit<1><<<blocks(n, 256), 256, 0, st>>>(t, xf, n, keys, child, parent, bmin, bmax, flags, req);
    }
    LbvhDev dev() const { return LbvhDev{n, keys, child, bmin, bmax}; }
};

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
    faceBvh_->alloc(t.nF, 0, bytes_);
    edgeBvh_->alloc(t.nE, 1, bytes_);
}

void ContactDetector::rebuild(const float4* xf, cudaStream_t st) {
    faceBvh_->build(t_, xf, st);
    edgeBvh_->build(t_, xf, st);
}

void ContactDetector::enqueue_detect(const float4* xf, float maxQueryDis, const int* d_req, cudaStream_t st) {
    faceBvh_->refit(t_, xf, d_req, st);
    edgeBvh_->refit(t_, xf, d_req, st);
    const int nr = std::max(t_.nF, 1);
    k_cd_reset<<<blocks(nr, 256), 256, 0, st>>>(t_, out_, maxQueryDis, d_req);
    if (t_.nV > 0) k_vf_query<<<blocks(t_.nV, 128), 128, 0, st>>>(t_, faceBvh_->dev(), xf, maxQueryDis, out_, d_req);
    if (t_.nSimF > 0) k_fv_sort<<<blocks(t_.nSimF, 128), 128, 0, st>>>(t_, out_, d_req);
    if (t_.nSimE > 0) k_ee_query<<<blocks(t_.nSimE, 128), 128, 0, st>>>(t_, edgeBvh_->dev(), xf, maxQueryDis, out_, d_req);
    CD_CUDA(cudaGetLastError());
}

}  // namespace cloth
}  // namespace gaia
