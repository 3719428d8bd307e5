// Contact detection of the cloth VBD step on the GPU: linear BVHs over all
// faces and all edges (Morton-ordered, Karras-style hierarchy, refit in place),
// the vertex-face radius query and the edge-edge query with the reference's
// topology filtering, de-duplication and feasible-region tests.
//
// Results do not depend on the BVH's traversal order: narrow-phase candidates
// are gathered first and then filtered in ascending primitive order, which is
// the order the CPU restatement uses. This replaces ClothContactDetector
// (CollisionDetector/ClothContactDetector.cpp:144-288, 731-813, 1052-1135),
// which runs Embree point queries on the host.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace gaia {
namespace cloth {

// Device pointers to the concatenated topology of all meshes (simulated meshes
// first, then colliders).
struct CDTopo {
    int nV = 0, nF = 0, nE = 0;              // all meshes
    int nSimV = 0, nSimF = 0, nSimE = 0;     // simulated prefix
    int numSimMeshes = 0;
    const int4* faces = nullptr;      // v0, v1, v2 (global vertex ids), mesh id
    const int4* faceEdges = nullptr;  // edges AB, BC, CA (global ids), local face id
    const int4* edges = nullptr;      // v1, v2, v12next, v21next (global ids, -1 on a boundary)
    const int4* edgeInfo = nullptr;   // f1, f2 (global ids, -1), mesh id, local edge id
    const int2* vInfo = nullptr;      // mesh id, local vertex id
    const int* nbrVOfs = nullptr;     // all vertices: neighbour vertices (global ids)
    const int* nbrV = nullptr;
};

// Detection results (device arrays owned by the detector).
struct CDOut {
    int* vfFace = nullptr;       // nV * VF_CAP: contacting faces (global ids), ascending
    int* vfCount = nullptr;      // nV
    float* vfMinDis = nullptr;   // nV: min distance to any face within the query radius
    int* fMinDisBits = nullptr;  // nF: per face min distance to any vertex (float bits)
    int* fvVert = nullptr;       // nSimF * FV_CAP: contacting vertices (global ids), ascending
    int* fvCount = nullptr;      // nSimF (may exceed FV_CAP: overflow)
    int* eeOther = nullptr;      // nSimE * EE_CAP: contacting edges (global ids), ascending
    int* eeCount = nullptr;      // nSimE
    float* eeMinDis = nullptr;   // nSimE
    unsigned long long* counters = nullptr;  // CC_* (cloth_dev.cuh)
};

class Lbvh;

class ContactDetector {
public:
    ContactDetector() = default;
    ~ContactDetector();
    ContactDetector(const ContactDetector&) = delete;
    ContactDetector& operator=(const ContactDetector&) = delete;

    // Allocate BVHs and result arrays for `t`; `counters` is a device array of CC_N.
    void init(const CDTopo& t, unsigned long long* counters, cudaStream_t st);
    // Rebuild both hierarchies (Morton codes, sort, topology) from positions `xf`
    // (float4 per vertex, all meshes). Not gated: call it where detection runs.
    void rebuild(const float4* xf, cudaStream_t st);
    // Refit and query when *d_req != 0 (every kernel returns at once otherwise), so
    // the sequence can sit in a CUDA graph and run only when a vertex left its bound.
    void enqueue_detect(const float4* xf, float maxQueryDis, const int* d_req, cudaStream_t st);
    const CDOut& out() const { return out_; }
    const CDTopo& topo() const { return t_; }
    size_t device_bytes() const { return bytes_; }

private:
    CDTopo t_;
    CDOut out_;
    Lbvh* faceBvh_ = nullptr;
    Lbvh* edgeBvh_ = nullptr;
    size_t bytes_ = 0;
};

}  // namespace cloth
}  // namespace gaia
