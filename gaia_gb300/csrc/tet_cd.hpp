// Contact detection of the tet VBD step on the GPU: which surface vertex touches which
// surface face, found once per substep (and optionally every few iterations), and the
// per-vertex contact records the block solve reads.
//
// Reference path: VBDPhysics::dcd / ccd / prepareCollisionDataGPU (VBD/VBDPhysics.cpp:
// 1812-1894, 1958-2156) with Embree's DCD (CollisionDetector/DiscreteCollisionDetector.cpp)
// and CCD (CollisionDetector/ContinuousCollisionDetector.cpp, CCDSolver.h) on the host.
// Here both run as kernels over one LBVH of the moving surface faces and one of the tets
// (lbvh.cuh), with the FP32 predicates evaluated in a fixed operation order without
// contraction so that they match the CPU oracle bit for bit.
//
// Everything is indexed by the engine's vertex slots; positions come in as one float4
// array of 2 * nslots entries: the current positions, then those at the start of the
// substep.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace gaia {
namespace tetcd {

struct Topo {
    int32_t nslots = 0;
    std::vector<int4> faces;        // per surface face (meshes concatenated): slots a, b, c; w = mesh
    std::vector<int4> face_nbr;     // per face: global face across edge AB, BC, CA (-1: none)
    std::vector<int32_t> face_ofs;  // first global face of each mesh (nmesh + 1)
    std::vector<int2> verts;        // per surface vertex (mesh-major, ascending): slot, mesh
    std::vector<int32_t> ring_ofs;  // per slot (nslots + 1): surface neighbours ...
    std::vector<int32_t> ring;      // ... as slots
    std::vector<int4> tets;         // per tet (meshes concatenated): slots
    std::vector<int32_t> tet_mesh;
    std::vector<int4> tet_nbr;      // per tet: global tet across the face omitting vertex x/y/z/w (-1: none)
    std::vector<int2> face_tet;     // per face: the global tet it bounds, the local vertex it omits
};

struct Params {
    bool ccd = true, dcd = true;   // allowCCD, allowDCD
    bool handle_self = true;       // handleSelfCollision
    bool check_feasible = true;    // checkFeasibleRegion
    float feasible_eps = 1e-2f;    // feasibleRegionEpsilon
    float off_height = 1e7f;       // collisionOffHeight (y)
    // the DCD closest-point query's tetrahedral traversal check
    bool check_traverse = true;     // checkTetTraverse
    bool traverse_non_self = true;  // tetrahedralTraverseForNonSelfIntersection
    bool stop_after_passing = true; // stopTraversingAfterPassingQueryPoint
    bool shift_to_center = true;    // shiftQueryPointToCenter
    bool static_traverse = true;    // useStaticTraverse
    float center_shift = 0.01f;     // centerShiftLevel
    float ray_eps = 1e-10f;         // rayTriIntersectionEPSILON
    float max_search_mult = 1.8f;   // maxSearchDistanceMultiplier
};

// What the solve reads, per slot:
//   info: bit 3 = the vertex has its own contact (own[slot]), bits 0-2 = number of
//         relations (contacts whose face holds this vertex, at most 4);
//   own:  the contact face's vertex slots (x, y, z) and mesh (w);
//   rel:  4 per slot, (colliding vertex slot << 2) | vertex order in the face;
//   list: the slots with info != 0, ascending, list[0 .. *nlist).
struct Records {
    const uint8_t* info = nullptr;
    const int4* own = nullptr;
    const int32_t* rel = nullptr;
    const int32_t* list = nullptr;
    const int32_t* nlist = nullptr;
};

class Detector {
public:
    Detector() = default;
    ~Detector();
    Detector(const Detector&) = delete;
    Detector& operator=(const Detector&) = delete;

    void init(const Topo& topo, const Params& prm, size_t& bytes);
    bool enabled() const { return prm_.ccd || prm_.dcd; }
    // Builds the face and tet hierarchies on the given positions (once, outside any
    // stream capture); later passes refit them.
    void build(const float4* xf, cudaStream_t st);
    // Clears every result and record (a state reset).
    void reset(cudaStream_t st);
    // Enqueues one detection pass (see the reference order in tet_cd.cu): at the start
    // of a substep (intermediate = false) or between iterations. rebuild = rebuild the
    // face hierarchy (otherwise refit); the tet hierarchy is refitted only when some tet
    // is large enough for the point-in-tet test.
    void enqueue(const float4* xf, bool intermediate, bool rebuild, cudaStream_t st);
    Records records() const;
    // Host copy of the current contacts: rows of (slot, face global index, hit kind:
    // 1 = CCD, 2 = DCD) for every surface vertex with a contact, in surface order.
    void contacts(std::vector<int32_t>& rows, cudaStream_t st) const;
    int32_t num_faces() const { return nf_; }
    int32_t num_surface_vertices() const { return nsv_; }
    void counters(unsigned long long* out, cudaStream_t st) const;  // CC_* counters of cloth_dev.cuh

private:
    void release();
    Params prm_;
    int32_t nslots_ = 0, nf_ = 0, nsv_ = 0, ntet_ = 0;
    struct Impl;
    Impl* d_ = nullptr;
};

}  // namespace tetcd
}  // namespace gaia
