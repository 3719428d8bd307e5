/*
 * Tet-mesh contact for the CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * Restates, on the CPU, the reference's vertex-face contact path of the GPU VBD
 * step for tet meshes:
 *   - surface extraction (faces that belong to one tet, oriented outward);
 *   - continuous collision detection of every surface vertex's trajectory against
 *     every moving surface triangle (CollisionDetector/ContinuousCollisionDetector.cpp:
 *     66-186, 346-377), with the moving-point / moving-triangle test of
 *     CollisionDetector/CCDSolver.h:97-196 and the cubic root finder it calls
 *     (Simulator/3rdParty/CyCodeBase/cyPolynomial.h: CubicRoots 800-903,
 *     RootFinderNewton::FindClosed 382-450, QuadraticRoots 597-621), evaluated in
 *     FP32 without contraction, as the reference's CCDDType = float;
 *   - the contact records the GPU solve reads (VBD/VBDPhysics.cpp:1812-1894,
 *     prepareCollisionDataGPU) and the per-contact force and Hessian
 *     (VBD/VBDPhysicsCompute.cu:1731-1773, 1812-1930).
 *
 * Parity anchor: the CCD restatement is checked bit-for-bit against the
 * reference's own CCDSolver.h compiled from the reference tree into
 * oracle/_ref/ (oracle/Makefile, target ref) where that tree is present.
 */
#ifndef GAIA_TET_CONTACT_ORACLE_H
#define GAIA_TET_CONTACT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
#include <vector>

namespace oracle_tc {

struct Surface {
    std::vector<int32_t> faces;     // 3 per face, mesh-local vertex ids, outward
    std::vector<int32_t> verts;     // surface vertices, ascending
    std::vector<int32_t> face_nbr;  // 3 per face: the face across edge AB, BC, CA (-1: none)
    std::vector<int32_t> ring_ofs, ring;  // per mesh vertex: its surface neighbours, ascending
    // tetrahedral traversal tables (TetMesh/TetMeshFEM.cpp:40-70, 173-214):
    std::vector<int32_t> face_tet;  // 2 per face: the tet it bounds, the local vertex it omits
    std::vector<int32_t> tet_nbr;   // 4 per tet: the tet across the face omitting local vertex k (-1: none)
};

// Boundary faces of a tet mesh in ascending (tet, local face) order; the face
// opposite local vertex k is (1,2,3), (0,3,2), (0,1,3), (0,2,1) for k = 0..3,
// reversed for tets of negative rest volume.
Surface extract_surface(int nv, int ntet, const int32_t* tets, const double* X);

// Moving point p[0] -> p[1] against the moving triangle x[0][*] -> x[1][*] (xyz
// triples). Returns 1 and the time of impact and the barycentrics on a hit.
int ccd_tri_point(const float x0[9], const float x1[9], const float p0[3], const float p1[3], float* tt,
                  float bary[3]);

// One mesh as the detector sees it: FP32 positions at the start of the substep
// (xprev) and now (x), 3 per vertex, its tets and its surface.
struct CcdMesh {
    const float* x;
    const float* xprev;
    const Surface* surf;
    int32_t ntet;
    const int32_t* tets;
};

struct CcdHit {
    int32_t fmesh = -1, face = -1;  // contact face (mesh, surface face index), -1: none
    float tt = 0.f, depth = 0.f;    // CCD: time of impact and tt * |trajectory|; DCD: tt = -1, distance
    float bary[3] = {0.f, 0.f, 0.f};
};

struct DcdParams {
    bool handle_self = true;       // handleSelfCollision
    bool check_feasible = true;    // checkFeasibleRegion
    float feasible_eps = 1e-2f;    // feasibleRegionEpsilon
    // the tetrahedral traversal check of the closest-point query
    // (CollisionDetector/CollisionDetertionParameters.h:51-77)
    bool check_traverse = true;     // checkTetTraverse
    bool traverse_non_self = true;  // tetrahedralTraverseForNonSelfIntersection
    bool stop_after_passing = true; // stopTraversingAfterPassingQueryPoint
    bool shift_to_center = true;    // shiftQueryPointToCenter
    bool static_traverse = true;    // useStaticTraverse
    float center_shift = 0.01f;     // centerShiftLevel
    float ray_eps = 1e-10f;         // rayTriIntersectionEPSILON
    float max_search_mult = 1.8f;   // maxSearchDistanceMultiplier
};

// Walk from surface face `face` of a mesh, along the ray from `origin` in direction `dir`,
// through the tets (tetrahedralTraverseTo / tetrahedralTraverseToDynamic,
// TetMesh/TetMeshFEM.cpp:503-740, 908-1100): true when the walk reaches `target`.
// max_dis <= 0 turns the pass-through test off. `status` gets 0, or 1 when the walk
// gave up on its size bounds (candidate stack or step count).
bool tet_traverse(const float* X, const int32_t* tets, const Surface& s, const float origin[3], const float dir[3],
                  float max_dis, int32_t face, int32_t target, float ray_eps, bool use_static, int* status);

// The two detectors of the tet-mesh contact path over all meshes:
//   ccd(m, i): vertexContinuousCollisionDetection (ContinuousCollisionDetector.cpp:
//     346-377 with the callback at 66-186): the face of any mesh (own mesh: not incident
//     to the vertex) whose moving triangle the trajectory xprev -> x of surface vertex i
//     of mesh m crosses first; equal depths go to the lower (mesh, face);
//   dcd(m, i): vertexCollisionDetection + closestPointQuery (DiscreteCollisionDetector.cpp:
//     12-95, 97-329, 517-660) at the positions given to build_tets: whether the vertex
//     lies strictly inside a tet (the lowest (mesh, tet) of any mesh; own mesh only when
//     handle_self and not incident), and then the nearest feasible surface face of that
//     tet's mesh (hit.face = -1 when none) from which the tetrahedral traversal
//     (tet_traverse) reaches the containing tet.
class Detector {
public:
    explicit Detector(const std::vector<CcdMesh>& meshes);
    ~Detector();
    Detector(const Detector&) = delete;
    Detector& operator=(const Detector&) = delete;
    void build_swept();              // broad phase of ccd()
    void build_tets(bool prev);      // broad phase of dcd(), on xprev or x
    CcdHit ccd(int m, int i) const;
    bool dcd(int m, int i, const DcdParams& p, CcdHit& hit) const;

private:
    struct Impl;
    Impl* d_;
};

}  // namespace oracle_tc
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Test entry points. */
int32_t oracle_ccd_tri_point(const float* x0, const float* x1, const float* p0, const float* p1, float* tt,
                             float* bary);
/* Tetrahedral walk of one tet mesh from surface face `face` toward tet `target` (1 reached,
   0 not, -1 bad index); status = 1 when the walk gave up on a size bound. */
int32_t oracle_tet_walk(int32_t nv, int32_t ntet, const int32_t* tets, const double* X, int32_t face, int32_t target,
                        const float* origin, const float* dir, float max_dis, float ray_eps, int32_t use_static,
                        int32_t* status);
/* Surface of one tet mesh: call with faces == NULL to get the counts. */
void oracle_tet_surface(int32_t nv, int32_t ntet, const int32_t* tets, const double* X, int32_t* nfaces,
                        int32_t* nverts, int32_t* faces, int32_t* verts);

#ifdef __cplusplus
}
#endif
#endif
