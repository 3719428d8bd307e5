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
};

// The two detectors of the tet-mesh contact path over all meshes:
//   ccd(m, i): vertexContinuousCollisionDetection (ContinuousCollisionDetector.cpp:
//     346-377 with the callback at 66-186): the face of any mesh (own mesh: not incident
//     to the vertex) whose moving triangle the trajectory xprev -> x of surface vertex i
//     of mesh m crosses first; equal depths go to the lower (mesh, face);
//   dcd(m, i): vertexCollisionDetection + closestPointQuery (DiscreteCollisionDetector.cpp:
//     12-95, 97-329, 517-660) at the positions given to build_tets: whether the vertex
//     lies strictly inside a tet (the lowest (mesh, tet) of any mesh; own mesh only when
//     handle_self and not incident), and then the nearest feasible surface face of that
//     tet's mesh (hit.face = -1 when none). The tetrahedral traversal check of the
//     closest-point query is not restated (it accepts every face of a convex mesh).
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
/* Surface of one tet mesh: call with faces == NULL to get the counts. */
void oracle_tet_surface(int32_t nv, int32_t ntet, const int32_t* tets, const double* X, int32_t* nfaces,
                        int32_t* nverts, int32_t* faces, int32_t* verts);

#ifdef __cplusplus
}
#endif
#endif
