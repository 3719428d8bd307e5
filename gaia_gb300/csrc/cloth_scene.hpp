// Host-side scene model for the cloth VBD step: the inputs Gaia's
// VBDClothSimulationFramework reads (Models.json / Parameters.json with
// PhysicsParams, ContactDetectorParams and ColliderParams), the triangle meshes
// with their topology (edges, per-vertex neighbour faces / edges / bending
// stencils), the rest shape, colorings and the merged parallel groups. All of
// it runs once at set-up; the per-step work lives in the CUDA cloth engine.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gaia {
namespace cloth {

// BasePhysicsParams (Parameters/PhysicsParameters.h:9-178) and
// VBDClothPhysicsParameters (VBDCloth/VBDClothPhysicsParameters.h:7-75), same
// defaults. Keys the reference does not read from JSON (contactEnergyTypes,
// boundaryContactStiffness) keep their defaults here too.
struct PhysicsParams {
    double gravity[3] = {0.0, -10.0, 0.0};
    double timeStep = 0.01666666666666666666;
    int numSubsteps = 20;
    int iterations = 1;
    double worldLo[3] = {-1e7, -1e7, -1e7};
    double worldHi[3] = {1e7, 1e7, 1e7};
    double boundaryFrictionDynamic = 0.1;
    double stepSize = 1.0;
    bool associateGravityWithInertia = true;
    bool handleCollision = true;
    double contactStiffness = 1e4;
    double contactRadius = 1.0;
    double thickness = 0.0;
    double conservativeStepRelaxation = 0.45;
    double boundaryContactStiffness = 1e4;  // not read from JSON by the reference
    double boundaryFrictionEpsValue = 1e-2;
    int contactEnergyTypes = 1;             // not read from JSON by the reference
    int contactBVHReconstructionSteps = 32;
    double degenerateTriangleThres = 1e-6;
    bool applyAcceleration = false;
    double acceleratorRho = 0.95;
    bool useNewton = false;
    // ClothContactDetectorParameters (CollisionDetector/ClothContactDetector.h:13-31):
    // the constructor body sets 0.4, which is what an absent key leaves.
    double maxQueryDis = 0.4;
    // derived (BasePhysicsFramework.cpp:245-249)
    double dt = -1.0, dtSqrReciprocal = -1.0;
    // GB300 engine keys (extensions; absent in reference files -> defaults)
    std::string gpuPrecision = "fp32";     // "fp32", "mixed" (FP32 arithmetic, double-float positions) or
                                           // "fp64" (the FP64 engine is the error reference)
    bool contactDetectionEveryIteration = false;  // also run detection when no vertex was truncated
    int blockSize = 128;
    int lanesPerVertex = 0;                // lanes per vertex of the solve; 0 = autotune per color
};

// ObjectParams (Materials/Materials.h:12-75) + TriMeshParams (TriMesh/TriMesh.h:27-50)
// + VBDObjectParamsTriMesh (VBDCloth/VBDBaseTriMesh.h:8-20) + VBDObjectParamsTriMeshStVk
// (VBDCloth/VBDTriMeshStVK.h:12-27), same defaults.
struct ObjectParams {
    std::string path;
    std::string verticesColoringCategoriesPath;
    double scale[3] = {1, 1, 1};
    double translation[3] = {0, 0, 0};
    double rotation[3] = {0, 0, 0};
    double density = 1.0;
    double maxVelocityMagnitude = -1.0;
    bool hasNoGravZone = false;
    double noGravZoneThreshold = 0.0;
    std::vector<int32_t> fixedPoints;
    bool use3DRestpose = true;
    double frictionDynamic = 0.1;
    double frictionEpsV = 0.1;
    double bendingStiffness = 0.0;
    double exponentialVelDamping = 1.0;
    double constantVelDamping = 0.0;
    int initializationType = 2;
    double miu = 1e4;
    double lambda = 1e4;
    double dampingStVK = 0.0;
    double dampingBending = 0.0;
};

// EdgeInfo (TriMesh/TriMesh.h:52-61).
struct Edge {
    int32_t v1, v2;      // first half-edge: v1 -> v2 in face f1
    int32_t v12next;     // vertex opposite (v1, v2) in f1
    int32_t v21next;     // vertex opposite (v2, v1) in f2, -1 on a boundary edge
    int32_t f1, f2;      // f2 = -1 on a boundary edge
};

struct TriMesh {
    int32_t nv = 0, nf = 0, ne = 0;
    std::vector<float> X;             // 3*nv positions after rotation / scale / translation
    std::vector<int32_t> faces;       // 3*nf
    std::vector<Edge> edges;
    std::vector<int32_t> faceEdges;   // 3*nf: edges AB, BC, CA of each face
    // per-vertex CSR lists, ascending ids
    std::vector<int32_t> nbrVOfs, nbrV;                     // neighbour vertices
    std::vector<int32_t> nbrFOfs, nbrF, nbrFOrder;          // incident faces, order of the vertex in the face
    std::vector<int32_t> nbrEOfs, nbrE, nbrEOrder;          // incident edges, 0 if the vertex is v1 else 1
    std::vector<int32_t> bendOfs, bendE, bendOrder;         // relevant bending stencils, order 0..3
    // simulated meshes only
    std::vector<double> dminv;        // 4*nf, 2x2 column-major inverse of the 2D rest edge matrix
    std::vector<double> area;         // nf rest areas
    std::vector<double> mass;         // nv
    std::vector<double> bendQ;        // 16*ne, 4x4 row-major quadratic form (zero for boundary edges)
    std::vector<uint8_t> fixed;       // nv
    std::vector<std::vector<int32_t>> colors;  // sorted by size, large to small
};

struct Scene {
    PhysicsParams p;
    std::vector<ObjectParams> objs;      // one per simulated mesh
    std::vector<TriMesh> meshes;         // simulated meshes, then collider meshes
    std::vector<double> colliderFriction;     // per collider: frictionDynamic, frictionEpsV
    int numSim = 0;
    std::vector<std::vector<int32_t>> groups;  // merged colors: (mesh, vertex) pairs
};

// Loading (throws std::runtime_error with a message on any failure).
void load_scene(const std::string& models_json, const std::string& params_json, const std::string& repo_root,
                Scene& s);
void load_obj(const std::string& path, std::vector<float>& X, std::vector<int32_t>& faces);
void build_topology(TriMesh& m);
void prepare_rest_shape(const ObjectParams& o, TriMesh& m);
void build_parallel_groups(Scene& s);
// Vertex graph of a triangle mesh (TriMeshVertexGraph.h:13-43): the two ends of
// every edge, plus with `bending` the two vertices across every interior edge.
void tri_vertex_graph(const TriMesh& m, bool bending, std::vector<int64_t>& ofs, std::vector<int32_t>& adj);

// Orthonormal tangent basis (t, b) of a unit normal n with t x b = n
// (Duff et al. 2017, "Building an Orthonormal Basis, Revisited").
void orthonormal_basis(const double n[3], double t[3], double b[3]);

}  // namespace cloth
}  // namespace gaia
