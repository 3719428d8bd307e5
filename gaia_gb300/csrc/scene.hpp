// Host-side scene model for the VBD step: the inputs Gaia's VBDPhysics reads
// (Models.json / Parameters.json), the tet meshes, colorings and the merged
// per-color "parallel groups". Everything here runs once at set-up on the
// host; the per-step work lives in the CUDA engine.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gaia {

// Hot-path keys of BasePhysicsParams (Parameters/PhysicsParameters.h:9-178) and
// VBDPhysicsParameters (VBD/VBDPhysicsParameters.h:5-147), with the same
// defaults. Keys the VBD step does not read are ignored.
struct PhysicsParams {
    double gravity[3] = {0.0, -10.0, 0.0};
    double timeStep = 0.01666666666666666666;
    int numSubsteps = 20;
    int iterations = 1;
    bool usePlaneGround = true;
    double worldLo[3] = {-1e7, -1e7, -1e7};
    double worldHi[3] = {1e7, 1e7, 1e7};
    double boundaryFrictionDynamic = 0.1;
    double boundaryFrictionEpsV = 1.0;
    double boundaryCollisionStiffness = 1e5;
    double stepSize = 1.0;
    double stepSizeGD = 1e-3;
    int frictionStartIter = 0;
    bool associateGravityWithInertia = true;
    bool useAccelerator = false;
    double acceleratorRho = 0.93;
    bool useGPU = true;
    bool handleCollision = false;
    double collisionStiffness = 1e5;
    double collisionOffHeight = 1e7;          // contact detection only below this height (y)
    int intermediateCollisionIterations = -1; // re-detect every n iterations (n > 0)
    // CollisionDetectionParamters (CollisionDetector/CollisionDetertionParameters.h:41-78),
    // "CollisionParams" in Parameters.json: the keys the VBD step uses
    bool allowCCD = true;
    bool allowDCD = true;
    bool handleSelfCollision = true;
    bool checkFeasibleRegion = true;
    double feasibleRegionEpsilon = 1e-2;
    // the DCD closest-point query's tetrahedral traversal check
    bool checkTetTraverse = true;
    bool tetrahedralTraverseForNonSelfIntersection = true;
    bool stopTraversingAfterPassingQueryPoint = true;
    bool shiftQueryPointToCenter = true;
    bool useStaticTraverse = true;
    bool loopLessTraverse = false;  // not supported (rejected)
    double centerShiftLevel = 0.01;
    double rayTriIntersectionEPSILON = 1e-10;
    double maxSearchDistanceMultiplier = 1.8;
    int numThreadsVBDSolve = 16;
    bool useDouble3x3 = false;
    bool evaluateConvergence = false;
    int evaluationSteps = 10;  // with evaluateConvergence: evaluate after iterations 0, n, 2n, ...
    // output of the frame loop (Parameters/PhysicsParameters.h:30, 87-99)
    int numFrames = 5000;
    bool saveOutputs = true;
    bool saveAllModelsTogether = true;
    std::string outputExt = "ply";
    int binaryModeVisualizationSteps = 100;
    bool outputRecoveryState = true;
    int outputRecoveryStateStep = 10;
    bool outputRecoveryStateBinary = true;
    // derived (BasePhysicsFramework.cpp:245-249)
    double dt = -1.0, dtSqrReciprocal = -1.0;
    // GB300 engine keys (extensions; absent in reference files -> defaults)
    std::string gpuPrecision = "mixed";  // "mixed" (double-float state, FP32 element math), "dfhi" (double-float
                                         // state read as FP32 by neighbours), "fp32" or "fp64"
    int lanesPerVertex = 0;              // 0 = autotune
    int blockSize = 0;                   // 0 = autotune
    bool autotune = true;
    bool usePDL = true;                  // programmatic dependent launch between color kernels
    int smallColorVertices = 16384;      // colors up to this size use one warp per vertex
    int solveVariant = -1;               // -1 autotune, 0 register-pipelined, 1 TMA-staged records, 4 deeper
                                         // register pipeline, 6 next wave's records prefetched into L2,
                                         // 7 double-buffered TMA tiles on a persistent grid
    std::string sweepMode = "auto";      // color scheduling: "auto", "merged", "scenes", "cluster", "grid"
    int clusterSize = 0;                 // blocks per cluster of the cluster sweep (0 = autotune; 2, 4, 8, 16)
    bool meshFrames = true;              // FP32-compute states relative to a per-mesh frame that follows
                                         // the mesh (no contact detection, no deformers)
    int waitPollLimit = -1;              // polls of a bounded device wait (-1: the built-in limit); tests
                                         // lower it to make the wait run out
};

// ObjectParams (Materials/Materials.h:12-75) + ObjectParamsVBD
// (VBD/VBD_BaseMaterial.h:21-49) + ObjectParametersVBDNeoHookean
// (VBD/VBD_NeoHookean.h:16-33), same defaults.
struct ObjectParams {
    std::string path;
    std::string materialName = "NeoHookean";
    std::string verticesColoringCategoriesPath;
    double translationBeforeScaling[3] = {0, 0, 0};
    double scale[3] = {1, 1, 1};
    double translation[3] = {0, 0, 0};
    double rotation[3] = {0, 0, 0};
    double initialVelocity[3] = {0, 0, 0};
    double density = 1.0;
    double maxVelocityMagnitude = -1.0;
    int frameToAppear = -1;
    std::vector<int32_t> fixedPoints;
    double frictionDynamic = 0.1;
    double frictionEpsV = 0.01;
    double exponentialVelDamping = 1.0;
    double constantVelDamping = 0.0;
    int initializationType = 0;
    double miu = 1e4;
    double lmbd = 1e4;
    double dampingDeviatoric = 0.0;
    double dampingHydrostatic = 0.0;
};

// Deformers[] entries of Parameters.json (VBD/VBDDeformer.h:175-221).
struct DeformerParams {
    int type = 0;  // 0 = Rotator, 1 = Translator
    double center[3] = {0, 0, 0};
    double axis[3] = {1, 0, 0};
    double angularVelocity = 0.0;
    double endTime = -1.0;
    double speed[3] = {0, 0, 0};
    std::vector<int32_t> selectedMeshes;
    std::vector<std::vector<int32_t>> selectedVertices;
};

struct TetMesh {
    int32_t nv = 0, ntet = 0;
    std::vector<float> X;          // 3*nv positions after rotation/scale/translation (FP32, as mVertPos)
    std::vector<float> V;          // 3*nv initial velocities
    std::vector<int32_t> tets;     // 4*ntet
    std::vector<double> dminv;     // 9*ntet column-major, FP64 precompute
    std::vector<double> vol;       // ntet
    std::vector<double> mass;      // nv
    std::vector<uint8_t> fixed;    // nv
    std::vector<std::vector<int32_t>> colors;  // sorted by size, large to small
    std::vector<int32_t> nbr_ofs, nbr_tet, nbr_order;  // CSR vertex -> incident tets
    // surface (see extract_surface)
    std::vector<int32_t> sfaces;               // 3 per boundary face, outward
    std::vector<int32_t> sverts;               // boundary vertices, ascending
    std::vector<int32_t> sface_nbr;            // 3 per face: face across edge AB, BC, CA (-1: none)
    std::vector<int32_t> sring_ofs, sring;     // per vertex: surface neighbours, ascending
    std::vector<int32_t> sface_tet;            // 2 per face: the tet it bounds, the local vertex it omits
    std::vector<int32_t> tet_nbr;              // 4 per tet: tet across the face omitting vertex k (-1: none)
};

struct Scene {
    PhysicsParams p;
    std::vector<ObjectParams> objs;
    std::vector<TetMesh> meshes;
    std::vector<DeformerParams> defs;
    std::vector<std::vector<int32_t>> groups;  // merged colors: (mesh, vertex) pairs
};

// Loading (throws std::runtime_error with a message on any failure).
void load_scene(const std::string& models_json, const std::string& params_json, const std::string& repo_root,
                Scene& scene);
void load_t(const std::string& path, std::vector<float>& X, std::vector<int32_t>& tets);
std::vector<std::vector<int32_t>> load_coloring(const std::string& path);
void prepare_mesh(const PhysicsParams& p, const ObjectParams& o, TetMesh& m);  // rest shape, CSR, fixed
void build_parallel_groups(Scene& scene);
// Boundary faces (faces of exactly one tet) in ascending (tet, local face) order; the
// face opposite local vertex k is (1,2,3), (0,3,2), (0,1,3), (0,2,1) for k = 0..3, which
// points out of a tet of positive rest volume, and is reversed for a negative one. Also
// the surface vertices, the face across each face edge and each vertex's surface ring.
void extract_surface(TetMesh& m);
void validate_coloring(const TetMesh& m);  // every vertex exactly once; no two tet-neighbours share a color

// Colorings (bit-exact with GraphColoring/mcs.cpp and gready.cpp, in O(E log V)).
int32_t color_mcs(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors);
int32_t color_greedy(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors);
// The same two algorithms on a vertex graph given as CSR with sorted unique
// neighbours (ofs has nv + 1 entries).
int32_t color_mcs_graph(int32_t nv, const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t* colors);
int32_t color_greedy_graph(int32_t nv, const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t* colors);
std::vector<std::vector<int32_t>> colors_to_categories(int32_t nv, const int32_t* colors);
// GraphColor::balanceColoredCategories (GraphColoring/ColoringAlgorithms.cpp:142-196), the
// GraphColoring tool's default post-pass (-b, ratio 1.05, GraphColoring.cpp:23-24, 182-189):
// move a vertex from the largest category (or, if none of its vertices can move, from the
// first other category that has one) to the smallest, until the largest/smallest size ratio
// measured before a move is at most goal; categories keep the reference's order (a moved
// vertex is erased from its list and appended to the destination's). Updates colors.
// Throws where the reference's loop would not end (moves cycling short of the goal).
void balance_categories(int32_t nv, const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t* colors,
                        std::vector<std::vector<int32_t>>& cats, float goal);
// The vertex graph of a tet mesh (all vertex pairs sharing a tet), CSR with sorted neighbours.
void tet_vertex_graph(int32_t nv, int32_t ntet, const int32_t* tets, std::vector<int64_t>& ofs, std::vector<int32_t>& adj);

void write_t(const std::string& path, int32_t nv, const double* X, int32_t ntet, const int32_t* tets);
void write_coloring(const std::string& path, const std::vector<std::vector<int32_t>>& cats);

}  // namespace gaia
