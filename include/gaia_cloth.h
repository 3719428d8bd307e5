/* C ABI of the GB300 cloth VBD step (libgaia_vbd.so).
 *
 * Drop-in for the GPU-relevant path of Gaia's VBDClothSimulationFramework:
 *   loadRunningparameters / initialize  (VBDCloth/VBDClothPhysics.cpp:19-64,
 *                                        Framework/BaseClothSimPhsicsFramework.cpp:17-78)
 *   runStep -> runStep_CDEveryIter      (VBDCloth/VBDClothPhysics.cpp:314-324, 389-518)
 *   ClothContactDetector queries        (CollisionDetector/ClothContactDetector.cpp:1052-1135)
 * reading the same Models.json / Parameters.json (PhysicsParams, ContactDetectorParams,
 * ColliderParams). Meshes are .obj triangle meshes with the StVK membrane and quadratic
 * bending material; colliders are static triangle meshes.
 *
 * Conventions as in gaia_vbd.h: every call returns a gaia_vbd_status code, 0 = OK; no
 * exception crosses the ABI; the handle owns all device memory and one CUDA stream;
 * calls on one handle must not overlap. Positions and velocities are 3 doubles per
 * vertex in the mesh's own vertex order. Mesh indices count the simulated meshes of
 * Models.json first, then the colliders of ColliderParams.ColliderMeshes.
 */
#ifndef GAIA_CLOTH_H
#define GAIA_CLOTH_H

#include <stdint.h>

#include "gaia_vbd.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gaia_cloth gaia_cloth;

typedef struct gaia_cloth_stats {
    int32_t precision;              /* 32, 48 (FP32 arithmetic on double-float positions:
                                       gpuPrecision "mixed") or 64 */
    int32_t num_groups;             /* merged colors */
    int64_t num_vertices;           /* all meshes, colliders included */
    int64_t num_sim_vertices;
    int64_t num_faces;
    int64_t num_edges;
    int64_t kernel_launches_per_step;
    int64_t detections;             /* contact detections run so far */
    int64_t truncations;            /* solves that hit their conservative bound */
    int64_t vf_overflow, ee_overflow, fv_overflow, candidate_overflow, stack_overflow;
    int64_t fp64_fallback_solves, failed_solves;
    int64_t device_bytes;
} gaia_cloth_stats;

/* VBDClothSimulationFramework::loadRunningparameters: parse the inputs and build
 * topology, rest shape, colorings and merged colors on the host (no device needed;
 * the topology, rest-shape and group getters work on a loaded handle). */
int gaia_cloth_load(const char* models_json, const char* params_json, const char* repo_root, gaia_cloth** out);
/* VBDClothSimulationFramework::initialize: upload to the current device, capture the
 * substep graph. */
int gaia_cloth_initialize(gaia_cloth* h);
/* gaia_cloth_load + gaia_cloth_initialize. */
int gaia_cloth_create(const char* models_json, const char* params_json, const char* repo_root, gaia_cloth** out);
void gaia_cloth_destroy(gaia_cloth* h);
const char* gaia_cloth_last_error(gaia_cloth* h);

/* n_steps calls of runStep (numSubsteps substeps each). Asynchronous. */
int gaia_cloth_run_step(gaia_cloth* h, int32_t n_steps);
/* The same, timed on the handle's stream with CUDA events. */
int gaia_cloth_run_step_timed(gaia_cloth* h, int32_t n_steps, float* total_ms);
int gaia_cloth_synchronize(gaia_cloth* h);
/* PhysicsState recovery file of the simulated meshes (same format as gaia_vbd_save_state). */
int gaia_cloth_save_state(gaia_cloth* h, const char* path, int32_t binary);
int gaia_cloth_load_state(gaia_cloth* h, const char* path);
/* Output frames of the simulated meshes (BaseClothSimPhsicsFramework.cpp:130-160,
 * IO/FileIO.cpp:86-117, 187-251): ASCII PLY of all vertices and faces, one file or one per
 * mesh (<dir>/<stem>Model_<%04d>[_<model stem>]_<ext>), or raw FP32 xyz. */
int gaia_cloth_write_ply(gaia_cloth* h, const char* path, int32_t all_in_one, int32_t add_model_name);
int gaia_cloth_write_binary(gaia_cloth* h, const char* path);


int gaia_cloth_num_meshes(gaia_cloth* h, int32_t* num_sim, int32_t* num_colliders);
int64_t gaia_cloth_num_vertices(gaia_cloth* h, int32_t mesh);
int64_t gaia_cloth_num_faces(gaia_cloth* h, int32_t mesh);
int64_t gaia_cloth_num_edges(gaia_cloth* h, int32_t mesh);

int gaia_cloth_get_positions(gaia_cloth* h, int32_t mesh, double* xyz);
int gaia_cloth_set_positions(gaia_cloth* h, int32_t mesh, const double* xyz);
int gaia_cloth_get_velocities(gaia_cloth* h, int32_t mesh, double* xyz);
int gaia_cloth_set_velocities(gaia_cloth* h, int32_t mesh, const double* xyz);

/* TriMeshTopology (TriMesh/TriMesh.h:52-120): per edge (v1, v2, v12next, v21next, f1, f2),
 * -1 across a boundary; per face its edges AB, BC, CA. */
int gaia_cloth_get_topology(gaia_cloth* h, int32_t mesh, int32_t* edges6, int32_t* face_edges3);
/* Rest shape of a simulated mesh: 2x2 column-major DmInv per face, rest area per face,
 * vertex mass. */
int gaia_cloth_get_rest_shape(gaia_cloth* h, int32_t mesh, double* dminv4, double* area, double* mass);
int gaia_cloth_num_groups(gaia_cloth* h);
int64_t gaia_cloth_group_size(gaia_cloth* h, int32_t group);
/* (mesh, vertex) pairs of one merged color. */
int gaia_cloth_get_group(gaia_cloth* h, int32_t group, int32_t* mesh_vertex_pairs);

/* ClothVBD applyCollisionDetection on the current positions (BVH rebuild and refit,
 * VF and EE queries, conservative bounds), then synchronize. */
int gaia_cloth_detect(gaia_cloth* h);
/* Contact pairs of the last detection. VF rows (vertex mesh, vertex, face mesh, face);
 * EE rows (mesh 1, edge 1, mesh 2, edge 2), edge 1 simulated. Rows are ordered by the
 * query primitive, then ascending target. *n receives the row count; at most cap rows
 * are written. */
int gaia_cloth_get_vf_contacts(gaia_cloth* h, int32_t* rows4, int64_t cap, int64_t* n);
int gaia_cloth_get_ee_contacts(gaia_cloth* h, int32_t* rows4, int64_t cap, int64_t* n);
/* Per simulated vertex of `mesh`: its conservative displacement bound of the last
 * detection (VBDClothPhysics.cpp:780-814). */
int gaia_cloth_get_bounds(gaia_cloth* h, int32_t mesh, double* bounds);
/* Minimum distances of the last detection: per vertex of `mesh` to any face, per face
 * of `mesh` to any vertex, per edge of a simulated `mesh` to any edge (maxQueryDis
 * where nothing is within reach). Any pointer may be NULL. */
int gaia_cloth_get_min_distances(gaia_cloth* h, int32_t mesh, float* vertex_face, float* face_vertex, float* edge_edge);

/* Force (3) and Hessian (3x3 row-major) the block solve of one simulated vertex would use
 * at the current positions and contact sets: VBDStepWithExistingCollisions up to the
 * solve (VBDClothPhysics.cpp:1026-1124). */
int gaia_cloth_vertex_force_hessian(gaia_cloth* h, int32_t mesh, int32_t v, double* f3, double* h9);

/* Re-time the lanes per vertex of every color's solve kernel on the current state and
 * capture the substep graph again (the simulation itself is unchanged). */
int gaia_cloth_autotune(gaia_cloth* h);
/* Lanes per vertex of each merged color's solve (num_groups entries). */
int gaia_cloth_get_group_lanes(gaia_cloth* h, int32_t* lanes);
/* Milliseconds of one sweep of the per-color solve kernels over all colors, timed with
 * CUDA events over `reps` sweeps on the current state; the state is restored. For
 * roofline accounting of the solve kernel. */
int gaia_cloth_time_solve(gaia_cloth* h, int32_t reps, float* ms_per_sweep);

int gaia_cloth_get_stats(gaia_cloth* h, gaia_cloth_stats* out);

/* GraphColoring tool on a triangle mesh (GraphColoring/GraphColoring.cpp:80-150 with
 * TriMeshVertexGraph.h:13-43): OrderedGreedy or MCS on the vertex graph of the mesh
 * edges, plus the two vertices across every interior edge when `bending` != 0.
 * Returns the number of colors, or -1 on bad input. */
int32_t gaia_cloth_color_greedy(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t* colors);
int32_t gaia_cloth_color_mcs(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t* colors);
/* The GraphColoring tool on a triangle mesh: MCS (0, default) or OrderedGreedy (1), then
 * balanceColoredCategories when balance != 0 (the tool's default, goal 1.05); `order`
 * (optional, nv ints) receives the categories' vertex order (see gaia_vbd_color_tool). */
int32_t gaia_cloth_color_tool(int32_t nv, int32_t nf, const int32_t* faces, int32_t bending, int32_t algorithm,
                              int32_t balance, float goal_ratio, int32_t* colors, int32_t* order);

#ifdef __cplusplus
}
#endif

#endif /* GAIA_CLOTH_H */
