/*
 * gaia_vbd.h — C ABI of the GB300-native VBD step (libgaia_vbd.so).
 *
 * This is the drop-in boundary for Gaia's Vertex Block Descent step. Each
 * entry point names the reference interface it replaces (paths relative to the
 * reference project's Simulator/ directory). The reference binds these
 * through C++ class methods of GAIA::VBDPhysics; here they are plain C symbols
 * with pointers and sizes, no exceptions cross the boundary, and every call
 * returns a status code (GAIA_VBD_OK = 0).
 *
 * Threading: one handle owns one CUDA stream and all its device memory. Calls
 * on one handle must not run concurrently; separate handles are independent.
 * Memory: arrays are caller-owned host memory unless stated otherwise.
 */
#ifndef GAIA_VBD_H
#define GAIA_VBD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GAIA_VBD_VERSION 1

/* Status codes. */
enum {
    GAIA_VBD_OK = 0,
    GAIA_VBD_E_INVALID_ARG = 1,  /* null pointer, index out of range, bad size */
    GAIA_VBD_E_INPUT = 2,        /* unreadable or malformed JSON / mesh / coloring file */
    GAIA_VBD_E_COLORING = 3,     /* coloring misses or repeats vertices, or is not an independent set */
    GAIA_VBD_E_MESH = 4,         /* degenerate tet (zero rest volume), bad fixed point */
    GAIA_VBD_E_CUDA = 5,         /* a CUDA runtime call failed (message in last_error) */
    GAIA_VBD_E_NONFINITE = 6,    /* a solve produced NaN/Inf; positions are left as they were written */
    GAIA_VBD_E_NO_DEVICE = 7,    /* no CUDA device is visible */
    GAIA_VBD_E_UNSUPPORTED = 8,  /* input asks for a feature outside the VBD tet step */
    GAIA_VBD_E_DEVICE_TIMEOUT = 9 /* a bounded device-side wait ran out: the blocks that gave up
                                     skipped their vertices (none of them moved) */
};
/* NONFINITE and DEVICE_TIMEOUT come from device work and are returned by the next
 * synchronizing call (synchronize, get_positions, ...). Each is returned once: that call
 * clears it, and gaia_vbd_get_stats keeps the running totals. */

typedef struct gaia_vbd gaia_vbd;

/* Run-time counters of one handle. */
typedef struct {
    int32_t precision;            /* state / arithmetic of the engine (gpuPrecision): 32 = "fp32",
                                     48 = "mixed" (double-float state), 40 = "dfhi" (double-float state,
                                     neighbours read in FP32), 64 = "fp64" (the plain FP64 engine) */
    int32_t lanes_per_vertex;     /* threads cooperating on one vertex solve */
    int32_t block_size;           /* threads per block of the solve kernel */
    int32_t num_groups;           /* merged colors ("parallel groups") */
    int64_t num_vertices;         /* all meshes */
    int64_t num_active_vertices;  /* vertices that are solved (not fixed) */
    int64_t num_incidences;       /* (vertex, incident tet) pairs over active vertices */
    int64_t kernel_launches_per_step;
    int64_t fp64_fallback_solves; /* FP32 3x3 solves redone in FP64 (cumulative) */
    int64_t failed_solves;        /* solves that fell back to the gradient step (cumulative) */
    int64_t device_bytes;         /* device memory owned by the handle */
    double autotune_ms_per_iteration; /* best measured sweep time per iteration (0 if not tuned) */
    int32_t solve_variant;        /* 0 = register-pipelined solve kernel, 1 = TMA-staged records,
                                     2 = scene-major persistent sweep, 3 = cluster sweep, 4 = register
                                     pipeline two records deep, 5 = grid sweep, 6 = register pipeline
                                     with the records of the next resident wave prefetched into L2,
                                     7 = double-buffered TMA tiles on a persistent grid (of the
                                     largest color) */
    int32_t mesh_frames;          /* 1: states are kept relative to a per-mesh frame offset that
                                     follows each mesh (PhysicsParams meshFrames; FP32-compute
                                     precisions without contact detection or deformers) */
    /* tet-mesh contact detection (cumulative; 0 when contact is off) */
    int64_t contact_detections;       /* detection passes run */
    int64_t contact_stack_overflow;   /* hierarchy traversals that dropped a node (stack full) */
    int64_t contact_traverse_bounds;  /* DCD tetrahedral walks that gave up on a size bound */
    int64_t device_timeouts;          /* blocks whose bounded wait (staged records, grid barrier) ran
                                         out; the call that reports it returns GAIA_VBD_E_DEVICE_TIMEOUT */
    int64_t nonfinite_solves;         /* vertex solves with a non-finite force or step (not written) */
    int32_t sweep_mode;               /* color scheduling: 0 = merged colors (a launch per merged color
                                         and iteration), 1 = scene-major persistent sweep, one block per
                                         scene (solve_variant 2), 2 = scene-major sweep on thread-block
                                         clusters with the scene in shared memory (solve_variant 3),
                                         3 = one cooperative launch per substep over the merged colors
                                         with a bounded grid barrier between colors (solve_variant 5) */
    int32_t cluster_size;             /* blocks per cluster of the cluster sweep (0 otherwise) */
    double sweep_ms_merged;           /* sweep time per iteration the autotuner measured for each */
    double sweep_ms_scenes;           /* schedule (0 where it did not time it) */
    double sweep_ms_cluster;
    double sweep_ms_grid;             /* (-1: the grid sweep could not be built here) */
} gaia_vbd_stats;

/* ---- life cycle ------------------------------------------------------------
 * gaia_vbd_create: VBDPhysics::loadRunningparameters (VBD/VBDPhysics.cpp:90-97)
 * followed by VBDPhysics::initialize (VBD/VBDPhysics.cpp:208-454) and
 * initializeGPU (:563-651). Reads Models.json and Parameters.json with the
 * reference's keys and defaults, substitutes ${REPO_ROOT} in paths
 * (Parser/InputHandler.h:128-185), loads the .t meshes and vertex colorings
 * (computing the reference's OrderedGreedy coloring when a model gives no
 * coloring file), precomputes the rest shape in FP64, merges colors into
 * parallel groups and uploads everything. repo_root may be NULL.
 * Extra PhysicsParams keys: "gpuPrecision" ("fp32" | "mixed" | "dfhi" | "fp64"),
 * "lanesPerVertex", "blockSize" (0 = autotune), "autotune" (bool), "sweepMode"
 * ("auto" | "merged" | "scenes" | "cluster" | "grid": color scheduling, see
 * gaia_vbd_stats.sweep_mode; auto times every schedule the scene allows and keeps the fastest;
 * the persistent sweeps need contact detection, the accelerator and evaluateConvergence off,
 * and the cluster sweep scenes that fit in the shared memory of a cluster), "clusterSize"
 * (0 = autotune, 2-16), "waitPollLimit" (polls of a bounded device wait before it gives up:
 * the staged records' wait and the grid barrier; default 2^20), "meshFrames" (default true:
 * FP32-compute states relative to a per-mesh offset that follows the mesh, see
 * gaia_vbd_stats.mesh_frames; positions in and out of the API are absolute either way).
 */
int gaia_vbd_create(const char* models_json, const char* params_json, const char* repo_root, gaia_vbd** out);
/* The two halves of gaia_vbd_create. gaia_vbd_load is host-only (no GPU needed):
 * VBDPhysics::loadRunningparameters plus the host part of initialize (meshes,
 * colorings, rest shape, parallel groups); the introspection calls below work on a
 * loaded handle. gaia_vbd_initialize builds the device layout and CUDA graphs
 * (VBDPhysics::initializeGPU, VBD/VBDPhysics.cpp:563-651). */
int gaia_vbd_load(const char* models_json, const char* params_json, const char* repo_root, gaia_vbd** out);
int gaia_vbd_initialize(gaia_vbd* h);
/* ~VBDPhysics. Safe on NULL. */
void gaia_vbd_destroy(gaia_vbd* h);
/* Message of the last failed call on this handle ("" if none). */
const char* gaia_vbd_last_error(const gaia_vbd* h);
/* Message of the last failed gaia_vbd_create or tool call on this thread. */
const char* gaia_vbd_last_global_error(void);

/* ---- stepping --------------------------------------------------------------
 * gaia_vbd_run_step: VBDPhysics::runStep -> runStepGPU (VBD/VBDPhysics.cpp:809-969),
 * n_steps times; each step runs numSubsteps substeps of: initial step +
 * deformers, `iterations` color sweeps of the per-vertex block solve
 * (VBDPhysicsCompute.cu:803-908 / VBDPhysics.cpp:2402-2483), velocity update.
 * Asynchronous on the handle's stream; errors of device work surface on the
 * next synchronizing call. */
int gaia_vbd_run_step(gaia_vbd* h, int32_t n_steps);
int gaia_vbd_synchronize(gaia_vbd* h);
/* PhysicsState recovery file (Framework/BasePhysicsFramework.h:127-319; written by
 * writeOutputs, read by recoverFromState, BasePhysicsFramework.cpp:264-282, 495-502):
 * frameId, curTime and every mesh's positions and velocities, inline ("text") or in
 * <name>.pos / <name>.vel FP32 files next to the JSON (binary != 0). Loading sets
 * positions, velocities, the frame counter and the simulated time. */
int gaia_vbd_save_state(gaia_vbd* h, const char* path, int32_t binary);
int gaia_vbd_load_state(gaia_vbd* h, const char* path);
/* Output frames as writeOutputs writes them (Framework/BasePhysicsFramework.cpp:442-489,
 * IO/FileIO.cpp): the surface of every tet mesh as ASCII PLY, in one file (all_in_one)
 * or one per mesh (<dir>/<stem>_Model_<%06d>[_<model stem>]<ext>), or the surface
 * vertices of all meshes as raw FP32 xyz (the "bin" output). Surface vertices are in
 * ascending vertex order. */
int gaia_vbd_write_ply(gaia_vbd* h, const char* path, int32_t all_in_one, int32_t add_model_name);
int gaia_vbd_write_binary(gaia_vbd* h, const char* path);

/* Tet-mesh vertex-face contact (VBDPhysics::dcd / ccd / prepareCollisionDataGPU,
 * VBD/VBDPhysics.cpp:1812-2156; DiscreteCollisionDetector / ContinuousCollisionDetector).
 * The step runs contact detection at the start of every substep (and every
 * intermediateCollisionIterations iterations) when CollisionParams allowCCD / allowDCD
 * are set (the reference's defaults). These calls expose it on its own:
 *   gaia_vbd_num_surface / gaia_vbd_get_surface: the boundary faces (3 ints each,
 *     outward, mesh-local vertex ids) and surface vertices of a mesh (host data, no GPU);
 *   gaia_vbd_set_prev_positions: the positions at the start of the substep (3 doubles
 *     per vertex), the trajectory origins of the continuous test;
 *   gaia_vbd_collide: one substep-start detection pass on the current positions;
 *   gaia_vbd_get_contacts: rows of 8 ints per vertex in contact, in (mesh, surface
 *     vertex) order: mesh, vertex, face mesh, face vertices 0..2, surface face, kind
 *     (1 = continuous, 2 = discrete: the vertex lies inside a tet). */
int gaia_vbd_num_surface(gaia_vbd* h, int32_t mesh, int32_t* nfaces, int32_t* nverts);
int gaia_vbd_get_surface(gaia_vbd* h, int32_t mesh, int32_t* faces, int32_t* verts);
int gaia_vbd_set_prev_positions(gaia_vbd* h, int32_t mesh, const double* xyz);
int gaia_vbd_collide(gaia_vbd* h, int32_t* n_contacts);
int gaia_vbd_get_contacts(gaia_vbd* h, int32_t* rows, int32_t cap, int32_t* n_rows);

/* Runs n_steps and times them with CUDA events on the handle's stream: total_ms = all
 * device work. With sweep_ms NULL the steps run as gaia_vbd_run_step runs them (one CUDA
 * graph per substep); otherwise each substep's initial step, color sweeps and velocity
 * update run as three graphs with events around the sweeps, and sweep_ms = the color
 * sweeps (solve kernels) only. */
int gaia_vbd_run_step_timed(gaia_vbd* h, int32_t n_steps, float* total_ms, float* sweep_ms);
/* Restore the state gaia_vbd_initialize produced: rest positions, initial velocities,
 * substep clock at 0 (counters are kept). The reference recovers a saved state with
 * BasePhysicFramework::recoverFromState (Framework/BasePhysicsFramework.cpp:264-282). */
int gaia_vbd_reset(gaia_vbd* h);
/* Re-run the autotuner (lanes per vertex x block size) on the current state;
 * the state is restored afterwards. */
int gaia_vbd_autotune(gaia_vbd* h);

/* ---- state access (TetMeshFEM positions()/velocities(); VBDPhysics::syncAllToCPU / syncAllToGPU,
 * VBD/VBDPhysics.h:266-299). Arrays are 3*num_vertices(mesh), x,y,z per vertex. Synchronous. */
int gaia_vbd_num_meshes(const gaia_vbd* h);
int64_t gaia_vbd_num_vertices(const gaia_vbd* h, int32_t mesh);
int64_t gaia_vbd_num_tets(const gaia_vbd* h, int32_t mesh);
int gaia_vbd_get_positions(gaia_vbd* h, int32_t mesh, double* out);
int gaia_vbd_set_positions(gaia_vbd* h, int32_t mesh, const double* in);
int gaia_vbd_get_velocities(gaia_vbd* h, int32_t mesh, double* out);
int gaia_vbd_set_velocities(gaia_vbd* h, int32_t mesh, const double* in);
/* Whole-scene FP32 state, meshes concatenated in Models.json order (3 floats per vertex).
 * set_state copies host->device and scatters on the device; get_positions gathers on the
 * device and copies device->host. Pass page-locked buffers for full copy bandwidth. */
int gaia_vbd_set_state_f32(gaia_vbd* h, const float* x, const float* v);
int gaia_vbd_get_positions_f32(gaia_vbd* h, float* x);
int gaia_vbd_get_velocities_f32(gaia_vbd* h, float* v);

/* ---- introspection ----------------------------------------------------------
 * Parallel groups (VBDPhysics::vertexParallelGroups, VBD/VBDPhysics.cpp:235-274):
 * group g holds size pairs (mesh, vertex), in the reference's order. */
int gaia_vbd_num_groups(const gaia_vbd* h);
int64_t gaia_vbd_group_size(const gaia_vbd* h, int32_t g);
int gaia_vbd_get_group(const gaia_vbd* h, int32_t g, int32_t* out_pairs);
/* Per-vertex color index (position in the size-sorted color list, TetMeshFEM.cpp:122-134). */
int gaia_vbd_get_coloring(const gaia_vbd* h, int32_t mesh, int32_t* colors);
/* FP64 rest shape: DmInv 9 per tet (column-major), rest volume per tet, lumped mass per vertex. */
int gaia_vbd_get_rest_shape(const gaia_vbd* h, int32_t mesh, double* dminv, double* vol, double* mass);
/* Total Neo-Hookean elastic energy (rest energy removed) plus inertia energy
 * (VBDPhysicsCompute.cu:1223-1237, 1775-1810; VBD_BaseMaterial.h:223-241), evaluated on
 * the device and reduced in FP64 in a fixed order (gaia_vbd_convergence). */
int gaia_vbd_energy(gaia_vbd* h, double* out);
/* evaluateConvergenceGPU (VBD/VBDPhysics.cpp:3508-3556, with evaluateMeritEnergyGPU :3851-3871)
 * on the current state, reduced in FP64 in a fixed order (repeated calls on one state
 * return bit-identical values): out4 = total energy, inertia energy (all vertices),
 * elastic energy, and the average over all vertices of the norm of the material (with
 * damping) plus inertia force, zero for fixed vertices. gaia_vbd_energy returns out4[0]. */
int gaia_vbd_convergence(gaia_vbd* h, double* out4);
/* With PhysicsParams evaluateConvergence, every step records the same four values on the
 * device, inside its CUDA graphs, at iteration -1 (the initial guess) and after iterations
 * 0, evaluationSteps, 2 * evaluationSteps, ... of every substep (VBDPhysics.cpp:866-870,
 * 948-951). This returns the last step's records, 6 doubles each: substep, iteration,
 * energy, inertia, elastic, average force norm (n_rows = count; at most cap written). */
int gaia_vbd_get_convergence_log(gaia_vbd* h, double* rows, int32_t cap, int32_t* n_rows);
/* Per-vertex force and 3x3 Hessian (material + inertia + ground) at the current state,
 * computed by the solve kernel without moving the vertex: f3 = 3 values, h9 = 9 (row-major). */
int gaia_vbd_vertex_force_hessian(gaia_vbd* h, int32_t mesh, int32_t vertex, int32_t apply_friction,
                                  double* f3, double* h9);
int gaia_vbd_get_stats(gaia_vbd* h, gaia_vbd_stats* out);

/* Output settings of the frame loop as Parameters.json gives them (PhysicsParams keys,
 * defaults of Parameters/PhysicsParameters.h:30, 87-99), read by simulate / writeOutputs
 * (Framework/BasePhysicsFramework.cpp:284-393, 442-506); frame = runStep calls since
 * initialize, or the frameId of the last loaded recovery state. Host data (no GPU). */
typedef struct {
    int32_t num_frames;                        /* numFrames */
    int32_t save_outputs;                      /* saveOutputs */
    int32_t save_all_models_together;          /* saveAllModelsTogether */
    int32_t binary_mode_visualization_steps;   /* binaryModeVisualizationSteps */
    int32_t output_recovery_state;             /* outputRecoveryState */
    int32_t output_recovery_state_step;        /* outputRecoveryStateStep */
    int32_t output_recovery_state_binary;      /* outputRecoveryStateBinary */
    int32_t reserved;
    char output_ext[16];                       /* outputExt, NUL-terminated ("ply", "bin", ...) */
} gaia_vbd_output_params;
int gaia_vbd_get_output_params(const gaia_vbd* h, gaia_vbd_output_params* out);
int64_t gaia_vbd_frame(const gaia_vbd* h);
/* Launch configuration the autotuner chose for merged color g (parallel group g):
 * lanes per vertex, block size, kernel variant (0 registers, 1 TMA-staged), and the
 * measured time of one launch in ms (0 when not tuned). Any pointer may be NULL.
 * The reference launches every color with one 32-thread block per vertex
 * (VBDPhysicsCompute.cu:114-123). */
int gaia_vbd_get_color_config(gaia_vbd* h, int32_t g, int32_t* lanes, int32_t* block, int32_t* variant,
                              float* tuned_ms);

/* ---- energy without device allocation -----------------------------------------
 * This entry point has no counterpart in the reference. It is for callers that
 * cannot call cudaMalloc: hosts that give all device memory to their own arena at
 * start-up, and real-time or plugin hosts that forbid allocation after start-up
 * because cudaMalloc / cudaFree synchronize the device. It returns the same total
 * as gaia_vbd_energy (Neo-Hookean energy with the rest energy removed, plus the
 * inertia energy when y is given) for one mesh held in caller-owned DEVICE arrays,
 * and allocates nothing:
 *   x 3*nv positions, y 3*nv inertia targets or NULL (then mass may be NULL too),
 *   mass nv lumped masses, tets 4*ntet, dminv 9*ntet (column-major), vol ntet,
 *   out 1 double (device); stream = cudaStream_t or NULL.
 * Its only scratch is a fixed array of 4096 partial sums (32 KiB) compiled into the
 * library, which every GPU that loads the library holds until the process exits.
 * Limits: nv and ntet each at most 2^24; larger calls fail with GAIA_VBD_E_INVALID_ARG
 * and a message in gaia_vbd_last_global_error. The first call on a device looks up
 * the scratch array's device address for that device; make that first call before
 * any stream capture. The address is kept for the life of the process: do not call this
 * on a device after a cudaDeviceReset of it. The call is asynchronous on `stream`. All calls share the one
 * scratch array: calls whose kernels overlap on the GPU (different streams or
 * threads) race and must be serialized by the caller. */
int gaia_vbd_energy_noalloc(const double* x, const double* y, const double* mass, int32_t nv,
                            const int32_t* tets, const double* dminv, const double* vol, int32_t ntet,
                            double mu, double lmbd, double dt, double* out, void* stream);

/* ---- tools -------------------------------------------------------------------
 * GraphColoring tool (GraphColoring/GraphColoring.cpp:157-196) on a tet list:
 * MCS (Modules/GraphColoring/mcs.cpp:14-168) and OrderedGreedy (gready.cpp:15-117),
 * bit-exact with the reference. Return the number of colors, or -1 on error. */
int32_t gaia_vbd_color_mcs(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors);
int32_t gaia_vbd_color_greedy(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors);
/* Jones-Plassmann coloring on the GPU (hashed vertex priorities from `seed`, lowest free
 * color): a faster alternative for meshes without a coloring file; not the reference's
 * coloring. Same graph and return value as the two above. */
int32_t gaia_vbd_color_gpu(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors, uint32_t seed);
/* The GraphColoring tool as a whole (GraphColoring/GraphColoring.cpp:157-196): MCS
 * (algorithm 0, the tool's default) or OrderedGreedy (1), then, with balance != 0 (the
 * tool's default, goal ratio 1.05), balanceColoredCategories. colors receives each
 * vertex's color; order (nv ints, optional) the vertices of every category in the order
 * the tool writes them. Returns the number of colors, or -1 on error. */
int32_t gaia_vbd_color_tool(int32_t nv, int32_t ntet, const int32_t* tets, int32_t algorithm, int32_t balance,
                            float goal_ratio, int32_t* colors, int32_t* order);
/* Write categories in a given vertex order (`order` from gaia_vbd_color_tool). */
int gaia_vbd_write_categories(const char* path, int32_t nv, const int32_t* colors, const int32_t* order);
/* Write a coloring as the reference's JSON list of lists (ColoringAlgorithms.cpp:200-211). */
int gaia_vbd_write_coloring(const char* path, int32_t nv, const int32_t* colors);
/* Write a .t mesh ("Vertex id x y z" / "Tet id a b c d"). */
int gaia_vbd_write_t(const char* path, int32_t nv, const double* X, int32_t ntet, const int32_t* tets);

#ifdef __cplusplus
}
#endif
#endif /* GAIA_VBD_H */
