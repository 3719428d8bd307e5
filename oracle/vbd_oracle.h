/*
 * CPU oracle for the VBD step — TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, on the CPU and in plain C++, the reference's own
 * algorithm for Gaia's Vertex Block Descent step so that the CUDA path can be
 * checked against it. Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs may load it. The product library
 * (libgaia_vbd.so) never links, loads or calls anything here.
 *
 * Parity anchors:
 *   - vertex coloring (MCS, OrderedGreedy): pinned bit-exactly against the
 *     reference's 18 shipped *.t.vertexColoring.json fixtures;
 *   - the VBD step: restated from the reference's CPU path
 *     (Simulator/Modules/VBD/VBDPhysics.cpp:1580-1632, 2402-2483;
 *      VBD_NeoHookean.cpp:379-581). The reference cannot be built here
 *     (its CuMatrix / MeshFrame2 submodules are empty), so per-step
 *     trajectories are "parity unpinned" beyond this restatement.
 */
#ifndef GAIA_VBD_ORACLE_H
#define GAIA_VBD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t nv, ntet;
    const double* X;            /* 3*nv initial positions (x,y,z per vertex) */
    const double* V0;           /* 3*nv initial velocities, or NULL = zero */
    const int32_t* tets;        /* 4*ntet vertex ids */
    const int8_t* fixed;        /* nv fixed flags, or NULL */
    int32_t ncolors;            /* vertex color categories as read from JSON (unsorted) */
    const int32_t* color_offsets; /* ncolors+1 */
    const int32_t* color_verts;
    double miu, lmbd, density;
    double damping_hydrostatic, damping_deviatoric;
    double exp_vel_damping, const_vel_damping;   /* raw JSON values */
    double friction_dynamic, friction_eps_v;
    int32_t init_type;
    int32_t active;             /* activeForMaterialSolve */
} OracleMesh;

typedef struct {
    double time_step;
    int32_t num_substeps, iterations;
    double gravity[3];
    double world_lo[3], world_hi[3];
    int32_t use_plane_ground;
    double boundary_stiffness, boundary_friction_mu, boundary_friction_eps_v;
    double step_size, step_size_gd;
    int32_t friction_start_iter;
    int32_t associate_gravity;
    int32_t use_accelerator;
    double accelerator_rho;
    /* tet-mesh contact (CollisionParams allowCCD / allowDCD; PhysicsParams
       collisionStiffness, collisionOffHeight, intermediateCollisionIterations) */
    int32_t allow_ccd, allow_dcd;
    double collision_stiffness, collision_off_height;
    int32_t intermediate_collision_iterations;
    int32_t handle_self_collision, check_feasible_region;
    double feasible_region_eps;
    /* the DCD closest-point query's tetrahedral traversal (CollisionParams
       checkTetTraverse, tetrahedralTraverseForNonSelfIntersection,
       stopTraversingAfterPassingQueryPoint, shiftQueryPointToCenter, useStaticTraverse,
       centerShiftLevel, rayTriIntersectionEPSILON, maxSearchDistanceMultiplier) */
    int32_t check_tet_traverse, traverse_non_self, stop_traversing_after_passing, shift_query_to_center,
        use_static_traverse;
    double center_shift_level, ray_tri_eps, max_search_mult;
} OracleParams;

typedef struct {
    int32_t type;               /* 0 = Rotator, 1 = Translator */
    double center[3], axis[3];
    double angular_velocity, end_time;
    double speed[3];
    int32_t nsel;               /* number of (mesh, vertex) pairs */
    const int32_t* sel_mesh;
    const int32_t* sel_vert;
} OracleDeformer;

/* .t reader: call with X == NULL to get the counts. Returns 0, or -1 if unreadable. */
int32_t oracle_read_t(const char* path, int32_t* nv, int32_t* ntet, double* X, int32_t* tets);

/* Graph coloring restatements (return number of colors, -1 on error). */
int32_t oracle_color_mcs(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors);
int32_t oracle_color_greedy(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors);
/* The GraphColoring tool: MCS (0) or OrderedGreedy (1), then balanceColoredCategories when
 * balance != 0; colors per vertex and the written categories' vertex order. */
int32_t oracle_color_tool(int32_t nv, int32_t ntet, const int32_t* tets, int32_t algorithm, int32_t balance,
                          float goal, int32_t* colors, int32_t* order);

/* Simulation. precision = 64 (double) or 32 (float). nthreads <= 0: all cores. */
void* oracle_create(int32_t precision, int32_t nmesh, const OracleMesh* meshes,
                    const OracleParams* params, int32_t ndef, const OracleDeformer* defs,
                    int32_t nthreads);
void oracle_destroy(void* h);
int32_t oracle_step(void* h, int32_t nsteps);
/* Run only `iterations` solver iterations of one substep (a bounded timing sample). */
int32_t oracle_substep_sample(void* h, int32_t iterations);
void oracle_get_positions(void* h, int32_t mesh, double* out);
void oracle_get_velocities(void* h, int32_t mesh, double* out);
void oracle_set_positions(void* h, int32_t mesh, const double* in);
void oracle_set_velocities(void* h, int32_t mesh, const double* in);
void oracle_get_rest(void* h, int32_t mesh, double* dminv, double* vol, double* mass);
int32_t oracle_num_groups(void* h);
int32_t oracle_group_size(void* h, int32_t g);          /* number of (mesh, vertex) pairs */
void oracle_group(void* h, int32_t g, int32_t* out);    /* 2*size ints: mesh, vertex */
/* Force and 3x3 Hessian of one vertex at the current state (material+inertia+boundary). */
void oracle_vertex_force_hessian(void* h, int32_t mesh, int32_t v, int32_t apply_friction,
                                 double* f3, double* h9);
/* Total elastic (Neo-Hookean, rest energy removed) + inertia energy, in double. */
double oracle_energy(void* h);
int32_t oracle_solve_failures(void* h);
/* evaluateConvergence in FP64: energy, inertia energy, elastic energy, average force norm
 * (material with damping plus inertia; zero for fixed vertices; over all vertices). */
void oracle_convergence(void* h, double* out4);
/* One tet's Neo-Hookean force (3) and Hessian (9, row-major) on its vertex `order` in
 * FP64, the per-tet term of oracle_vertex_force_hessian; accumulated into f and h. */
void oracle_nh_element(const double* x12, const double* xprev12, const double* dminv9, double mu, double lmbd,
                       double A, int32_t order, double kh, double kd, double dt, double* f, double* h);

/* Tet-mesh contact. oracle_collide runs the substep-start detection on the current
 * positions (trajectories from the previous positions) and builds the contact
 * records the solve reads; it returns the number of vertices in contact (v side).
 * oracle_get_contacts writes, per such vertex in (mesh, surface vertex) order,
 * 8 ints: mesh, vertex, face mesh, face vertex 0..2, surface face index, kind
 * (1 = CCD, 2 = DCD); it returns the row count (rows beyond cap are not written). */
void oracle_set_prev_positions(void* h, int32_t mesh, const double* in);
int32_t oracle_collide(void* h);
int32_t oracle_get_contacts(void* h, int32_t* rows, int32_t cap);
int32_t oracle_num_surface(void* h, int32_t mesh, int32_t* nverts);

#ifdef __cplusplus
}
#endif
#endif
