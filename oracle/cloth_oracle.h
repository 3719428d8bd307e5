/* Test infrastructure only: CPU restatement of Gaia's cloth VBD step, the checker
 * of the GPU cloth path. Nothing in the product links or calls it. */
#ifndef GAIA_CLOTH_ORACLE_H
#define GAIA_CLOTH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ClothOracleMesh {
    int32_t nv, nf;
    const double* X;          /* 3*nv positions (already rotated / scaled / translated, FP32 values) */
    const int32_t* faces;     /* 3*nf */
    int32_t is_collider;
    /* simulated meshes: */
    const int8_t* fixed;      /* nv */
    int32_t ncolors;
    const int32_t* color_offsets; /* ncolors + 1 */
    const int32_t* color_verts;   /* colors in file order (sorted large to small by the oracle) */
    double density, miu, lambda_, damping_stvk, damping_bending, bending_stiffness;
    double friction_dynamic, friction_eps_v, exp_vel_damping, const_vel_damping, max_velocity, no_grav_threshold;
    int32_t has_no_grav_zone, init_type;
} ClothOracleMesh;

typedef struct ClothOracleParams {
    double gravity[3];
    double dt;                /* substep length */
    int32_t num_substeps, iterations;
    double world_lo[3], world_hi[3];
    double boundary_friction_dynamic, boundary_contact_stiffness, boundary_friction_eps;
    double step_size;
    int32_t associate_gravity, handle_collision, apply_acceleration, cd_every_iteration;
    double contact_stiffness, contact_radius, thickness, relaxation, degenerate_thres, accelerator_rho;
    double max_query_dis;
} ClothOracleParams;

void* cloth_oracle_create(int32_t nmesh, const ClothOracleMesh* meshes, const ClothOracleParams* p, int32_t nthreads);
void cloth_oracle_destroy(void* h);
const char* cloth_oracle_error(void);
void cloth_oracle_step(void* h, int32_t n);
void cloth_oracle_get_positions(void* h, int32_t mesh, double* out);
void cloth_oracle_set_positions(void* h, int32_t mesh, const double* in);
void cloth_oracle_get_velocities(void* h, int32_t mesh, double* out);
void cloth_oracle_detect(void* h);
int64_t cloth_oracle_vf_contacts(void* h, int32_t* rows4, int64_t cap);
int64_t cloth_oracle_ee_contacts(void* h, int32_t* rows4, int64_t cap);
void cloth_oracle_bounds(void* h, int32_t mesh, double* out);
void cloth_oracle_min_distances(void* h, int32_t mesh, float* vf, float* fv, float* ee);
int32_t cloth_oracle_num_edges(void* h, int32_t mesh);
void cloth_oracle_topology(void* h, int32_t mesh, int32_t* edges6, int32_t* face_edges3);
void cloth_oracle_rest(void* h, int32_t mesh, double* dminv4, double* area, double* mass);
int32_t cloth_oracle_num_groups(void* h);
int64_t cloth_oracle_group(void* h, int32_t g, int32_t* pairs);
/* Elastic energy (membrane + bending) of a simulated mesh at the current positions and
 * the force / 3x3 Hessian of those two terms at one vertex (no damping). */
double cloth_oracle_elastic_energy(void* h, int32_t mesh);
void cloth_oracle_elastic_force_hessian(void* h, int32_t mesh, int32_t v, double* f3, double* h9);
/* Force and Hessian the block solve of one vertex would use (contacts, inertia, membrane
 * with damping, bending, world box). */
void cloth_oracle_vertex_force_hessian(void* h, int32_t mesh, int32_t v, double* f3, double* h9);
int64_t cloth_oracle_counter(void* h, int32_t which); /* 0 detections, 1 truncations, 2 failed solves */

#ifdef __cplusplus
}
#endif
#endif
