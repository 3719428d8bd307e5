// Checker build of the reference's own VBD device functions — TEST INFRASTRUCTURE ONLY.
//
// `make -C oracle ref` compiles this file into oracle/_ref/libvbd_ref32.so and, with
// REF_AS_DOUBLE, into oracle/_ref/libvbd_ref64.so. It includes the reference's device
// headers from the reference tree (VBD/VBDPhysicsCompute.h, VBD/VBD_GeneralCompute.h and
// what they include; VBD_GeneralCompute.h through a generated copy that only drops the
// redundant GAIA:: qualifiers GCC rejects) and the bodies of its host/device functions taken unchanged from
// VBD/VBDPhysicsCompute.cu by oracle/extract_ref.py (that file also holds the kernels,
// which do not compile on the host):
//   evaluateNeoHookeanMaterialForceAndHessian (:2035-2232) with assembleVertexVForceAndHessian
//     (:36-94), evaluateNeoHookeanEnergy (:1775-1810),
//   accumulateCollisionForceAndHessian (:1731-1773), accumlateCollisionForceAndHessianPerCollision_v2
//     (:1812-1930), updateVertexVelocity (:1250-1260), dampVelocity (:1397-1413);
// from VBD_GeneralCompute.h: accumulateInertiaForceAndHessian (:68-85),
// accumulateBoundaryForceAndHessianGPU (:87-166) with accumulateVertexFrictionGPU (:10-66),
// closestPointTriangle (:180-268).
// The CuMatrix helpers they call come from ref_shim/ (the submodule is empty; conventions
// stated there). The float build is the reference's arithmetic (FloatingTypeGPU = float,
// TetMesh/TetMeshFEMGPU.h:6); the double build compiles the same bodies with `float`
// defined as `double`, which gives the reference's formulas in FP64 for a tight pin.
//
// What this file adds is only the composition the reference's kernels perform around
// those functions, restated here because __global__ code does not run on the host:
//   * ref_vertex_force_hessian: VBDSolveParallelGroup_allInOne_kernel_V2
//     (VBDPhysicsCompute.cu:803-908) for one vertex: 32 per-thread force/Hessian slots,
//     incident tets beyond 32 accumulated into slot (index mod 32), the shared-memory tree
//     reduction j = 16, 8, 4, 2, 1, then inertia, collision and boundary terms;
//   * ref_step: runStepGPU (VBD/VBDPhysics.cpp:839-969) without contact detection, deformers
//     or accelerator: initial step (VBD_BaseMaterial.h:201-259, VBD_BaseMaterial.cpp:7-31,
//     initialization type 0), per iteration every parallel group solved Jacobi-style into
//     positionsNew and committed (VBDSolveParallelGroup_updateVertexPosition_kernel,
//     :946-968), the CMP_EPSILON2 gate (Types/Types.h:20-21) and the fallback step along the
//     force when the 3x3 solve fails, then VBDUpdateVelocity_kernel (:190-215). The 3x3
//     solve is CuMatrix::solve3x3_psd_stable, whose source is absent: it is the LDL^T with a
//     relative pivot threshold that the oracle and the CUDA kernels also use.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef REF_AS_DOUBLE
#define float double
#endif

#include "VBDPhysicsCompute.h"
// VBD_GeneralCompute.h as written, less the redundant GAIA:: qualifiers of the definitions
// inside its namespace, which GCC rejects (extract_ref.py --host-header)
#include "VBD_GeneralCompute_host.h"

using namespace GAIA;

#include "vbd_compute_functions.inc"

typedef FloatingTypeGPU FT;

namespace {

// Same LDL^T as the oracle's solve3x3_ldlt (row-major 3x3 in, x out).
bool ldlt_solve(const FT* H, const FT* b, FT* x, FT rel_tol) {
    FT scale = std::fabs(H[0]);
    if (std::fabs(H[4]) > scale) scale = std::fabs(H[4]);
    if (std::fabs(H[8]) > scale) scale = std::fabs(H[8]);
    if (!(scale > FT(0))) return false;
    const FT tol = rel_tol * scale;
    const FT d0 = H[0];
    if (!(d0 > tol)) return false;
    const FT l10 = H[3] / d0, l20 = H[6] / d0;
    const FT d1 = H[4] - l10 * H[3];
    if (!(d1 > tol)) return false;
    const FT l21 = (H[7] - l20 * H[3]) / d1;
    const FT d2 = H[8] - l20 * H[6] - l21 * l21 * d1;
    if (!(d2 > tol)) return false;
    FT z0 = b[0], z1 = b[1] - l10 * z0, z2 = b[2] - l20 * z0 - l21 * z1;
    z0 /= d0;
    z1 /= d1;
    z2 /= d2;
    x[2] = z2;
    x[1] = z1 - l21 * x[2];
    x[0] = z0 - l10 * x[1] - l20 * x[2];
    return std::isfinite(x[0]) && std::isfinite(x[1]) && std::isfinite(x[2]);
}

}  // namespace

extern "C" {

// One mesh, host arrays in the reference's device layout (3 values per vertex, DmInv 9
// per tet column-major, CSR of incident tets as vertexNeighborTets_infos (start, count)).
struct RefMesh {
    int32_t nv, ntet;
    FT* pos;             // 3 nv
    FT* prev;            // 3 nv
    FT* inertia;         // 3 nv
    FT* vel;             // 3 nv
    FT* pos_new;         // 3 nv scratch
    const FT* mass;      // nv
    const int8_t* fixed; // nv
    const int32_t* tets; // 4 ntet
    const FT* dminv;     // 9 ntet
    const FT* vol;       // ntet
    const int32_t* nbr_info;   // 2 nv
    const int32_t* nbr_tet;    // incidences
    const int32_t* nbr_order;  // incidences
    FT mu, lmbd, kh, kd;
    FT friction_dynamic, friction_eps_v;
    FT max_velocity, exp_vel_damping, const_vel_damping;
    // collision records, 23 ints per vertex (or null): activeColliding, closest face
    // vertices (3), face id, face mesh, number of relations, 4 x (mesh, primitive, type, order)
    const int32_t* coll;
};

struct RefPhysics {
    FT dt, dt_sqr_recip;
    FT world[6];
    FT boundary_stiffness, boundary_friction_mu, boundary_friction_eps_v;
    FT collision_stiffness;
    FT step_size, step_size_gd;
    FT gravity[3];
    FT pivot_tol;  // relative LDL^T pivot threshold of the 3x3 solve
};

int ref_float_bytes() { return int(sizeof(FT)); }

// evaluateNeoHookeanMaterialForceAndHessian on one tet (tetId 0, vertices 0..3 in x);
// accumulates into f (3) and h (9, column-major as the kernel's hessian).
void ref_nh_element(const FT* x, const FT* xprev, const FT* dminv, FT mu, FT lmbd, FT A, int32_t vorder, FT kh,
                    FT kd, FT dt, FT* f, FT* h) {
    const int32_t ids[4] = {0, 1, 2, 3};
    evaluateNeoHookeanMaterialForceAndHessian(mu, lmbd, A, 0, vorder, ids, x, xprev, dminv, f, h, kh, kd, dt);
}

FT ref_nh_energy(const FT* x, const FT* dminv, FT mu, FT lmbd, FT A) {
    const int32_t ids[4] = {0, 1, 2, 3};
    std::vector<FT> xs(x, x + 12);
    return evaluateNeoHookeanEnergy(mu, lmbd, A, 0, ids, xs.data(), dminv);
}

}  // extern "C"

namespace {

// The device structs of the reference over a scene's host arrays.
struct Scene {
    std::vector<TetMeshTopologyGPU> topo;
    std::vector<VBDTetMeshNeoHookeanGPU> meshes;
    std::vector<VBDBaseTetMeshGPU*> mesh_ptrs;
    std::vector<std::vector<CollisionDataGPU>> coll;
    std::vector<std::vector<int8_t>> active;
    std::vector<std::vector<int32_t>> nbr_pairs;
    VBDPhysicsDataGPU phys{};

    Scene(RefMesh* ms, int nmesh, const RefPhysics* p) {
        topo.resize(nmesh);
        meshes.resize(nmesh);
        coll.resize(nmesh);
        active.resize(nmesh);
        nbr_pairs.resize(nmesh);
        for (int m = 0; m < nmesh; ++m) {
            RefMesh& R = ms[m];
            TetMeshTopologyGPU& T = topo[m];
            std::memset(&T, 0, sizeof(T));
            T.tetVIds = const_cast<int32_t*>(R.tets);
            T.vertexNeighborTets = const_cast<int32_t*>(R.nbr_tet);
            T.vertexNeighborTets_vertexOrder = const_cast<int32_t*>(R.nbr_order);
            T.vertexNeighborTets_infos = const_cast<int32_t*>(R.nbr_info);
            T.nVerts = R.nv;
            T.nTets = R.ntet;
            VBDTetMeshNeoHookeanGPU& M = meshes[m];
            std::memset(static_cast<void*>(&M), 0, sizeof(M));
            M.pTopology = &T;
            M.vertexMass = const_cast<FT*>(R.mass);
            M.DmInvs = const_cast<FT*>(R.dminv);
            M.tetRestVolume = const_cast<FT*>(R.vol);
            M.vertPos = R.pos;
            M.vertPrevPos = R.prev;
            M.velocity = R.vel;
            M.vertexFixedMask = const_cast<int8_t*>(R.fixed);
            M.activeForCollision = true;
            M.activeForMaterialSolve = true;
            M.positionsNew = R.pos_new;
            M.inertia = R.inertia;
            coll[m].assign(size_t(R.nv), CollisionDataGPU{});
            for (int32_t v = 0; v < R.nv; ++v) {
                CollisionDataGPU& c = coll[m][size_t(v)];
                std::memset(&c, 0, sizeof(c));
                if (!R.coll) continue;
                const int32_t* r = R.coll + 23 * size_t(v);
                c.activeColliding = r[0];
                c.closestSurfaceFaceVIds[0] = r[1];
                c.closestSurfaceFaceVIds[1] = r[2];
                c.closestSurfaceFaceVIds[2] = r[3];
                c.closestSurfaceFaceId = r[4];
                c.intersectedTMeshId = r[5];
                c.numCollisionRelations = r[6];
                for (int k = 0; k < GPU_COLLISION_RELATION_PREALLOCATION_SIZE; ++k) {
                    c.collisionRelations[k].meshId = r[7 + 4 * k];
                    c.collisionRelations[k].collisionPrimitiveId = r[8 + 4 * k];
                    c.collisionRelations[k].collisionType = r[9 + 4 * k];
                    c.collisionRelations[k].collisionVertexOrder = r[10 + 4 * k];
                }
            }
            M.collisionData = coll[m].data();
            active[m].assign(size_t(R.nv), 0);
            M.activeCollisionMask = active[m].data();
            M.maxVelocityMagnitude = R.max_velocity;
            M.exponentialVelDamping = R.exp_vel_damping;
            M.constantVelDamping = R.const_vel_damping;
            M.frictionDynamic = R.friction_dynamic;
            M.frictionEpsV = R.friction_eps_v;
            M.lmbd = R.lmbd;
            M.miu = R.mu;
            M.dampingHydrostatic = R.kh;
            M.dampingDeviatoric = R.kd;
        }
        for (auto& M : meshes) mesh_ptrs.push_back(&M);
        phys.dt = p->dt;
        phys.tetMeshes = mesh_ptrs.data();
        phys.numMeshes = nmesh;
        for (int k = 0; k < 6; ++k) phys.worldBounds[k] = p->world[k];
        phys.boundaryCollisionStiffness = p->boundary_stiffness;
        phys.boundaryFrictionDynamic = p->boundary_friction_mu;
        phys.boundaryFrictionEpsV = p->boundary_friction_eps_v;
        phys.collisionStiffness = p->collision_stiffness;
        phys.dtSqrReciprocal = p->dt_sqr_recip;
        phys.stepSize = p->step_size;
        phys.stepSizeGD = p->step_size_gd;
    }
};

constexpr int kThreads = NUM_THREADS_VERTEX_SWEEP;

// The per-vertex part of VBDSolveParallelGroup_allInOne_kernel_V2 up to the 3x3 solve:
// force (3) and Hessian (9, column-major) of vertex v of mesh m, in the kernel's order.
void vertex_force_hessian(Scene& S, int m, int v, FT* out12) {
    VBDTetMeshNeoHookeanGPU* pTetMeshGPU = &S.meshes[size_t(m)];
    const TetMeshTopologyGPU* pTopology = pTetMeshGPU->pTopology;
    FT slots[kThreads][12];
    std::memset(slots, 0, sizeof(slots));
    const int32_t start = pTopology->vertexNeighborTets_infos[v * 2];
    const int32_t num = pTopology->vertexNeighborTets_infos[v * 2 + 1];
    for (int tid = 0; tid < kThreads; ++tid) {
        FT* forceAndHessian = slots[tid];
        FT* hessian = forceAndHessian + 3;
        auto one = [&](int index) {
            const int32_t tet = pTopology->vertexNeighborTets[start + index];
            const int32_t order = pTopology->vertexNeighborTets_vertexOrder[start + index];
            const int32_t* tetVIds = pTopology->tetVIds + 4 * tet;
            evaluateNeoHookeanMaterialForceAndHessian(pTetMeshGPU->miu, pTetMeshGPU->lmbd, pTetMeshGPU->tetRestVolume[tet],
                                                      tet, order, tetVIds, pTetMeshGPU->vertPos, pTetMeshGPU->vertPrevPos,
                                                      pTetMeshGPU->DmInvs, forceAndHessian, hessian,
                                                      pTetMeshGPU->dampingHydrostatic, pTetMeshGPU->dampingDeviatoric,
                                                      S.phys.dt);
        };
        if (tid < num) one(tid);
        if (num > kThreads) {
            const int extra = num - kThreads;
            for (int i = 0; i < extra; i += kThreads) {
                const int index = tid + kThreads + i;
                if (index < num) one(index);
            }
        }
    }
    for (int j = kThreads / 2; j > 0; j >>= 1)
        for (int tid = 0; tid < j; ++tid)
            for (int k = 0; k < 12; ++k) slots[tid][k] = slots[tid][k] + slots[tid + j][k];
    FT* forceAndHessian = slots[0];
    FT* hessian = forceAndHessian + 3;
    accumulateInertiaForceAndHessian(pTetMeshGPU, v, S.phys.dtSqrReciprocal, forceAndHessian, hessian);
    accumulateCollisionForceAndHessian(&S.phys, pTetMeshGPU, v, forceAndHessian, hessian);
    accumulateBoundaryForceAndHessianGPU(&S.phys, pTetMeshGPU, v, forceAndHessian, hessian);
    std::memcpy(out12, forceAndHessian, 12 * sizeof(FT));
}

}  // namespace

extern "C" {

// Force (3) and Hessian (9, column-major) of one vertex, composed as the V2 kernel does.
int ref_vertex_force_hessian(RefMesh* meshes, int32_t nmesh, const RefPhysics* p, int32_t mesh, int32_t vertex,
                             FT* f3, FT* h9) {
    if (mesh < 0 || mesh >= nmesh || vertex < 0 || vertex >= meshes[mesh].nv) return -1;
    Scene S(meshes, nmesh, p);
    FT out[12];
    vertex_force_hessian(S, mesh, vertex, out);
    std::memcpy(f3, out, 3 * sizeof(FT));
    std::memcpy(h9, out + 3, 9 * sizeof(FT));
    return 0;
}

// n_steps steps of runStepGPU with one substep, `iterations` iterations, no contact
// detection (collision records as given, usually none), no deformers and no accelerator.
// groups: the parallel groups as (mesh, vertex) pairs, group g in
// pairs[2 * group_ofs[g] .. 2 * group_ofs[g + 1]). Returns the number of failed solves.
int ref_step(RefMesh* meshes, int32_t nmesh, const RefPhysics* p, int32_t ngroups, const int32_t* group_ofs,
             const int32_t* pairs, int32_t iterations, int32_t n_steps) {
    Scene S(meshes, nmesh, p);
    int failed = 0;
    for (int step = 0; step < n_steps; ++step) {
        // initial step: x_prev = x, v += dt g, inertia y = x + dt v, x = y
        for (int m = 0; m < nmesh; ++m) {
            RefMesh& R = meshes[m];
            for (int32_t v = 0; v < R.nv; ++v) {
                FT* x = R.pos + 3 * v;
                FT* vel = R.vel + 3 * v;
                for (int k = 0; k < 3; ++k) {
                    R.prev[3 * v + k] = x[k];
                    vel[k] += p->dt * p->gravity[k];
                    if (R.fixed[v]) vel[k] = 0;
                    R.inertia[3 * v + k] = x[k] + p->dt * vel[k];
                    x[k] = R.inertia[3 * v + k];
                }
            }
        }
        for (int it = 0; it < iterations; ++it) {
            for (int g = 0; g < ngroups; ++g) {
                for (int32_t i = group_ofs[g]; i < group_ofs[g + 1]; ++i) {
                    const int m = pairs[2 * i], v = pairs[2 * i + 1];
                    VBDTetMeshNeoHookeanGPU* M = &S.meshes[size_t(m)];
                    if (M->vertexFixedMask[v]) continue;
                    FT fh[12];
                    vertex_force_hessian(S, m, v, fh);
                    FT vNew[3];
                    CuMatrix::vec3Set(vNew, M->getVert(v));
                    if (CuMatrix::vec3NormSquare(fh) > FT(1e-5f) * FT(1e-5f)) {
                        // column-major 9 = row-major for the symmetric block
                        FT dx[3];
                        const bool ok = ldlt_solve(fh + 3, fh, dx, p->pivot_tol);
                        FT stepSize = ok ? S.phys.stepSize : S.phys.stepSizeGD;
                        if (!ok) {
                            ++failed;
                            CuMatrix::vec3Set(dx, fh);
                        }
                        CuMatrix::vec3MulAddTo(dx, stepSize, vNew);
                    }
                    CuMatrix::vec3Set(M->getVertPosNew(v), vNew);
                }
                for (int32_t i = group_ofs[g]; i < group_ofs[g + 1]; ++i) {
                    const int m = pairs[2 * i], v = pairs[2 * i + 1];
                    VBDTetMeshNeoHookeanGPU* M = &S.meshes[size_t(m)];
                    if (!M->vertexFixedMask[v]) CuMatrix::vec3Set(M->getVert(v), M->getVertPosNew(v));
                }
            }
        }
        for (int m = 0; m < nmesh; ++m) {
            VBDTetMeshNeoHookeanGPU* M = &S.meshes[size_t(m)];
            for (int32_t v = 0; v < meshes[m].nv; ++v) {
                FT* vel = M->velocity + 3 * v;
                if (M->vertexFixedMask[v]) {
                    vel[0] = vel[1] = vel[2] = 0;
                } else {
                    updateVertexVelocity(M, v, S.phys.dt);
                    dampVelocity(vel, M->maxVelocityMagnitude, M->exponentialVelDamping, M->constantVelDamping);
                }
            }
        }
    }
    return failed;
}

}  // extern "C"
