// GB300 VBD engine (the class template behind every handle of libgaia_vbd.so).
//
// One handle = one scene on one GPU: device buffers in the slot layout
// described in vbd_kernels.cuh, one CUDA stream, and three CUDA graphs per
// substep (initial step + deformers | all color sweeps of all iterations |
// velocity update). The graphs replace the reference's per-iteration graph
// (VBDPhysics.cpp:1546-1570) and its host<->device syncs per substep.
//
// Each precision mode instantiates the template in a translation unit of its own
// (vbd_engine_<mode>.cu, through the make_engine_* factories), so that they compile in
// parallel; the C ABI (vbd_engine.cu) holds only the base class.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gaia_vbd.h"
#include "scene.hpp"
#include "state_io.hpp"
#include "tet_cd.hpp"
#include "vbd_cluster.cuh"
#include "vbd_convergence.cuh"
#include "vbd_grid.cuh"
#include "vbd_kernels.cuh"

namespace gaia {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// A bounded device-side wait ran out (GAIA_VBD_E_DEVICE_TIMEOUT).
struct DeviceTimeout : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define GAIA_CUDA(call)                                                                                  \
    do {                                                                                                 \
        cudaError_t e__ = (call);                                                                        \
        if (e__ != cudaSuccess)                                                                          \
            throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e__) + " (" + __FILE__ + ":" + \
                            std::to_string(__LINE__) + ")");                                             \
    } while (0)

namespace {

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    void alloc(size_t count, size_t* total) {
        if (p) cudaFree(p);
        p = nullptr;
        n = count;
        if (count) {
            GAIA_CUDA(cudaMalloc(&p, count * sizeof(T)));
            if (total) *total += count * sizeof(T);
        }
    }
    void upload(const std::vector<T>& h, size_t* total, cudaStream_t st) {
        alloc(h.size(), total);
        if (!h.empty()) GAIA_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    }
};

inline int div_up(int64_t a, int64_t b) { return int((a + b - 1) / b); }

}  // namespace

// One incidence record (layout in vbd_kernels.cuh).
template <typename R>
void make_record(int4& n, dev::R4<R>& a, dev::R4<R>& b, R* c, const int* nb, double mv[3][3]);
template <>
inline void make_record<float>(int4& n, dev::R4<float>& a, dev::R4<float>& b, float*, const int* nb,
                               double mv[3][3]) {
    float m2z = float(mv[2][2]);
    int bits;
    std::memcpy(&bits, &m2z, 4);
    n = make_int4(nb[0], nb[1], nb[2], bits);
    a = dev::R4<float>{float(mv[0][0]), float(mv[0][1]), float(mv[0][2]), float(mv[1][0])};
    b = dev::R4<float>{float(mv[1][1]), float(mv[1][2]), float(mv[2][0]), float(mv[2][1])};
}
template <>
inline void make_record<double>(int4& n, dev::R4<double>& a, dev::R4<double>& b, double* c, const int* nb,
                                double mv[3][3]) {
    n = make_int4(nb[0], nb[1], nb[2], 0);
    a = dev::R4<double>{mv[0][0], mv[0][1], mv[0][2], mv[1][0]};
    b = dev::R4<double>{mv[1][1], mv[1][2], mv[2][0], mv[2][1]};
    *c = mv[2][2];
}

enum { kSweepMerged = 0, kSweepScenes = 1, kSweepCluster = 2, kSweepGrid = 3 };
constexpr int kVariantDeep = 4;  // solve variant: k_solve_deep
constexpr int kVariantGrid = 5;  // solve variant: k_sweep_grid
constexpr int kVariantPrefetch = 6;  // solve variant: k_solve with the next wave's records prefetched into L2
constexpr int kVariantPipe = 7;      // solve variant: k_solve_pipe, double-buffered TMA tiles on a persistent grid

class EngineBase {
public:
    virtual ~EngineBase() {}
    virtual int mode() const = 0;
    virtual double tuned_ms() const = 0;
    virtual double measure_sweep_ms() = 0;
    virtual void run_steps(int n) = 0;
    virtual void run_steps_timed(int n, float* total_ms, float* sweep_ms) = 0;
    virtual void autotune() = 0;
    virtual void reset() = 0;
    virtual void get_positions(int mesh, double* out) = 0;
    virtual void set_positions(int mesh, const double* in) = 0;
    virtual void get_velocities(int mesh, double* out) = 0;
    virtual void set_velocities(int mesh, const double* in) = 0;
    virtual void set_state_f32(const float* x, const float* v) = 0;
    virtual void get_positions_f32(float* x) = 0;
    virtual void get_velocities_f32(float* v) = 0;
    virtual double energy() = 0;
    virtual void convergence(double* out4) = 0;
    virtual void convergence_log(std::vector<double>& rows) = 0;
    virtual void vertex_force_hessian(int mesh, int v, int friction, double* f3, double* h9) = 0;
    virtual void stats(gaia_vbd_stats* s) = 0;
    virtual void sync() = 0;
    virtual void color_config(int g, int32_t* L, int32_t* B, int32_t* variant, float* ms) const = 0;
    virtual double get_time() = 0;
    virtual void set_time(double t) = 0;
    // tet-mesh contact
    virtual void set_prev_positions(int mesh, const double* in) = 0;
    virtual int collide() = 0;
    virtual void contacts(std::vector<int32_t>& rows) = 0;
};

template <typename ST, typename R>
class Engine : public EngineBase {
    using S4 = typename ST::U;   // per-vertex displacement state
    using V4 = typename ST::V;   // per-vertex velocity
    using Sc = typename ST::Sc;
    using R4 = dev::R4<R>;

public:
    // cluster mode: a cluster size whose blocks hold every scene (states and owned records)
    struct ClusterFit {
        int C;
        int32_t pos_cap, rec_cap;
        size_t bytes;
    };

    // mode: kSweepMerged (one launch per merged color and iteration), kSweepScenes (one
    // persistent launch per substep running every scene's iterations, scene-major slots),
    // kSweepCluster (the same on thread-block clusters with the scene in shared memory) or
    // kSweepGrid (one cooperative launch per substep over the merged colors, a bounded grid
    // barrier between colors)
    Engine(const Scene& s, int mode) : sc_(s), mode_(mode) {
        GAIA_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        GAIA_CUDA(cudaEventCreate(&ev_a_));
        GAIA_CUDA(cudaEventCreate(&ev_b_));
        GAIA_CUDA(cudaEventCreate(&ev_c_));
        build_layout();
        upload();
        setup_contact();
        setup_frames();
        lanes_ = sc_.p.lanesPerVertex;
        block_ = sc_.p.blockSize;
        if (lanes_ != 0 && lanes_ != 2 && lanes_ != 4 && lanes_ != 8 && lanes_ != 16 && lanes_ != 32)
            throw std::runtime_error("lanesPerVertex must be 2, 4, 8, 16 or 32");
        if (block_ != 0 && (block_ < 64 || block_ > 256 || block_ % 32))
            throw std::runtime_error("blockSize must be a multiple of 32 in [64, 256]");
        use_pdl_ = sc_.p.usePDL;
        small_color_ = sc_.p.smallColorVertices;
        set_tma_smem_limits();
        variant_fixed_ = sc_.p.solveVariant;
        if (variant_fixed_ != -1 && variant_fixed_ != 0 && variant_fixed_ != 1 && variant_fixed_ != kVariantDeep &&
            variant_fixed_ != kVariantPrefetch && variant_fixed_ != kVariantPipe)
            throw std::runtime_error("solveVariant must be -1 (autotune), 0 (registers), 1 (TMA-staged), 4 (registers, "
                                     "deeper record pipeline), 6 (registers, next wave's records prefetched into L2) or "
                                     "7 (double-buffered TMA tiles on a persistent grid)");
        // the FP64 engine has neither the TMA variants nor the record prefetch
        if ((variant_fixed_ == 1 || variant_fixed_ == kVariantPrefetch || variant_fixed_ == kVariantPipe) &&
            sizeof(R) != 4)
            variant_fixed_ = 0;
        if (variant_fixed_ >= 0) variant_ = variant_fixed_;
        if (mode_ == kSweepScenes) {
            setup_scenes();
            if ((lanes_ == 0 || block_ == 0) && sc_.p.autotune) autotune_scenes();
            finalize_scenes();
        } else if (mode_ == kSweepCluster) {
            setup_scenes();
            setup_cluster();
            if ((lanes_ == 0 || block_ == 0 || sc_.p.clusterSize == 0) && sc_.p.autotune) autotune_cluster();
            finalize_cluster();
        } else if (mode_ == kSweepGrid) {
            setup_grid();
            if ((lanes_ == 0 || block_ == 0) && sc_.p.autotune) autotune_grid();
            finalize_grid();
        } else {
            if ((lanes_ == 0 || block_ == 0 || variant_fixed_ < 0) && sc_.p.autotune) autotune_impl();
            finalize_cfg();
        }
        if (sc_.p.evaluateConvergence) setup_conv();
        capture();
    }

    int mode() const override { return mode_; }

    void color_config(int g, int32_t* L, int32_t* B, int32_t* variant, float* ms) const override {
        if (g < 0 || size_t(g) >= ccfg_.size()) throw std::invalid_argument("color index out of range");
        if (L) *L = ccfg_[g].L;
        if (B) *B = ccfg_[g].B;
        if (variant) *variant = ccfg_[g].variant;
        if (ms) *ms = ccfg_[g].ms;
    }

    ~Engine() override {
        destroy_graphs();
        if (ev_a_) cudaEventDestroy(ev_a_);
        if (ev_b_) cudaEventDestroy(ev_b_);
        if (ev_c_) cudaEventDestroy(ev_c_);
        if (st_) cudaStreamDestroy(st_);
    }

    // ---- layout ---------------------------------------------------------------
    void build_layout() {
        const auto& meshes = sc_.meshes;
        nmesh_ = int(meshes.size());
        mesh_off_.assign(nmesh_ + 1, 0);
        for (int m = 0; m < nmesh_; ++m) mesh_off_[m + 1] = mesh_off_[m] + meshes[m].nv;
        nslots_ = mesh_off_[nmesh_];
        if (nslots_ > int64_t(INT32_MAX) / 2) throw std::runtime_error("scene too large for 32-bit vertex indices");
        slot_of_.assign(nslots_, -1);
        int32_t slot = 0;
        group_beg_.clear();
        group_end_.clear();
        scene_colors_.clear();
        scene_ofs_.assign(1, 0);
        if (mode_ == kSweepScenes || mode_ == kSweepCluster) {
            // scene-major: mesh by mesh, within a mesh its vertices of merged color 0, 1, ...
            std::vector<std::vector<std::vector<int32_t>>> per(size_t(nmesh_),
                                                               std::vector<std::vector<int32_t>>(sc_.groups.size()));
            for (size_t gi = 0; gi < sc_.groups.size(); ++gi) {
                const auto& g = sc_.groups[gi];
                for (size_t i = 0; i + 1 < g.size(); i += 2) {
                    const int m = g[i], v = g[i + 1];
                    if (!meshes[m].fixed[v]) per[size_t(m)][gi].push_back(v);
                }
            }
            for (int m = 0; m < nmesh_; ++m) {
                for (auto& verts : per[size_t(m)]) {
                    if (verts.empty()) continue;
                    const int32_t beg = slot;
                    for (int32_t v : verts) slot_of_[mesh_off_[m] + v] = slot++;
                    scene_colors_.push_back(make_int2(beg, slot));
                }
                scene_ofs_.push_back(int32_t(scene_colors_.size()));
            }
        } else {
            for (auto& g : sc_.groups) {
                group_beg_.push_back(slot);
                for (size_t i = 0; i + 1 < g.size(); i += 2) {
                    int m = g[i], v = g[i + 1];
                    if (!meshes[m].fixed[v]) slot_of_[mesh_off_[m] + v] = slot++;
                }
                group_end_.push_back(slot);
            }
        }
        nactive_ = slot;
        for (int64_t gi = 0; gi < nslots_; ++gi)
            if (slot_of_[gi] < 0) slot_of_[gi] = slot++;
        if (slot != nslots_) throw std::runtime_error("internal: slot assignment incomplete");
        orig_of_.assign(nslots_, 0);
        for (int64_t gi = 0; gi < nslots_; ++gi) orig_of_[slot_of_[gi]] = int32_t(gi);
        slot_mesh_.assign(nslots_, 0);
        for (int m = 0; m < nmesh_; ++m)
            for (int v = 0; v < meshes[m].nv; ++v) slot_mesh_[slot_of_[mesh_off_[m] + v]] = m;

        // incidence records in slot order
        inc_ofs_.assign(size_t(nactive_) + 1, 0);
        for (int32_t s = 0; s < nactive_; ++s) {
            int32_t gi = orig_of_[s];
            int m = slot_mesh_[s];
            int v = gi - int32_t(mesh_off_[m]);
            inc_ofs_[s + 1] = inc_ofs_[s] + (meshes[m].nbr_ofs[v + 1] - meshes[m].nbr_ofs[v]);
        }
        ninc_ = inc_ofs_[nactive_];
        if (int64_t(ninc_) > int64_t(INT32_MAX)) throw std::runtime_error("too many incidences");
        h_rec_n_.resize(ninc_);
        h_rec_a_.resize(ninc_);
        h_rec_b_.resize(ninc_);
        if (sizeof(R) == 8) h_rec_c_.resize(ninc_);
        for (int32_t s = 0; s < nactive_; ++s) {
            int32_t gi = orig_of_[s];
            int m = slot_mesh_[s];
            const TetMesh& M = meshes[m];
            int v = gi - int32_t(mesh_off_[m]);
            int32_t r = inc_ofs_[s];
            for (int k = M.nbr_ofs[v]; k < M.nbr_ofs[v + 1]; ++k, ++r) {
                int t = M.nbr_tet[k], o = M.nbr_order[k];
                const double* Di = &M.dminv[9 * size_t(t)];
                int others[3], q = 0;
                for (int j = 0; j < 4; ++j)
                    if (j != o) others[q++] = j;
                if (o & 1) std::swap(others[0], others[1]);  // keeps det[m0;m1;m2] = det(DmInv)
                double mv[3][3];
                int nb[3];
                for (int i = 0; i < 3; ++i) {
                    int j = others[i];
                    for (int c = 0; c < 3; ++c)
                        mv[i][c] = j == 0 ? -(Di[3 * c] + Di[3 * c + 1] + Di[3 * c + 2]) : Di[3 * c + (j - 1)];
                    nb[i] = slot_of_[mesh_off_[m] + M.tets[4 * size_t(t) + j]];
                }
                set_record(r, nb, mv);
            }
        }
        // per-slot state
        h_pos_.resize(nslots_);
        h_vel_.resize(nslots_);
        h_rest_.resize(nslots_);
        for (int m = 0; m < nmesh_; ++m) {
            const TetMesh& M = meshes[m];
            for (int v = 0; v < M.nv; ++v) {
                int32_t s = slot_of_[mesh_off_[m] + v];
                h_rest_[s] = make_float4(M.X[3 * size_t(v)], M.X[3 * size_t(v) + 1], M.X[3 * size_t(v) + 2], 0.f);
                const double zero[3] = {0.0, 0.0, 0.0};
                h_pos_[s] = ST::from_d(zero, M.mass[v]);  // displacement from rest, mass
                h_vel_[s] = V4{Sc(M.V[3 * size_t(v)]), Sc(M.V[3 * size_t(v) + 1]), Sc(M.V[3 * size_t(v) + 2]), Sc(0)};
            }
        }
        // materials
        h_mats_.resize(nmesh_);
        for (int m = 0; m < nmesh_; ++m) {
            const ObjectParams& o = sc_.objs[m];
            dev::MeshMat<R> mm{};
            mm.mu = R(o.miu);
            mm.lmbd = R(o.lmbd);
            mm.a = R(1.0 + o.miu / o.lmbd);
            mm.kh = R(o.dampingHydrostatic);
            mm.kd = R(o.dampingDeviatoric);
            mm.exp_damp = R(std::pow(o.exponentialVelDamping, sc_.p.dt));  // VBDPhysics.cpp:794-807
            mm.const_damp = R(o.constantVelDamping * sc_.p.dt);
            mm.init_type = o.initializationType;
            h_mats_[m] = mm;
        }
        // deformers
        for (size_t di = 0; di < sc_.defs.size(); ++di) {
            const DeformerParams& d = sc_.defs[di];
            dev::DeformerDev dd{};
            dd.type = d.type;
            for (int k = 0; k < 3; ++k) {
                dd.axis[k] = d.axis[k];
                dd.speed[k] = d.speed[k];
            }
            dd.omega = d.angularVelocity;
            dd.end_time = d.endTime;
            h_defs_.push_back(dd);
            for (size_t k = 0; k < d.selectedMeshes.size(); ++k) {
                int m = d.selectedMeshes[k];
                for (int32_t v : d.selectedVertices[k]) {
                    const float* X = &meshes[m].X[3 * size_t(v)];
                    double P[3] = {X[0], X[1], X[2]};
                    h_def_slot_.push_back(slot_of_[mesh_off_[m] + v]);
                    h_def_idx_.push_back(int32_t(di));
                    if (d.type == 0) {
                        double OP[3] = {P[0] - d.center[0], P[1] - d.center[1], P[2] - d.center[2]};
                        double dot = OP[0] * d.axis[0] + OP[1] * d.axis[1] + OP[2] * d.axis[2];
                        for (int c = 0; c < 3; ++c) {
                            double root = dot * d.axis[c];
                            h_def_a_.push_back(root);
                            h_def_b_.push_back(P[c] - root);
                        }
                    } else {
                        for (int c = 0; c < 3; ++c) {
                            h_def_a_.push_back(P[c]);
                            h_def_b_.push_back(0.0);
                        }
                    }
                }
            }
        }
        // constants
        const PhysicsParams& p = sc_.p;
        c_.dt = R(p.dt);
        c_.inv_dt = R(1.0 / p.dt);
        c_.dt2inv = R(p.dtSqrReciprocal);
        c_.dt_d = p.dt;
        c_.dt_f = float(p.dt);
        for (int k = 0; k < 3; ++k) {
            c_.g[k] = p.gravity[k];
            c_.lo[k] = p.worldLo[k];
            c_.hi[k] = p.worldHi[k];
            c_.g_f[k] = float(p.gravity[k]);
            c_.lo_f[k] = float(p.worldLo[k]);
            c_.hi_f[k] = float(p.worldHi[k]);
        }
        c_.kb = R(p.boundaryCollisionStiffness);
        c_.kc = R(p.collisionStiffness);
        c_.fr_mu = R(p.boundaryFrictionDynamic);
        c_.fr_epsU = R(p.boundaryFrictionEpsV * p.dt);
        c_.step = R(p.stepSize);
        c_.step_gd = R(p.stepSizeGD);
        c_.plane = p.usePlaneGround ? 1 : 0;
        c_.assoc_grav = p.associateGravityWithInertia ? 1 : 0;
        c_.spin_limit = p.waitPollLimit >= 0 ? p.waitPollLimit : dev::kMbarSpinLimit;
    }

    void set_record(int32_t r, const int* nb, double mv[3][3]) {
        make_record<R>(h_rec_n_[r], h_rec_a_[r], h_rec_b_[r], sizeof(R) == 8 ? &h_rec_c_[r] : nullptr, nb, mv);
    }

    void upload() {
        bytes_ = 0;
        d_pos_.upload(h_pos_, &bytes_, st_);
        d_rest_.upload(h_rest_, &bytes_, st_);
        d_vel_.upload(h_vel_, &bytes_, st_);
        d_y_.upload(h_pos_, &bytes_, st_);
        d_xprev_.upload(h_pos_, &bytes_, st_);
        d_vprev_.upload(h_vel_, &bytes_, st_);
        d_inc_ofs_.upload(inc_ofs_, &bytes_, st_);
        d_rec_n_.upload(h_rec_n_, &bytes_, st_);
        d_rec_a_.upload(h_rec_a_, &bytes_, st_);
        d_rec_b_.upload(h_rec_b_, &bytes_, st_);
        d_rec_c_.upload(h_rec_c_, &bytes_, st_);
        d_slot_mesh_.upload(slot_mesh_, &bytes_, st_);
        d_mats_.upload(h_mats_, &bytes_, st_);
        d_slot_of_.upload(slot_of_, &bytes_, st_);
        d_counters_.alloc(dev::CNT_N, &bytes_);
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p, 0, dev::CNT_N * sizeof(unsigned long long), st_));
        d_time_.alloc(1, &bytes_);
        GAIA_CUDA(cudaMemsetAsync(d_time_.p, 0, sizeof(double), st_));
        d_def_slot_.upload(h_def_slot_, &bytes_, st_);
        d_def_idx_.upload(h_def_idx_, &bytes_, st_);
        d_def_a_.upload(h_def_a_, &bytes_, st_);
        d_def_b_.upload(h_def_b_, &bytes_, st_);
        d_defs_.upload(h_defs_, &bytes_, st_);
        if (sc_.p.useAccelerator) {
            d_acc_pp_.alloc(nslots_, &bytes_);
            d_acc_prev_.alloc(nslots_, &bytes_);
        }
        d_stage_f32_.alloc(6 * size_t(nslots_), &bytes_);
        d_stage_f64_.alloc(3 * size_t(nslots_), &bytes_);
        d_probe_.alloc(12, &bytes_);
        GAIA_CUDA(cudaStreamSynchronize(st_));
        // keep host copies small: records are device-only from here on
        std::vector<int4>().swap(h_rec_n_);
        std::vector<R4>().swap(h_rec_a_);
        std::vector<R4>().swap(h_rec_b_);
        std::vector<R>().swap(h_rec_c_);
    }

    dev::Ptrs<ST, R> ptrs() const {
        dev::Ptrs<ST, R> P;
        P.u = d_pos_.p;
        P.rest = d_rest_.p;
        P.y = d_y_.p;
        P.xprev = d_xprev_.p;
        P.vel = d_vel_.p;
        P.vprev = d_vprev_.p;
        P.inc_ofs = d_inc_ofs_.p;
        P.rec_n = d_rec_n_.p;
        P.rec_a = d_rec_a_.p;
        P.rec_b = d_rec_b_.p;
        P.rec_c = d_rec_c_.p;
        P.slot_mesh = d_slot_mesh_.p;
        P.mats = d_mats_.p;
        P.counters = d_counters_.p;
        P.nactive = nactive_;
        P.nslots = int32_t(nslots_);
        const tetcd::Records rc = cd_.records();
        P.col_info = rc.info;
        P.col_own = rc.own;
        P.col_rel = rc.rel;
        P.mesh_fric = d_mesh_fric_.p;
        P.col_scratch = d_col_scratch_.p;
        P.frame_shift = frames_ ? d_frame_shift_.p : nullptr;
        P.frame_F = frames_ ? d_frame_F_.p : nullptr;
        P.rest_fh = frames_ ? d_rest_fh_.p : nullptr;
        P.rest_fl = frames_ ? d_rest_fl_.p : nullptr;
        return P;
    }

    // ---- mesh frames --------------------------------------------------------------------
    // FP32-compute engines keep each mesh's states relative to a frame offset F that follows
    // the mesh (k_frame_update, once per substep). Off with contact detection (contacts
    // couple meshes, whose frames differ) and with deformers (they set absolute positions).
    void setup_frames() {
        frames_ = sizeof(R) == 4 && sc_.p.meshFrames && !cd_.enabled() && h_def_slot_.empty() && nmesh_ > 0;
        if (!frames_) return;
        std::vector<int32_t> ref(size_t(nmesh_), -1);
        for (int m = 0; m < nmesh_; ++m)
            for (int v = 0; v < sc_.meshes[m].nv; ++v)
                if (!sc_.meshes[m].fixed[v]) {
                    ref[size_t(m)] = slot_of_[mesh_off_[m] + v];
                    break;
                }
        d_frame_ref_.upload(ref, &bytes_, st_);
        d_frame_F_.alloc(nmesh_, &bytes_);
        d_frame_shift_.alloc(nmesh_, &bytes_);
        d_rest_fh_.alloc(nslots_, &bytes_);
        d_rest_fl_.alloc(nslots_, &bytes_);
        reset_frames();
    }

    // F = 0, no shift, X + F = X
    void reset_frames() {
        if (!frames_) return;
        GAIA_CUDA(cudaMemsetAsync(d_frame_F_.p, 0, nmesh_ * sizeof(double4), st_));
        GAIA_CUDA(cudaMemsetAsync(d_frame_shift_.p, 0, nmesh_ * sizeof(float4), st_));
        GAIA_CUDA(cudaMemcpyAsync(d_rest_fh_.p, d_rest_.p, nslots_ * sizeof(float4), cudaMemcpyDeviceToDevice, st_));
        GAIA_CUDA(cudaMemsetAsync(d_rest_fl_.p, 0, nslots_ * sizeof(float4), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    const double4* frame_ptr() const { return frames_ ? d_frame_F_.p : nullptr; }

    // ---- tet-mesh contact -----------------------------------------------------------
    // Surface faces / vertices, surface rings and tets of all meshes in slot terms for
    // the detector, the detector itself, and the first hierarchies.
    void setup_contact() {
        const PhysicsParams& p = sc_.p;
        tetcd::Params prm;
        prm.ccd = p.allowCCD;
        prm.dcd = p.allowDCD;
        prm.handle_self = p.handleSelfCollision;
        prm.check_feasible = p.checkFeasibleRegion;
        prm.feasible_eps = float(p.feasibleRegionEpsilon);
        prm.off_height = float(p.collisionOffHeight);
        prm.check_traverse = p.checkTetTraverse;
        prm.traverse_non_self = p.tetrahedralTraverseForNonSelfIntersection;
        prm.stop_after_passing = p.stopTraversingAfterPassingQueryPoint;
        prm.shift_to_center = p.shiftQueryPointToCenter;
        prm.static_traverse = p.useStaticTraverse;
        prm.center_shift = float(p.centerShiftLevel);
        prm.ray_eps = float(p.rayTriIntersectionEPSILON);
        prm.max_search_mult = float(p.maxSearchDistanceMultiplier);
        tetcd::Topo t;
        t.nslots = int32_t(nslots_);
        t.face_ofs.assign(nmesh_ + 1, 0);
        std::vector<std::vector<int32_t>> ring(static_cast<size_t>(nslots_));
        for (int m = 0; m < nmesh_; ++m) {
            const TetMesh& M = sc_.meshes[m];
            auto slot = [&](int32_t v) { return slot_of_[mesh_off_[m] + v]; };
            const int32_t f0 = int32_t(t.faces.size());
            const size_t nf = M.sfaces.size() / 3;
            t.face_ofs[m + 1] = f0 + int32_t(nf);
            for (size_t f = 0; f < nf; ++f) {
                t.faces.push_back(make_int4(slot(M.sfaces[3 * f]), slot(M.sfaces[3 * f + 1]), slot(M.sfaces[3 * f + 2]), m));
                int32_t nb[3];
                for (int k = 0; k < 3; ++k) nb[k] = M.sface_nbr[3 * f + k] < 0 ? -1 : f0 + M.sface_nbr[3 * f + k];
                t.face_nbr.push_back(make_int4(nb[0], nb[1], nb[2], 0));
            }
            for (int32_t v : M.sverts) t.verts.push_back(make_int2(slot(v), m));
            for (int32_t v = 0; v < M.nv; ++v)
                for (int32_t r = M.sring_ofs[v]; r < M.sring_ofs[v + 1]; ++r) ring[slot(v)].push_back(slot(M.sring[r]));
            const int32_t t0 = int32_t(t.tets.size());
            for (size_t f = 0; f < nf; ++f) t.face_tet.push_back(make_int2(t0 + M.sface_tet[2 * f], M.sface_tet[2 * f + 1]));
            for (int32_t k = 0; k < M.ntet; ++k) {
                const int32_t* tv = &M.tets[4 * size_t(k)];
                t.tets.push_back(make_int4(slot(tv[0]), slot(tv[1]), slot(tv[2]), slot(tv[3])));
                t.tet_mesh.push_back(m);
                int32_t nb[4];
                for (int j = 0; j < 4; ++j) nb[j] = M.tet_nbr[4 * size_t(k) + j] < 0 ? -1 : t0 + M.tet_nbr[4 * size_t(k) + j];
                t.tet_nbr.push_back(make_int4(nb[0], nb[1], nb[2], nb[3]));
            }
        }
        t.ring_ofs.assign(size_t(nslots_) + 1, 0);
        for (int64_t s = 0; s < nslots_; ++s) {
            t.ring.insert(t.ring.end(), ring[s].begin(), ring[s].end());
            t.ring_ofs[s + 1] = int32_t(t.ring.size());
        }
        cd_.init(t, prm, bytes_);
        if (!cd_.enabled()) return;
        std::vector<double2> fr(nmesh_);
        for (int m = 0; m < nmesh_; ++m) fr[m] = make_double2(sc_.objs[m].frictionDynamic, sc_.objs[m].frictionEpsV);
        d_mesh_fric_.upload(fr, &bytes_, st_);
        d_xf_.alloc(2 * size_t(nslots_), &bytes_);
        d_col_scratch_.alloc(9 * size_t(nslots_), &bytes_);
        enqueue_gather();
        cd_.build(d_xf_.p, st_);
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    void enqueue_gather() {
        dev::k_gather_xf<ST><<<div_up(nslots_, 256), 256, 0, st_>>>(d_pos_.p, d_xprev_.p, d_rest_.p, d_xf_.p, int32_t(nslots_));
        GAIA_CUDA(cudaGetLastError());
    }

    // One detection pass on the current and start-of-substep positions.
    void enqueue_detection(bool intermediate, bool rebuild) {
        if (!cd_.enabled()) return;
        enqueue_gather();
        cd_.enqueue(d_xf_.p, intermediate, rebuild, st_);
    }

    // Contact sums of the vertices with records in [beg, end), before that color's solve.
    void launch_contact_color(int beg, int end, bool pdl) {
        const tetcd::Records rc = cd_.records();
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kContactBlocks);
        cfg.blockDim = dim3(128);
        cfg.stream = st_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = pdl ? attr : nullptr;
        cfg.numAttrs = pdl ? 1 : 0;
        GAIA_CUDA(cudaLaunchKernelEx(&cfg, dev::k_contact_color<ST, R>, ptrs(), c_, beg, end, rc.list, rc.nlist));
    }

    // ---- kernels ----------------------------------------------------------------
    // Launch of one color's solve. pdl: launched as a programmatic dependent of
    // the previous kernel in the stream (its static-data prologue overlaps that
    // kernel's tail; k_solve waits on griddepcontrol before reading positions).
    template <bool PROBE, int L>
    void launch_solve_l(int grid, int B, int beg, int end, int friction, double* probe, bool pdl, int pf = 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(B);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = pdl ? attr : nullptr;
        cfg.numAttrs = pdl ? 1 : 0;
        GAIA_CUDA(cudaLaunchKernelEx(&cfg, dev::k_solve<L, ST, R, PROBE>, ptrs(), c_, beg, end, friction, probe, pf));
    }

    // Largest record count of any block of vpb consecutive vertices in [beg, end).
    int max_records(int beg, int end, int vpb) {
        auto key = std::make_pair(beg, vpb);
        auto it = maxrec_cache_.find(key);
        if (it != maxrec_cache_.end()) return it->second;
        int m = 0;
        for (int v0 = beg; v0 < end; v0 += vpb) m = std::max(m, inc_ofs_[std::min(end, v0 + vpb)] - inc_ofs_[v0]);
        maxrec_cache_[key] = m;
        return m;
    }

    template <int L>
    bool launch_solve_tma_l(int B, int beg, int end, int friction, bool pdl) {
        if constexpr (sizeof(R) != 4) {
            return false;
        } else {
            const int vpb = B / L;
            const int mr = max_records(beg, end, vpb);
            const size_t smem = 16 + 48 * size_t(mr);
            if (smem > kTmaSmemMax) return false;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(div_up(end - beg, vpb));
            cfg.blockDim = dim3(B);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st_;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = pdl ? attr : nullptr;
            cfg.numAttrs = pdl ? 1 : 0;
            GAIA_CUDA(cudaLaunchKernelEx(&cfg, dev::k_solve_tma<L, ST>, ptrs(), c_, beg, end, friction, mr));
            return true;
        }
    }

    // Double-buffered TMA pipeline on a persistent grid (FP32 compute, both tile buffers fit).
    template <int L>
    bool launch_solve_pipe_l(int B, int beg, int end, int friction, bool pdl) {
        if constexpr (sizeof(R) != 4) {
            return false;
        } else {
            const int vpt = B / L;
            const int mr = max_records(beg, end, vpt);
            const size_t smem = 16 + 2 * 48 * size_t(mr);
            if (smem > kTmaSmemMax) return false;
            auto kern = dev::k_solve_pipe<L, ST>;
            const auto key = std::make_pair(L * 100000 + B, int(smem));
            int per_sm = 0;
            auto it = pipe_occ_.find(key);
            if (it != pipe_occ_.end()) {
                per_sm = it->second;
            } else {
                GAIA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, B, smem));
                pipe_occ_[key] = per_sm;
            }
            if (per_sm < 1) return false;
            int dev = 0, sms = 0;
            GAIA_CUDA(cudaGetDevice(&dev));
            GAIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            const int ntiles = div_up(end - beg, vpt);
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(unsigned(std::min(ntiles, per_sm * sms)));
            cfg.blockDim = dim3(B);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st_;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = pdl ? attr : nullptr;
            cfg.numAttrs = pdl ? 1 : 0;
            GAIA_CUDA(cudaLaunchKernelEx(&cfg, kern, ptrs(), c_, beg, end, friction, mr));
            return true;
        }
    }

    bool launch_solve_pipe(int L, int B, int beg, int end, int friction, bool pdl) {
        switch (L) {
            case 2: return launch_solve_pipe_l<2>(B, beg, end, friction, pdl);
            case 4: return launch_solve_pipe_l<4>(B, beg, end, friction, pdl);
            case 8: return launch_solve_pipe_l<8>(B, beg, end, friction, pdl);
            case 16: return launch_solve_pipe_l<16>(B, beg, end, friction, pdl);
            default: return launch_solve_pipe_l<32>(B, beg, end, friction, pdl);
        }
    }

    // TMA-staged launch if this engine computes in FP32 and the block's records fit.
    bool launch_solve_tma(int L, int B, int beg, int end, int friction, bool pdl) {
        switch (L) {
            case 2: return launch_solve_tma_l<2>(B, beg, end, friction, pdl);
            case 4: return launch_solve_tma_l<4>(B, beg, end, friction, pdl);
            case 8: return launch_solve_tma_l<8>(B, beg, end, friction, pdl);
            case 16: return launch_solve_tma_l<16>(B, beg, end, friction, pdl);
            default: return launch_solve_tma_l<32>(B, beg, end, friction, pdl);
        }
    }

    void set_tma_smem_limits() {
        if constexpr (sizeof(R) == 4) {
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_tma<2, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_tma<4, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_tma<8, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_tma<16, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_tma<32, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_pipe<2, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_pipe<4, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_pipe<8, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_pipe<16, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
            GAIA_CUDA(cudaFuncSetAttribute(dev::k_solve_pipe<32, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaSmemMax)));
        }
    }

    template <int L>
    void launch_solve_deep_l(int grid, int B, int beg, int end, int friction, bool pdl) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(B);
        cfg.stream = st_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = pdl ? attr : nullptr;
        cfg.numAttrs = pdl ? 1 : 0;
        GAIA_CUDA(cudaLaunchKernelEx(&cfg, dev::k_solve_deep<L, ST, R>, ptrs(), c_, beg, end, friction));
    }

    template <bool PROBE>
    void launch_solve(int L, int B, int beg, int end, int friction, double* probe, bool pdl = false,
                      int variant = 0) {
        if (end <= beg) return;
        if (!PROBE && variant == 1 && launch_solve_tma(L, B, beg, end, friction, pdl)) return;
        if (!PROBE && variant == kVariantPipe && launch_solve_pipe(L, B, beg, end, friction, pdl)) return;
        if (!PROBE && variant == kVariantDeep) {
            const int grid = div_up(int64_t(end - beg) * L, B);
            switch (L) {
                case 2: launch_solve_deep_l<2>(grid, B, beg, end, friction, pdl); break;
                case 4: launch_solve_deep_l<4>(grid, B, beg, end, friction, pdl); break;
                case 8: launch_solve_deep_l<8>(grid, B, beg, end, friction, pdl); break;
                case 16: launch_solve_deep_l<16>(grid, B, beg, end, friction, pdl); break;
                default: launch_solve_deep_l<32>(grid, B, beg, end, friction, pdl); break;
            }
            return;
        }
        int grid = div_up(int64_t(end - beg) * L, B);
        const bool pf = !PROBE && variant == kVariantPrefetch;
        switch (L) {
            case 2: launch_solve_l<PROBE, 2>(grid, B, beg, end, friction, probe, pdl, pf ? wave_blocks<2>(B) : 0); break;
            case 4: launch_solve_l<PROBE, 4>(grid, B, beg, end, friction, probe, pdl, pf ? wave_blocks<4>(B) : 0); break;
            case 8: launch_solve_l<PROBE, 8>(grid, B, beg, end, friction, probe, pdl, pf ? wave_blocks<8>(B) : 0); break;
            case 16:
                launch_solve_l<PROBE, 16>(grid, B, beg, end, friction, probe, pdl, pf ? wave_blocks<16>(B) : 0);
                break;
            default:
                launch_solve_l<PROBE, 32>(grid, B, beg, end, friction, probe, pdl, pf ? wave_blocks<32>(B) : 0);
                break;
        }
    }

    // Blocks of k_solve<L> resident on the whole device at once (one wave): the distance at
    // which the prefetching variant fetches records ahead.
    template <int L>
    int wave_blocks(int B) {
        const auto key = std::make_pair(L, B);
        auto it = wave_cache_.find(key);
        if (it != wave_cache_.end()) return it->second;
        int per_sm = 0, dev = 0, sms = 0;
        GAIA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::k_solve<L, ST, R, false>, B, 0));
        GAIA_CUDA(cudaGetDevice(&dev));
        GAIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int w = std::max(1, per_sm * sms);
        wave_cache_[key] = w;
        return w;
    }

    // Launch configuration of every merged color. Colors differ in size and in
    // vertex degree (on a 5-tet lattice the largest color holds the vertices with
    // 8 incident tets, the next ones those with 32), so the autotuner picks lanes
    // per vertex, block size and kernel variant per color.
    struct ColorCfg {
        int L = 4, B = 128, variant = 0;
        float ms = 0.f;
    };

    // One configuration for all colors; small colors, which cannot fill the GPU,
    // use one warp per vertex (one incidence per lane, the shortest load chain).
    void uniform_cfg(int L, int B, int variant) {
        ccfg_.assign(group_beg_.size(), ColorCfg{});
        for (size_t g = 0; g < group_beg_.size(); ++g) {
            const int n = group_end_[g] - group_beg_[g];
            ccfg_[g] = ColorCfg{n <= small_color_ ? 32 : L, B, variant, 0.f};
        }
    }

    void enqueue_init(bool rebuild) {
        auto P = ptrs();
        if (frames_) {
            dev::k_frame_update<ST><<<div_up(nmesh_, 128), 128, 0, st_>>>(d_pos_.p, d_frame_ref_.p, d_frame_F_.p,
                                                                         d_frame_shift_.p, nmesh_);
            GAIA_CUDA(cudaGetLastError());
        }
        dev::k_initial_step<ST, R><<<div_up(nslots_, 256), 256, 0, st_>>>(P, c_);
        GAIA_CUDA(cudaGetLastError());
        // contacts: DCD on the start-of-substep positions, CCD on the trajectories to the
        // initial guess, before the deformers move their vertices (VBDPhysics.cpp:846-859)
        enqueue_detection(false, rebuild);
        if (!h_def_slot_.empty()) {
            dev::DeformVerts D;
            D.slot = d_def_slot_.p;
            D.def = d_def_idx_.p;
            D.a = d_def_a_.p;
            D.b = d_def_b_.p;
            D.defs = d_defs_.p;
            D.n = int32_t(h_def_slot_.size());
            dev::k_deformers<ST><<<div_up(D.n, 256), 256, 0, st_>>>(d_pos_.p, d_rest_.p, D, d_time_.p, sc_.p.dt);
            GAIA_CUDA(cudaGetLastError());
        }
        if (sc_.p.useAccelerator)
            GAIA_CUDA(cudaMemcpyAsync(d_acc_pp_.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
    }

    // One iteration's color sweep: VBDPhysics.cpp:879-953 (graph of per-color kernels).
    void enqueue_iteration(int it, double* omega, bool accel) {
        int friction = it >= sc_.p.frictionStartIter ? 1 : 0;
        // intermediateCollisionDetection (VBDPhysics.cpp:878-884)
        const int ici = sc_.p.intermediateCollisionIterations;
        if (ici > 0 && it % ici == 0 && it) enqueue_detection(true, false);
        if (accel) {
            // getAcceleratorOmega (VBDPhysics.cpp:3558-3574)
            double rho = sc_.p.acceleratorRho;
            int order = it + 1;
            *omega = order == 1 ? 1.0 : (order == 2 ? 2.0 / (2.0 - rho * rho) : 4.0 / (4.0 - rho * rho * *omega));
            GAIA_CUDA(cudaMemcpyAsync(d_acc_prev_.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        }
        // programmatic launch only directly after another solve kernel in the stream
        // (k_contact_color and k_solve read no dynamic data before griddepcontrol.wait)
        bool after_solve = it > 0 && !accel;
        const bool contacts = cd_.enabled();
        for (size_t g = 0; g < group_beg_.size(); ++g) {
            const int n = group_end_[g] - group_beg_[g];
            if (n <= 0) continue;
            const ColorCfg& cc = ccfg_[g];
            if (contacts) {
                launch_contact_color(group_beg_[g], group_end_[g], use_pdl_ && after_solve);
                after_solve = true;
            }
            launch_solve<false>(cc.L, cc.B, group_beg_[g], group_end_[g], friction, nullptr,
                                use_pdl_ && after_solve, cc.variant);
            after_solve = true;
        }
        if (accel) {
            dev::k_accel_apply<ST><<<div_up(nactive_, 256), 256, 0, st_>>>(d_pos_.p, d_acc_pp_.p, d_acc_prev_.p, nactive_,
                                                                          *omega, cd_.records().info);
            GAIA_CUDA(cudaGetLastError());
        }
        // evaluateConvergence (VBDPhysics.cpp:948-951): a record after iterations 0, n, 2n, ...
        if (sc_.p.evaluateConvergence && it % sc_.p.evaluationSteps == 0) enqueue_conv(true);
    }

    void enqueue_velocity() {
        dev::k_velocity<ST, R><<<div_up(nslots_, 256), 256, 0, st_>>>(ptrs(), c_, d_time_.p);
        GAIA_CUDA(cudaGetLastError());
    }

    // ---- graphs -----------------------------------------------------------------
    void destroy_graphs() {
        for (auto* g : {&g_init_, &g_init_rb_, &g_sweep_, &g_vel_, &g_step_, &g_step_rb_})
            if (*g) {
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
    }

    template <typename Fn>
    cudaGraphExec_t capture_one(Fn&& fn, int64_t* kernels = nullptr) {
        cudaGraph_t graph = nullptr;
        GAIA_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        try {
            fn();
        } catch (...) {
            cudaStreamEndCapture(st_, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        GAIA_CUDA(cudaStreamEndCapture(st_, &graph));
        if (kernels) {
            // kernel nodes of the captured work: the launches one replay makes
            size_t n = 0;
            GAIA_CUDA(cudaGraphGetNodes(graph, nullptr, &n));
            std::vector<cudaGraphNode_t> nodes(n);
            if (n) GAIA_CUDA(cudaGraphGetNodes(graph, nodes.data(), &n));
            int64_t k = 0;
            for (auto nd : nodes) {
                cudaGraphNodeType t;
                GAIA_CUDA(cudaGraphNodeGetType(nd, &t));
                k += t == cudaGraphNodeTypeKernel ? 1 : 0;
            }
            *kernels = k;
        }
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        GAIA_CUDA(e);
        return exec;
    }

    void capture() {
        destroy_graphs();
        int64_t k_init = 0, k_init_rb = 0, k_sweep = 0, k_vel = 0;
        g_init_ = capture_one([&] { enqueue_init(false); }, &k_init);
        g_init_rb_ = cd_.enabled() ? capture_one([&] { enqueue_init(true); }, &k_init_rb) : nullptr;
        g_sweep_ = capture_one([&] { enqueue_sweep(); }, &k_sweep);
        g_vel_ = capture_one([&] { enqueue_velocity(); }, &k_vel);
        // the whole substep as one graph (no gaps between the three): for untimed steps and
        // for timed steps whose sweep time is measured apart
        g_step_ = capture_one([&] {
            enqueue_init(false);
            enqueue_sweep();
            enqueue_velocity();
        });
        g_step_rb_ = cd_.enabled() ? capture_one([&] {
            enqueue_init(true);
            enqueue_sweep();
            enqueue_velocity();
        })
                                   : nullptr;
        const int64_t nsub = sc_.p.numSubsteps;
        launches_per_step_ = nsub * (k_init + k_sweep + k_vel) + (g_init_rb_ ? k_init_rb - k_init : 0);
        launches_per_substep_ = (launches_per_step_ + nsub - 1) / nsub;
    }

    // One substep's iterations (the sweep graph's content).
    void enqueue_sweep() {
        if (mode_ == kSweepScenes) {
            enqueue_scenes_sweep(scene_L_, scene_B_);
            return;
        }
        if (mode_ == kSweepCluster) {
            enqueue_cluster_sweep(scene_C_, scene_L_, scene_B_);
            return;
        }
        if (mode_ == kSweepGrid) {
            enqueue_grid_sweep(scene_L_, scene_B_);
            return;
        }
        // evaluateConvergence at iteration -1, on the initial guess (VBDPhysics.cpp:866-870)
        if (sc_.p.evaluateConvergence) enqueue_conv(true);
        double omega = 1.0;
        for (int it = 0; it < sc_.p.iterations; ++it) enqueue_iteration(it, &omega, sc_.p.useAccelerator);
    }

    // The face hierarchy of the contact detector is rebuilt at the first substep of a
    // step and refitted in the others.
    cudaGraphExec_t init_graph(int sub) const { return sub == 0 && g_init_rb_ ? g_init_rb_ : g_init_; }
    cudaGraphExec_t step_graph(int sub) const { return sub == 0 && g_step_rb_ ? g_step_rb_ : g_step_; }

    // The convergence log holds the records of the last step.
    void start_step_log() {
        if (sc_.p.evaluateConvergence) GAIA_CUDA(cudaMemsetAsync(d_conv_count_.p, 0, sizeof(int32_t), st_));
    }

    void run_steps(int n) override {
        for (int k = 0; k < n; ++k)
            for (int sub = 0; sub < sc_.p.numSubsteps; ++sub) {
                if (sub == 0) start_step_log();
                GAIA_CUDA(cudaGraphLaunch(step_graph(sub), st_));
            }
    }

    // Device time of n steps. Without sweep_ms the steps run as run_steps runs them (one
    // graph per substep) and are timed as a whole; with it the substep's initial step, sweep
    // and velocity update run as three graphs with events around every sweep, so that the
    // solve kernels are timed apart.
    void run_steps_timed(int n, float* total_ms, float* sweep_ms) override {
        if (!sweep_ms) {
            GAIA_CUDA(cudaEventRecord(ev_a_, st_));
            run_steps(n);
            GAIA_CUDA(cudaEventRecord(ev_b_, st_));
            GAIA_CUDA(cudaEventSynchronize(ev_b_));
            float tot = 0.f;
            GAIA_CUDA(cudaEventElapsedTime(&tot, ev_a_, ev_b_));
            if (total_ms) *total_ms = tot;
            return;
        }
        // per-substep sweep events: [start, end] pairs recorded around the sweep graph
        int nsub = n * sc_.p.numSubsteps;
        std::vector<cudaEvent_t> ev(2 * size_t(nsub));
        for (auto& e : ev) GAIA_CUDA(cudaEventCreate(&e));
        GAIA_CUDA(cudaEventRecord(ev_a_, st_));
        int q = 0;
        for (int k = 0; k < n; ++k)
            for (int sub = 0; sub < sc_.p.numSubsteps; ++sub, ++q) {
                if (sub == 0) start_step_log();
                GAIA_CUDA(cudaGraphLaunch(init_graph(sub), st_));
                GAIA_CUDA(cudaEventRecord(ev[2 * q], st_));
                GAIA_CUDA(cudaGraphLaunch(g_sweep_, st_));
                GAIA_CUDA(cudaEventRecord(ev[2 * q + 1], st_));
                GAIA_CUDA(cudaGraphLaunch(g_vel_, st_));
            }
        GAIA_CUDA(cudaEventRecord(ev_b_, st_));
        GAIA_CUDA(cudaEventSynchronize(ev_b_));
        float tot = 0.f, sw = 0.f;
        GAIA_CUDA(cudaEventElapsedTime(&tot, ev_a_, ev_b_));
        for (int i = 0; i < nsub; ++i) {
            float t = 0.f;
            GAIA_CUDA(cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]));
            sw += t;
        }
        for (auto& e : ev) cudaEventDestroy(e);
        if (total_ms) *total_ms = tot;
        if (sweep_ms) *sweep_ms = sw;
    }

    // Autotuner: per merged color, every (kernel variant, lanes per vertex, block
    // size) is timed on that color's kernel alone (CUDA events around repeated
    // launches on the current state, positions restored afterwards) and the
    // fastest is kept. Fixed lanesPerVertex / blockSize / solveVariant
    // parameters restrict the search.
    void autotune_impl() {
        if (nactive_ == 0) return;
        DevBuf<S4> save;
        save.alloc(nslots_, nullptr);
        GAIA_CUDA(cudaMemcpyAsync(save.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        const int Ls[] = {2, 4, 8, 16, 32};
        // blocks of 64 too for the tile pipeline, whose two tile buffers bound the blocks per SM
        const std::vector<int> Bs = {128, 256}, Bs_pipe = {64, 128, 256};
        // kernel variants: 0 register-pipelined, 1 TMA-staged (FP32 compute only), 4 deeper
        // register pipeline, 6 register-pipelined with the records of the block one resident
        // wave ahead bulk-prefetched into L2 (FP32 compute only), 7 double-buffered TMA tiles
        // on a persistent grid (FP32 compute only)
        std::vector<int> variants = {0, kVariantDeep};
        if (sizeof(R) == 4) {
            variants.push_back(1);
            variants.push_back(kVariantPrefetch);
            variants.push_back(kVariantPipe);
        }
        const int reps = 4;
        ccfg_.assign(group_beg_.size(), ColorCfg{});
        double total = 0.0;
        for (size_t g = 0; g < group_beg_.size(); ++g) {
            const int beg = group_beg_[g], end = group_end_[g];
            if (end <= beg) continue;
            ColorCfg best;
            best.ms = 1e30f;
            for (int var : variants) {
                if (variant_fixed_ >= 0 && var != variant_fixed_) continue;
                for (int L : Ls) {
                    if (lanes_ && L != lanes_) continue;
                    for (int B : var == kVariantPipe ? Bs_pipe : Bs) {
                        if (block_ && B != block_) continue;
                        launch_solve<false>(L, B, beg, end, 1, nullptr, false, var);  // warm-up
                        GAIA_CUDA(cudaEventRecord(ev_a_, st_));
                        for (int r = 0; r < reps; ++r) launch_solve<false>(L, B, beg, end, 1, nullptr, false, var);
                        GAIA_CUDA(cudaEventRecord(ev_b_, st_));
                        GAIA_CUDA(cudaEventSynchronize(ev_b_));
                        float ms = 0.f;
                        GAIA_CUDA(cudaEventElapsedTime(&ms, ev_a_, ev_b_));
                        ms /= reps;
                        if (ms < best.ms) best = ColorCfg{L, B, var, ms};
                    }
                }
            }
            ccfg_[g] = best;
            total += best.ms;
            GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        }
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p, 0, dev::CNT_N * sizeof(unsigned long long), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        tuned_ms_ = total;
        tuned_ = true;
    }

    // After construction or a re-tune: per-color configurations in place, and the
    // configuration of the largest color reported as the engine's.
    void finalize_cfg() {
        if (!tuned_) uniform_cfg(lanes_ ? lanes_ : 4, block_ ? block_ : 128, variant_);
        size_t big = 0;
        for (size_t g = 0; g < group_beg_.size(); ++g)
            if (group_end_[g] - group_beg_[g] > group_end_[big] - group_beg_[big]) big = g;
        if (!ccfg_.empty()) {
            lanes_ = ccfg_[big].L;
            block_ = ccfg_[big].B;
            variant_ = ccfg_[big].variant;
        }
    }

    // ---- persistent scene-major sweep (k_sweep_scenes) ------------------------------
    void setup_scenes() {
        std::vector<int64_t> work(size_t(nmesh_), 0);
        for (int m = 0; m < nmesh_; ++m)
            for (int32_t ci = scene_ofs_[m]; ci < scene_ofs_[m + 1]; ++ci)
                work[size_t(m)] += inc_ofs_[scene_colors_[ci].y] - inc_ofs_[scene_colors_[ci].x];
        std::vector<int32_t> order;
        for (int m = 0; m < nmesh_; ++m)
            if (scene_ofs_[m + 1] > scene_ofs_[m]) order.push_back(m);
        // largest scene first: the work counter hands them out in this order
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[size_t(a)] > work[size_t(b)]; });
        nscenes_ = int32_t(order.size());
        d_scene_colors_.upload(scene_colors_, &bytes_, st_);
        d_scene_ofs_.upload(scene_ofs_, &bytes_, st_);
        d_scene_order_.upload(order, &bytes_, st_);
        d_scene_work_.alloc(1, &bytes_);
        GAIA_CUDA(cudaMemsetAsync(d_scene_work_.p, 0, sizeof(int32_t), st_));
        int dev = 0;
        GAIA_CUDA(cudaGetDevice(&dev));
        GAIA_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    template <int L, int MAXB>
    void launch_scenes_lb(int B) {
        auto kern = dev::k_sweep_scenes<L, ST, R, MAXB>;
        int per_sm = 0;
        GAIA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, B, 0));
        const int grid = std::max(1, std::min(nscenes_, std::max(per_sm, 1) * num_sms_));
        kern<<<grid, B, 0, st_>>>(ptrs(), c_, d_scene_colors_.p, d_scene_ofs_.p, d_scene_order_.p, nscenes_,
                                  sc_.p.iterations, sc_.p.frictionStartIter, d_scene_work_.p);
        GAIA_CUDA(cudaGetLastError());
    }

    template <int L>
    void launch_scenes_l(int B) {
        if (B <= 256) launch_scenes_lb<L, 256>(B);
        else launch_scenes_lb<L, 1024>(B);
    }

    // One substep's iterations: reset the work counter, one persistent launch.
    void enqueue_scenes_sweep(int L, int B) {
        if (nscenes_ == 0 || sc_.p.iterations == 0) return;
        GAIA_CUDA(cudaMemsetAsync(d_scene_work_.p, 0, sizeof(int32_t), st_));
        switch (L) {
            case 2: launch_scenes_l<2>(B); break;
            case 4: launch_scenes_l<4>(B); break;
            case 8: launch_scenes_l<8>(B); break;
            case 16: launch_scenes_l<16>(B); break;
            default: launch_scenes_l<32>(B); break;
        }
    }

    // Lanes per vertex and block size of the persistent sweep: every pair timed on a full
    // sweep of the current state (restored afterwards); ms per iteration of the fastest.
    void autotune_scenes() {
        if (nactive_ == 0 || nscenes_ == 0 || sc_.p.iterations == 0) return;
        DevBuf<S4> save;
        save.alloc(nslots_, nullptr);
        GAIA_CUDA(cudaMemcpyAsync(save.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        const int Ls[] = {4, 8, 16, 32};
        const int Bs[] = {256, 512, 1024};
        float best = 1e30f;
        for (int L : Ls) {
            if (lanes_ && L != lanes_) continue;
            for (int B : Bs) {
                if (block_ && B != block_) continue;
                enqueue_scenes_sweep(L, B);  // warm-up
                GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
                GAIA_CUDA(cudaEventRecord(ev_a_, st_));
                enqueue_scenes_sweep(L, B);
                GAIA_CUDA(cudaEventRecord(ev_b_, st_));
                GAIA_CUDA(cudaEventSynchronize(ev_b_));
                float ms = 0.f;
                GAIA_CUDA(cudaEventElapsedTime(&ms, ev_a_, ev_b_));
                GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
                if (ms < best) {
                    best = ms;
                    scene_L_ = L;
                    scene_B_ = B;
                }
            }
        }
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p, 0, dev::CNT_N * sizeof(unsigned long long), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        tuned_ms_ = double(best) / sc_.p.iterations;
        tuned_ = true;
    }

    // ---- cluster sweep (vbd_cluster.cuh) ---------------------------------------------
    // Per scene: its active and fixed slot ranges, and how many states and records one
    // block of a C-block cluster holds; the cluster sizes whose largest block fits.
    void setup_cluster() {
        std::vector<int4> slots(size_t(nmesh_), make_int4(0, 0, 0, 0));
        int64_t f0 = nactive_;
        for (int m = 0; m < nmesh_; ++m) {
            int32_t a0 = 0, a1 = 0;
            if (scene_ofs_[m + 1] > scene_ofs_[m]) {
                a0 = scene_colors_[scene_ofs_[m]].x;
                a1 = scene_colors_[scene_ofs_[m + 1] - 1].y;
            }
            int64_t nf = 0;
            for (int v = 0; v < sc_.meshes[m].nv; ++v) nf += sc_.meshes[m].fixed[v] ? 1 : 0;
            slots[size_t(m)] = make_int4(a0, a1, int32_t(f0), int32_t(f0 + nf));
            f0 += nf;
        }
        int dev = 0;
        GAIA_CUDA(cudaGetDevice(&dev));
        int smem_optin = 0;
        GAIA_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const size_t budget = size_t(std::max(0, smem_optin - 4096));  // static shared memory and slack
        cluster_fits_.clear();
        for (int C : {2, 4, 8, 16}) {
            int64_t pos_cap = 0, rec_cap = 0;
            bool ok = true;
            for (int m = 0; m < nmesh_ && ok; ++m) {
                const int4 sl = slots[size_t(m)];
                pos_cap = std::max<int64_t>(pos_cap, int64_t(sl.y - sl.x) + (sl.w - sl.z));
                if (scene_ofs_[m + 1] - scene_ofs_[m] > dev::kClusterMaxColors) ok = false;
                std::vector<int64_t> per_rank(size_t(C), 0);
                for (int32_t ci = scene_ofs_[m]; ci < scene_ofs_[m + 1]; ++ci) {
                    const int2 rg = scene_colors_[ci];
                    const int per = (rg.y - rg.x + C - 1) / C;
                    for (int r = 0; r < C; ++r) {
                        const int beg = std::min(rg.y, rg.x + r * per), end = std::min(rg.y, beg + per);
                        per_rank[size_t(r)] += inc_ofs_[end] - inc_ofs_[beg];
                    }
                }
                for (int64_t x : per_rank) rec_cap = std::max(rec_cap, x);
            }
            const size_t bytes = sizeof(S4) * size_t(pos_cap) + sizeof(dev::RecS<R>) * size_t(rec_cap);
            if (ok && bytes <= budget) cluster_fits_.push_back({C, int32_t(pos_cap), int32_t(rec_cap), bytes});
        }
        if (cluster_fits_.empty())
            throw std::runtime_error("sweepMode \"cluster\" is not supported: a scene does not fit in the shared "
                                     "memory of a 16-block cluster");
        if (sc_.p.clusterSize && !cluster_fit(sc_.p.clusterSize))
            throw std::runtime_error("sweepMode \"cluster\" is not supported with clusterSize " +
                                     std::to_string(sc_.p.clusterSize) + ": a scene does not fit in the shared "
                                     "memory of a cluster of that many blocks");
        d_scene_slots_.upload(slots, &bytes_, st_);
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    const ClusterFit* cluster_fit(int C) const {
        for (auto& f : cluster_fits_)
            if (f.C == C) return &f;
        return nullptr;
    }

    template <int L>
    void launch_cluster_l(const ClusterFit& f, int B) {
        auto kern = dev::k_sweep_cluster<L, ST, R>;
        GAIA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(f.bytes)));
        if (f.C > 8) GAIA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = unsigned(f.C);
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.blockDim = dim3(unsigned(B));
        cfg.dynamicSmemBytes = f.bytes;
        cfg.stream = st_;
        cfg.gridDim = dim3(unsigned(f.C));
        int nclusters = 0;
        GAIA_CUDA(cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg));
        if (nclusters < 1) throw std::runtime_error("no cluster of this size fits on the device");
        cfg.gridDim = dim3(unsigned(f.C * std::min(nscenes_, nclusters)));
        dev::ClusterScenes S;
        S.colors = d_scene_colors_.p;
        S.scene_ofs = d_scene_ofs_.p;
        S.scene_order = d_scene_order_.p;
        S.scene_slots = d_scene_slots_.p;
        S.nscenes = nscenes_;
        S.iterations = sc_.p.iterations;
        S.friction_start = sc_.p.frictionStartIter;
        S.pos_cap = f.pos_cap;
        S.rec_cap = f.rec_cap;
        GAIA_CUDA(cudaLaunchKernelEx(&cfg, kern, ptrs(), c_, S, d_scene_work_.p));
    }

    void enqueue_cluster_sweep(int C, int L, int B) {
        if (nscenes_ == 0 || sc_.p.iterations == 0) return;
        const ClusterFit* f = cluster_fit(C);
        if (!f) throw std::runtime_error("clusterSize: scenes do not fit a cluster of " + std::to_string(C) + " blocks");
        GAIA_CUDA(cudaMemsetAsync(d_scene_work_.p, 0, sizeof(int32_t), st_));
        switch (L) {
            case 4: launch_cluster_l<4>(*f, B); break;
            case 8: launch_cluster_l<8>(*f, B); break;
            case 16: launch_cluster_l<16>(*f, B); break;
            default: launch_cluster_l<32>(*f, B); break;
        }
    }

    // Cluster size, lanes per vertex and block size of the cluster sweep, each combination
    // timed on a full sweep of the current state (restored afterwards).
    void autotune_cluster() {
        if (nactive_ == 0 || nscenes_ == 0 || sc_.p.iterations == 0) return;
        DevBuf<S4> save;
        save.alloc(nslots_, nullptr);
        GAIA_CUDA(cudaMemcpyAsync(save.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        float best = 1e30f;
        for (const ClusterFit& f : cluster_fits_) {
            if (sc_.p.clusterSize && f.C != sc_.p.clusterSize) continue;
            for (int L : {4, 8, 16, 32}) {
                if (lanes_ && L != lanes_) continue;
                for (int B : {128, 256}) {
                    if (block_ && B != block_) continue;
                    enqueue_cluster_sweep(f.C, L, B);  // warm-up
                    GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
                    GAIA_CUDA(cudaEventRecord(ev_a_, st_));
                    enqueue_cluster_sweep(f.C, L, B);
                    GAIA_CUDA(cudaEventRecord(ev_b_, st_));
                    GAIA_CUDA(cudaEventSynchronize(ev_b_));
                    float ms = 0.f;
                    GAIA_CUDA(cudaEventElapsedTime(&ms, ev_a_, ev_b_));
                    GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
                    if (ms < best) {
                        best = ms;
                        scene_C_ = f.C;
                        scene_L_ = L;
                        scene_B_ = B;
                    }
                }
            }
        }
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p, 0, dev::CNT_N * sizeof(unsigned long long), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        if (!(best < 1e30f)) throw std::runtime_error("cluster sweep: no configuration was timed");
        tuned_ms_ = double(best) / sc_.p.iterations;
        tuned_ = true;
    }

    void finalize_cluster() {
        if (!tuned_) {
            scene_C_ = sc_.p.clusterSize ? sc_.p.clusterSize : cluster_fits_.back().C;
            scene_L_ = lanes_ ? lanes_ : 8;
            scene_B_ = block_ ? block_ : 128;
        }
        if (!cluster_fit(scene_C_))
            throw std::runtime_error("clusterSize: scenes do not fit a cluster of " + std::to_string(scene_C_) + " blocks");
        lanes_ = scene_L_;
        block_ = scene_B_;
        variant_ = 3;
        ccfg_.assign(sc_.groups.size(), ColorCfg{scene_L_, scene_B_, 3, float(tuned_ms_)});
    }

    // ---- grid sweep (vbd_grid.cuh) -----------------------------------------------------
    void setup_grid() {
        std::vector<int2> colors;
        for (size_t g = 0; g < group_beg_.size(); ++g)
            if (group_end_[g] > group_beg_[g]) colors.push_back(make_int2(group_beg_[g], group_end_[g]));
        grid_ncolors_ = int32_t(colors.size());
        grid_max_color_ = 0;
        for (const int2& c : colors) grid_max_color_ = std::max(grid_max_color_, c.y - c.x);
        d_grid_colors_.upload(colors, &bytes_, st_);
        d_grid_bar_.alloc(2, &bytes_);
        int dev = 0, coop = 0;
        GAIA_CUDA(cudaGetDevice(&dev));
        GAIA_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
        GAIA_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) throw std::runtime_error("sweepMode \"grid\" is not supported: no cooperative launch on this device");
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    // Blocks of the grid sweep: enough for the largest color at one vertex per group, at most
    // as many as are resident at once (the cooperative launch requires it).
    template <int L>
    int grid_blocks(int B) const {
        int per_sm = 0;
        GAIA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::k_sweep_grid<L, ST, R>, B, 0));
        if (per_sm < 1) throw std::runtime_error("grid sweep: no block of this size fits on an SM");
        const int need = std::max(1, int(div_up(int64_t(grid_max_color_) * L, B)));
        return std::min(need, per_sm * num_sms_);
    }

    template <int L>
    void launch_grid_l(int B) {
        dev::GridSweep G;
        G.colors = d_grid_colors_.p;
        G.ncolors = grid_ncolors_;
        G.iterations = sc_.p.iterations;
        G.friction_start = sc_.p.frictionStartIter;
        G.bar = d_grid_bar_.p;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.gridDim = dim3(unsigned(grid_blocks<L>(B)));
        cfg.blockDim = dim3(unsigned(B));
        cfg.stream = st_;
        GAIA_CUDA(cudaLaunchKernelEx(&cfg, dev::k_sweep_grid<L, ST, R>, ptrs(), c_, G));
    }

    // One substep's iterations: the barrier's counter and flag zeroed, one cooperative launch.
    void enqueue_grid_sweep(int L, int B) {
        if (grid_ncolors_ == 0 || sc_.p.iterations == 0) return;
        GAIA_CUDA(cudaMemsetAsync(d_grid_bar_.p, 0, 2 * sizeof(uint32_t), st_));
        switch (L) {
            case 2: launch_grid_l<2>(B); break;
            case 4: launch_grid_l<4>(B); break;
            case 8: launch_grid_l<8>(B); break;
            case 16: launch_grid_l<16>(B); break;
            default: launch_grid_l<32>(B); break;
        }
    }

    // Lanes per vertex and block size of the grid sweep, each pair timed on a full sweep of
    // the current state (restored afterwards).
    void autotune_grid() {
        if (nactive_ == 0 || grid_ncolors_ == 0 || sc_.p.iterations == 0) return;
        DevBuf<S4> save;
        save.alloc(nslots_, nullptr);
        GAIA_CUDA(cudaMemcpyAsync(save.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        float best = 1e30f;
        for (int L : {4, 8, 16, 32}) {
            if (lanes_ && L != lanes_) continue;
            for (int B : {128, 256}) {
                if (block_ && B != block_) continue;
                enqueue_grid_sweep(L, B);  // warm-up
                GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
                GAIA_CUDA(cudaEventRecord(ev_a_, st_));
                enqueue_grid_sweep(L, B);
                GAIA_CUDA(cudaEventRecord(ev_b_, st_));
                GAIA_CUDA(cudaEventSynchronize(ev_b_));
                float ms = 0.f;
                GAIA_CUDA(cudaEventElapsedTime(&ms, ev_a_, ev_b_));
                GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
                if (ms < best) {
                    best = ms;
                    scene_L_ = L;
                    scene_B_ = B;
                }
            }
        }
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p, 0, dev::CNT_N * sizeof(unsigned long long), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        if (!(best < 1e30f)) throw std::runtime_error("grid sweep: no configuration was timed");
        tuned_ms_ = double(best) / sc_.p.iterations;
        tuned_ = true;
    }

    void finalize_grid() {
        if (!tuned_) {
            scene_L_ = lanes_ ? lanes_ : 16;
            scene_B_ = block_ ? block_ : 256;
        }
        lanes_ = scene_L_;
        block_ = scene_B_;
        variant_ = kVariantGrid;
        ccfg_.assign(sc_.groups.size(), ColorCfg{scene_L_, scene_B_, kVariantGrid, float(tuned_ms_)});
    }

    void finalize_scenes() {
        if (!tuned_) {
            scene_L_ = lanes_ ? lanes_ : 8;
            scene_B_ = block_ ? block_ : 512;
        }
        lanes_ = scene_L_;
        block_ = scene_B_;
        variant_ = 2;
        ccfg_.assign(sc_.groups.size(), ColorCfg{scene_L_, scene_B_, 2, float(tuned_ms_)});
    }

    double get_time() override {
        double t = 0.0;
        GAIA_CUDA(cudaMemcpyAsync(&t, d_time_.p, sizeof(double), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        return t;
    }
    void set_time(double t) override {
        GAIA_CUDA(cudaMemcpyAsync(d_time_.p, &t, sizeof(double), cudaMemcpyHostToDevice, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    void reset() override {
        GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, h_pos_.data(), nslots_ * sizeof(S4), cudaMemcpyHostToDevice, st_));
        GAIA_CUDA(cudaMemcpyAsync(d_vel_.p, h_vel_.data(), nslots_ * sizeof(V4), cudaMemcpyHostToDevice, st_));
        GAIA_CUDA(cudaMemcpyAsync(d_y_.p, h_pos_.data(), nslots_ * sizeof(S4), cudaMemcpyHostToDevice, st_));
        GAIA_CUDA(cudaMemcpyAsync(d_xprev_.p, h_pos_.data(), nslots_ * sizeof(S4), cudaMemcpyHostToDevice, st_));
        GAIA_CUDA(cudaMemsetAsync(d_time_.p, 0, sizeof(double), st_));
        // the status counters (non-finite solves, device timeouts) start again from zero
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p + dev::CNT_NONFINITE, 0, 3 * sizeof(unsigned long long), st_));
        cd_.reset(st_);
        GAIA_CUDA(cudaStreamSynchronize(st_));
        reset_frames();
    }

    void autotune() override {
        lanes_ = sc_.p.lanesPerVertex;
        block_ = sc_.p.blockSize;
        tuned_ = false;
        if (mode_ == kSweepScenes) {
            autotune_scenes();
            finalize_scenes();
        } else if (mode_ == kSweepCluster) {
            autotune_cluster();
            finalize_cluster();
        } else if (mode_ == kSweepGrid) {
            autotune_grid();
            finalize_grid();
        } else {
            autotune_impl();
            finalize_cfg();
        }
        capture();
    }

    double tuned_ms() const override { return tuned_ms_; }

    // Device time of the captured sweep graph (all iterations of one substep) on the
    // current state, per iteration; the state is restored afterwards.
    double measure_sweep_ms() override {
        DevBuf<S4> save;
        save.alloc(nslots_, nullptr);
        GAIA_CUDA(cudaMemcpyAsync(save.p, d_pos_.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        GAIA_CUDA(cudaGraphLaunch(g_sweep_, st_));  // warm-up
        const int reps = 3;
        float total = 0.f;
        for (int r = 0; r < reps; ++r) {
            GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
            GAIA_CUDA(cudaEventRecord(ev_a_, st_));
            GAIA_CUDA(cudaGraphLaunch(g_sweep_, st_));
            GAIA_CUDA(cudaEventRecord(ev_b_, st_));
            GAIA_CUDA(cudaEventSynchronize(ev_b_));
            float ms = 0.f;
            GAIA_CUDA(cudaEventElapsedTime(&ms, ev_a_, ev_b_));
            total += ms;
        }
        GAIA_CUDA(cudaMemcpyAsync(d_pos_.p, save.p, nslots_ * sizeof(S4), cudaMemcpyDeviceToDevice, st_));
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p, 0, dev::CNT_N * sizeof(unsigned long long), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        return double(total) / reps / std::max(sc_.p.iterations, 1);
    }

    // ---- state access -------------------------------------------------------------
    // Status of the device work so far: a bounded wait that ran out, then non-finite solves.
    // Each is reported once: the call that throws moves the device counts into the handle's
    // totals (stats) and clears them, so the calls after it see the state as it was left.
    void check_nonfinite() {
        unsigned long long h[dev::CNT_N];
        GAIA_CUDA(cudaMemcpyAsync(h, d_counters_.p, sizeof(h), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        if (!h[dev::CNT_TIMEOUT] && !h[dev::CNT_NONFINITE]) return;
        reported_timeouts_ += int64_t(h[dev::CNT_TIMEOUT]);
        reported_nonfinite_ += int64_t(h[dev::CNT_NONFINITE]);
        GAIA_CUDA(cudaMemsetAsync(d_counters_.p + dev::CNT_NONFINITE, 0, 3 * sizeof(unsigned long long), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        if (h[dev::CNT_TIMEOUT])
            throw DeviceTimeout(std::to_string(h[dev::CNT_TIMEOUT]) +
                                " solve block(s) gave up on a bounded device wait and skipped their vertices" +
                                (h[dev::CNT_DRAIN] ? " (" + std::to_string(h[dev::CNT_DRAIN]) +
                                                         " still had copies in flight)"
                                                   : std::string()));
        if (h[dev::CNT_NONFINITE])
            throw std::domain_error(std::to_string(h[dev::CNT_NONFINITE]) +
                                    " vertex solve(s) met a non-finite force or step (not written)");
    }

    void sync() override {
        GAIA_CUDA(cudaStreamSynchronize(st_));
        check_nonfinite();
    }

    void mesh_range(int mesh, int64_t& off, int64_t& n) {
        if (mesh < 0 || mesh >= nmesh_) throw std::invalid_argument("mesh index out of range");
        off = mesh_off_[mesh];
        n = mesh_off_[mesh + 1] - off;
    }

    void get_positions(int mesh, double* out) override {
        check_nonfinite();
        int64_t off, n;
        mesh_range(mesh, off, n);
        if (n == 0) return;
        dev::k_gather_positions<ST><<<div_up(n, 256), 256, 0, st_>>>(d_pos_.p, d_rest_.p, nullptr, d_stage_f64_.p,
                                                                     d_slot_of_.p + off, int32_t(n), frame_ptr(),
                                                                     d_slot_mesh_.p);
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaMemcpyAsync(out, d_stage_f64_.p, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }
    void get_velocities(int mesh, double* out) override {
        int64_t off, n;
        mesh_range(mesh, off, n);
        if (n == 0) return;
        dev::k_gather_velocities<V4><<<div_up(n, 256), 256, 0, st_>>>(d_vel_.p, nullptr, d_stage_f64_.p,
                                                                      d_slot_of_.p + off, int32_t(n));
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaMemcpyAsync(out, d_stage_f64_.p, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }
    void set_positions(int mesh, const double* in) override {
        int64_t off, n;
        mesh_range(mesh, off, n);
        if (n == 0) return;
        GAIA_CUDA(cudaMemcpyAsync(d_stage_f64_.p, in, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st_));
        dev::k_scatter_positions_f64<ST><<<div_up(n, 256), 256, 0, st_>>>(d_pos_.p, d_rest_.p, d_stage_f64_.p,
                                                                          d_slot_of_.p + off, int32_t(n), frame_ptr(),
                                                                          d_slot_mesh_.p);
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }
    void set_prev_positions(int mesh, const double* in) override {
        int64_t off, n;
        mesh_range(mesh, off, n);
        if (n == 0) return;
        GAIA_CUDA(cudaMemcpyAsync(d_stage_f64_.p, in, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st_));
        dev::k_scatter_positions_f64<ST><<<div_up(n, 256), 256, 0, st_>>>(d_xprev_.p, d_rest_.p, d_stage_f64_.p,
                                                                          d_slot_of_.p + off, int32_t(n), frame_ptr(),
                                                                          d_slot_mesh_.p);
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    // A substep-start detection pass on the current positions (trajectories from the
    // start-of-substep positions); returns the number of vertices with a contact.
    int collide() override {
        if (!cd_.enabled()) return 0;
        enqueue_detection(false, true);
        std::vector<int32_t> rows;
        cd_.contacts(rows, st_);
        return int(rows.size() / 3);
    }

    // Rows of 8: mesh, vertex, face mesh, face vertices (3, mesh-local), surface face
    // (mesh-local), kind (1 = CCD, 2 = DCD), in (mesh, surface vertex) order.
    void contacts(std::vector<int32_t>& out) override {
        out.clear();
        if (!cd_.enabled()) return;
        std::vector<int32_t> rows;
        cd_.contacts(rows, st_);
        std::vector<int32_t> face_ofs(nmesh_ + 1, 0);
        for (int m = 0; m < nmesh_; ++m) face_ofs[m + 1] = face_ofs[m] + int32_t(sc_.meshes[m].sfaces.size() / 3);
        for (size_t r = 0; r + 2 < rows.size(); r += 3) {
            const int32_t gi = orig_of_[rows[r]];
            const int m = int(std::upper_bound(mesh_off_.begin(), mesh_off_.end(), int64_t(gi)) - mesh_off_.begin()) - 1;
            const int32_t g = rows[r + 1];
            const int fm = int(std::upper_bound(face_ofs.begin(), face_ofs.end(), g) - face_ofs.begin()) - 1;
            const int32_t f = g - face_ofs[fm];
            const int32_t* fv = &sc_.meshes[fm].sfaces[3 * size_t(f)];
            const int32_t row[8] = {m, gi - int32_t(mesh_off_[m]), fm, fv[0], fv[1], fv[2], f, rows[r + 2]};
            out.insert(out.end(), row, row + 8);
        }
    }

    void set_velocities(int mesh, const double* in) override {
        int64_t off, n;
        mesh_range(mesh, off, n);
        if (n == 0) return;
        GAIA_CUDA(cudaMemcpyAsync(d_stage_f64_.p, in, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st_));
        dev::k_scatter_velocities_f64<ST><<<div_up(n, 256), 256, 0, st_>>>(d_vel_.p, d_stage_f64_.p,
                                                                           d_slot_of_.p + off, int32_t(n));
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    void set_state_f32(const float* x, const float* v) override {
        float* dx = d_stage_f32_.p;
        float* dv = d_stage_f32_.p + 3 * size_t(nslots_);
        if (x) GAIA_CUDA(cudaMemcpyAsync(dx, x, 3 * nslots_ * sizeof(float), cudaMemcpyHostToDevice, st_));
        if (v) GAIA_CUDA(cudaMemcpyAsync(dv, v, 3 * nslots_ * sizeof(float), cudaMemcpyHostToDevice, st_));
        dev::k_scatter_state<ST><<<div_up(nslots_, 256), 256, 0, st_>>>(d_pos_.p, d_rest_.p, d_vel_.p, x ? dx : nullptr,
                                                                       v ? dv : nullptr, d_slot_of_.p,
                                                                       int32_t(nslots_), frame_ptr(), d_slot_mesh_.p);
        GAIA_CUDA(cudaGetLastError());
    }

    void get_positions_f32(float* x) override {
        dev::k_gather_positions<ST><<<div_up(nslots_, 256), 256, 0, st_>>>(d_pos_.p, d_rest_.p, d_stage_f32_.p,
                                                                          nullptr, d_slot_of_.p, int32_t(nslots_),
                                                                          frame_ptr(), d_slot_mesh_.p);
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaMemcpyAsync(x, d_stage_f32_.p, 3 * nslots_ * sizeof(float), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        check_nonfinite();
    }
    void get_velocities_f32(float* v) override {
        dev::k_gather_velocities<V4><<<div_up(nslots_, 256), 256, 0, st_>>>(d_vel_.p, d_stage_f32_.p, nullptr,
                                                                            d_slot_of_.p, int32_t(nslots_));
        GAIA_CUDA(cudaGetLastError());
        GAIA_CUDA(cudaMemcpyAsync(v, d_stage_f32_.p, 3 * nslots_ * sizeof(float), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    // ---- FP64 convergence reduction (vbd_convergence.cuh) -----------------------------
    // Per-tet FP64 data (global tet order: meshes in order, tets in order), each active
    // slot's incidences as (tet, order) in the solve's CSR, partial-sum buffers and the
    // record log; built on first use, or at construction when the step logs records.
    void setup_conv() {
        if (conv_ready_) return;
        std::vector<int4> ts;
        std::vector<double> dm, vol;
        std::vector<int32_t> tm, tet_off(nmesh_ + 1, 0);
        for (int m = 0; m < nmesh_; ++m) {
            const TetMesh& M = sc_.meshes[m];
            tet_off[m + 1] = tet_off[m] + M.ntet;
            for (int t = 0; t < M.ntet; ++t) {
                const int32_t* tv = &M.tets[4 * size_t(t)];
                ts.push_back(make_int4(slot_of_[mesh_off_[m] + tv[0]], slot_of_[mesh_off_[m] + tv[1]],
                                       slot_of_[mesh_off_[m] + tv[2]], slot_of_[mesh_off_[m] + tv[3]]));
                dm.insert(dm.end(), M.dminv.begin() + 9 * size_t(t), M.dminv.begin() + 9 * size_t(t) + 9);
                vol.push_back(M.vol[t]);
                tm.push_back(m);
            }
        }
        // incidences in slot order, as the solve's records are stored
        std::vector<int32_t> inc_tet;
        std::vector<int8_t> inc_ord;
        inc_tet.reserve(size_t(ninc_));
        inc_ord.reserve(size_t(ninc_));
        for (int32_t sl = 0; sl < nactive_; ++sl) {
            const int m = slot_mesh_[sl];
            const TetMesh& M = sc_.meshes[m];
            const int v = orig_of_[sl] - int32_t(mesh_off_[m]);
            const int32_t base = tet_off[m];
            for (int k = M.nbr_ofs[v]; k < M.nbr_ofs[v + 1]; ++k) {
                inc_tet.push_back(base + M.nbr_tet[k]);
                inc_ord.push_back(static_cast<int8_t>(M.nbr_order[k]));
            }
        }
        std::vector<double4> mat(nmesh_);
        for (int m = 0; m < nmesh_; ++m) {
            const ObjectParams& o = sc_.objs[m];
            mat[m] = make_double4(o.miu, o.lmbd, o.dampingHydrostatic, o.dampingDeviatoric);
        }
        std::vector<double> mass(size_t(nslots_), 0.0);
        for (int m = 0; m < nmesh_; ++m)
            for (int v = 0; v < sc_.meshes[m].nv; ++v) mass[size_t(slot_of_[mesh_off_[m] + v])] = sc_.meshes[m].mass[v];
        d_tet_slots_.upload(ts, &bytes_, st_);
        d_tet_dminv_.upload(dm, &bytes_, st_);
        d_tet_vol_.upload(vol, &bytes_, st_);
        d_tet_mesh_.upload(tm, &bytes_, st_);
        d_conv_inc_tet_.upload(inc_tet, &bytes_, st_);
        d_conv_inc_ord_.upload(inc_ord, &bytes_, st_);
        d_conv_mat_.upload(mat, &bytes_, st_);
        d_conv_mass_.upload(mass, &bytes_, st_);
        conv_nb_t_ = std::max(1, div_up(int64_t(ts.size()), dev::kConvThreads));
        conv_nb_v_ = std::max(1, div_up(nslots_, dev::kConvThreads));
        d_conv_part_.alloc(size_t(conv_nb_t_) + 2 * size_t(conv_nb_v_), &bytes_);
        d_conv_out_.alloc(4, &bytes_);
        conv_per_substep_ = 1 + (sc_.p.iterations + sc_.p.evaluationSteps - 1) / sc_.p.evaluationSteps;
        if (sc_.p.iterations == 0) conv_per_substep_ = 1;
        conv_cap_ = sc_.p.evaluateConvergence ? conv_per_substep_ * sc_.p.numSubsteps : 0;
        d_conv_log_.alloc(4 * size_t(std::max(conv_cap_, 1)), &bytes_);
        d_conv_count_.alloc(1, &bytes_);
        GAIA_CUDA(cudaMemsetAsync(d_conv_count_.p, 0, sizeof(int32_t), st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        conv_ready_ = true;
    }

    dev::ConvData conv_data() const {
        dev::ConvData D;
        D.tet_slots = d_tet_slots_.p;
        D.tet_dminv = d_tet_dminv_.p;
        D.tet_vol = d_tet_vol_.p;
        D.tet_mesh = d_tet_mesh_.p;
        D.mesh_mat = d_conv_mat_.p;
        D.slot_mesh = d_slot_mesh_.p;
        D.slot_mass = d_conv_mass_.p;
        D.inc_ofs = d_inc_ofs_.p;
        D.inc_tet = d_conv_inc_tet_.p;
        D.inc_ord = d_conv_inc_ord_.p;
        D.ntet = int32_t(d_tet_slots_.n);
        D.nactive = nactive_;
        D.nslots = int32_t(nslots_);
        D.dt2inv = sc_.p.dtSqrReciprocal;
        D.inv_dt = 1.0 / sc_.p.dt;
        return D;
    }

    // Three kernels: elastic partials, inertia / force-norm partials, the fixed-order finish
    // into the log (to_log) or into the single-record output.
    void enqueue_conv(bool to_log) {
        const dev::ConvData D = conv_data();
        double* pe = d_conv_part_.p;
        double* pi = pe + conv_nb_t_;
        double* pf = pi + conv_nb_v_;
        if (D.ntet) dev::k_conv_tets<ST><<<conv_nb_t_, dev::kConvThreads, 0, st_>>>(d_pos_.p, d_rest_.p, D, pe);
        else GAIA_CUDA(cudaMemsetAsync(pe, 0, sizeof(double), st_));
        dev::k_conv_verts<ST><<<conv_nb_v_, dev::kConvThreads, 0, st_>>>(d_pos_.p, d_y_.p, d_xprev_.p, d_rest_.p, D, pi,
                                                                         pf);
        dev::k_conv_finish<<<1, dev::kConvThreads, 0, st_>>>(pe, D.ntet ? conv_nb_t_ : 1, pi, pf, conv_nb_v_,
                                                             1.0 / double(std::max<int64_t>(nslots_, 1)),
                                                             to_log ? d_conv_log_.p : d_conv_out_.p,
                                                             to_log ? d_conv_count_.p : nullptr,
                                                             to_log ? conv_cap_ : 1);
        GAIA_CUDA(cudaGetLastError());
    }

    // evaluateConvergenceGPU on the current state: energy, inertia, elastic, average force norm.
    void convergence(double* out4) override {
        setup_conv();
        enqueue_conv(false);
        GAIA_CUDA(cudaMemcpyAsync(out4, d_conv_out_.p, 4 * sizeof(double), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
    }

    double energy() override {
        double out[4];
        convergence(out);
        return out[0];
    }

    // Records of the last step: (substep, iteration, energy, inertia, elastic, average force norm).
    void convergence_log(std::vector<double>& rows) override {
        rows.clear();
        if (!sc_.p.evaluateConvergence) return;
        int32_t n = 0;
        GAIA_CUDA(cudaMemcpyAsync(&n, d_conv_count_.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        n = std::min(n, conv_cap_);
        std::vector<double> log(4 * size_t(std::max(n, 1)));
        if (n) GAIA_CUDA(cudaMemcpyAsync(log.data(), d_conv_log_.p, 4 * size_t(n) * sizeof(double),
                                         cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        for (int k = 0; k < n; ++k) {
            const int sub = k / conv_per_substep_, e = k % conv_per_substep_;
            rows.push_back(double(sub));
            rows.push_back(e == 0 ? -1.0 : double((e - 1) * sc_.p.evaluationSteps));
            rows.insert(rows.end(), log.begin() + 4 * size_t(k), log.begin() + 4 * size_t(k) + 4);
        }
    }

    void vertex_force_hessian(int mesh, int v, int friction, double* f3, double* h9) override {
        int64_t off, n;
        mesh_range(mesh, off, n);
        if (v < 0 || v >= n) throw std::invalid_argument("vertex index out of range");
        int32_t s = slot_of_[off + v];
        if (s >= nactive_) throw std::invalid_argument("vertex is fixed (not solved)");
        if (cd_.enabled()) launch_contact_color(s, s + 1, false);
        launch_solve<true>(lanes_, block_, s, s + 1, friction, d_probe_.p);
        double h[12];
        GAIA_CUDA(cudaMemcpyAsync(h, d_probe_.p, sizeof(h), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        for (int i = 0; i < 3; ++i) f3[i] = h[i];
        for (int i = 0; i < 9; ++i) h9[i] = h[3 + i];
    }

    void stats(gaia_vbd_stats* s) override {
        unsigned long long h[dev::CNT_N];
        GAIA_CUDA(cudaMemcpyAsync(h, d_counters_.p, sizeof(h), cudaMemcpyDeviceToHost, st_));
        GAIA_CUDA(cudaStreamSynchronize(st_));
        s->precision = ST::kCode;
        s->lanes_per_vertex = lanes_;
        s->block_size = block_;
        s->num_groups = int32_t(sc_.groups.size());
        s->sweep_mode = mode_;
        s->cluster_size = mode_ == kSweepCluster ? scene_C_ : 0;
        s->num_vertices = nslots_;
        s->num_active_vertices = nactive_;
        s->num_incidences = ninc_;
        s->kernel_launches_per_step = launches_per_step_;
        s->fp64_fallback_solves = int64_t(h[dev::CNT_FP64_SOLVES]);
        s->failed_solves = int64_t(h[dev::CNT_FAILED_SOLVES]);
        s->device_bytes = int64_t(bytes_);
        s->autotune_ms_per_iteration = tuned_ms_;
        s->solve_variant = variant_;
        s->mesh_frames = frames_ ? 1 : 0;
        unsigned long long cc[cloth::CC_N];
        cd_.counters(cc, st_);
        s->contact_detections = int64_t(cc[cloth::CC_DETECTIONS]);
        s->contact_stack_overflow = int64_t(cc[cloth::CC_STACK_OVERFLOW]);
        s->contact_traverse_bounds = int64_t(cc[cloth::CC_TRUNCATIONS]);
        s->device_timeouts = reported_timeouts_ + int64_t(h[dev::CNT_TIMEOUT]);
        s->nonfinite_solves = reported_nonfinite_ + int64_t(h[dev::CNT_NONFINITE]);
    }

private:
    const Scene& sc_;
    cudaStream_t st_ = nullptr;
    cudaEvent_t ev_a_ = nullptr, ev_b_ = nullptr, ev_c_ = nullptr;
    cudaGraphExec_t g_init_ = nullptr, g_init_rb_ = nullptr, g_sweep_ = nullptr, g_vel_ = nullptr;
    cudaGraphExec_t g_step_ = nullptr, g_step_rb_ = nullptr;  // init + sweep + velocity of one substep
    tetcd::Detector cd_;
    DevBuf<float4> d_xf_;
    DevBuf<double2> d_mesh_fric_;
    DevBuf<R> d_col_scratch_;
    int nmesh_ = 0;
    int64_t nslots_ = 0;
    int32_t nactive_ = 0, ninc_ = 0;
    int lanes_ = 0, block_ = 0;
    std::vector<ColorCfg> ccfg_;
    bool tuned_ = false;
    bool use_pdl_ = true;
    int small_color_ = 16384;
    int variant_ = 0;          // 0 = register-pipelined k_solve, 1 = TMA-staged k_solve_tma, 2 = k_sweep_scenes,
                               // 3 = k_sweep_cluster, 4 = k_solve_deep, 5 = k_sweep_grid, 6 = k_solve with L2
                               // prefetch of the next wave's records, 7 = k_solve_pipe
    int mode_ = 0;             // kSweepMerged, kSweepScenes, kSweepCluster or kSweepGrid
    // scene-major mode: per mesh its color slot ranges, in sweep order
    std::vector<int2> scene_colors_;
    std::vector<int32_t> scene_ofs_;
    int32_t nscenes_ = 0;
    int scene_L_ = 8, scene_B_ = 512, scene_C_ = 8, num_sms_ = 1;
    DevBuf<int2> d_scene_colors_;
    DevBuf<int32_t> d_scene_ofs_, d_scene_order_, d_scene_work_;
    std::vector<ClusterFit> cluster_fits_;
    DevBuf<int4> d_scene_slots_;
    // grid mode: the merged colors' slot ranges, the barrier's counter and abort flag
    DevBuf<int2> d_grid_colors_;
    // mesh frames: per mesh the reference slot, the FP64 offset, this substep's shift, the planes
    bool frames_ = false;
    DevBuf<int32_t> d_frame_ref_;
    DevBuf<double4> d_frame_F_;
    DevBuf<float4> d_frame_shift_;
    DevBuf<float4> d_rest_fh_, d_rest_fl_;
    DevBuf<uint32_t> d_grid_bar_;
    int32_t grid_ncolors_ = 0, grid_max_color_ = 0;
    int variant_fixed_ = -1;   // from PhysicsParams solveVariant (-1 = autotune)
    std::map<std::pair<int, int>, int> maxrec_cache_;
    std::map<std::pair<int, int>, int> wave_cache_;  // (lanes, block) -> resident blocks of k_solve
    std::map<std::pair<int, int>, int> pipe_occ_;    // (lanes and block, shared bytes) -> k_solve_pipe blocks per SM
    static constexpr size_t kTmaSmemMax = 200 * 1024;
    static constexpr int kContactBlocks = 64;
    double tuned_ms_ = 0.0;
    int64_t launches_per_substep_ = 0, launches_per_step_ = 0;
    int64_t reported_timeouts_ = 0, reported_nonfinite_ = 0;  // status counts already reported
    size_t bytes_ = 0;
    dev::Consts<R> c_{};
    std::vector<int64_t> mesh_off_;
    std::vector<int32_t> slot_of_, orig_of_, slot_mesh_, inc_ofs_, group_beg_, group_end_;
    std::vector<int4> h_rec_n_;
    std::vector<R4> h_rec_a_, h_rec_b_;
    std::vector<S4> h_pos_;
    std::vector<V4> h_vel_;
    std::vector<float4> h_rest_;
    std::vector<R> h_rec_c_;
    std::vector<dev::MeshMat<R>> h_mats_;
    std::vector<dev::DeformerDev> h_defs_;
    std::vector<int32_t> h_def_slot_, h_def_idx_;
    std::vector<double> h_def_a_, h_def_b_;
    DevBuf<S4> d_pos_, d_y_, d_xprev_, d_acc_pp_, d_acc_prev_;
    DevBuf<V4> d_vel_, d_vprev_;
    DevBuf<int32_t> d_inc_ofs_, d_slot_mesh_, d_slot_of_, d_def_slot_, d_def_idx_, d_tet_mesh_;
    DevBuf<int4> d_rec_n_, d_tet_slots_;
    DevBuf<R4> d_rec_a_, d_rec_b_;
    DevBuf<R> d_rec_c_;
    DevBuf<dev::MeshMat<R>> d_mats_;
    DevBuf<unsigned long long> d_counters_;
    DevBuf<double> d_time_, d_def_a_, d_def_b_, d_stage_f64_, d_probe_, d_tet_dminv_, d_tet_vol_;
    // convergence reduction
    bool conv_ready_ = false;
    int conv_nb_t_ = 1, conv_nb_v_ = 1, conv_per_substep_ = 1, conv_cap_ = 0;
    DevBuf<int32_t> d_conv_inc_tet_, d_conv_count_;
    DevBuf<int8_t> d_conv_inc_ord_;
    DevBuf<double4> d_conv_mat_;
    DevBuf<double> d_conv_part_, d_conv_out_, d_conv_log_, d_conv_mass_;
    DevBuf<dev::DeformerDev> d_defs_;
    DevBuf<float4> d_rest_;
    DevBuf<float> d_stage_f32_;
};

// The engine of each precision mode, built in its own translation unit.
EngineBase* make_engine_f32(const Scene& s, int mode);
EngineBase* make_engine_df(const Scene& s, int mode);
EngineBase* make_engine_dfh(const Scene& s, int mode);
EngineBase* make_engine_f64(const Scene& s, int mode);

}  // namespace gaia

