// C ABI of libgaia_vbd.so (declared in include/gaia_vbd.h) over the engines of
// vbd_engine.cuh.
#include "vbd_engine.cuh"

namespace gaia {
namespace {
thread_local std::string g_last_error;
}  // namespace

// Message for gaia_vbd_last_global_error from entry points defined in other files.
void set_last_global_error(const std::string& msg) { g_last_error = msg; }

}  // namespace gaia

// =============================================================================
// C ABI
// =============================================================================
struct gaia_vbd {
    gaia::Scene scene;
    std::unique_ptr<gaia::EngineBase> eng;
    std::string err;
    int64_t frame = 0;  // runStep calls since initialize / the last loaded state
    double sweep_ms[4] = {0.0, 0.0, 0.0, 0.0};  // autotuned schedule choice: measured ms per iteration,
                                                // merged / scenes / cluster / grid (0 where not timed)
};

namespace {

template <typename Fn>
int guarded(gaia_vbd* h, Fn&& fn) {
    try {
        fn();
        if (h) h->err.clear();
        return GAIA_VBD_OK;
    } catch (const gaia::CudaError& e) {
        (h ? h->err : gaia::g_last_error) = e.what();
        return GAIA_VBD_E_CUDA;
    } catch (const std::invalid_argument& e) {
        (h ? h->err : gaia::g_last_error) = e.what();
        return GAIA_VBD_E_INVALID_ARG;
    } catch (const std::domain_error& e) {
        (h ? h->err : gaia::g_last_error) = e.what();
        return GAIA_VBD_E_NONFINITE;
    } catch (const gaia::DeviceTimeout& e) {
        (h ? h->err : gaia::g_last_error) = e.what();
        return GAIA_VBD_E_DEVICE_TIMEOUT;
    } catch (const std::exception& e) {
        (h ? h->err : gaia::g_last_error) = e.what();
        std::string m = e.what();
        if (m.find("coloring") != std::string::npos) return GAIA_VBD_E_COLORING;
        if (m.find("degenerate") != std::string::npos || m.find("fixed point") != std::string::npos ||
            m.find("out of range") != std::string::npos)
            return GAIA_VBD_E_MESH;
        if (m.find("not supported") != std::string::npos) return GAIA_VBD_E_UNSUPPORTED;
        return GAIA_VBD_E_INPUT;
    } catch (...) {
        (h ? h->err : gaia::g_last_error) = "unknown error";
        return GAIA_VBD_E_INPUT;
    }
}

}  // namespace

extern "C" {

int gaia_vbd_load(const char* models_json, const char* params_json, const char* repo_root, gaia_vbd** out) {
    if (!models_json || !params_json || !out) {
        gaia::g_last_error = "null argument";
        return GAIA_VBD_E_INVALID_ARG;
    }
    *out = nullptr;
    std::unique_ptr<gaia_vbd> h(new gaia_vbd());
    int rc = guarded(nullptr, [&] { gaia::load_scene(models_json, params_json, repo_root ? repo_root : "", h->scene); });
    if (rc) return rc;
    *out = h.release();
    return GAIA_VBD_OK;
}

int gaia_vbd_initialize(gaia_vbd* h) {
    if (!h) return GAIA_VBD_E_INVALID_ARG;
    if (h->eng) return GAIA_VBD_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        h->err = gaia::g_last_error = "no CUDA device is visible";
        return GAIA_VBD_E_NO_DEVICE;
    }
    return guarded(h, [&] {
        const gaia::PhysicsParams& p = h->scene.p;
        auto make = [&](int mode) -> gaia::EngineBase* {
            if (p.gpuPrecision == "fp64") return gaia::make_engine_f64(h->scene, mode);
            if (p.gpuPrecision == "fp32") return gaia::make_engine_f32(h->scene, mode);
            if (p.gpuPrecision == "dfhi") return gaia::make_engine_dfh(h->scene, mode);
            return gaia::make_engine_df(h->scene, mode);
        };
        // color scheduling: merged colors (one launch per merged color and iteration), scene-major
        // (one persistent launch per substep) or the grid sweep (one cooperative launch per
        // substep over the merged colors). The persistent sweeps need no per-iteration work
        // outside the solve; the scene-major ones also meshes that do not interact.
        const bool scenes_ok = !(p.allowCCD || p.allowDCD) && !p.useAccelerator && !p.evaluateConvergence &&
                               p.iterations > 0;
        if ((p.sweepMode == "scenes" || p.sweepMode == "cluster" || p.sweepMode == "grid") && !scenes_ok)
            throw std::runtime_error("sweepMode \"" + p.sweepMode + "\" is not supported with contact detection, "
                                     "the accelerator or evaluateConvergence");
        if (p.sweepMode == "merged" || !scenes_ok || (p.sweepMode == "auto" && !p.autotune)) {
            h->eng.reset(make(gaia::kSweepMerged));
        } else if (p.sweepMode == "scenes") {
            h->eng.reset(make(gaia::kSweepScenes));
        } else if (p.sweepMode == "cluster") {
            h->eng.reset(make(gaia::kSweepCluster));
        } else if (p.sweepMode == "grid") {
            h->eng.reset(make(gaia::kSweepGrid));
        } else {
            // autotuned: every schedule the scene allows is built and its sweep graph timed;
            // the fastest is kept (the cluster sweep only where every scene fits on-chip)
            std::unique_ptr<gaia::EngineBase> best(make(gaia::kSweepMerged));
            h->sweep_ms[0] = best->measure_sweep_ms();
            double tbest = h->sweep_ms[0];
            // a scene-major sweep runs each scene on one block (or one cluster): a scene much
            // larger than a block can hold on-chip only serialises its work, so the autotuner
            // does not time those schedules when a mesh has more than kSceneMajorMaxVertices
            int64_t largest = 0;
            for (const auto& m : h->scene.meshes) {
                int64_t n = 0;
                for (uint8_t f : m.fixed) n += f ? 0 : 1;
                largest = std::max(largest, n);
            }
            constexpr int64_t kSceneMajorMaxVertices = 65536;
            for (int mode : {gaia::kSweepGrid, gaia::kSweepScenes, gaia::kSweepCluster}) {
                if (mode != gaia::kSweepGrid && largest > kSceneMajorMaxVertices) break;
                std::unique_ptr<gaia::EngineBase> e;
                if (mode == gaia::kSweepCluster) {
                    try {
                        e.reset(make(mode));
                    } catch (const std::runtime_error& ex) {
                        if (std::string(ex.what()).find("does not fit") == std::string::npos) throw;
                        continue;  // a scene too large for a cluster's shared memory
                    }
                } else if (mode == gaia::kSweepGrid) {
                    // a device or driver without cooperative launches in captured graphs: the
                    // schedule is left out (sweep_ms_grid = -1); an explicit "grid" reports it
                    try {
                        e.reset(make(mode));
                    } catch (const std::runtime_error&) {
                        (void)cudaGetLastError();
                        h->sweep_ms[mode] = -1.0;
                        continue;
                    }
                } else {
                    e.reset(make(mode));
                }
                const double t = e->measure_sweep_ms();
                h->sweep_ms[mode] = t;
                if (t < tbest) {
                    tbest = t;
                    best = std::move(e);
                }
            }
            h->eng = std::move(best);
        }
    });
}

int gaia_vbd_create(const char* models_json, const char* params_json, const char* repo_root, gaia_vbd** out) {
    gaia_vbd* h = nullptr;
    int rc = gaia_vbd_load(models_json, params_json, repo_root, &h);
    if (rc) return rc;
    rc = gaia_vbd_initialize(h);
    if (rc) {
        gaia::g_last_error = h->err;
        delete h;
        return rc;
    }
    *out = h;
    return GAIA_VBD_OK;
}

void gaia_vbd_destroy(gaia_vbd* h) { delete h; }

const char* gaia_vbd_last_error(const gaia_vbd* h) { return h ? h->err.c_str() : gaia::g_last_error.c_str(); }
const char* gaia_vbd_last_global_error(void) { return gaia::g_last_error.c_str(); }

#define GAIA_NEED(h)                                                   \
    do {                                                               \
        if (!(h)) return GAIA_VBD_E_INVALID_ARG;                       \
        if (!(h)->eng) {                                               \
            (h)->err = "handle is not initialized (gaia_vbd_initialize)"; \
            return GAIA_VBD_E_INVALID_ARG;                             \
        }                                                              \
    } while (0)

int gaia_vbd_run_step(gaia_vbd* h, int32_t n_steps) {
    GAIA_NEED(h);
    if (n_steps < 0) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] {
        h->eng->run_steps(n_steps);
        h->frame += n_steps;
    });
}

namespace {
// Surface vertices (FP32 positions) and surface faces in surface-vertex numbering of every
// mesh: what TetMeshFEM::saveAsPLY and writeAllToBinary write (surfaceVIds order here is
// ascending vertex id).
std::vector<gaia::FrameMesh> tet_frame(gaia_vbd* h) {
    std::vector<gaia::FrameMesh> out;
    for (size_t m = 0; m < h->scene.meshes.size(); ++m) {
        const gaia::TetMesh& M = h->scene.meshes[m];
        std::vector<double> x(3 * size_t(M.nv));
        h->eng->get_positions(int(m), x.data());
        gaia::FrameMesh fm;
        std::vector<int32_t> local(size_t(M.nv), -1);
        for (size_t i = 0; i < M.sverts.size(); ++i) {
            const int32_t v = M.sverts[i];
            local[size_t(v)] = int32_t(i);
            for (int d = 0; d < 3; ++d) fm.X.push_back(float(x[3 * size_t(v) + d]));
        }
        for (int32_t v : M.sfaces) fm.faces.push_back(local[size_t(v)]);
        fm.model_path = h->scene.objs[m].path;
        out.push_back(std::move(fm));
    }
    return out;
}
}  // namespace

int gaia_vbd_write_ply(gaia_vbd* h, const char* path, int32_t all_in_one, int32_t add_model_name) {
    GAIA_NEED(h);
    if (!path) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { gaia::write_frame_ply(path, tet_frame(h), all_in_one != 0, add_model_name != 0, false); });
}

int gaia_vbd_write_binary(gaia_vbd* h, const char* path) {
    GAIA_NEED(h);
    if (!path) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { gaia::write_frame_binary(path, tet_frame(h)); });
}

int gaia_vbd_save_state(gaia_vbd* h, const char* path, int32_t binary) {
    GAIA_NEED(h);
    if (!path) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] {
        gaia::PhysicsStateFile st;
        st.frameId = int(h->frame);
        st.curTime = h->eng->get_time();
        for (size_t m = 0; m < h->scene.meshes.size(); ++m) {
            const size_t nv = size_t(h->scene.meshes[m].nv);
            std::vector<double> x(3 * nv), v(3 * nv);
            h->eng->get_positions(int(m), x.data());
            h->eng->get_velocities(int(m), v.data());
            st.position.emplace_back(x.begin(), x.end());
            st.velocity.emplace_back(v.begin(), v.end());
        }
        gaia::write_physics_state(path, st, binary != 0);
    });
}

int gaia_vbd_load_state(gaia_vbd* h, const char* path) {
    GAIA_NEED(h);
    if (!path) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] {
        gaia::PhysicsStateFile st = gaia::read_physics_state(path);
        // BasePhysicFramework::recoverFromState / PhysicsState::initializePhysics: meshes
        // beyond the file's are left as they are
        for (size_t m = 0; m < h->scene.meshes.size() && m < st.position.size(); ++m) {
            const size_t nv = size_t(h->scene.meshes[m].nv);
            if (st.position[m].size() != 3 * nv)
                throw std::invalid_argument("state file mesh " + std::to_string(m) + " has " +
                                            std::to_string(st.position[m].size() / 3) + " vertices, the scene " +
                                            std::to_string(nv));
            std::vector<double> x(st.position[m].begin(), st.position[m].end());
            std::vector<double> v(st.velocity[m].begin(), st.velocity[m].end());
            h->eng->set_positions(int(m), x.data());
            h->eng->set_velocities(int(m), v.data());
        }
        h->frame = st.frameId;
        h->eng->set_time(st.curTime);
    });
}

int gaia_vbd_synchronize(gaia_vbd* h) {
    GAIA_NEED(h);
    return guarded(h, [&] { h->eng->sync(); });
}

int gaia_vbd_run_step_timed(gaia_vbd* h, int32_t n_steps, float* total_ms, float* sweep_ms) {
    GAIA_NEED(h);
    if (n_steps <= 0) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->run_steps_timed(n_steps, total_ms, sweep_ms); });
}

int gaia_vbd_num_surface(gaia_vbd* h, int32_t mesh, int32_t* nfaces, int32_t* nverts) {
    if (!h) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] {
        if (mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) throw std::invalid_argument("mesh index out of range");
        const gaia::TetMesh& m = h->scene.meshes[mesh];
        if (nfaces) *nfaces = int32_t(m.sfaces.size() / 3);
        if (nverts) *nverts = int32_t(m.sverts.size());
    });
}

int gaia_vbd_get_surface(gaia_vbd* h, int32_t mesh, int32_t* faces, int32_t* verts) {
    if (!h) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] {
        if (mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) throw std::invalid_argument("mesh index out of range");
        const gaia::TetMesh& m = h->scene.meshes[mesh];
        if (faces) std::copy(m.sfaces.begin(), m.sfaces.end(), faces);
        if (verts) std::copy(m.sverts.begin(), m.sverts.end(), verts);
    });
}

int gaia_vbd_set_prev_positions(gaia_vbd* h, int32_t mesh, const double* xyz) {
    GAIA_NEED(h);
    if (!xyz) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->set_prev_positions(mesh, xyz); });
}

int gaia_vbd_collide(gaia_vbd* h, int32_t* n_contacts) {
    GAIA_NEED(h);
    return guarded(h, [&] {
        const int n = h->eng->collide();
        if (n_contacts) *n_contacts = n;
    });
}

int gaia_vbd_get_contacts(gaia_vbd* h, int32_t* rows, int32_t cap, int32_t* n_rows) {
    GAIA_NEED(h);
    return guarded(h, [&] {
        std::vector<int32_t> r;
        h->eng->contacts(r);
        const int32_t n = int32_t(r.size() / 8);
        if (n_rows) *n_rows = n;
        if (rows) std::copy(r.begin(), r.begin() + 8 * std::min(n, std::max(cap, 0)), rows);
    });
}

int gaia_vbd_reset(gaia_vbd* h) {
    GAIA_NEED(h);
    return guarded(h, [&] {
        h->eng->reset();
        h->frame = 0;
    });
}

int gaia_vbd_autotune(gaia_vbd* h) {
    GAIA_NEED(h);
    return guarded(h, [&] { h->eng->autotune(); });
}

int gaia_vbd_num_meshes(const gaia_vbd* h) { return h ? int(h->scene.meshes.size()) : -1; }

int64_t gaia_vbd_num_vertices(const gaia_vbd* h, int32_t mesh) {
    if (!h || mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) return -1;
    return h->scene.meshes[mesh].nv;
}

int64_t gaia_vbd_num_tets(const gaia_vbd* h, int32_t mesh) {
    if (!h || mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) return -1;
    return h->scene.meshes[mesh].ntet;
}

int gaia_vbd_get_positions(gaia_vbd* h, int32_t mesh, double* out) {
    GAIA_NEED(h);
    if (!out) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->get_positions(mesh, out); });
}
int gaia_vbd_set_positions(gaia_vbd* h, int32_t mesh, const double* in) {
    GAIA_NEED(h);
    if (!in) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->set_positions(mesh, in); });
}
int gaia_vbd_get_velocities(gaia_vbd* h, int32_t mesh, double* out) {
    GAIA_NEED(h);
    if (!out) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->get_velocities(mesh, out); });
}
int gaia_vbd_set_velocities(gaia_vbd* h, int32_t mesh, const double* in) {
    GAIA_NEED(h);
    if (!in) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->set_velocities(mesh, in); });
}
int gaia_vbd_set_state_f32(gaia_vbd* h, const float* x, const float* v) {
    GAIA_NEED(h);
    return guarded(h, [&] { h->eng->set_state_f32(x, v); });
}
int gaia_vbd_get_positions_f32(gaia_vbd* h, float* x) {
    GAIA_NEED(h);
    if (!x) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->get_positions_f32(x); });
}
int gaia_vbd_get_velocities_f32(gaia_vbd* h, float* v) {
    GAIA_NEED(h);
    if (!v) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->get_velocities_f32(v); });
}

int gaia_vbd_num_groups(const gaia_vbd* h) { return h ? int(h->scene.groups.size()) : -1; }

int64_t gaia_vbd_group_size(const gaia_vbd* h, int32_t g) {
    if (!h || g < 0 || size_t(g) >= h->scene.groups.size()) return -1;
    return int64_t(h->scene.groups[g].size() / 2);
}

int gaia_vbd_get_group(const gaia_vbd* h, int32_t g, int32_t* out_pairs) {
    if (!h || !out_pairs || g < 0 || size_t(g) >= h->scene.groups.size()) return GAIA_VBD_E_INVALID_ARG;
    std::copy(h->scene.groups[g].begin(), h->scene.groups[g].end(), out_pairs);
    return GAIA_VBD_OK;
}

int gaia_vbd_get_coloring(const gaia_vbd* h, int32_t mesh, int32_t* colors) {
    if (!h || !colors || mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) return GAIA_VBD_E_INVALID_ARG;
    const auto& M = h->scene.meshes[mesh];
    for (size_t c = 0; c < M.colors.size(); ++c)
        for (int32_t v : M.colors[c]) colors[v] = int32_t(c);
    return GAIA_VBD_OK;
}

int gaia_vbd_get_rest_shape(const gaia_vbd* h, int32_t mesh, double* dminv, double* vol, double* mass) {
    if (!h || mesh < 0 || size_t(mesh) >= h->scene.meshes.size()) return GAIA_VBD_E_INVALID_ARG;
    const auto& M = h->scene.meshes[mesh];
    if (dminv) std::copy(M.dminv.begin(), M.dminv.end(), dminv);
    if (vol) std::copy(M.vol.begin(), M.vol.end(), vol);
    if (mass) std::copy(M.mass.begin(), M.mass.end(), mass);
    return GAIA_VBD_OK;
}

int gaia_vbd_energy(gaia_vbd* h, double* out) {
    GAIA_NEED(h);
    if (!out) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { *out = h->eng->energy(); });
}

int gaia_vbd_convergence(gaia_vbd* h, double* out4) {
    GAIA_NEED(h);
    if (!out4) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->convergence(out4); });
}

int gaia_vbd_get_convergence_log(gaia_vbd* h, double* rows, int32_t cap, int32_t* n_rows) {
    GAIA_NEED(h);
    return guarded(h, [&] {
        std::vector<double> r;
        h->eng->convergence_log(r);
        const int32_t n = int32_t(r.size() / 6);
        if (n_rows) *n_rows = n;
        if (rows) std::copy(r.begin(), r.begin() + 6 * std::min(n, std::max(cap, 0)), rows);
    });
}

int gaia_vbd_vertex_force_hessian(gaia_vbd* h, int32_t mesh, int32_t vertex, int32_t apply_friction, double* f3,
                                  double* h9) {
    GAIA_NEED(h);
    if (!f3 || !h9) return GAIA_VBD_E_INVALID_ARG;
    return guarded(h, [&] { h->eng->vertex_force_hessian(mesh, vertex, apply_friction, f3, h9); });
}

int gaia_vbd_get_color_config(gaia_vbd* h, int32_t g, int32_t* lanes, int32_t* block, int32_t* variant,
                              float* tuned_ms) {
    GAIA_NEED(h);
    return guarded(h, [&] { h->eng->color_config(g, lanes, block, variant, tuned_ms); });
}

int gaia_vbd_get_stats(gaia_vbd* h, gaia_vbd_stats* out) {
    GAIA_NEED(h);
    if (!out) return GAIA_VBD_E_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    return guarded(h, [&] {
        h->eng->stats(out);
        out->sweep_ms_merged = h->sweep_ms[0];
        out->sweep_ms_scenes = h->sweep_ms[1];
        out->sweep_ms_cluster = h->sweep_ms[2];
        out->sweep_ms_grid = h->sweep_ms[3];
    });
}

int gaia_vbd_get_output_params(const gaia_vbd* h, gaia_vbd_output_params* out) {
    if (!h) return GAIA_VBD_E_INVALID_ARG;
    if (!out) return GAIA_VBD_E_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    const gaia::PhysicsParams& p = h->scene.p;
    out->num_frames = p.numFrames;
    out->save_outputs = p.saveOutputs;
    out->save_all_models_together = p.saveAllModelsTogether;
    out->binary_mode_visualization_steps = p.binaryModeVisualizationSteps;
    out->output_recovery_state = p.outputRecoveryState;
    out->output_recovery_state_step = p.outputRecoveryStateStep;
    out->output_recovery_state_binary = p.outputRecoveryStateBinary;
    std::snprintf(out->output_ext, sizeof(out->output_ext), "%s", p.outputExt.c_str());
    return GAIA_VBD_OK;
}

int64_t gaia_vbd_frame(const gaia_vbd* h) { return h ? h->frame : -1; }

int32_t gaia_vbd_color_mcs(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors) {
    if (nv <= 0 || ntet < 0 || (!tets && ntet) || !colors) return -1;
    int32_t n = -1;
    if (guarded(nullptr, [&] { n = gaia::color_mcs(nv, ntet, tets, colors); })) return -1;
    return n;
}

int32_t gaia_vbd_color_greedy(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors) {
    if (nv <= 0 || ntet < 0 || (!tets && ntet) || !colors) return -1;
    int32_t n = -1;
    if (guarded(nullptr, [&] { n = gaia::color_greedy(nv, ntet, tets, colors); })) return -1;
    return n;
}

int32_t gaia_vbd_color_tool(int32_t nv, int32_t ntet, const int32_t* tets, int32_t algorithm, int32_t balance,
                            float goal_ratio, int32_t* colors, int32_t* order) {
    if (nv <= 0 || ntet < 0 || (!tets && ntet) || !colors || (algorithm != 0 && algorithm != 1)) return -1;
    int32_t n = -1;
    if (guarded(nullptr, [&] {
            n = algorithm == 0 ? gaia::color_mcs(nv, ntet, tets, colors) : gaia::color_greedy(nv, ntet, tets, colors);
            auto cats = gaia::colors_to_categories(nv, colors);
            if (balance) {
                std::vector<int64_t> ofs;
                std::vector<int32_t> adj;
                gaia::tet_vertex_graph(nv, ntet, tets, ofs, adj);
                gaia::balance_categories(nv, ofs, adj, colors, cats, goal_ratio);
            }
            if (order) {
                size_t k = 0;
                for (auto& c : cats)
                    for (int32_t v : c) order[k++] = v;
            }
        }))
        return -1;
    return n;
}

int gaia_vbd_write_categories(const char* path, int32_t nv, const int32_t* colors, const int32_t* order) {
    if (!path || nv <= 0 || !colors || !order) return GAIA_VBD_E_INVALID_ARG;
    return guarded(nullptr, [&] {
        int32_t n = 0;
        for (int32_t i = 0; i < nv; ++i) {
            if (colors[i] < 0) throw std::invalid_argument("negative color");
            n = std::max(n, colors[i] + 1);
        }
        std::vector<std::vector<int32_t>> cats(n);
        for (int32_t i = 0; i < nv; ++i) cats[colors[order[i]]].push_back(order[i]);
        gaia::write_coloring(path, cats);
    });
}

int gaia_vbd_write_coloring(const char* path, int32_t nv, const int32_t* colors) {
    if (!path || nv <= 0 || !colors) return GAIA_VBD_E_INVALID_ARG;
    return guarded(nullptr, [&] {
        for (int32_t i = 0; i < nv; ++i)
            if (colors[i] < 0) throw std::invalid_argument("negative color");
        gaia::write_coloring(path, gaia::colors_to_categories(nv, colors));
    });
}

int gaia_vbd_write_t(const char* path, int32_t nv, const double* X, int32_t ntet, const int32_t* tets) {
    if (!path || nv <= 0 || !X || ntet < 0 || (!tets && ntet)) return GAIA_VBD_E_INVALID_ARG;
    return guarded(nullptr, [&] { gaia::write_t(path, nv, X, ntet, tets); });
}

}  // extern "C"
