/*
 * gaia_vbd.hpp — header-only C++ facade over the C ABI of gaia_vbd.h with the method
 * names of the reference's physics framework, for C++ callers that used GAIA::VBDPhysics:
 *
 *   loadRunningparameters  VBD/VBDPhysics.cpp:90-97 (+ ${REPO_ROOT}, Parser/InputHandler.h)
 *   initialize             VBD/VBDPhysics.cpp:208-454
 *   runStep                VBD/VBDPhysics.cpp:809-837
 *   simulate               Framework/BasePhysicsFramework.cpp:284-393 (setUpOutputFolders
 *                          :414-440; the viewer thread and statistics files are not part of it)
 *   writeOutputs           Framework/BasePhysicsFramework.cpp:442-506
 *   recoverFromState       Framework/BasePhysicsFramework.cpp:264-282
 *
 * Failures throw gaia::VBDError with the library's message (the C ABI itself never
 * throws). The object owns its handle; it is movable, not copyable.
 */
#ifndef GAIA_VBD_HPP
#define GAIA_VBD_HPP

#include <cstdio>
#include <filesystem>
#include <stdexcept>
#include <string>
#include <system_error>
#include <utility>
#include <vector>

#include "gaia_vbd.h"

namespace gaia {

class VBDError : public std::runtime_error {
public:
    VBDError(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

class VBDPhysics {
public:
    VBDPhysics() = default;
    ~VBDPhysics() { gaia_vbd_destroy(h_); }
    VBDPhysics(const VBDPhysics&) = delete;
    VBDPhysics& operator=(const VBDPhysics&) = delete;
    VBDPhysics(VBDPhysics&& o) noexcept : h_(std::exchange(o.h_, nullptr)), outputFolder(std::move(o.outputFolder)) {}
    VBDPhysics& operator=(VBDPhysics&& o) noexcept {
        if (this != &o) {
            gaia_vbd_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
            outputFolder = std::move(o.outputFolder);
        }
        return *this;
    }

    // Parses Models.json / Parameters.json, loads meshes and colorings (no GPU needed).
    // "${REPO_ROOT}" in the three paths and in the files' paths becomes repoRoot.
    void loadRunningparameters(std::string modelsFile, std::string paramsFile, std::string outFolder = "",
                               const std::string& repoRoot = "") {
        if (!repoRoot.empty()) {
            modelsFile = replace_root(modelsFile, repoRoot);
            paramsFile = replace_root(paramsFile, repoRoot);
            outFolder = replace_root(outFolder, repoRoot);
        }
        gaia_vbd* h = nullptr;
        const int rc = gaia_vbd_load(modelsFile.c_str(), paramsFile.c_str(), repoRoot.empty() ? nullptr : repoRoot.c_str(), &h);
        if (rc != GAIA_VBD_OK) throw VBDError(rc, std::string("loadRunningparameters: ") + gaia_vbd_last_global_error());
        gaia_vbd_destroy(h_);
        h_ = h;
        outputFolder = std::move(outFolder);
    }
    // Device layout, autotuning and the step's CUDA graphs.
    void initialize() { check(gaia_vbd_initialize(handle()), "initialize"); }
    // One frame: numSubsteps substeps (asynchronous; errors surface on the next sync).
    void runStep() { check(gaia_vbd_run_step(handle(), 1), "runStep"); }
    void synchronize() { check(gaia_vbd_synchronize(handle()), "synchronize"); }
    void recoverFromState(const std::string& stateFile) {
        check(gaia_vbd_load_state(handle(), stateFile.c_str()), "recoverFromState");
    }
    void saveState(const std::string& stateFile, bool binary) {
        check(gaia_vbd_save_state(handle(), stateFile.c_str(), binary ? 1 : 0), "saveState");
    }

    gaia_vbd_output_params outputParams() const {
        gaia_vbd_output_params o;
        check(gaia_vbd_get_output_params(handle(), &o), "outputParams");
        return o;
    }
    // frameId: runStep calls since initialize, or the frame of the recovered state.
    int frameId() const { return int(gaia_vbd_frame(handle())); }
    int numMeshes() const { return gaia_vbd_num_meshes(handle()); }
    std::vector<double> positions(int mesh) {
        const int64_t nv = gaia_vbd_num_vertices(handle(), mesh);
        if (nv < 0) throw VBDError(GAIA_VBD_E_INVALID_ARG, "positions: mesh index out of range");
        std::vector<double> x(3 * size_t(nv));
        check(gaia_vbd_get_positions(handle(), mesh, x.data()), "positions");
        return x;
    }

    // The reference's writeOutputs: frame files A<frame>.<ext> ("ply": all models together
    // or one file per model, as saveAllModelsTogether says; "bin": surface positions, with
    // TemplateMesh/TemplateMesh.ply per model at frame 0 and a PLY every
    // binaryModeVisualizationSteps frames; "obj" writes no frame) and, every
    // outputRecoveryStateStep frames, RecoveryStates/A<frame>.json.
    void writeOutputs(const std::string& outFolder, int frame) {
        const gaia_vbd_output_params o = outputParams();
        char num[16];
        std::snprintf(num, sizeof(num), "%08d", frame);
        const std::string ext = o.output_ext, base = outFolder + "/A" + num;
        const int together = o.save_all_models_together ? 1 : 0;
        if (ext == "bin") {
            if (frame == 0) {
                make_dir(outFolder + "/TemplateMesh");
                check(gaia_vbd_write_ply(handle(), (outFolder + "/TemplateMesh/TemplateMesh.ply").c_str(), 0, 1),
                      "writeOutputs");
            }
            check(gaia_vbd_write_binary(handle(), (base + ".bin").c_str()), "writeOutputs");
            const int vis = o.binary_mode_visualization_steps > 0 ? o.binary_mode_visualization_steps : 1;
            if (!(frame % vis))
                check(gaia_vbd_write_ply(handle(), (base + ".ply").c_str(), together, together), "writeOutputs");
        } else if (ext == "ply") {
            check(gaia_vbd_write_ply(handle(), (base + ".ply").c_str(), together, together), "writeOutputs");
        } else if (ext != "obj") {
            std::fprintf(stderr, "[Error] Unsupported output EXT name: %s\n", ext.c_str());
            return;
        }
        const int step = o.output_recovery_state_step > 0 ? o.output_recovery_state_step : 1;
        if (o.output_recovery_state && !(frame % step))
            check(gaia_vbd_save_state(handle(), (outFolder + "/RecoveryStates/A" + num + ".json").c_str(),
                                      o.output_recovery_state_binary),
                  "writeOutputs");
    }

    // The reference's simulate: output folders, frame frameId, then runStep and the
    // outputs of every frame up to numFrames (outputs after frame 0 only while
    // saveOutputs holds; setSaveOutputs(false) is what the command line does for
    // "noOutput"). Returns the number of frames stepped.
    int simulate() {
        const gaia_vbd_output_params o = outputParams();
        const bool save = saveOutputs_ < 0 ? o.save_outputs != 0 : saveOutputs_ != 0;
        make_dir(outputFolder);
        if (o.output_recovery_state) make_dir(outputFolder + "/RecoveryStates");
        int frame = frameId();
        writeOutputs(outputFolder, frame);
        int steps = 0;
        while (frame < o.num_frames) {
            runStep();
            ++frame;
            ++steps;
            if (save) writeOutputs(outputFolder, frame);
        }
        synchronize();
        return steps;
    }
    void setSaveOutputs(bool save) { saveOutputs_ = save ? 1 : 0; }

    gaia_vbd* handle() const {
        if (!h_) throw VBDError(GAIA_VBD_E_INVALID_ARG, "call loadRunningparameters first");
        return h_;
    }

    std::string outputFolder;

private:
    void check(int rc, const char* what) const {
        if (rc != GAIA_VBD_OK) throw VBDError(rc, std::string(what) + ": " + gaia_vbd_last_error(h_));
    }
    static std::string replace_root(std::string s, const std::string& root) {
        const std::string key = "${REPO_ROOT}";
        for (size_t k = s.find(key); k != std::string::npos; k = s.find(key, k + root.size()))
            s.replace(k, key.size(), root);
        return s;
    }
    static void make_dir(const std::string& d) {  // MF::IO::createFolder: parents too, no error if present
        std::error_code ec;
        std::filesystem::create_directories(d, ec);
    }

    gaia_vbd* h_ = nullptr;
    int saveOutputs_ = -1;  // -1: Parameters.json's saveOutputs
};

}  // namespace gaia

#endif
