// Command-line runner with the reference's VBDDynamics interface
// (Simulator/VBDDynamics/main.cpp, BasePhysicFramework::simulate and writeOutputs,
// Modules/Framework/BasePhysicsFramework.cpp:284-393, 442-506), on the C ABI:
//
//   vbd_dynamics Models.json Parameters.json outFolder [-R repoRoot] [-r recoveryState.json]
//
// Loads and initializes the scene, optionally recovers a PhysicsState, writes frame 0 (as the
// reference does, whatever saveOutputs says), then runs steps until frame numFrames, writing
// after each one while saveOutputs holds (outFolder "noOutput" clears it). "${REPO_ROOT}" in
// the three paths is replaced by -R, as InputHandlerVBD::handleInput does:
// outputExt "ply" -> <out>/A<%08d>.ply (all models together or one file per model, as
// saveAllModelsTogether says); "bin" -> <out>/A<%08d>.bin, the template mesh
// <out>/TemplateMesh/TemplateMesh.ply at frame 0 and a PLY every binaryModeVisualizationSteps
// frames; recovery states <out>/RecoveryStates/A<%08d>.json every outputRecoveryStateStep
// frames (outputRecoveryState, outputRecoveryStateBinary). The frame loop, output layout and
// parameter keys follow the reference; the step itself is the library's.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <system_error>

#include "gaia_vbd.h"
#include "json_get.hpp"
#include "json_lite.hpp"

namespace {

struct OutputParams {
    int numFrames = 5000;
    bool saveOutputs = true;
    bool saveAllModelsTogether = true;
    std::string outputExt = "ply";
    int binaryModeVisualizationSteps = 100;
    bool outputRecoveryState = true;
    int outputRecoveryStateStep = 10;
    bool outputRecoveryStateBinary = true;
};

// MF::IO::createFolder: the folder and its parents, no error if it exists
void make_dir(const std::string& d) {
    std::error_code ec;
    std::filesystem::create_directories(d, ec);
}

std::string frame_name(int frame) {
    char b[16];
    std::snprintf(b, sizeof(b), "%08d", frame);
    return b;
}

int fail(gaia_vbd* h, const char* what) {
    std::fprintf(stderr, "%s failed: %s\n", what, h ? gaia_vbd_last_error(h) : gaia_vbd_last_global_error());
    return 1;
}

// writeOutputs (BasePhysicsFramework.cpp:442-506)
int write_outputs(gaia_vbd* h, const std::string& out, int frame, const OutputParams& o) {
    const std::string num = frame_name(frame);
    if (o.outputExt == "bin") {
        if (frame == 0) {
            make_dir(out + "/TemplateMesh");
            if (gaia_vbd_write_ply(h, (out + "/TemplateMesh/TemplateMesh.ply").c_str(), 0, 1)) return fail(h, "write");
        }
        if (gaia_vbd_write_binary(h, (out + "/A" + num + ".bin").c_str())) return fail(h, "write");
        if (!(frame % o.binaryModeVisualizationSteps))
            if (gaia_vbd_write_ply(h, (out + "/A" + num + ".ply").c_str(), o.saveAllModelsTogether, o.saveAllModelsTogether))
                return fail(h, "write");
    } else if (o.outputExt == "ply") {
        if (gaia_vbd_write_ply(h, (out + "/A" + num + ".ply").c_str(), o.saveAllModelsTogether, o.saveAllModelsTogether))
            return fail(h, "write");
    } else if (o.outputExt != "obj") {  // "obj" writes no frame in the reference either
        std::fprintf(stderr, "[Error] Unsupported output EXT name: %s\n", o.outputExt.c_str());
        return 0;
    }
    if (o.outputRecoveryState && !(frame % o.outputRecoveryStateStep))
        if (gaia_vbd_save_state(h, (out + "/RecoveryStates/A" + num + ".json").c_str(), o.outputRecoveryStateBinary))
            return fail(h, "save state");
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s Models.json Parameters.json outFolder [-R repoRoot] [-r recoveryState.json]\n",
                     argv[0]);
        return 2;
    }
    std::string models = argv[1], params = argv[2], out = argv[3];
    std::string root, recovery;
    for (int i = 4; i + 1 < argc; i += 2) {
        if (!std::strcmp(argv[i], "-R") || !std::strcmp(argv[i], "--repoRoot")) root = argv[i + 1];
        else if (!std::strcmp(argv[i], "-r") || !std::strcmp(argv[i], "--recoveryState")) recovery = argv[i + 1];
        else {
            std::fprintf(stderr, "unknown option %s\n", argv[i]);
            return 2;
        }
    }
    if (!root.empty()) {
        using gaia::jsonio::replace_all;
        models = replace_all(models, "${REPO_ROOT}", root);
        params = replace_all(params, "${REPO_ROOT}", root);
        out = replace_all(out, "${REPO_ROOT}", root);
    }
    OutputParams o;
    try {
        gaia::json::Value P = gaia::json::parse(gaia::jsonio::read_file(params));
        if (const gaia::json::Value* pp = P.find("PhysicsParams")) {
            using gaia::jsonio::get;
            get(*pp, "numFrames", o.numFrames);
            get(*pp, "saveOutputs", o.saveOutputs);
            get(*pp, "saveAllModelsTogether", o.saveAllModelsTogether);
            get(*pp, "outputExt", o.outputExt);
            get(*pp, "binaryModeVisualizationSteps", o.binaryModeVisualizationSteps);
            get(*pp, "outputRecoveryState", o.outputRecoveryState);
            get(*pp, "outputRecoveryStateStep", o.outputRecoveryStateStep);
            get(*pp, "outputRecoveryStateBinary", o.outputRecoveryStateBinary);
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "cannot read %s: %s\n", params.c_str(), e.what());
        return 1;
    }
    if (out == "noOutput") o.saveOutputs = false;
    if (o.binaryModeVisualizationSteps <= 0) o.binaryModeVisualizationSteps = 1;
    if (o.outputRecoveryStateStep <= 0) o.outputRecoveryStateStep = 1;

    gaia_vbd* h = nullptr;
    if (gaia_vbd_create(models.c_str(), params.c_str(), root.empty() ? nullptr : root.c_str(), &h))
        return fail(nullptr, "create");
    int frame = 0;
    if (!recovery.empty()) {
        if (gaia_vbd_load_state(h, recovery.c_str())) return fail(h, "recoverFromState");
        try {
            gaia::json::Value S = gaia::json::parse(gaia::jsonio::read_file(recovery));
            gaia::jsonio::get(S, "frameId", frame);
        } catch (const std::exception&) {
        }
        if (frame < 0) frame = 0;
    }
    // handleInput and setUpOutputFolders (BasePhysicsFramework.cpp:414-440), then frame 0
    make_dir(out);
    if (o.outputRecoveryState) make_dir(out + "/RecoveryStates");
    if (write_outputs(h, out, frame, o)) return 1;
    const auto t0 = std::chrono::steady_clock::now();
    int steps = 0;
    while (frame < o.numFrames) {
        if (gaia_vbd_run_step(h, 1)) return fail(h, "runStep");
        ++frame;
        ++steps;
        if (o.saveOutputs && write_outputs(h, out, frame, o)) return 1;
    }
    if (gaia_vbd_synchronize(h)) return fail(h, "synchronize");
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("%d frames in %.3f s (%.2f frames/s)\n", steps, s, steps > 0 ? steps / s : 0.0);
    gaia_vbd_destroy(h);
    return 0;
}
