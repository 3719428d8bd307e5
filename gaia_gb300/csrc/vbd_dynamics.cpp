// Command-line runner with the reference's VBDDynamics interface (Simulator/VBDDynamics/
// main.cpp:7-32), on the C++ facade of include/gaia_vbd.hpp:
//
//   vbd_dynamics Models.json Parameters.json outFolder [-R repoRoot] [-r recoveryState.json]
//
// loadRunningparameters ("${REPO_ROOT}" in the three paths replaced by -R, as
// InputHandlerVBD::handleInput does), initialize, recoverFromState when -r is given,
// saveOutputs cleared when outFolder is "noOutput", then simulate: frame frameId is written
// before the loop (whatever saveOutputs says, as in the reference) and the frames up to
// numFrames after it.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>

#include "gaia_vbd.hpp"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s Models.json Parameters.json outFolder [-R repoRoot] [-r recoveryState.json]\n",
                     argv[0]);
        return 2;
    }
    std::string root, recovery;
    for (int i = 4; i < argc; i += 2) {
        if (i + 1 >= argc) {
            std::fprintf(stderr, "option %s needs a value\n", argv[i]);
            return 2;
        }
        if (!std::strcmp(argv[i], "-R") || !std::strcmp(argv[i], "--repoRoot")) root = argv[i + 1];
        else if (!std::strcmp(argv[i], "-r") || !std::strcmp(argv[i], "--recoveryState")) recovery = argv[i + 1];
        else {
            std::fprintf(stderr, "unknown option %s\n", argv[i]);
            return 2;
        }
    }
    try {
        gaia::VBDPhysics physics;
        physics.loadRunningparameters(argv[1], argv[2], argv[3], root);
        physics.initialize();
        if (!recovery.empty()) physics.recoverFromState(recovery);
        if (physics.outputFolder == "noOutput") physics.setSaveOutputs(false);
        const auto t0 = std::chrono::steady_clock::now();
        const int steps = physics.simulate();
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("%d frames in %.3f s (%.2f frames/s)\n", steps, s, steps > 0 ? steps / s : 0.0);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
