// PhysicsState recovery files (Framework/BasePhysicsFramework.h:127-319): a JSON file
// with frameId, curTime and per-mesh positions and velocities, either inline ("text") or
// in two raw FP32 files next to it ("binary": <name>.pos / <name>.vel, meshes
// concatenated, xyz per vertex). Used by the tet and cloth handles' save/load calls.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gaia {

struct PhysicsStateFile {
    int frameId = -1;
    double curTime = 0.0;
    std::vector<std::vector<float>> position;  // per mesh, 3 floats per vertex
    std::vector<std::vector<float>> velocity;
};

void write_physics_state(const std::string& path, const PhysicsStateFile& s, bool binary);
// Throws std::runtime_error on unreadable or inconsistent files.
PhysicsStateFile read_physics_state(const std::string& path);

}  // namespace gaia
