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

// Output frames (IO/FileIO.cpp): the surface of every mesh as PLY (GAIA::saveAsPly,
// FileIO.cpp:8-49: ASCII, "%f" coordinates, triangle lists) or all vertex positions as raw
// FP32 xyz (writeAllToBinary, :52-117).
struct FrameMesh {
    std::vector<float> X;          // 3 per written vertex
    std::vector<int32_t> faces;    // 3 per face, indices into X
    std::string model_path;        // ObjectParams path (for the model-name suffix)
};
// all_in_one: one file with the meshes' vertices and faces concatenated (face indices
// offset); otherwise one file per mesh named as writeAllToPLY names it: tet meshes
// <dir>/<stem>_Model_<%06d mesh>[_<model stem>]<ext>, triangle meshes
// <dir>/<stem>Model_<%04d mesh>[_<model stem>]_<ext> (FileIO.cpp:119-251).
void write_frame_ply(const std::string& output, const std::vector<FrameMesh>& meshes, bool all_in_one,
                     bool add_model_name, bool tri_mesh_naming);
void write_frame_binary(const std::string& output, const std::vector<FrameMesh>& meshes);

}  // namespace gaia
