// Stand-in for the reference's MeshFrame tet-mesh header (an empty submodule in the
// reference tree) for the checker build of its coloring code: GraphColoring/Graph.h only
// names these types in typedefs, and mcs.cpp / gready.cpp / ColoringAlgorithms.cpp do not
// use them. TEST INFRASTRUCTURE ONLY.
#pragma once
#include <array>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

namespace MF {
namespace TetMesh {
struct TMeshStaticF {};
template <typename M>
struct TIterators {};
}  // namespace TetMesh
}  // namespace MF
