// Stand-in for the reference's MeshFrame triangle-mesh header (see TMeshStaticLibHeaders.h).
// TEST INFRASTRUCTURE ONLY.
#pragma once

namespace MF {
namespace TriMesh {
struct TriMeshStaticF {};
struct TriMeshStaticIteratorF {};
}  // namespace TriMesh
}  // namespace MF
