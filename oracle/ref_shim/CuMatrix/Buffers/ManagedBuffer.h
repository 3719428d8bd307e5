// Checker-build stand-in for the CuMatrix submodule's ManagedBuffer.h (the submodule is
// empty in the reference tree) — TEST INFRASTRUCTURE ONLY. The reference's device-data
// headers (TetMesh/TetMeshFEMGPU.h) include it for its host/device function qualifier;
// for a host build of the reference's GPU_CPU_INLINE_FUNC code it is plain `inline`.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>

#ifndef GPU_CPU_INLINE_FUNC
#define GPU_CPU_INLINE_FUNC inline
#endif
