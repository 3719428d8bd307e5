// Checker build of the reference's own moving-point / moving-triangle CCD test —
// TEST INFRASTRUCTURE ONLY. Compiled by `make -C oracle ref` against the
// reference tree (CollisionDetector/CCDSolver.h and the CyCodeBase headers it
// includes), where that tree is present, into oracle/_ref/libccd_ref.so. The
// tests compare the oracle's FP32 restatement (tet_contact.cpp) with it bit for bit.
#include <cstdint>

#include "CCDSolver.h"

extern "C" int32_t ref_ccd_tri_point(const float* x0, const float* x1, const float* p0, const float* p1, float* tt,
                                     float* bary) {
    cy::Vec3<float> x[2][3];
    cy::Vec3<float> p[2];
    for (int i = 0; i < 3; ++i) {
        x[0][i] = cy::Vec3<float>(x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]);
        x[1][i] = cy::Vec3<float>(x1[3 * i], x1[3 * i + 1], x1[3 * i + 2]);
    }
    p[0] = cy::Vec3<float>(p0[0], p0[1], p0[2]);
    p[1] = cy::Vec3<float>(p1[0], p1[1], p1[2]);
    float t = -1.0f;
    cy::Vec3<float> b(0.0f, 0.0f, 0.0f);
    const bool hit = cy::IntersectContinuousTriPoint<float>(t, x, p, b);
    *tt = t;
    bary[0] = b.x;
    bary[1] = b.y;
    bary[2] = b.z;
    return hit ? 1 : 0;
}
