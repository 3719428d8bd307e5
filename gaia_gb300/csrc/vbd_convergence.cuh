// Deterministic FP64 convergence reduction of the VBD step: total energy (Neo-Hookean
// elastic with the rest energy removed, plus inertia) and the average norm of the
// per-vertex force (material with damping, plus inertia), the quantities of the
// reference's evaluateConvergenceGPU / evaluateMeritEnergyGPU (VBD/VBDPhysics.cpp:3459-3556,
// 3851-3871; VBDPhysicsCompute.cu:1775-1810; VBD_BaseMaterial.h:223-241).
//
// Everything is evaluated in FP64 from the FP64 rest shape, whatever the engine's state
// precision. Each pass writes one partial sum per block (a fixed shuffle tree inside the
// block), and one finishing block adds the partials in index order: the result depends
// only on the data and the launch shape, so repeated evaluations of one state are
// bit-identical (no floating-point atomics).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_state.cuh"

namespace gaia {
namespace dev {

constexpr int kConvThreads = 256;

struct ConvData {
    const int4* tet_slots;     // 4 slots per tet
    const double* tet_dminv;   // 9 per tet, column-major
    const double* tet_vol;     // rest volume per tet
    const int32_t* tet_mesh;   // mesh of each tet
    const double4* mesh_mat;   // per mesh: mu, lambda, dampingHydrostatic, dampingDeviatoric
    const int32_t* slot_mesh;  // mesh of each slot
    const double* slot_mass;   // FP64 lumped mass of each slot (the states hold it in their own precision)
    const int32_t* inc_ofs;    // per active slot: its incidences [inc_ofs[s], inc_ofs[s + 1])
    const int32_t* inc_tet;    // tet of each incidence
    const int8_t* inc_ord;     // the slot's vertex order in that tet
    int32_t ntet, nactive, nslots;
    double dt2inv, inv_dt;
};

// Sum of v over the block in a fixed order; the total is valid in thread 0.
__device__ __forceinline__ double block_sum_fixed(double v) {
    __shared__ double part[kConvThreads / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) part[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < int(blockDim.x >> 5); ++i) s += part[i];
    __syncthreads();
    return s;
}

template <typename ST>
__device__ __forceinline__ void conv_pos(const typename ST::U* u, const float4* rest, int s, double* p) {
    ST::to_d(u[s], p);
    const float4 X = rest[s];
    p[0] += double(X.x);
    p[1] += double(X.y);
    p[2] += double(X.z);
}

// F = Ds DmInv of tet t (column-major), its determinant and cofactor dJ/dF (column-major).
template <typename ST>
__device__ __forceinline__ void conv_tet_F(const typename ST::U* u, const float4* rest, const ConvData& D, int t,
                                           double* F, double& J, double* cof) {
    const int4 sv = D.tet_slots[t];
    double p0[3], p[3];
    conv_pos<ST>(u, rest, sv.x, p0);
    double Ds[9];
    const int o[3] = {sv.y, sv.z, sv.w};
    for (int c = 0; c < 3; ++c) {
        conv_pos<ST>(u, rest, o[c], p);
        for (int r = 0; r < 3; ++r) Ds[3 * c + r] = p[r] - p0[r];
    }
    const double* Di = D.tet_dminv + 9 * size_t(t);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) F[3 * c + r] = Ds[r] * Di[3 * c] + Ds[3 + r] * Di[3 * c + 1] + Ds[6 + r] * Di[3 * c + 2];
    auto f = [&](int r, int c) { return F[3 * c + r]; };
    cof[0] = f(1, 1) * f(2, 2) - f(1, 2) * f(2, 1);
    cof[1] = f(0, 2) * f(2, 1) - f(0, 1) * f(2, 2);
    cof[2] = f(0, 1) * f(1, 2) - f(0, 2) * f(1, 1);
    cof[3] = f(1, 2) * f(2, 0) - f(1, 0) * f(2, 2);
    cof[4] = f(0, 0) * f(2, 2) - f(0, 2) * f(2, 0);
    cof[5] = f(0, 2) * f(1, 0) - f(0, 0) * f(1, 2);
    cof[6] = f(1, 0) * f(2, 1) - f(1, 1) * f(2, 0);
    cof[7] = f(0, 1) * f(2, 0) - f(0, 0) * f(2, 1);
    cof[8] = f(0, 0) * f(1, 1) - f(0, 1) * f(1, 0);
    J = f(0, 0) * cof[0] + f(1, 0) * cof[1] + f(2, 0) * cof[2];
}

// Pass 1a: elastic energy of every tet, one partial per block.
template <typename ST>
__global__ void __launch_bounds__(kConvThreads) k_conv_tets(const typename ST::U* u, const float4* rest, ConvData D,
                                                            double* part) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (t < D.ntet) {
        double F[9], cof[9], J;
        conv_tet_F<ST>(u, rest, D, t, F, J, cof);
        double n2 = 0.0;
        for (int i = 0; i < 9; ++i) n2 += F[i] * F[i];
        const double4 m = D.mesh_mat[D.tet_mesh[t]];
        const double a = 1.0 + m.x / m.y, A = D.tet_vol[t];
        e = A * (m.x * 0.5 * (n2 - 3.0) + m.y * 0.5 * (J - a) * (J - a)) - 0.5 * A * m.y * (1.0 - a) * (1.0 - a);
    }
    const double s = block_sum_fixed(e);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Pass 1b: per slot, the inertia energy (all slots) and the norm of the force (material
// with damping, plus inertia; zero for fixed slots), one partial of each per block.
template <typename ST>
__global__ void __launch_bounds__(kConvThreads) k_conv_verts(const typename ST::U* u, const typename ST::U* y,
                                                             const typename ST::U* xprev, const float4* rest,
                                                             ConvData D, double* part_inertia, double* part_fnorm) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double ei = 0.0, fn = 0.0;
    if (s < D.nslots) {
        double x[3], yy[3];
        ST::to_d(u[s], x);
        ST::to_d(y[s], yy);
        const double mass = D.slot_mass[s];
        const double w = mass * D.dt2inv;
        const double d0 = yy[0] - x[0], d1 = yy[1] - x[1], d2 = yy[2] - x[2];
        ei = 0.5 * w * (d0 * d0 + d1 * d1 + d2 * d2);
        if (s < D.nactive) {
            double f[3] = {w * d0, w * d1, w * d2};
            double xp[3];
            ST::to_d(xprev[s], xp);
            const double disp[3] = {x[0] - xp[0], x[1] - xp[1], x[2] - xp[2]};
            const double4 m = D.mesh_mat[D.slot_mesh[s]];
            const double a = 1.0 + m.x / m.y;
            for (int k = D.inc_ofs[s]; k < D.inc_ofs[s + 1]; ++k) {
                const int t = D.inc_tet[k];
                const int ord = D.inc_ord[k];
                double F[9], cof[9], J;
                conv_tet_F<ST>(u, rest, D, t, F, J, cof);
                const double* Di = D.tet_dminv + 9 * size_t(t);
                double mv[3];
                for (int c = 0; c < 3; ++c)
                    mv[c] = ord == 0 ? -(Di[3 * c] + Di[3 * c + 1] + Di[3 * c + 2]) : Di[3 * c + ord - 1];
                const double A = D.tet_vol[t];
                double g[3], P[3];
                for (int r = 0; r < 3; ++r) {
                    g[r] = cof[r] * mv[0] + cof[3 + r] * mv[1] + cof[6 + r] * mv[2];
                    P[r] = F[r] * mv[0] + F[3 + r] * mv[1] + F[6 + r] * mv[2];
                }
                // -dE/dx_o = -A (mu F + lambda (J - a) cof F) m_o
                for (int r = 0; r < 3; ++r) f[r] -= A * (m.x * P[r] + m.y * (J - a) * g[r]);
                if (m.z > 0.0 || m.w > 0.0) {
                    // damping (k_h lambda A g g^T + k_d mu A |m|^2 I) / dt times the displacement
                    const double gd = g[0] * disp[0] + g[1] * disp[1] + g[2] * disp[2];
                    const double S = m.x * A * (mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]);
                    for (int r = 0; r < 3; ++r) f[r] -= (m.z * m.y * A * g[r] * gd + m.w * S * disp[r]) * D.inv_dt;
                }
            }
            fn = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
        }
    }
    const double si = block_sum_fixed(ei);
    const double sf = block_sum_fixed(fn);
    if (threadIdx.x == 0) {
        part_inertia[blockIdx.x] = si;
        part_fnorm[blockIdx.x] = sf;
    }
}

// Pass 2: one block adds each quantity's partials in index order and writes one record
// (energy, inertia, elastic, average force norm) to out[4 * k], k = *counter (then
// incremented) when a counter is given, else k = 0; records beyond cap are dropped.
static __global__ void __launch_bounds__(kConvThreads) k_conv_finish(const double* part_elastic, int nb_t,
                                                              const double* part_inertia, const double* part_fnorm,
                                                              int nb_v, double inv_nslots, double* out,
                                                              int32_t* counter, int32_t cap) {
    double e = 0.0, i = 0.0, f = 0.0;
    for (int k = threadIdx.x; k < nb_t; k += blockDim.x) e += part_elastic[k];
    for (int k = threadIdx.x; k < nb_v; k += blockDim.x) {
        i += part_inertia[k];
        f += part_fnorm[k];
    }
    e = block_sum_fixed(e);
    i = block_sum_fixed(i);
    f = block_sum_fixed(f);
    if (threadIdx.x == 0) {
        int k = 0;
        if (counter) {
            k = *counter;
            *counter = k + 1;
        }
        if (k < cap) {
            double* o = out + 4 * size_t(k);
            o[0] = e + i;
            o[1] = i;
            o[2] = e;
            o[3] = f * inv_nslots;
        }
    }
}

}  // namespace dev
}  // namespace gaia
