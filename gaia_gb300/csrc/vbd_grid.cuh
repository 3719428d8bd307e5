// Merged-color persistent sweep on a co-resident grid with a bounded device-wide barrier.
//
// One cooperative launch per substep runs all its iterations over the merged colors (the
// color-major slot layout of the per-color launches): the grid's vertex groups stride over
// the color's slot range, then every block arrives at a grid barrier before the next color
// reads the updated states. The barrier replaces the kernel boundary between two color
// launches (VBDPhysics.cpp:879-953 launches one kernel per color): no launch, and the
// states written by other blocks are read through L2 (ldcg), since the reading SM's L1 may
// hold a line from an earlier color.
//
// The barrier is bounded: a block whose arrival count has not reached its target after
// spin_limit polls gives up, raises the abort flag (every waiting block then gives up at
// its next poll), counts a device timeout and returns. Blocks never wait on anything but
// that counter and flag, which every block of the co-resident grid reaches, so in a correct
// launch the barrier completes; the limit only turns a lost block into a status.
// The per-vertex arithmetic is k_solve's (same incidence loop and lane assignment, same
// reduction and tail), so for the same lanes per vertex the result equals the per-color
// launches' bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_kernels.cuh"

namespace gaia {
namespace dev {

struct GridSweep {
    const int2* colors;  // slot ranges of the merged colors, in sweep order
    int32_t ncolors, iterations, friction_start;
    uint32_t* bar;       // [0] arrivals (monotonic within a launch), [1] abort flag; zeroed before each launch
};

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Arrive and wait until `target` arrivals (this block's included) or give up: at most
// `limit` polls, or the abort flag raised by another block that gave up. Returns whether
// the barrier completed; every thread of the block gets the same answer.
__device__ __forceinline__ bool grid_barrier(uint32_t* bar, uint32_t target, int limit,
                                             unsigned long long* counters) {
    __shared__ int s_ok;
    __syncthreads();  // the block's state writes are done
    if (threadIdx.x == 0) {
        __threadfence();  // ... and visible device-wide before the arrival
        const uint32_t arrived = atomicAdd(bar, 1u) + 1u;
        int ok = arrived >= target ? 1 : 0;
        for (int i = 0; !ok && i < limit; ++i) {
            if (ld_acquire_gpu(bar) >= target) ok = 1;
            else if (ld_acquire_gpu(bar + 1)) break;
        }
        if (!ok) {
            atomicExch(bar + 1, 1u);
            atomicAdd(&counters[CNT_TIMEOUT], 1ull);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <int L, typename ST, typename R>
__global__ void __launch_bounds__(256) k_sweep_grid(Ptrs<ST, R> P, Consts<R> c, GridSweep G) {
    using U = typename ST::U;
    const int per_block = int(blockDim.x) / L;
    const int ngroups = int(gridDim.x) * per_block;
    const int gid = int(blockIdx.x) * per_block + int(threadIdx.x) / L;
    const int lane = int(threadIdx.x) & (L - 1);
    uint32_t target = 0;
    for (int it = 0; it < G.iterations; ++it) {
        const int friction = it >= G.friction_start ? 1 : 0;
        for (int ci = 0; ci < G.ncolors; ++ci) {
            const int2 rg = G.colors[ci];
            for (int base = rg.x; base < rg.y; base += ngroups) {
                const int v = base + gid;
                const bool valid = v < rg.y;
                Acc<R> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                U uo{};
                MeshMat<R> mat;
                if (valid) {
                    mat = P.mats[P.slot_mesh[v]];
                    const int r = P.inc_ofs[v] + lane, e = P.inc_ofs[v + 1];
                    RecRaw<R> cur;
                    if (r < e) cur.load_kept(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r);
                    if (lane == 0) prefetch_tail(P, v);
                    uo = ST::ldcg_own(P.u, v);
                    accumulate_records<L, ST, R, kStateGrid>(P, r, e, cur, uo, mat.mu, mat.lmbd, acc);
                }
                reduce_group<L, R>(acc);
                if (valid && lane == 0) vertex_tail<ST, R, false>(P, c, v, uo, mat, acc, friction, nullptr, rg.x, rg.y);
            }
            if (it + 1 == G.iterations && ci + 1 == G.ncolors) break;  // the kernel's end orders the last color
            target += gridDim.x;
            if (!grid_barrier(G.bar, target, c.spin_limit, P.counters)) return;
        }
    }
}

}  // namespace dev
}  // namespace gaia
