// Scene-major sweep on a thread-block cluster with the scene in distributed shared memory.
//
// For scenes small enough to live on-chip (the CPU-runnable 10^3 drop: 1000 vertices,
// 14.6k incidences), a cluster of C blocks (C <= 16, one per SM) takes one scene at a
// time from a work counter and runs all its iterations without touching global memory
// for positions or records:
//   * every block holds a copy of all the scene's states (active and fixed vertices) in
//     its shared memory, and the incidence records of the vertices it owns: of each
//     color, the block of rank r owns a contiguous chunk, whose records are one
//     contiguous range of the record arrays;
//   * per color, each block solves its chunk (L lanes per vertex, neighbour states and
//     records from its own shared memory) and writes every new state into all C copies:
//     its own, and the other blocks' through distributed shared memory;
//   * a cluster barrier (release / acquire at cluster scope) separates colors, so the
//     next color reads the updated states from the local copy;
//   * after the last iteration each block writes its owned vertices back to global memory.
// Per color the critical path is shared-memory loads, the element arithmetic, the lane
// reduction, the 3x3 solve, C remote stores and one cluster barrier: no launch and no
// L2 round trip between colors. The per-vertex arithmetic is the solve kernels' (same
// incidence function, lane reduction and tail), so the results equal the merged and the
// single-block scene sweeps' for the same lanes per vertex.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_kernels.cuh"

namespace gaia {
namespace dev {

namespace cg = cooperative_groups;

constexpr int kClusterMaxColors = 64;  // colors per scene that the per-block color table holds

// One incidence record in shared memory.
template <typename R>
struct RecS;
template <>
struct RecS<float> {
    RecRaw<float> r;
    __device__ __forceinline__ void from_global(const int4* n, const R4<float>* a, const R4<float>* b, const float*,
                                                int i) {
        r.n = n[i];
        r.a = reinterpret_cast<const float4*>(a)[i];
        r.b = reinterpret_cast<const float4*>(b)[i];
    }
};
template <>
struct RecS<double> {
    RecRaw<double> r;
    __device__ __forceinline__ void from_global(const int4* n, const R4<double>* a, const R4<double>* b,
                                                const double* c, int i) {
        r.n = n[i];
        const double2* pa = reinterpret_cast<const double2*>(a + i);
        const double2* pb = reinterpret_cast<const double2*>(b + i);
        r.a0 = pa[0];
        r.a1 = pa[1];
        r.b0 = pb[0];
        r.b1 = pb[1];
        r.c = c[i];
    }
};

struct ClusterScenes {
    const int2* colors;        // slot ranges of the scenes' colors (scene-major slot layout)
    const int32_t* scene_ofs;  // colors of scene m: colors[scene_ofs[m] .. scene_ofs[m + 1])
    const int32_t* scene_order;
    const int4* scene_slots;   // per scene: active slots [x, y), fixed slots [z, w)
    int32_t nscenes, iterations, friction_start;
    int32_t pos_cap;           // states each block's shared copy holds
    int32_t rec_cap;           // records each block holds
};

// A state broadcast from lane src of the warp (every field of the trait's state type).
template <typename ST>
__device__ __forceinline__ typename ST::U shfl_state(typename ST::U u, int src) {
    constexpr int kWords = int(sizeof(typename ST::U) / 4);
    static_assert(sizeof(typename ST::U) % 4 == 0, "state of whole 32-bit words");
    uint32_t w[kWords];
    memcpy(w, &u, sizeof(u));
#pragma unroll
    for (int k = 0; k < kWords; ++k) w[k] = __shfl_sync(0xffffffffu, w[k], src);
    memcpy(&u, w, sizeof(u));
    return u;
}

template <int L, typename ST, typename R>
__global__ void __launch_bounds__(256) k_sweep_cluster(Ptrs<ST, R> P, Consts<R> c, ClusterScenes S, int32_t* work) {
    using U = typename ST::U;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = int(cluster.block_rank());
    const int C = int(cluster.num_blocks());
    extern __shared__ __align__(16) unsigned char smem[];
    U* spos = reinterpret_cast<U*>(smem);
    RecS<R>* srec = reinterpret_cast<RecS<R>*>(smem + sizeof(U) * size_t(S.pos_cap));
    __shared__ int s_scene;
    __shared__ int s_rec_base[kClusterMaxColors + 1];
    const int groups = int(blockDim.x) / L;
    const int g = int(threadIdx.x) / L;
    const int lane = int(threadIdx.x) & (L - 1);
    for (;;) {
        // rank 0 takes the next scene and hands it to every block of the cluster
        if (rank == 0 && threadIdx.x == 0) {
            const int k = atomicAdd(work, 1);
            for (int r = 0; r < C; ++r) *cluster.map_shared_rank(&s_scene, r) = k;
        }
        cluster.sync();
        const int k = s_scene;
        if (k >= S.nscenes) return;
        const int sc = S.scene_order[k];
        const int c0 = S.scene_ofs[sc], c1 = S.scene_ofs[sc + 1];
        const int4 sl = S.scene_slots[sc];
        const int na = sl.y - sl.x;
        auto loc = [&](int s) { return s < sl.y ? s - sl.x : na + (s - sl.z); };
        // this block's chunk of color ci: [beg, end)
        auto chunk = [&](int ci, int& beg, int& end) {
            const int2 rg = S.colors[ci];
            const int per = (rg.y - rg.x + C - 1) / C;
            beg = min(rg.y, rg.x + rank * per);
            end = min(rg.y, beg + per);
        };
        if (threadIdx.x == 0) {
            int base = 0;
            for (int ci = c0; ci < c1; ++ci) {
                int beg, end;
                chunk(ci, beg, end);
                s_rec_base[ci - c0] = base;
                base += P.inc_ofs[end] - P.inc_ofs[beg];
            }
            s_rec_base[c1 - c0] = base;
        }
        // stage: all the scene's states, this block's records
        const int nloc = na + (sl.w - sl.z);
        for (int i = threadIdx.x; i < nloc; i += blockDim.x) spos[i] = P.u[i < na ? sl.x + i : sl.z + (i - na)];
        __syncthreads();
        for (int ci = c0; ci < c1; ++ci) {
            int beg, end;
            chunk(ci, beg, end);
            const int r0 = P.inc_ofs[beg], nr = P.inc_ofs[end] - r0, b = s_rec_base[ci - c0];
            for (int i = threadIdx.x; i < nr; i += blockDim.x)
                srec[b + i].from_global(P.rec_n, P.rec_a, P.rec_b, P.rec_c, r0 + i);
        }
        cluster.sync();  // every copy staged before any block writes into another's
        for (int it = 0; it < S.iterations; ++it) {
            const int friction = it >= S.friction_start ? 1 : 0;
            for (int ci = c0; ci < c1; ++ci) {
                int beg, end;
                chunk(ci, beg, end);
                const int rb = s_rec_base[ci - c0], r0 = P.inc_ofs[beg];
                for (int base = beg; base < end; base += groups) {
                    const int v = base + g;
                    const bool valid = v < end;
                    Acc<R> acc = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                    U uo{};
                    MeshMat<R> mat;
                    if (valid) {
                        if (lane == 0) prefetch_tail(P, v);
                        mat = P.mats[P.slot_mesh[v]];
                        uo = spos[v - sl.x];
                        const U uon = ST::nb(uo);
                        const int e = rb + P.inc_ofs[v + 1] - r0;
                        for (int r = rb + P.inc_ofs[v] - r0 + lane; r < e; r += L) {
                            const RecRaw<R>& rec = srec[r].r;
                            const U q0 = ST::nb(spos[loc(rec.n.x)]), q1 = ST::nb(spos[loc(rec.n.y)]),
                                    q2 = ST::nb(spos[loc(rec.n.z)]);
                            R m0[3], m1[3], m2[3];
                            rec.rows(m0, m1, m2);
                            R e0[3], e1[3], e2[3];
                            ST::diff(q0, uon, e0);
                            ST::diff(q1, uon, e1);
                            ST::diff(q2, uon, e2);
                            incidence<R>(e0, e1, e2, m0, m1, m2, mat.mu, mat.lmbd, acc);
                        }
                    }
                    reduce_group<L, R>(acc);
                    // lane 0 solves; the group's lanes then write the new state into the C
                    // copies, one remote store each, instead of lane 0 writing all of them
                    U un{};
                    int moved = 0;
                    if (valid && lane == 0)
                        moved = vertex_tail<ST, R, false>(P, c, v, uo, mat, acc, friction, nullptr, beg, end, &un) ? 1 : 0;
                    const int src = int(threadIdx.x) & ~(L - 1) & 31;
                    moved = __shfl_sync(0xffffffffu, moved, src);
                    un = shfl_state<ST>(un, src);
                    if (valid && moved) {
                        const int lv = v - sl.x;
                        for (int r = lane; r < C; r += L) *cluster.map_shared_rank(&spos[lv], r) = un;
                    }
                }
                cluster.sync();  // this color's states in every copy before the next color
            }
        }
        // the owned vertices back to global memory
        for (int ci = c0; ci < c1; ++ci) {
            int beg, end;
            chunk(ci, beg, end);
            for (int v = beg + int(threadIdx.x); v < end; v += blockDim.x) P.u[v] = spos[v - sl.x];
        }
        cluster.sync();  // no block stages the next scene while another still reads this one
    }
}

}  // namespace dev
}  // namespace gaia
