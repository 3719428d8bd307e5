// Vertex coloring of a tet mesh on the GPU (an option next to the reference's MCS and
// OrderedGreedy, GraphColoring/mcs.cpp, gready.cpp, which this library reproduces on the
// host): the vertex graph (every pair of vertices sharing a tet) is built with a radix
// sort of the tets' directed vertex pairs, then colored by Jones-Plassmann rounds
// (Jones & Plassmann, "A parallel graph coloring heuristic", SIAM J. Sci. Comput. 1993):
// every uncolored vertex whose hashed priority is the largest among its uncolored
// neighbours takes the lowest color its colored neighbours do not use. Vertices colored
// in one round are pairwise non-adjacent, so the result does not depend on thread order;
// it depends only on the mesh and the seed.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "gaia_vbd.h"

namespace gaia {
namespace jp {
namespace {

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
#define JP_CUDA(x) check((x), #x)

template <typename T>
struct Dev {
    T* p = nullptr;
    explicit Dev(size_t n) { JP_CUDA(cudaMalloc(&p, (n ? n : 1) * sizeof(T))); }
    ~Dev() { cudaFree(p); }
    Dev(const Dev&) = delete;
    Dev& operator=(const Dev&) = delete;
};

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

__global__ void k_pairs(const int4* tets, int32_t ntet, int32_t nv, unsigned long long* keys, int* bad) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntet) return;
    const int4 q = tets[t];
    const int v[4] = {q.x, q.y, q.z, q.w};
    int k = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (v[i] < 0 || v[i] >= nv) atomicOr(bad, 1);
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (i != j) {
                const bool ok = v[i] != v[j] && v[i] >= 0 && v[i] < nv && v[j] >= 0 && v[j] < nv;
                keys[12 * t + k++] = ok ? (static_cast<unsigned long long>(v[i]) << 32) | static_cast<unsigned>(v[j])
                                        : ~0ull;
            }
    }
}

// CSR from sorted (a << 32 | b) keys: first occurrence of each distinct key goes in,
// per-vertex counts by the first key of each vertex.
__global__ void k_mark_unique(const unsigned long long* keys, int64_t n, int32_t* flag) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = keys[i] != ~0ull && (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_scatter_adj(const unsigned long long* keys, const int32_t* flag, const int32_t* pos, int64_t n,
                              int32_t* adj, int32_t* deg) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const int32_t a = int32_t(keys[i] >> 32);
    adj[pos[i]] = int32_t(keys[i] & 0xffffffffull);
    atomicAdd(&deg[a], 1);
}

__device__ __forceinline__ uint32_t prio(uint32_t v, uint32_t seed) {
    // a 32-bit integer mixer (the finalizer of MurmurHash3)
    uint32_t h = v ^ (seed * 0x9e3779b9u);
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// One round. state[v] = -1 while uncolored, else (round << 16) | color. A neighbour colored
// in this same round counts as uncolored (it has the higher priority, so v waits), which
// makes the round's outcome independent of the order in which threads see the writes.
__global__ void k_jp_round(const int32_t* ofs, const int32_t* adj, int32_t nv, uint32_t seed, int32_t round,
                           int32_t* state, int32_t* remaining) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv || state[v] >= 0) return;
    const uint32_t pv = prio(uint32_t(v), seed);
    const int b = ofs[v], e = ofs[v + 1];
    for (int k = b; k < e; ++k) {
        const int u = adj[k];
        const int su = state[u];
        if (su >= 0 && (su >> 16) != round) continue;
        const uint32_t pu = prio(uint32_t(u), seed);
        if (pu > pv || (pu == pv && u > v)) {
            atomicAdd(remaining, 1);
            return;
        }
    }
    // lowest color unused by the neighbours colored in earlier rounds: 64 colors per pass
    for (int base = 0;; base += 64) {
        unsigned long long used = 0;
        for (int k = b; k < e; ++k) {
            const int su = state[adj[k]];
            if (su < 0 || (su >> 16) == round) continue;
            const int c = (su & 0xffff) - base;
            if (c >= 0 && c < 64) used |= 1ull << c;
        }
        if (~used) {
            state[v] = (round << 16) | (base + __ffsll(static_cast<long long>(~used)) - 1);
            return;
        }
    }
}

__global__ void k_jp_colors(const int32_t* state, int32_t nv, int32_t* colors) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv) colors[v] = state[v] & 0xffff;
}

}  // namespace
}  // namespace jp
}  // namespace gaia

extern "C" int32_t gaia_vbd_color_gpu(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors, uint32_t seed) {
    using namespace gaia::jp;
    if (nv <= 0 || ntet < 0 || (!tets && ntet) || !colors) return -1;
    try {
        const int64_t np = 12 * int64_t(ntet);
        Dev<int4> d_tets(ntet);
        Dev<unsigned long long> keys(np), sorted(np);
        Dev<int32_t> flag(np), pos(np), ofs(int64_t(nv) + 1), deg(nv), col(nv), rem(1);
        Dev<int> bad(1);
        JP_CUDA(cudaMemset(bad.p, 0, sizeof(int)));
        if (ntet) JP_CUDA(cudaMemcpy(d_tets.p, tets, sizeof(int4) * size_t(ntet), cudaMemcpyHostToDevice));
        k_pairs<<<blocks(ntet, 256), 256>>>(d_tets.p, ntet, nv, keys.p, bad.p);
        size_t tb = 0;
        JP_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, keys.p, sorted.p, np));
        size_t sb = 0;
        JP_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb, flag.p, pos.p, np));
        size_t sb2 = 0;
        JP_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb2, deg.p, ofs.p, int64_t(nv) + 1));
        Dev<char> tmp(std::max(tb, std::max(sb, sb2)));
        JP_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, tb, keys.p, sorted.p, np));
        k_mark_unique<<<blocks(np, 256), 256>>>(sorted.p, np, flag.p);
        JP_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, flag.p, pos.p, np));
        int32_t last_pos = 0, last_flag = 0;
        if (np) {
            JP_CUDA(cudaMemcpy(&last_pos, pos.p + np - 1, sizeof(int32_t), cudaMemcpyDeviceToHost));
            JP_CUDA(cudaMemcpy(&last_flag, flag.p + np - 1, sizeof(int32_t), cudaMemcpyDeviceToHost));
        }
        Dev<int32_t> adj(int64_t(last_pos) + last_flag);
        JP_CUDA(cudaMemset(deg.p, 0, sizeof(int32_t) * size_t(nv)));
        k_scatter_adj<<<blocks(np, 256), 256>>>(sorted.p, flag.p, pos.p, np, adj.p, deg.p);
        // ofs = exclusive sum of deg over nv + 1 entries (the last reads one past deg: use
        // a zero-padded copy)
        Dev<int32_t> deg1(int64_t(nv) + 1);
        JP_CUDA(cudaMemset(deg1.p, 0, sizeof(int32_t) * (size_t(nv) + 1)));
        JP_CUDA(cudaMemcpy(deg1.p, deg.p, sizeof(int32_t) * size_t(nv), cudaMemcpyDeviceToDevice));
        JP_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb2, deg1.p, ofs.p, int64_t(nv) + 1));
        int hbad = 0;
        JP_CUDA(cudaMemcpy(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (hbad) throw std::invalid_argument("tet references vertex out of range");
        JP_CUDA(cudaMemset(col.p, 0xff, sizeof(int32_t) * size_t(nv)));
        int32_t remaining = nv;
        for (int32_t round = 0; remaining > 0; ++round) {
            // every round colors at least the uncolored vertex of highest priority
            if (round >= 32767) throw std::runtime_error("Jones-Plassmann coloring did not finish");
            JP_CUDA(cudaMemset(rem.p, 0, sizeof(int32_t)));
            k_jp_round<<<blocks(nv, 256), 256>>>(ofs.p, adj.p, nv, seed, round, col.p, rem.p);
            JP_CUDA(cudaMemcpy(&remaining, rem.p, sizeof(int32_t), cudaMemcpyDeviceToHost));
        }
        Dev<int32_t> out(nv);
        k_jp_colors<<<blocks(nv, 256), 256>>>(col.p, nv, out.p);
        JP_CUDA(cudaMemcpy(colors, out.p, sizeof(int32_t) * size_t(nv), cudaMemcpyDeviceToHost));
        int32_t nc = 0;
        for (int32_t i = 0; i < nv; ++i) nc = colors[i] + 1 > nc ? colors[i] + 1 : nc;
        return nc;
    } catch (const std::exception&) {
        return -1;
    }
}
