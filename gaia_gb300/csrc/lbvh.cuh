// Linear BVH on the GPU: 30-bit Morton codes of primitive box centres in the scene box,
// a CUB radix sort of (code, index) keys, Karras' parallel hierarchy ("Maximizing
// parallelism in the construction of BVHs, octrees and k-d trees", HPG 2012), a
// bottom-up refit in which the second thread to reach a node forms its box, and a
// stack traversal that visits every primitive whose box is within a radius of a point.
// Used by the cloth contact detector and the tet-mesh collision detector; each
// including translation unit gets its own copy (anonymous namespace).
#pragma once
#include <cub/cub.cuh>

#include <algorithm>
#include <stdexcept>
#include <string>

#include "cloth_dev.cuh"

namespace gaia {
namespace bvh {
namespace {

using cloth::ld3;
using cloth::v3;
using cloth::CC_STACK_OVERFLOW;

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
#define BVH_CUDA(x) ::gaia::bvh::check((x), #x)

template <typename T>
T* dalloc(size_t n, size_t& bytes) {
    T* p = nullptr;
    if (n == 0) n = 1;
    BVH_CUDA(cudaMalloc(&p, n * sizeof(T)));
    bytes += n * sizeof(T);
    return p;
}

inline int blocks(int n, int b) { return (n + b - 1) / b; }

// Order-preserving int encoding of a float (for atomicMin / atomicMax on floats).
__device__ __forceinline__ int ford(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fdec(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ unsigned int expand_bits(unsigned int v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Primitives: an int4 of vertex ids per primitive, of which the first k (2 = edge,
// 3 = triangle, 4 = tet) are used. swept != 0: the box also covers the same vertices at
// id + swept (a second set of positions in the same array, e.g. those at the start of a
// time step), which bounds the primitive's linear motion between the two.
struct Prims {
    const int4* idx;
    int k;
    int swept = 0;
};

__device__ __forceinline__ void prim_box(const Prims& P, const float4* xf, int p, float3& lo, float3& hi) {
    const int4 q = P.idx[p];
    const float3 a = ld3(xf, q.x), b = ld3(xf, q.y);
    lo = v3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z));
    hi = v3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z));
    if (P.k >= 3) {
        const float3 c = ld3(xf, q.z);
        lo = v3(fminf(lo.x, c.x), fminf(lo.y, c.y), fminf(lo.z, c.z));
        hi = v3(fmaxf(hi.x, c.x), fmaxf(hi.y, c.y), fmaxf(hi.z, c.z));
    }
    if (P.k >= 4) {
        const float3 d = ld3(xf, q.w);
        lo = v3(fminf(lo.x, d.x), fminf(lo.y, d.y), fminf(lo.z, d.z));
        hi = v3(fmaxf(hi.x, d.x), fmaxf(hi.y, d.y), fmaxf(hi.z, d.z));
    }
    if (P.swept) {
        const int ids[4] = {q.x, q.y, q.z, q.w};
        for (int j = 0; j < P.k; ++j) {
            const float3 e = ld3(xf, ids[j] + P.swept);
            lo = v3(fminf(lo.x, e.x), fminf(lo.y, e.y), fminf(lo.z, e.z));
            hi = v3(fmaxf(hi.x, e.x), fmaxf(hi.y, e.y), fmaxf(hi.z, e.z));
        }
    }
}

struct MinOp {
    __device__ __forceinline__ float operator()(float a, float b) const { return fminf(a, b); }
};

__global__ void k_centroid_bounds(Prims t, const float4* xf, int n, int* bounds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float3 lo = v3(3.4e38f, 3.4e38f, 3.4e38f), hi = v3(-3.4e38f, -3.4e38f, -3.4e38f);
    if (i < n) {
        float3 a, b;
        prim_box(t, xf, i, a, b);
        lo = v3(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z));
        hi = lo;
    }
    using BR = cub::BlockReduce<float, 256>;
    __shared__ typename BR::TempStorage tmp;
    float vals[6] = {lo.x, lo.y, lo.z, -hi.x, -hi.y, -hi.z};
    for (int k = 0; k < 6; ++k) {
        float m = BR(tmp).Reduce(vals[k], MinOp());
        __syncthreads();
        if (threadIdx.x == 0) atomicMin(&bounds[k], ford(m));
    }
}

__global__ void k_bounds_init(int* bounds) {
    if (threadIdx.x < 6) bounds[threadIdx.x] = ford(3.4e38f);
}

__global__ void k_morton(Prims t, const float4* xf, int n, const int* bounds, unsigned long long* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 a, b;
    prim_box(t, xf, i, a, b);
    const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned int code = 0;
    for (int k = 0; k < 3; ++k) {
        const float lo = fdec(bounds[k]), hi = -fdec(bounds[3 + k]);
        const float ext = hi - lo;
        float u = ext > 0.f ? (c[k] - lo) / ext : 0.f;
        u = fminf(fmaxf(u * 1024.f, 0.f), 1023.f);
        code |= expand_bits((unsigned int)u) << (2 - k);
    }
    keys[i] = (static_cast<unsigned long long>(code) << 32) | static_cast<unsigned int>(i);
}

__device__ __forceinline__ int delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    return __clzll(k[i] ^ k[j]);
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and k-d
// trees": internal node i spans a key range found by binary search; keys are unique.
__global__ void k_karras(const unsigned long long* keys, int n, int2* child, int* parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int s = lmax / 2; s >= 1; s /= 2)
        if (delta(keys, n, i, i + (l + s) * d) > dmin) l += s;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0, tt = l;
    do {
        tt = (tt + 1) >> 1;
        if (delta(keys, n, i, i + (s + tt) * d) > dnode) s += tt;
    } while (tt > 1);
    const int gamma = i + s * d + min(d, 0);
    const int left = (min(i, j) == gamma) ? (n - 1) + gamma : gamma;
    const int right = (max(i, j) == gamma + 1) ? (n - 1) + gamma + 1 : gamma + 1;
    child[i] = make_int2(left, right);
    parent[left] = i;
    parent[right] = i;
    if (i == 0) parent[0] = -1;
}

// Arrival at an internal node of the refit: acquire-release at device scope, so the box
// this thread wrote before is visible to the thread that arrives second, and that thread
// sees the first one's box (no separate fences on the path up).
__device__ __forceinline__ int refit_arrive(int* flag) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(flag) : "memory");
    return old;
}

// Leaf boxes from the current positions, then bottom-up unions: the second thread to
// reach an internal node computes its box (the first returns) and resets its flag. The
// thread carries the box of the child it comes from in registers and loads only the
// sibling's; the length of the walk (the hierarchy's depth, a few tens of levels) is the
// kernel's critical path, one atomic and one box load per level.
__global__ void k_refit(Prims t, const float4* xf, int n, const unsigned long long* keys, const int2* child,
                        const int* parent, float4* bmin, float4* bmax, int* flags, const int* req) {
    if (req && *req == 0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = (n - 1) + i;
    float3 lo, hi;
    prim_box(t, xf, int(keys[i] & 0xffffffffull), lo, hi);
    bmin[node] = make_float4(lo.x, lo.y, lo.z, 0.f);
    bmax[node] = make_float4(hi.x, hi.y, hi.z, 0.f);
    if (n == 1) return;
    int p = __ldg(&parent[node]);
    while (p >= 0) {
        const int2 c = __ldg(&child[p]);
        const int pp = __ldg(&parent[p]);
        if (refit_arrive(&flags[p]) == 0) return;
        flags[p] = 0;
        const int sib = c.x == node ? c.y : c.x;
        const float4 s0 = __ldcg(&bmin[sib]), s1 = __ldcg(&bmax[sib]);
        lo = make_float3(fminf(lo.x, s0.x), fminf(lo.y, s0.y), fminf(lo.z, s0.z));
        hi = make_float3(fmaxf(hi.x, s1.x), fmaxf(hi.y, s1.y), fmaxf(hi.z, s1.z));
        bmin[p] = make_float4(lo.x, lo.y, lo.z, 0.f);
        bmax[p] = make_float4(hi.x, hi.y, hi.z, 0.f);
        node = p;
        p = pp;
    }
}

struct LbvhDev {
    int n;
    const unsigned long long* keys;
    const int2* child;
    const float4* bmin;
    const float4* bmax;
};

__device__ __forceinline__ bool sphere_box(float3 p, float r2, float4 lo, float4 hi) {
    const float dx = fmaxf(fmaxf(lo.x - p.x, 0.f), p.x - hi.x);
    const float dy = fmaxf(fmaxf(lo.y - p.y, 0.f), p.y - hi.y);
    const float dz = fmaxf(fmaxf(lo.z - p.z, 0.f), p.z - hi.z);
    return dx * dx + dy * dy + dz * dz <= r2;
}

// Visits every primitive whose box is within sqrt(r2) of p, that is every leaf whose box
// and whose ancestors' boxes all pass the test (stack traversal). Both children of a node
// are tested together when the node is popped (two independent box loads in flight), a
// leaf that passes is visited at once, and only passing internal nodes are pushed; the
// set of visited leaves is that of a one-node-at-a-time traversal, the order differs.
template <typename F>
__device__ __forceinline__ void traverse(const LbvhDev& b, float3 p, float r2, unsigned long long* counters, F&& leaf) {
    if (b.n <= 0) return;
    if (!sphere_box(p, r2, b.bmin[0], b.bmax[0])) return;
    if (b.n == 1) {
        leaf(int(b.keys[0] & 0xffffffffull));
        return;
    }
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const int2 c = b.child[node];
        const float4 lo0 = b.bmin[c.x], hi0 = b.bmax[c.x], lo1 = b.bmin[c.y], hi1 = b.bmax[c.y];
        const bool h0 = sphere_box(p, r2, lo0, hi0), h1 = sphere_box(p, r2, lo1, hi1);
        const int ch[2] = {c.x, c.y};
        const bool hit[2] = {h0, h1};
#pragma unroll
        for (int k = 1; k >= 0; --k) {  // c.x ends on top of the stack, as before
            if (!hit[k]) continue;
            if (ch[k] >= b.n - 1) {
                leaf(int(b.keys[ch[k] - (b.n - 1)] & 0xffffffffull));
            } else if (sp + 1 > 64) {
                atomicAdd(&counters[CC_STACK_OVERFLOW], 1ull);
            } else {
                stack[sp++] = ch[k];
            }
        }
    }
}

// Packet traversal: the warp walks the hierarchy once for all its lanes' queries (lane i its
// own sphere p, r2; lanes without a query take part with active = false). A node is
// descended when its box passes the test of any lane; a leaf is visited by exactly the
// lanes whose own test its box passes — the leaves traverse() visits for that lane, since a
// node's box contains its children's — and the visiting lanes take the same primitive at
// the same time. For queries that are neighbours in space (a warp of consecutive grid
// vertices, or of consecutive leaves in Morton order) the warp's walk is little longer than
// one lane's, and the node loads and tests are shared instead of diverging. Every lane of
// the warp calls it.
template <typename F>
__device__ __forceinline__ void traverse_warp(const LbvhDev& b, float3 p, float r2, bool active,
                                              unsigned long long* counters, F&& leaf) {
    const unsigned full = 0xffffffffu;
    if (b.n <= 0) return;
    const bool hr = active && sphere_box(p, r2, b.bmin[0], b.bmax[0]);
    if (!__any_sync(full, hr)) return;
    if (b.n == 1) {
        if (hr) leaf(int(b.keys[0] & 0xffffffffull));
        return;
    }
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const int2 c = b.child[node];
        const float4 lo0 = b.bmin[c.x], hi0 = b.bmax[c.x], lo1 = b.bmin[c.y], hi1 = b.bmax[c.y];
        const bool h0 = active && sphere_box(p, r2, lo0, hi0), h1 = active && sphere_box(p, r2, lo1, hi1);
        const bool a0 = __any_sync(full, h0), a1 = __any_sync(full, h1);
        const int ch[2] = {c.x, c.y};
        const bool hit[2] = {h0, h1}, any[2] = {a0, a1};
#pragma unroll
        for (int k = 1; k >= 0; --k) {
            if (!any[k]) continue;
            if (ch[k] >= b.n - 1) {
                if (hit[k]) leaf(int(b.keys[ch[k] - (b.n - 1)] & 0xffffffffull));
            } else if (sp + 1 > 64) {
                if ((threadIdx.x & 31) == 0) atomicAdd(&counters[CC_STACK_OVERFLOW], 1ull);
            } else {
                stack[sp++] = ch[k];
            }
        }
    }
}

class Lbvh {
public:
    int n = 0;
    Prims prims{nullptr, 0};
    unsigned long long* keys = nullptr;
    unsigned long long* keysTmp = nullptr;
    int2* child = nullptr;
    int* parent = nullptr;
    float4* bmin = nullptr;
    float4* bmax = nullptr;
    int* flags = nullptr;
    int* bounds = nullptr;
    void* temp = nullptr;
    size_t tempBytes = 0;

    void alloc(int n_, Prims p, size_t& bytes) {
        n = n_;
        prims = p;
        if (n == 0) return;
        keys = dalloc<unsigned long long>(n, bytes);
        keysTmp = dalloc<unsigned long long>(n, bytes);
        child = dalloc<int2>(std::max(n - 1, 1), bytes);
        parent = dalloc<int>(2 * n - 1, bytes);
        bmin = dalloc<float4>(2 * n - 1, bytes);
        bmax = dalloc<float4>(2 * n - 1, bytes);
        flags = dalloc<int>(std::max(n - 1, 1), bytes);
        bounds = dalloc<int>(6, bytes);
        BVH_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tempBytes, keysTmp, keys, n, 0, 62));
        temp = dalloc<char>(tempBytes, bytes);
        BVH_CUDA(cudaMemset(flags, 0, sizeof(int) * std::max(n - 1, 1)));
        BVH_CUDA(cudaMemset(parent, 0xff, sizeof(int) * (2 * n - 1)));
    }
    void release() {
        for (void* p : {(void*)keys, (void*)keysTmp, (void*)child, (void*)parent, (void*)bmin, (void*)bmax,
                        (void*)flags, (void*)bounds, temp})
            if (p) cudaFree(p);
        keys = keysTmp = nullptr;
        child = nullptr;
        parent = flags = bounds = nullptr;
        bmin = bmax = nullptr;
        temp = nullptr;
    }
    // Morton codes of the primitive box centres, sorted (code, index) keys, hierarchy, boxes.
    void build(const float4* xf, cudaStream_t st) {
        if (n == 0) return;
        k_bounds_init<<<1, 32, 0, st>>>(bounds);
        k_centroid_bounds<<<blocks(n, 256), 256, 0, st>>>(prims, xf, n, bounds);
        k_morton<<<blocks(n, 256), 256, 0, st>>>(prims, xf, n, bounds, keysTmp);
        size_t tb = tempBytes;
        BVH_CUDA(cub::DeviceRadixSort::SortKeys(temp, tb, keysTmp, keys, n, 0, 62, st));
        if (n > 1) k_karras<<<blocks(n - 1, 256), 256, 0, st>>>(keys, n, child, parent);
        refit(xf, nullptr, st);
        BVH_CUDA(cudaGetLastError());
    }
    // Boxes from the current positions (when *req != 0, or always when req is null).
    void refit(const float4* xf, const int* req, cudaStream_t st) {
        if (n == 0) return;
        k_refit<<<blocks(n, 256), 256, 0, st>>>(prims, xf, n, keys, child, parent, bmin, bmax, flags, req);
    }
    LbvhDev dev() const { return LbvhDev{n, keys, child, bmin, bmax}; }
};


}  // namespace
}  // namespace bvh
}  // namespace gaia
