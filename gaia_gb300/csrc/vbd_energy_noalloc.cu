// Energy evaluation that allocates no device memory: gaia_vbd_energy_noalloc.
//
// Some callers cannot call cudaMalloc: hosts that hand the whole device memory
// to their own arena at start-up, and real-time or plugin hosts that forbid
// allocation after start-up because cudaMalloc / cudaFree synchronize the
// device and stall everything else running on it. For them this file provides
// the Neo-Hookean + inertia energy of gaia_vbd_energy as a stand-alone call on
// caller-owned device arrays, whose only scratch (one partial sum per block)
// lives in the fixed-size array below. The array is part of the library image:
// every GPU that loads the library holds its 32 KiB until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/gaia_vbd.h"

namespace gaia {
// Sets the message returned by gaia_vbd_last_global_error (vbd_engine.cu).
void set_last_global_error(const std::string& msg);

namespace noalloc {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 4096;              // partial sums held by the scratch array
constexpr int64_t kMaxItems = int64_t(1) << 24;  // largest nv or ntet accepted per call
constexpr int kMaxDevices = 64;

// Partial sums, one per block of the first pass. In host code this name is only a
// stand-in for the symbol: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_partials[kMaxBlocks];

std::mutex g_mutex;
double* g_scratch[kMaxDevices] = {};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double part[kThreads / 32];
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) part[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = l < kThreads / 32 ? part[l] : 0.0;
        v = warp_sum(v);
    }
    return v;  // valid in thread 0
}

// Pass 1: every block sums its grid-stride share of tets (elastic energy with the rest
// energy removed, VBDPhysicsCompute.cu:1775-1810) and of vertices (inertia energy
// m |x - y|^2 / (2 dt^2), VBD_BaseMaterial.h:223-241) into partials[blockIdx.x].
__global__ void __launch_bounds__(kThreads) k_energy_partials(const double* x, const double* y, const double* mass,
                                                              int32_t nv, const int32_t* tets, const double* dminv,
                                                              const double* vol, int32_t ntet, double mu,
                                                              double lmbd, double half_dt2inv, double* partials) {
    double e = 0.0;
    const double a = 1.0 + mu / lmbd;
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntet; t += stride) {
        const int32_t* tv = tets + 4 * size_t(t);
        const double* p0 = x + 3 * size_t(tv[0]);
        double Ds[9];
        for (int c = 0; c < 3; ++c) {
            const double* pc = x + 3 * size_t(tv[c + 1]);
            for (int r = 0; r < 3; ++r) Ds[3 * c + r] = pc[r] - p0[r];
        }
        const double* Di = dminv + 9 * size_t(t);
        double F[9];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                F[3 * c + r] = Ds[r] * Di[3 * c] + Ds[3 + r] * Di[3 * c + 1] + Ds[6 + r] * Di[3 * c + 2];
        const double det = F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                           F[6] * (F[1] * F[5] - F[4] * F[2]);
        double n2 = 0.0;
        for (int i = 0; i < 9; ++i) n2 += F[i] * F[i];
        const double A = vol[t];
        e += A * (mu * 0.5 * (n2 - 3.0) + lmbd * 0.5 * (det - a) * (det - a)) - 0.5 * A * lmbd * (1.0 - a) * (1.0 - a);
    }
    if (y) {
        for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += stride) {
            double d2 = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double d = x[3 * size_t(v) + k] - y[3 * size_t(v) + k];
                d2 += d * d;
            }
            e += half_dt2inv * mass[v] * d2;
        }
    }
    e = block_sum(e);
    if (threadIdx.x == 0) partials[blockIdx.x] = e;
}

// Pass 2: one block adds the nblocks partials of this call in a fixed order.
__global__ void __launch_bounds__(kThreads) k_energy_finish(const double* partials, int nblocks, double* out) {
    double e = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) e += partials[i];
    e = block_sum(e);
    if (threadIdx.x == 0) *out = e;
}

// Device address of the scratch array on the current device, looked up once per device and
// kept for the life of the process. A cudaDeviceReset of that device unloads the module and
// makes the kept address stale, so the entry point must not be called on a device after it
// was reset (the library would have to be loaded again).
cudaError_t scratch_for_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess) return e;
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

}  // namespace noalloc
}  // namespace gaia

extern "C" int gaia_vbd_energy_noalloc(const double* x, const double* y, const double* mass, int32_t nv,
                                       const int32_t* tets, const double* dminv, const double* vol, int32_t ntet,
                                       double mu, double lmbd, double dt, double* out, void* stream) {
    using namespace gaia::noalloc;
    if (!x || !tets || !dminv || !vol || !out || nv < 0 || ntet < 0 || (y && !mass) || !(lmbd != 0.0)) {
        gaia::set_last_global_error("gaia_vbd_energy_noalloc: null pointer or invalid size / material");
        return GAIA_VBD_E_INVALID_ARG;
    }
    if (y && !(dt > 0.0)) {
        gaia::set_last_global_error("gaia_vbd_energy_noalloc: dt must be positive when inertia targets are given");
        return GAIA_VBD_E_INVALID_ARG;
    }
    if (int64_t(nv) > kMaxItems || int64_t(ntet) > kMaxItems) {
        gaia::set_last_global_error("gaia_vbd_energy_noalloc: at most " + std::to_string(kMaxItems) +
                                    " vertices and tets per call (fixed scratch of " + std::to_string(kMaxBlocks) +
                                    " partial sums)");
        return GAIA_VBD_E_INVALID_ARG;
    }
    double* partials = nullptr;
    cudaError_t e = scratch_for_current_device(&partials);
    if (e != cudaSuccess) {
        gaia::set_last_global_error(std::string("gaia_vbd_energy_noalloc: scratch lookup failed: ") +
                                    cudaGetErrorString(e));
        return GAIA_VBD_E_CUDA;
    }
    const int64_t items = std::max<int64_t>(std::max<int64_t>(nv, ntet), 1);
    const int blocks = int(std::min<int64_t>(kMaxBlocks, (items + kThreads - 1) / kThreads));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const double half_dt2inv = y ? 0.5 / (dt * dt) : 0.0;
    k_energy_partials<<<blocks, kThreads, 0, st>>>(x, y, mass, nv, tets, dminv, vol, ntet, mu, lmbd, half_dt2inv,
                                                   partials);
    k_energy_finish<<<1, kThreads, 0, st>>>(partials, blocks, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        gaia::set_last_global_error(std::string("gaia_vbd_energy_noalloc: launch failed: ") + cudaGetErrorString(e));
        return GAIA_VBD_E_CUDA;
    }
    return GAIA_VBD_OK;
}

