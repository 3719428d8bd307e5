// Per-vertex state storage of the three precision modes.
//
//   StF32 : displacement as FP32                          (16 B per vertex, w = mass)
//   StDF  : displacement as a double-float pair hi + lo,  (32 B per vertex, hi.w = mass)
//           both FP32; |lo| <= ulp(hi) / 2. Differences and updates use FP32
//           operations only (error-free two-sum), so the state carries ~48
//           significant bits while no FP64 instruction runs per incidence:
//           GB300 executes FP64 at a small fraction of its FP32 rate.
//   StDFH : StDF state whose neighbour reads load the FP32 high part only (see below)
//   StF64 : displacement as FP64                          (32 B per vertex, w = mass)
//
// Each trait provides read-only (ldg) and coherent (ld) loads, a - b rounded to the
// compute type R, a + d for a delta d in the velocity type, conversions from
// and to double, and (c - X - u) for the world-box tests.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gaia {
namespace dev {

template <typename R>
struct alignas(4 * sizeof(R)) R4 {
    R x, y, z, w;
};

struct alignas(32) DF4 {
    float hx, hy, hz, w;   // high parts, mass
    float lx, ly, lz, pad; // low parts
};

// error-free a + b = s + e (Knuth two-sum), in round-to-nearest FP32 without contraction
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) + d, renormalized
__device__ __forceinline__ void df_add(float& hi, float& lo, float d) {
    float s, e;
    two_sum(hi, d, s, e);
    e = __fadd_rn(e, lo);
    two_sum(s, e, hi, lo);
}

struct StF32 {
    using U = R4<float>;
    using V = R4<float>;
    using Sc = float;
    static constexpr int kCode = 32;  // gaia_vbd_stats.precision
    __host__ __device__ static U from_d(const double* x, double w) {
        return U{float(x[0]), float(x[1]), float(x[2]), float(w)};
    }
    __device__ static void to_d(const U& u, double* x) { x[0] = u.x; x[1] = u.y; x[2] = u.z; }
    __device__ static Sc mass(const U& u) { return u.w; }
    __device__ static U ldg(const U* p, int i) {
        float4 v = __ldg(reinterpret_cast<const float4*>(p) + i);
        return U{v.x, v.y, v.z, v.w};
    }
    // coherent load: for state written earlier in the same kernel by the same block
    // (ordered by a block barrier)
    __device__ static U ld(const U* p, int i) {
        float4 v = reinterpret_cast<const float4*>(p)[i];
        return U{v.x, v.y, v.z, v.w};
    }
    // load through L2 only: for state written earlier in the same kernel by other blocks
    // (ordered by a grid barrier; the reading SM's L1 may hold an older copy of the line)
    __device__ static U ldcg(const U* p, int i) {
        float4 v = __ldcg(reinterpret_cast<const float4*>(p) + i);
        return U{v.x, v.y, v.z, v.w};
    }
    // the vertex's own state in full (ld / ldcg return what the incidence loop reads)
    __device__ static U ld_own(const U* p, int i) { return ld(p, i); }
    __device__ static U ldcg_own(const U* p, int i) { return ldcg(p, i); }
    // the state as the incidence loop uses it (the vertex's own, like its neighbours')
    __device__ static U nb(const U& u) { return u; }
    template <typename R>
    __device__ static void diff(const U& a, const U& b, R* o) {
        o[0] = R(a.x - b.x); o[1] = R(a.y - b.y); o[2] = R(a.z - b.z);
    }
    __device__ static U add(U a, Sc d0, Sc d1, Sc d2) {
        a.x += d0; a.y += d1; a.z += d2;
        return a;
    }
    __device__ static float comp(const U& u, int d) { return d == 0 ? u.x : (d == 1 ? u.y : u.z); }
    // the state moved into a frame shifted by (sx, sy, sz): u - s
    __device__ static U shift(U u, float sx, float sy, float sz) {
        u.x = __fsub_rn(u.x, sx);
        u.y = __fsub_rn(u.y, sy);
        u.z = __fsub_rn(u.z, sz);
        return u;
    }
    // the FP32 part that a frame shift takes out (the state itself)
    __device__ static float4 head(const U& u) { return make_float4(u.x, u.y, u.z, 0.f); }
    // c - (Xh + Xl) - u for a reference position split in two floats (X + F in a mesh frame)
    template <typename R>
    __device__ static R sub_plane(Sc c, float Xh, float Xl, const U& u, int d) {
        return R(__fsub_rn(__fsub_rn(__fsub_rn(c, Xh), comp(u, d)), Xl));
    }
    template <typename R>
    __device__ static R sub_from(Sc c, float X, const U& u, int d) {
        return R((c - X) - comp(u, d));
    }
};

struct StF64 {
    using U = R4<double>;
    using V = R4<double>;
    using Sc = double;
    static constexpr int kCode = 64;
    __host__ __device__ static U from_d(const double* x, double w) { return U{x[0], x[1], x[2], w}; }
    __device__ static void to_d(const U& u, double* x) { x[0] = u.x; x[1] = u.y; x[2] = u.z; }
    __device__ static Sc mass(const U& u) { return u.w; }
    __device__ static U ldg(const U* p, int i) {
        const double2* q = reinterpret_cast<const double2*>(p + i);
        double2 a = __ldg(q), b = __ldg(q + 1);
        return U{a.x, a.y, b.x, b.y};
    }
    __device__ static U ld(const U* p, int i) {
        const double2* q = reinterpret_cast<const double2*>(p + i);
        double2 a = q[0], b = q[1];
        return U{a.x, a.y, b.x, b.y};
    }
    __device__ static U ldcg(const U* p, int i) {
        const double2* q = reinterpret_cast<const double2*>(p + i);
        double2 a = __ldcg(q), b = __ldcg(q + 1);
        return U{a.x, a.y, b.x, b.y};
    }
    __device__ static U ld_own(const U* p, int i) { return ld(p, i); }
    __device__ static U ldcg_own(const U* p, int i) { return ldcg(p, i); }
    __device__ static U nb(const U& u) { return u; }
    template <typename R>
    __device__ static void diff(const U& a, const U& b, R* o) {
        o[0] = R(a.x - b.x); o[1] = R(a.y - b.y); o[2] = R(a.z - b.z);
    }
    __device__ static U add(U a, Sc d0, Sc d1, Sc d2) {
        a.x += d0; a.y += d1; a.z += d2;
        return a;
    }
    __device__ static double comp(const U& u, int d) { return d == 0 ? u.x : (d == 1 ? u.y : u.z); }
    __device__ static U shift(U u, float sx, float sy, float sz) {
        u.x -= double(sx);
        u.y -= double(sy);
        u.z -= double(sz);
        return u;
    }
    __device__ static float4 head(const U& u) { return make_float4(float(u.x), float(u.y), float(u.z), 0.f); }
    template <typename R>
    __device__ static R sub_plane(Sc c, float Xh, float Xl, const U& u, int d) {
        return R(((c - double(Xh)) - double(Xl)) - comp(u, d));
    }
    template <typename R>
    __device__ static R sub_from(Sc c, float X, const U& u, int d) {
        return R((c - double(X)) - comp(u, d));
    }
};

struct StDF {
    using U = DF4;
    using V = R4<float>;
    using Sc = float;
    static constexpr int kCode = 48;
    __host__ __device__ static U from_d(const double* x, double w) {
        U u;
        u.hx = float(x[0]); u.lx = float(x[0] - double(u.hx));
        u.hy = float(x[1]); u.ly = float(x[1] - double(u.hy));
        u.hz = float(x[2]); u.lz = float(x[2] - double(u.hz));
        u.w = float(w);
        u.pad = 0.f;
        return u;
    }
    __device__ static void to_d(const U& u, double* x) {
        x[0] = double(u.hx) + double(u.lx);
        x[1] = double(u.hy) + double(u.ly);
        x[2] = double(u.hz) + double(u.lz);
    }
    __device__ static Sc mass(const U& u) { return u.w; }
    __device__ static U ldg(const U* p, int i) {
        const float4* q = reinterpret_cast<const float4*>(p + i);
        float4 a = __ldg(q), b = __ldg(q + 1);
        return U{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    }
    __device__ static U ld(const U* p, int i) {
        const float4* q = reinterpret_cast<const float4*>(p + i);
        float4 a = q[0], b = q[1];
        return U{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    }
    __device__ static U ldcg(const U* p, int i) {
        const float4* q = reinterpret_cast<const float4*>(p + i);
        float4 a = __ldcg(q), b = __ldcg(q + 1);
        return U{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    }
    __device__ static U ld_own(const U* p, int i) { return ld(p, i); }
    __device__ static U ldcg_own(const U* p, int i) { return ldcg(p, i); }
    __device__ static U nb(const U& u) { return u; }
    // (a.hi - b.hi) + (a.lo - b.lo): relative error ~2^-23 of the result
    template <typename R>
    __device__ static void diff(const U& a, const U& b, R* o) {
        o[0] = R(__fadd_rn(__fsub_rn(a.hx, b.hx), __fsub_rn(a.lx, b.lx)));
        o[1] = R(__fadd_rn(__fsub_rn(a.hy, b.hy), __fsub_rn(a.ly, b.ly)));
        o[2] = R(__fadd_rn(__fsub_rn(a.hz, b.hz), __fsub_rn(a.lz, b.lz)));
    }
    __device__ static U add(U a, Sc d0, Sc d1, Sc d2) {
        df_add(a.hx, a.lx, d0);
        df_add(a.hy, a.ly, d1);
        df_add(a.hz, a.lz, d2);
        return a;
    }
    template <typename R>
    __device__ static R sub_from(Sc c, float X, const U& u, int d) {
        float h = d == 0 ? u.hx : (d == 1 ? u.hy : u.hz);
        float l = d == 0 ? u.lx : (d == 1 ? u.ly : u.lz);
        return R(__fsub_rn(__fsub_rn(__fsub_rn(c, X), h), l));
    }
    // exact (double-float) u - s
    __device__ static U shift(U u, float sx, float sy, float sz) {
        df_add(u.hx, u.lx, -sx);
        df_add(u.hy, u.ly, -sy);
        df_add(u.hz, u.lz, -sz);
        return u;
    }
    __device__ static float4 head(const U& u) { return make_float4(u.hx, u.hy, u.hz, 0.f); }
    template <typename R>
    __device__ static R sub_plane(Sc c, float Xh, float Xl, const U& u, int d) {
        float h = d == 0 ? u.hx : (d == 1 ? u.hy : u.hz);
        float l = d == 0 ? u.lx : (d == 1 ? u.ly : u.lz);
        return R(__fsub_rn(__fsub_rn(__fsub_rn(c, Xh), h), __fadd_rn(Xl, l)));
    }
};

// Double-float state read as FP32 in the incidence loop: a vertex's own state (its update,
// its inertia, damping, friction and ground terms) keeps both parts, so positions do not
// drift by FP32 rounding from update to update, while the incidence loop works on the high
// halves only, the neighbours' (whose gathers load 16 B instead of 32 B) and the vertex's
// own alike (nb): the element forces are those of the FP32 mode on the rounded positions,
// consistent between the vertices of a tet (with the own low half but not the neighbours',
// the forces of a tet's vertices would not balance and a body would drift), without the
// FP32 mode's accumulation of rounded updates.
struct StDFH : StDF {
    static constexpr int kCode = 40;
    __device__ static U ldg(const U* p, int i) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(p + i));
        return U{a.x, a.y, a.z, a.w, 0.f, 0.f, 0.f, 0.f};
    }
    __device__ static U ld(const U* p, int i) {
        const float4 a = reinterpret_cast<const float4*>(p + i)[0];
        return U{a.x, a.y, a.z, a.w, 0.f, 0.f, 0.f, 0.f};
    }
    __device__ static U ldcg(const U* p, int i) {
        const float4 a = __ldcg(reinterpret_cast<const float4*>(p + i));
        return U{a.x, a.y, a.z, a.w, 0.f, 0.f, 0.f, 0.f};
    }
    // the own state keeps its low half (the update accumulates into both)
    __device__ static U ld_own(const U* p, int i) { return StDF::ld(p, i); }
    __device__ static U ldcg_own(const U* p, int i) { return StDF::ldcg(p, i); }
    __device__ static U nb(const U& u) { return U{u.hx, u.hy, u.hz, u.w, 0.f, 0.f, 0.f, 0.f}; }
};

}  // namespace dev
}  // namespace gaia
