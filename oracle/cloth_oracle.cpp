// Test infrastructure only: CPU restatement of Gaia's cloth VBD step. It is the
// checker of the GPU cloth path (tests, smoke, the CPU baseline of the bench);
// nothing in the product links or calls it.
//
// Follows, in serial semantics:
//   VBDClothSimulationFramework::runStep_CDEveryIter  VBDCloth/VBDClothPhysics.cpp:389-518
//   VBDStepWithExistingCollisions                     VBDCloth/VBDClothPhysics.cpp:1026-1154
//   accumulateVF/EEContactForceAndHessian             VBDCloth/VBDClothPhysics.cpp:1248-1399
//   accumlateBoundaryForceAndHessian, computeFriction, computeContactRepulsiveForce
//                                                     VBDCloth/VBDClothPhysics.cpp:1401-1579
//   applyConservativeBoundTruncation, applyAcceleration, updateVelocity
//                                                     VBDCloth/VBDClothPhysics.cpp:1223-1246, 893-915, 2318-2360
//   applyCollisionDetection (bounds)                  VBDCloth/VBDClothPhysics.cpp:735-814
//   applyInitialStep / forwardStep_intertia           VBDCloth/VBDBaseTriMesh.cpp:55-196
//   accumlateStVKForceAndHessian (6x6 d2W/dF2 form)   VBDCloth/VBDTriMeshStVK.cpp:721-911
//   accumlateBendingForceAndHessian, quadratic forms  VBDCloth/VBDTriMeshStVK.cpp:50-89, 913-982
//   rest shape, topology                              TriMesh/TriMesh.cpp:213-244, 481-750
//   contact queries and feasible regions              CollisionDetector/ClothContactDetector.cpp:144-288,
//                                                     440-560, 731-813, 1052-1135;
//                                                     CollisionDetector/TriMeshCollisionGeometry.cpp:7-195;
//                                                     CollisionDetector/CollisionGeometry.h:84-255
// The solve is FP64; contact detection is FP32 on a float copy of the positions,
// with candidates taken in ascending (mesh, primitive) order. The rest-shape 2D
// frame here is aligned with each face's first edge (any in-plane frame gives the
// same energy).
#include "cloth_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

std::string g_err;

// ---------------------------------------------------------------- thread pool
class Pool {
public:
    explicit Pool(int n) {
        for (int i = 1; i < n; ++i) th_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
    }
    void run(int64_t n, const std::function<void(int64_t)>& fn) {
        if (th_.empty() || n < 64) {
            for (int64_t i = 0; i < n; ++i) fn(i);
            return;
        }
        {
            std::lock_guard<std::mutex> l(m_);
            fn_ = &fn;
            n_ = n;
            next_.store(0);
            busy_ = int(th_.size());
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> l(m_);
        done_.wait(l, [this] { return busy_ == 0; });
        fn_ = nullptr;
    }

private:
    void work() {
        for (;;) {
            int64_t b = next_.fetch_add(64);
            if (b >= n_) break;
            int64_t e = std::min(n_, b + 64);
            for (int64_t i = b; i < e; ++i) (*fn_)(i);
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
            std::lock_guard<std::mutex> l(m_);
            if (--busy_ == 0) done_.notify_all();
        }
    }
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    const std::function<void(int64_t)>* fn_ = nullptr;
    std::atomic<int64_t> next_{0};
    int64_t n_ = 0;
    int busy_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

// ---------------------------------------------------------------- small vectors
template <typename T>
struct V3 {
    T x, y, z;
};
template <typename T>
inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T>
inline T dotp(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T>
inline V3<T> crossp(V3<T> a, V3<T> b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
template <typename T>
inline V3<T> unit_or_zero(V3<T> a) {
    T n2 = dotp(a, a);
    return n2 > T(0) ? (T(1) / std::sqrt(n2)) * a : a;
}
using D3 = V3<double>;
using F3 = V3<float>;

enum { AtA = 0, AtB, AtC, AtAB, AtBC, AtAC, AtInterior, NotFound };

// CollisionGeometry.h:84-145
template <typename T>
int closest_on_triangle(V3<T> p, V3<T> a, V3<T> b, V3<T> c, V3<T>& bary, V3<T>& q) {
    const V3<T> ab = b - a, ac = c - a, ap = p - a;
    const T d1 = dotp(ab, ap), d2 = dotp(ac, ap);
    if (d1 <= T(0) && d2 <= T(0)) {
        bary = {T(1), T(0), T(0)};
        q = a;
        return AtA;
    }
    const V3<T> bp = p - b;
    const T d3 = dotp(ab, bp), d4 = dotp(ac, bp);
    if (d3 >= T(0) && d4 <= d3) {
        bary = {T(0), T(1), T(0)};
        q = b;
        return AtB;
    }
    const V3<T> cp = p - c;
    const T d5 = dotp(ab, cp), d6 = dotp(ac, cp);
    if (d6 >= T(0) && d5 <= d6) {
        bary = {T(0), T(0), T(1)};
        q = c;
        return AtC;
    }
    const T vc = d1 * d4 - d3 * d2;
    if (vc <= T(0) && d1 >= T(0) && d3 <= T(0)) {
        const T v = d1 / (d1 - d3);
        bary = {T(1) - v, v, T(0)};
        q = a + v * ab;
        return AtAB;
    }
    const T vb = d5 * d2 - d1 * d6;
    if (vb <= T(0) && d2 >= T(0) && d6 <= T(0)) {
        const T v = d2 / (d2 - d6);
        bary = {T(1) - v, T(0), v};
        q = a + v * ac;
        return AtAC;
    }
    const T va = d3 * d6 - d5 * d4;
    if (va <= T(0) && (d4 - d3) >= T(0) && (d5 - d6) >= T(0)) {
        const T v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary = {T(0), T(1) - v, v};
        q = b + v * (c - b);
        return AtBC;
    }
    const T denom = T(1) / (va + vb + vc);
    const T v = vb * denom, w = vc * denom;
    bary = {T(1) - v - w, v, w};
    q = (a + v * ab) + w * ac;
    return AtInterior;
}

// CollisionGeometry.h:147-255
template <typename T>
void closest_on_segments(V3<T> p0, V3<T> p1, V3<T> q0, V3<T> q1, V3<T>& cp, V3<T>& cq, T& s, T& t) {
    const V3<T> p = p1 - p0, q = q1 - q0, r = p0 - q0;
    const T a = dotp(p, p), b = dotp(p, q), c = dotp(q, q), d = dotp(p, r), e = dotp(q, r);
    s = T(0);
    t = T(0);
    const T det = a * c - b * b;
    if (det > T(1e-5f)) {
        const T bte = b * e, ctd = c * d;
        if (bte <= ctd) {
            if (e <= T(0)) {
                s = (-d >= a ? T(1) : (-d > T(0) ? -d / a : T(0)));
                t = T(0);
            } else if (e < c) {
                s = T(0);
                t = e / c;
            } else {
                s = (b - d >= a ? T(1) : (b - d > T(0) ? (b - d) / a : T(0)));
                t = T(1);
            }
        } else {
            s = bte - ctd;
            if (s >= det) {
                if (b + e <= T(0)) {
                    s = (-d <= T(0) ? T(0) : (-d < a ? -d / a : T(1)));
                    t = T(0);
                } else if (b + e < c) {
                    s = T(1);
                    t = (b + e) / c;
                } else {
                    s = (b - d <= T(0) ? T(0) : (b - d < a ? (b - d) / a : T(1)));
                    t = T(1);
                }
            } else {
                const T ate = a * e, btd = b * d;
                if (ate <= btd) {
                    s = (-d <= T(0) ? T(0) : (-d >= a ? T(1) : -d / a));
                    t = T(0);
                } else {
                    t = ate - btd;
                    if (t >= det) {
                        s = (b - d <= T(0) ? T(0) : (b - d >= a ? T(1) : (b - d) / a));
                        t = T(1);
                    } else {
                        s /= det;
                        t /= det;
                    }
                }
            }
        }
    } else {
        if (e <= T(0)) {
            s = (-d <= T(0) ? T(0) : (-d >= a ? T(1) : -d / a));
            t = T(0);
        } else if (e >= c) {
            s = (b - d <= T(0) ? T(0) : (b - d >= a ? T(1) : (b - d) / a));
            t = T(1);
        } else {
            s = T(0);
            t = e / c;
        }
    }
    cp = (T(1) - s) * p0 + s * p1;
    cq = (T(1) - t) * q0 + t * q1;
}

// LDL^T solve of a symmetric 3x3 with a relative pivot threshold (shared definition
// with the GPU kernels: the reference's solve3x3_psd_stable is not in its sources).
bool solve3(const double H[3][3], const double b[3], double x[3]) {
    const double scale = std::max(std::fabs(H[0][0]), std::max(std::fabs(H[1][1]), std::fabs(H[2][2])));
    if (!(scale > 0)) return false;
    const double tol = 1e-12 * scale;
    const double d0 = H[0][0];
    if (!(d0 > tol)) return false;
    const double l10 = H[0][1] / d0, l20 = H[0][2] / d0;
    const double d1 = H[1][1] - l10 * H[0][1];
    if (!(d1 > tol)) return false;
    const double l21 = (H[1][2] - l20 * H[0][1]) / d1;
    const double d2 = H[2][2] - l20 * H[0][2] - l21 * l21 * d1;
    if (!(d2 > tol)) return false;
    double z0 = b[0], z1 = b[1] - l10 * z0, z2 = b[2] - l20 * z0 - l21 * z1;
    z0 /= d0;
    z1 /= d1;
    z2 /= d2;
    x[2] = z2;
    x[1] = z1 - l21 * x[2];
    x[0] = z0 - l10 * x[1] - l20 * x[2];
    return std::isfinite(x[0]) && std::isfinite(x[1]) && std::isfinite(x[2]);
}

struct EdgeT {
    int v1, v2, n12, n21, f1, f2;
};

struct Mesh {
    int nv = 0, nf = 0, ne = 0;
    bool collider = false;
    ClothOracleMesh prm{};
    std::vector<D3> x0;                  // loaded positions
    std::vector<int> faces;              // 3*nf
    std::vector<EdgeT> edges;
    std::vector<int> fedges;             // 3*nf
    std::vector<std::vector<int>> vv;    // neighbour vertices
    std::vector<std::vector<std::pair<int, int>>> vf, ve, vb;  // (face|edge, order)
    std::vector<double> dminv, area, mass, Q;  // 4*nf, nf, nv, 16*ne
    std::vector<int8_t> fixed;
    std::vector<std::vector<int>> colors;
};

struct Scene {
    ClothOracleParams p{};
    std::vector<Mesh> m;
    int ns = 0;
    std::vector<int> vbase, fbase, ebase;
    int nV = 0, nF = 0, nE = 0, nSimV = 0, nSimF = 0, nSimE = 0;
    std::vector<int> vmesh, fmesh, emesh;
    // state (global vertex index)
    std::vector<D3> x, xprev, y, v, vprev, acc, xnext, xcd, xPrevIter;
    std::vector<double> bound;
    std::vector<char> active;
    std::vector<std::vector<std::pair<int, int>>> groups;
    // detection results (global ids)
    std::vector<std::vector<int>> vfFaces;
    std::vector<float> vfMin, fMin, eeMin;
    std::vector<std::vector<int>> fvVerts, eeOther;
    std::atomic<bool> cdRequired{false};
    int64_t nInit = 0;
    int64_t detections = 0;
    std::atomic<int64_t> truncations{0}, failed{0};
    std::unique_ptr<Pool> pool;
};

void build_topology(Mesh& M) {
    std::map<std::pair<int, int>, int> key;
    M.fedges.assign(3 * size_t(M.nf), -1);
    for (int f = 0; f < M.nf; ++f)
        for (int i = 0; i < 3; ++i) {
            const int a = M.faces[3 * f + i], b = M.faces[3 * f + (i + 1) % 3], c = M.faces[3 * f + (i + 2) % 3];
            auto k = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = key.find(k);
            if (it == key.end()) {
                key[k] = int(M.edges.size());
                M.fedges[3 * f + i] = int(M.edges.size());
                M.edges.push_back({a, b, c, -1, f, -1});
            } else {
                EdgeT& E = M.edges[it->second];
                if (E.f2 != -1 || E.v1 != b) throw std::runtime_error("non-manifold or inconsistently oriented mesh");
                E.f2 = f;
                E.n21 = c;
                M.fedges[3 * f + i] = it->second;
            }
        }
    M.ne = int(M.edges.size());
    M.vv.assign(M.nv, {});
    M.vf.assign(M.nv, {});
    M.ve.assign(M.nv, {});
    M.vb.assign(M.nv, {});
    for (int f = 0; f < M.nf; ++f)
        for (int i = 0; i < 3; ++i) M.vf[M.faces[3 * f + i]].push_back({f, i});
    for (int e = 0; e < M.ne; ++e) {
        const EdgeT& E = M.edges[e];
        M.vv[E.v1].push_back(E.v2);
        M.vv[E.v2].push_back(E.v1);
        M.ve[E.v1].push_back({e, 0});
        M.ve[E.v2].push_back({e, 1});
    }
    for (int v = 0; v < M.nv; ++v) {
        std::sort(M.vv[v].begin(), M.vv[v].end());
        for (auto& eo : M.ve[v])
            if (M.edges[eo.first].f2 != -1) M.vb[v].push_back(eo);
        for (auto& fo : M.vf[v]) {
            const int e = M.fedges[3 * fo.first + (fo.second + 1) % 3];
            const EdgeT& E = M.edges[e];
            if (E.f2 == -1) continue;
            M.vb[v].push_back({e, E.f1 == fo.first ? 2 : 3});
        }
    }
}

void rest_shape(Mesh& M) {
    M.dminv.assign(4 * size_t(M.nf), 0.0);
    M.area.assign(M.nf, 0.0);
    M.mass.assign(M.nv, 0.0);
    for (int f = 0; f < M.nf; ++f) {
        const D3 a = M.x0[M.faces[3 * f]], b = M.x0[M.faces[3 * f + 1]], c = M.x0[M.faces[3 * f + 2]];
        const D3 e1 = b - a, e2 = c - a;
        const D3 n = unit_or_zero(crossp(e1, e2));
        const D3 t = unit_or_zero(e1);
        const D3 s = crossp(n, t);
        const double D00 = dotp(t, e1), D01 = dotp(t, e2), D10 = dotp(s, e1), D11 = dotp(s, e2);
        const double det = D00 * D11 - D01 * D10;
        if (!(det > 0)) throw std::runtime_error("degenerate face in the oracle");
        M.area[f] = 0.5 * det;
        M.dminv[4 * f + 0] = D11 / det;
        M.dminv[4 * f + 1] = -D10 / det;
        M.dminv[4 * f + 2] = -D01 / det;
        M.dminv[4 * f + 3] = D00 / det;
        for (int i = 0; i < 3; ++i) M.mass[M.faces[3 * f + i]] += M.prm.density * M.area[f] / 3.0;
    }
    M.Q.assign(16 * size_t(M.ne), 0.0);
    auto cot = [](D3 u, D3 w) { return dotp(u, w) / std::sqrt(dotp(crossp(u, w), crossp(u, w))); };
    for (int e = 0; e < M.ne; ++e) {
        const EdgeT& E = M.edges[e];
        if (E.f2 == -1) continue;
        const D3 x0 = M.x0[E.v1], x1 = M.x0[E.v2], x2 = M.x0[E.n12], x3 = M.x0[E.n21];
        const D3 e01 = x1 - x0, e02 = x2 - x0, e03 = x3 - x0, e12 = x2 - x1, e13 = x3 - x1;
        const D3 m01 = -1.0 * e01;
        const double c01 = cot(e02, e01), c02 = cot(e01, e03), c03 = cot(m01, e12), c04 = cot(m01, e13);
        const double K[4] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
        auto farea = [&](int f) {
            const D3 a = M.x0[M.faces[3 * f]], b = M.x0[M.faces[3 * f + 1]], c = M.x0[M.faces[3 * f + 2]];
            const D3 n = crossp(b - a, c - a);
            return std::sqrt(dotp(n, n));
        };
        const double s = farea(E.f1) + farea(E.f2);
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) M.Q[16 * e + 4 * i + j] = 3.0 * K[i] * K[j] / s;
    }
}

// VBDClothSimulationFramework::initializeParallelGroups (VBDClothPhysics.cpp:72-138)
void merge_groups(Scene& S) {
    size_t ng = 0;
    for (int i = 0; i < S.ns; ++i) ng = std::max(ng, S.m[i].colors.size());
    S.groups.assign(ng, {});
    for (int i = 0; i < S.ns; ++i) {
        const size_t nc = S.m[i].colors.size();
        for (size_t c = 0; c < nc; ++c) {
            size_t best = 0;
            for (size_t g = 1; g < nc; ++g)
                if (S.groups[g].size() < S.groups[best].size()) best = g;
            for (int v : S.m[i].colors[c]) S.groups[best].push_back({i, v});
        }
    }
}

// ---------------------------------------------------------------- detection
struct Grid {
    float h = 1;
    std::unordered_map<int64_t, std::vector<int>> cells;
    static int64_t key(int i, int j, int k) {
        return (int64_t(i) & 0x1fffff) | ((int64_t(j) & 0x1fffff) << 21) | ((int64_t(k) & 0x1fffff) << 42);
    }
    int cell(float x) const { return int(std::floor(x / h)); }
    void insert(int id, F3 lo, F3 hi) {
        for (int i = cell(lo.x); i <= cell(hi.x); ++i)
            for (int j = cell(lo.y); j <= cell(hi.y); ++j)
                for (int k = cell(lo.z); k <= cell(hi.z); ++k) cells[key(i, j, k)].push_back(id);
    }
    // ids of every primitive whose cells overlap the box [p - r, p + r], ascending and unique
    void query(F3 p, float r, std::vector<int>& out) const {
        out.clear();
        for (int i = cell(p.x - r); i <= cell(p.x + r); ++i)
            for (int j = cell(p.y - r); j <= cell(p.y + r); ++j)
                for (int k = cell(p.z - r); k <= cell(p.z + r); ++k) {
                    auto it = cells.find(key(i, j, k));
                    if (it != cells.end()) out.insert(out.end(), it->second.begin(), it->second.end());
                }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
};

F3 fpos(const std::vector<F3>& xf, int i) { return xf[i]; }

bool vertex_feasible(const Scene& S, const std::vector<F3>& xf, F3 p, int m, int a) {
    const int gb = S.vbase[m];
    const F3 A = xf[gb + a];
    const F3 AP = p - A;
    const float relaxed = -1e-3f - 1e-6f;
    for (int b : S.m[m].vv[a]) {
        const F3 BA = A - xf[gb + b];
        if (dotp(AP, BA) < relaxed) return false;
    }
    return true;
}

bool edge_feasible(const Scene& S, const std::vector<F3>& xf, F3 p, int m, int e) {
    const int gb = S.vbase[m];
    const EdgeT& E = S.m[m].edges[e];
    const F3 v1 = xf[gb + E.v1], v2 = xf[gb + E.v2];
    const F3 AP = p - v1, BP = p - v2, AB = v2 - v1;
    const float relaxed = 1e-3f + 1e-6f;
    if (dotp(AP, AB) < -relaxed) return false;
    if (dotp(BP, AB) > relaxed) return false;
    const float ABsq = dotp(AB, AB);
    if (ABsq < 1e-5f * 1e-5f) return false;
    for (int o : {E.n12, E.n21}) {
        if (o == -1) continue;
        const F3 vo = xf[gb + o];
        const float t = dotp(AB, vo - v1) / ABsq;
        const F3 foot = v1 + t * AB;
        if (dotp(vo - foot, p - foot) > relaxed) return false;
    }
    return true;
}

void detect(Scene& S) {
    const float r = float(S.p.max_query_dis);
    std::vector<F3> xf(S.nV);
    for (int g = 0; g < S.nV; ++g) xf[g] = {float(S.x[g].x), float(S.x[g].y), float(S.x[g].z)};
    for (int g = 0; g < S.nSimV; ++g) S.xcd[g] = S.x[g];
    // face and edge grids (cell = query radius, at least)
    double avg = 0;
    int cnt = 0;
    for (int mi = 0; mi < int(S.m.size()); ++mi)
        for (const EdgeT& E : S.m[mi].edges) {
            const F3 d = xf[S.vbase[mi] + E.v1] - xf[S.vbase[mi] + E.v2];
            avg += std::sqrt(dotp(d, d));
            ++cnt;
        }
    Grid fg, eg;
    fg.h = eg.h = std::max(r, float(cnt ? avg / cnt : r));
    for (int f = 0; f < S.nF; ++f) {
        const int m = S.fmesh[f], lf = f - S.fbase[m], gb = S.vbase[m];
        const F3 a = xf[gb + S.m[m].faces[3 * lf]], b = xf[gb + S.m[m].faces[3 * lf + 1]], c = xf[gb + S.m[m].faces[3 * lf + 2]];
        fg.insert(f, {std::min({a.x, b.x, c.x}), std::min({a.y, b.y, c.y}), std::min({a.z, b.z, c.z})},
                  {std::max({a.x, b.x, c.x}), std::max({a.y, b.y, c.y}), std::max({a.z, b.z, c.z})});
    }
    for (int e = 0; e < S.nE; ++e) {
        const int m = S.emesh[e], le = e - S.ebase[m], gb = S.vbase[m];
        const F3 a = xf[gb + S.m[m].edges[le].v1], b = xf[gb + S.m[m].edges[le].v2];
        eg.insert(e, {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)},
                  {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)});
    }

    // vertex-face queries
    S.vfFaces.assign(S.nV, {});
    S.vfMin.assign(S.nV, r);
    std::vector<std::vector<std::pair<int, float>>> hits(S.nV);
    S.pool->run(S.nV, [&](int64_t gi) {
        const int g = int(gi);
        const int mq = S.vmesh[g], lv = g - S.vbase[mq];
        const bool qSim = mq < S.ns;
        const F3 p = xf[g];
        std::vector<int> cand;
        fg.query(p, r * 1.0001f, cand);
        std::vector<std::pair<int, int>> acc;  // (face, type), ascending face
        float mn = r;
        for (int f : cand) {
            const int mf = S.fmesh[f], lf = f - S.fbase[mf], gb = S.vbase[mf];
            const bool fSim = mf < S.ns;
            if (!fSim && !qSim) continue;
            const int* fv = &S.m[mf].faces[3 * lf];
            if (mf == mq && (fv[0] == lv || fv[1] == lv || fv[2] == lv)) continue;
            F3 bary, q;
            const int type = closest_on_triangle<float>(p, xf[gb + fv[0]], xf[gb + fv[1]], xf[gb + fv[2]], bary, q);
            const F3 d3 = p - q;
            const float d = std::sqrt(dotp(d3, d3));
            if (!(d < r)) continue;
            mn = std::min(mn, d);
            hits[g].push_back({f, d});
            acc.push_back({f, type});
        }
        S.vfMin[g] = mn;
        std::vector<std::pair<int, int>> seen;  // (primitive type, mesh-local id)
        for (auto& ft : acc) {
            const int f = ft.first, type = ft.second;
            const int mf = S.fmesh[f], lf = f - S.fbase[mf];
            const Mesh& M = S.m[mf];
            int ptype, pid;
            if (type <= AtC) {
                ptype = 0;
                pid = M.faces[3 * lf + type];
            } else if (type <= AtAC) {
                ptype = 1;
                pid = M.fedges[3 * lf + (type == AtAB ? 0 : (type == AtBC ? 1 : 2))];
            } else {
                ptype = 2;
                pid = lf;
            }
            if (std::find(seen.begin(), seen.end(), std::make_pair(ptype, pid)) != seen.end()) continue;
            bool ok;
            if (type == AtInterior) ok = true;
            else if (type <= AtC) ok = vertex_feasible(S, xf, p, mf, M.faces[3 * lf + type]);
            else ok = edge_feasible(S, xf, p, mf, pid);
            if (!ok) continue;
            if (int(seen.size()) >= 32) break;  // VF_CAP of the GPU detector
            seen.push_back({ptype, pid});
            S.vfFaces[g].push_back(f);
        }
    });
    S.fMin.assign(S.nF, r);
    for (int g = 0; g < S.nV; ++g)
        for (auto& fd : hits[g]) S.fMin[fd.first] = std::min(S.fMin[fd.first], fd.second);
    S.fvVerts.assign(S.nSimF, {});
    for (int g = 0; g < S.nV; ++g)
        for (int f : S.vfFaces[g])
            if (f < S.nSimF && S.fvVerts[f].size() < 32) S.fvVerts[f].push_back(g);

    // edge-edge queries
    S.eeOther.assign(S.nSimE, {});
    S.eeMin.assign(S.nSimE, r);
    S.pool->run(S.nSimE, [&](int64_t ei) {
        const int e = int(ei);
        const int m1 = S.emesh[e], le = e - S.ebase[m1], gb1 = S.vbase[m1];
        const EdgeT& E = S.m[m1].edges[le];
        const F3 p1 = xf[gb1 + E.v1], p2 = xf[gb1 + E.v2];
        const F3 dd = p1 - p2;
        const float half = std::sqrt(dotp(dd, dd)) * 0.5f;
        const F3 c = 0.5f * (p1 + p2);
        std::vector<int> cand;
        eg.query(c, (r + half) * 1.0001f, cand);
        float mn = r;
        for (int e2 : cand) {
            const int m2 = S.emesh[e2], le2 = e2 - S.ebase[m2], gb2 = S.vbase[m2];
            const EdgeT& F = S.m[m2].edges[le2];
            if (m1 == m2) {
                if (le2 == le) continue;
                if (E.v1 == F.v1 || E.v1 == F.v2 || E.v2 == F.v1 || E.v2 == F.v2) continue;
            }
            const F3 q1 = xf[gb2 + F.v1], q2 = xf[gb2 + F.v2];
            F3 c1, c2;
            float s, t;
            closest_on_segments<float>(p1, p2, q1, q2, c1, c2, s, t);
            const F3 df = c1 - c2;
            const float d = std::sqrt(dotp(df, df));
            mn = std::min(mn, d);
            if (!(d < r)) continue;
            const F3 ev1 = p2 - p1, ev2 = q2 - q1;
            const bool ok = (dotp(c2 - p1, ev1) >= 0.f && dotp(p2 - c2, ev1) >= 0.f) ||
                            (dotp(c1 - q1, ev2) >= 0.f && dotp(q2 - c1, ev2) >= 0.f);
            if (!ok) continue;
            if (S.eeOther[e].size() < 64) S.eeOther[e].push_back(e2);  // EE_CAP
        }
        S.eeMin[e] = mn;
    });

    // conservative bounds (VBDClothPhysics.cpp:780-814)
    for (int m = 0; m < S.ns; ++m) {
        const Mesh& M = S.m[m];
        for (int lv = 0; lv < M.nv; ++lv) {
            const int g = S.vbase[m] + lv;
            float dMin = float(S.p.max_query_dis);
            dMin = std::min(dMin, S.vfMin[g]);
            bool act = !S.vfFaces[g].empty();
            for (auto& fo : M.vf[lv]) {
                const int f = S.fbase[m] + fo.first;
                dMin = std::min(dMin, S.fMin[f]);
                act = act || !S.fvVerts[f].empty();
            }
            for (auto& eo : M.ve[lv]) {
                const int e = S.ebase[m] + eo.first;
                dMin = std::min(dMin, S.eeMin[e]);
                act = act || !S.eeOther[e].empty();
            }
            dMin = std::max(0.f, dMin - float(S.p.thickness));
            S.bound[g] = double(dMin * float(S.p.relaxation));
            if (act) S.active[g] = 1;
        }
    }
    S.cdRequired = false;
    ++S.detections;
}

// ---------------------------------------------------------------- per-vertex solve
void repulsion(const ClothOracleParams& p, double dis, double& dEdD, double& d2E) {
    const double dadj = dis - p.thickness;
    const double r = p.contact_radius, k = p.contact_stiffness;
    const double tau = r * 0.5;
    if (dadj < tau && dadj > double(1e-5f)) {
        const double k2 = 0.5 * tau * tau * k;
        dEdD = -k2 / dadj;
        d2E = k2 / (dadj * dadj);
    } else {
        dEdD = -k * (r - dadj);
        d2E = k;
    }
}

void friction(double mu, double lambda, D3 t0, D3 t1, D3 dx, double epsU, double b, D3& f, double H[3][3]) {
    const double u0 = dotp(t0, dx), u1 = dotp(t1, dx);
    const double un = std::sqrt(u0 * u0 + u1 * u1);
    if (!(un > 0)) return;
    const double f1 = un > epsU ? 1.0 / un : (-un / epsU + 2.0) / epsU;
    f = f + (-mu * lambda * f1 * b) * (u0 * t0 + u1 * t1);
    const double T[2][3] = {{t0.x, t0.y, t0.z}, {t1.x, t1.y, t1.z}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] += mu * lambda * f1 * b * b * (T[0][i] * T[0][j] + T[1][i] * T[1][j]);
}

void add_nn(double H[3][3], double s, D3 n) {
    const double a[3] = {n.x, n.y, n.z};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] += s * a[i] * a[j];
}

const ClothOracleMesh& mprm(const Scene& S, int m) { return S.m[m].prm; }

void vf_force(const Scene& S, int u, int f, int order, D3& force, double H[3][3]) {
    const int mf = S.fmesh[f], lf = f - S.fbase[mf], gb = S.vbase[mf];
    const int* fv = &S.m[mf].faces[3 * lf];
    const int t0 = gb + fv[0], t1 = gb + fv[1], t2 = gb + fv[2];
    const D3 xu = S.x[u];
    D3 bary, q;
    closest_on_triangle<double>(xu, S.x[t0], S.x[t1], S.x[t2], bary, q);
    const D3 diff = xu - q;
    const D3 n = unit_or_zero(diff);
    const double dis = dotp(diff, n);
    if (!(dis < S.p.contact_radius + S.p.thickness)) return;
    const double bs[4] = {-bary.x, -bary.y, -bary.z, 1.0};
    const double b = bs[order];
    double dEdD, d2E;
    repulsion(S.p, dis, dEdD, d2E);
    const double lambda = -dEdD;
    force = force + (b * lambda) * n;
    add_nn(H, d2E * b * b, n);
    const D3 dx3 = xu - S.xprev[u];
    const D3 qprev = (bary.x * S.xprev[t0] + bary.y * S.xprev[t1]) + bary.z * S.xprev[t2];
    const D3 dx = dx3 - (q - qprev);
    const D3 e0 = unit_or_zero(S.x[t1] - S.x[t0]);
    const D3 e1 = unit_or_zero(crossp(e0, n));
    const ClothOracleMesh &pf = mprm(S, mf), &pu = mprm(S, S.vmesh[u]);
    const double mu = (pf.friction_dynamic + pu.friction_dynamic) * 0.5;
    const double epsU = (pf.friction_eps_v + pu.friction_eps_v) * 0.5 * S.p.dt;
    friction(mu, lambda, e0, e1, dx, epsU, b, force, H);
}

void ee_force(const Scene& S, int e, int e2, int order, D3& force, double H[3][3]) {
    const int m1 = S.emesh[e], m2 = S.emesh[e2];
    const EdgeT& E = S.m[m1].edges[e - S.ebase[m1]];
    const EdgeT& F = S.m[m2].edges[e2 - S.ebase[m2]];
    const int a1 = S.vbase[m1] + E.v1, a2 = S.vbase[m1] + E.v2, b1 = S.vbase[m2] + F.v1, b2 = S.vbase[m2] + F.v2;
    D3 c1, c2;
    double s, t;
    closest_on_segments<double>(S.x[a1], S.x[a2], S.x[b1], S.x[b2], c1, c2, s, t);
    const D3 diff = c1 - c2;
    const double dis = std::sqrt(dotp(diff, diff));
    const D3 v1 = S.x[a2] - S.x[a1], v2 = S.x[b2] - S.x[b1];
    const D3 cr = crossp(v1, v2);
    const double par = dotp(cr, cr) / (std::sqrt(dotp(v1, v1)) * std::sqrt(dotp(v2, v2)));
    if (!(dis < S.p.contact_radius + S.p.thickness && par > double(1e-5f))) return;
    const D3 n = (1.0 / dis) * diff;
    const double bs[4] = {1.0 - s, s, -1.0 + t, -t};
    const double b = bs[order];
    double dEdD, d2E;
    repulsion(S.p, dis, dEdD, d2E);
    const double lambda = -dEdD;
    force = force + (b * lambda) * n;
    add_nn(H, d2E * b * b, n);
    const D3 c1p = (1.0 - s) * S.xprev[a1] + s * S.xprev[a2];
    const D3 c2p = (1.0 - t) * S.xprev[b1] + t * S.xprev[b2];
    const D3 dx = (c1 - c1p) - (c2 - c2p);
    const D3 e0 = unit_or_zero(v1);
    const D3 e1 = unit_or_zero(crossp(e0, n));
    const ClothOracleMesh &p1 = mprm(S, m1), &p2 = mprm(S, m2);
    const double mu = (p1.friction_dynamic + p2.friction_dynamic) * 0.5;
    const double epsU = (p1.friction_eps_v + p2.friction_eps_v) * 0.5 * S.p.dt;
    friction(mu, lambda, e0, e1, dx, epsU, b, force, H);
}

// StVK membrane of one face at one vertex, literally as VBDTriMeshStVK.cpp:721-911:
// F = Ds DmInv, S = 2 mu G + lambda tr(G) I, F12 = -A F S DmInv^T, the 6x6 d2W/dF2 and
// assembleMembraneHessian (VBDCloth/VBDBaseTriMesh.h:149-160).
void stvk_face(const Scene& S, int m, int lf, int order, D3& force, double H[3][3]) {
    const Mesh& M = S.m[m];
    const int gb = S.vbase[m];
    const D3 x0 = S.x[gb + M.faces[3 * lf]], x1 = S.x[gb + M.faces[3 * lf + 1]], x2 = S.x[gb + M.faces[3 * lf + 2]];
    const double* Di = &M.dminv[4 * lf];  // column-major: Di[0]=(0,0) Di[1]=(1,0) Di[2]=(0,1) Di[3]=(1,1)
    const double Dm[2][2] = {{Di[0], Di[2]}, {Di[1], Di[3]}};
    const D3 c0 = x1 - x0, c1 = x2 - x0;
    double F[3][2];
    const double cc0[3] = {c0.x, c0.y, c0.z}, cc1[3] = {c1.x, c1.y, c1.z};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) F[i][j] = cc0[i] * Dm[0][j] + cc1[i] * Dm[1][j];
    double G[2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            double s = 0;
            for (int i = 0; i < 3; ++i) s += F[i][a] * F[i][b];
            G[a][b] = 0.5 * (s - (a == b ? 1.0 : 0.0));
        }
    const double mu = M.prm.miu, la = M.prm.lambda_;
    const double tr = G[0][0] + G[1][1];
    double Sm[2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) Sm[a][b] = 2.0 * mu * G[a][b] + (a == b ? la * tr : 0.0);
    const double A = M.area[lf];
    double F12[3][2];  // -A F S DmInv^T
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) {
            double s = 0;
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) s += F[i][a] * Sm[a][b] * Dm[j][b];
            F12[i][j] = -A * s;
        }
    const double F11 = F[0][0], F21 = F[1][0], F31 = F[2][0], F12_ = F[0][1], F22 = F[1][1], F32 = F[2][1];
    const double euu = G[0][0], evv = G[1][1], euv = G[0][1], es = euu + evv;
    double D[6][6];
    D[0][0] = F11 * (F11 * la + 2 * F11 * mu) + 2 * mu * euu + la * es + F12_ * F12_ * mu;
    D[0][1] = F11 * (F21 * la + 2 * F21 * mu) + F12_ * F22 * mu;
    D[0][2] = F11 * (F31 * la + 2 * F31 * mu) + F12_ * F32 * mu;
    D[0][3] = 2 * mu * euv + F11 * F12_ * la + F11 * F12_ * mu;
    D[0][4] = F11 * F22 * la + F12_ * F21 * mu;
    D[0][5] = F11 * F32 * la + F12_ * F31 * mu;
    D[1][1] = F21 * (F21 * la + 2 * F21 * mu) + 2 * mu * euu + la * es + F22 * F22 * mu;
    D[1][2] = F21 * (F31 * la + 2 * F31 * mu) + F22 * F32 * mu;
    D[1][3] = F12_ * F21 * la + F11 * F22 * mu;
    D[1][4] = 2 * mu * euv + F21 * F22 * la + F21 * F22 * mu;
    D[1][5] = F21 * F32 * la + F22 * F31 * mu;
    D[2][2] = F31 * (F31 * la + 2 * F31 * mu) + 2 * mu * euu + la * es + F32 * F32 * mu;
    D[2][3] = F12_ * F31 * la + F11 * F32 * mu;
    D[2][4] = F22 * F31 * la + F21 * F32 * mu;
    D[2][5] = 2 * mu * euv + F31 * F32 * la + F31 * F32 * mu;
    D[3][3] = F12_ * (F12_ * la + 2 * F12_ * mu) + 2 * mu * evv + la * es + F11 * F11 * mu;
    D[3][4] = F12_ * (F22 * la + 2 * F22 * mu) + F11 * F21 * mu;
    D[3][5] = F12_ * (F32 * la + 2 * F32 * mu) + F11 * F31 * mu;
    D[4][4] = F22 * (F22 * la + 2 * F22 * mu) + 2 * mu * evv + la * es + F21 * F21 * mu;
    D[4][5] = F22 * (F32 * la + 2 * F32 * mu) + F21 * F31 * mu;
    D[5][5] = F32 * (F32 * la + 2 * F32 * mu) + 2 * mu * evv + la * es + F31 * F31 * mu;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < i; ++j) D[i][j] = D[j][i];
    double m1, m2;
    if (order == 0) {
        m1 = -Dm[0][0] - Dm[1][0];
        m2 = -Dm[0][1] - Dm[1][1];
        force = force + D3{-F12[0][0] - F12[0][1], -F12[1][0] - F12[1][1], -F12[2][0] - F12[2][1]};
    } else if (order == 1) {
        m1 = Dm[0][0];
        m2 = Dm[0][1];
        force = force + D3{F12[0][0], F12[1][0], F12[2][0]};
    } else {
        m1 = Dm[1][0];
        m2 = Dm[1][1];
        force = force + D3{F12[0][1], F12[1][1], F12[2][1]};
    }
    double HL[3][6];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 6; ++c) HL[r][c] = A * (D[r][c] * m1 + D[r + 3][c] * m2);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) H[r][c] += HL[r][c] * m1 + HL[r][c + 3] * m2;
}

double stvk_energy(const Scene& S, int m, int lf) {
    const Mesh& M = S.m[m];
    const int gb = S.vbase[m];
    const D3 x0 = S.x[gb + M.faces[3 * lf]], x1 = S.x[gb + M.faces[3 * lf + 1]], x2 = S.x[gb + M.faces[3 * lf + 2]];
    const double* Di = &M.dminv[4 * lf];
    const D3 c0 = x1 - x0, c1 = x2 - x0;
    const D3 f0 = Di[0] * c0 + Di[1] * c1, f1 = Di[2] * c0 + Di[3] * c1;
    const double euu = 0.5 * (dotp(f0, f0) - 1), evv = 0.5 * (dotp(f1, f1) - 1), euv = 0.5 * dotp(f0, f1);
    return M.area[lf] * (0.5 * M.prm.lambda_ * (euu + evv) * (euu + evv) + M.prm.miu * (euu * euu + evv * evv + 2 * euv * euv));
}

void bending(const Scene& S, int m, int e, int order, D3 xv, D3 xp, bool damping, D3& force, double H[3][3]) {
    const Mesh& M = S.m[m];
    const EdgeT& E = M.edges[e];
    const int gb = S.vbase[m];
    const D3 X[4] = {S.x[gb + E.v1], S.x[gb + E.v2], S.x[gb + E.n12], S.x[gb + E.n21]};
    const D3 n1 = crossp(X[1] - X[0], X[2] - X[0]);
    const D3 n2 = crossp(X[2] - X[3], X[1] - X[3]);
    const double thr = S.p.degenerate_thres;
    if (dotp(n1, n1) < thr * thr || dotp(n2, n2) < thr * thr) return;
    const double k = M.prm.bending_stiffness;
    const double db = damping ? M.prm.damping_bending / S.p.dt : 0.0;
    const double* Q = &M.Q[16 * e];
    D3 g{0, 0, 0};
    for (int j = 0; j < 4; ++j) g = g + (k * Q[4 * order + j]) * X[j];
    const double hq = k * Q[4 * order + order];
    force = force - (g + (hq * db) * (xv - xp));
    for (int i = 0; i < 3; ++i) H[i][i] += hq * (1.0 + db);
}

void accumulate(const Scene& S, int m, int lv, D3& f, double H[3][3]) {
    const int g = S.vbase[m] + lv;
    const Mesh& M = S.m[m];
    const D3 x = S.x[g], xp = S.xprev[g];
    for (int face : S.vfFaces[g]) vf_force(S, g, face, 3, f, H);
    for (auto& fo : M.vf[lv]) {
        const int gf = S.fbase[m] + fo.first;
        for (int u : S.fvVerts[gf]) vf_force(S, u, gf, fo.second, f, H);
    }
    for (auto& eo : M.ve[lv]) {
        const int ge = S.ebase[m] + eo.first;
        for (int e2 : S.eeOther[ge]) ee_force(S, ge, e2, eo.second, f, H);
    }
    // inertia
    const double mh = M.mass[lv] / (S.p.dt * S.p.dt);
    f = f + mh * (S.y[g] - x);
    for (int i = 0; i < 3; ++i) H[i][i] += mh;
    // StVK with damping on its own Hessian
    double Hm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (auto& fo : M.vf[lv]) stvk_face(S, m, fo.first, fo.second, f, Hm);
    const double dmp = M.prm.damping_stvk / S.p.dt;
    const D3 du = x - xp;
    const double dd[3] = {du.x, du.y, du.z};
    double df[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) df[i] += Hm[i][j] * dmp * dd[j];
    f = f - D3{df[0], df[1], df[2]};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[i][j] += Hm[i][j] * (1.0 + dmp);
    // bending
    for (auto& eo : M.vb[lv]) bending(S, m, eo.first, eo.second, x, xp, true, f, H);
    // world box
    const double xs[3] = {x.x, x.y, x.z};
    const D3 dx = x - xp;
    for (int d = 0; d < 3; ++d) {
        double pen;
        double fd[3] = {0, 0, 0};
        if (xs[d] < S.p.world_lo[d]) {
            pen = S.p.world_lo[d] - xs[d];
            fd[d] = pen * S.p.boundary_contact_stiffness;
        } else if (xs[d] > S.p.world_hi[d]) {
            pen = xs[d] - S.p.world_hi[d];
            fd[d] = -pen * S.p.boundary_contact_stiffness;
        } else {
            continue;
        }
        f = f + D3{fd[0], fd[1], fd[2]};
        H[d][d] += S.p.boundary_contact_stiffness;
        double T0[3] = {0, 0, 0}, T1[3] = {0, 0, 0};
        T0[(d + 1) % 3] = 1;
        T1[(d + 2) % 3] = 1;
        friction(S.p.boundary_friction_dynamic, pen * S.p.boundary_contact_stiffness, D3{T0[0], T0[1], T0[2]},
                 D3{T1[0], T1[1], T1[2]}, dx, S.p.boundary_friction_eps * S.p.dt, 1.0, f, H);
    }
}

void vertex_solve(Scene& S, int m, int lv) {
    const int g = S.vbase[m] + lv;
    D3 f{0, 0, 0};
    double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    accumulate(S, m, lv, f, H);
    const D3 x = S.x[g];
    double sol[3];
    const double b[3] = {f.x, f.y, f.z};
    D3 xn = x;
    if (solve3(H, b, sol)) {
        xn = x + S.p.step_size * D3{sol[0], sol[1], sol[2]};
        const D3 disp = xn - S.xcd[g];
        const double s = std::sqrt(dotp(disp, disp));
        if (s > S.bound[g]) {
            xn = S.xcd[g] + (S.bound[g] / s) * disp;
            S.cdRequired = true;
            ++S.truncations;
        }
    } else {
        ++S.failed;
    }
    S.xnext[g] = xn;
}

void initial_step(Scene& S) {
    const bool hasPrev = S.nInit > 0;
    const D3 g3{S.p.gravity[0], S.p.gravity[1], S.p.gravity[2]};
    for (int m = 0; m < S.ns; ++m) {
        const Mesh& M = S.m[m];
        for (int lv = 0; lv < M.nv; ++lv) {
            const int g = S.vbase[m] + lv;
            const D3 x = S.x[g];
            S.xprev[g] = x;
            D3 vel = S.v[g];
            if (hasPrev) S.acc[g] = (1.0 / S.p.dt) * (vel - S.vprev[g]);
            const D3 vp = vel;
            S.vprev[g] = vel;
            if (S.p.associate_gravity) vel = vel + S.p.dt * g3;
            if (M.fixed[lv]) vel = {0, 0, 0};
            S.v[g] = vel;
            S.y[g] = x + S.p.dt * vel;
            switch (M.prm.init_type) {
                case 0: S.x[g] = S.y[g]; break;
                case 1:
                    if (hasPrev) {
                        const double gn = std::sqrt(dotp(g3, g3));
                        const D3 gd = (1.0 / gn) * g3;
                        double ac = dotp(S.acc[g], gd);
                        ac = ac < gn ? ac : gn;
                        ac = ac > 1e-5 ? ac : 0.0;
                        S.x[g] = (x + S.p.dt * vp) + (S.p.dt * S.p.dt * ac) * gd;
                    } else {
                        S.x[g] = S.y[g];
                    }
                    break;
                case 3: {
                    D3 st = S.y[g] - x;
                    const double sz = std::sqrt(dotp(st, st));
                    if (S.p.handle_collision && sz > S.bound[g] && sz != 0.0) st = (S.bound[g] / sz) * st;
                    S.x[g] = x + st;
                    break;
                }
                default: break;
            }
        }
    }
    ++S.nInit;
}

void velocity_update(Scene& S) {
    for (int m = 0; m < S.ns; ++m) {
        const Mesh& M = S.m[m];
        for (int lv = 0; lv < M.nv; ++lv) {
            const int g = S.vbase[m] + lv;
            D3 vel = (1.0 / S.p.dt) * (S.x[g] - S.xprev[g]);
            const double vm = std::sqrt(dotp(vel, vel));
            if (M.prm.has_no_grav_zone && M.prm.max_velocity > 0 && vel.y > M.prm.no_grav_threshold) {
                if (vm > M.prm.max_velocity) vel = (M.prm.max_velocity / vm) * vel;
            } else if (vm > 1e-6) {
                double vn = vm * M.prm.exp_vel_damping - M.prm.const_vel_damping;
                vn = vn > 1e-6 ? vn : 0.0;
                vel = (vn / vm) * vel;
            } else {
                vel = {0, 0, 0};
            }
            if (M.fixed[lv]) vel = {0, 0, 0};
            S.v[g] = vel;
        }
    }
}

void substep(Scene& S) {
    double omega = 1.0;
    for (int it = 0; it < S.p.iterations; ++it) {
        if (it == 0) std::fill(S.active.begin(), S.active.end(), 0);
        if (S.p.handle_collision) {
            if (it == 0 || S.cdRequired || S.p.cd_every_iteration) detect(S);
        } else if (it == 0) {
            for (int g = 0; g < S.nSimV; ++g) S.bound[g] = double(std::numeric_limits<float>::max());
        }
        if (S.p.apply_acceleration) S.xPrevIter = S.x;
        if (it == 0) initial_step(S);
        for (auto& grp : S.groups) {
            std::vector<char> trunc(1, 0);
            S.pool->run(int64_t(grp.size()), [&](int64_t k) {
                const int m = grp[k].first, lv = grp[k].second;
                if (S.m[m].fixed[lv]) return;
                vertex_solve(S, m, lv);
            });
            for (auto& mv : grp)
                if (!S.m[mv.first].fixed[mv.second]) {
                    const int g = S.vbase[mv.first] + mv.second;
                    S.x[g] = S.xnext[g];
                }
        }
        if (S.p.apply_acceleration) {
            const double rho = double(float(S.p.accelerator_rho));
            const int order = it + 1;
            if (rho == 0.0 || order == 1) omega = 1.0;
            else if (order == 2) omega = 2.0 / (2.0 - rho * rho);
            else omega = 4.0 / (4.0 - rho * rho * omega);
            if (omega > 1.0)
                for (int g = 0; g < S.nSimV; ++g) {
                    if (S.active[g]) continue;
                    D3 xn = omega * (S.x[g] - S.xPrevIter[g]) + S.xPrevIter[g];
                    const D3 disp = xn - S.xcd[g];
                    const double s = std::sqrt(dotp(disp, disp));
                    if (s > S.bound[g]) {
                        xn = S.xcd[g] + (S.bound[g] / s) * disp;
                        S.cdRequired = true;
                    }
                    S.x[g] = xn;
                }
        }
    }
    velocity_update(S);
}

}  // namespace

extern "C" {

const char* cloth_oracle_error(void) { return g_err.c_str(); }

void* cloth_oracle_create(int32_t nmesh, const ClothOracleMesh* meshes, const ClothOracleParams* p, int32_t nthreads) {
    try {
        auto S = std::make_unique<Scene>();
        S->p = *p;
        S->m.resize(nmesh);
        for (int i = 0; i < nmesh; ++i) {
            Mesh& M = S->m[i];
            M.prm = meshes[i];
            M.collider = meshes[i].is_collider != 0;
            M.nv = meshes[i].nv;
            M.nf = meshes[i].nf;
            M.x0.resize(M.nv);
            for (int v = 0; v < M.nv; ++v) M.x0[v] = {meshes[i].X[3 * v], meshes[i].X[3 * v + 1], meshes[i].X[3 * v + 2]};
            M.faces.assign(meshes[i].faces, meshes[i].faces + 3 * size_t(M.nf));
            build_topology(M);
            if (!M.collider) {
                if (i != S->ns) throw std::runtime_error("simulated meshes must precede colliders");
                ++S->ns;
                rest_shape(M);
                M.fixed.assign(meshes[i].fixed, meshes[i].fixed + M.nv);
                for (int c = 0; c < meshes[i].ncolors; ++c)
                    M.colors.emplace_back(meshes[i].color_verts + meshes[i].color_offsets[c],
                                          meshes[i].color_verts + meshes[i].color_offsets[c + 1]);
                std::sort(M.colors.begin(), M.colors.end(),
                          [](const std::vector<int>& a, const std::vector<int>& b) { return a.size() > b.size(); });
            }
        }
        Scene& s = *S;
        s.vbase.assign(nmesh + 1, 0);
        s.fbase.assign(nmesh + 1, 0);
        s.ebase.assign(nmesh + 1, 0);
        for (int i = 0; i < nmesh; ++i) {
            s.vbase[i + 1] = s.vbase[i] + s.m[i].nv;
            s.fbase[i + 1] = s.fbase[i] + s.m[i].nf;
            s.ebase[i + 1] = s.ebase[i] + s.m[i].ne;
        }
        s.nV = s.vbase[nmesh];
        s.nF = s.fbase[nmesh];
        s.nE = s.ebase[nmesh];
        s.nSimV = s.vbase[s.ns];
        s.nSimF = s.fbase[s.ns];
        s.nSimE = s.ebase[s.ns];
        for (int i = 0; i < nmesh; ++i) {
            for (int k = 0; k < s.m[i].nv; ++k) s.vmesh.push_back(i);
            for (int k = 0; k < s.m[i].nf; ++k) s.fmesh.push_back(i);
            for (int k = 0; k < s.m[i].ne; ++k) s.emesh.push_back(i);
        }
        s.x.resize(s.nV);
        for (int i = 0; i < nmesh; ++i)
            for (int k = 0; k < s.m[i].nv; ++k) s.x[s.vbase[i] + k] = s.m[i].x0[k];
        s.xprev = s.x;
        s.y = s.x;
        s.xnext = s.x;
        s.xcd = s.x;
        s.xPrevIter = s.x;
        s.v.assign(s.nV, D3{0, 0, 0});
        s.vprev = s.v;
        s.acc = s.v;
        s.bound.assign(s.nV, double(std::numeric_limits<float>::max()));
        s.active.assign(s.nV, 0);
        s.vfFaces.assign(s.nV, {});
        s.vfMin.assign(s.nV, float(p->max_query_dis));
        s.fMin.assign(s.nF, float(p->max_query_dis));
        s.fvVerts.assign(s.nSimF, {});
        s.eeOther.assign(s.nSimE, {});
        s.eeMin.assign(s.nSimE, float(p->max_query_dis));
        merge_groups(s);
        s.pool.reset(new Pool(nthreads > 0 ? nthreads : int(std::max(1u, std::thread::hardware_concurrency()))));
        return S.release();
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void cloth_oracle_destroy(void* h) { delete static_cast<Scene*>(h); }

void cloth_oracle_step(void* h, int32_t n) {
    Scene& S = *static_cast<Scene*>(h);
    for (int i = 0; i < n; ++i)
        for (int s = 0; s < S.p.num_substeps; ++s) substep(S);
}

void cloth_oracle_get_positions(void* h, int32_t mesh, double* out) {
    Scene& S = *static_cast<Scene*>(h);
    for (int k = 0; k < S.m[mesh].nv; ++k) {
        const D3 x = S.x[S.vbase[mesh] + k];
        out[3 * k] = x.x;
        out[3 * k + 1] = x.y;
        out[3 * k + 2] = x.z;
    }
}

void cloth_oracle_set_positions(void* h, int32_t mesh, const double* in) {
    Scene& S = *static_cast<Scene*>(h);
    for (int k = 0; k < S.m[mesh].nv; ++k) {
        S.x[S.vbase[mesh] + k] = {in[3 * k], in[3 * k + 1], in[3 * k + 2]};
        if (S.m[mesh].collider) S.xprev[S.vbase[mesh] + k] = S.x[S.vbase[mesh] + k];
    }
}

void cloth_oracle_get_velocities(void* h, int32_t mesh, double* out) {
    Scene& S = *static_cast<Scene*>(h);
    for (int k = 0; k < S.m[mesh].nv; ++k) {
        const D3 v = S.v[S.vbase[mesh] + k];
        out[3 * k] = v.x;
        out[3 * k + 1] = v.y;
        out[3 * k + 2] = v.z;
    }
}

void cloth_oracle_detect(void* h) { detect(*static_cast<Scene*>(h)); }

int64_t cloth_oracle_vf_contacts(void* h, int32_t* rows, int64_t cap) {
    Scene& S = *static_cast<Scene*>(h);
    int64_t n = 0;
    for (int g = 0; g < S.nV; ++g)
        for (int f : S.vfFaces[g]) {
            if (n < cap) {
                rows[4 * n] = S.vmesh[g];
                rows[4 * n + 1] = g - S.vbase[S.vmesh[g]];
                rows[4 * n + 2] = S.fmesh[f];
                rows[4 * n + 3] = f - S.fbase[S.fmesh[f]];
            }
            ++n;
        }
    return n;
}

int64_t cloth_oracle_ee_contacts(void* h, int32_t* rows, int64_t cap) {
    Scene& S = *static_cast<Scene*>(h);
    int64_t n = 0;
    for (int e = 0; e < S.nSimE; ++e)
        for (int e2 : S.eeOther[e]) {
            if (n < cap) {
                rows[4 * n] = S.emesh[e];
                rows[4 * n + 1] = e - S.ebase[S.emesh[e]];
                rows[4 * n + 2] = S.emesh[e2];
                rows[4 * n + 3] = e2 - S.ebase[S.emesh[e2]];
            }
            ++n;
        }
    return n;
}

void cloth_oracle_bounds(void* h, int32_t mesh, double* out) {
    Scene& S = *static_cast<Scene*>(h);
    for (int k = 0; k < S.m[mesh].nv; ++k) out[k] = S.bound[S.vbase[mesh] + k];
}

void cloth_oracle_min_distances(void* h, int32_t mesh, float* vf, float* fv, float* ee) {
    Scene& S = *static_cast<Scene*>(h);
    if (vf)
        for (int k = 0; k < S.m[mesh].nv; ++k) vf[k] = S.vfMin[S.vbase[mesh] + k];
    if (fv)
        for (int k = 0; k < S.m[mesh].nf; ++k) fv[k] = S.fMin[S.fbase[mesh] + k];
    if (ee && mesh < S.ns)
        for (int k = 0; k < S.m[mesh].ne; ++k) ee[k] = S.eeMin[S.ebase[mesh] + k];
}

int32_t cloth_oracle_num_edges(void* h, int32_t mesh) { return static_cast<Scene*>(h)->m[mesh].ne; }

void cloth_oracle_topology(void* h, int32_t mesh, int32_t* edges6, int32_t* fe3) {
    const Mesh& M = static_cast<Scene*>(h)->m[mesh];
    for (int e = 0; e < M.ne; ++e) {
        const EdgeT& E = M.edges[e];
        const int32_t r[6] = {E.v1, E.v2, E.n12, E.n21, E.f1, E.f2};
        std::memcpy(edges6 + 6 * e, r, sizeof(r));
    }
    std::memcpy(fe3, M.fedges.data(), M.fedges.size() * sizeof(int32_t));
}

void cloth_oracle_rest(void* h, int32_t mesh, double* dminv4, double* area, double* mass) {
    const Mesh& M = static_cast<Scene*>(h)->m[mesh];
    if (dminv4) std::memcpy(dminv4, M.dminv.data(), M.dminv.size() * sizeof(double));
    if (area) std::memcpy(area, M.area.data(), M.area.size() * sizeof(double));
    if (mass) std::memcpy(mass, M.mass.data(), M.mass.size() * sizeof(double));
}

int32_t cloth_oracle_num_groups(void* h) { return int32_t(static_cast<Scene*>(h)->groups.size()); }

int64_t cloth_oracle_group(void* h, int32_t g, int32_t* pairs) {
    const auto& G = static_cast<Scene*>(h)->groups[g];
    if (pairs)
        for (size_t k = 0; k < G.size(); ++k) {
            pairs[2 * k] = G[k].first;
            pairs[2 * k + 1] = G[k].second;
        }
    return int64_t(G.size());
}

double cloth_oracle_elastic_energy(void* h, int32_t mesh) {
    Scene& S = *static_cast<Scene*>(h);
    const Mesh& M = S.m[mesh];
    double E = 0;
    for (int f = 0; f < M.nf; ++f) E += stvk_energy(S, mesh, f);
    const int gb = S.vbase[mesh];
    for (int e = 0; e < M.ne; ++e) {
        const EdgeT& Ed = M.edges[e];
        if (Ed.f2 == -1) continue;
        const D3 X[4] = {S.x[gb + Ed.v1], S.x[gb + Ed.v2], S.x[gb + Ed.n12], S.x[gb + Ed.n21]};
        double q = 0;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) q += M.Q[16 * e + 4 * i + j] * dotp(X[i], X[j]);
        E += 0.5 * M.prm.bending_stiffness * q;
    }
    return E;
}

void cloth_oracle_elastic_force_hessian(void* h, int32_t mesh, int32_t v, double* f3, double* h9) {
    Scene& S = *static_cast<Scene*>(h);
    const Mesh& M = S.m[mesh];
    D3 f{0, 0, 0};
    double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (auto& fo : M.vf[v]) stvk_face(S, mesh, fo.first, fo.second, f, H);
    const D3 x = S.x[S.vbase[mesh] + v];
    for (auto& eo : M.vb[v]) bending(S, mesh, eo.first, eo.second, x, x, false, f, H);
    f3[0] = f.x;
    f3[1] = f.y;
    f3[2] = f.z;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) h9[3 * i + j] = H[i][j];
}

void cloth_oracle_vertex_force_hessian(void* h, int32_t mesh, int32_t v, double* f3, double* h9) {
    Scene& S = *static_cast<Scene*>(h);
    D3 f{0, 0, 0};
    double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    accumulate(S, mesh, v, f, H);
    f3[0] = f.x;
    f3[1] = f.y;
    f3[2] = f.z;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) h9[3 * i + j] = H[i][j];
}

int64_t cloth_oracle_counter(void* h, int32_t which) {
    Scene& S = *static_cast<Scene*>(h);
    return which == 0 ? S.detections : (which == 1 ? S.truncations.load() : S.failed.load());
}

}  // extern "C"
