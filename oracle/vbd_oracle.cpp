// CPU oracle for the VBD step — TEST INFRASTRUCTURE ONLY (see vbd_oracle.h).
//
// Each function cites the reference file:line it restates. Paths are relative
// to the reference project's Simulator/Modules directory.
#include "vbd_oracle.h"
#include "tet_contact.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <string>
#include <functional>
#include <mutex>
#include <queue>
#include <set>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Vertex graph of a tet mesh: every pair of vertices that shares a tet, as a
// sorted edge set. GraphColoring/TetMeshVertexGraph.h:14-41 (edges of a tet
// mesh = all 6 vertex pairs of every tet), ColoringAlgorithms.cpp:11-26.
// ---------------------------------------------------------------------------
std::vector<std::vector<int>> vertex_graph(int nv, int ntet, const int32_t* tets) {
    std::set<std::array<int, 2>> edges;
    for (int t = 0; t < ntet; ++t)
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j) {
                int a = tets[4 * t + i], b = tets[4 * t + j];
                if (a == b) continue;
                edges.insert({std::min(a, b), std::max(a, b)});
            }
    std::vector<std::vector<int>> g(nv);
    for (auto& e : edges) {
        g[e[0]].push_back(e[1]);
        g[e[1]].push_back(e[0]);
    }
    return g;
}

// ---------------------------------------------------------------------------
// Thread pool: persistent workers, one parallel-for at a time.
// Stands in for the reference's TBB cpu_parallel_for
// (Parallelization/CPUParallelization.h:19-28).
// ---------------------------------------------------------------------------
class Pool {
public:
    explicit Pool(int n) : n_(std::max(1, n)) {
        for (int i = 1; i < n_; ++i) workers_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    int size() const { return n_; }
    void run(int64_t n, const std::function<void(int64_t, int64_t)>& fn) {
        if (n <= 0) return;
        if (n_ == 1 || n < 64) { fn(0, n); return; }
        fn_ = &fn;
        total_ = n;
        chunk_ = std::max<int64_t>(16, n / (int64_t(n_) * 8));
        next_.store(0);
        done_.store(0);
        {
            std::lock_guard<std::mutex> lk(m_);
            ++gen_;
        }
        cv_.notify_all();
        work();
        while (done_.load(std::memory_order_acquire) < n_ - 1) std::this_thread::yield();
    }

private:
    void work() {
        for (;;) {
            int64_t s = next_.fetch_add(chunk_);
            if (s >= total_) break;
            (*fn_)(s, std::min(total_, s + chunk_));
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            work();
            done_.fetch_add(1, std::memory_order_release);
        }
    }
    int n_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_;
    uint64_t gen_ = 0;
    bool stop_ = false;
    const std::function<void(int64_t, int64_t)>* fn_ = nullptr;
    int64_t total_ = 0, chunk_ = 1;
    std::atomic<int64_t> next_{0};
    std::atomic<int> done_{0};
};

// ---------------------------------------------------------------------------
// 3x3 symmetric solve used in place of CuMatrix::solve3x3_psd_stable, whose
// source is not in the reference tree (call sites VBDPhysics.cpp:2439-2450,
// VBDPhysicsCompute.cu:896). LDL^T without pivoting; fails when a pivot is
// not above rel_tol * max|diag|. The CUDA path uses the same algorithm.
// ---------------------------------------------------------------------------
template <typename R>
bool solve3x3_ldlt(const R* H, const R* b, R* x, R rel_tol) {
    R scale = std::max(std::fabs(H[0]), std::max(std::fabs(H[4]), std::fabs(H[8])));
    if (!(scale > R(0))) return false;
    R tol = rel_tol * scale;
    R d0 = H[0];
    if (!(d0 > tol)) return false;
    R l10 = H[3] / d0, l20 = H[6] / d0;
    R d1 = H[4] - l10 * H[3];
    if (!(d1 > tol)) return false;
    R l21 = (H[7] - l20 * H[3]) / d1;
    R d2 = H[8] - l20 * H[6] - l21 * l21 * d1;
    if (!(d2 > tol)) return false;
    R z0 = b[0];
    R z1 = b[1] - l10 * z0;
    R z2 = b[2] - l20 * z0 - l21 * z1;
    z0 /= d0; z1 /= d1; z2 /= d2;
    x[2] = z2;
    x[1] = z1 - l21 * x[2];
    x[0] = z0 - l10 * x[1] - l20 * x[2];
    return std::isfinite(x[0]) && std::isfinite(x[1]) && std::isfinite(x[2]);
}

// The solve policy of the mixed-precision path: FP32 attempt, FP64 retry
// when the FP32 pivots are too small, failure only when FP64 fails too. The retry
// solves an FP32-accumulated block, whose pivots below 2e-6 of the largest diagonal
// are rounding noise: it treats them as singular (the same thresholds as the GPU).
template <typename R>
bool solve3x3(const R* H, const R* b, R* x, int* fp64_used);
template <>
bool solve3x3<double>(const double* H, const double* b, double* x, int*) {
    return solve3x3_ldlt<double>(H, b, x, 1e-12);
}
template <>
bool solve3x3<float>(const float* H, const float* b, float* x, int* fp64_used) {
    if (solve3x3_ldlt<float>(H, b, x, 1e-5f)) return true;
    double Hd[9], bd[3], xd[3];
    for (int i = 0; i < 9; ++i) Hd[i] = H[i];
    for (int i = 0; i < 3; ++i) bd[i] = b[i];
    if (fp64_used) ++*fp64_used;
    if (!solve3x3_ldlt<double>(Hd, bd, xd, 2e-6)) return false;
    for (int i = 0; i < 3; ++i) x[i] = float(xd[i]);
    return true;
}

// ---------------------------------------------------------------------------
// Per-mesh and scene state.
// ---------------------------------------------------------------------------
template <typename R>
struct Mesh {
    int nv = 0, ntet = 0;
    std::vector<R> x, xprev, v, vprev, y;     // 3*nv
    std::vector<int32_t> tets;                // 4*ntet
    std::vector<R> dminv;                     // 9*ntet, column-major (TetMeshFEM.cpp:409-418)
    std::vector<R> vol;                       // ntet
    std::vector<R> mass;                      // nv
    std::vector<int32_t> nbr_ofs, nbr_tet, nbr_order;  // CSR vertex -> incident tets
    std::vector<int8_t> fixed;
    std::vector<std::vector<int32_t>> colors; // sorted by size, descending
    R miu, lmbd, density, kh, kd, exp_damp, const_damp, fr_mu, fr_eps;
    int init_type = 0;
    bool active = true;
    // accelerator buffers (VBDPhysicsCompute.cu:910-944)
    std::vector<R> prev_iter, prevprev_iter;
    // contact: surface, detector results per surface vertex, and the per-vertex
    // records of VBD_BaseMeshGPU.h:18-43 (v side: face mesh + face vertices; up to
    // four relations to contacts whose face holds this vertex: mesh, vertex, order)
    oracle_tc::Surface surf;
    std::vector<oracle_tc::CcdHit> hits;
    std::vector<char> penetrated;             // per surface vertex: DCD found it inside a tet
    std::vector<char> col_active, col_mask;
    std::vector<int32_t> col_fmesh, col_fv, col_face, col_kind, col_nrel, col_rel;
};

struct Deformer {
    int type;
    double center[3], axis[3], omega, end_time, speed[3];
    std::vector<int32_t> sel_mesh, sel_vert;
    std::vector<std::array<double, 3>> root, rootp, orig;
};

struct SceneBase {
    virtual ~SceneBase() {}
};

template <typename R>
struct Scene : SceneBase {
    std::vector<Mesh<R>> meshes;
    OracleParams p;
    double dt, dt2inv, cur_time = 0.0;
    std::vector<std::vector<int32_t>> groups;  // (mesh, vertex) pairs
    std::vector<Deformer> defs;
    Pool* pool = nullptr;
    std::atomic<int> fp64_solves{0};
    std::atomic<int> failures{0};
    ~Scene() { delete pool; }
};

// Rest shape: TetMeshFEM.cpp:409-429 (Dm = [x1-x0, x2-x0, x3-x0], DmInv = Dm^-1,
// volume = det(Dm)/6, lumped mass += density*volume/4), computed in double.
template <typename R>
void rest_shape(Mesh<R>& m) {
    m.dminv.assign(9 * size_t(m.ntet), R(0));
    m.vol.assign(m.ntet, R(0));
    std::vector<double> mass(m.nv, 0.0);
    for (int t = 0; t < m.ntet; ++t) {
        const int32_t* tv = &m.tets[4 * size_t(t)];
        double D[9];  // column-major
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                D[3 * c + r] = double(m.x[3 * size_t(tv[c + 1]) + r]) - double(m.x[3 * size_t(tv[0]) + r]);
        // cofactor inverse of a column-major 3x3
        auto A = [&](int r, int c) { return D[3 * c + r]; };
        double c00 = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
        double c01 = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
        double c02 = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
        double det = A(0, 0) * c00 + A(0, 1) * c01 + A(0, 2) * c02;
        double inv[9];
        double id = 1.0 / det;
        // inverse(r,c) = cofactor(c,r)/det, stored column-major
        inv[0 + 3 * 0] = c00 * id;
        inv[0 + 3 * 1] = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) * id;
        inv[0 + 3 * 2] = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) * id;
        inv[1 + 3 * 0] = c01 * id;
        inv[1 + 3 * 1] = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) * id;
        inv[1 + 3 * 2] = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) * id;
        inv[2 + 3 * 0] = c02 * id;
        inv[2 + 3 * 1] = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) * id;
        inv[2 + 3 * 2] = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) * id;
        for (int i = 0; i < 9; ++i) m.dminv[9 * size_t(t) + i] = R(inv[i]);
        double vol = det / 6.0;
        m.vol[t] = R(vol);
        for (int i = 0; i < 4; ++i) mass[tv[i]] += 0.25 * vol * double(m.density);
    }
    m.mass.resize(m.nv);
    for (int i = 0; i < m.nv; ++i) m.mass[i] = R(mass[i]);
}

// CSR vertex -> incident tets with the vertex's order in each tet
// (TetMesh/TetMeshFEM.cpp:276-324). Incident tets are listed in ascending tet id.
template <typename R>
void build_adjacency(Mesh<R>& m) {
    std::vector<int32_t> cnt(m.nv + 1, 0);
    for (int t = 0; t < m.ntet; ++t)
        for (int i = 0; i < 4; ++i) cnt[m.tets[4 * size_t(t) + i] + 1]++;
    for (int i = 0; i < m.nv; ++i) cnt[i + 1] += cnt[i];
    m.nbr_ofs = cnt;
    m.nbr_tet.assign(cnt[m.nv], 0);
    m.nbr_order.assign(cnt[m.nv], 0);
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int t = 0; t < m.ntet; ++t)
        for (int i = 0; i < 4; ++i) {
            int v = m.tets[4 * size_t(t) + i];
            m.nbr_tet[fill[v]] = t;
            m.nbr_order[fill[v]] = i;
            fill[v]++;
        }
}

// Neo-Hookean force and Hessian of one tet on one of its vertices, restating
// VBD_NeoHookean.cpp:379-581 (accumlateMaterialForceAndHessian2): the 9x9
// d2E/dF2 = A*lambda*(g g^T + (detF - a) * d2det/dF2) contracted with the
// vertex's row of dF/dx, mu*A*|m|^2 added on the 3x3 diagonal, and the
// Rayleigh-like damping Hessian (k_h * H_lambda + k_d * mu*A*|m|^2 I)/dt.
// xt: the tet's 4 vertex positions (3 each); disp = x_v - x_prev,v of the vertex;
// force (3) and H (9, row-major) are accumulated.
template <typename R>
void tet_force_hessian(const R* xt, const R* Dinv, R A, int ord, R miu, R lmbd, R kh, R kd, R dt, const R* disp,
                       R* force, R* H) {
    const R a = R(1) + miu / lmbd;
    R Ds[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Ds[3 * c + r] = xt[3 * (c + 1) + r] - xt[r];
    R F[9];  // column-major F = Ds * DmInv
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            R s = 0;
            for (int q = 0; q < 3; ++q) s += Ds[3 * q + r] * Dinv[3 * c + q];
            F[3 * c + r] = s;
        }
    auto f = [&](int r, int c) { return F[3 * c + r]; };
    // d(det F)/dF, column-major (VBD_NeoHookean.cpp:424-433)
    R g[9];
    g[0] = f(1, 1) * f(2, 2) - f(1, 2) * f(2, 1);
    g[1] = f(0, 2) * f(2, 1) - f(0, 1) * f(2, 2);
    g[2] = f(0, 1) * f(1, 2) - f(0, 2) * f(1, 1);
    g[3] = f(1, 2) * f(2, 0) - f(1, 0) * f(2, 2);
    g[4] = f(0, 0) * f(2, 2) - f(0, 2) * f(2, 0);
    g[5] = f(0, 2) * f(1, 0) - f(0, 0) * f(1, 2);
    g[6] = f(1, 0) * f(2, 1) - f(1, 1) * f(2, 0);
    g[7] = f(0, 1) * f(2, 0) - f(0, 0) * f(2, 1);
    g[8] = f(0, 0) * f(1, 1) - f(0, 1) * f(1, 0);
    R detF = f(0, 0) * g[0] + f(1, 0) * g[1] + f(2, 0) * g[2];
    R kk = detF - a;
    // d2E/dF2 without the mu term (VBD_NeoHookean.cpp:436-494), times A.
    // The second derivative of det F: d2J/dF_pj dF_ql = sum_rs eps_pqr eps_jls F_rs,
    // which has a single non-zero term (r = 3-p-q, s = 3-j-l) when p != q and j != l.
    auto eps = [](int a, int b, int c) { return (a - b) * (b - c) * (c - a) / 2; };
    R d2[9][9];
    for (int j = 0; j < 3; ++j)
        for (int p = 0; p < 3; ++p)
            for (int l = 0; l < 3; ++l)
                for (int q = 0; q < 3; ++q) {
                    int I = p + 3 * j, J = q + 3 * l;
                    R hd = 0;
                    if (p != q && j != l) {
                        int r = 3 - p - q, s = 3 - j - l;
                        hd = R(eps(p, q, r) * eps(j, l, s)) * f(r, s);
                    }
                    d2[I][J] = (g[I] * g[J] + kk * hd) * lmbd * A;
                }
    R dEdF[9];
    for (int i = 0; i < 9; ++i) dEdF[i] = A * (miu * F[i] + lmbd * kk * g[i]);
    // rows of dF/dx: VBD_NeoHookean.cpp:526-553
    R mv[3];
    if (ord == 0) {
        for (int c = 0; c < 3; ++c) mv[c] = -Dinv[3 * c + 0] - Dinv[3 * c + 1] - Dinv[3 * c + 2];
    } else {
        for (int c = 0; c < 3; ++c) mv[c] = Dinv[3 * c + (ord - 1)];
    }
    R dEdx[3], Hl[9];
    for (int i = 0; i < 3; ++i) {
        R s = 0;
        for (int j = 0; j < 3; ++j) s += dEdF[i + 3 * j] * mv[j];
        dEdx[i] = s;
    }
    for (int i = 0; i < 3; ++i)
        for (int q = 0; q < 3; ++q) {
            R s = 0;
            for (int j = 0; j < 3; ++j)
                for (int l = 0; l < 3; ++l) s += mv[j] * mv[l] * d2[i + 3 * j][q + 3 * l];
            Hl[3 * i + q] = s;
        }
    R dampH[9];
    for (int i = 0; i < 9; ++i) dampH[i] = Hl[i] * kh;
    R tmp = (mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]) * miu * A;
    Hl[0] += tmp; Hl[4] += tmp; Hl[8] += tmp;
    tmp *= kd;
    dampH[0] += tmp; dampH[4] += tmp; dampH[8] += tmp;
    for (int i = 0; i < 9; ++i) dampH[i] /= dt;
    for (int i = 0; i < 3; ++i) {
        R df = dampH[3 * i + 0] * disp[0] + dampH[3 * i + 1] * disp[1] + dampH[3 * i + 2] * disp[2];
        force[i] -= dEdx[i] + df;
    }
    for (int i = 0; i < 9; ++i) H[i] += Hl[i] + dampH[i];
}

// Neo-Hookean per-vertex force and Hessian: the incident tets in ascending id.
template <typename R>
void material_force_hessian(const Mesh<R>& m, int iv, R dt, R* force, R* H) {
    R disp[3];
    for (int d = 0; d < 3; ++d) disp[d] = m.x[3 * size_t(iv) + d] - m.xprev[3 * size_t(iv) + d];
    for (int k = m.nbr_ofs[iv]; k < m.nbr_ofs[iv + 1]; ++k) {
        int t = m.nbr_tet[k];
        const int32_t* tv = &m.tets[4 * size_t(t)];
        R xt[12];
        for (int j = 0; j < 4; ++j)
            for (int r = 0; r < 3; ++r) xt[3 * j + r] = m.x[3 * size_t(tv[j]) + r];
        tet_force_hessian<R>(xt, &m.dminv[9 * size_t(t)], m.vol[t], m.nbr_order[k], m.miu, m.lmbd, m.kh, m.kd, dt,
                             disp, force, H);
    }
}

// IPC-style lagged friction (VBDPhysics.cpp:2563-2592, computeVertexFriction).
// T is 3x2 column-major: T[0..2] first tangent, T[3..5] second.
template <typename R>
void vertex_friction(R mu, R lambda, const R* T, const R* u, R epsU, R* force, R* H) {
    R un = std::sqrt(u[0] * u[0] + u[1] * u[1]);
    if (!(un > R(0))) return;
    R f1;
    if (un > epsU) f1 = R(1) / un;
    else f1 = (-un / epsU + R(2)) / epsU;
    R s = mu * lambda * f1;
    for (int r = 0; r < 3; ++r) {
        force[r] += -s * (T[r] * u[0] + T[3 + r] * u[1]);
        for (int c = 0; c < 3; ++c) H[3 * r + c] += s * (T[r] * T[c] + T[3 + r] * T[3 + c]);
    }
}

// Plane-ground / world-box penalty with friction on every violated axis
// (VBDPhysics.cpp:2858-2953, the usePlaneGround branch).
template <typename R>
void boundary_force_hessian(const Scene<R>& s, const Mesh<R>& m, int iv, bool apply_friction, R* force, R* H) {
    if (!s.p.use_plane_ground) return;
    const R k = R(s.p.boundary_stiffness);
    const R* x = &m.x[3 * size_t(iv)];
    for (int d = 0; d < 3; ++d) {
        R lo = R(s.p.world_lo[d]), hi = R(s.p.world_hi[d]);
        R depth;
        if (x[d] < lo) {
            depth = lo - x[d];
            force[d] += depth * k;
        } else if (x[d] > hi) {
            depth = x[d] - hi;
            force[d] -= depth * k;
        } else {
            continue;
        }
        H[4 * d] += k;
        if (apply_friction) {
            R dx[3];
            for (int c = 0; c < 3; ++c) dx[c] = x[c] - m.xprev[3 * size_t(iv) + c];
            R T[6] = {0, 0, 0, 0, 0, 0};
            T[(d + 1) % 3] = 1;
            T[3 + (d + 2) % 3] = 1;
            R u[2] = {T[0] * dx[0] + T[1] * dx[1] + T[2] * dx[2], T[3] * dx[0] + T[4] * dx[1] + T[5] * dx[2]};
            R lambda = depth * k;
            R epsU = R(s.p.boundary_friction_eps_v) * R(s.dt);
            vertex_friction<R>(R(s.p.boundary_friction_mu), lambda, T, u, epsU, force, H);
        }
    }
}

// Inertia: VBD_BaseMaterial.h:359-366.
template <typename R>
void inertia_force_hessian(const Scene<R>& s, const Mesh<R>& m, int iv, R* force, R* H) {
    R w = m.mass[iv] * R(s.dt2inv);
    for (int d = 0; d < 3; ++d) force[d] += w * (m.y[3 * size_t(iv) + d] - m.x[3 * size_t(iv) + d]);
    H[0] += w; H[4] += w; H[8] += w;
}

// ---------------------------------------------------------------------------
// Tet-mesh contact (v-f): detection at the start of a substep, the contact
// records, and the per-contact force and Hessian.
// ---------------------------------------------------------------------------

// Closest point on triangle abc (VBD/VBD_GeneralCompute.h:180-268, the Voronoi
// region walk of Ericson's "Real-Time Collision Detection" 5.1.5). 6 = interior.
template <typename R>
int closest_point_triangle(const R* p, const R* a, const R* b, const R* c, R* bary, R* cp) {
    R ab[3], ac[3], ap[3], bp[3], cpv[3];
    for (int d = 0; d < 3; ++d) {
        ab[d] = b[d] - a[d];
        ac[d] = c[d] - a[d];
        ap[d] = p[d] - a[d];
    }
    auto dot = [](const R* u, const R* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
    const R d1 = dot(ab, ap), d2 = dot(ac, ap);
    auto set = [&](R u, R v, R w) {
        bary[0] = u; bary[1] = v; bary[2] = w;
        for (int d = 0; d < 3; ++d) cp[d] = u * a[d] + v * b[d] + w * c[d];
    };
    if (d1 <= 0 && d2 <= 0) { set(1, 0, 0); for (int d = 0; d < 3; ++d) cp[d] = a[d]; return 0; }
    for (int d = 0; d < 3; ++d) bp[d] = p[d] - b[d];
    const R d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) { set(0, 1, 0); for (int d = 0; d < 3; ++d) cp[d] = b[d]; return 1; }
    for (int d = 0; d < 3; ++d) cpv[d] = p[d] - c[d];
    const R d5 = dot(ab, cpv), d6 = dot(ac, cpv);
    if (d6 >= 0 && d5 <= d6) { set(0, 0, 1); for (int d = 0; d < 3; ++d) cp[d] = c[d]; return 2; }
    const R vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        const R v = d1 / (d1 - d3);
        bary[0] = 1 - v; bary[1] = v; bary[2] = 0;
        for (int d = 0; d < 3; ++d) cp[d] = a[d] + v * ab[d];
        return 3;
    }
    const R vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
        const R v = d2 / (d2 - d6);
        bary[0] = 1 - v; bary[1] = 0; bary[2] = v;
        for (int d = 0; d < 3; ++d) cp[d] = a[d] + v * ac[d];
        return 5;
    }
    const R va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        const R v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary[0] = 0; bary[1] = 1 - v; bary[2] = v;
        for (int d = 0; d < 3; ++d) cp[d] = b[d] + v * (c[d] - b[d]);
        return 4;
    }
    const R denom = R(1) / (va + vb + vc);
    const R v = vb * denom, w = vc * denom;
    bary[0] = 1 - v - w; bary[1] = v; bary[2] = w;
    for (int d = 0; d < 3; ++d) cp[d] = a[d] + v * ab[d] + w * ac[d];
    return 6;
}

// accumlateCollisionForceAndHessianPerCollision_v2 (VBDPhysicsCompute.cu:1812-1930):
// the contact of vertex qv of mesh qm with its recorded face, evaluated at the current
// positions, acting on the vertex of that contact with index `order` (3 = the
// colliding vertex, 0..2 = a face vertex): penalty k * depth along the face normal
// (interior) or along the closest-point direction, with lagged IPC friction in the
// frame (edge AB, edge x normal); force * b and Hessian * b^2 with b = 1 for the
// vertex and -barycentric for a face vertex.
template <typename R>
void contact_term(const Scene<R>& s, int qm, int qv, int order, R* force, R* H) {
    const Mesh<R>& Q = s.meshes[qm];
    const Mesh<R>& F = s.meshes[Q.col_fmesh[qv]];
    const int32_t* fv = &Q.col_fv[3 * size_t(qv)];
    const R* p = &Q.x[3 * size_t(qv)];
    const R* A = &F.x[3 * size_t(fv[0])];
    const R* B = &F.x[3 * size_t(fv[1])];
    const R* C = &F.x[3 * size_t(fv[2])];
    R bary[3], cp[3];
    const int type = closest_point_triangle<R>(p, A, B, C, bary, cp);
    R e1[3], e2[3], fn[3], diff[3], n[3];
    for (int d = 0; d < 3; ++d) {
        e1[d] = B[d] - A[d];
        e2[d] = C[d] - A[d];
        diff[d] = cp[d] - p[d];
    }
    fn[0] = e1[1] * e2[2] - e1[2] * e2[1];
    fn[1] = e1[2] * e2[0] - e1[0] * e2[2];
    fn[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const R fl = std::sqrt(fn[0] * fn[0] + fn[1] * fn[1] + fn[2] * fn[2]);
    for (int d = 0; d < 3; ++d) fn[d] /= fl;
    if (type == 6) {
        for (int d = 0; d < 3; ++d) n[d] = fn[d];
    } else {
        const R inv = R(1) / std::sqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
        for (int d = 0; d < 3; ++d) n[d] = diff[d] * inv;
        if (n[0] * fn[0] + n[1] * fn[1] + n[2] * fn[2] < 0)
            for (int d = 0; d < 3; ++d) n[d] = -n[d];
    }
    const R depth = diff[0] * n[0] + diff[1] * n[1] + diff[2] * n[2];
    if (!(depth > 0)) return;
    const R b = order == 3 ? R(1) : -bary[order];
    const R k = R(s.p.collision_stiffness);
    const R lambda = depth * k;
    R cf[3], cH[9];
    for (int r = 0; r < 3; ++r) {
        cf[r] = n[r] * lambda;
        for (int c = 0; c < 3; ++c) cH[3 * r + c] = n[r] * n[c] * k;
    }
    R dx[3];
    for (int d = 0; d < 3; ++d) {
        const R d3 = p[d] - Q.xprev[3 * size_t(qv) + d];
        const R d0 = A[d] - F.xprev[3 * size_t(fv[0]) + d];
        const R d1 = B[d] - F.xprev[3 * size_t(fv[1]) + d];
        const R d2 = C[d] - F.xprev[3 * size_t(fv[2]) + d];
        dx[d] = d3 - (bary[0] * d0 + bary[1] * d1 + bary[2] * d2);
    }
    R t0[3] = {e1[0], e1[1], e1[2]};
    const R l0 = std::sqrt(t0[0] * t0[0] + t0[1] * t0[1] + t0[2] * t0[2]);
    for (int d = 0; d < 3; ++d) t0[d] /= l0;
    R t1[3] = {t0[1] * n[2] - t0[2] * n[1], t0[2] * n[0] - t0[0] * n[2], t0[0] * n[1] - t0[1] * n[0]};
    const R l1 = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (int d = 0; d < 3; ++d) t1[d] /= l1;
    const R T[6] = {t0[0], t0[1], t0[2], t1[0], t1[1], t1[2]};
    const R u[2] = {t0[0] * dx[0] + t0[1] * dx[1] + t0[2] * dx[2], t1[0] * dx[0] + t1[1] * dx[1] + t1[2] * dx[2]};
    const R mu = (Q.fr_mu + F.fr_mu) * R(0.5);
    const R epsV = (Q.fr_eps + F.fr_eps) * R(0.5);
    vertex_friction<R>(mu, lambda, T, u, epsV * R(s.dt), cf, cH);
    for (int r = 0; r < 3; ++r) force[r] += b * cf[r];
    for (int i = 0; i < 9; ++i) H[i] += b * b * cH[i];
}

// accumulateCollisionForceAndHessian (VBDPhysicsCompute.cu:1731-1773): the vertex's
// own contact, then its relations in record order.
template <typename R>
void collision_force_hessian(const Scene<R>& s, int im, int iv, R* force, R* H) {
    const Mesh<R>& m = s.meshes[im];
    if (m.col_active.empty()) return;
    if (m.col_active[iv]) contact_term(s, im, iv, 3, force, H);
    for (int j = 0; j < m.col_nrel[iv]; ++j) {
        const int32_t* r = &m.col_rel[12 * size_t(iv) + 3 * j];
        contact_term(s, r[0], r[1], r[2], force, H);
    }
}

// prepareCollisionDataGPU (VBDPhysics.cpp:1812-1894): clear, then, mesh by mesh and
// surface vertex by surface vertex, record every hit as the vertex's contact and
// append a relation to each of the face's vertices that has fewer than four.
template <typename R>
void build_contact_records(Scene<R>& s) {
    for (auto& m : s.meshes) {
        m.col_active.assign(size_t(m.nv), 0);
        m.col_mask.assign(size_t(m.nv), 0);
        m.col_nrel.assign(size_t(m.nv), 0);
        m.col_fmesh.assign(size_t(m.nv), -1);
        m.col_face.assign(size_t(m.nv), -1);
        m.col_kind.assign(size_t(m.nv), 0);
        m.col_fv.assign(3 * size_t(m.nv), -1);
        m.col_rel.assign(12 * size_t(m.nv), -1);
    }
    for (size_t im = 0; im < s.meshes.size(); ++im) {
        auto& m = s.meshes[im];
        for (size_t i = 0; i < m.surf.verts.size(); ++i) {
            const oracle_tc::CcdHit& h = m.hits[i];
            if (h.face < 0) continue;
            const int v = m.surf.verts[i];
            m.col_active[v] = 1;
            m.col_mask[v] = 1;
            m.col_fmesh[v] = h.fmesh;
            m.col_face[v] = h.face;
            m.col_kind[v] = h.tt < 0.f ? 2 : 1;
            auto& F = s.meshes[h.fmesh];
            for (int j = 0; j < 3; ++j) {
                const int fv = F.surf.faces[3 * size_t(h.face) + j];
                m.col_fv[3 * size_t(v) + j] = fv;
                if (F.col_nrel[fv] < 4) {
                    int32_t* r = &F.col_rel[12 * size_t(fv) + 3 * F.col_nrel[fv]];
                    r[0] = int32_t(im);
                    r[1] = v;
                    r[2] = j;
                    F.col_nrel[fv]++;
                    F.col_mask[fv] = 1;
                }
            }
        }
    }
}

// Contact detection of one substep (VBDPhysics.cpp:1958-2035 dcd, 2078-2116 ccd) or of
// an intermediate pass (:2037-2076, 2118-2156), on FP32 copies of the positions:
//   substep start: DCD (run before the initial step, so on the previous positions) for
//   the surface vertices below collisionOffHeight, marking the ones inside a tet as
//   penetrated; without DCD all results are cleared; then CCD for the vertices below
//   the height that DCD did not mark;
//   intermediate: DCD (current positions) for the penetrated vertices, or for all when
//   CCD is off; CCD as above on the current positions.
// Entries the reference does not revisit keep their previous result.
template <typename R>
void detect_contacts(Scene<R>& s, bool intermediate) {
    const bool ccd = s.p.allow_ccd != 0, dcd = s.p.allow_dcd != 0;
    if (!ccd && !dcd) return;
    const float off = float(s.p.collision_off_height);
    oracle_tc::DcdParams dp;
    dp.handle_self = s.p.handle_self_collision != 0;
    dp.check_feasible = s.p.check_feasible_region != 0;
    dp.feasible_eps = float(s.p.feasible_region_eps);
    dp.check_traverse = s.p.check_tet_traverse != 0;
    dp.traverse_non_self = s.p.traverse_non_self != 0;
    dp.stop_after_passing = s.p.stop_traversing_after_passing != 0;
    dp.shift_to_center = s.p.shift_query_to_center != 0;
    dp.static_traverse = s.p.use_static_traverse != 0;
    dp.center_shift = float(s.p.center_shift_level);
    dp.ray_eps = float(s.p.ray_tri_eps);
    dp.max_search_mult = float(s.p.max_search_mult);
    std::vector<std::vector<float>> xf(s.meshes.size()), pf(s.meshes.size());
    std::vector<oracle_tc::CcdMesh> cm(s.meshes.size());
    for (size_t im = 0; im < s.meshes.size(); ++im) {
        auto& m = s.meshes[im];
        xf[im].resize(m.x.size());
        pf[im].resize(m.x.size());
        for (size_t i = 0; i < m.x.size(); ++i) {
            xf[im][i] = float(m.x[i]);
            pf[im][i] = float(m.xprev[i]);
        }
        cm[im] = oracle_tc::CcdMesh{xf[im].data(), pf[im].data(), &m.surf, m.ntet, m.tets.data()};
        if (m.hits.size() != m.surf.verts.size()) m.hits.assign(m.surf.verts.size(), oracle_tc::CcdHit{});
        if (m.penetrated.size() != m.surf.verts.size()) m.penetrated.assign(m.surf.verts.size(), 0);
    }
    oracle_tc::Detector det(cm);
    auto height = [&](size_t im, size_t i, bool prev) {
        return (prev ? pf : xf)[im][3 * size_t(s.meshes[im].surf.verts[i]) + 1];
    };
    if (dcd) {
        det.build_tets(!intermediate);
        for (size_t im = 0; im < s.meshes.size(); ++im) {
            auto& m = s.meshes[im];
            if (!intermediate) std::fill(m.penetrated.begin(), m.penetrated.end(), 0);
            for (size_t i = 0; i < m.surf.verts.size(); ++i) {
                const bool query = intermediate ? (m.penetrated[i] || !ccd) : height(im, i, true) < off;
                if (!query) continue;
                oracle_tc::CcdHit h;
                const bool inside = det.dcd(int(im), int(i), dp, h);
                m.hits[i] = h;
                if (inside && !intermediate) m.penetrated[i] = 1;
            }
        }
    } else if (!intermediate) {
        for (auto& m : s.meshes) std::fill(m.hits.begin(), m.hits.end(), oracle_tc::CcdHit{});
    }
    if (ccd) {
        det.build_swept();
        for (size_t im = 0; im < s.meshes.size(); ++im) {
            auto& m = s.meshes[im];
            for (size_t i = 0; i < m.surf.verts.size(); ++i)
                if (height(im, i, false) < off && !m.penetrated[i]) m.hits[i] = det.ccd(int(im), int(i));
        }
    }
    build_contact_records(s);
}

template <typename R>
void vertex_force_hessian(const Scene<R>& s, const Mesh<R>& m, int iv, bool apply_friction, R* force, R* H) {
    for (int i = 0; i < 3; ++i) force[i] = 0;
    for (int i = 0; i < 9; ++i) H[i] = 0;
    material_force_hessian(m, iv, R(s.dt), force, H);
    inertia_force_hessian(s, m, iv, force, H);
    collision_force_hessian(s, int(&m - s.meshes.data()), iv, force, H);
    boundary_force_hessian(s, m, iv, apply_friction, force, H);
}

// One block-descent update of one vertex: VBDPhysics.cpp:2402-2483
// (VBDStepWithCollision without line search), written to out[3] (the new position).
template <typename R>
void vbd_vertex_step(Scene<R>& s, Mesh<R>& m, int iv, bool apply_friction, R* out) {
    R force[3], H[9];
    vertex_force_hessian(s, m, iv, apply_friction, force, H);
    for (int d = 0; d < 3; ++d) out[d] = m.x[3 * size_t(iv) + d];
    R n2 = force[0] * force[0] + force[1] * force[1] + force[2] * force[2];
    if (!(n2 > R(1e-10))) return;  // CMP_EPSILON2, Types/Types.h:20-21
    R dx[3];
    R step = R(s.p.step_size);
    int fp64 = 0;
    bool ok = solve3x3<R>(H, force, dx, &fp64);
    if (fp64) s.fp64_solves.fetch_add(fp64);
    if (!ok) {
        step = R(s.p.step_size_gd);
        for (int d = 0; d < 3; ++d) dx[d] = force[d];
        s.failures.fetch_add(1);
    }
    for (int d = 0; d < 3; ++d) out[d] += step * dx[d];
}

// Parallel-group merge: VBDPhysics.cpp:99-122 (findSmallestParallelGroup) and
// :235-274 — each mesh's colors go, in order, to the globally smallest group
// this mesh has not used yet (first smallest wins ties).
template <typename R>
void build_groups(Scene<R>& s) {
    size_t ng = 0;
    for (auto& m : s.meshes) ng = std::max(ng, m.colors.size());
    s.groups.assign(ng, {});
    for (size_t im = 0; im < s.meshes.size(); ++im) {
        auto& m = s.meshes[im];
        std::vector<int> avail(m.colors.size());
        for (size_t c = 0; c < avail.size(); ++c) avail[c] = int(c);
        for (size_t c = 0; c < m.colors.size(); ++c) {
            size_t best = s.groups[avail[0]].size();
            int bestId = avail[0];
            size_t bestI = 0;
            for (size_t i = 1; i < avail.size(); ++i)
                if (s.groups[avail[i]].size() < best) {
                    best = s.groups[avail[i]].size();
                    bestId = avail[i];
                    bestI = i;
                }
            avail.erase(avail.begin() + bestI);
            for (int32_t v : m.colors[c]) {
                s.groups[bestId].push_back(int32_t(im));
                s.groups[bestId].push_back(v);
            }
        }
    }
}

// Deformer set-up and application: VBD/VBDDeformer.h:45-172.
template <typename R>
void init_deformers(Scene<R>& s) {
    for (auto& d : s.defs) {
        for (size_t i = 0; i < d.sel_mesh.size(); ++i) {
            auto& m = s.meshes[d.sel_mesh[i]];
            int v = d.sel_vert[i];
            m.fixed[v] = 1;  // setFixed (VBDDeformer.h:20-43)
            std::array<double, 3> P = {double(m.x[3 * v]), double(m.x[3 * v + 1]), double(m.x[3 * v + 2])};
            if (d.type == 0) {
                double OP[3] = {P[0] - d.center[0], P[1] - d.center[1], P[2] - d.center[2]};
                double dot = OP[0] * d.axis[0] + OP[1] * d.axis[1] + OP[2] * d.axis[2];
                std::array<double, 3> root = {dot * d.axis[0], dot * d.axis[1], dot * d.axis[2]};
                d.root.push_back(root);
                d.rootp.push_back({P[0] - root[0], P[1] - root[1], P[2] - root[2]});
            } else {
                d.orig.push_back(P);
            }
        }
    }
}

template <typename R>
void apply_deformers(Scene<R>& s) {
    for (auto& d : s.defs) {
        double t = s.cur_time;
        if (t >= d.end_time && d.end_time > 0) t = d.end_time;
        if (d.type == 0) {
            double th = t * d.omega;
            double c = std::cos(th), sn = std::sin(th);
            double ux = d.axis[0], uy = d.axis[1], uz = d.axis[2];
            double Rm[9] = {c + ux * ux * (1 - c), ux * uy * (1 - c) - uz * sn, ux * uz * (1 - c) + uy * sn,
                            uy * ux * (1 - c) + uz * sn, c + uy * uy * (1 - c), uy * uz * (1 - c) - ux * sn,
                            uz * ux * (1 - c) - uy * sn, uz * uy * (1 - c) + ux * sn, c + uz * uz * (1 - c)};
            for (size_t i = 0; i < d.sel_mesh.size(); ++i) {
                auto& m = s.meshes[d.sel_mesh[i]];
                int v = d.sel_vert[i];
                for (int r = 0; r < 3; ++r) {
                    double q = d.root[i][r] + Rm[3 * r] * d.rootp[i][0] + Rm[3 * r + 1] * d.rootp[i][1] +
                               Rm[3 * r + 2] * d.rootp[i][2];
                    m.x[3 * size_t(v) + r] = R(q);
                }
            }
        } else {
            for (size_t i = 0; i < d.sel_mesh.size(); ++i) {
                auto& m = s.meshes[d.sel_mesh[i]];
                int v = d.sel_vert[i];
                for (int r = 0; r < 3; ++r) m.x[3 * size_t(v) + r] = R(d.speed[r] * t + d.orig[i][r]);
            }
        }
    }
}

// Initial step: VBD_BaseMaterial.h:244-259 (applyInitialStep), :201-221
// (computeInertia: v += dt*g, fixed velocities zeroed, y = x + dt*v) and
// VBD_BaseMaterial.cpp:7-31 (forwardStep, initialization types 0-4).
template <typename R>
void initial_step(Scene<R>& s, Mesh<R>& m) {
    const R dt = R(s.dt);
    m.xprev = m.x;
    m.vprev = m.v;
    for (int i = 0; i < m.nv; ++i) {
        for (int d = 0; d < 3; ++d) {
            if (s.p.associate_gravity) m.v[3 * size_t(i) + d] += dt * R(s.p.gravity[d]);
        }
        if (m.fixed[i])
            for (int d = 0; d < 3; ++d) m.v[3 * size_t(i) + d] = 0;
        for (int d = 0; d < 3; ++d) m.y[3 * size_t(i) + d] = m.x[3 * size_t(i) + d] + dt * m.v[3 * size_t(i) + d];
    }
    for (int i = 0; i < m.nv; ++i)
        for (int d = 0; d < 3; ++d) {
            size_t k = 3 * size_t(i) + d;
            switch (m.init_type) {
                case 0: m.x[k] = m.y[k]; break;
                case 1: break;
                case 2: m.x[k] = m.xprev[k] + dt * m.vprev[k]; break;
                case 3: m.x[k] = R(0.5) * m.x[k] + R(0.5) * m.y[k]; break;
                case 4: m.x[k] = m.x[k] + dt * m.vprev[k] + dt * dt * R(0.5) * R(s.p.gravity[d]); break;
                default: m.x[k] = m.y[k]; break;
            }
        }
}

// Velocity update and damping, CPU semantics: VBDPhysics.cpp:2486-2561.
template <typename R>
void update_velocities(Scene<R>& s, Mesh<R>& m) {
    const R dt = R(s.dt);
    s.pool->run(m.nv, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            R* v = &m.v[3 * size_t(i)];
            for (int d = 0; d < 3; ++d) v[d] = (m.x[3 * size_t(i) + d] - m.xprev[3 * size_t(i) + d]) / dt;
            R vm = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (vm > R(1e-6)) {
                R vn = vm * m.exp_damp - m.const_damp;
                vn = vn > R(1e-6) ? vn : R(0);
                for (int d = 0; d < 3; ++d) v[d] *= vn / vm;
            } else {
                for (int d = 0; d < 3; ++d) v[d] *= R(0);
            }
            if (m.fixed[i])
                for (int d = 0; d < 3; ++d) v[d] = 0;
        }
    });
}

// Chebyshev over-relaxation weight: VBDPhysics.cpp:3558-3574.
double accel_omega(int order, double rho, double prev) {
    if (order == 1) return 1.0;
    if (order == 2) return 2.0 / (2.0 - rho * rho);
    return 4.0 / (4.0 - rho * rho * prev);
}

// One substep: VBDPhysics.cpp:1580-1632 (runStep_serialCollisionHandling),
// with the optional accelerator of runStepGPU (:879-953, VBDPhysicsCompute.cu:910-944).
template <typename R>
void substep(Scene<R>& s, int iterations) {
    s.cur_time += s.dt;
    for (auto& m : s.meshes)
        if (m.active) initial_step(s, m);
    detect_contacts(s, false);
    apply_deformers(s);
    double omega = 1.0;
    if (s.p.use_accelerator)
        for (auto& m : s.meshes) m.prevprev_iter = m.x;
    for (int it = 0; it < iterations; ++it) {
        bool fric = it >= s.p.friction_start_iter;
        // intermediateCollisionDetection (VBDPhysics.cpp:878-884, 2158-2172)
        const int ici = s.p.intermediate_collision_iterations;
        if (ici > 0 && it % ici == 0 && it) detect_contacts(s, true);
        if (s.p.use_accelerator) {
            omega = accel_omega(it + 1, s.p.accelerator_rho, omega);
            for (auto& m : s.meshes) m.prev_iter = m.x;
        }
        // a group (merged color) is updated Jacobi-style, as the GPU path does
        // (positionsNew, then commit: VBDPhysicsCompute.cu:803-908, 946-968): no vertex of
        // a group sees another's new position. Tet neighbours are never in one group, so
        // this only matters for contact partners.
        std::vector<R> xnew;
        for (auto& g : s.groups) {
            int64_t n = int64_t(g.size() / 2);
            xnew.resize(3 * size_t(n));
            s.pool->run(n, [&](int64_t b, int64_t e) {
                for (int64_t i = b; i < e; ++i) {
                    auto& m = s.meshes[g[2 * i]];
                    int v = g[2 * i + 1];
                    R* out = &xnew[3 * size_t(i)];
                    if (!m.fixed[v] && m.active) vbd_vertex_step(s, m, v, fric, out);
                    else for (int d = 0; d < 3; ++d) out[d] = m.x[3 * size_t(v) + d];
                }
            });
            for (int64_t i = 0; i < n; ++i) {
                auto& m = s.meshes[g[2 * i]];
                int v = g[2 * i + 1];
                for (int d = 0; d < 3; ++d) m.x[3 * size_t(v) + d] = xnew[3 * size_t(i) + d];
            }
        }
        if (s.p.use_accelerator) {
            const R om = R(omega);
            for (auto& m : s.meshes) {
                if (!m.active) continue;
                for (int i = 0; i < m.nv; ++i) {
                    if (m.fixed[i]) continue;
                    const bool colliding = !m.col_mask.empty() && m.col_mask[i];
                    for (int d = 0; d < 3; ++d) {
                        size_t k = 3 * size_t(i) + d;
                        if (!colliding) {
                            R diff = m.x[k] - m.prevprev_iter[k];
                            m.x[k] = m.prevprev_iter[k] + om * diff;
                        }
                        m.prevprev_iter[k] = m.prev_iter[k];
                    }
                }
            }
        }
    }
    for (auto& m : s.meshes)
        if (m.active) update_velocities(s, m);
}

template <typename R>
Scene<R>* create(int nmesh, const OracleMesh* meshes, const OracleParams* params, int ndef,
                 const OracleDeformer* defs, int nthreads) {
    auto* s = new Scene<R>();
    s->p = *params;
    // BasePhysicsFramework.cpp:245-249 and VBDPhysics.cpp:794-807
    s->dt = params->time_step / params->num_substeps;
    s->dt2inv = 1.0 / (s->dt * s->dt);
    if (nthreads <= 0) nthreads = int(std::thread::hardware_concurrency());
    s->pool = new Pool(nthreads);
    s->meshes.resize(nmesh);
    for (int im = 0; im < nmesh; ++im) {
        const OracleMesh& in = meshes[im];
        Mesh<R>& m = s->meshes[im];
        m.nv = in.nv;
        m.ntet = in.ntet;
        m.x.resize(3 * size_t(m.nv));
        for (size_t i = 0; i < m.x.size(); ++i) m.x[i] = R(in.X[i]);
        m.v.assign(3 * size_t(m.nv), R(0));
        if (in.V0)
            for (size_t i = 0; i < m.v.size(); ++i) m.v[i] = R(in.V0[i]);
        m.xprev = m.x;
        m.vprev = m.v;
        m.y = m.x;
        m.tets.assign(in.tets, in.tets + 4 * size_t(m.ntet));
        m.fixed.assign(m.nv, 0);
        if (in.fixed)
            for (int i = 0; i < m.nv; ++i) m.fixed[i] = in.fixed[i] ? 1 : 0;
        m.miu = R(in.miu); m.lmbd = R(in.lmbd); m.density = R(in.density);
        m.kh = R(in.damping_hydrostatic); m.kd = R(in.damping_deviatoric);
        m.exp_damp = R(std::pow(in.exp_vel_damping, s->dt));
        m.const_damp = R(in.const_vel_damping * s->dt);
        m.fr_mu = R(in.friction_dynamic); m.fr_eps = R(in.friction_eps_v);
        m.init_type = in.init_type;
        m.active = in.active != 0;
        for (int c = 0; c < in.ncolors; ++c)
            m.colors.emplace_back(in.color_verts + in.color_offsets[c], in.color_verts + in.color_offsets[c + 1]);
        // TetMeshFEM.cpp:122-134: sort colors large to small (std::sort, not stable)
        std::sort(m.colors.begin(), m.colors.end(),
                  [](const std::vector<int32_t>& a, const std::vector<int32_t>& b) { return a.size() > b.size(); });
        rest_shape(m);
        build_adjacency(m);
        m.surf = oracle_tc::extract_surface(m.nv, m.ntet, in.tets, in.X);
        m.hits.assign(m.surf.verts.size(), oracle_tc::CcdHit{});
    }
    for (int i = 0; i < ndef; ++i) {
        Deformer d;
        d.type = defs[i].type;
        for (int k = 0; k < 3; ++k) {
            d.center[k] = defs[i].center[k];
            d.axis[k] = defs[i].axis[k];
            d.speed[k] = defs[i].speed[k];
        }
        d.omega = defs[i].angular_velocity;
        d.end_time = defs[i].end_time;
        d.sel_mesh.assign(defs[i].sel_mesh, defs[i].sel_mesh + defs[i].nsel);
        d.sel_vert.assign(defs[i].sel_vert, defs[i].sel_vert + defs[i].nsel);
        s->defs.push_back(d);
    }
    build_groups(*s);
    init_deformers(*s);
    return s;
}

struct Handle {
    int precision;
    Scene<double>* d = nullptr;
    Scene<float>* f = nullptr;
};

template <typename Fn>
auto dispatch(void* h, Fn&& fn) {
    Handle* H = static_cast<Handle*>(h);
    if (H->precision == 64) return fn(*H->d);
    return fn(*H->f);
}

template <typename R>
double energy(Scene<R>& s) {
    double E = 0;
    for (auto& m : s.meshes) {
        double a = 1.0 + double(m.miu) / double(m.lmbd);
        for (int t = 0; t < m.ntet; ++t) {
            const int32_t* tv = &m.tets[4 * size_t(t)];
            double Ds[9], F[9];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r)
                    Ds[3 * c + r] = double(m.x[3 * size_t(tv[c + 1]) + r]) - double(m.x[3 * size_t(tv[0]) + r]);
            const R* Di = &m.dminv[9 * size_t(t)];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    double sum = 0;
                    for (int q = 0; q < 3; ++q) sum += Ds[3 * q + r] * double(Di[3 * c + q]);
                    F[3 * c + r] = sum;
                }
            double det = F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                         F[6] * (F[1] * F[5] - F[4] * F[2]);
            double n2 = 0;
            for (int i = 0; i < 9; ++i) n2 += F[i] * F[i];
            double A = double(m.vol[t]);
            // VBDPhysicsCompute.cu:1775-1810 (energy with the rest energy removed)
            E += A * (double(m.miu) * 0.5 * (n2 - 3.0) + double(m.lmbd) * 0.5 * (det - a) * (det - a));
            E -= 0.5 * A * double(m.lmbd) * (1.0 - a) * (1.0 - a);
        }
        for (int i = 0; i < m.nv; ++i) {
            double d2 = 0;
            for (int d = 0; d < 3; ++d) {
                double q = double(m.x[3 * size_t(i) + d]) - double(m.y[3 * size_t(i) + d]);
                d2 += q * q;
            }
            E += 0.5 * s.dt2inv * double(m.mass[i]) * d2;
        }
    }
    return E;
}

// evaluateConvergence (VBDPhysics.cpp:3459-3506) in FP64: energy, inertia, elastic, and
// the average over all vertices of |material force (with damping) + inertia force|,
// zero for fixed vertices.
template <typename R>
void convergence(Scene<R>& s, double* out) {
    double total = energy(s), inertia = 0.0, fsum = 0.0;
    int64_t nall = 0;
    for (auto& m : s.meshes) {
        for (int i = 0; i < m.nv; ++i) {
            double d2 = 0;
            for (int d = 0; d < 3; ++d) {
                const double q = double(m.x[3 * size_t(i) + d]) - double(m.y[3 * size_t(i) + d]);
                d2 += q * q;
            }
            inertia += 0.5 * s.dt2inv * double(m.mass[i]) * d2;
        }
        nall += m.nv;
        if (!m.active) continue;
        std::vector<double> fn(size_t(m.nv), 0.0);
        s.pool->run(m.nv, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i) {
                if (m.fixed[i]) continue;
                R f[3] = {0, 0, 0}, H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                material_force_hessian<R>(m, int(i), R(s.dt), f, H);
                const double w = double(m.mass[i]) * s.dt2inv;
                double g[3];
                for (int d = 0; d < 3; ++d)
                    g[d] = double(f[d]) + w * (double(m.y[3 * size_t(i) + d]) - double(m.x[3 * size_t(i) + d]));
                fn[size_t(i)] = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            }
        });
        for (double v : fn) fsum += v;
    }
    out[0] = total;
    out[1] = inertia;
    out[2] = total - inertia;
    out[3] = nall ? fsum / double(nall) : 0.0;
}

}  // namespace

extern "C" {

// .t mesh reader ("Vertex id x y z" / "Tet id a b c d", vertex ids in file order).
// Call with X == nullptr to get the counts, then again with buffers.
int32_t oracle_read_t(const char* path, int32_t* nv, int32_t* ntet, double* X, int32_t* tets) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::string text(size_t(n), '\0');
    size_t got = std::fread(&text[0], 1, size_t(n), f);
    std::fclose(f);
    if (got != size_t(n)) return -1;
    int32_t cv = 0, ct = 0;
    const char* p = text.c_str();
    const char* end = p + text.size();
    while (p < end) {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
        if (p >= end) break;
        const char* line = p;
        while (p < end && *p != '\n') ++p;
        char* q = nullptr;
        if (std::strncmp(line, "Vertex", 6) == 0) {
            std::strtol(line + 6, &q, 10);
            if (X) for (int k = 0; k < 3; ++k) X[3 * size_t(cv) + k] = std::strtod(q, &q);
            ++cv;
        } else if (std::strncmp(line, "Tet", 3) == 0) {
            std::strtol(line + 3, &q, 10);
            if (tets) for (int k = 0; k < 4; ++k) tets[4 * size_t(ct) + k] = int32_t(std::strtol(q, &q, 10));
            ++ct;
        }
    }
    *nv = cv;
    *ntet = ct;
    return 0;
}

// MCS coloring, restating GraphColoring/mcs.cpp:14-168. The time-seeded
// shuffle there (mcs.cpp:50-52) only decides when the candidate list is
// compacted, never which node is picked, so it is left out: the node picked
// each round is the first maximum-weight node in index order.
int32_t oracle_color_mcs(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors) {
    auto g = vertex_graph(nv, ntet, tets);
    std::vector<int> weight(nv, 0), picked(nv, 0), order;
    order.reserve(nv);
    for (int i = 0; i < nv; ++i) {
        int best = -1, bw = -1;
        for (int j = 0; j < nv; ++j)
            if (!picked[j] && weight[j] > bw) { bw = weight[j]; best = j; }
        if (best < 0) return -1;
        order.push_back(best);
        picked[best] = 1;
        for (int nb : g[best]) weight[nb] += 1;
    }
    for (int i = 0; i < nv; ++i) colors[i] = -1;
    int ncol = 0;
    for (int node : order) {
        std::vector<int> used;
        for (int nb : g[node]) used.push_back(colors[nb]);
        std::sort(used.begin(), used.end());
        used.erase(std::unique(used.begin(), used.end()), used.end());
        int c = 0;
        for (int u : used)
            if (u == c) ++c;
        colors[node] = c;
        ncol = std::max(ncol, c + 1);
    }
    return ncol;
}

// OrderedGreedy coloring, restating GraphColoring/gready.cpp:15-117: repeatedly
// take the uncolored node of minimum remaining degree (lowest index on ties),
// give it the lowest color its colored neighbours do not use, and decrement
// the remaining degree of its uncolored neighbours.
int32_t oracle_color_greedy(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors) {
    auto g = vertex_graph(nv, ntet, tets);
    std::vector<int> deg(nv);
    for (int i = 0; i < nv; ++i) { deg[i] = int(g[i].size()); colors[i] = -1; }
    int maxColor = -1;
    for (int n = 0; n < nv; ++n) {
        int node = -1, md = nv + 1;
        for (int i = 0; i < nv; ++i) {
            if (deg[i] == -1) continue;
            if (md > deg[i]) { md = deg[i]; node = i; }
        }
        if (node < 0) return -1;
        if (maxColor == -1) {
            maxColor = 0;
            colors[node] = 0;
        } else {
            std::vector<char> used(maxColor + 1, 0);
            for (int nb : g[node])
                if (colors[nb] >= 0) used[colors[nb]] = 1;
            int c = -1;
            for (int k = 0; k <= maxColor; ++k)
                if (!used[k]) { c = k; break; }
            if (c == -1) c = ++maxColor;
            colors[node] = c;
        }
        deg[node] = -1;
        for (int nb : g[node])
            if (deg[nb] != -1) deg[nb]--;
    }
    return maxColor + 1;
}

// One tet's Neo-Hookean force (3) and Hessian (9, row-major) on its vertex `order`, in FP64
// (the per-tet term of the vertex block; accumulated into f and h).
void oracle_nh_element(const double* x12, const double* xprev12, const double* dminv9, double mu, double lmbd,
                       double A, int32_t order, double kh, double kd, double dt, double* f, double* h) {
    double disp[3];
    for (int d = 0; d < 3; ++d) disp[d] = x12[3 * order + d] - xprev12[3 * order + d];
    tet_force_hessian<double>(x12, dminv9, A, order, mu, lmbd, kh, kd, dt, disp, f, h);
}

// The GraphColoring tool's pipeline (GraphColoring/GraphColoring.cpp:170-189): MCS
// (algorithm 0) or OrderedGreedy (1), categories in color order with vertices ascending,
// then, with balance, balanceColoredCategories (ColoringAlgorithms.cpp:142-196): move the
// first vertex of the largest category (or of the first other category that has one) that
// no neighbour of the smallest category blocks to the end of the smallest, the loop body
// running once before the max/min size ratio is compared with the goal. colors: each
// vertex's color; order: the vertices of every category in the order the tool writes them.
int32_t oracle_color_tool(int32_t nv, int32_t ntet, const int32_t* tets, int32_t algorithm, int32_t balance,
                          float goal, int32_t* colors, int32_t* order) {
    const int32_t n = algorithm == 0 ? oracle_color_mcs(nv, ntet, tets, colors)
                                     : oracle_color_greedy(nv, ntet, tets, colors);
    if (n <= 0) return n;
    std::vector<std::vector<int>> cats(static_cast<size_t>(n));
    for (int v = 0; v < nv; ++v) cats[size_t(colors[v])].push_back(v);
    if (balance) {
        auto g = vertex_graph(nv, ntet, tets);
        auto free_in = [&](int src, int dst) {
            const auto& c = cats[size_t(src)];
            for (size_t i = 0; i < c.size(); ++i) {
                bool ok = true;
                for (int nb : g[size_t(c[i])])
                    if (colors[nb] == dst) { ok = false; break; }
                if (ok) return int(i);
            }
            return -1;
        };
        const int64_t cap = 64 * int64_t(nv) + 1024;
        int64_t moves = 0;
        float ratio;
        do {
            if (++moves > cap) return -1;
            int big = 0, small = 0;
            for (int c = 0; c < n; ++c) {
                if (cats[size_t(big)].size() < cats[size_t(c)].size()) big = c;
                if (cats[size_t(small)].size() > cats[size_t(c)].size()) small = c;
            }
            ratio = float(cats[size_t(big)].size()) / float(cats[size_t(small)].size());
            int id = free_in(big, small);
            if (id < 0)
                for (int c = 0; c < n && id < 0; ++c) {
                    if (c == big || c == small) continue;
                    id = free_in(c, small);
                    if (id >= 0) big = c;
                }
            if (id < 0) break;
            const int node = cats[size_t(big)][size_t(id)];
            colors[node] = small;
            cats[size_t(big)].erase(cats[size_t(big)].begin() + id);
            cats[size_t(small)].push_back(node);
        } while (ratio > goal);
    }
    if (order) {
        size_t k = 0;
        for (auto& c : cats)
            for (int v : c) order[k++] = v;
    }
    return n;
}

void* oracle_create(int32_t precision, int32_t nmesh, const OracleMesh* meshes, const OracleParams* params,
                    int32_t ndef, const OracleDeformer* defs, int32_t nthreads) {
    Handle* h = new Handle();
    h->precision = precision == 32 ? 32 : 64;
    if (h->precision == 64) h->d = create<double>(nmesh, meshes, params, ndef, defs, nthreads);
    else h->f = create<float>(nmesh, meshes, params, ndef, defs, nthreads);
    return h;
}

void oracle_destroy(void* h) {
    Handle* H = static_cast<Handle*>(h);
    delete H->d;
    delete H->f;
    delete H;
}

int32_t oracle_step(void* h, int32_t nsteps) {
    return dispatch(h, [&](auto& s) {
        for (int k = 0; k < nsteps; ++k)
            for (int sub = 0; sub < s.p.num_substeps; ++sub) substep(s, s.p.iterations);
        return int32_t(0);
    });
}

int32_t oracle_substep_sample(void* h, int32_t iterations) {
    return dispatch(h, [&](auto& s) {
        substep(s, iterations);
        return int32_t(0);
    });
}

void oracle_get_positions(void* h, int32_t mesh, double* out) {
    dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        for (size_t i = 0; i < m.x.size(); ++i) out[i] = double(m.x[i]);
        return 0;
    });
}
void oracle_get_velocities(void* h, int32_t mesh, double* out) {
    dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        for (size_t i = 0; i < m.v.size(); ++i) out[i] = double(m.v[i]);
        return 0;
    });
}
void oracle_set_positions(void* h, int32_t mesh, const double* in) {
    dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        using R = typename std::decay_t<decltype(m.x)>::value_type;
        for (size_t i = 0; i < m.x.size(); ++i) m.x[i] = R(in[i]);
        return 0;
    });
}
void oracle_set_velocities(void* h, int32_t mesh, const double* in) {
    dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        using R = typename std::decay_t<decltype(m.v)>::value_type;
        for (size_t i = 0; i < m.v.size(); ++i) m.v[i] = R(in[i]);
        return 0;
    });
}
void oracle_get_rest(void* h, int32_t mesh, double* dminv, double* vol, double* mass) {
    dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        if (dminv) for (size_t i = 0; i < m.dminv.size(); ++i) dminv[i] = double(m.dminv[i]);
        if (vol) for (size_t i = 0; i < m.vol.size(); ++i) vol[i] = double(m.vol[i]);
        if (mass) for (size_t i = 0; i < m.mass.size(); ++i) mass[i] = double(m.mass[i]);
        return 0;
    });
}
int32_t oracle_num_groups(void* h) {
    return dispatch(h, [&](auto& s) { return int32_t(s.groups.size()); });
}
int32_t oracle_group_size(void* h, int32_t g) {
    return dispatch(h, [&](auto& s) { return int32_t(s.groups[g].size() / 2); });
}
void oracle_group(void* h, int32_t g, int32_t* out) {
    dispatch(h, [&](auto& s) {
        std::copy(s.groups[g].begin(), s.groups[g].end(), out);
        return 0;
    });
}
void oracle_vertex_force_hessian(void* h, int32_t mesh, int32_t v, int32_t apply_friction, double* f3, double* h9) {
    dispatch(h, [&](auto& s) {
        using R = typename std::decay_t<decltype(s.meshes[0].x)>::value_type;
        R f[3], H[9];
        vertex_force_hessian(s, s.meshes[mesh], v, apply_friction != 0, f, H);
        for (int i = 0; i < 3; ++i) f3[i] = double(f[i]);
        for (int i = 0; i < 9; ++i) h9[i] = double(H[i]);
        return 0;
    });
}
double oracle_energy(void* h) {
    return dispatch(h, [&](auto& s) { return energy(s); });
}
void oracle_convergence(void* h, double* out4) {
    dispatch(h, [&](auto& s) { convergence(s, out4); });
}

int32_t oracle_solve_failures(void* h) {
    return dispatch(h, [&](auto& s) { return int32_t(s.failures.load()); });
}

void oracle_set_prev_positions(void* h, int32_t mesh, const double* in) {
    dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        using R = typename std::decay_t<decltype(m.x)>::value_type;
        for (size_t i = 0; i < m.xprev.size(); ++i) m.xprev[i] = R(in[i]);
        return 0;
    });
}
int32_t oracle_collide(void* h) {
    return dispatch(h, [&](auto& s) {
        detect_contacts(s, false);
        int32_t n = 0;
        for (auto& m : s.meshes)
            for (char a : m.col_active) n += a ? 1 : 0;
        return n;
    });
}
int32_t oracle_get_contacts(void* h, int32_t* rows, int32_t cap) {
    return dispatch(h, [&](auto& s) {
        int32_t n = 0;
        for (size_t im = 0; im < s.meshes.size(); ++im) {
            auto& m = s.meshes[im];
            if (m.col_active.empty()) continue;
            for (int32_t v : m.surf.verts) {
                if (!m.col_active[v]) continue;
                if (n < cap) {
                    int32_t* r = rows + 8 * size_t(n);
                    r[0] = int32_t(im);
                    r[1] = v;
                    r[2] = m.col_fmesh[v];
                    for (int j = 0; j < 3; ++j) r[3 + j] = m.col_fv[3 * size_t(v) + j];
                    r[6] = m.col_face[v];
                    r[7] = m.col_kind[v];
                }
                ++n;
            }
        }
        return n;
    });
}
int32_t oracle_num_surface(void* h, int32_t mesh, int32_t* nverts) {
    return dispatch(h, [&](auto& s) {
        auto& m = s.meshes[mesh];
        if (nverts) *nverts = int32_t(m.surf.verts.size());
        return int32_t(m.surf.faces.size() / 3);
    });
}

}  // extern "C"
