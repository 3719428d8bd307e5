// Host-side scene set-up: JSON inputs, .t meshes, colorings, rest shape and
// parallel-group merge. See scene.hpp.
#include "scene.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <queue>
#include <sstream>
#include <stdexcept>

#include "json_get.hpp"
#include "json_lite.hpp"

namespace gaia {

namespace {

using namespace jsonio;

// Vertex graph of a tet mesh as CSR with sorted unique neighbours
// (GraphColoring/TetMeshVertexGraph.h:14-41: all vertex pairs sharing a tet).
void vertex_graph(int32_t nv, int32_t ntet, const int32_t* tets, std::vector<int64_t>& ofs, std::vector<int32_t>& adj) {
    std::vector<int64_t> cnt(size_t(nv) + 1, 0);
    for (int64_t t = 0; t < ntet; ++t)
        for (int i = 0; i < 4; ++i) {
            int32_t a = tets[4 * t + i];
            if (a < 0 || a >= nv) throw std::runtime_error("tet references vertex out of range");
            cnt[size_t(a) + 1] += 3;
        }
    for (int32_t i = 0; i < nv; ++i) cnt[i + 1] += cnt[i];
    std::vector<int32_t> raw(cnt[nv]);
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t t = 0; t < ntet; ++t)
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                if (i != j) {
                    int32_t a = tets[4 * t + i], b = tets[4 * t + j];
                    if (a != b) raw[fill[a]++] = b;
                }
    ofs.assign(size_t(nv) + 1, 0);
    adj.clear();
    adj.reserve(raw.size() / 2 + 1);
    for (int32_t v = 0; v < nv; ++v) {
        auto b = raw.begin() + cnt[v], e = raw.begin() + fill[v];
        std::sort(b, e);
        auto u = std::unique(b, e);
        adj.insert(adj.end(), b, u);
        ofs[v + 1] = int64_t(adj.size());
    }
}

// Lowest color not used by already colored neighbours.
int32_t lowest_free_color(const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t node,
                          const int32_t* colors, std::vector<int32_t>& scratch) {
    scratch.clear();
    for (int64_t k = ofs[node]; k < ofs[node + 1]; ++k) {
        int32_t c = colors[adj[k]];
        if (c >= 0) scratch.push_back(c);
    }
    std::sort(scratch.begin(), scratch.end());
    int32_t c = 0;
    for (int32_t u : scratch)
        if (u == c) ++c;
    return c;
}

}  // namespace

// MCS (GraphColoring/mcs.cpp:14-168): visit order = repeatedly the unvisited node
// of largest weight (number of visited neighbours), lowest index on ties; then
// color in visit order with the lowest free color. A lazy max-heap keyed on
// (weight, -index) reproduces the reference's linear scan exactly.
int32_t color_mcs(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors) {
    std::vector<int64_t> ofs;
    std::vector<int32_t> adj;
    vertex_graph(nv, ntet, tets, ofs, adj);
    return color_mcs_graph(nv, ofs, adj, colors);
}

int32_t color_mcs_graph(int32_t nv, const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t* colors) {
    std::vector<int32_t> weight(nv, 0), order;
    std::vector<uint8_t> done(nv, 0);
    order.reserve(nv);
    using E = std::pair<int32_t, int32_t>;  // (weight, -index)
    std::priority_queue<E> pq;
    for (int32_t i = 0; i < nv; ++i) pq.push({0, -i});
    while (!pq.empty()) {
        E e = pq.top();
        pq.pop();
        int32_t v = -e.second;
        if (done[v] || e.first != weight[v]) continue;
        done[v] = 1;
        order.push_back(v);
        for (int64_t k = ofs[v]; k < ofs[v + 1]; ++k) {
            int32_t u = adj[k];
            weight[u] += 1;
            if (!done[u]) pq.push({weight[u], -u});
        }
    }
    if (int32_t(order.size()) != nv) return -1;
    for (int32_t i = 0; i < nv; ++i) colors[i] = -1;
    int32_t ncol = 0;
    std::vector<int32_t> scratch;
    for (int32_t v : order) {
        int32_t c = lowest_free_color(ofs, adj, v, colors, scratch);
        colors[v] = c;
        ncol = std::max(ncol, c + 1);
    }
    return ncol;
}

// OrderedGreedy (GraphColoring/gready.cpp:15-117): repeatedly the uncolored node
// of smallest remaining degree (lowest index on ties) takes the lowest free color;
// its uncolored neighbours' remaining degrees drop by one. Lazy min-heap.
int32_t color_greedy(int32_t nv, int32_t ntet, const int32_t* tets, int32_t* colors) {
    std::vector<int64_t> ofs;
    std::vector<int32_t> adj;
    vertex_graph(nv, ntet, tets, ofs, adj);
    return color_greedy_graph(nv, ofs, adj, colors);
}

int32_t color_greedy_graph(int32_t nv, const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t* colors) {
    std::vector<int32_t> deg(nv);
    using E = std::pair<int32_t, int32_t>;  // (degree, index), min-heap
    std::priority_queue<E, std::vector<E>, std::greater<E>> pq;
    for (int32_t i = 0; i < nv; ++i) {
        deg[i] = int32_t(ofs[i + 1] - ofs[i]);
        colors[i] = -1;
        pq.push({deg[i], i});
    }
    int32_t ncol = 0, ncolored = 0;
    std::vector<int32_t> scratch;
    while (!pq.empty()) {
        E e = pq.top();
        pq.pop();
        int32_t v = e.second;
        if (deg[v] == -1 || e.first != deg[v]) continue;
        int32_t c = lowest_free_color(ofs, adj, v, colors, scratch);
        colors[v] = c;
        ncol = std::max(ncol, c + 1);
        ++ncolored;
        deg[v] = -1;
        for (int64_t k = ofs[v]; k < ofs[v + 1]; ++k) {
            int32_t u = adj[k];
            if (deg[u] != -1) {
                deg[u] -= 1;
                pq.push({deg[u], u});
            }
        }
    }
    return ncolored == nv ? ncol : -1;
}

// ColoringAlgorithms.cpp:69-80 (convertToColoredCategories).
void tet_vertex_graph(int32_t nv, int32_t ntet, const int32_t* tets, std::vector<int64_t>& ofs, std::vector<int32_t>& adj) {
    vertex_graph(nv, ntet, tets, ofs, adj);
}

void balance_categories(int32_t nv, const std::vector<int64_t>& ofs, const std::vector<int32_t>& adj, int32_t* colors,
                        std::vector<std::vector<int32_t>>& cats, float goal) {
    auto movable = [&](int32_t node, int32_t dst) {
        for (int64_t k = ofs[node]; k < ofs[node + 1]; ++k)
            if (colors[adj[k]] == dst) return false;
        return true;
    };
    auto first_movable = [&](int32_t src, int32_t dst) -> int64_t {
        const auto& c = cats[size_t(src)];
        for (size_t i = 0; i < c.size(); ++i)
            if (movable(c[i], dst)) return int64_t(i);
        return -1;
    };
    if (cats.empty()) return;
    // the reference's loop has no bound and does not end on some graphs (moves can cycle
    // between categories without reaching the goal); stop with an error instead
    const int64_t max_moves = 64 * int64_t(nv) + 1024;
    int64_t moves = 0;
    float ratio;
    do {
        if (++moves > max_moves)
            throw std::runtime_error("color balancing did not reach the goal ratio (the reference's loop would not end)");
        // findLargestSmallestCategories: first largest, first smallest in color order
        size_t big = 0, small = 0;
        for (size_t c = 0; c < cats.size(); ++c) {
            if (cats[big].size() < cats[c].size()) big = c;
            if (cats[small].size() > cats[c].size()) small = c;
        }
        ratio = float(cats[big].size()) / float(cats[small].size());
        int64_t id = first_movable(int32_t(big), int32_t(small));
        if (id < 0)
            for (size_t c = 0; c < cats.size(); ++c) {
                if (c == big || c == small) continue;
                id = first_movable(int32_t(c), int32_t(small));
                if (id >= 0) {
                    big = c;
                    break;
                }
            }
        if (id < 0) return;  // "not optimizable anymore"
        const int32_t node = cats[big][size_t(id)];
        colors[node] = int32_t(small);
        cats[big].erase(cats[big].begin() + id);
        cats[small].push_back(node);
    } while (ratio > goal);
}

std::vector<std::vector<int32_t>> colors_to_categories(int32_t nv, const int32_t* colors) {
    int32_t n = 0;
    for (int32_t i = 0; i < nv; ++i) n = std::max(n, colors[i] + 1);
    std::vector<std::vector<int32_t>> cats(n);
    for (int32_t i = 0; i < nv; ++i) cats[colors[i]].push_back(i);
    return cats;
}

// .t format read by MeshFrame's load_t: "Vertex <id> x y z" and "Tet <id> a b c d".
// Vertex ids map to file order; tets reference vertex ids.
void load_t(const std::string& path, std::vector<float>& X, std::vector<int32_t>& tets) {
    std::string text = read_file(path);
    X.clear();
    tets.clear();
    std::vector<int64_t> ids;
    bool identity = true;
    const char* p = text.c_str();
    const char* end = p + text.size();
    std::vector<int64_t> rawTets;
    while (p < end) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
        if (p >= end) break;
        const char* line = p;
        while (p < end && *p != '\n') ++p;
        if (std::strncmp(line, "Vertex", 6) == 0) {
            char* q = nullptr;
            long long id = std::strtoll(line + 6, &q, 10);
            double x = std::strtod(q, &q), y = std::strtod(q, &q), z = std::strtod(q, &q);
            if (int64_t(id) != int64_t(ids.size())) identity = false;
            ids.push_back(id);
            X.push_back(float(x));
            X.push_back(float(y));
            X.push_back(float(z));
        } else if (std::strncmp(line, "Tet", 3) == 0) {
            char* q = nullptr;
            std::strtoll(line + 3, &q, 10);
            for (int i = 0; i < 4; ++i) rawTets.push_back(std::strtoll(q, &q, 10));
        }
    }
    if (X.empty()) throw std::runtime_error("no vertices in mesh file: " + path);
    int64_t nv = int64_t(ids.size());
    tets.resize(rawTets.size());
    if (identity) {
        for (size_t i = 0; i < rawTets.size(); ++i) {
            if (rawTets[i] < 0 || rawTets[i] >= nv) throw std::runtime_error("tet vertex id out of range in " + path);
            tets[i] = int32_t(rawTets[i]);
        }
    } else {
        std::vector<std::pair<int64_t, int32_t>> map;
        for (int64_t i = 0; i < nv; ++i) map.push_back({ids[i], int32_t(i)});
        std::sort(map.begin(), map.end());
        for (size_t i = 0; i < rawTets.size(); ++i) {
            auto it = std::lower_bound(map.begin(), map.end(), std::make_pair(rawTets[i], int32_t(-1)));
            if (it == map.end() || it->first != rawTets[i]) throw std::runtime_error("unknown vertex id in " + path);
            tets[i] = it->second;
        }
    }
}

std::vector<std::vector<int32_t>> load_coloring(const std::string& path) {
    json::Value v = json::parse(read_file(path));
    if (!v.is_array()) throw std::runtime_error("coloring file is not a list of lists: " + path);
    std::vector<std::vector<int32_t>> cats;
    for (auto& c : v.arr) {
        if (!c.is_array()) throw std::runtime_error("coloring file is not a list of lists: " + path);
        std::vector<int32_t> cat;
        cat.reserve(c.arr.size());
        for (auto& e : c.arr) cat.push_back(int32_t(e.num));
        cats.push_back(std::move(cat));
    }
    return cats;
}

void validate_coloring(const TetMesh& m) {
    std::vector<int32_t> color(m.nv, -1);
    for (size_t c = 0; c < m.colors.size(); ++c)
        for (int32_t v : m.colors[c]) {
            if (v < 0 || v >= m.nv) throw std::runtime_error("coloring lists a vertex out of range");
            if (color[v] != -1) throw std::runtime_error("coloring lists a vertex twice");
            color[v] = int32_t(c);
        }
    for (int32_t v = 0; v < m.nv; ++v)
        if (color[v] == -1) throw std::runtime_error("coloring misses vertex " + std::to_string(v));
    for (int32_t t = 0; t < m.ntet; ++t)
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j)
                if (color[m.tets[4 * size_t(t) + i]] == color[m.tets[4 * size_t(t) + j]])
                    throw std::runtime_error("invalid coloring: tet " + std::to_string(t) + " has two vertices of one color");
}

void extract_surface(TetMesh& m) {
    static const int kFace[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
    struct Key {
        int32_t a, b, c, id;  // sorted vertex ids, 4 * tet + local face
    };
    std::vector<Key> keys(4 * size_t(m.ntet));
    for (int32_t t = 0; t < m.ntet; ++t)
        for (int k = 0; k < 4; ++k) {
            int32_t v[3] = {m.tets[4 * size_t(t) + kFace[k][0]], m.tets[4 * size_t(t) + kFace[k][1]],
                            m.tets[4 * size_t(t) + kFace[k][2]]};
            std::sort(v, v + 3);
            keys[4 * size_t(t) + k] = Key{v[0], v[1], v[2], 4 * t + k};
        }
    auto less3 = [](const Key& x, const Key& y) {
        return x.a != y.a ? x.a < y.a : (x.b != y.b ? x.b < y.b : x.c < y.c);
    };
    std::sort(keys.begin(), keys.end(), [&](const Key& x, const Key& y) { return less3(x, y) || (!less3(y, x) && x.id < y.id); });
    std::vector<char> boundary(4 * size_t(m.ntet), 0);
    // tetsNeighborTets (TetMesh/TetMeshFEM.cpp:40-70): the other tet of a face two tets share
    m.tet_nbr.assign(4 * size_t(m.ntet), -1);
    for (size_t i = 0; i < keys.size();) {
        size_t j = i + 1;
        while (j < keys.size() && !less3(keys[i], keys[j])) ++j;
        if (j - i == 1) boundary[size_t(keys[i].id)] = 1;
        if (j - i == 2) {
            m.tet_nbr[size_t(keys[i].id)] = keys[i + 1].id / 4;
            m.tet_nbr[size_t(keys[i + 1].id)] = keys[i].id / 4;
        }
        i = j;
    }
    m.sfaces.clear();
    m.sface_tet.clear();
    std::vector<char> on(size_t(m.nv), 0);
    for (int32_t t = 0; t < m.ntet; ++t) {
        const int32_t* tv = &m.tets[4 * size_t(t)];
        double e[3][3];
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) e[i][d] = double(m.X[3 * size_t(tv[i + 1]) + d]) - double(m.X[3 * size_t(tv[0]) + d]);
        const double vol = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
        for (int k = 0; k < 4; ++k) {
            if (!boundary[4 * size_t(t) + k]) continue;
            int32_t f[3] = {tv[kFace[k][0]], tv[kFace[k][1]], tv[kFace[k][2]]};
            if (vol < 0) std::swap(f[1], f[2]);
            m.sface_tet.push_back(t);
            m.sface_tet.push_back(k);
            for (int i = 0; i < 3; ++i) {
                m.sfaces.push_back(f[i]);
                on[size_t(f[i])] = 1;
            }
        }
    }
    m.sverts.clear();
    for (int32_t v = 0; v < m.nv; ++v)
        if (on[size_t(v)]) m.sverts.push_back(v);
    // face across each edge, and the surface ring of every vertex
    const size_t nf = m.sfaces.size() / 3;
    struct Edge {
        int32_t lo, hi, face, k;
    };
    std::vector<Edge> edges;
    edges.reserve(3 * nf);
    for (size_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) {
            const int32_t a = m.sfaces[3 * f + k], b = m.sfaces[3 * f + (k + 1) % 3];
            edges.push_back(Edge{std::min(a, b), std::max(a, b), int32_t(f), k});
        }
    std::sort(edges.begin(), edges.end(), [](const Edge& x, const Edge& y) {
        return x.lo != y.lo ? x.lo < y.lo : (x.hi != y.hi ? x.hi < y.hi : x.face < y.face);
    });
    m.sface_nbr.assign(3 * nf, -1);
    std::vector<std::vector<int32_t>> ring(static_cast<size_t>(m.nv));
    for (size_t i = 0; i < edges.size();) {
        size_t j = i;
        while (j < edges.size() && edges[j].lo == edges[i].lo && edges[j].hi == edges[i].hi) ++j;
        // each face takes the first other face on the edge
        for (size_t a = i; a < j; ++a)
            for (size_t b = i; b < j; ++b)
                if (edges[b].face != edges[a].face) {
                    m.sface_nbr[3 * size_t(edges[a].face) + size_t(edges[a].k)] = edges[b].face;
                    break;
                }
        ring[size_t(edges[i].lo)].push_back(edges[i].hi);
        ring[size_t(edges[i].hi)].push_back(edges[i].lo);
        i = j;
    }
    m.sring_ofs.assign(size_t(m.nv) + 1, 0);
    m.sring.clear();
    for (int32_t v = 0; v < m.nv; ++v) {
        auto& r = ring[size_t(v)];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        m.sring.insert(m.sring.end(), r.begin(), r.end());
        m.sring_ofs[size_t(v) + 1] = int32_t(m.sring.size());
    }
}

// Rest shape (TetMesh/TetMeshFEM.cpp:332-443): rotation (axis-angle), scale,
// translation; Dm = [x1-x0, x2-x0, x3-x0], DmInv = Dm^-1, volume = det/6,
// lumped mass. DmInv/volume/mass are computed in FP64 from the FP32 positions.
void prepare_mesh(const PhysicsParams& p, const ObjectParams& o, TetMesh& m) {
    (void)p;
    m.nv = int32_t(m.X.size() / 3);
    m.ntet = int32_t(m.tets.size() / 4);
    double rot = std::sqrt(o.rotation[0] * o.rotation[0] + o.rotation[1] * o.rotation[1] + o.rotation[2] * o.rotation[2]);
    if (rot > 0) {
        double a[3] = {o.rotation[0] / rot, o.rotation[1] / rot, o.rotation[2] / rot};
        double c = std::cos(rot), s = std::sin(rot), C = 1 - c;
        double R[9] = {c + a[0] * a[0] * C, a[0] * a[1] * C - a[2] * s, a[0] * a[2] * C + a[1] * s,
                       a[1] * a[0] * C + a[2] * s, c + a[1] * a[1] * C, a[1] * a[2] * C - a[0] * s,
                       a[2] * a[0] * C - a[1] * s, a[2] * a[1] * C + a[0] * s, c + a[2] * a[2] * C};
        for (int32_t v = 0; v < m.nv; ++v) {
            double x[3] = {m.X[3 * size_t(v)], m.X[3 * size_t(v) + 1], m.X[3 * size_t(v) + 2]};
            for (int r = 0; r < 3; ++r) m.X[3 * size_t(v) + r] = float(R[3 * r] * x[0] + R[3 * r + 1] * x[1] + R[3 * r + 2] * x[2]);
        }
    }
    for (int32_t v = 0; v < m.nv; ++v)
        for (int r = 0; r < 3; ++r) {
            float& x = m.X[3 * size_t(v) + r];
            x = x * float(o.scale[r]);
            x = x + float(o.translation[r]);
        }
    m.V.assign(3 * size_t(m.nv), 0.f);
    for (int32_t v = 0; v < m.nv; ++v)
        for (int r = 0; r < 3; ++r) m.V[3 * size_t(v) + r] = float(o.initialVelocity[r]);

    m.dminv.assign(9 * size_t(m.ntet), 0.0);
    m.vol.assign(m.ntet, 0.0);
    m.mass.assign(m.nv, 0.0);
    for (int32_t t = 0; t < m.ntet; ++t) {
        const int32_t* tv = &m.tets[4 * size_t(t)];
        double D[9];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                D[3 * c + r] = double(m.X[3 * size_t(tv[c + 1]) + r]) - double(m.X[3 * size_t(tv[0]) + r]);
        auto A = [&](int r, int c) { return D[3 * c + r]; };
        double c00 = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
        double c01 = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
        double c02 = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
        double det = A(0, 0) * c00 + A(0, 1) * c01 + A(0, 2) * c02;
        if (!(std::fabs(det) > 0.0) || !std::isfinite(det))
            throw std::runtime_error("degenerate tet " + std::to_string(t) + " (zero rest volume)");
        double id = 1.0 / det;
        double* inv = &m.dminv[9 * size_t(t)];
        inv[0] = c00 * id;
        inv[3] = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) * id;
        inv[6] = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) * id;
        inv[1] = c01 * id;
        inv[4] = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) * id;
        inv[7] = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) * id;
        inv[2] = c02 * id;
        inv[5] = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) * id;
        inv[8] = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) * id;
        double vol = det / 6.0;
        m.vol[t] = vol;
        for (int i = 0; i < 4; ++i) m.mass[tv[i]] += 0.25 * vol * o.density;
    }
    // CSR vertex -> incident tets, ascending tet id (TetMeshFEM.cpp:276-324)
    m.nbr_ofs.assign(size_t(m.nv) + 1, 0);
    for (int32_t t = 0; t < m.ntet; ++t)
        for (int i = 0; i < 4; ++i) m.nbr_ofs[m.tets[4 * size_t(t) + i] + 1]++;
    for (int32_t v = 0; v < m.nv; ++v) m.nbr_ofs[v + 1] += m.nbr_ofs[v];
    m.nbr_tet.assign(m.nbr_ofs[m.nv], 0);
    m.nbr_order.assign(m.nbr_ofs[m.nv], 0);
    std::vector<int32_t> fill(m.nbr_ofs.begin(), m.nbr_ofs.end() - 1);
    for (int32_t t = 0; t < m.ntet; ++t)
        for (int i = 0; i < 4; ++i) {
            int32_t v = m.tets[4 * size_t(t) + i];
            m.nbr_tet[fill[v]] = t;
            m.nbr_order[fill[v]] = i;
            fill[v]++;
        }
    m.fixed.assign(m.nv, 0);
    for (int32_t v : o.fixedPoints) {
        if (v < 0 || v >= m.nv) throw std::runtime_error("fixed point " + std::to_string(v) + " out of range");
        m.fixed[v] = 1;
    }
}

// VBDPhysics.cpp:99-122 and 235-274: each mesh's colors (already sorted large
// to small) go, in order, to the smallest group this mesh has not used yet.
void build_parallel_groups(Scene& s) {
    size_t ng = 0;
    for (auto& m : s.meshes) ng = std::max(ng, m.colors.size());
    s.groups.assign(ng, {});
    for (size_t im = 0; im < s.meshes.size(); ++im) {
        auto& m = s.meshes[im];
        std::vector<int32_t> avail(m.colors.size());
        for (size_t c = 0; c < avail.size(); ++c) avail[c] = int32_t(c);
        for (size_t c = 0; c < m.colors.size(); ++c) {
            size_t best = s.groups[avail[0]].size(), bestI = 0;
            int32_t bestId = avail[0];
            for (size_t i = 1; i < avail.size(); ++i)
                if (s.groups[avail[i]].size() < best) {
                    best = s.groups[avail[i]].size();
                    bestId = avail[i];
                    bestI = i;
                }
            avail.erase(avail.begin() + bestI);
            auto& g = s.groups[bestId];
            for (int32_t v : m.colors[c]) {
                g.push_back(int32_t(im));
                g.push_back(v);
            }
        }
    }
}

void load_scene(const std::string& models_json, const std::string& params_json, const std::string& repo_root,
                Scene& s) {
    auto subst = [&](const std::string& x) { return repo_root.empty() ? x : replace_all(x, "${REPO_ROOT}", repo_root); };
    json::Value models = json::parse(read_file(subst(models_json)));
    json::Value params = json::parse(read_file(subst(params_json)));

    PhysicsParams& p = s.p;
    if (const json::Value* pp = params.find("PhysicsParams")) {
        get3(*pp, "gravity", p.gravity);
        get(*pp, "timeStep", p.timeStep);
        get(*pp, "numSubsteps", p.numSubsteps);
        get(*pp, "iterations", p.iterations);
        get(*pp, "usePlaneGround", p.usePlaneGround);
        if (auto* wb = pp->find("worldBounds")) {
            if (!wb->is_array() || wb->arr.size() != 2) throw std::runtime_error("worldBounds must be [[lo x,y,z],[hi x,y,z]]");
            for (int i = 0; i < 3; ++i) {
                p.worldLo[i] = wb->arr[0].arr.at(i).num;
                p.worldHi[i] = wb->arr[1].arr.at(i).num;
            }
        }
        get(*pp, "boundaryFrictionDynamic", p.boundaryFrictionDynamic);
        get(*pp, "boundaryFrictionEpsV", p.boundaryFrictionEpsV);
        get(*pp, "boundaryCollisionStiffness", p.boundaryCollisionStiffness);
        get(*pp, "stepSize", p.stepSize);
        get(*pp, "stepSizeGD", p.stepSizeGD);
        get(*pp, "frictionStartIter", p.frictionStartIter);
        get(*pp, "associateGravityWithInertia", p.associateGravityWithInertia);
        get(*pp, "useAccelerator", p.useAccelerator);
        get(*pp, "acceleratorRho", p.acceleratorRho);
        get(*pp, "useGPU", p.useGPU);
        get(*pp, "handleCollision", p.handleCollision);
        get(*pp, "collisionStiffness", p.collisionStiffness);
        get(*pp, "collisionOffHeight", p.collisionOffHeight);
        get(*pp, "intermediateCollisionIterations", p.intermediateCollisionIterations);
        get(*pp, "numThreadsVBDSolve", p.numThreadsVBDSolve);
        get(*pp, "useDouble3x3", p.useDouble3x3);
        get(*pp, "evaluateConvergence", p.evaluateConvergence);
        get(*pp, "evaluationSteps", p.evaluationSteps);
        get(*pp, "numFrames", p.numFrames);
        get(*pp, "saveOutputs", p.saveOutputs);
        get(*pp, "saveAllModelsTogether", p.saveAllModelsTogether);
        get(*pp, "outputExt", p.outputExt);
        get(*pp, "binaryModeVisualizationSteps", p.binaryModeVisualizationSteps);
        get(*pp, "outputRecoveryState", p.outputRecoveryState);
        get(*pp, "outputRecoveryStateStep", p.outputRecoveryStateStep);
        get(*pp, "outputRecoveryStateBinary", p.outputRecoveryStateBinary);
        get(*pp, "gpuPrecision", p.gpuPrecision);
        get(*pp, "lanesPerVertex", p.lanesPerVertex);
        get(*pp, "blockSize", p.blockSize);
        get(*pp, "autotune", p.autotune);
        get(*pp, "usePDL", p.usePDL);
        get(*pp, "smallColorVertices", p.smallColorVertices);
        get(*pp, "solveVariant", p.solveVariant);
        get(*pp, "waitPollLimit", p.waitPollLimit);
        get(*pp, "sweepMode", p.sweepMode);
        get(*pp, "clusterSize", p.clusterSize);
        get(*pp, "meshFrames", p.meshFrames);
    }
    if (const json::Value* cp = params.find("CollisionParams")) {
        get(*cp, "allowCCD", p.allowCCD);
        get(*cp, "allowDCD", p.allowDCD);
        get(*cp, "handleSelfCollision", p.handleSelfCollision);
        get(*cp, "checkFeasibleRegion", p.checkFeasibleRegion);
        get(*cp, "feasibleRegionEpsilon", p.feasibleRegionEpsilon);
        get(*cp, "checkTetTraverse", p.checkTetTraverse);
        get(*cp, "tetrahedralTraverseForNonSelfIntersection", p.tetrahedralTraverseForNonSelfIntersection);
        get(*cp, "stopTraversingAfterPassingQueryPoint", p.stopTraversingAfterPassingQueryPoint);
        get(*cp, "shiftQueryPointToCenter", p.shiftQueryPointToCenter);
        get(*cp, "useStaticTraverse", p.useStaticTraverse);
        get(*cp, "loopLessTraverse", p.loopLessTraverse);
        get(*cp, "centerShiftLevel", p.centerShiftLevel);
        get(*cp, "rayTriIntersectionEPSILON", p.rayTriIntersectionEPSILON);
        get(*cp, "maxSearchDistanceMultiplier", p.maxSearchDistanceMultiplier);
        if (p.loopLessTraverse) throw std::runtime_error("CollisionParams loopLessTraverse is not supported");
    }
    if (p.numSubsteps <= 0 || p.timeStep <= 0) throw std::runtime_error("timeStep and numSubsteps must be positive");
    if (p.iterations < 0) throw std::runtime_error("iterations must be >= 0");
    if (p.evaluationSteps < 1) throw std::runtime_error("evaluationSteps must be >= 1");
    if (p.sweepMode != "auto" && p.sweepMode != "merged" && p.sweepMode != "scenes" && p.sweepMode != "cluster" &&
        p.sweepMode != "grid")
        throw std::runtime_error("sweepMode must be \"auto\", \"merged\", \"scenes\", \"cluster\" or \"grid\"");
    if (p.clusterSize != 0 && p.clusterSize != 2 && p.clusterSize != 4 && p.clusterSize != 8 && p.clusterSize != 16)
        throw std::runtime_error("clusterSize must be 0 (autotune), 2, 4, 8 or 16");
    if (p.gpuPrecision != "fp32" && p.gpuPrecision != "mixed" && p.gpuPrecision != "dfhi" && p.gpuPrecision != "fp64")
        throw std::runtime_error("gpuPrecision must be \"mixed\", \"dfhi\", \"fp32\" or \"fp64\"");
    p.dt = p.timeStep / p.numSubsteps;
    p.dtSqrReciprocal = 1.0 / (p.dt * p.dt);

    const json::Value* ml = models.find("Models");
    if (!ml || !ml->is_array()) throw std::runtime_error("Models.json has no \"Models\" list");
    for (auto& mj : ml->arr) {
        ObjectParams o;
        get(mj, "materialName", o.materialName);
        if (o.materialName != "NeoHookean")
            throw std::runtime_error("material '" + o.materialName + "' is not supported by the VBD tet step (NeoHookean only)");
        get(mj, "path", o.path);
        get(mj, "verticesColoringCategoriesPath", o.verticesColoringCategoriesPath);
        get3(mj, "translationBeforeScaling", o.translationBeforeScaling);
        get3(mj, "scale", o.scale);
        get3(mj, "translation", o.translation);
        get3(mj, "rotation", o.rotation);
        get3(mj, "initialVelocity", o.initialVelocity);
        get(mj, "density", o.density);
        get(mj, "maxVelocityMagnitude", o.maxVelocityMagnitude);
        get(mj, "frameToAppear", o.frameToAppear);
        get_ints(mj, "fixedPoints", o.fixedPoints);
        get(mj, "frictionDynamic", o.frictionDynamic);
        get(mj, "frictionEpsV", o.frictionEpsV);
        get(mj, "exponentialVelDamping", o.exponentialVelDamping);
        get(mj, "constantVelDamping", o.constantVelDamping);
        get(mj, "initializationType", o.initializationType);
        get(mj, "miu", o.miu);
        get(mj, "lmbd", o.lmbd);
        get(mj, "dampingDeviatoric", o.dampingDeviatoric);
        get(mj, "dampingHydrostatic", o.dampingHydrostatic);
        if (!(o.lmbd != 0.0)) throw std::runtime_error("lmbd must be non-zero");
        if (o.initializationType < 0 || o.initializationType > 4)
            throw std::runtime_error("initializationType must be 0..4 for the VBD step");
        o.path = subst(o.path);
        o.verticesColoringCategoriesPath = subst(o.verticesColoringCategoriesPath);
        s.objs.push_back(o);
    }
    if (s.objs.empty()) throw std::runtime_error("Models.json lists no models");

    s.meshes.resize(s.objs.size());
    for (size_t i = 0; i < s.objs.size(); ++i) {
        TetMesh& m = s.meshes[i];
        load_t(s.objs[i].path, m.X, m.tets);
        prepare_mesh(p, s.objs[i], m);
        extract_surface(m);
        if (!s.objs[i].verticesColoringCategoriesPath.empty()) {
            m.colors = load_coloring(s.objs[i].verticesColoringCategoriesPath);
        } else {
            std::vector<int32_t> col(m.nv);
            if (color_greedy(m.nv, m.ntet, m.tets.data(), col.data()) < 0)
                throw std::runtime_error("greedy coloring failed for " + s.objs[i].path);
            m.colors = colors_to_categories(m.nv, col.data());
        }
        validate_coloring(m);
        // TetMeshFEM.cpp:122-134: large to small, std::sort (not stable), as in the reference
        std::sort(m.colors.begin(), m.colors.end(),
                  [](const std::vector<int32_t>& a, const std::vector<int32_t>& b) { return a.size() > b.size(); });
    }

    if (const json::Value* dl = params.find("Deformers")) {
        if (!dl->is_array()) throw std::runtime_error("Deformers must be a list");
        for (auto& dj : dl->arr) {
            DeformerParams d;
            std::string name;
            get(dj, "DeformerName", name);
            if (name == "Rotator") {
                d.type = 0;
                get3(dj, "center", d.center);
                get3(dj, "axis", d.axis);
                get(dj, "angularVelocity", d.angularVelocity);
                get(dj, "rotationEndTime", d.endTime);
            } else if (name == "Translator") {
                d.type = 1;
                get3(dj, "speed", d.speed);
                get(dj, "deformationEndTime", d.endTime);
            } else {
                throw std::runtime_error("unrecognized deformer: " + name);
            }
            get_ints(dj, "selectedMeshes", d.selectedMeshes);
            if (auto* sv = dj.find("selectedVertices")) {
                for (auto& l : sv->arr) {
                    std::vector<int32_t> vs;
                    for (auto& e : l.arr) vs.push_back(int32_t(e.num));
                    d.selectedVertices.push_back(vs);
                }
            }
            if (d.selectedVertices.size() != d.selectedMeshes.size())
                throw std::runtime_error("deformer selectedMeshes / selectedVertices size mismatch");
            for (size_t k = 0; k < d.selectedMeshes.size(); ++k) {
                int32_t mi = d.selectedMeshes[k];
                if (mi < 0 || size_t(mi) >= s.meshes.size()) throw std::runtime_error("deformer mesh index out of range");
                for (int32_t v : d.selectedVertices[k]) {
                    if (v < 0 || v >= s.meshes[mi].nv) throw std::runtime_error("deformer vertex out of range");
                    s.meshes[mi].fixed[v] = 1;  // setFixed (VBDDeformer.h:20-43)
                }
            }
            s.defs.push_back(d);
        }
    }
    build_parallel_groups(s);
}

void write_t(const std::string& path, int32_t nv, const double* X, int32_t ntet, const int32_t* tets) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::vector<char> buf(1 << 20);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    for (int32_t v = 0; v < nv; ++v)
        std::fprintf(f, "Vertex %d %.9g %.9g %.9g\n", v, X[3 * size_t(v)], X[3 * size_t(v) + 1], X[3 * size_t(v) + 2]);
    for (int32_t t = 0; t < ntet; ++t)
        std::fprintf(f, "Tet %d %d %d %d %d\n", t, tets[4 * size_t(t)], tets[4 * size_t(t) + 1], tets[4 * size_t(t) + 2],
                     tets[4 * size_t(t) + 3]);
    std::fclose(f);
}

void write_coloring(const std::string& path, const std::vector<std::vector<int32_t>>& cats) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fputc('[', f);
    for (size_t c = 0; c < cats.size(); ++c) {
        if (c) std::fputc(',', f);
        std::fputc('[', f);
        for (size_t i = 0; i < cats[c].size(); ++i) std::fprintf(f, i ? ",%d" : "%d", cats[c][i]);
        std::fputc(']', f);
    }
    std::fputc(']', f);
    std::fclose(f);
}

}  // namespace gaia
