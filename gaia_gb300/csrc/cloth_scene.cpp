// Host-side cloth scene set-up: JSON inputs, .obj meshes, topology, rest shape,
// colorings and parallel-group merge. See cloth_scene.hpp.
#include "cloth_scene.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>

#include "json_get.hpp"
#include "scene.hpp"

namespace gaia {
namespace cloth {

using namespace jsonio;

// TriMeshFEM::loadObj (TriMesh/TriMesh.cpp:280-407): "v x y z" lines and the
// first three vertex indices of every "f" line (1-based, "a/b/c" accepted).
// Coordinates are parsed as double and rounded to float.
void load_obj(const std::string& path, std::vector<float>& X, std::vector<int32_t>& faces) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) throw std::runtime_error("cannot open mesh file: " + path);
    X.clear();
    faces.clear();
    char line[4096];
    while (std::fgets(line, sizeof(line), f)) {
        char* s = line;
        while (*s == ' ' || *s == '\t') ++s;
        if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
            char* p = s + 2;
            for (int i = 0; i < 3; ++i) {
                char* e = nullptr;
                double d = std::strtod(p, &e);
                if (e == p) {
                    std::fclose(f);
                    throw std::runtime_error("bad vertex line in " + path);
                }
                X.push_back(float(d));
                p = e;
            }
        } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
            char* p = s + 2;
            int32_t idx[3];
            for (int i = 0; i < 3; ++i) {
                char* e = nullptr;
                long v = std::strtol(p, &e, 10);
                if (e == p) {
                    std::fclose(f);
                    throw std::runtime_error("bad face line in " + path);
                }
                idx[i] = int32_t(v - 1);
                p = e;
                while (*p && *p != ' ' && *p != '\t' && *p != '\n' && *p != '\r') ++p;  // skip "/uv/n"
            }
            faces.insert(faces.end(), idx, idx + 3);
        }
    }
    std::fclose(f);
    const int32_t nv = int32_t(X.size() / 3);
    for (int32_t v : faces)
        if (v < 0 || v >= nv) throw std::runtime_error("face references a vertex out of range in " + path);
}

namespace {

// TriMeshFEM::applyRotationScalingTranslation (TriMesh/TriMesh.cpp:113-132):
// axis-angle rotation, then per-axis scale, then translation.
void apply_transform(const double* rotation, const double* scale, const double* translation, std::vector<float>& X) {
    const size_t nv = X.size() / 3;
    double rot = std::sqrt(rotation[0] * rotation[0] + rotation[1] * rotation[1] + rotation[2] * rotation[2]);
    if (rot > 0) {
        double a[3] = {rotation[0] / rot, rotation[1] / rot, rotation[2] / rot};
        double c = std::cos(rot), s = std::sin(rot), C = 1 - c;
        double R[9] = {c + a[0] * a[0] * C, a[0] * a[1] * C - a[2] * s, a[0] * a[2] * C + a[1] * s,
                       a[1] * a[0] * C + a[2] * s, c + a[1] * a[1] * C, a[1] * a[2] * C - a[0] * s,
                       a[2] * a[0] * C - a[1] * s, a[2] * a[1] * C + a[0] * s, c + a[2] * a[2] * C};
        for (size_t v = 0; v < nv; ++v) {
            double x[3] = {X[3 * v], X[3 * v + 1], X[3 * v + 2]};
            for (int r = 0; r < 3; ++r) X[3 * v + r] = float(R[3 * r] * x[0] + R[3 * r + 1] * x[1] + R[3 * r + 2] * x[2]);
        }
    }
    for (size_t v = 0; v < nv; ++v)
        for (int r = 0; r < 3; ++r) {
            float& x = X[3 * v + r];
            x = x * float(scale[r]);
            x = x + float(translation[r]);
        }
}

void csr_from_lists(const std::vector<std::vector<std::pair<int32_t, int32_t>>>& lists, std::vector<int32_t>& ofs,
                    std::vector<int32_t>& ids, std::vector<int32_t>* order) {
    ofs.assign(lists.size() + 1, 0);
    ids.clear();
    if (order) order->clear();
    for (size_t v = 0; v < lists.size(); ++v) {
        for (auto& e : lists[v]) {
            ids.push_back(e.first);
            if (order) order->push_back(e.second);
        }
        ofs[v + 1] = int32_t(ids.size());
    }
}

double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
double norm3(const double* a) { return std::sqrt(dot3(a, a)); }

}  // namespace

void orthonormal_basis(const double n[3], double t[3], double b[3]) {
    const double sign = std::copysign(1.0, n[2]);
    const double a = -1.0 / (sign + n[2]);
    const double bb = n[0] * n[1] * a;
    t[0] = 1.0 + sign * n[0] * n[0] * a;
    t[1] = sign * bb;
    t[2] = -sign * n[0];
    b[0] = bb;
    b[1] = sign + n[1] * n[1] * a;
    b[2] = -n[1];
}

// TriMeshTopology::initialize (TriMesh/TriMesh.cpp:481-750). Edges are numbered in
// order of first appearance over the faces' half-edges (f0->f1, f1->f2, f2->f0);
// the first half-edge of an edge gives v1, v2, f1 and v12next, the opposite
// half-edge f2 and v21next. Neighbour lists are in ascending id order.
void build_topology(TriMesh& m) {
    m.nv = int32_t(m.X.size() / 3);
    m.nf = int32_t(m.faces.size() / 3);
    m.edges.clear();
    m.faceEdges.assign(3 * size_t(m.nf), -1);
    std::map<std::pair<int32_t, int32_t>, int32_t> key;
    for (int32_t f = 0; f < m.nf; ++f) {
        const int32_t* fv = &m.faces[3 * size_t(f)];
        if (fv[0] == fv[1] || fv[1] == fv[2] || fv[0] == fv[2])
            throw std::runtime_error("degenerate face " + std::to_string(f) + " (repeated vertex)");
        for (int i = 0; i < 3; ++i) {
            int32_t a = fv[i], b = fv[(i + 1) % 3], c = fv[(i + 2) % 3];
            auto k = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = key.find(k);
            if (it == key.end()) {
                Edge e{a, b, c, -1, f, -1};
                key.emplace(k, int32_t(m.edges.size()));
                m.faceEdges[3 * size_t(f) + i] = int32_t(m.edges.size());
                m.edges.push_back(e);
            } else {
                Edge& e = m.edges[it->second];
                if (e.f2 != -1) throw std::runtime_error("non-manifold edge (" + std::to_string(a) + ", " +
                                                         std::to_string(b) + "): more than two faces");
                if (e.v1 != b || e.v2 != a)
                    throw std::runtime_error("inconsistently oriented faces at edge (" + std::to_string(a) + ", " +
                                             std::to_string(b) + ")");
                e.f2 = f;
                e.v21next = c;
                m.faceEdges[3 * size_t(f) + i] = it->second;
            }
        }
    }
    m.ne = int32_t(m.edges.size());

    std::vector<std::vector<std::pair<int32_t, int32_t>>> vv(m.nv), vf(m.nv), ve(m.nv), vb(m.nv);
    for (int32_t f = 0; f < m.nf; ++f)
        for (int i = 0; i < 3; ++i) vf[m.faces[3 * size_t(f) + i]].push_back({f, i});
    for (int32_t e = 0; e < m.ne; ++e) {
        const Edge& E = m.edges[e];
        vv[E.v1].push_back({E.v2, 0});
        vv[E.v2].push_back({E.v1, 0});
        ve[E.v1].push_back({e, 0});
        ve[E.v2].push_back({e, 1});
    }
    for (int32_t v = 0; v < m.nv; ++v) {
        std::sort(vv[v].begin(), vv[v].end());
        std::sort(vf[v].begin(), vf[v].end());
        std::sort(ve[v].begin(), ve[v].end());
        // relevant bendings (TriMesh.cpp:660-716): interior edges through v (order 0 / 1),
        // then for every incident face the interior edge across from v (order 2 when the
        // face is the edge's f1, i.e. v is v12next, else 3)
        for (auto& e : ve[v])
            if (m.edges[e.first].f2 != -1) vb[v].push_back(e);
        for (auto& fo : vf[v]) {
            int32_t f = fo.first, i = fo.second;
            int32_t e = m.faceEdges[3 * size_t(f) + (i + 1) % 3];  // edge opposite vertex i
            const Edge& E = m.edges[e];
            if (E.f2 == -1) continue;
            vb[v].push_back({e, E.f1 == f ? 2 : 3});
        }
    }
    csr_from_lists(vv, m.nbrVOfs, m.nbrV, nullptr);
    csr_from_lists(vf, m.nbrFOfs, m.nbrF, &m.nbrFOrder);
    csr_from_lists(ve, m.nbrEOfs, m.nbrE, &m.nbrEOrder);
    csr_from_lists(vb, m.bendOfs, m.bendE, &m.bendOrder);
}

// Rest shape of a simulated mesh: TriMeshFEM::computeRestposeTrianglesFrom3D
// (TriMesh/TriMesh.cpp:213-244): each face projected to 2D on an orthonormal basis
// of its normal, Dm = [x1 - x0, x2 - x0] in that basis, area = det(Dm) / 2,
// DmInv = Dm^-1, vertex mass += density * area / 3; and the bending quadratic
// forms of VBDTriMeshStVk::intializeEdgeQuadraticForms (VBDCloth/VBDTriMeshStVK.cpp:50-89):
// Q = 3 K K^T / (A0 + A1) with cotangent weights K and A = |cross| of the two faces.
// FP64 throughout.
void prepare_rest_shape(const ObjectParams& o, TriMesh& m) {
    if (!o.use3DRestpose)
        throw std::runtime_error("use3DRestpose = false (UV rest shape) is not supported by the cloth step");
    auto X = [&](int32_t v, double* out) {
        for (int r = 0; r < 3; ++r) out[r] = double(m.X[3 * size_t(v) + r]);
    };
    m.dminv.assign(4 * size_t(m.nf), 0.0);
    m.area.assign(m.nf, 0.0);
    m.mass.assign(m.nv, 0.0);
    for (int32_t f = 0; f < m.nf; ++f) {
        const int32_t* fv = &m.faces[3 * size_t(f)];
        double x0[3], x1[3], x2[3], e1[3], e2[3], n[3];
        X(fv[0], x0);
        X(fv[1], x1);
        X(fv[2], x2);
        for (int r = 0; r < 3; ++r) {
            e1[r] = x1[r] - x0[r];
            e2[r] = x2[r] - x0[r];
        }
        cross3(e1, e2, n);
        double nn = norm3(n);
        if (!(nn > 0.0)) throw std::runtime_error("degenerate face " + std::to_string(f) + " (zero rest area)");
        for (int r = 0; r < 3; ++r) n[r] /= nn;
        double t[3], b[3];
        orthonormal_basis(n, t, b);
        double D00 = dot3(t, e1), D10 = dot3(b, e1), D01 = dot3(t, e2), D11 = dot3(b, e2);
        double det = D00 * D11 - D01 * D10;
        m.area[f] = 0.5 * det;
        double* inv = &m.dminv[4 * size_t(f)];  // column-major 2x2
        inv[0] = D11 / det;
        inv[1] = -D10 / det;
        inv[2] = -D01 / det;
        inv[3] = D00 / det;
        for (int i = 0; i < 3; ++i) m.mass[fv[i]] += o.density * m.area[f] / 3.0;
    }
    m.bendQ.assign(16 * size_t(m.ne), 0.0);
    for (int32_t e = 0; e < m.ne; ++e) {
        const Edge& E = m.edges[e];
        if (E.f2 == -1) continue;
        double p0[3], p1[3], p2[3], p3[3];
        X(E.v1, p0);
        X(E.v2, p1);
        X(E.v12next, p2);
        X(E.v21next, p3);
        double e01[3], e02[3], e03[3], e12[3], e13[3], m01[3];
        for (int r = 0; r < 3; ++r) {
            e01[r] = p1[r] - p0[r];
            e02[r] = p2[r] - p0[r];
            e03[r] = p3[r] - p0[r];
            e12[r] = p2[r] - p1[r];
            e13[r] = p3[r] - p1[r];
            m01[r] = -e01[r];
        }
        auto cot = [](const double* a, const double* b) {
            double c[3];
            cross3(a, b, c);
            return dot3(a, b) / norm3(c);
        };
        double c01 = cot(e02, e01), c02 = cot(e01, e03), c03 = cot(m01, e12), c04 = cot(m01, e13);
        double K[4] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
        double n1[3], n2[3], a1[3], a2[3], b1[3], b2[3];
        const int32_t* f1 = &m.faces[3 * size_t(E.f1)];
        const int32_t* f2 = &m.faces[3 * size_t(E.f2)];
        double q0[3], q1[3], q2[3];
        X(f1[0], q0);
        X(f1[1], q1);
        X(f1[2], q2);
        for (int r = 0; r < 3; ++r) {
            a1[r] = q1[r] - q0[r];
            b1[r] = q2[r] - q0[r];
        }
        X(f2[0], q0);
        X(f2[1], q1);
        X(f2[2], q2);
        for (int r = 0; r < 3; ++r) {
            a2[r] = q1[r] - q0[r];
            b2[r] = q2[r] - q0[r];
        }
        cross3(a1, b1, n1);
        cross3(a2, b2, n2);
        double A0 = norm3(n1), A1 = norm3(n2);
        double* Q = &m.bendQ[16 * size_t(e)];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) Q[4 * i + j] = 3.0 * K[i] * K[j] / (A0 + A1);
    }
    m.fixed.assign(m.nv, 0);
    for (int32_t v : o.fixedPoints) {
        if (v < 0 || v >= m.nv) throw std::runtime_error("fixed point index out of range");
        m.fixed[v] = 1;
    }
}

void tri_vertex_graph(const TriMesh& m, bool bending, std::vector<int64_t>& ofs, std::vector<int32_t>& adj) {
    std::vector<std::vector<int32_t>> nb(m.nv);
    for (const Edge& E : m.edges) {
        nb[E.v1].push_back(E.v2);
        nb[E.v2].push_back(E.v1);
        if (bending && E.f2 != -1) {
            nb[E.v12next].push_back(E.v21next);
            nb[E.v21next].push_back(E.v12next);
        }
    }
    ofs.assign(size_t(m.nv) + 1, 0);
    adj.clear();
    for (int32_t v = 0; v < m.nv; ++v) {
        std::sort(nb[v].begin(), nb[v].end());
        nb[v].erase(std::unique(nb[v].begin(), nb[v].end()), nb[v].end());
        adj.insert(adj.end(), nb[v].begin(), nb[v].end());
        ofs[v + 1] = int64_t(adj.size());
    }
}

// VBDClothSimulationFramework::initializeParallelGroups (VBDCloth/VBDClothPhysics.cpp:72-138):
// the number of groups is the largest color count of any mesh; each color of each mesh
// joins the currently smallest group among the first (its mesh's color count) groups,
// lowest index on ties. Unlike the tet merge, a group is not removed from the candidates
// after a color of the same mesh joined it.
void build_parallel_groups(Scene& s) {
    size_t ng = 0;
    for (int i = 0; i < s.numSim; ++i) ng = std::max(ng, s.meshes[i].colors.size());
    s.groups.assign(ng, {});
    for (int i = 0; i < s.numSim; ++i) {
        const TriMesh& m = s.meshes[i];
        const size_t nc = m.colors.size();
        for (size_t c = 0; c < nc; ++c) {
            size_t best = 0;
            for (size_t g = 1; g < nc; ++g)
                if (s.groups[g].size() < s.groups[best].size()) best = g;
            for (int32_t v : m.colors[c]) {
                s.groups[best].push_back(i);
                s.groups[best].push_back(v);
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
        if (auto* wb = pp->find("worldBounds")) {
            if (!wb->is_array() || wb->arr.size() != 2) throw std::runtime_error("worldBounds must be [[lo x,y,z],[hi x,y,z]]");
            for (int i = 0; i < 3; ++i) {
                p.worldLo[i] = wb->arr[0].arr.at(i).num;
                p.worldHi[i] = wb->arr[1].arr.at(i).num;
            }
        }
        get(*pp, "boundaryFrictionDynamic", p.boundaryFrictionDynamic);
        get(*pp, "stepSize", p.stepSize);
        get(*pp, "associateGravityWithInertia", p.associateGravityWithInertia);
        get(*pp, "handleCollision", p.handleCollision);
        get(*pp, "contactStiffness", p.contactStiffness);
        get(*pp, "contactRadius", p.contactRadius);
        get(*pp, "thickness", p.thickness);
        get(*pp, "conservativeStepRelaxation", p.conservativeStepRelaxation);
        get(*pp, "boundaryFrictionEpsValue", p.boundaryFrictionEpsValue);
        get(*pp, "contactBVHReconstructionSteps", p.contactBVHReconstructionSteps);
        get(*pp, "applyAcceleration", p.applyAcceleration);
        get(*pp, "acceleratorRho", p.acceleratorRho);
        get(*pp, "useNewton", p.useNewton);
        get(*pp, "gpuPrecision", p.gpuPrecision);
        get(*pp, "contactDetectionEveryIteration", p.contactDetectionEveryIteration);
        get(*pp, "blockSize", p.blockSize);
        get(*pp, "lanesPerVertex", p.lanesPerVertex);
    }
    if (const json::Value* cp = params.find("ContactDetectorParams")) get(*cp, "maxQueryDis", p.maxQueryDis);
    if (p.numSubsteps <= 0 || p.timeStep <= 0) throw std::runtime_error("timeStep and numSubsteps must be positive");
    if (p.iterations < 0) throw std::runtime_error("iterations must be >= 0");
    if (p.useNewton) throw std::runtime_error("useNewton = true (Newton solver) is not part of the VBD cloth step");
    if (p.gpuPrecision != "fp32" && p.gpuPrecision != "fp64" && p.gpuPrecision != "mixed")
        throw std::runtime_error("cloth gpuPrecision must be \"fp32\", \"mixed\" or \"fp64\"");
    if (p.blockSize < 32 || p.blockSize > 128 || p.blockSize % 32)
        throw std::runtime_error("blockSize must be 32, 64, 96 or 128");
    if (p.lanesPerVertex != 0 && p.lanesPerVertex != 1 && p.lanesPerVertex != 2 && p.lanesPerVertex != 4 &&
        p.lanesPerVertex != 8 && p.lanesPerVertex != 16 && p.lanesPerVertex != 32)
        throw std::runtime_error("lanesPerVertex must be 0 (autotune), 1, 2, 4, 8, 16 or 32");
    if (!(p.maxQueryDis > 0)) throw std::runtime_error("maxQueryDis must be positive");
    p.dt = p.timeStep / p.numSubsteps;
    p.dtSqrReciprocal = 1.0 / (p.dt * p.dt);

    const json::Value* ml = models.find("Models");
    if (!ml || !ml->is_array()) throw std::runtime_error("Models.json has no \"Models\" list");
    for (auto& mj : ml->arr) {
        ObjectParams o;
        std::string material = "StVK_triMesh";
        get(mj, "materialName", material);
        if (material != "StVK_triMesh" && material != "StVK")
            throw std::runtime_error("material '" + material + "' is not supported by the cloth VBD step (StVK_triMesh)");
        get(mj, "path", o.path);
        o.path = subst(o.path);
        get(mj, "verticesColoringCategoriesPath", o.verticesColoringCategoriesPath);
        o.verticesColoringCategoriesPath = subst(o.verticesColoringCategoriesPath);
        get3(mj, "scale", o.scale);
        get3(mj, "translation", o.translation);
        get3(mj, "rotation", o.rotation);
        get(mj, "density", o.density);
        get(mj, "maxVelocityMagnitude", o.maxVelocityMagnitude);
        get(mj, "hasNoGravZone", o.hasNoGravZone);
        get(mj, "noGravZoneThreshold", o.noGravZoneThreshold);
        get_ints(mj, "fixedPoints", o.fixedPoints);
        get(mj, "use3DRestpose", o.use3DRestpose);
        get(mj, "frictionDynamic", o.frictionDynamic);
        get(mj, "frictionEpsV", o.frictionEpsV);
        get(mj, "bendingStiffness", o.bendingStiffness);
        get(mj, "exponentialVelDamping", o.exponentialVelDamping);
        get(mj, "constantVelDamping", o.constantVelDamping);
        get(mj, "initializationType", o.initializationType);
        get(mj, "miu", o.miu);
        get(mj, "lambda", o.lambda);
        get(mj, "dampingStVK", o.dampingStVK);
        get(mj, "dampingBending", o.dampingBending);
        if (o.initializationType < 0 || o.initializationType > 4)
            throw std::runtime_error("initializationType must be 0..4");
        s.objs.push_back(o);
    }
    s.numSim = int(s.objs.size());
    s.meshes.resize(s.numSim);
    for (int i = 0; i < s.numSim; ++i) {
        const ObjectParams& o = s.objs[i];
        TriMesh& m = s.meshes[i];
        if (o.path.size() < 4 || o.path.substr(o.path.size() - 4) != ".obj")
            throw std::runtime_error("cloth mesh must be an .obj file: " + o.path);
        load_obj(o.path, m.X, m.faces);
        apply_transform(o.rotation, o.scale, o.translation, m.X);
        build_topology(m);
        prepare_rest_shape(o, m);
        if (!o.verticesColoringCategoriesPath.empty()) {
            m.colors = load_coloring(o.verticesColoringCategoriesPath);
        } else {
            std::vector<int64_t> ofs;
            std::vector<int32_t> adj;
            tri_vertex_graph(m, false, ofs, adj);
            std::vector<int32_t> col(m.nv);
            if (color_greedy_graph(m.nv, ofs, adj, col.data()) < 0) throw std::runtime_error("greedy coloring failed");
            m.colors = colors_to_categories(m.nv, col.data());
        }
        std::vector<int32_t> seen(m.nv, 0);
        for (auto& c : m.colors)
            for (int32_t v : c) {
                if (v < 0 || v >= m.nv) throw std::runtime_error("coloring references a vertex out of range");
                seen[v] += 1;
            }
        for (int32_t v = 0; v < m.nv; ++v)
            if (seen[v] != 1) throw std::runtime_error("coloring does not cover every vertex exactly once");
        // TriMesh.cpp:744-749: sorted large to small
        std::sort(m.colors.begin(), m.colors.end(),
                  [](const std::vector<int32_t>& a, const std::vector<int32_t>& b) { return a.size() > b.size(); });
    }

    // ColliderParams.ColliderMeshes (Framework/BaseClothSimPhsicsFramework.cpp:80-112): static
    // "TriMeshSequence" colliders with one mesh file
    if (const json::Value* cp = params.find("ColliderParams")) {
        if (const json::Value* cl = cp->find("ColliderMeshes")) {
            for (auto& cj : cl->arr) {
                std::string type;
                get(cj, "colliderType", type);
                if (type != "TriMeshSequence") throw std::runtime_error("unrecognized collider type: " + type);
                std::vector<std::string> files;
                if (auto* mf = cj.find("meshFiles"))
                    for (auto& e : mf->arr) files.push_back(subst(e.str));
                if (files.size() != 1)
                    throw std::runtime_error("only static colliders (one entry in meshFiles) are supported");
                ObjectParams o;
                get3(cj, "scale", o.scale);
                get3(cj, "translation", o.translation);
                get3(cj, "rotation", o.rotation);
                get(cj, "frictionDynamic", o.frictionDynamic);
                get(cj, "frictionEpsV", o.frictionEpsV);
                TriMesh m;
                load_obj(files[0], m.X, m.faces);
                apply_transform(o.rotation, o.scale, o.translation, m.X);
                build_topology(m);
                s.meshes.push_back(std::move(m));
                s.colliderFriction.push_back(o.frictionDynamic);
                s.colliderFriction.push_back(o.frictionEpsV);
            }
        }
    }
    build_parallel_groups(s);
}

}  // namespace cloth
}  // namespace gaia
