// PhysicsState recovery files. See state_io.hpp.
#include "state_io.hpp"

#include <cstdio>
#include <fstream>
#include <stdexcept>

#include "json_get.hpp"
#include "json_lite.hpp"

namespace gaia {

namespace {

std::string dir_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string(".") : path.substr(0, k);
}

// file name without directory and extension (MF::IO::FileParts::name)
std::string stem_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    std::string name = k == std::string::npos ? path : path.substr(k + 1);
    const size_t d = name.find_last_of('.');
    return d == std::string::npos ? name : name.substr(0, d);
}

void put_float(std::string& out, float v) {
    char buf[32];
    std::snprintf(buf, sizeof(buf), "%.9g", double(v));
    out += buf;
}

void put_vec3_list(std::string& out, const std::vector<float>& a) {
    out += "[";
    for (size_t i = 0; i + 2 < a.size(); i += 3) {
        if (i) out += ", ";
        out += "[";
        put_float(out, a[i]);
        out += ", ";
        put_float(out, a[i + 1]);
        out += ", ";
        put_float(out, a[i + 2]);
        out += "]";
    }
    out += "]";
}

std::vector<float> get_vec3_list(const json::Value& v, const char* what) {
    if (!v.is_array()) throw std::runtime_error(std::string("state file: ") + what + " is not a list");
    std::vector<float> out;
    out.reserve(3 * v.arr.size());
    for (auto& p : v.arr) {
        if (!p.is_array() || p.arr.size() != 3) throw std::runtime_error(std::string("state file: bad entry in ") + what);
        for (int k = 0; k < 3; ++k) out.push_back(float(p.arr[k].num));
    }
    return out;
}

}  // namespace

void write_physics_state(const std::string& path, const PhysicsStateFile& s, bool binary) {
    if (s.position.size() != s.velocity.size()) throw std::invalid_argument("state: position/velocity mesh counts differ");
    std::string j = "{\n  \"frameId\": " + std::to_string(s.frameId) + ",\n  \"curTime\": ";
    char buf[40];
    std::snprintf(buf, sizeof(buf), "%.17g", s.curTime);
    j += buf;
    if (binary) {
        const std::string base = stem_of(path);
        const std::string dir = dir_of(path);
        std::ofstream vf(dir + "/" + base + ".vel", std::ios::binary), pf(dir + "/" + base + ".pos", std::ios::binary);
        if (!vf || !pf) throw std::runtime_error("cannot write state files next to " + path);
        std::string nverts;
        for (size_t m = 0; m < s.position.size(); ++m) {
            if (s.position[m].size() != s.velocity[m].size())
                throw std::invalid_argument("state: position/velocity sizes differ");
            vf.write(reinterpret_cast<const char*>(s.velocity[m].data()), std::streamsize(s.velocity[m].size() * sizeof(float)));
            pf.write(reinterpret_cast<const char*>(s.position[m].data()), std::streamsize(s.position[m].size() * sizeof(float)));
            nverts += (m ? ", " : "") + std::to_string(s.position[m].size() / 3);
        }
        j += ",\n  \"format\": \"binary\",\n  \"nMeshes\": " + std::to_string(s.position.size()) +
             ",\n  \"meshesState\": {\"nVerts\": [" + nverts + "], \"velocities_file\": \"" + base +
             ".vel\", \"position_file\": \"" + base + ".pos\"}\n}\n";
    } else {
        j += ",\n  \"format\": \"text\",\n  \"meshesState\": [";
        for (size_t m = 0; m < s.position.size(); ++m) {
            j += m ? ",\n    {\"velocities\": " : "\n    {\"velocities\": ";
            put_vec3_list(j, s.velocity[m]);
            j += ", \"position\": ";
            put_vec3_list(j, s.position[m]);
            j += "}";
        }
        j += "\n  ]\n}\n";
    }
    std::ofstream f(path);
    if (!f) throw std::runtime_error("cannot write state file: " + path);
    f << j;
}

PhysicsStateFile read_physics_state(const std::string& path) {
    json::Value root = json::parse(jsonio::read_file(path));
    PhysicsStateFile s;
    jsonio::get(root, "frameId", s.frameId);
    jsonio::get(root, "curTime", s.curTime);
    std::string format = "text";
    jsonio::get(root, "format", format);
    const json::Value* ms = root.find("meshesState");
    if (!ms) throw std::runtime_error("state file has no meshesState: " + path);
    if (format == "binary") {
        int n = 0;
        jsonio::get(root, "nMeshes", n);
        std::vector<int32_t> nv;
        jsonio::get_ints(*ms, "nVerts", nv);
        std::string vfile, pfile;
        jsonio::get(*ms, "velocities_file", vfile);
        jsonio::get(*ms, "position_file", pfile);
        if (int(nv.size()) < n) throw std::runtime_error("state file: nVerts shorter than nMeshes");
        const std::string dir = dir_of(path);
        std::ifstream vf(dir + "/" + vfile, std::ios::binary), pf(dir + "/" + pfile, std::ios::binary);
        if (!vf || !pf) throw std::runtime_error("cannot open the binary state files of " + path);
        for (int m = 0; m < n; ++m) {
            std::vector<float> v(3 * size_t(nv[m])), p(3 * size_t(nv[m]));
            vf.read(reinterpret_cast<char*>(v.data()), std::streamsize(v.size() * sizeof(float)));
            pf.read(reinterpret_cast<char*>(p.data()), std::streamsize(p.size() * sizeof(float)));
            if (!vf || !pf) throw std::runtime_error("binary state files are shorter than nVerts says: " + path);
            s.velocity.push_back(std::move(v));
            s.position.push_back(std::move(p));
        }
    } else if (format == "text") {
        if (!ms->is_array()) throw std::runtime_error("state file: meshesState is not a list");
        for (auto& m : ms->arr) {
            const json::Value* v = m.find("velocities");
            const json::Value* p = m.find("position");
            if (!v || !p) throw std::runtime_error("state file: mesh entry without velocities/position");
            s.velocity.push_back(get_vec3_list(*v, "velocities"));
            s.position.push_back(get_vec3_list(*p, "position"));
            if (s.velocity.back().size() != s.position.back().size())
                throw std::runtime_error("state file: velocities and positions differ in length");
        }
    } else {
        throw std::runtime_error("state file: unknown format " + format);
    }
    return s;
}

namespace {

std::string ext_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    const std::string name = k == std::string::npos ? path : path.substr(k + 1);
    const size_t d = name.find_last_of('.');
    return d == std::string::npos ? std::string() : name.substr(d);
}

void save_ply(const std::string& path, const std::vector<float>& X, const std::vector<int32_t>& F) {
    FILE* fp = std::fopen(path.c_str(), "w");
    if (!fp) throw std::runtime_error("cannot write " + path);
    const size_t nv = X.size() / 3, nf = F.size() / 3;
    std::fprintf(fp, "ply\nformat ascii 1.0\ncomment Mocap generated\nelement vertex %zu\n", nv);
    std::fprintf(fp, "property float x\nproperty float y\nproperty float z\n");
    if (nf) std::fprintf(fp, "element face %zu \nproperty list uchar int vertex_indices\n", nf);
    std::fprintf(fp, "end_header\n");
    for (size_t i = 0; i < nv; ++i) std::fprintf(fp, "%f %f %f\n", double(X[3 * i]), double(X[3 * i + 1]), double(X[3 * i + 2]));
    for (size_t i = 0; i < nf; ++i) std::fprintf(fp, "3 %d %d %d\n", F[3 * i], F[3 * i + 1], F[3 * i + 2]);
    std::fclose(fp);
}

}  // namespace

void write_frame_ply(const std::string& output, const std::vector<FrameMesh>& meshes, bool all_in_one,
                     bool add_model_name, bool tri_mesh_naming) {
    if (all_in_one) {
        std::vector<float> X;
        std::vector<int32_t> F;
        int32_t off = 0;
        for (const FrameMesh& m : meshes) {
            X.insert(X.end(), m.X.begin(), m.X.end());
            for (int32_t f : m.faces) F.push_back(f + off);
            off += int32_t(m.X.size() / 3);
        }
        save_ply(output, X, F);
        return;
    }
    const std::string dir = dir_of(output), stem = stem_of(output), ext = ext_of(output);
    for (size_t i = 0; i < meshes.size(); ++i) {
        char num[16];
        std::snprintf(num, sizeof(num), tri_mesh_naming ? "%04d" : "%06d", int(i));
        std::string name = dir + "/" + stem + (tri_mesh_naming ? "Model_" : "_Model_") + num;
        if (add_model_name) name += "_" + stem_of(meshes[i].model_path);
        name += tri_mesh_naming ? "_" + ext : ext;
        save_ply(name, meshes[i].X, meshes[i].faces);
    }
}

void write_frame_binary(const std::string& output, const std::vector<FrameMesh>& meshes) {
    std::ofstream f(output, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + output);
    for (const FrameMesh& m : meshes)
        f.write(reinterpret_cast<const char*>(m.X.data()), std::streamsize(m.X.size() * sizeof(float)));
}

}  // namespace gaia
