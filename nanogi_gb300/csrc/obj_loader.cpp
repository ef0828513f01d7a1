// Wavefront OBJ reader (see obj_loader.hpp).
#include "obj_loader.hpp"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <unordered_map>

namespace ngi {

namespace {

struct Corner {
    int64_t v, vt, vn;  // 0-based, -1 = absent
};

struct TripleHash {
    size_t operator()(const Corner& c) const {
        uint64_t h = (uint64_t)c.v * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)(c.vt + 1) * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
        h ^= (uint64_t)(c.vn + 1) * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};
struct TripleEq {
    bool operator()(const Corner& a, const Corner& b) const { return a.v == b.v && a.vt == b.vt && a.vn == b.vn; }
};

// Parses one float the way the file states it, rounded to float32 (Assimp's storage type).
bool ParseFloat(const char*& p, float& out) {
    while (*p == ' ' || *p == '\t') p++;
    if (*p == '\0' || *p == '\n') return false;
    char* end = nullptr;
    double d = std::strtod(p, &end);
    if (end == p) return false;
    p = end;
    out = (float)d;
    return true;
}

int64_t ResolveIndex(long long idx, size_t count, const std::string& name, int lineno) {
    long long r;
    if (idx > 0)
        r = idx - 1;
    else if (idx < 0)
        r = (long long)count + idx;
    else
        throw ObjError(name + ":" + std::to_string(lineno) + ": index 0 is invalid in OBJ");
    if (r < 0 || r >= (long long)count)
        throw ObjError(name + ":" + std::to_string(lineno) + ": index out of range");
    return r;
}

}  // namespace

ObjMesh ParseObj(const std::string& text, bool gen_smooth_normals, const std::string& name) {
    std::vector<float> v, vn, vt;
    v.reserve(1 << 16);
    std::vector<std::vector<Corner>> polys;  // faces of the first mesh group
    bool group_has_faces = false;
    bool group_closed = false;
    std::string current_mtl;
    bool have_mtl = false;

    std::istringstream in(text);
    std::string line;
    int lineno = 0;
    while (std::getline(in, line)) {
        lineno++;
        const char* p = line.c_str();
        while (*p == ' ' || *p == '\t') p++;
        if (*p == '#' || *p == '\0' || *p == '\r') continue;
        if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
            p += 2;
            float x, y, z;
            if (!ParseFloat(p, x) || !ParseFloat(p, y) || !ParseFloat(p, z))
                throw ObjError(name + ":" + std::to_string(lineno) + ": malformed vertex");
            v.push_back(x); v.push_back(y); v.push_back(z);
        } else if (p[0] == 'v' && p[1] == 'n' && (p[2] == ' ' || p[2] == '\t')) {
            p += 3;
            float x, y, z;
            if (!ParseFloat(p, x) || !ParseFloat(p, y) || !ParseFloat(p, z))
                throw ObjError(name + ":" + std::to_string(lineno) + ": malformed normal");
            vn.push_back(x); vn.push_back(y); vn.push_back(z);
        } else if (p[0] == 'v' && p[1] == 't' && (p[2] == ' ' || p[2] == '\t')) {
            p += 3;
            float x, y = 0.0f;
            if (!ParseFloat(p, x))
                throw ObjError(name + ":" + std::to_string(lineno) + ": malformed texcoord");
            ParseFloat(p, y);
            vt.push_back(x); vt.push_back(y);
        } else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
            p += 2;
            if (group_closed) continue;  // faces of later meshes are not imported
            std::vector<Corner> poly;
            while (true) {
                while (*p == ' ' || *p == '\t' || *p == '\r') p++;
                if (*p == '\0') break;
                Corner c{-1, -1, -1};
                char* end = nullptr;
                long long a = std::strtoll(p, &end, 10);
                if (end == p) throw ObjError(name + ":" + std::to_string(lineno) + ": malformed face");
                p = end;
                c.v = ResolveIndex(a, v.size() / 3, name, lineno);
                if (*p == '/') {
                    p++;
                    if (*p != '/') {
                        long long b = std::strtoll(p, &end, 10);
                        if (end == p) throw ObjError(name + ":" + std::to_string(lineno) + ": malformed face");
                        p = end;
                        c.vt = ResolveIndex(b, vt.size() / 2, name, lineno);
                    }
                    if (*p == '/') {
                        p++;
                        long long d = std::strtoll(p, &end, 10);
                        if (end == p) throw ObjError(name + ":" + std::to_string(lineno) + ": malformed face");
                        p = end;
                        c.vn = ResolveIndex(d, vn.size() / 3, name, lineno);
                    }
                }
                poly.push_back(c);
            }
            if (poly.size() < 3) continue;  // points and lines are not triangles
            polys.push_back(std::move(poly));
            group_has_faces = true;
        } else if ((p[0] == 'o' || p[0] == 'g') && (p[1] == ' ' || p[1] == '\t' || p[1] == '\0' || p[1] == '\r')) {
            if (group_has_faces) group_closed = true;
        } else if (std::strncmp(p, "usemtl", 6) == 0) {
            std::string m(p + 6);
            size_t b = m.find_first_not_of(" \t");
            m = b == std::string::npos ? std::string() : m.substr(b);
            while (!m.empty() && (m.back() == '\r' || m.back() == ' ')) m.pop_back();
            if (have_mtl && m != current_mtl && group_has_faces) group_closed = true;
            current_mtl = m;
            have_mtl = true;
        }
        // mtllib, s, l, p and unknown statements carry nothing the renderer reads.
    }
    if (polys.empty()) throw ObjError("No mesh is found in " + name);

    ObjMesh mesh;
    std::unordered_map<Corner, uint32_t, TripleHash, TripleEq> index;
    bool all_have_vn = true, any_vt = false;
    for (auto& poly : polys)
        for (auto& c : poly) {
            if (c.vn < 0) all_have_vn = false;
            if (c.vt >= 0) any_vt = true;
        }
    mesh.file_had_normals = all_have_vn;
    auto corner_index = [&](const Corner& c) -> uint32_t {
        auto it = index.find(c);
        if (it != index.end()) return it->second;
        uint32_t id = (uint32_t)(mesh.positions.size() / 3);
        for (int k = 0; k < 3; k++) mesh.positions.push_back((double)v[3 * c.v + k]);
        for (int k = 0; k < 3; k++) mesh.normals.push_back(all_have_vn ? (double)vn[3 * c.vn + k] : 0.0);
        if (any_vt) {
            mesh.texcoords.push_back(c.vt >= 0 ? (double)vt[2 * c.vt] : 0.0);
            mesh.texcoords.push_back(c.vt >= 0 ? (double)vt[2 * c.vt + 1] : 0.0);
        }
        index.emplace(c, id);
        return id;
    };
    for (auto& poly : polys) {
        // fan triangulation from the first corner
        for (size_t k = 1; k + 1 < poly.size(); k++) {
            mesh.faces.push_back(corner_index(poly[0]));
            mesh.faces.push_back(corner_index(poly[k]));
            mesh.faces.push_back(corner_index(poly[k + 1]));
        }
    }

    if (!all_have_vn) {
        const size_t nv = mesh.positions.size() / 3;
        const size_t nf = mesh.faces.size() / 3;
        auto P = [&](uint32_t i, int k) { return mesh.positions[3 * i + k]; };
        if (!gen_smooth_normals) {
            // Flat normals: every corner gets its own vertex carrying the face normal.
            ObjMesh flat;
            flat.file_had_normals = false;
            for (size_t f = 0; f < nf; f++) {
                uint32_t i0 = mesh.faces[3 * f], i1 = mesh.faces[3 * f + 1], i2 = mesh.faces[3 * f + 2];
                double e1[3], e2[3], n[3];
                for (int k = 0; k < 3; k++) { e1[k] = P(i1, k) - P(i0, k); e2[k] = P(i2, k) - P(i0, k); }
                n[0] = e1[1] * e2[2] - e1[2] * e2[1];
                n[1] = e1[2] * e2[0] - e1[0] * e2[2];
                n[2] = e1[0] * e2[1] - e1[1] * e2[0];
                double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                for (int k = 0; k < 3; k++) n[k] = l > 0 ? (double)(float)(n[k] / l) : 0.0;
                for (uint32_t c : {i0, i1, i2}) {
                    flat.faces.push_back((uint32_t)(flat.positions.size() / 3));
                    for (int k = 0; k < 3; k++) flat.positions.push_back(P(c, k));
                    for (int k = 0; k < 3; k++) flat.normals.push_back(n[k]);
                    if (!mesh.texcoords.empty()) {
                        flat.texcoords.push_back(mesh.texcoords[2 * c]);
                        flat.texcoords.push_back(mesh.texcoords[2 * c + 1]);
                    }
                }
            }
            return flat;
        }
        // Smooth normals: area-weighted sum of face normals over vertices sharing a position.
        std::vector<double> acc(3 * nv, 0.0);
        for (size_t f = 0; f < nf; f++) {
            uint32_t i0 = mesh.faces[3 * f], i1 = mesh.faces[3 * f + 1], i2 = mesh.faces[3 * f + 2];
            double e1[3], e2[3], n[3];
            for (int k = 0; k < 3; k++) { e1[k] = P(i1, k) - P(i0, k); e2[k] = P(i2, k) - P(i0, k); }
            n[0] = e1[1] * e2[2] - e1[2] * e2[1];
            n[1] = e1[2] * e2[0] - e1[0] * e2[2];
            n[2] = e1[0] * e2[1] - e1[1] * e2[0];
            for (uint32_t c : {i0, i1, i2})
                for (int k = 0; k < 3; k++) acc[3 * c + k] += n[k];
        }
        for (size_t i = 0; i < nv; i++) {
            double l = std::sqrt(acc[3 * i] * acc[3 * i] + acc[3 * i + 1] * acc[3 * i + 1] + acc[3 * i + 2] * acc[3 * i + 2]);
            for (int k = 0; k < 3; k++) mesh.normals[3 * i + k] = l > 0 ? (double)(float)(acc[3 * i + k] / l) : 0.0;
        }
    }
    return mesh;
}

ObjMesh LoadObj(const std::string& path, bool gen_smooth_normals) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::ios_base::failure("Unable to open file \"" + path + "\".");
    std::stringstream ss;
    ss << f.rdbuf();
    return ParseObj(ss.str(), gen_smooth_normals, path);
}

}  // namespace ngi
