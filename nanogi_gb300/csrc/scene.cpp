// Scene loading: YAML scene schema (schema.yml:33-334) -> HostScene.
// Follows Scene::Load in include/nanogi/rt.hpp:1519-2154 step by step.
#include "scene.hpp"

#include <cmath>
#include <fstream>

#include "image_io.hpp"
#include "obj_loader.hpp"
#include "texture.hpp"
#include "yaml_lite.hpp"

namespace ngi {

namespace {

constexpr int kVersionMin = 3;  // AppConfigVersionMin rt.hpp:1484
constexpr int kVersionMax = 5;  // AppConfigVersionMax rt.hpp:1485
constexpr double kPi = 3.14159265358979323846;

// NGI status codes (include/nanogi.h) used when throwing SceneError.
constexpr int kErrArg = 1, kErrIO = 2, kErrParse = 3, kErrUnsupported = 7;

void ParseVec3(const YamlNode& n, double out[3], const std::string& what) {
    // ParseVec3 rt.hpp:61-64
    if (!n.IsSequence() || n.size() != 3) throw SceneError(kErrParse, what + " must be a 3-element sequence");
    for (int k = 0; k < 3; k++) out[k] = n[k].AsDouble();
}

std::string ParentDir(const std::string& p) {
    size_t s = p.find_last_of('/');
    if (s == std::string::npos) return "";
    return p.substr(0, s + 1);
}

// glm::normalize: v * inversesqrt(dot(v, v))
void Normalize(double v[3]) {
    const double inv = 1.0 / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; k++) v[k] *= inv;
}

void Cross(const double a[3], const double b[3], double out[3]) {
    out[0] = a[1] * b[2] - a[2] * b[1];
    out[1] = a[2] * b[0] - a[0] * b[2];
    out[2] = a[0] * b[1] - a[1] * b[0];
}

// CreateTriangleAreaDist (rt.hpp:1747-1765): FP64 cdf over triangle areas.
void CreateTriangleAreaDist(const HostScene& s, HostPrimitive& prim) {
    prim.area_cdf.assign(1, 0.0);
    double sum = 0;
    for (int64_t i = 0; i < prim.tri_count; i++) {
        const float* P = &s.tri_pos[9 * (prim.tri_first + i)];
        double e1[3], e2[3], c[3];
        for (int k = 0; k < 3; k++) {
            e1[k] = (double)P[3 + k] - (double)P[k];
            e2[k] = (double)P[6 + k] - (double)P[k];
        }
        Cross(e1, e2, c);
        const double area = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * 0.5;
        prim.area_cdf.push_back(prim.area_cdf.back() + area);
        sum += area;
    }
    const double inv = 1.0 / prim.area_cdf.back();
    for (auto& v : prim.area_cdf) v *= inv;
    prim.inv_area = 1.0 / sum;
}

}  // namespace

namespace {

// Appends a caller-held mesh to the flattened triangle arrays; returns its vertex count.
int64_t AppendMemoryMesh(HostScene& scene, HostPrimitive& prim, const MemoryMesh& m, double* bmin, double* bmax) {
    prim.has_mesh = true;
    prim.has_uv = m.texcoords != nullptr;
    prim.tri_first = scene.NumTriangles();
    prim.tri_count = m.num_triangles;
    const size_t nt = (size_t)m.num_triangles;
    const size_t base = scene.tri_pos.size() / 9;
    scene.tri_pos.resize(9 * (base + nt));
    scene.tri_nrm.resize(9 * (base + nt));
    scene.tri_uv.resize(6 * (base + nt), 0.0f);
    scene.tri_prim.resize(base + nt, (int32_t)scene.prims.size());
    for (int64_t v = 0; v < m.num_vertices; v++)
        for (int k = 0; k < 3; k++) {
            bmin[k] = std::fmin(bmin[k], (double)m.positions[3 * v + k]);
            bmax[k] = std::fmax(bmax[k], (double)m.positions[3 * v + k]);
        }
    float* P = scene.tri_pos.data() + 9 * base;
    float* N = scene.tri_nrm.data() + 9 * base;
    float* T = scene.tri_uv.data() + 6 * base;
    for (size_t f = 0; f < nt; f++) {
        const uint32_t* ix = m.faces + 3 * f;
        for (int c = 0; c < 3; c++) {
            for (int k = 0; k < 3; k++) P[9 * f + 3 * c + k] = m.positions[3 * (size_t)ix[c] + k];
            if (m.normals)
                for (int k = 0; k < 3; k++) N[9 * f + 3 * c + k] = m.normals[3 * (size_t)ix[c] + k];
            if (m.texcoords)
                for (int k = 0; k < 2; k++) T[6 * f + 2 * c + k] = m.texcoords[2 * (size_t)ix[c] + k];
        }
        if (!m.normals) {
            // flat normals (aiProcess_GenNormals, rt.hpp:1655-1663)
            const float* q = P + 9 * f;
            const double e1[3] = {(double)q[3] - q[0], (double)q[4] - q[1], (double)q[5] - q[2]};
            const double e2[3] = {(double)q[6] - q[0], (double)q[7] - q[1], (double)q[8] - q[2]};
            double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int k = 0; k < 3; k++) n[k] = l > 0 ? n[k] / l : 0.0;
            for (int c = 0; c < 3; c++)
                for (int k = 0; k < 3; k++) N[9 * f + 3 * c + k] = (float)n[k];
        }
    }
    return m.num_vertices;
}

}  // namespace

std::unique_ptr<HostScene> LoadScene(const std::string& path, double aspect, const std::vector<MemoryMesh>* memory) {
    if (!(aspect > 0) || !std::isfinite(aspect)) throw SceneError(kErrArg, "aspect must be positive and finite");
    {
        std::ifstream probe(path);
        if (!probe) throw SceneError(kErrIO, "cannot open scene file " + path);
    }
    std::shared_ptr<YamlNode> root;
    try {
        root = YamlLoadFile(path);
    } catch (const YamlError& e) {
        throw SceneError(kErrParse, std::string("YAML exception: ") + e.what());
    }

    auto scene = std::make_unique<HostScene>();
    scene->path = path;
    const std::string base = ParentDir(path);
    // LoadTexture (rt.hpp:1775-1802): one image per distinct path, relative to the scene file.
    // A texture that does not load fails the scene (the reference logs it and renders black).
    std::vector<std::string> texture_paths;
    auto load_texture = [&](const std::string& local) -> int {
        const std::string tp = base + local;
        for (size_t i = 0; i < texture_paths.size(); i++)
            if (texture_paths[i] == tp) return (int)i;
        try {
            scene->textures.push_back(LoadTexture(tp));
        } catch (const ImageError& e) {
            throw SceneError(e.code, e.what());
        }
        texture_paths.push_back(tp);
        return (int)texture_paths.size() - 1;
    };

    try {
        const YamlNode& doc = *root;
        if (!doc.Has("version")) throw SceneError(kErrParse, "missing 'version'");
        const int version = doc["version"].AsInt();
        if (version < kVersionMin || kVersionMax < version)
            throw SceneError(kErrParse, "Invalid config version [Min 3, Max 5, Actual " + std::to_string(version) + "]");

        const YamlNode& prims = doc["scene"]["primitives"];
        if (!prims.IsSequence()) throw SceneError(kErrParse, "missing 'scene.primitives' sequence");

        double bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};

        for (size_t i = 0; i < prims.size(); i++) {
            const YamlNode& pn = prims[i];
            HostPrimitive prim;
            const std::string where = "primitive " + std::to_string(i);

            // Primitive type (rt.hpp:1587-1616)
            const YamlNode& tn = pn["type"];
            if (!tn.IsSequence()) throw SceneError(kErrParse, where + ": 'type' must be a sequence");
            for (size_t j = 0; j < tn.size(); j++) {
                const std::string t = tn[j].AsString();
                if (t == "D") prim.type |= PT_D;
                else if (t == "G") prim.type |= PT_G;
                else if (t == "S") prim.type |= PT_S;
                else if (t == "L") prim.type |= PT_L;
                else if (t == "E") prim.type |= PT_E;
            }
            if (prim.type == 0 || ((prim.type & PT_L) && (prim.type & PT_E)))
                throw SceneError(kErrParse, where + ": Invalid primitive type");
            if (prim.type & PT_E) scene->sensor_prim = (int)scene->prims.size();
            if (prim.type & PT_L) scene->light_prims.push_back((int)scene->prims.size());

            // Mesh (rt.hpp:1624-1738)
            if (pn.Has("mesh")) {
                const YamlNode& mn = pn["mesh"];
                const std::string local = mn["path"].AsString();
                bool smooth = false;
                if (mn.Has("postprocess")) {
                    const YamlNode& pp = mn["postprocess"];
                    smooth = pp.Has("generate_smooth_normals") && pp["generate_smooth_normals"].AsBool();
                }
                const MemoryMesh* held = nullptr;
                if (memory)
                    for (const MemoryMesh& m : *memory)
                        if (m.path == local) held = &m;
                if (held) {
                    scene->num_vertices += AppendMemoryMesh(*scene, prim, *held, bmin, bmax);
                } else {
                    ObjMesh mesh;
                    try {
                        mesh = LoadObj(base + local, smooth);
                    } catch (const std::ios_base::failure& e) {
                        throw SceneError(kErrIO, e.what());
                    } catch (const ObjError& e) {
                        throw SceneError(kErrParse, e.what());
                    }
                    prim.has_mesh = true;
                    prim.has_uv = !mesh.texcoords.empty();
                    prim.tri_first = scene->NumTriangles();
                    prim.tri_count = (int64_t)(mesh.faces.size() / 3);
                    const size_t nv = mesh.positions.size() / 3;
                    for (size_t v = 0; v < nv; v++)
                        for (int k = 0; k < 3; k++) {
                            bmin[k] = std::fmin(bmin[k], mesh.positions[3 * v + k]);
                            bmax[k] = std::fmax(bmax[k], mesh.positions[3 * v + k]);
                        }
                    scene->num_vertices += (int64_t)nv;
                    for (int64_t f = 0; f < prim.tri_count; f++) {
                        for (int c = 0; c < 3; c++) {
                            const uint32_t vi = mesh.faces[3 * f + c];
                            for (int k = 0; k < 3; k++) {
                                scene->tri_pos.push_back((float)mesh.positions[3 * vi + k]);
                                scene->tri_nrm.push_back((float)mesh.normals[3 * vi + k]);
                            }
                            for (int k = 0; k < 2; k++)
                                scene->tri_uv.push_back(prim.has_uv ? (float)mesh.texcoords[2 * vi + k] : 0.0f);
                        }
                        scene->tri_prim.push_back((int32_t)scene->prims.size());
                    }
                }
            }

            // Parameters (rt.hpp:1767-2043)
            const YamlNode& params = pn["params"];
            if (prim.type & PT_L) {
                const YamlNode& L = params["L"];
                const std::string lt = L["type"].AsString();
                if (lt == "area") {
                    prim.l_type = L_AREA;
                    ParseVec3(L["area"]["Le"], prim.Le, where + " L.area.Le");
                    if (!prim.has_mesh) throw SceneError(kErrParse, where + ": Area light must be associated with mesh");
                    CreateTriangleAreaDist(*scene, prim);
                } else if (lt == "point") {
                    prim.l_type = L_POINT;
                    ParseVec3(L["point"]["Le"], prim.Le, where + " L.point.Le");
                    ParseVec3(L["point"]["position"], prim.l_position, where + " L.point.position");
                } else if (lt == "directional") {
                    prim.l_type = L_DIRECTIONAL;
                    ParseVec3(L["directional"]["Le"], prim.Le, where + " L.directional.Le");
                    ParseVec3(L["directional"]["direction"], prim.l_direction, where + " L.directional.direction");
                } else {
                    throw SceneError(kErrParse, where + ": unknown light type '" + lt + "'");
                }
            }
            if (prim.type & PT_E) {
                const YamlNode& E = params["E"];
                const std::string et = E["type"].AsString();
                if (et == "pinhole") {
                    const YamlNode& ph = E["pinhole"];
                    double eye[3], center[3], up[3];
                    ParseVec3(ph["view"]["eye"], eye, where + " eye");
                    ParseVec3(ph["view"]["center"], center, where + " center");
                    ParseVec3(ph["view"]["up"], up, where + " up");
                    prim.e_type = E_PINHOLE;
                    ParseVec3(ph["We"], prim.We, where + " We");
                    for (int k = 0; k < 3; k++) prim.eye[k] = eye[k];
                    prim.fov = ph["perspective"]["fov"].AsDouble() * kPi / 180.0;  // glm::radians
                    for (int k = 0; k < 3; k++) prim.Vz[k] = eye[k] - center[k];
                    Normalize(prim.Vz);
                    Cross(up, prim.Vz, prim.Vx);
                    Normalize(prim.Vx);
                    Cross(prim.Vz, prim.Vx, prim.Vy);
                    prim.aspect = aspect;
                } else if (et == "area") {
                    prim.e_type = E_AREA;
                    ParseVec3(E["area"]["We"], prim.We, where + " We");
                    if (!prim.has_mesh || !prim.has_uv)
                        throw SceneError(kErrParse, where + ": Raw sensor must be associated with mesh with UV coordinates");
                    CreateTriangleAreaDist(*scene, prim);
                } else {
                    throw SceneError(kErrParse, where + ": unknown sensor type '" + et + "'");
                }
            }
            if (prim.type & PT_D) {
                const YamlNode& D = params["D"];
                if (D.Has("R")) {
                    ParseVec3(D["R"], prim.D_R, where + " D.R");
                } else if (D.Has("TexR")) {
                    prim.D_tex = load_texture(D["TexR"].AsString());
                } else {
                    throw SceneError(kErrParse, where + ": D needs R");
                }
            }
            if (prim.type & PT_G) {
                const YamlNode& G = params["G"];
                ParseVec3(G["Eta"], prim.G_eta, where + " G.Eta");
                ParseVec3(G["K"], prim.G_k, where + " G.K");
                prim.G_roughness = G["Roughness"].AsDouble();
                if (G.Has("R")) {
                    ParseVec3(G["R"], prim.G_R, where + " G.R");
                } else if (G.Has("TexR")) {
                    prim.G_tex = load_texture(G["TexR"].AsString());
                } else {
                    throw SceneError(kErrParse, where + ": G needs R");
                }
            }
            if (prim.type & PT_S) {
                const YamlNode& S = params["S"];
                const std::string st = S["type"].AsString();
                if (st == "reflection") {
                    prim.s_type = S_REFLECTION;
                    ParseVec3(S["reflection"]["R"], prim.S_R, where + " S.reflection.R");
                } else if (st == "refraction") {
                    prim.s_type = S_REFRACTION;
                    ParseVec3(S["refraction"]["R"], prim.S_R, where + " S.refraction.R");
                    prim.S_eta1 = S["refraction"]["eta1"].AsDouble();
                    prim.S_eta2 = S["refraction"]["eta2"].AsDouble();
                } else if (st == "fresnel") {
                    prim.s_type = S_FRESNEL;
                    ParseVec3(S["fresnel"]["R"], prim.S_R, where + " S.fresnel.R");
                    prim.S_eta1 = S["fresnel"]["eta1"].AsDouble();
                    prim.S_eta2 = S["fresnel"]["eta2"].AsDouble();
                } else {
                    throw SceneError(kErrParse, where + ": unknown specular type '" + st + "'");
                }
            }
            scene->prims.push_back(std::move(prim));
        }

        // Post-configuration of directional lights from the scene bound (rt.hpp:2059-2079)
        for (auto& prim : scene->prims) {
            if ((prim.type & PT_L) && prim.l_type == L_DIRECTIONAL) {
                double d[3];
                for (int k = 0; k < 3; k++) {
                    prim.l_center[k] = (bmax[k] + bmin[k]) * 0.5;
                    d[k] = prim.l_center[k] - bmax[k];
                }
                prim.l_radius = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * 1.01;
                prim.inv_area = 1.0 / (2.0 * kPi * prim.l_radius * prim.l_radius);
            }
        }
        for (int k = 0; k < 3; k++) {
            scene->bmin[k] = scene->NumTriangles() ? bmin[k] : 0.0;
            scene->bmax[k] = scene->NumTriangles() ? bmax[k] : 0.0;
        }
    } catch (const YamlError& e) {
        throw SceneError(kErrParse, std::string("YAML exception: ") + e.what());
    }
    if (scene->NumTriangles() > (int64_t)0x7fffffff)
        throw SceneError(kErrUnsupported, "more than 2^31-1 triangles");
    return scene;
}

}  // namespace ngi
