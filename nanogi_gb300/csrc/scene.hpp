// Host-side scene: the reference's Scene/Primitive/Mesh (include/nanogi/rt.hpp:148-155,
// 379-477, 1488-1500) flattened into plain arrays ready for upload to the GPU.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "texture.hpp"

namespace ngi {

// PrimitiveType bits (rt.hpp:338-351).
enum : int { PT_D = 1, PT_G = 2, PT_S = 4, PT_L = 8, PT_E = 16, PT_BSDF = 7, PT_EMITTER = 24 };
enum : int { L_AREA = 0, L_POINT = 1, L_DIRECTIONAL = 2 };   // LType rt.hpp:353-358
enum : int { E_AREA = 0, E_PINHOLE = 1 };                    // EType rt.hpp:360-364
enum : int { S_REFLECTION = 0, S_REFRACTION = 1, S_FRESNEL = 2 };  // SType rt.hpp:366-371

// Primitive::Params (rt.hpp:389-477), host copy in double precision.
struct HostPrimitive {
    int type = 0;
    bool has_mesh = false;
    bool has_uv = false;
    int64_t tri_first = 0;  // range in the global triangle arrays
    int64_t tri_count = 0;

    // L
    int l_type = L_AREA;
    double Le[3] = {0, 0, 0};
    double l_position[3] = {0, 0, 0};
    double l_direction[3] = {0, 0, 0};
    double l_center[3] = {0, 0, 0};
    double l_radius = 0;
    double inv_area = 0;            // area light / area sensor / directional (2*pi*r^2)^-1
    std::vector<double> area_cdf;   // Distribution1D cdf, tri_count+1 entries (basic.hpp:440-497)

    // E
    int e_type = E_PINHOLE;
    double We[3] = {0, 0, 0};
    double eye[3] = {0, 0, 0};
    double Vx[3] = {0, 0, 0}, Vy[3] = {0, 0, 0}, Vz[3] = {0, 0, 0};
    double fov = 0;                 // radians
    double aspect = 1;

    // D
    double D_R[3] = {0, 0, 0};
    int D_tex = -1;                 // TexR: index into HostScene::textures, -1 = the constant R
    // G
    double G_R[3] = {0, 0, 0}, G_eta[3] = {0, 0, 0}, G_k[3] = {0, 0, 0};
    int G_tex = -1;
    double G_roughness = 0;
    // S
    int s_type = S_REFLECTION;
    double S_R[3] = {0, 0, 0};
    double S_eta1 = 1, S_eta2 = 1;
};

struct DeviceScene;  // device buffers, defined in the CUDA translation units

struct HostScene {
    std::string path;
    std::vector<HostPrimitive> prims;
    std::vector<int> light_prims;   // LightPrimitiveIndices (rt.hpp:1499)
    int sensor_prim = -1;           // SensorPrimitiveIndex (rt.hpp:1498): the last E primitive

    // Flattened triangles; global triangle index = primitives in YAML order, faces in
    // mesh order. Values are float32 (what Assimp stores and Embree consumes).
    std::vector<float> tri_pos;     // 9 per triangle (p1, p2, p3)
    std::vector<float> tri_nrm;     // 9 per triangle (n1, n2, n3)
    std::vector<float> tri_uv;      // 6 per triangle (zeros when the mesh has none)
    std::vector<int32_t> tri_prim;  // owning primitive
    std::vector<TextureImage> textures;  // TexR images (Scene::Textures, rt.hpp:1495)
    int64_t num_vertices = 0;
    double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};

    DeviceScene* dev = nullptr;

    int64_t NumTriangles() const { return (int64_t)tri_prim.size(); }
};

// A caller-held indexed triangle mesh that replaces the file a primitive's `mesh: path:`
// names (Mesh::Positions / Normals / Texcoords / Faces, rt.hpp:148-155).
struct MemoryMesh {
    std::string path;
    const float* positions = nullptr;   // 3 per vertex
    const float* normals = nullptr;     // 3 per vertex, or null: flat face normals
    const float* texcoords = nullptr;   // 2 per vertex, or null
    const uint32_t* faces = nullptr;    // 3 per triangle
    int64_t num_vertices = 0;
    int64_t num_triangles = 0;
};

// Scene::Load (rt.hpp:1519-2154). Throws ngi::SceneError / YamlError / ObjError. A mesh
// path equal to the path of one of `memory` (verbatim) takes that mesh instead of a file.
std::unique_ptr<HostScene> LoadScene(const std::string& yaml_path, double aspect,
                                     const std::vector<MemoryMesh>* memory = nullptr);

struct SceneError : std::runtime_error {
    int code;
    SceneError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

}  // namespace ngi
