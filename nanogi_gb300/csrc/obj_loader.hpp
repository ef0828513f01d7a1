// Wavefront OBJ reader for nanogi meshes.
//
// The reference imports meshes with Assimp (include/nanogi/rt.hpp:1640-1730): it keeps
// only the FIRST mesh of the file (scene->mMeshes[0], rt.hpp:1679), triangulates
// polygons, joins identical vertices and reads positions, normals and the first UV set.
// Assimp's OBJ importer emits one mesh per object ("o"/"g") and material ("usemtl")
// group, so "first mesh" is the first such group that holds faces. This reader
// reproduces that behaviour: fan triangulation from the polygon's first corner, one
// vertex per distinct (position, uv, normal) index triple, and optional flat or smooth
// normal generation (aiProcess_GenNormals / aiProcess_GenSmoothNormals, rt.hpp:1655-1663).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace ngi {

struct ObjError : std::runtime_error {
    explicit ObjError(const std::string& m) : std::runtime_error(m) {}
};

struct ObjMesh {
    // Per unique vertex; values are the float32 numbers the file holds (Assimp stores
    // aiVector3D as float), widened to double like Mesh::Positions (rt.hpp:148-155).
    std::vector<double> positions;  // 3 per vertex
    std::vector<double> normals;    // 3 per vertex (always filled)
    std::vector<double> texcoords;  // 2 per vertex, empty when the file has none
    std::vector<uint32_t> faces;    // 3 per triangle
    bool file_had_normals = false;
};

enum class ObjNormalMode { FromFile, Flat, Smooth };

// Loads the first mesh of an OBJ file. When the mesh has no normals, normals are
// generated (flat unless smooth is requested).
ObjMesh LoadObj(const std::string& path, bool gen_smooth_normals);

// Same, from an in-memory OBJ text (used by tests).
ObjMesh ParseObj(const std::string& text, bool gen_smooth_normals, const std::string& name = "<memory>");

}  // namespace ngi
