// Device-resident scene layout (HBM) for the GB300 path tracer.
//
//   nodes    : compressed 8-wide BVH, 80 B per node (5 x 16 B vector loads)
//   tris     : triangles in BVH leaf order, 48 B each: float4 p1 (w = global triangle id),
//              float4 p2, float4 p3 -- read with 16 B loads by the triangle test
//   nrm      : per BVH-order triangle, float4 n1 (w = primitive id), float4 n2, float4 n3
//   uv       : per BVH-order triangle, float2 x 3 (only read for area sensors)
//   mats_f/d : per primitive material/emitter record, float and double copies
//   lights   : per light (LightPrimitiveIndices order) record + FP64 area CDF
#pragma once

#include <cstdint>

#include "ngi_math.cuh"

namespace ngi {

// PrimitiveType bits (include/nanogi/rt.hpp:338-351)
enum : int { DT_D = 1, DT_G = 2, DT_S = 4, DT_L = 8, DT_E = 16 };
enum : int { BSDF_NONE = 0, BSDF_D = 1, BSDF_G = 2, BSDF_S = 3 };
enum : int { LT_AREA = 0, LT_POINT = 1, LT_DIRECTIONAL = 2 };
enum : int { ET_AREA = 0, ET_PINHOLE = 1 };
enum : int { ST_REFLECTION = 0, ST_REFRACTION = 1, ST_FRESNEL = 2 };

constexpr float kEpsF = 1e-4f;               // EpsF (include/nanogi/basic.hpp:85)
constexpr float kInfF = 3.402823466e+38f;    // InfF (basic.hpp:84)

// One compressed BVH8 node (Ylitie, Karras, Laine, HPG 2017 layout).
struct alignas(16) CwNode {
    float px, py, pz;         // quantisation origin
    uint8_t ex, ey, ez;       // biased float exponents of the per-axis scale 2^(e-127)
    uint8_t imask;            // bit s set: slot s holds an internal node
    uint32_t child_base;      // first child node (internal children are contiguous, slot order)
    uint32_t tri_base;        // first triangle of this node's leaves
    uint8_t meta[8];          // 0 = empty; internal: 0x38+slot; leaf: (unary count << 5) | tri offset
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(CwNode) == 80, "CwNode must be 80 bytes");

// Material + emitter record of a primitive (Primitive::Params, rt.hpp:389-477).
template <typename R>
struct DevMaterial {
    int type;      // PrimitiveType bits
    int bsdf;      // BSDF used at hits: first of D, G, S present (the reference tests D, then G, then S)
    int s_type;
    int l_type;
    V3<R> R_;      // D.R / G.R / S.*.R of the chosen BSDF
    V3<R> eta, k;  // G conductor
    R roughness;
    R eta1, eta2;  // S refraction / fresnel
    V3<R> Le;      // area light radiance (hit emission in pt)
    V3<R> We;      // area sensor importance (hit with the sensor in lt)
    int light_index;
    int e_type;    // ET_* of a sensor primitive
    int tex;       // TexR of the chosen D / G BSDF: index into SceneView::tex_info, -1 = the constant R_
    int pad;
};

// Light record (rt.hpp:389-416 + the area CDF of rt.hpp:1747-1765).
template <typename R>
struct DevLight {
    int type;          // LT_*
    int prim;
    int tri_count;
    int tri_base;      // first triangle of this light's mesh in the emitter arrays
    int cdf_offset;    // index of this light's first cdf entry in the shared cdf array
    int sensor_facing; // 0: every triangle faces away from the pinhole eye (no sensor connection)
    V3<R> Le;
    R inv_area;
    V3<R> position;    // point light
    V3<R> direction;   // directional light
    V3<R> center;
    R radius;
};

// Sensor record (rt.hpp:418-437).
template <typename R>
struct DevSensor {
    int type;          // ET_*
    int prim;
    int tri_count;
    int tri_base;
    int cdf_offset;
    int pad;
    V3<R> eye, Vx, Vy, Vz;
    R tan_fov, aspect;
    V3<R> We;
    R inv_area;
};

template <typename R>
struct SceneView {
    const CwNode* nodes;
    const float4* tris;        // 3 per triangle, BVH order
    const float4* nrm;         // 3 per triangle, BVH order
    const float2* uv;          // 3 per triangle, BVH order
    const DevMaterial<R>* mats;
    const DevLight<R>* lights;
    int num_lights;
    int num_nodes;
    const double* cdf;         // FP64 emitter-area cdfs
    const float* emit_tri_pos; // 9 floats per emitter triangle (original order), light/sensor meshes
    const float* emit_tri_uv;  // 6 floats per emitter triangle
    const float4* texels;      // TexR images, rgb + pad per texel, rows top first
    const int4* tex_info;      // per texture: first texel, width, height
    int num_textures;
    DevSensor<R> sensor;
};

}  // namespace ngi
