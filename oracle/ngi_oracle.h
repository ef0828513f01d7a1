/*
 * CPU oracle for nanogi's `pt` / `ptdirect` path (TEST INFRASTRUCTURE ONLY).
 *
 * An FP64 restatement of the reference's algorithm, written independently of the GPU
 * product code. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it, and only as the checker / the timed CPU baseline -- never as a product path.
 *
 * PARITY UNPINNED: the reference (lighttransport/nanogi) has no tests, golden images or
 * known-answer vectors, and it cannot be built here (Embree 2, yaml-cpp, Assimp, Boost,
 * TBB, glm and FreeImage are absent), so this restatement is checked against analytic
 * known answers (furnace, energy and reciprocity of each BSDF, published RNG vectors)
 * rather than against outputs of the reference itself.
 */
#ifndef NGI_ORACLE_H
#define NGI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One primitive (Primitive::Params, include/nanogi/rt.hpp:379-477). */
typedef struct ora_prim_desc {
    int32_t type;        /* PrimitiveType bits: D=1 G=2 S=4 L=8 E=16 */
    int32_t has_mesh;
    int64_t tri_first;   /* range in the flattened triangle arrays */
    int64_t tri_count;
    int32_t l_type;      /* 0 area, 1 point, 2 directional */
    int32_t e_type;      /* 0 area, 1 pinhole */
    double Le[3];
    double l_position[3];
    double l_direction[3];
    double We[3];
    double eye[3], center[3], up[3];
    double fov_deg;
    double D_R[3];
    double G_R[3], G_eta[3], G_k[3];
    double G_roughness;
    int32_t s_type;      /* 0 reflection, 1 refraction, 2 fresnel */
    int32_t has_uv;
    double S_R[3];
    double S_eta1, S_eta2;
    /* TexR images (rt.hpp:157-270): rgb floats, row 0 = the image's top row; NULL = constant R.
     * Copied by ora_scene_create. */
    const float* D_tex;
    int32_t D_tex_w, D_tex_h;
    const float* G_tex;
    int32_t G_tex_w, G_tex_h;
} ora_prim_desc;

typedef struct ora_render_params {
    int32_t renderer;       /* 0 pt, 1 ptdirect */
    int32_t max_vertices;   /* -1 = unbounded */
    int64_t num_samples;
    int32_t width, height;
    uint64_t seed;
    int64_t sample_offset;
    int32_t rng_mode;       /* 0: reference stream (mt19937 per thread), 1: Philox replay keys */
    int32_t raster_mode;    /* replay mode only: 0 stratified, 1 uniform over the image */
    int32_t num_threads;    /* 0 = all hardware threads */
    int32_t use_bvh;        /* 1: own BVH (fast), 0: brute force (truth) */
    int64_t grain_size;     /* samples per work item (TBB grain size, src/nanogi.cpp:2014) */
    int32_t ray_offset;     /* 0: absolute tmin = EpsF (rt.hpp:2248); 1: scale-aware origin offset, tmin 0 */
    int32_t pad_;
} ora_render_params;

typedef struct ora_render_stats {
    int64_t camera_rays, extension_rays, shadow_rays;
    double seconds;
    int32_t threads;
    int64_t extension_misses;  /* extension rays (camera rays included) that hit nothing */
} ora_render_stats;

typedef struct ora_scene ora_scene;

ora_scene* ora_scene_create(const ora_prim_desc* prims, int32_t n_prims, const float* tri_pos,
                            const float* tri_nrm, const float* tri_uv, int64_t n_tris, double aspect);
void ora_scene_free(ora_scene* s);
const char* ora_last_error(void);

/* FP32 nearest hit over [tmin, tmax): rays n*8 floats (o, tmin, d, tmax). */
int ora_intersect(ora_scene* s, const float* rays, int64_t n, int32_t use_bvh, int32_t* prim, float* t, float* uv);
/* Scene::Visible for n point pairs (6 doubles each). */
int ora_visible(ora_scene* s, const double* pts, int64_t n, int32_t use_bvh, uint8_t* vis);
/* Normalised film (W*H*3, row 0 bottom), like Renderer::Render. */
int ora_render(ora_scene* s, const ora_render_params* p, double* film, ora_render_stats* stats);

/* Known-answer hooks */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint32_t ora_mt19937_nth(uint32_t seed, int64_t n);   /* n-th output (1-based) */
double ora_mt19937_uniform(uint32_t seed, int64_t n); /* n-th uniform_real_distribution<double> */

/* Single-vertex BSDF hooks (for energy / reciprocity tests). Frame: shading normal = +z. */
int ora_bsdf_sample(const ora_prim_desc* prim, const double wi[3], const double u[3], double wo[3],
                    double* pdf, double fs[3]);
int ora_bsdf_eval(const ora_prim_desc* prim, const double wi[3], const double wo[3], int force_degenerated,
                  double fs[3], double* pdf);

#ifdef __cplusplus
}
#endif

#endif
