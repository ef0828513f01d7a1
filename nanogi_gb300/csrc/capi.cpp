// C ABI of nanogi-gb300 (include/nanogi.h): status codes, thread-local error text, no
// exception ever crosses the boundary.
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/nanogi.h"
#include "device_scene.hpp"
#include "image_io.hpp"
#include "texture.hpp"
#include "obj_loader.hpp"
#include "scene.hpp"
#include "yaml_lite.hpp"

struct ngi_scene {
    std::unique_ptr<ngi::HostScene> host;
};

namespace {

thread_local std::string g_last_error;

ngi_status Fail(ngi_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

template <typename F>
ngi_status Guard(F&& f) {
    try {
        g_last_error.clear();
        return f();
    } catch (const ngi::SceneError& e) {
        return Fail((ngi_status)e.code, e.what());
    } catch (const ngi::DeviceError& e) {
        return Fail((ngi_status)e.code, e.what());
    } catch (const ngi::ImageError& e) {
        return Fail((ngi_status)e.code, e.what());
    } catch (const ngi::YamlError& e) {
        return Fail(NGI_ERR_PARSE, e.what());
    } catch (const ngi::ObjError& e) {
        return Fail(NGI_ERR_PARSE, e.what());
    } catch (const std::bad_alloc&) {
        return Fail(NGI_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return Fail(NGI_ERR_INVALID_ARGUMENT, e.what());
    } catch (...) {
        return Fail(NGI_ERR_INVALID_ARGUMENT, "unknown error");
    }
}

ngi_status CheckParams(const ngi_scene* scene, const ngi_render_params* p) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (!p) return Fail(NGI_ERR_INVALID_ARGUMENT, "params is NULL");
    if (p->renderer < NGI_RENDERER_PT || p->renderer > NGI_RENDERER_BDPT)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "renderer must be pt, ptdirect, lt, ltdirect or bdpt");
    if (p->width <= 0 || p->height <= 0) return Fail(NGI_ERR_INVALID_ARGUMENT, "width and height must be positive");
    if ((int64_t)p->width * (int64_t)p->height > ((int64_t)1 << 31) - 1)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "width*height must fit in 31 bits");
    if (p->num_samples < 0) return Fail(NGI_ERR_INVALID_ARGUMENT, "num_samples must be >= 0");
    if (p->sample_offset < 0) return Fail(NGI_ERR_INVALID_ARGUMENT, "sample_offset must be >= 0");
    if (p->max_num_vertices < -1 || p->max_num_vertices == 0)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "max_num_vertices must be -1 or >= 1");
    if (p->precision != NGI_PRECISION_FP32 && p->precision != NGI_PRECISION_FP64)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "precision must be FP32 or FP64");
    if (p->raster_mode != NGI_RASTER_STRATIFIED && p->raster_mode != NGI_RASTER_UNIFORM)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "raster_mode must be STRATIFIED or UNIFORM");
    if (p->wave_size < 0 || p->iterations_per_graph < 0 || p->iterations_per_graph > 64)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "wave_size / iterations_per_graph out of range");
    if (p->trace_refill < 0 || p->trace_refill > 32)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "trace_refill must be 0 (auto) or 1..32");
    if (p->reserved != 0) return Fail(NGI_ERR_INVALID_ARGUMENT, "the reserved field must be 0");
    if (p->ray_offset != NGI_RAY_OFFSET_REFERENCE && p->ray_offset != NGI_RAY_OFFSET_SCALED)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "ray_offset must be REFERENCE or SCALED");
    return NGI_OK;
}

// The batch, adjoint and allocation-free paths run the camera-path tracers only.
ngi_status CheckCameraRenderer(const ngi_render_params* p) {
    if (p->renderer != NGI_RENDERER_PT && p->renderer != NGI_RENDERER_PTDIRECT)
        return Fail(NGI_ERR_UNSUPPORTED, "this entry point runs pt and ptdirect only");
    return NGI_OK;
}

}  // namespace

extern "C" {

NGI_API const char* ngi_last_error(void) { return g_last_error.c_str(); }

NGI_API int32_t ngi_abi_version(void) { return NGI_ABI_VERSION; }

NGI_API ngi_status ngi_scene_load(const char* yaml_path, double aspect, ngi_scene** out_scene) {
    if (!out_scene) return Fail(NGI_ERR_INVALID_ARGUMENT, "out_scene is NULL");
    *out_scene = nullptr;
    if (!yaml_path) return Fail(NGI_ERR_INVALID_ARGUMENT, "path is NULL");
    return Guard([&]() {
        auto host = ngi::LoadScene(yaml_path, aspect);
        auto* s = new ngi_scene();
        s->host = std::move(host);
        *out_scene = s;
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_scene_load_with_meshes(const char* yaml_path, double aspect, const ngi_mesh_data* meshes,
                                              int32_t num_meshes, ngi_scene** out_scene) {
    if (!out_scene) return Fail(NGI_ERR_INVALID_ARGUMENT, "out_scene is NULL");
    *out_scene = nullptr;
    if (!yaml_path) return Fail(NGI_ERR_INVALID_ARGUMENT, "path is NULL");
    if (num_meshes < 0 || (num_meshes > 0 && !meshes))
        return Fail(NGI_ERR_INVALID_ARGUMENT, "meshes is NULL or num_meshes is negative");
    std::vector<ngi::MemoryMesh> held((size_t)num_meshes);
    for (int32_t i = 0; i < num_meshes; i++) {
        const ngi_mesh_data& m = meshes[i];
        const std::string which = "mesh " + std::to_string(i);
        if (!m.path) return Fail(NGI_ERR_INVALID_ARGUMENT, which + ": path is NULL");
        if (m.num_vertices < 0 || m.num_triangles < 0)
            return Fail(NGI_ERR_INVALID_ARGUMENT, which + ": negative vertex or triangle count");
        if (m.num_triangles > 0 && (!m.positions || !m.faces))
            return Fail(NGI_ERR_INVALID_ARGUMENT, which + ": positions or faces is NULL");
        if (m.num_vertices > 0xFFFFFFFFll || m.num_triangles > 0x7FFFFFFFll)
            return Fail(NGI_ERR_INVALID_ARGUMENT, which + ": too many vertices or triangles");
        for (int64_t k = 0; k < 3 * m.num_triangles; k++)
            if ((int64_t)m.faces[k] >= m.num_vertices)
                return Fail(NGI_ERR_INVALID_ARGUMENT, which + ": face index out of range");
        held[i].path = m.path;
        held[i].positions = m.positions;
        held[i].normals = m.normals;
        held[i].texcoords = m.texcoords;
        held[i].faces = m.faces;
        held[i].num_vertices = m.num_vertices;
        held[i].num_triangles = m.num_triangles;
    }
    return Guard([&]() {
        auto host = ngi::LoadScene(yaml_path, aspect, &held);
        auto* s = new ngi_scene();
        s->host = std::move(host);
        *out_scene = s;
        return NGI_OK;
    });
}

NGI_API void ngi_scene_free(ngi_scene* scene) {
    if (!scene) return;
    try {
        if (scene->host) ngi::DeviceFree(*scene->host);
    } catch (...) {
    }
    delete scene;
}

NGI_API ngi_status ngi_scene_get_info(const ngi_scene* scene, ngi_scene_info* out) {
    if (!scene || !scene->host || !out) return Fail(NGI_ERR_INVALID_ARGUMENT, "NULL argument");
    const ngi::HostScene& h = *scene->host;
    std::memset(out, 0, sizeof(*out));
    out->num_primitives = (int32_t)h.prims.size();
    out->num_lights = (int32_t)h.light_prims.size();
    out->sensor_index = h.sensor_prim;
    out->sensor_type = h.sensor_prim >= 0 ? h.prims[h.sensor_prim].e_type : -1;
    out->num_triangles = h.NumTriangles();
    out->num_vertices = h.num_vertices;
    for (int k = 0; k < 3; k++) {
        out->bound_min[k] = h.bmin[k];
        out->bound_max[k] = h.bmax[k];
    }
    if (h.dev) {
        out->device_ready = 1;
        out->bvh_nodes = h.dev->num_nodes;
        out->bvh_bytes = (int64_t)h.dev->num_nodes * 80 + (int64_t)h.dev->num_tris * 48;
        out->bvh_build_ms = h.dev->build_ms;
    }
    g_last_error.clear();
    return NGI_OK;
}

NGI_API ngi_status ngi_scene_get_triangles(const ngi_scene* scene, float* pos, float* nrm, float* uv, int32_t* prim) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    const ngi::HostScene& h = *scene->host;
    if (pos && !h.tri_pos.empty()) std::memcpy(pos, h.tri_pos.data(), h.tri_pos.size() * sizeof(float));
    if (nrm && !h.tri_nrm.empty()) std::memcpy(nrm, h.tri_nrm.data(), h.tri_nrm.size() * sizeof(float));
    if (uv && !h.tri_uv.empty()) std::memcpy(uv, h.tri_uv.data(), h.tri_uv.size() * sizeof(float));
    if (prim && !h.tri_prim.empty()) std::memcpy(prim, h.tri_prim.data(), h.tri_prim.size() * sizeof(int32_t));
    g_last_error.clear();
    return NGI_OK;
}

NGI_API ngi_status ngi_scene_build(ngi_scene* scene) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    return Guard([&]() {
        ngi::DeviceUpload(*scene->host);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_scene_release_buffers(ngi_scene* scene) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    return Guard([&]() {
        ngi::DeviceReleaseBuffers(*scene->host);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_render(ngi_scene* scene, const ngi_render_params* params, double* film_rgb) {
    const ngi_status st = CheckParams(scene, params);
    if (st != NGI_OK) return st;
    if (!film_rgb) return Fail(NGI_ERR_INVALID_ARGUMENT, "film is NULL");
    return Guard([&]() {
        ngi::DeviceRenderToHost(*scene->host, *params, film_rgb);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_render_device(ngi_scene* scene, const ngi_render_params* params, double* d_film_rgb,
                                     void* stream) {
    const ngi_status st = CheckParams(scene, params);
    if (st != NGI_OK) return st;
    if (!d_film_rgb) return Fail(NGI_ERR_INVALID_ARGUMENT, "film is NULL");
    return Guard([&]() {
        ngi::DeviceRender(*scene->host, *params, d_film_rgb, (cudaStream_t)stream);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_render_device_noalloc(ngi_scene* scene, const ngi_render_params* params, double* d_film_rgb,
                                             void* stream) {
    const ngi_status st = CheckParams(scene, params);
    if (st != NGI_OK) return st;
    if (CheckCameraRenderer(params) != NGI_OK) return NGI_ERR_UNSUPPORTED;
    if (!d_film_rgb) return Fail(NGI_ERR_INVALID_ARGUMENT, "film is NULL");
    return Guard([&]() {
        ngi::DeviceRenderNoAlloc(*scene->host, *params, d_film_rgb, (cudaStream_t)stream);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_get_render_stats(const ngi_scene* scene, ngi_render_stats* out) {
    if (!scene || !scene->host || !out) return Fail(NGI_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!scene->host->dev) {
        std::memset(out, 0, sizeof(*out));
    } else {
        *out = scene->host->dev->last_stats;
    }
    g_last_error.clear();
    return NGI_OK;
}

NGI_API ngi_status ngi_render_batch(ngi_scene* const* scenes, const ngi_render_params* params, int32_t num_jobs,
                                    double* const* films, const ngi_batch_options* options, ngi_batch_stats* stats) {
    if (num_jobs < 0 || (num_jobs > 0 && (!scenes || !params)))
        return Fail(NGI_ERR_INVALID_ARGUMENT, "bad job arrays");
    std::vector<ngi::HostScene*> hs((size_t)num_jobs);
    std::vector<ngi_render_params> ps((size_t)num_jobs);
    for (int32_t j = 0; j < num_jobs; j++) {
        const ngi_status st = CheckParams(scenes[j], &params[j]);
        if (st != NGI_OK) return Fail(st, "job " + std::to_string(j) + ": " + g_last_error);
        if (CheckCameraRenderer(&params[j]) != NGI_OK) return NGI_ERR_UNSUPPORTED;
        hs[(size_t)j] = scenes[j]->host.get();
        ps[(size_t)j] = params[j];
    }
    ngi_batch_options opt{};
    if (options) opt = *options;
    if (opt.wave_size < 0 || opt.trace_refill < 0 || opt.trace_refill > 32 || opt.iterations_per_graph < 0 ||
        opt.iterations_per_graph > 64 || !(opt.autotune_fraction >= 0.0) || opt.autotune_fraction > 1.0)
        return Fail(NGI_ERR_INVALID_ARGUMENT, "batch options out of range");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (num_jobs == 0) {
        g_last_error.clear();
        return NGI_OK;
    }
    return Guard([&]() {
        ngi::DeviceRenderBatch(hs, ps, films, opt, stats);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_scene_get_parameters(const ngi_scene* scene, double* albedo, double* emission) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    const ngi::HostScene& h = *scene->host;
    for (size_t i = 0; i < h.prims.size(); i++) {
        const ngi::HostPrimitive& p = h.prims[i];
        const double* r = (p.type & ngi::PT_D) ? p.D_R : (p.type & ngi::PT_G) ? p.G_R : (p.type & ngi::PT_S) ? p.S_R : nullptr;
        for (int k = 0; k < 3; k++) {
            if (albedo) albedo[3 * i + k] = r ? r[k] : 0.0;
            if (emission) emission[3 * i + k] = (p.type & ngi::PT_L) ? p.Le[k] : 0.0;
        }
    }
    g_last_error.clear();
    return NGI_OK;
}

NGI_API ngi_status ngi_scene_set_parameters(ngi_scene* scene, const double* albedo, const double* emission) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    return Guard([&]() {
        ngi::HostScene& h = *scene->host;
        for (size_t i = 0; i < h.prims.size(); i++) {
            ngi::HostPrimitive& p = h.prims[i];
            double* r = (p.type & ngi::PT_D) ? p.D_R : (p.type & ngi::PT_G) ? p.G_R : (p.type & ngi::PT_S) ? p.S_R : nullptr;
            for (int k = 0; k < 3; k++) {
                if (albedo && r) {
                    if (!std::isfinite(albedo[3 * i + k])) return Fail(NGI_ERR_INVALID_ARGUMENT, "albedo must be finite");
                    r[k] = albedo[3 * i + k];
                }
                if (emission && (p.type & ngi::PT_L)) {
                    if (!std::isfinite(emission[3 * i + k])) return Fail(NGI_ERR_INVALID_ARGUMENT, "emission must be finite");
                    p.Le[k] = emission[3 * i + k];
                }
            }
        }
        ngi::DeviceUpdateTables(h);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_render_backward(ngi_scene* scene, const ngi_render_params* params, const double* d_film,
                                       double* grad_albedo, double* grad_emission) {
    const ngi_status st = CheckParams(scene, params);
    if (st != NGI_OK) return st;
    if (CheckCameraRenderer(params) != NGI_OK) return NGI_ERR_UNSUPPORTED;
    if (!scene->host->textures.empty())
        return Fail(NGI_ERR_UNSUPPORTED, "the adjoint differentiates constant albedos; the scene has TexR textures");
    if (!d_film) return Fail(NGI_ERR_INVALID_ARGUMENT, "d_film is NULL");
    return Guard([&]() {
        ngi::DeviceRenderBackward(*scene->host, *params, d_film, grad_albedo, grad_emission);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_intersect(ngi_scene* scene, const float* rays, int64_t n, int32_t* prim_out, float* t_out,
                                 float* uv_out) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n < 0 || (n > 0 && !rays)) return Fail(NGI_ERR_INVALID_ARGUMENT, "bad ray array");
    return Guard([&]() {
        ngi::DeviceIntersect(*scene->host, rays, n, prim_out, t_out, uv_out);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_visible(ngi_scene* scene, const double* points, int64_t n, uint8_t* visible_out) {
    if (!scene || !scene->host) return Fail(NGI_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (n < 0 || (n > 0 && (!points || !visible_out))) return Fail(NGI_ERR_INVALID_ARGUMENT, "bad point array");
    return Guard([&]() {
        ngi::DeviceVisible(*scene->host, points, n, visible_out);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_save_image(const char* path, const double* film_rgb, int32_t width, int32_t height) {
    if (!path || !film_rgb) return Fail(NGI_ERR_INVALID_ARGUMENT, "NULL argument");
    return Guard([&]() {
        ngi::SaveImage(path, film_rgb, width, height);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_load_hdr(const char* path, double* film_rgb, int32_t width, int32_t height) {
    if (!path || !film_rgb || width <= 0 || height <= 0) return Fail(NGI_ERR_INVALID_ARGUMENT, "bad argument");
    return Guard([&]() {
        ngi::LoadHdr(path, film_rgb, width, height);
        return NGI_OK;
    });
}

NGI_API ngi_status ngi_load_texture(const char* path, float* rgb, int32_t* width, int32_t* height) {
    if (!path || !width || !height) return Fail(NGI_ERR_INVALID_ARGUMENT, "NULL argument");
    return Guard([&]() {
        const ngi::TextureImage t = ngi::LoadTexture(path);
        *width = t.width;
        *height = t.height;
        if (rgb) std::memcpy(rgb, t.rgb.data(), t.rgb.size() * sizeof(float));
        return NGI_OK;
    });
}

}  // extern "C"
