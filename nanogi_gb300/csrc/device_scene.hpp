// Device side of a scene handle: HBM buffers, the scene stream and the render wave.
// Plain C++ (no device code) so the host translation units can include it.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nanogi.h"

namespace ngi {

struct HostScene;
struct CwNode;
struct RenderWave;  // wave buffers, defined in render.cu

struct DeviceError : std::runtime_error {
    int code;
    explicit DeviceError(const std::string& m, int c = NGI_ERR_CUDA) : std::runtime_error(m), code(c) {}
};

struct DeviceScene {
    int device = 0;
    cudaStream_t stream = nullptr;

    // geometry in HBM
    CwNode* nodes = nullptr;
    float4* tris = nullptr;   // 3 per triangle, leaf order
    float4* nrm = nullptr;    // 3 per triangle, leaf order
    float2* uv = nullptr;     // 3 per triangle, leaf order
    int num_nodes = 0;
    int num_tris = 0;
    int bvh_depth = 0;
    float build_ms = 0;

    // primitive / emitter tables (float and double copies)
    void* mats_f = nullptr;
    void* mats_d = nullptr;
    void* lights_f = nullptr;
    void* lights_d = nullptr;
    double* cdf = nullptr;
    float* emit_pos = nullptr;
    float* emit_uv = nullptr;
    float4* texels = nullptr;      // TexR images (see SceneView::texels)
    int4* tex_info = nullptr;
    int num_textures = 0;
    int num_lights = 0;
    // sensor records (host copies, passed by value to kernels)
    unsigned char sensor_f[256];
    unsigned char sensor_d[256];

    RenderWave* wave = nullptr;
    ngi_render_stats last_stats{};

    // film used by the host-buffer render entry point (kept between calls)
    double* film = nullptr;
    size_t film_elems = 0;
    // adjoint: dLoss/dfilm and the gradient accumulators (kept between calls)
    double* adj = nullptr;
    size_t adj_elems = 0;
    double* grads = nullptr;
    size_t grad_elems = 0;
};

// Uploads the flattened scene and builds the BVH on the current device.
void DeviceUpload(HostScene& scene);
void DeviceFree(HostScene& scene);
void DeviceReleaseBuffers(HostScene& scene);  // the cached wave of path slots
void BuildBvh(DeviceScene& ds, const float* d_pos, const float* d_nrm, const float* d_uv, const int* d_tri_prim,
              int n, cudaStream_t stream);

// Wavefront render of params into the device film (raw sums added to its contents).
void DeviceRender(HostScene& scene, const ngi_render_params& params, double* d_film, cudaStream_t stream);

// Host-buffer render: clears the scene's device film, renders, scales by W*H/N on the
// device and copies the normalised film into host memory.
void DeviceRenderToHost(HostScene& scene, const ngi_render_params& params, double* h_film);

// Same render with all scratch in a fixed file-scope device array: allocates nothing.
// Needs the scene built beforehand; bounds the wave at 65536 path slots.
void DeviceRenderNoAlloc(HostScene& scene, const ngi_render_params& params, double* d_film, cudaStream_t stream);

// Path-replay adjoint of DeviceRenderToHost: replays the same paths and accumulates
// dLoss/dR (BSDF albedo) and dLoss/dLe per primitive from h_dfilm = dLoss/d(normalised film).
void DeviceRenderBackward(HostScene& scene, const ngi_render_params& params, const double* h_dfilm,
                          double* grad_albedo, double* grad_emission);

// Renders many independent jobs in one persistent wave (one CUDA graph), optionally after
// autotuning the wave size / refill threshold / graph length on a sample of every job.
void DeviceRenderBatch(std::vector<HostScene*>& scenes, const std::vector<ngi_render_params>& params,
                       double* const* films, const ngi_batch_options& options, ngi_batch_stats* stats);

// Pushes the host copy of the materials / lights (after a parameter update) to the device.
void DeviceUpdateTables(HostScene& scene);

// Parity hooks.
void DeviceIntersect(HostScene& scene, const float* h_rays, int64_t n, int32_t* prim, float* t, float* uv);
void DeviceVisible(HostScene& scene, const double* h_points, int64_t n, uint8_t* visible);

}  // namespace ngi
