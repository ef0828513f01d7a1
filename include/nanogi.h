/*
 * nanogi-gb300 C ABI: the single host<->device boundary of the GB300 path tracer.
 *
 * The reference (lighttransport/nanogi) has no plugin or FFI layer. Its renderer
 * interface is (i) the command line, (ii) the YAML scene schema and (iii) the film
 * file, with the C++ entry points listed next to each function below. This header
 * exposes exactly those entry points as plain C: opaque handles, plain pointers and
 * sizes, integer status codes, and no exceptions or C++/torch types crossing it.
 *
 * Conventions shared by every function:
 *   - Every call returns an ngi_status; NGI_OK is 0. On failure a human-readable
 *     message is available from ngi_last_error() (thread-local, valid until the next
 *     call on the same thread).
 *   - Films are W*H*3 doubles, row 0 = the BOTTOM scanline, pixel index = y*W + x,
 *     exactly the layout of std::vector<glm::dvec3> film in the reference
 *     (src/nanogi.cpp:429-437, include/nanogi/rt.hpp:135-140).
 *   - A scene handle owns its host copy, its device buffers, its CUDA stream and its
 *     wave buffers. A handle must not be used from two host threads at once.
 */
#ifndef NANOGI_GB300_H
#define NANOGI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define NGI_API __declspec(dllexport)
#else
#define NGI_API __attribute__((visibility("default")))
#endif

#define NGI_ABI_VERSION 1

typedef enum ngi_status {
    NGI_OK = 0,
    NGI_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or parameter */
    NGI_ERR_IO = 2,               /* file missing / unreadable / unwritable */
    NGI_ERR_PARSE = 3,            /* malformed YAML or OBJ, schema violation */
    NGI_ERR_CUDA = 4,             /* CUDA runtime error (message carries the CUDA string) */
    NGI_ERR_OUT_OF_MEMORY = 5,    /* host or device allocation failed */
    NGI_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up */
    NGI_ERR_UNSUPPORTED = 7,      /* valid input the reference rejects or crashes on */
    NGI_ERR_NO_DEVICE = 8         /* no CUDA device visible */
} ngi_status;

/* Renderer names of the reference (src/nanogi.cpp:51-69). All five estimators are built; ptmnee is not. */
typedef enum ngi_renderer_type {
    NGI_RENDERER_PT = 0,       /* "pt"       : ProcessSample_PT       src/nanogi.cpp:446-607 */
    NGI_RENDERER_PTDIRECT = 1, /* "ptdirect" : ProcessSample_PTDirect src/nanogi.cpp:609-802 */
    NGI_RENDERER_LT = 2,       /* "lt"       : ProcessSample_LT       src/nanogi.cpp:804-955 */
    NGI_RENDERER_LTDIRECT = 3, /* "ltdirect" : ProcessSample_LTDirect src/nanogi.cpp:957-1131 */
    NGI_RENDERER_BDPT = 4      /* "bdpt"     : ProcessSample_BDPT     src/nanogi.cpp:1133-1194, include/nanogi/bdpt.hpp;
                                  subpaths keep at most 32 vertices */
} ngi_renderer_type;

/* Arithmetic of the shading stage. Traversal is FP32 and accumulation FP64 in both. */
typedef enum ngi_precision {
    NGI_PRECISION_FP32 = 0,   /* tuned path: FP32 shading, FP64 film */
    NGI_PRECISION_FP64 = 1    /* plain path: FP64 shading and path state, FP64 film */
} ngi_precision;

/* Sample -> raster mapping. The reference draws every sample uniformly over the whole
 * image (include/nanogi/rt.hpp:733-739 with u from src/nanogi.cpp:495); STRATIFIED gives
 * each pixel an equal share of whole passes (same expectation, lower variance). */
typedef enum ngi_raster_mode {
    NGI_RASTER_STRATIFIED = 0,
    NGI_RASTER_UNIFORM = 1
} ngi_raster_mode;

/* Renderer parameters: the reference's Renderer::Params (src/nanogi.cpp:85-97) plus the
 * replay seed and the GPU-only knobs. */
typedef struct ngi_render_params {
    int32_t renderer;          /* ngi_renderer_type */
    int32_t max_num_vertices;  /* -m; -1 = unbounded (src/nanogi.cpp:2007) */
    int64_t num_samples;       /* -n; TOTAL samples over the image (src/nanogi.cpp:2006) */
    int32_t width;             /* -w */
    int32_t height;            /* -h */
    uint64_t seed;             /* Philox key: (seed, sample index) makes every path replayable */
    int64_t sample_offset;     /* first global sample index (sharded / resumed renders) */
    int32_t precision;         /* ngi_precision */
    int32_t raster_mode;       /* ngi_raster_mode */
    int32_t wave_size;         /* path slots resident on the device; 0 = auto (2^25 for ptdirect and for pt
                                  renders of at most 2^25 samples, 2^18 for bdpt, 2^23 otherwise, never above
                                  the samples) */
    int32_t iterations_per_graph; /* wave iterations per CUDA-graph launch; 0 = auto (6 for a ptdirect
                                     or pt wave that holds every sample, else 4) */
    int32_t flags;             /* NGI_RENDER_* measurement flags, 0 for normal renders */
    int32_t trace_refill;      /* idle lanes that make a traversal warp fetch new rays (1..32); 0 = auto */
    int32_t reserved;          /* must be 0 */
    int32_t ray_offset;        /* ngi_ray_offset: how rays leave a surface */
} ngi_render_params;

/* How a ray leaves a surface point. REFERENCE keeps the reference's absolute tmin = EpsF = 1e-4
 * scene units (Scene::Intersect rt.hpp:2248, Visible rt.hpp:2260); SCALED moves the origin a
 * fixed number of float ulps along the geometric normal and uses tmin = 0, which holds at any
 * scene scale (Waechter and Binder, Ray Tracing Gems 2019, ch. 6). */
typedef enum ngi_ray_offset {
    NGI_RAY_OFFSET_REFERENCE = 0,
    NGI_RAY_OFFSET_SCALED = 1
} ngi_ray_offset;

/* Render flags. The first two are measurement flags (results in ngi_render_stats); none of the
 * three changes the film. */
#define NGI_RENDER_KERNEL_TIMING 1        /* launch without graphs, CUDA events around each kernel */
#define NGI_RENDER_TRAVERSAL_COUNTERS 2   /* count BVH nodes and triangles visited per ray */
/* ptdirect and ltdirect score only through connections made at vertices that survive Russian
 * roulette, and the roulette variable of a path's next hit is drawn with its current vertex: by
 * default an extension ray whose hit the roulette (or the length limit) will end is not traced. The film is
 * the same sample for sample; extension_rays counts the rays traced. This flag traces them all,
 * as the reference does (ray counts then match the reference's). */
#define NGI_RENDER_TRACE_ALL_RAYS 4

/* Counters of the last render on a scene handle (per-stage ray counts etc). */
typedef struct ngi_render_stats {
    int64_t camera_rays;       /* paths started (= samples processed) */
    int64_t extension_rays;    /* closest-hit rays traced (camera rays included) */
    int64_t shadow_rays;       /* visibility rays traced (NEE) */
    int64_t film_contributions;/* non-zero contributions added to the film */
    int64_t iterations;        /* wave iterations executed */
    int64_t nonfinite;         /* NaN/Inf contributions dropped (reported, never trapped) */
    double render_ms;          /* device time of the render (CUDA events on the render stream) */
    /* NGI_RENDER_KERNEL_TIMING: summed device time and launch count per kernel. One traversal
     * launch per iteration traces both the extension and the shadow queue: extend_* cover that
     * launch, and shadow_ms / shadow_launches are 0. */
    double logic_ms, extend_ms, shadow_ms;
    int64_t logic_launches, extend_launches, shadow_launches;
    /* NGI_RENDER_TRAVERSAL_COUNTERS: nodes / triangles visited, over all rays of each kind */
    int64_t extend_nodes, extend_tris, shadow_nodes, shadow_tris;
    /* pt / ptdirect camera paths: once every sample is claimed and few paths remain, one launch
     * runs each remaining path to its end (one thread per path). The paths it ran; 0 when the wave
     * drained without it. */
    int64_t finish_paths;
} ngi_render_stats;

/* Scene summary (host side; available without a GPU). */
typedef struct ngi_scene_info {
    int32_t num_primitives;
    int32_t num_lights;
    int32_t sensor_index;      /* index of the E primitive, -1 if none */
    int32_t sensor_type;       /* 0 = area, 1 = pinhole (EType, rt.hpp:360-364) */
    int64_t num_triangles;
    int64_t num_vertices;
    double bound_min[3];
    double bound_max[3];
    int32_t device_ready;      /* 1 once the BVH has been built on the device */
    int32_t bvh_nodes;         /* compressed 8-wide nodes */
    int64_t bvh_bytes;         /* node + triangle bytes resident in HBM */
    double bvh_build_ms;       /* device time of the last BVH build */
} ngi_scene_info;

typedef struct ngi_scene ngi_scene;

/* ---- errors / version ---------------------------------------------------------- */

/* Message of the last failed call on this thread ("" if none). */
NGI_API const char* ngi_last_error(void);
NGI_API int32_t ngi_abi_version(void);

/* ---- scene ------------------------------------------------------------------------ */

/* Scene::Load(const std::string& path, double aspect)  include/nanogi/rt.hpp:1519-2154.
 * Parses the YAML scene (schema versions 3..5, schema.yml:33-334) and its OBJ meshes,
 * flattens them into host SoA arrays. Does not touch the GPU. */
NGI_API ngi_status ngi_scene_load(const char* yaml_path, double aspect, ngi_scene** out_scene);

/* A triangle mesh held by the caller (Mesh::Positions / Normals / Texcoords / Faces,
 * rt.hpp:148-155). It stands in for the mesh file that a primitive's `mesh: path:` names. */
typedef struct ngi_mesh_data {
    const char* path;            /* matched verbatim against the scene file's mesh paths */
    const float* positions;      /* 3 per vertex */
    const float* normals;        /* 3 per vertex, or NULL for flat face normals */
    const float* texcoords;      /* 2 per vertex, or NULL */
    const uint32_t* faces;       /* 3 vertex indices per triangle, 0-based */
    int64_t num_vertices;
    int64_t num_triangles;
} ngi_mesh_data;

/* ngi_scene_load, with meshes taken from memory: a primitive whose mesh path equals the path
 * of one of `meshes` reads that mesh instead of the file (other paths still load from disk).
 * The arrays are copied; the caller may free them on return. No reference counterpart: the
 * reference reads every mesh through Assimp (rt.hpp:1640-1730). */
NGI_API ngi_status ngi_scene_load_with_meshes(const char* yaml_path, double aspect, const ngi_mesh_data* meshes,
                                              int32_t num_meshes, ngi_scene** out_scene);

/* Scene::~Scene  include/nanogi/rt.hpp:1509-1513. Frees host and device memory. */
NGI_API void ngi_scene_free(ngi_scene* scene);

NGI_API ngi_status ngi_scene_get_info(const ngi_scene* scene, ngi_scene_info* out_info);

/* Copies the flattened host triangle arrays (what Scene::Load produced, rt.hpp:1676-1731):
 * pos/nrm: num_triangles*9 floats (p1,p2,p3 / n1,n2,n3), uv: num_triangles*6 floats (zeros
 * when the mesh has none), prim: owning primitive per triangle. Any pointer may be NULL.
 * Host only; no GPU needed. */
NGI_API ngi_status ngi_scene_get_triangles(const ngi_scene* scene, float* pos, float* nrm, float* uv, int32_t* prim);

/* Uploads the flattened scene and builds the compressed 8-wide BVH on the GPU: the
 * counterpart of the Embree build in include/nanogi/rt.hpp:2087-2143. Called implicitly
 * by the first render/intersect; explicit so its cost can be measured apart. */
NGI_API ngi_status ngi_scene_build(ngi_scene* scene);

/* Frees the render buffers a scene handle keeps between renders (its wave of path slots and
 * queues: at most 2^25 slots, about 8.6 GB in FP32 and 13.4 GB in FP64, never more slots than a
 * render's samples); the scene itself stays on the device and the next render allocates them
 * again. For programs that keep many scene handles alive. Not in the reference (its per-thread
 * contexts live for one render, nanogi.cpp:281-319). */
NGI_API ngi_status ngi_scene_release_buffers(ngi_scene* scene);

/* ---- rendering --------------------------------------------------------------------- */

/* Renderer::Render(const Scene&, std::vector<glm::dvec3>& film)  src/nanogi.cpp:182-221
 * with RenderProcess's gather and W*H/N normalisation (src/nanogi.cpp:429-437).
 * film_rgb: HOST array of width*height*3 doubles, overwritten with the normalised film. */
NGI_API ngi_status ngi_render(ngi_scene* scene, const ngi_render_params* params, double* film_rgb);

/* Same render, film left on the device: d_film_rgb is a DEVICE pointer to width*height*3
 * doubles which receives the RAW (un-normalised) sums added to its current contents; the
 * caller scales by width*height/num_samples. stream: cudaStream_t or NULL for the scene's
 * own stream. Returns after the work is enqueued AND complete. */
NGI_API ngi_status ngi_render_device(ngi_scene* scene, const ngi_render_params* params,
                                     double* d_film_rgb, void* stream);

NGI_API ngi_status ngi_get_render_stats(const ngi_scene* scene, ngi_render_stats* out_stats);

/* Allocation-free variant of ngi_render_device. It has no counterpart in the reference.
 *
 * For callers that cannot allocate device memory while they render: an application whose
 * own allocator owns the whole device, a real-time loop that cannot take the device-wide
 * synchronisation cudaMalloc / cudaFree may cause, or a process held to a fixed memory
 * budget. The call allocates nothing (no cudaMalloc, cudaFree, graph or event creation):
 * the render's scratch -- its wave of path slots, queues and counters -- lives in one
 * 32 MiB file-scope device array.
 *
 * Limits and rules:
 *   - pt and ptdirect only; lt, ltdirect and bdpt return NGI_ERR_UNSUPPORTED;
 *   - the scene must already be on the device (ngi_scene_build), else NGI_ERR_INVALID_ARGUMENT,
 *     and that device must be the current one, else NGI_ERR_INVALID_ARGUMENT;
 *   - params->wave_size must be 0 (= 65536) or at most 65536 path slots, else
 *     NGI_ERR_INVALID_ARGUMENT; num_samples is not bounded (samples stream through the wave);
 *   - params->flags may hold NGI_RENDER_TRACE_ALL_RAYS and nothing else (the measurement
 *     flags need buffers of their own), else NGI_ERR_INVALID_ARGUMENT;
 *   - params->iterations_per_graph sets how many wave iterations run between two reads of the
 *     wave's counters (0 = 4; odd counts are rounded up to even);
 *   - the caller passes the output: d_film_rgb, a DEVICE array of width*height*3 doubles that
 *     receives the raw sums added to its contents, as with ngi_render_device;
 *   - the 32 MiB are reserved on a device the first time this library's render code runs
 *     there (CUDA loads it lazily) and are held until the process exits. A caller whose own
 *     allocator will take the whole device makes one call first, before that allocator starts:
 *     a call with num_samples = 0 does this set-up (and looks up the array's device address)
 *     without rendering;
 *   - every call reads the wave's counters back to the host and synchronises the stream, so it
 *     cannot be made while the stream is being captured into a CUDA graph;
 *   - every call shares the array and clears what must start at zero; calls that overlap on
 *     the GPU (e.g. from two streams at once) race on it and must not be made. */
NGI_API ngi_status ngi_render_device_noalloc(ngi_scene* scene, const ngi_render_params* params,
                                             double* d_film_rgb, void* stream);

/* ---- batches (no counterpart in the reference: it renders one scene per process) ------ */

typedef struct ngi_batch_options {
    int32_t autotune;             /* 1: choose wave size, refill threshold and graph length by
                                     short timed trials on a sample of every job first */
    int32_t wave_size;            /* path slots; 0 = auto (the starting point of the autotuner) */
    int32_t trace_refill;         /* 0 = auto */
    int32_t iterations_per_graph; /* 0 = auto */
    double autotune_fraction;     /* share of each job's samples per trial; 0 = 0.02 */
} ngi_batch_options;

typedef struct ngi_batch_stats {
    double render_ms;             /* device time of the batch render (autotuning excluded) */
    double autotune_ms;           /* device time of the autotuning trials */
    int64_t samples;
    int64_t extension_rays;
    int64_t shadow_rays;
    int64_t iterations;
    int32_t wave_size;            /* the configuration used */
    int32_t trace_refill;
    int32_t iterations_per_graph;
    int32_t trials;
} ngi_batch_stats;

/* Renders num_jobs independent jobs -- scenes[i] with params[i] into the HOST film films[i]
 * (width*height*3 doubles, normalised as ngi_render does) -- through ONE shared wave of
 * path slots replayed from one CUDA graph: every job's samples share the slots, so small
 * jobs never leave the GPU idle. Jobs may differ in scene, renderer, resolution, samples,
 * max vertices and seed; all must use the same precision. The same scene handle may appear
 * in several jobs. films[i] may be NULL. stats may be NULL. */
NGI_API ngi_status ngi_render_batch(ngi_scene* const* scenes, const ngi_render_params* params, int32_t num_jobs,
                                    double* const* films, const ngi_batch_options* options, ngi_batch_stats* stats);

/* ---- differentiable rendering (no counterpart in the reference) ---------------------- */

/* Reads / replaces the differentiable parameters of every primitive: `albedo` is the R of
 * the BSDF used at hits (D.R, else G.R, else S.*.R; rt.hpp:439-476), `emission` the Le of a
 * light (rt.hpp:395-415). Arrays hold num_primitives*3 doubles; either may be NULL. Entries of
 * primitives without a BSDF / without L are ignored on write and zero on read. Updates the
 * device tables in place when the scene is built (no reload, no BVH rebuild). */
NGI_API ngi_status ngi_scene_get_parameters(const ngi_scene* scene, double* albedo, double* emission);
NGI_API ngi_status ngi_scene_set_parameters(ngi_scene* scene, const double* albedo, const double* emission);

/* Path-replay adjoint of ngi_render with the same params (seed included): replays the same
 * paths, recomputing rather than storing them, and returns dLoss/dalbedo and dLoss/demission
 * (num_primitives*3 doubles each, overwritten) for d_film = dLoss/d(film), the HOST gradient
 * of the normalised film ngi_render returned. Requires max_num_vertices in 1..17. */
NGI_API ngi_status ngi_render_backward(ngi_scene* scene, const ngi_render_params* params, const double* d_film,
                                       double* grad_albedo, double* grad_emission);

/* ---- parity hooks ------------------------------------------------------------------ */

/* Scene::Intersect(ray, isect, minT, maxT)  include/nanogi/rt.hpp:2162-2244, restricted
 * to what the Embree query returns: nearest triangle, t and barycentric u, v.
 * rays: HOST array of n*8 floats (ox, oy, oz, tmin, dx, dy, dz, tmax).
 * prim_out[i] = global triangle index (primitives in YAML order, faces in mesh order)
 * or -1 on a miss; t_out[i]; uv_out[2i..2i+1] = (u, v) with hit point
 * (1-u-v)*p0 + u*p1 + v*p2 (Embree convention, rt.hpp:2212). Any output may be NULL. */
NGI_API ngi_status ngi_intersect(ngi_scene* scene, const float* rays, int64_t n,
                                 int32_t* prim_out, float* t_out, float* uv_out);

/* Scene::Visible(p1, p2)  include/nanogi/rt.hpp:2251-2261 for n point pairs.
 * points: HOST array of n*6 doubles (p1.xyz, p2.xyz). visible_out[i] = 1 if unoccluded. */
NGI_API ngi_status ngi_visible(ngi_scene* scene, const double* points, int64_t n,
                               uint8_t* visible_out);

/* ---- film I/O ------------------------------------------------------------------------ */

/* SaveImage(path, film, w, h)  include/nanogi/basic.hpp:506-672 for ".hdr" (Radiance
 * RGBE, upright image: the bottom film row is written last) and ".pfm". */
NGI_API ngi_status ngi_save_image(const char* path, const double* film_rgb, int32_t width, int32_t height);

/* Reads back a ".hdr" written by ngi_save_image into width*height*3 doubles, row 0 =
 * bottom (test helper; no reference counterpart beyond Texture::Load of .hdr, rt.hpp:168). */
NGI_API ngi_status ngi_load_hdr(const char* path, double* film_rgb, int32_t width, int32_t height);

/* Texture::Load (rt.hpp:167-256): decodes a TexR image (PNG 8-bit RGB/RGBA, PPM P6, BMP
 * 24/32-bit, Radiance .hdr, PFM) into 3 floats per texel, row 0 = the image's top row, 8-bit
 * values as v/255. With rgb == NULL only *width and *height are filled in. */
NGI_API ngi_status ngi_load_texture(const char* path, float* rgb, int32_t* width, int32_t* height);

#ifdef __cplusplus
}
#endif

#endif /* NANOGI_GB300_H */
