// Wavefront path tracing on GB300: the `pt` and `ptdirect` estimators of
// src/nanogi.cpp:446-607 and :609-802 reorganised as a persistent wave of path slots.
//
// One wave iteration = three kernels over HBM-resident SoA state:
//   k_logic  : per slot, consume the previous extension hit (emission for pt, Russian
//              roulette, vertex update), do next-event estimation (ptdirect) and sample the
//              next direction; a finished slot immediately claims the next sample index
//              (path regeneration) and starts a camera path. Extension and shadow rays are
//              appended to compacted queues with one atomic per warp.
//   k_trace<extension> : closest-hit traversal of the extension queue (compressed BVH8)
//   k_trace<shadow>    : any-hit traversal of the shadow queue; unoccluded contributions
//                        are added to the FP64 film with atomics.
// Both traversal kernels are persistent: resident warps refill idle lanes from the queue.
// Iterations are captured in a CUDA graph and replayed until every slot has drained.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device_scene.hpp"
#include "ngi_bdpt.cuh"
#include "ngi_shade.cuh"
#include "ngi_trace.cuh"
#include "scene.hpp"

namespace ngi {

#define CUDA_CHECK(x)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw DeviceError(std::string(cudaGetErrorString(e_)) + " (" #x ")",                   \
                              e_ == cudaErrorMemoryAllocation ? NGI_ERR_OUT_OF_MEMORY : NGI_ERR_CUDA); \
    } while (0)

template <typename R> struct alignas(4 * sizeof(R)) Vec4T { R x, y, z, w; };
// Wave records written and read once per iteration (rays, hits, shadow rays) move with the
// cache-streaming hint (evict first), so that L2 keeps the BVH nodes and triangles the rays share.
template <typename R>
__device__ __forceinline__ Vec4T<R> ld_stream(const Vec4T<R>* p) {
    if constexpr (sizeof(R) == 4) {
        const float4 v = __ldcs(reinterpret_cast<const float4*>(p));
        return Vec4T<R>{v.x, v.y, v.z, v.w};
    } else {
        return *p;
    }
}
template <typename R>
__device__ __forceinline__ void st_stream(Vec4T<R>* p, const Vec4T<R>& v) {
    if constexpr (sizeof(R) == 4) __stcs(reinterpret_cast<float4*>(p), make_float4(v.x, v.y, v.z, v.w));
    else *p = v;
}

// Resident 256-thread blocks per SM the path-logic kernel is compiled for. 2 leaves ptdirect's
// FP32 logic at 128 registers (25% occupancy); 4 caps it at 64 registers with ~250 B of spills
// to L1, and was faster on the terrain (1384 vs 1322 Mrays/s): the kernel waits on HBM.
// Also measured and not kept: 3 blocks (1579 vs 1621-1631 Mrays/s), and a bulk L2 prefetch
// (cp.async.bulk.prefetch) of the next loop iteration's slot arrays, alone (1460-1586) or with
// the next hit's triangle and normals (1551); the prefetched lines likely compete with the BVH for L2.
// No change (1875-1880 against 1875): loading the hit record together with the slot state, and an
// emitter cdf search in float pairs instead of FP64 (the FP64 pipe is 23% busy in this kernel).
constexpr int kLogicMinBlocks = 4;
// Minimum resident blocks per SM asked of the traversal kernels (register budget). 8 blocks of
// 128 give 64 registers and no spills. Measured on the 1.55M-triangle terrain (Mrays/s, two runs
// each): 8: 1809, 6 (80 registers): 1723, 10 (51, 132 B of spills): 1739, 12 (42): 1617.
constexpr int kTraceMinBlocks = 8;

enum : uint8_t { SLOT_EMPTY = 0, SLOT_ACTIVE = 1, SLOT_DONE = 2 };

// Kernels add to these with one atomic per warp (queue appends, sample claims) or per block
// (event counts, see BlockCounts); per-thread atomics on them queued at one L2 slice and cost the
// terrain 8% and the Cornell box a third of their throughput. Placing each counter on its own
// 128-byte line made no difference once they were gone.
struct WaveCounters {
    unsigned long long next_sample;   // samples claimed so far (local index)
    int ext_count;                    // reset before every iteration: ext_count .. sh_fetch
    int sh_count;
    int active;
    int ext_fetch;                    // rays handed out by the persistent traversal kernel
    int sh_fetch;                     // rays handed out by the shadow-only traversal kernel
    int regen_count;                  // slots handed from path shading to regeneration
    int error_flags;                  // bit 0: traversal stack overflow, 1: adjoint prefix, 2: wave-end vertex cap
    int ext_count_b;                  // compacted shading: count of the second extension queue
    int carry_count[2];               //   and of the two carry queues (reset per iteration by parity)
    int regen_seed;                   //   and the regeneration queue's length in the first iteration
    unsigned long long stat_camera;
    unsigned long long stat_ext;
    unsigned long long stat_shadow;
    unsigned long long stat_contrib;
    unsigned long long stat_nonfinite;
    unsigned long long ext_nodes, ext_tris, sh_nodes, sh_tris;  // traversal counters
};

struct RenderConsts {
    int renderer;
    int max_vertices;
    long long num_samples;
    long long sample_offset;
    unsigned long long seed;
    int width, height;
    int stratified;
    long long strat_end;    // global sample indices below this are pixel-stratified
    int trace_refill;       // idle lanes that trigger a traversal warp's refill
    int num_prims;          // primitives of the scene (adjoint gradient layout)
    int ray_offset;         // NGI_RAY_OFFSET_*: absolute tmin = EpsF, or scale-aware origin offsets
    int trace_all;          // NGI_RENDER_TRACE_ALL_RAYS: trace the rays toward hits that cannot score
    int one_pass;           // the queued wave holds every sample: no regeneration after the first iteration
};

// One job of a batch render: its scene, parameters, device film and first batch sample.
template <typename R>
struct JobView {
    SceneView<R> sv;
    RenderConsts rc;
    double* film;
    long long sample_base;
};

template <typename R>
struct WaveView {
    int Q;
    float4* ray_o;           // extension ray origin (xyz), tmin (w)
    float4* ray_d;           // direction (xyz), tmax (w)
    float4* hit;             // t, u, v, leaf-order triangle index (-1 = miss)
    Vec4T<R>* thr;           // throughput
    Vec4T<double>* od_o;     // FP64 path: exact origin
    Vec4T<double>* od_d;     // FP64 path: exact direction
    uint32_t* pixel;
    unsigned long long* sample;
    int* nverts;
    uint8_t* state;
    int* ext_queue;          // the iteration's extension rays (slot ids), traced by k_trace
    int* ext_count;          // their number (a counter in ctr)
    int* regen_queue;        // slots whose path ended this iteration (split path logic)
    // compacted shading (ptdirect): the slots to shade are the previous iteration's extension
    // queue and the slots regeneration left empty; both are double-buffered by iteration parity
    const int* ext_in;
    const int* ext_in_count;
    const int* carry_in;
    const int* carry_in_count;
    int* carry_out;
    int* carry_out_count;
    int* ext_queue_b;        // the second extension-queue buffer and the two carry buffers
    int* carry_a;
    int* carry_b;
    float4* sh_o;
    float4* sh_d;
    Vec4T<R>* sh_c;
    uint32_t* sh_pix;
    WaveCounters* ctr;
    double* film;
    // path-replay adjoint only (null otherwise)
    uint4* pre;              // per slot: 2 x uint4 = up to 16 primitive ids (uint16) of the path's surface vertices
    uint4* sh_pre;           // per shadow ray: the same prefix
    int2* sh_info;           // per shadow ray: x = prefix length | (NEE-vertex primitive + 1) << 8, y = light primitive
    const double* adj;       // dLoss/dfilm per pixel and channel, scaled by W*H/N
    double* grad_albedo;     // per primitive x 3
    double* grad_emission;   // per primitive x 3
    // batches only (null otherwise)
    int* job;                // per slot: job of the path
    int* sh_job;             // per shadow ray: job of the ray
    // bdpt only (null otherwise)
    BdVert<R>* bd_verts;     // per slot: light subpath then eye subpath, kBdptMaxVertices each
    int4* bd_info;           // per slot: phase | pending << 8, #light vertices, #eye vertices, cursor n << 8 | s
};

// Longest surface-vertex prefix the adjoint carries: paths of up to 17 vertices.
constexpr int kAdjMaxPrefix = 16;

// A wave's executable graphs, one pair per kind of wave run (an instantiation of run_wave and a graph
// length). Each render captures its graphs again (the launches take the render's constants by value)
// and updates the executable graphs in place, which costs far less than instantiating them.
struct WaveGraphs {
    const void* kind = nullptr;
    int iters = 0;
    bool one_pass = false;  // the wave holds every sample: regeneration in the first iteration only
    cudaGraphExec_t main = nullptr, drain = nullptr;
};

struct RenderWave {
    int Q = 0;
    int precision = -1;
    bool adjoint_buffers = false;
    int bdpt_precision = -1;  // precision the bdpt vertex arrays were sized for
    std::vector<void*> bufs;
    WaveCounters* ctr = nullptr;
    WaveCounters* h_ctr = nullptr;   // pinned
    WaveView<float> vf{};
    WaveView<double> vd{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<WaveGraphs> graphs;
};

// ---- warp helpers ----------------------------------------------------------------------
NGI_D unsigned lane_id() { return threadIdx.x & 31u; }
NGI_D unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// Warp-aggregated append: every lane of the warp calls this; returns the slot index for
// lanes with want == true.
NGI_D int warp_append(int* counter, bool want) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, want);
    if (mask == 0u) return -1;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return want ? base + __popc(mask & lanemask_lt()) : -1;
}
// The same for the lanes of a warp that are executing together (any subset of the warp): one
// atomic for those lanes.
NGI_D int coalesced_append(int* counter, bool want) {
    const unsigned act = __activemask();
    const unsigned mask = __ballot_sync(act, want);
    if (mask == 0u) return -1;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(act, base, leader);
    return want ? base + __popc(mask & lanemask_lt()) : -1;
}
// Block-wide claim: every thread of the block calls it, and the block takes its threads' wanted
// entries with one atomic (shared scratch: s_warp[kLogicBlock / 32], s_base). Returns the entry of a
// thread with want == true.
template <typename T>
NGI_D T block_claim(T* counter, bool want, int* s_warp, T* s_base) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, want);
    const int warp = (int)(threadIdx.x >> 5);
    if (lane_id() == 0) s_warp[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        int total = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            const int c = s_warp[k];
            s_warp[k] = total;
            total += c;
        }
        *s_base = total ? atomicAdd(counter, (T)total) : (T)0;
    }
    __syncthreads();
    const T idx = *s_base + (T)(s_warp[warp] + __popc(m & lanemask_lt()));
    __syncthreads();  // the scratch is reused by the next claim
    return idx;
}
// Two block-wide claims in one step (three barriers instead of six): entries of c0 for the threads
// with w0, of c1 for those with w1. c0 may be null (no claim; w0 must then be false).
NGI_D void block_claim2(int* c0, bool w0, int* c1, bool w1, int& q0, int& q1, int* s_warp0, int* s_warp1,
                        int* s_base) {
    const unsigned m0 = __ballot_sync(0xFFFFFFFFu, w0), m1 = __ballot_sync(0xFFFFFFFFu, w1);
    const int warp = (int)(threadIdx.x >> 5);
    if (lane_id() == 0) {
        s_warp0[warp] = __popc(m0);
        s_warp1[warp] = __popc(m1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int t0 = 0, t1 = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            const int a = s_warp0[k], b = s_warp1[k];
            s_warp0[k] = t0;
            s_warp1[k] = t1;
            t0 += a;
            t1 += b;
        }
        s_base[0] = t0 ? atomicAdd(c0, t0) : 0;
        s_base[1] = t1 ? atomicAdd(c1, t1) : 0;
    }
    __syncthreads();
    q0 = s_base[0] + s_warp0[warp] + __popc(m0 & lanemask_lt());
    q1 = s_base[1] + s_warp1[warp] + __popc(m1 & lanemask_lt());
    __syncthreads();  // the scratch is reused by the next claim
}
// Adds per-thread counts (traversal statistics) into a global counter with one atomic per warp;
// called where every lane of the warp is present.
NGI_D void warp_sum_add(unsigned long long* counter, uint32_t v) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
    if (lane_id() == 0 && x) atomicAdd(counter, x);
}

// Event counts of a logic kernel's block (slots in flight, samples started, film
// contributions), kept in shared memory and added to the wave's counters once when the block
// ends. Measured and not kept: one set per warp flushed without the block barrier (2039 vs
// 2043 Mrays/s on the terrain, 3881 vs 4093 on the Cornell box), one out-of-line copy of the
// random number generator instead of six inlined (2025 / 3813) and an out-of-line next-event
// estimation (1837 / 3816), both tried against the instruction-cache stalls ncu reports.
constexpr int kLogicBlock = 256;  // threads per block of every logic kernel
struct BlockCounts {
    unsigned int active, camera, contrib, nonfinite;
};
#define NGI_COUNTS_DECL __shared__ BlockCounts bc;
NGI_D void block_counts_init(BlockCounts& b) {
    if (threadIdx.x == 0) b = BlockCounts{0u, 0u, 0u, 0u};
    __syncthreads();
}
// warp vote, one shared-memory add per warp (all lanes of the warp present)
NGI_D void block_count_warp(unsigned int* c, bool flag) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, flag);
    if (lane_id() == 0 && m) atomicAdd(c, (unsigned)__popc(m));
}
NGI_D void block_counts_flush(const BlockCounts& b, WaveCounters* ctr) {
    __syncthreads();
    if (threadIdx.x == 0) {
        if (b.active) atomicAdd(&ctr->active, (int)b.active);
        if (b.camera) atomicAdd(&ctr->stat_camera, (unsigned long long)b.camera);
        if (b.contrib) atomicAdd(&ctr->stat_contrib, (unsigned long long)b.contrib);
        if (b.nonfinite) atomicAdd(&ctr->stat_nonfinite, (unsigned long long)b.nonfinite);
    }
}

template <typename R>
NGI_D bool finite3(V3<R> c) { return isfinite(c.x) && isfinite(c.y) && isfinite(c.z); }

template <typename R>
NGI_D void film_add(double* film, uint32_t pixel, V3<R> c) {
    double* f = film + 3 * (size_t)pixel;
    atomicAdd(f + 0, (double)c.x);
    atomicAdd(f + 1, (double)c.y);
    atomicAdd(f + 2, (double)c.z);
}

// A pending shadow ray held in registers until the warp appends it.
template <typename R>
struct ShadowRay {
    bool valid;
    float ox, oy, oz, dx, dy, dz, tmin, tmax;
    V3<R> c;
    uint32_t pixel;
    int light_prim;  // adjoint: primitive whose Le scales the contribution
};

// Ray origins. REFERENCE: the surface point itself with the reference's absolute
// tmin = EpsF (Scene::Intersect / Visible, rt.hpp:2248, 2260). SCALED: tmin = 0 and the point
// moves off its surface, to the side the ray leaves by, by 2^-17 of the largest |coordinate|
// of the surface triangle. Hit points are affine combinations of that triangle's vertices, so
// their distance from its plane is a few ulps of that magnitude, and so is the error of a
// later plane test against them; 2^-17 is 64..128 such ulps. The offset follows the local
// geometry, not the scene, so millimetre triangles near the origin and kilometre walls both
// stay clear of self-intersection. Shadow rays move both ends and run between the moved
// points, stopping 2^-16 of their length short of the target.
constexpr float kOffsetScale = 1.0f / 131072.0f;
constexpr float kShadowShrink = 1.0f / 65536.0f;

// g moved off its surface toward direction `toward` (unchanged off surfaces).
template <typename R>
NGI_D V3<R> offset_point(const Geom<R>& g, V3<R> toward) {
    if (g.degenerated || !(g.ext > 0.0f)) return g.p;
    const R delta = (R)(g.ext * kOffsetScale);
    return g.p + g.gn * (dot(g.gn, toward) >= R(0) ? delta : -delta);
}

// Scene::Visible (rt.hpp:2251-2261): the shadow ray from surface point a to b.
template <typename R>
NGI_D void shadow_segment(const Geom<R>& a, const Geom<R>& b, int mode, ShadowRay<R>& out) {
    out.valid = true;
    if (mode == NGI_RAY_OFFSET_SCALED) {
        const V3<R> pa = offset_point(a, b.p - a.p);
        const V3<R> pb = offset_point(b, a.p - b.p);
        out.ox = (float)pa.x; out.oy = (float)pa.y; out.oz = (float)pa.z;
        const V3<R> d = pb - v3<R>((R)out.ox, (R)out.oy, (R)out.oz);
        const R len = sqrt_(dot(d, d));
        const V3<R> dn = d / len;
        out.dx = (float)dn.x; out.dy = (float)dn.y; out.dz = (float)dn.z;
        out.tmin = 0.0f;
        out.tmax = (float)len * (1.0f - kShadowShrink);
    } else {
        const V3<R> d = b.p - a.p;
        const R len = sqrt_(dot(d, d));
        const V3<R> dn = d / len;
        out.ox = (float)a.p.x; out.oy = (float)a.p.y; out.oz = (float)a.p.z;
        out.dx = (float)dn.x; out.dy = (float)dn.y; out.dz = (float)dn.z;
        out.tmin = kEpsF;
        out.tmax = (float)len * (1.0f - kEpsF);
    }
}

template <typename R>
NGI_D float4 ray_origin(const Geom<R>& g, V3<R> d, int mode) {
    if (mode != NGI_RAY_OFFSET_SCALED) return make_float4((float)g.p.x, (float)g.p.y, (float)g.p.z, kEpsF);
    const V3<R> o = offset_point(g, d);
    return make_float4((float)o.x, (float)o.y, (float)o.z, 0.0f);
}


// Primitive id k of a path prefix held in two uint4 (16 x uint16).
NGI_D uint32_t prefix_get(const uint4& a, const uint4& b, int k) {
    const uint4& q = k < 8 ? a : b;
    const int j = (k & 7) >> 1;
    const uint32_t word = j == 0 ? q.x : (j == 1 ? q.y : (j == 2 ? q.z : q.w));
    return (k & 1) ? (word >> 16) : (word & 0xFFFFu);
}
NGI_D void prefix_set(uint4& a, uint4& b, int k, uint32_t prim) {
    uint4& q = k < 8 ? a : b;
    const int j = (k & 7) >> 1;
    uint32_t& word = j == 0 ? q.x : (j == 1 ? q.y : (j == 2 ? q.z : q.w));
    word = (k & 1) ? ((word & 0x0000FFFFu) | (prim << 16)) : ((word & 0xFFFF0000u) | (prim & 0xFFFFu));
}

// Path-replay gradient of one film contribution C at `pixel` (Vicini, Speierer, Jakob 2021):
// every sampling decision of pt/ptdirect is independent of the albedo R and the emission Le,
// and C is a product holding R of each surface vertex on its path (the prefix, plus the
// NEE vertex) and one Le, so dC/dR_m = C * n_m / R_m and dC/dLe = C / Le, channel by channel.
//
// The sums go to a per-block shared-memory accumulator when the scene is small enough
// (smem != null: 6 floats per primitive, albedo then emission), flushed once per block by
// adj_flush; otherwise straight to the FP64 global gradients.
template <typename R>
NGI_D void adj_accumulate(const WaveView<R>& w, const SceneView<R>& sv, uint32_t pixel, V3<R> C, const uint4& pa,
                          const uint4& pb, int count, int vertex_prim, int light_prim, float* smem, int num_prims) {
    const double* a = w.adj + 3 * (size_t)pixel;
    const double wc[3] = {a[0] * (double)C.x, a[1] * (double)C.y, a[2] * (double)C.z};
    if (wc[0] == 0.0 && wc[1] == 0.0 && wc[2] == 0.0) return;
    auto add = [&](int index, double v) {
        if (smem) atomicAdd(smem + index, (float)v);
        else atomicAdd(index < 3 * num_prims ? w.grad_albedo + index : w.grad_emission + (index - 3 * num_prims), v);
    };
    auto add_albedo = [&](int m) {
        const V3<R> r = sv.mats[m].R_;
        const double rc[3] = {(double)r.x, (double)r.y, (double)r.z};
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (rc[c] != 0.0) add(3 * m + c, wc[c] / rc[c]);
    };
    for (int k = 0; k < count; k++) add_albedo((int)prefix_get(pa, pb, k));
    if (vertex_prim >= 0) add_albedo(vertex_prim);
    if (light_prim >= 0) {
        const V3<R> le = sv.mats[light_prim].Le;
        const double lc[3] = {(double)le.x, (double)le.y, (double)le.z};
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (lc[c] != 0.0) add(3 * num_prims + 3 * light_prim + c, wc[c] / lc[c]);
    }
}

// Largest scene (primitives) whose gradients fit the per-block shared-memory accumulator.
constexpr int kAdjSmemPrims = 1024;

NGI_D void adj_smem_clear(float* smem, int num_prims) {
    if (!smem) return;
    for (int i = threadIdx.x; i < 6 * num_prims; i += blockDim.x) smem[i] = 0.0f;
    __syncthreads();
}
template <typename R>
NGI_D void adj_flush(const WaveView<R>& w, float* smem, int num_prims) {
    if (!smem) return;
    __syncthreads();
    for (int i = threadIdx.x; i < 6 * num_prims; i += blockDim.x) {
        const float v = smem[i];
        if (v != 0.0f)
            atomicAdd(i < 3 * num_prims ? w.grad_albedo + i : w.grad_emission + (i - 3 * num_prims), (double)v);
    }
}

// Appends a pending shadow ray to the wave's shadow queue, with its batch job and, for the
// adjoint, the path prefix it scales (count surface vertices of pa/pb, plus vprim, the vertex
// the connection starts from; -1 at the sensor). Called by every lane of the group executing
// it, straight after the next-event estimation, so the ray's registers are free again before
// the BSDF sampling that follows.
template <typename R, bool ADJ, bool BATCH>
NGI_D void emit_shadow(const WaveView<R>& w, const ShadowRay<R>& sr, int job, const uint4& pa, const uint4& pb,
                       int count, int vprim) {
    const int q = coalesced_append(&w.ctr->sh_count, sr.valid);
    if (!sr.valid) return;
    __stcs(w.sh_o + q, make_float4(sr.ox, sr.oy, sr.oz, sr.tmin));
    __stcs(w.sh_d + q, make_float4(sr.dx, sr.dy, sr.dz, sr.tmax));
    st_stream(w.sh_c + q, Vec4T<R>{sr.c.x, sr.c.y, sr.c.z, R(0)});
    __stcs(w.sh_pix + q, sr.pixel);
    if (BATCH) w.sh_job[q] = job;
    if (ADJ) {
        if (count > 0) {
            w.sh_pre[2 * (size_t)q] = pa;
            w.sh_pre[2 * (size_t)q + 1] = pb;
        }
        w.sh_info[q] = make_int2(count | ((vprim + 1) << 8), sr.light_prim);
    }
}

// The shading kernel stages its shadow rays in shared memory instead: one entry per thread and
// item, claimed in the global shadow queue with the block's other claims (one atomic per block).
template <typename R>
struct StagedShadow {  // float4 members: 16-byte aligned (32 with a double colour)
    float4 o, d;
    Vec4T<R> c;
    uint32_t pixel;
};
template <typename R>
NGI_D StagedShadow<R>* shadow_stage() {
    __shared__ StagedShadow<R> stage[kLogicBlock];
    return stage;
}
template <typename R>
NGI_D void stage_shadow(const ShadowRay<R>& sr, StagedShadow<R>* stage, int* count) {
    if (!sr.valid) return;
    const int i = atomicAdd(count, 1);  // shared memory: at most one ray per thread and item
    stage[i].o = make_float4(sr.ox, sr.oy, sr.oz, sr.tmin);
    stage[i].d = make_float4(sr.dx, sr.dy, sr.dz, sr.tmax);
    stage[i].c = Vec4T<R>{sr.c.x, sr.c.y, sr.c.z, R(0)};
    stage[i].pixel = sr.pixel;
}

// Next-event estimation at a vertex (src/nanogi.cpp:654-707).
template <typename R>
NGI_D void next_event(const SceneView<R>& sv, const RenderConsts& rc, const Geom<R>& g, bool at_sensor,
                      const DevMaterial<R>* mat, V3<R> wi, V3<R> thr, uint32_t pixel, float4 u, ShadowRay<R>& out) {
    out.valid = false;
    const int nl = sv.num_lights;
    int li = (int)((R)u.x * (R)nl);
    li = li < 0 ? 0 : (li > nl - 1 ? nl - 1 : li);
    const DevLight<R>& L = sv.lights[li];
    if (L.type == LT_DIRECTIONAL) return;  // Le is 0 without forceDegenerated (rt.hpp:934-937)
    if (at_sensor && !L.sensor_facing) return;  // every point of L faces away from the pinhole eye
    Geom<R> gl;
    R pdf_pos;
    if (L.type == LT_AREA) {
        sample_mesh_position(sv, L.tri_base, L.tri_count, L.cdf_offset, (R)u.y, (R)u.z, gl);
        pdf_pos = L.inv_area;
    } else {
        gl.p = L.position;
        gl.degenerated = true;
        gl.ext = 0.0f;
        pdf_pos = R(1);
    }
    const V3<R> ppl = normalize(gl.p - g.p);
    V3<R> fs_e;
    if (at_sensor) {
        if (sv.sensor.type == ET_PINHOLE) {
            const R w = pinhole_importance(sv.sensor, ppl);
            fs_e = v3<R>(w, w, w);
        } else {
            fs_e = dot(g.sn, ppl) > R(0) ? sv.sensor.We : v3<R>(0, 0, 0);
        }
    } else {
        fs_e = bsdf_eval(*mat, material_albedo(sv, *mat, g), g, wi, ppl, false);
    }
    if (is_zero(fs_e)) return;
    V3<R> fs_l = L.Le;
    if (L.type == LT_AREA && !(dot(gl.sn, -ppl) > R(0))) return;
    const R G = geometry_term(g, gl);
    const R pdf_l = R(1) / (R)nl;
    const V3<R> C = thr * fs_e * G * fs_l / pdf_l / pdf_pos;
    if (is_zero(C)) return;
    uint32_t pix = pixel;
    if (at_sensor) {
        R rx, ry;
        if (sv.sensor.type == ET_PINHOLE) {
            pinhole_raster(sv.sensor, ppl, rx, ry);
        } else {
            rx = g.uvx; ry = g.uvy;
        }
        pix = (uint32_t)pixel_index(rx, ry, rc.width, rc.height);
    }
    shadow_segment(g, gl, rc.ray_offset, out);
    out.c = C;
    out.pixel = pix;
    out.light_prim = L.prim;
}

template <typename R>
NGI_D void store_ray(const WaveView<R>& w, int s, const Geom<R>& g, V3<R> d, int mode) {
    const V3<R> o = g.p;
    const float4 ro = ray_origin(g, d, mode);
    __stcs(w.ray_o + s, ro);
    __stcs(w.ray_d + s, make_float4((float)d.x, (float)d.y, (float)d.z, kInfF));
    if (sizeof(R) == 8) {
        // the hit point is reconstructed from the origin the ray was traced from
        if (mode == NGI_RAY_OFFSET_SCALED) w.od_o[s] = Vec4T<double>{(double)ro.x, (double)ro.y, (double)ro.z, 0.0};
        else w.od_o[s] = Vec4T<double>{(double)o.x, (double)o.y, (double)o.z, 0.0};
        w.od_d[s] = Vec4T<double>{(double)d.x, (double)d.y, (double)d.z, 0.0};
    }
}

// BATCH: every slot belongs to one job of a batch; its scene, parameters, film and renderer
// come from the device job table (one persistent wave serves every job).
// Hit reconstruction (Scene::Intersect rt.hpp:2196-2233): the surface geometry where the ray
// of slot s hit triangle h.w at distance h.x with barycentrics (h.y, h.z), the ray direction,
// and the primitive hit. Scaled ray offsets place the point on the triangle (barycentric),
// the reference mode at o + t d. Texture coordinates only when `with_uv` is set.
template <typename R>
NGI_D int hit_geometry(const SceneView<R>& sv, const RenderConsts& rc, const WaveView<R>& w, int s, float4 h, V3<R>& d,
                       Geom<R>& g, bool with_uv) {
    const int ti = __float_as_int(h.w);
    V3<R> o;
    if (sizeof(R) == 8) {
        const Vec4T<double> a = w.od_o[s], b = w.od_d[s];
        o = v3<R>((R)a.x, (R)a.y, (R)a.z);
        d = v3<R>((R)b.x, (R)b.y, (R)b.z);
    } else {
        const float4 a = __ldcs(w.ray_o + s), b = __ldcs(w.ray_d + s);
        o = v3<R>((R)a.x, (R)a.y, (R)a.z);
        d = v3<R>((R)b.x, (R)b.y, (R)b.z);
    }
    const float4* tp = sv.tris + 3 * (size_t)ti;
    const float4 q1 = tp[0], q2 = tp[1], q3 = tp[2];
    const V3<R> p1 = v3<R>(q1.x, q1.y, q1.z), p2 = v3<R>(q2.x, q2.y, q2.z), p3 = v3<R>(q3.x, q3.y, q3.z);
    g.gn = normalize(cross(p2 - p1, p3 - p1));
    const float4* np = sv.nrm + 3 * (size_t)ti;
    const float4 m1 = np[0], m2 = np[1], m3 = np[2];
    const float bw = 1.0f - h.y - h.z;
    if (rc.ray_offset == NGI_RAY_OFFSET_SCALED) {
        // on the triangle itself, whatever the distance travelled
        g.p = p1 * (R)bw + p2 * (R)h.y + p3 * (R)h.z;
        g.ext = max_abs3(p1, p2, p3);
    } else {
        g.p = o + d * (R)h.x;
        g.ext = 0.0f;
    }
    g.sn = normalize(v3<R>(m1.x, m1.y, m1.z) * (R)bw + v3<R>(m2.x, m2.y, m2.z) * (R)h.y +
                     v3<R>(m3.x, m3.y, m3.z) * (R)h.z);
    if (isnan_(g.sn.x) || isnan_(g.sn.y) || isnan_(g.sn.z)) g.sn = g.gn;
    g.degenerated = false;
    if (with_uv || sv.num_textures > 0) {
        const float2* up = sv.uv + 3 * (size_t)ti;
        const float2 t1 = up[0], t2 = up[1], t3 = up[2];
        g.uvx = (R)t1.x * (R)bw + (R)t2.x * (R)h.y + (R)t3.x * (R)h.z;
        g.uvy = (R)t1.y * (R)bw + (R)t2.y * (R)h.y + (R)t3.y * (R)h.z;
    } else {
        g.uvx = R(0);
        g.uvy = R(0);
    }
    return __float_as_int(m1.w);
}

// ptdirect scores only through next-event estimation, which a vertex does after it survives
// Russian roulette (src/nanogi.cpp:646-785: NEE at the loop top, the roulette right after the
// intersection); ltdirect likewise only through its sensor connections (src/nanogi.cpp:955-1130). The roulette variable of the next hit is the .w of the Philox call this vertex
// already drew for its own next-event estimation, so a path that the roulette -- or the length
// limit -- ends at its next hit gains nothing from that hit: its extension ray is not traced.
// The film is the same, sample for sample; fewer rays are traced per sample (terrain: 0.93
// instead of 1.62, 1784 instead of 1294 Msamples/s). NGI_RENDER_TRACE_ALL_RAYS traces them all.
NGI_D bool next_hit_is_dead(const RenderConsts& rc, float next_rr, int nv) {
    if (rc.trace_all) return false;
    return next_rr > 0.5f || (rc.max_vertices != -1 && nv + 1 >= rc.max_vertices);
}

// One path vertex of pt / ptdirect at the hit h of slot s's extension ray (src/nanogi.cpp:557-603
// and 646-799): emission on a light hit (pt), Russian roulette, next-event estimation (ptdirect; its
// shadow ray goes to emit(ray, prefix length, vertex primitive) at once, so that it holds no registers
// during the BSDF sampling), the BSDF sample, and the continuation ray stored in the slot. Returns true
// when the path continues. The adjoint's surface-vertex prefix is pa / pb.
template <typename R, bool ADJ, typename Emit>
NGI_D bool shade_vertex(const SceneView<R>& sv, const RenderConsts& rc, double* film, bool direct,
                        const WaveView<R>& w, int s, float4 h, uint4& pa, uint4& pb, float* gsm, BlockCounts& bc,
                        Emit&& emit) {
    V3<R> d;
    Geom<R> g;
    const int prim = hit_geometry(sv, rc, w, s, h, d, g, false);
    const Vec4T<R> t4 = w.thr[s];
    V3<R> thr = v3<R>(t4.x, t4.y, t4.z);
    const uint32_t pixel = w.pixel[s];
    const unsigned long long sample = w.sample[s];
    int nv = w.nverts[s];
    const RngKey rk = make_rng(rc.seed, sample);

    const DevMaterial<R>& mat = sv.mats[prim];
    if (ADJ) {
        pa = w.pre[2 * (size_t)s];
        pb = w.pre[2 * (size_t)s + 1];
    }

    if (!direct && (mat.type & DT_L) && mat.l_type == LT_AREA) {
        // Emission on a light hit (src/nanogi.cpp:568-575)
        if (dot(g.sn, -d) > R(0)) {
            const V3<R> c = thr * mat.Le;
            if (!is_zero(c)) {
                if (finite3(c)) {
                    film_add(film, pixel, c);
                    atomicAdd(&bc.contrib, 1u);
                    if (ADJ) adj_accumulate(w, sv, pixel, c, pa, pb, nv - 1, -1, prim, gsm, rc.num_prims);
                } else {
                    atomicAdd(&bc.nonfinite, 1u);
                }
            }
        }
    }
    // Russian roulette after every hit (src/nanogi.cpp:583-591)
    const float rr = rng4(rk, (uint32_t)nv, RNG_NEE_RR).w;
    if (rr > 0.5f) return false;
    thr = thr / R(0.5);
    nv++;
    if ((rc.max_vertices != -1 && nv >= rc.max_vertices) || mat.bsdf == BSDF_NONE) return false;
    tangent_space(g);
    const V3<R> wi = -d;
    bool dead = false;
    if (direct) {
        const float4 un = rng4(rk, (uint32_t)nv, RNG_NEE_RR);
        ShadowRay<R> sa;
        next_event(sv, rc, g, false, &mat, wi, thr, pixel, un, sa);
        emit(sa, nv - 2, prim);
        dead = next_hit_is_dead(rc, un.w, nv);
    }
    const float4 ud = rng4(rk, (uint32_t)nv, RNG_DIR);
    V3<R> wo, wgt;
    if (dead || !bsdf_sample_weight(mat, material_albedo(sv, mat, g), g, wi, (R)ud.x, (R)ud.y, (R)ud.z, wo, wgt))
        return false;
    thr = thr * wgt;
    if (ADJ) {
        if (nv - 2 >= kAdjMaxPrefix) {
            atomicOr(&w.ctr->error_flags, 2);
        } else {
            prefix_set(pa, pb, nv - 2, (uint32_t)prim);
            w.pre[2 * (size_t)s] = pa;
            w.pre[2 * (size_t)s + 1] = pb;
        }
    }
    store_ray(w, s, g, wo, rc.ray_offset);
    w.thr[s] = Vec4T<R>{thr.x, thr.y, thr.z, R(0)};
    w.nverts[s] = nv;
    return true;
}

// PART: kLogicFused does both halves of an iteration in one kernel; kLogicShadeQ consumes the
// hits, does next-event estimation and continues the paths, handing the slots whose path ended to
// kLogicRegen, which starts new samples in them (two kernels of half the code each: the fused
// kernel stalls on instruction fetch). ptdirect runs split (terrain 2091 vs 2059 Mrays/s fused);
// pt, with no next-event estimation to separate, stays fused (Cornell box 4038 vs 3640 split).
// The shading half reads its slots from queues (the slots whose extension ray hit something, and
// the slots regeneration left empty) instead of scanning every slot of the wave: terrain 1950
// against 1830 Msamples/s, the 10M-triangle interior 334 against 308.
constexpr int kLogicFused = 0, kLogicRegen = 2, kLogicShadeQ = 3;
constexpr int kRegenAttempts = 2;  // samples a slot may claim per iteration
// Shadow-queue entries per path slot and iteration: one next-event estimation at the slot's
// vertex plus one sensor connection per sample claimed (bdpt: two connections).
constexpr size_t kShadowPerSlot = 1 + (kRegenAttempts > 1 ? kRegenAttempts : 1);
// Resident blocks per SM the two ptdirect halves are compiled for (64 registers each). 5 or 6
// blocks (48 / 40 registers) were slower on the terrain: 2066-2083 against 2103 Mrays/s.
// (3 blocks for the shading kernel, about 85 registers and fewer spills with the fast FP32 division:
// 13.83 against 13.55 ms per 16-spp terrain render)
constexpr int kShadeMinBlocks = 4, kRegenMinBlocks = 4;
// Measured and not kept: sorting each block's 256 items by class (BSDF of the hit primitive,
// miss, empty slot) in shared memory before shading: 1798-1802 against 1803-1804 Mrays/s on the
// terrain, the logic's share of GPU time unchanged at 36%. The shading warps do not diverge on
// the material type.

template <typename R, bool DIRECT, bool ADJ, bool BATCH = false, int PART = kLogicFused>
__global__ void __launch_bounds__(256, PART == kLogicFused    ? kLogicMinBlocks
                                       : PART == kLogicShadeQ ? kShadeMinBlocks
                                                              : kRegenMinBlocks) k_logic(SceneView<R> sv0, WaveView<R> w, RenderConsts rc0,
                                               const JobView<R>* __restrict__ jobs, int num_jobs) {
    extern __shared__ float adj_smem[];
    float* gsm = (ADJ && !DIRECT && rc0.num_prims <= kAdjSmemPrims) ? adj_smem : nullptr;
    if (ADJ && !DIRECT) adj_smem_clear(gsm, rc0.num_prims);
    // block-wide claims (block_claim). All of a block's threads run the
    // same item iterations, so they all reach every claim. Measured on the 1.55M-triangle terrain
    // against one atomic per warp: 1939 against 1805 Mrays/s, the logic kernels' time per iteration
    // 0.276 against 0.338 ms (regeneration alone: 1872 and 0.307 ms). The warps of a wave's logic
    // kernels all claim from the same few counters, and those returning atomics queue at one L2 slice.
    __shared__ int s_warp[kLogicBlock / 32], s_warp2[kLogicBlock / 32];
    __shared__ unsigned long long s_base64;
    __shared__ int s_base32, s_base32b, s_base2[2];
    // shading: shadow rays staged in shared memory this item, and their claimed queue range
    __shared__ int s_staged, s_staged_n, s_staged_base;
    if (threadIdx.x == 0) s_staged = 0;  // the first barrier below comes before any staging
    const int stride = gridDim.x * blockDim.x;
    NGI_COUNTS_DECL
    block_counts_init(bc);
    // kLogicRegen walks the queue of ended paths, kLogicShadeQ the previous iteration's extension
    // queue followed by the slots regeneration left empty, the others every slot (Q is a multiple
    // of the block size). n_items is the same for every thread of a block, so all of them run the
    // same iterations.
    // (every queue holds at most one entry per slot; the clamps only keep a corrupted count in bounds)
    const int n_ext_in = PART == kLogicShadeQ ? min(*w.ext_in_count, w.Q) : 0;
    const int n_items = PART == kLogicRegen    ? min(w.ctr->regen_count, w.Q)
                        : PART == kLogicShadeQ ? n_ext_in + min(*w.carry_in_count, w.Q - n_ext_in)
                                               : w.Q;
    for (int base = blockIdx.x * blockDim.x; base < n_items; base += stride) {
        const int item = base + (int)threadIdx.x;
        const bool valid = item < n_items;  // false only past the end of a queue
        int s = item;
        uint8_t st;
        if (PART == kLogicRegen) {
            s = valid ? w.regen_queue[item] : 0;
            st = SLOT_EMPTY;
        } else if (PART == kLogicShadeQ) {
            s = !valid ? 0 : (item < n_ext_in ? w.ext_in[item] : w.carry_in[item - n_ext_in]);
            st = !valid ? (uint8_t)SLOT_DONE : (item < n_ext_in ? (uint8_t)SLOT_ACTIVE : (uint8_t)SLOT_EMPTY);
        } else {
            st = w.state[s];
        }
        bool need_new = valid && st == SLOT_EMPTY;
        bool want_ext = false;
        uint4 pa = make_uint4(0u, 0u, 0u, 0u), pb = pa;  // adjoint: surface-vertex prefix of the path

        if (PART != kLogicRegen && st == SLOT_ACTIVE) {
            // ---- consume the extension hit (src/nanogi.cpp:557-603 / 767-799) ----
            bool alive = false;
            const float4 h = __ldcs(w.hit + s);
            if (__float_as_int(h.w) >= 0) {
                const int job = BATCH ? w.job[s] : 0;
                const SceneView<R>& sv = BATCH ? jobs[job].sv : sv0;
                const RenderConsts& rc = BATCH ? jobs[job].rc : rc0;
                double* const film = BATCH ? jobs[job].film : w.film;
                const bool direct = BATCH ? rc.renderer == NGI_RENDERER_PTDIRECT : DIRECT;
                alive = shade_vertex<R, ADJ>(sv, rc, film, direct, w, s, h, pa, pb, gsm, bc,
                                             [&](const ShadowRay<R>& sa, int count, int vprim) {
                                                 if constexpr (PART == kLogicShadeQ && !ADJ)
                                                     stage_shadow(sa, shadow_stage<R>(), &s_staged);
                                                 else
                                                     emit_shadow<R, ADJ, BATCH>(w, sa, job, pa, pb, count, vprim);
                                             });
                want_ext = alive;
            }
            if (!alive) need_new = true;
        }

        if constexpr (PART == kLogicShadeQ) {
            // ---- hand the slots whose path ended to the regeneration kernel, queue the continuing
            // paths' rays and the staged shadow rays: one atomic per queue for the whole block ----
            // (the slot state array is not written: compacted shading knows a slot's state from the
            // queue it comes from, and only the fused kernel reads the array)
            if (!want_ext && st == SLOT_ACTIVE) st = SLOT_EMPTY;
            if (want_ext) st = SLOT_ACTIVE;
            // ended paths go to regeneration unless the wave holds every sample (nothing regenerates then)
            const bool to_regen = need_new && !rc0.one_pass;
            const unsigned mr = __ballot_sync(0xFFFFFFFFu, to_regen), me = __ballot_sync(0xFFFFFFFFu, want_ext);
            const int warp = (int)(threadIdx.x >> 5);
            if (lane_id() == 0) {
                s_warp[warp] = __popc(mr);
                s_warp2[warp] = __popc(me);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int tr = 0, te = 0;
                for (int k = 0; k < kLogicBlock / 32; k++) {
                    const int cr = s_warp[k], ce = s_warp2[k];
                    s_warp[k] = tr;
                    s_warp2[k] = te;
                    tr += cr;
                    te += ce;
                }
                s_base32 = tr ? atomicAdd(&w.ctr->regen_count, tr) : 0;
                s_base32b = te ? atomicAdd(w.ext_count, te) : 0;
                if constexpr (!ADJ) {
                    s_staged_n = s_staged;
                    s_staged_base = s_staged ? atomicAdd(&w.ctr->sh_count, s_staged) : 0;
                    s_staged = 0;  // every thread has staged this item's ray (it passed the barrier above)
                }
            }
            __syncthreads();
            if (to_regen) w.regen_queue[s_base32 + s_warp[warp] + __popc(mr & lanemask_lt())] = s;
            if (want_ext) w.ext_queue[s_base32b + s_warp2[warp] + __popc(me & lanemask_lt())] = s;
            if constexpr (!ADJ) {
                const StagedShadow<R>* stage = shadow_stage<R>();
                for (int t = (int)threadIdx.x; t < s_staged_n; t += kLogicBlock) {
                    const int q = s_staged_base + t;
                    __stcs(w.sh_o + q, stage[t].o);
                    __stcs(w.sh_d + q, stage[t].d);
                    st_stream(w.sh_c + q, stage[t].c);
                    __stcs(w.sh_pix + q, stage[t].pixel);
                }
            }
            __syncthreads();  // the scratch and the stage are reused by the next item
            block_count_warp(&bc.active, st != SLOT_DONE && !need_new);  // the others: counted by regeneration
        } else {
            // ---- claim a new sample for finished slots (path regeneration) ----
            // A claimed sample whose camera ray is not traced (its first hit is dead, or the ray leaves
            // the raster) leaves the slot empty; the slot then claims the next sample, up to
            // kRegenAttempts samples per iteration (each may add its sensor connection to the shadow
            // queue). Terrain, ptdirect: 1 attempt 1776, 2 attempts 1833, 3 attempts 1824 Msamples/s.
            for (int attempt = 0; attempt < kRegenAttempts; attempt++) {
                {
                    // one atomic per block on the sample counter every slot of the wave claims from; a
                    // wave that holds every sample gives the slot at queue position i (slot i of the
                    // identity queue it starts from) sample i instead (block-uniform branch)
                    const unsigned long long k = rc0.one_pass
                                                     ? (unsigned long long)item
                                                     : block_claim(&w.ctr->next_sample, need_new, s_warp, &s_base64);
                    if (need_new) {
                        int job = 0;
                        unsigned long long local = k;
                        if (BATCH && k < (unsigned long long)rc0.num_samples) {
                            // job of batch sample k: last job whose first sample is <= k
                            int lo = 0, hi = num_jobs - 1;
                            while (lo < hi) {
                                const int mid = (lo + hi + 1) >> 1;
                                if ((unsigned long long)jobs[mid].sample_base <= k) lo = mid; else hi = mid - 1;
                            }
                            job = lo;
                            local = k - (unsigned long long)jobs[job].sample_base;
                        }
                        const SceneView<R>& sv = BATCH ? jobs[job].sv : sv0;
                        const RenderConsts& rc = BATCH ? jobs[job].rc : rc0;
                        const bool direct = BATCH ? rc.renderer == NGI_RENDERER_PTDIRECT : DIRECT;
                        if (k >= (unsigned long long)rc0.num_samples) {
                            st = SLOT_DONE;
                        } else if (rc.max_vertices == 1) {
                            // the loop's first test ends the path before the sensor vertex does anything
                            // (src/nanogi.cpp:485, 647): the sample counts, nothing is traced
                            st = SLOT_EMPTY;
                        } else {
                            // ---- sensor vertex (src/nanogi.cpp:450-479, 609-641) ----
                            const unsigned long long gsample = (unsigned long long)rc.sample_offset + local;
                            const RngKey rk = make_rng(rc.seed, gsample);
                            Geom<R> ge;
                            V3<R> thr;
                            const DevSensor<R>& cam = sv.sensor;
                            bool ok = true;
                            if (cam.type == ET_PINHOLE) {
                                ge.p = cam.eye;
                                ge.degenerated = true;
                                ge.ext = 0.0f;
                                ge.sn = ge.gn = ge.du = ge.dv = v3<R>(0, 0, 0);
                                ge.uvx = ge.uvy = R(0);
                                thr = v3<R>(1, 1, 1);
                            } else {
                                const float4 us = rng4(rk, 1u, RNG_SENSOR);
                                sample_mesh_position(sv, cam.tri_base, cam.tri_count, cam.cdf_offset, (R)us.x, (R)us.y,
                                                     ge);
                                const R a = R(1) / cam.inv_area;
                                thr = v3<R>(a, a, a);
                            }
                            if (direct) {
                                const float4 un = rng4(rk, 1u, RNG_NEE_RR);
                                ShadowRay<R> sb;
                                next_event(sv, rc, ge, true, (const DevMaterial<R>*)nullptr, v3<R>(0, 0, 0), thr, 0u,
                                           un, sb);
                                // sensor vertex: no surface factors for the adjoint
                                emit_shadow<R, ADJ, BATCH>(w, sb, job, pa, pb, 0, -1);
                                if (next_hit_is_dead(rc, un.w, 1)) ok = false;  // the sample ends at the sensor vertex
                            }
                            const float4 ud = rng4(rk, 1u, RNG_DIR);
                            V3<R> wo;
                            uint32_t pix = 0;
                            if (cam.type == ET_PINHOLE) {
                                R rx, ry;
                                if (rc.stratified && (long long)gsample < rc.strat_end) {
                                    // 32-bit division where the sample index fits (a film has fewer
                                    // than 2^31 pixels); 64-bit division is far slower on the GPU
                                    const uint32_t wh = (uint32_t)rc.width * (uint32_t)rc.height;
                                    const uint32_t pidx = (gsample >> 32) == 0ull
                                                              ? (uint32_t)gsample % wh
                                                              : (uint32_t)(gsample % (unsigned long long)wh);
                                    const int px = (int)(pidx % (uint32_t)rc.width);
                                    const int py = (int)(pidx / (uint32_t)rc.width);
                                    rx = ((R)px + (R)ud.x) / (R)rc.width;
                                    ry = ((R)py + (R)ud.y) / (R)rc.height;
                                } else {
                                    rx = (R)ud.x;
                                    ry = (R)ud.y;
                                }
                                wo = pinhole_direction(cam, rx, ry);
                                R qx, qy;
                                if (!pinhole_raster(cam, wo, qx, qy)) ok = false;
                                else {
                                    pix = (uint32_t)pixel_index(qx, qy, rc.width, rc.height);
                                    const R W = pinhole_importance(cam, wo);
                                    if (W == R(0)) ok = false;
                                    else thr = thr * (W / W);
                                }
                            } else {
                                const V3<R> l = cosine_hemisphere((R)ud.x, (R)ud.y);
                                wo = to_world(ge, l);
                                pix = (uint32_t)pixel_index(ge.uvx, ge.uvy, rc.width, rc.height);
                                const V3<R> lw = to_local(ge, wo);
                                if (!(lw.z > R(0)) || is_zero(cam.We)) ok = false;
                                else thr = thr * cam.We / kInvPi_<R>();
                            }
                            if (ok) {
                                store_ray(w, s, ge, wo, rc.ray_offset);
                                w.thr[s] = Vec4T<R>{thr.x, thr.y, thr.z, R(0)};
                                w.pixel[s] = pix;
                                w.sample[s] = gsample;
                                if (BATCH) w.job[s] = job;
                                w.nverts[s] = 1;
                                want_ext = true;
                                st = SLOT_ACTIVE;
                            } else {
                                st = SLOT_EMPTY;
                            }
                        }
                    }
                    block_count_warp(&bc.camera, need_new && st != SLOT_DONE);
                }
                need_new = need_new && st == SLOT_EMPTY;
                // block-uniform (the claims are block-wide); a wave that holds every sample has
                // claimed them all with the first attempts of its slots, so it makes no second one
                if (!__syncthreads_or(need_new) || rc0.one_pass) break;
            }
            if (rc0.one_pass && need_new) st = SLOT_DONE;  // its sample ended at the sensor vertex
            if (!want_ext && st == SLOT_ACTIVE) st = SLOT_EMPTY;
            if (want_ext) st = SLOT_ACTIVE;
            if (PART == kLogicFused && valid) w.state[s] = st;  // read only by the fused kernel
            {
                // compacted shading visits only queued slots: one left empty waits in the carry queue
                const bool carry = PART == kLogicRegen && w.carry_out && valid && st == SLOT_EMPTY;
                int qc, qe;
                block_claim2(w.carry_out_count, carry, w.ext_count, want_ext, qc, qe, s_warp, s_warp2, s_base2);
                if (carry) w.carry_out[qc] = s;
                if (want_ext) w.ext_queue[qe] = s;
            }
            block_count_warp(&bc.active, valid && st != SLOT_DONE);
        }
    }
    block_counts_flush(bc, w.ctr);  // every thread of the block ran the same iterations
    if (ADJ && !DIRECT) adj_flush(w, gsm, rc0.num_prims);
}

// Direct sensor sampling of ltdirect (src/nanogi.cpp:1001-1051): connects vertex g -- a light
// vertex when `light` is set, else a BSDF vertex of material `mat` reached from wi -- to a
// position on the sensor, with the LE BSDF. The contribution is divided by the position pdf
// of the path's light (`light_pos_pdf`), as the reference does (src/nanogi.cpp:1017 passes
// the sampled sensor position to L->EvaluatePositionPDF): ltdirect images are the light
// tracer's estimate scaled by that light's area.
template <typename R>
NGI_D void sensor_connect(const SceneView<R>& sv, const RenderConsts& rc, const Geom<R>& g, const DevLight<R>* light,
                          const DevMaterial<R>* mat, V3<R> wi, V3<R> thr, R light_pos_pdf, float4 un,
                          ShadowRay<R>& out) {
    const DevSensor<R>& cam = sv.sensor;
    Geom<R> ge;
    if (cam.type == ET_PINHOLE) {
        ge.p = cam.eye;
        ge.degenerated = true;
        ge.ext = 0.0f;
        ge.sn = ge.gn = ge.du = ge.dv = v3<R>(0, 0, 0);
        ge.uvx = ge.uvy = R(0);
    } else {
        sample_mesh_position(sv, cam.tri_base, cam.tri_count, cam.cdf_offset, (R)un.y, (R)un.z, ge);
    }
    const V3<R> ppe = normalize(ge.p - g.p);
    V3<R> fs_l;
    if (light) {
        if (light->type == LT_DIRECTIONAL) return;  // Le is 0 without forceDegenerated (rt.hpp:934-937)
        if (light->type == LT_AREA && !(to_local(g, ppe).z > R(0))) return;
        fs_l = light->Le;
    } else {
        fs_l = bsdf_eval(*mat, material_albedo(sv, *mat, g), g, wi, ppe, false, true);
    }
    if (is_zero(fs_l)) return;
    V3<R> fs_e;
    R rx = R(0), ry = R(0);
    if (cam.type == ET_PINHOLE) {
        const R W = pinhole_importance(cam, -ppe);
        if (W == R(0)) return;
        fs_e = v3<R>(W, W, W);
        pinhole_raster(cam, -ppe, rx, ry);
    } else {
        if (!(dot(ge.sn, -ppe) > R(0))) return;
        fs_e = cam.We;
        rx = ge.uvx;
        ry = ge.uvy;
    }
    const R G = geometry_term(g, ge);
    const V3<R> C = thr * fs_l * G * fs_e / light_pos_pdf;
    if (is_zero(C)) return;
    shadow_segment(g, ge, rc.ray_offset, out);
    out.c = C;
    out.pixel = (uint32_t)pixel_index(rx, ry, rc.width, rc.height);
    out.light_prim = -1;
}

// Position pdf of a light with forceDegenerated (rt.hpp:643-664).
template <typename R>
NGI_D R light_position_pdf(const DevLight<R>& L) {
    return L.type == LT_POINT ? R(1) : L.inv_area;
}

// One wavefront step of the light tracers lt / ltdirect (ProcessSample_LT / _LTDirect,
// src/nanogi.cpp:804-1131), the mirror of k_logic: paths start on a light picked uniformly,
// leave it by its emission lobe and continue with LE BSDF sampling. lt scores where an
// extension ray hits an area sensor; ltdirect connects every vertex, the light's own
// included, to the sensor through a shadow ray. Random numbers per (sample, vertex):
// RNG_SENSOR .z light pick, .xy position on it; RNG_NEE_RR .yz sensor position, .w Russian
// roulette; RNG_DIR .xy direction, .z component choice.
template <typename R, bool DIRECT>
__global__ void __launch_bounds__(256) k_logic_lt(SceneView<R> sv, WaveView<R> w, RenderConsts rc) {
    const int stride = gridDim.x * blockDim.x;
    NGI_COUNTS_DECL
    block_counts_init(bc);
    for (int base = blockIdx.x * blockDim.x; base < w.Q; base += stride) {
        const int s = base + (int)threadIdx.x;  // Q is a multiple of the block size
        uint8_t st = w.state[s];
        bool need_new = st == SLOT_EMPTY;
        bool want_ext = false;
        ShadowRay<R> sa;
        sa.valid = false;

        if (st == SLOT_ACTIVE) {
            bool alive = false;
            const float4 h = w.hit[s];
            if (__float_as_int(h.w) >= 0) {
                V3<R> d;
                Geom<R> g;
                const int prim = hit_geometry(sv, rc, w, s, h, d, g, !DIRECT);
                const DevMaterial<R>& mat = sv.mats[prim];
                const Vec4T<R> t4 = w.thr[s];
                V3<R> thr = v3<R>(t4.x, t4.y, t4.z);
                const unsigned long long sample = w.sample[s];
                int nv = w.nverts[s];
                const RngKey rk = make_rng(rc.seed, sample);
                if (!DIRECT && (mat.type & DT_E) && mat.e_type == ET_AREA) {
                    // Hit with the sensor (src/nanogi.cpp:871-896): raster position = uv
                    if (dot(g.sn, -d) > R(0)) {
                        const V3<R> c = thr * mat.We;
                        if (!is_zero(c)) {
                            if (finite3(c)) {
                                film_add(w.film, (uint32_t)pixel_index(g.uvx, g.uvy, rc.width, rc.height), c);
                                atomicAdd(&bc.contrib, 1u);
                            } else {
                                atomicAdd(&bc.nonfinite, 1u);
                            }
                        }
                    }
                }
                // Russian roulette after every hit (src/nanogi.cpp:898-909)
                const float rr = rng4(rk, (uint32_t)nv, RNG_NEE_RR).w;
                if (!(rr > 0.5f)) {
                    thr = thr / R(0.5);
                    nv++;
                    if (!(rc.max_vertices != -1 && nv >= rc.max_vertices) && mat.bsdf != BSDF_NONE) {
                        tangent_space(g);
                        const V3<R> wi = -d;
                        bool dead = false;
                        if (DIRECT) {
                            const float4 un = rng4(rk, (uint32_t)nv, RNG_NEE_RR);
                            const R pdf_pe = light_position_pdf(sv.lights[w.pixel[s]]);
                            sensor_connect(sv, rc, g, (const DevLight<R>*)nullptr, &mat, wi, thr, pdf_pe, un, sa);
                            dead = next_hit_is_dead(rc, un.w, nv);  // ltdirect scores only by connections
                        }
                        const float4 ud = rng4(rk, (uint32_t)nv, RNG_DIR);
                        V3<R> wo, wgt;
                        if (!dead && bsdf_sample_weight(mat, material_albedo(sv, mat, g), g, wi, (R)ud.x, (R)ud.y,
                                                        (R)ud.z, wo, wgt, true)) {
                            thr = thr * wgt;
                            store_ray(w, s, g, wo, rc.ray_offset);
                            w.thr[s] = Vec4T<R>{thr.x, thr.y, thr.z, R(0)};
                            w.nverts[s] = nv;
                            alive = true;
                            want_ext = true;
                        }
                    }
                }
            }
            if (!alive) need_new = true;
        }
        {
            const int q = warp_append(&w.ctr->sh_count, sa.valid);
            if (sa.valid) {
                w.sh_o[q] = make_float4(sa.ox, sa.oy, sa.oz, sa.tmin);
                w.sh_d[q] = make_float4(sa.dx, sa.dy, sa.dz, sa.tmax);
                w.sh_c[q] = Vec4T<R>{sa.c.x, sa.c.y, sa.c.z, R(0)};
                w.sh_pix[q] = sa.pixel;
            }
        }

        // ---- claim a new sample for finished slots: the light vertex ----
        ShadowRay<R> sb;
        sb.valid = false;
        {
            const unsigned mask = __ballot_sync(0xFFFFFFFFu, need_new);
            unsigned long long k = 0;
            if (mask != 0u) {
                const int leader = __ffs(mask) - 1;
                unsigned long long b = 0;
                if ((int)lane_id() == leader) b = atomicAdd(&w.ctr->next_sample, (unsigned long long)__popc(mask));
                b = __shfl_sync(0xFFFFFFFFu, b, leader);
                k = b + (unsigned long long)__popc(mask & lanemask_lt());
            }
            if (need_new) {
                if (k >= (unsigned long long)rc.num_samples) {
                    st = SLOT_DONE;
                } else if (rc.max_vertices == 1) {
                    st = SLOT_EMPTY;  // the loop ends before the light vertex does anything
                } else {
                    const unsigned long long gsample = (unsigned long long)rc.sample_offset + k;
                    const RngKey rk = make_rng(rc.seed, gsample);
                    const float4 ul = rng4(rk, 1u, RNG_SENSOR);
                    const int nl = sv.num_lights;
                    int li = (int)((R)ul.z * (R)nl);
                    li = li < 0 ? 0 : (li > nl - 1 ? nl - 1 : li);
                    const DevLight<R>& L = sv.lights[li];
                    Geom<R> gl;
                    sample_light_position(sv, L, (R)ul.x, (R)ul.y, gl);
                    const R pdf_pl = light_position_pdf(L);
                    V3<R> thr = v3<R>(1, 1, 1) / pdf_pl / (R(1) / (R)nl);  // pdfL = 1 / #lights
                    bool dead = false;
                    if (DIRECT) {
                        const float4 un = rng4(rk, 1u, RNG_NEE_RR);
                        sensor_connect(sv, rc, gl, &L, (const DevMaterial<R>*)nullptr, v3<R>(0, 0, 0), thr, pdf_pl, un,
                                       sb);
                        dead = next_hit_is_dead(rc, un.w, 1);
                    }
                    const float4 ud = rng4(rk, 1u, RNG_DIR);
                    V3<R> wo, wgt;
                    if (!dead && light_sample_direction(L, gl, (R)ud.x, (R)ud.y, wo, wgt)) {
                        thr = thr * wgt;
                        store_ray(w, s, gl, wo, rc.ray_offset);
                        w.thr[s] = Vec4T<R>{thr.x, thr.y, thr.z, R(0)};
                        w.pixel[s] = (uint32_t)li;  // the path's light (its position pdf scales ltdirect)
                        w.sample[s] = gsample;
                        w.nverts[s] = 1;
                        want_ext = true;
                        st = SLOT_ACTIVE;
                    } else {
                        st = SLOT_EMPTY;
                    }
                }
            }
            block_count_warp(&bc.camera, need_new && st != SLOT_DONE);
        }
        if (!want_ext && st == SLOT_ACTIVE) st = SLOT_EMPTY;
        if (want_ext) st = SLOT_ACTIVE;
        w.state[s] = st;
        {
            const int q = warp_append(&w.ctr->sh_count, sb.valid);
            if (sb.valid) {
                w.sh_o[q] = make_float4(sb.ox, sb.oy, sb.oz, sb.tmin);
                w.sh_d[q] = make_float4(sb.dx, sb.dy, sb.dz, sb.tmax);
                w.sh_c[q] = Vec4T<R>{sb.c.x, sb.c.y, sb.c.z, R(0)};
                w.sh_pix[q] = sb.pixel;
            }
        }
        {
            const int q = warp_append(w.ext_count, want_ext);
            if (want_ext) w.ext_queue[q] = s;
        }
        block_count_warp(&bc.active, st != SLOT_DONE);
    }
    block_counts_flush(bc, w.ctr);
}

// ---- bdpt (ProcessSample_BDPT, src/nanogi.cpp:1133-1194) ---------------------------------------
// Leaves vertex V[nv-1] of a subpath (Path::SampleSubpath, bdpt.hpp:86-104): samples the next
// direction with the vertex's own sampling routine and queues the extension ray, or returns
// false where the subpath ends (length limit or a zero f). Random numbers: vertex j leaves with
// (vbase + j + 2, RNG_DIR).
template <typename R>
NGI_D bool bd_extend(const SceneView<R>& sv, const RenderConsts& rc, const WaveView<R>& w, int s, const BdVert<R>* V,
                     int nv, uint32_t vbase, const RngKey& rk, bool le) {
    if ((rc.max_vertices != -1 && nv >= rc.max_vertices) || nv >= kBdptMaxVertices) return false;
    const int j = nv - 1;
    const BdVert<R>& v = V[j];
    const Geom<R> g = bd_geom(v);
    const V3<R> wi = j >= 1 ? bd_dir(v, V[j - 1]) : v3<R>(0, 0, 0);
    const float4 ud = rng4(rk, vbase + (uint32_t)j + 2u, RNG_DIR);
    const DevMaterial<R>& m = sv.mats[v.prim];
    V3<R> wo;
    if (v.type & DT_L) {
        V3<R> wgt;
        if (!light_sample_direction(sv.lights[m.light_index], g, (R)ud.x, (R)ud.y, wo, wgt)) return false;
    } else if (v.type & DT_E) {
        const DevSensor<R>& cam = sv.sensor;
        if (cam.type == ET_PINHOLE) {
            wo = pinhole_direction(cam, (R)ud.x, (R)ud.y);
            if (pinhole_importance(cam, wo) == R(0)) return false;
        } else {
            wo = to_world(g, cosine_hemisphere((R)ud.x, (R)ud.y));
            if (!(to_local(g, wo).z > R(0)) || is_zero(cam.We)) return false;
        }
    } else {
        if (!bsdf_sample(m, g, wi, (R)ud.x, (R)ud.y, (R)ud.z, wo)) return false;
        if (is_zero(bsdf_eval(m, material_albedo(sv, m, g), g, wi, wo, true, le))) return false;
    }
    store_ray(w, s, g, wo, rc.ray_offset);
    return true;
}

// Vertex 0 of a subpath (bdpt.hpp:62-78): a light chosen uniformly (light subpath) or the
// sensor, and a position on it, from (vbase + 1, RNG_SENSOR): .z the choice, .xy the position.
template <typename R>
NGI_D void bd_first_vertex(const SceneView<R>& sv, BdVert<R>* V, uint32_t vbase, const RngKey& rk, bool light) {
    const float4 u = rng4(rk, vbase + 1u, RNG_SENSOR);
    Geom<R> g;
    if (light) {
        const int nl = sv.num_lights;
        int li = (int)((R)u.z * (R)nl);
        li = li < 0 ? 0 : (li > nl - 1 ? nl - 1 : li);
        const DevLight<R>& L = sv.lights[li];
        sample_light_position(sv, L, (R)u.x, (R)u.y, g);
        V[0] = bd_vert(g, L.prim, DT_L);
    } else {
        const DevSensor<R>& cam = sv.sensor;
        if (cam.type == ET_PINHOLE) {
            g.p = cam.eye;
            g.degenerated = true;
            g.ext = 0.0f;
            g.sn = g.gn = g.du = g.dv = v3<R>(0, 0, 0);
            g.uvx = g.uvy = R(0);
        } else {
            sample_mesh_position(sv, cam.tri_base, cam.tri_count, cam.cdf_offset, (R)u.x, (R)u.y, g);
        }
        V[0] = bd_vert(g, cam.prim, DT_E);
    }
}

// Evaluates strategies (n, s) of a sample from the cursor on (Path::Connect and
// EvaluateContribution / SelectionProb, bdpt.hpp:133-211): strategies without a connection
// (s = 0 or t = 0) go to the film, the others become at most two shadow rays. Returns true
// when every strategy is done; otherwise `cursor` holds the next one.
template <typename R>
NGI_D bool bd_connect(const SceneView<R>& sv, const RenderConsts& rc, const WaveView<R>& w, const BdVert<R>* VL,
                      const BdVert<R>* VE, int nL, int nE, int& cursor, ShadowRay<R>* out, BlockCounts& bc) {
    int emitted = 0;
    int n = cursor >> 8, s0 = cursor & 0xFF;
    for (; n <= nL + nE; n++, s0 = -1) {
        if (rc.max_vertices != -1 && n > rc.max_vertices) continue;
        const int smin = n - nE > 0 ? n - nE : 0, smax = nL < n ? nL : n;
        for (int s = s0 > smin ? s0 : smin; s <= smax; s++) {
            if (emitted == 2) {
                cursor = (n << 8) | s;
                return false;
            }
            const int t = n - s;
            if (s == 0 && !(sv.mats[VE[t - 1].prim].type & DT_L)) continue;
            if (t == 0 && !(sv.mats[VL[s - 1].prim].type & DT_E)) continue;
            BdPath<R> x;
            x.L = VL;
            x.E = VE;
            x.s = s;
            x.n = n;
            V3<R> C = bd_unweighted(sv, x);
            if (is_zero(C)) continue;
            C = C * bd_mis_weight(sv, x) / bd_selection_prob<R>(n, s);
            if (is_zero(C)) continue;
            if (!finite3(C)) {
                atomicAdd(&bc.nonfinite, 1u);
                continue;
            }
            // Path::RasterPosition (bdpt.hpp:204-211)
            const BdVert<R>& v = x.at(n - 1);
            R rx = R(0), ry = R(0);
            if (sv.mats[v.prim].e_type == ET_PINHOLE) pinhole_raster(sv.sensor, bd_dir(v, x.at(n - 2)), rx, ry);
            else { rx = v.uvx; ry = v.uvy; }
            const uint32_t pixel = (uint32_t)pixel_index(rx, ry, rc.width, rc.height);
            if (s > 0 && t > 0) {
                ShadowRay<R>& o = out[emitted++];
                shadow_segment(bd_geom(VL[s - 1]), bd_geom(VE[t - 1]), rc.ray_offset, o);
                o.c = C;
                o.pixel = pixel;
                o.light_prim = -1;
            } else {
                film_add(w.film, pixel, C);
                atomicAdd(&bc.contrib, 1u);
            }
        }
    }
    cursor = (n << 8);
    return true;
}

// One wavefront step of bdpt. A slot traces its sample's light subpath, then its eye subpath
// (one extension ray per step), then evaluates its strategies, at most two shadow rays per
// step. Subpath vertex j is kept in HBM (kBdptMaxVertices per subpath); random numbers of the
// light subpath use vertex keys 1.., those of the eye subpath 65.., Russian roulette of vertex
// j on (vbase + j + 1, RNG_NEE_RR).w.
template <typename R>
__global__ void __launch_bounds__(256) k_logic_bdpt(SceneView<R> sv, WaveView<R> w, RenderConsts rc) {
    const int stride = gridDim.x * blockDim.x;
    NGI_COUNTS_DECL
    block_counts_init(bc);
    for (int base = blockIdx.x * blockDim.x; base < w.Q; base += stride) {
        const int s = base + (int)threadIdx.x;  // Q is a multiple of the block size
        uint8_t st = w.state[s];
        int4 bi = w.bd_info[s];
        int phase = bi.x & 0xFF;
        bool pending = ((bi.x >> 8) & 1) != 0;
        int nL = bi.y, nE = bi.z, cursor = bi.w;
        BdVert<R>* VL = w.bd_verts + (size_t)s * 2 * kBdptMaxVertices;
        BdVert<R>* VE = VL + kBdptMaxVertices;
        unsigned long long sample = w.sample[s];
        bool need_new = st == SLOT_EMPTY;
        ShadowRay<R> sh[2];
        sh[0].valid = sh[1].valid = false;

        if (st == SLOT_ACTIVE) {
            const RngKey rk = make_rng(rc.seed, sample);
            if (phase < 2 && pending) {
                // the extension hit of subpath `phase` (bdpt.hpp:106-129)
                pending = false;
                const float4 h = w.hit[s];
                if (__float_as_int(h.w) >= 0) {
                    BdVert<R>* V = phase == 0 ? VL : VE;
                    int& nv = phase == 0 ? nL : nE;
                    const uint32_t vbase = phase == 0 ? 0u : 64u;
                    V3<R> d;
                    Geom<R> g;
                    const int prim = hit_geometry(sv, rc, w, s, h, d, g, true);
                    V[nv] = bd_vert(g, prim, sv.mats[prim].type & ~(DT_L | DT_E));
                    const float rr = rng4(rk, vbase + (uint32_t)nv + 1u, RNG_NEE_RR).w;
                    nv++;
                    if (!(rr > 0.5f)) pending = bd_extend(sv, rc, w, s, V, nv, vbase, rk, phase == 0);
                }
            }
            if (phase == 0 && !pending) {
                phase = 1;
                bd_first_vertex(sv, VE, 64u, rk, false);
                nE = 1;
                pending = bd_extend(sv, rc, w, s, VE, 1, 64u, rk, false);
            }
            if (phase == 1 && !pending) {
                phase = 2;
                cursor = 2 << 8;
            }
            if (phase == 2) {
                if (bd_connect(sv, rc, w, VL, VE, nL, nE, cursor, sh, bc)) {
                    need_new = true;
                    st = SLOT_EMPTY;
                }
            }
        }

        // ---- claim a new sample: its light subpath starts here ----
        {
            const unsigned mask = __ballot_sync(0xFFFFFFFFu, need_new);
            unsigned long long k = 0;
            if (mask != 0u) {
                const int leader = __ffs(mask) - 1;
                unsigned long long b = 0;
                if ((int)lane_id() == leader) b = atomicAdd(&w.ctr->next_sample, (unsigned long long)__popc(mask));
                b = __shfl_sync(0xFFFFFFFFu, b, leader);
                k = b + (unsigned long long)__popc(mask & lanemask_lt());
            }
            if (need_new) {
                if (k >= (unsigned long long)rc.num_samples) {
                    st = SLOT_DONE;
                } else {
                    sample = (unsigned long long)rc.sample_offset + k;
                    const RngKey rk = make_rng(rc.seed, sample);
                    bd_first_vertex(sv, VL, 0u, rk, true);
                    nL = 1;
                    nE = 0;
                    phase = 0;
                    pending = bd_extend(sv, rc, w, s, VL, 1, 0u, rk, true);
                    if (!pending) {
                        phase = 1;
                        bd_first_vertex(sv, VE, 64u, rk, false);
                        nE = 1;
                        pending = bd_extend(sv, rc, w, s, VE, 1, 64u, rk, false);
                        if (!pending) {
                            phase = 2;  // evaluated from the next step on
                            cursor = 2 << 8;
                        }
                    }
                    st = SLOT_ACTIVE;
                }
            }
            block_count_warp(&bc.camera, need_new && st != SLOT_DONE);
        }
        w.state[s] = st;
        w.sample[s] = sample;
        w.bd_info[s] = make_int4(phase | (pending ? 0x100 : 0), nL, nE, cursor);
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int q = warp_append(&w.ctr->sh_count, sh[r].valid);
            if (sh[r].valid) {
                w.sh_o[q] = make_float4(sh[r].ox, sh[r].oy, sh[r].oz, sh[r].tmin);
                w.sh_d[q] = make_float4(sh[r].dx, sh[r].dy, sh[r].dz, sh[r].tmax);
                w.sh_c[q] = Vec4T<R>{sh[r].c.x, sh[r].c.y, sh[r].c.z, R(0)};
                w.sh_pix[q] = sh[r].pixel;
            }
        }
        {
            const bool want_ext = st == SLOT_ACTIVE && pending;
            const int q = warp_append(w.ext_count, want_ext);
            if (want_ext) w.ext_queue[q] = s;
        }
        block_count_warp(&bc.active, st != SLOT_DONE);
    }
    block_counts_flush(bc, w.ctr);
}

// Which logic kernel a wave runs.
// kLogicCameraQ: camera paths with queued (compacted) shading whatever the renderer (pt renders
// whose samples all fit in one wave)
constexpr int kLogicCamera = 0, kLogicLight = 1, kLogicBdpt = 2, kLogicCameraQ = 3;


// ---- persistent traversal -------------------------------------------------------------------
// Warps stay resident and trace until both the queue and their lanes are empty. A lane
// whose ray has finished sits idle until at least `refill` lanes of its warp are idle; then
// the warp fetches that many new rays with one atomic and the lanes start them while the
// others carry on. This keeps SIMD lanes busy on incoherent rays (Aila and Laine, HPG 2009)
// and removes the tail of a fixed grid.
// One launch traces both queues: extension items first, then shadow items, each lane tracing its
// own kind, so shadow rays fill the tail of the extension work instead of a second launch
// (terrain 1483 against 1417 Mrays/s for two launches).
template <typename R, bool STATS, bool ADJ = false, bool BATCH = false>
__global__ void __launch_bounds__(128, kTraceMinBlocks) k_trace(SceneView<R> sv, WaveView<R> w, int refill,
                                                                 int num_prims, const JobView<R>* __restrict__ jobs) {
    extern __shared__ float adj_smem[];
    float* gsm = (ADJ && num_prims <= kAdjSmemPrims) ? adj_smem : nullptr;
    if (ADJ) adj_smem_clear(gsm, num_prims);
    const int n_ext = *w.ext_count;
    const int n = n_ext + w.ctr->sh_count;
    int* fetch = &w.ctr->ext_fetch;
    TravState s;
    uint2 stack[kTraversalStack];
    int item = -1, slot = -1, job = 0;
    bool shadow = false;
    const CwNode* nodes = sv.nodes;
    const float4* tris = sv.tris;
    int num_nodes = sv.num_nodes;
    bool exhausted = false;
    bool overflow = false;
    TraceStats ts{0u, 0u}, ts_sh{0u, 0u};
    // film contributions of the block, counted in shared memory (no register kept for them)
    __shared__ unsigned int blk_contrib;
    if (threadIdx.x == 0) blk_contrib = 0u;
    __syncthreads();
    while (true) {
        const bool idle = item < 0;
        const unsigned idle_mask = __ballot_sync(0xFFFFFFFFu, idle);
        if (!exhausted && __popc(idle_mask) >= refill) {
            const int leader = __ffs(idle_mask) - 1;
            int base = 0;
            if ((int)lane_id() == leader) base = atomicAdd(fetch, __popc(idle_mask));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (base + __popc(idle_mask) >= n) exhausted = true;
            if (idle) {
                const int i = base + __popc(idle_mask & lanemask_lt());
                if (i < n) {
                    shadow = i >= n_ext;
                    item = shadow ? i - n_ext : i;
                    float4 o, d;
                    if (shadow) {
                        o = __ldcs(w.sh_o + item);
                        d = __ldcs(w.sh_d + item);
                        if (BATCH) job = w.sh_job[item];
                    } else {
                        slot = __ldcs(w.ext_queue + item);
                        o = __ldcs(w.ray_o + slot);
                        d = __ldcs(w.ray_d + slot);
                        if (BATCH) job = w.job[slot];
                    }
                    if (BATCH) {
                        nodes = jobs[job].sv.nodes;
                        tris = jobs[job].sv.tris;
                        num_nodes = jobs[job].sv.num_nodes;
                    }
                    trav_init(s, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w);
                }
            }
        }
        const unsigned busy = __ballot_sync(0xFFFFFFFFu, item >= 0);
        if (busy == 0u) break;  // no lane has a ray: the refill above found the queue empty
        if (item >= 0) {
            const bool done = num_nodes == 0 ||
                              trav_step<STATS>(s, stack, nodes, tris, overflow, shadow ? &ts_sh : &ts, shadow);
            if (done) {
                if (shadow) {
                    if (s.hit < 0) {
                        const Vec4T<R> c = ld_stream(w.sh_c + item);
                        const V3<R> cc = v3<R>(c.x, c.y, c.z);
                        if (finite3(cc)) {
                            const uint32_t pix = __ldcs(w.sh_pix + item);
                            film_add(BATCH ? jobs[job].film : w.film, pix, cc);
                            atomicAdd(&blk_contrib, 1u);
                            if (ADJ) {
                                const int2 info = w.sh_info[item];
                                const int count = info.x & 0xFF;
                                uint4 qa = make_uint4(0u, 0u, 0u, 0u), qb = qa;
                                if (count > 0) {
                                    qa = w.sh_pre[2 * (size_t)item];
                                    qb = w.sh_pre[2 * (size_t)item + 1];
                                }
                                adj_accumulate(w, sv, pix, cc, qa, qb, count, (info.x >> 8) - 1, info.y, gsm,
                                               num_prims);
                            }
                        } else {
                            atomicAdd(&w.ctr->stat_nonfinite, 1ull);  // rare: no register kept for it
                        }
                    }
                } else {
                    __stcs(w.hit + slot, make_float4(s.tmax, s.hu, s.hv, __int_as_float(s.hit)));
                }
                item = -1;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && blk_contrib) atomicAdd(&w.ctr->stat_contrib, (unsigned long long)blk_contrib);
    if (ADJ) adj_flush(w, gsm, num_prims);
    if (overflow) atomicOr(&w.ctr->error_flags, 1);
    if (STATS) {
        warp_sum_add(&w.ctr->ext_nodes, ts.nodes);
        warp_sum_add(&w.ctr->ext_tris, ts.tris);
        warp_sum_add(&w.ctr->sh_nodes, ts_sh.nodes);
        warp_sum_add(&w.ctr->sh_tris, ts_sh.tris);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&w.ctr->stat_ext, (unsigned long long)n_ext);
        atomicAdd(&w.ctr->stat_shadow, (unsigned long long)(n - n_ext));
    }
}

// ---- the end of a wave ----------------------------------------------------------------------------
// Once every sample has been claimed, the paths still in flight only get fewer with each iteration,
// and the wave's last iterations run a handful of rays each at the price of a full set of launches.
// k_finish takes over then: one thread per pending path runs it to its end, vertex after vertex, with
// the shading of the wavefront kernels (shade_vertex) and the traversal inline (trace_ray: the closest
// hit of each extension ray and the any-hit test of each shadow ray, which adds an unoccluded
// contribution to the film). Every path follows the same Philox draws and traversal as in the
// wavefront, so the film is the same up to the order of its FP64 sums. BATCH: each path renders with
// its own job's scene, parameters, film and renderer. ADJ: the backward pass; an unoccluded shadow
// ray also adds its gradients (adj_accumulate with the path's prefix at that vertex, as the traversal
// kernel does from the shadow queue), summed per block in shared memory when the scene is small.
// Measured and not kept: tracing each vertex's shadow and extension rays together, their
// traversal steps interleaved in the thread (13.54 against 13.54 ms per 16-spp terrain render,
// 52.84 against 52.72 ms per 64-spp render; 168 registers instead of 123).
constexpr int kFinishBlock = 128;
constexpr int kFinishMaxVertices = 4096;
// Paths left in flight below which the wave hands them to k_finish: its time grows with the paths it
// gets (the longest of them sets it), while one more drain iteration costs a full set of launches.
// Terrain, ptdirect, 2^25-slot wave: 8192 paths 14.59 ms per 16-spp render, 32768 14.43, 131072
// 14.36; per 64-spp render 55.33, 55.10 and 54.89 ms. Later kernels, 131072 against larger limits:
// the terrain keeps 292,617 paths after four iterations, so 262144 is the same (12.73 ms) and 524288
// finishes all of them at once (13.26 ms); the interior (1024^2, max length 32) 15.23 against 15.61
// (262144) and 15.67 ms (524288).
constexpr int kFinishMaxPaths = 131072;
template <typename R, bool DIRECT, bool BATCH, bool ADJ>
__global__ void __launch_bounds__(kFinishBlock)
    k_finish(SceneView<R> sv0, WaveView<R> w, RenderConsts rc0, const JobView<R>* __restrict__ jobs) {
    NGI_COUNTS_DECL
    block_counts_init(bc);
    extern __shared__ float adj_smem_finish[];
    float* gsm = (ADJ && rc0.num_prims <= kAdjSmemPrims) ? adj_smem_finish : nullptr;
    if (ADJ) adj_smem_clear(gsm, rc0.num_prims);
    __shared__ unsigned long long blk_ext, blk_sh;
    if (threadIdx.x == 0) blk_ext = blk_sh = 0ull;
    __syncthreads();
    bool overflow = false;
    uint32_t n_ext = 0, n_sh = 0;
    const int n = min(*w.ext_count, w.Q);
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < n; item += gridDim.x * blockDim.x) {
        const int s = w.ext_queue[item];
        const int job = BATCH ? w.job[s] : 0;
        const SceneView<R>& sv = BATCH ? jobs[job].sv : sv0;
        const RenderConsts& rc = BATCH ? jobs[job].rc : rc0;
        double* const film = BATCH ? jobs[job].film : w.film;
        const bool direct = BATCH ? rc.renderer == NGI_RENDERER_PTDIRECT : DIRECT;
        float4 h = w.hit[s];
        uint4 pa = make_uint4(0u, 0u, 0u, 0u), pb = pa;
        // a path ends by Russian roulette with probability 1/2 per vertex; the cap only bounds the loop
        for (int vertex = 0; __float_as_int(h.w) >= 0; vertex++) {
            if (vertex == kFinishMaxVertices) {
                atomicOr(&w.ctr->error_flags, 4);
                break;
            }
            const bool alive = shade_vertex<R, ADJ>(
                sv, rc, film, direct, w, s, h, pa, pb, gsm, bc, [&](const ShadowRay<R>& sa, int count, int vprim) {
                    if (!sa.valid) return;
                    float tmax = sa.tmax, u = 0.0f, v = 0.0f;
                    const int occ = trace_ray<true, false>(sv.nodes, sv.tris, sv.num_nodes, sa.ox, sa.oy, sa.oz, sa.dx,
                                                           sa.dy, sa.dz, sa.tmin, tmax, u, v, overflow, nullptr);
                    n_sh++;
                    if (occ >= 0) return;
                    if (finite3(sa.c)) {
                        film_add(film, sa.pixel, sa.c);
                        atomicAdd(&bc.contrib, 1u);
                        if (ADJ) adj_accumulate(w, sv, sa.pixel, sa.c, pa, pb, count, vprim, sa.light_prim, gsm,
                                                rc.num_prims);
                    } else {
                        atomicAdd(&bc.nonfinite, 1u);
                    }
                });
            if (!alive) break;
            const float4 o = w.ray_o[s], d = w.ray_d[s];
            float tmax = d.w, u = 0.0f, v = 0.0f;
            const int ti = trace_ray<false, false>(sv.nodes, sv.tris, sv.num_nodes, o.x, o.y, o.z, d.x, d.y, d.z, o.w,
                                                   tmax, u, v, overflow, nullptr);
            n_ext++;
            h = make_float4(ti >= 0 ? tmax : d.w, u, v, __int_as_float(ti));
        }
    }
    if (n_ext) atomicAdd(&blk_ext, (unsigned long long)n_ext);
    if (n_sh) atomicAdd(&blk_sh, (unsigned long long)n_sh);
    if (overflow) atomicOr(&w.ctr->error_flags, 1);
    if (ADJ) adj_flush(w, gsm, rc0.num_prims);  // synchronises the block first
    block_counts_flush(bc, w.ctr);  // synchronises the block first
    if (threadIdx.x == 0) {
        if (blk_ext) atomicAdd(&w.ctr->stat_ext, blk_ext);
        if (blk_sh) atomicAdd(&w.ctr->stat_shadow, blk_sh);
    }
}

// ---- parity hooks --------------------------------------------------------------------------
__global__ void k_intersect(const CwNode* nodes, const float4* tris, int num_nodes, const float4* rays, int64_t n,
                            int32_t* prim, float* t_out, float* uv_out, int* err) {
    bool overflow = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = rays[2 * i], b = rays[2 * i + 1];
        float tmax = b.w, u = 0.0f, v = 0.0f;
        const int ti = trace_ray<false, false>(nodes, tris, num_nodes, a.x, a.y, a.z, b.x, b.y, b.z, a.w, tmax, u, v,
                                               overflow, nullptr);
        prim[i] = ti >= 0 ? (int32_t)__float_as_uint(tris[3 * (size_t)ti].w) : -1;
        t_out[i] = ti >= 0 ? tmax : INFINITY;
        uv_out[2 * i] = ti >= 0 ? u : 0.0f;
        uv_out[2 * i + 1] = ti >= 0 ? v : 0.0f;
    }
    if (overflow) atomicOr(err, 1);
}

__global__ void k_visible(const CwNode* nodes, const float4* tris, int num_nodes, const double* pts, int64_t n,
                          uint8_t* vis, int* err) {
    bool overflow = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double* p = pts + 6 * i;
        const V3<double> a = v3<double>(p[0], p[1], p[2]), b = v3<double>(p[3], p[4], p[5]);
        const V3<double> d = b - a;
        const double len = sqrt(dot(d, d));
        const V3<double> dn = d / len;
        float tmax = (float)len * (1.0f - kEpsF), u, v;
        const int ti = trace_ray<true, false>(nodes, tris, num_nodes, (float)a.x, (float)a.y, (float)a.z, (float)dn.x,
                                              (float)dn.y, (float)dn.z, kEpsF, tmax, u, v, overflow, nullptr);
        vis[i] = ti < 0 ? 1 : 0;
    }
    if (overflow) atomicOr(err, 1);
}

// ---- upload -----------------------------------------------------------------------------------
namespace {

template <typename T>
T* upload(const void* src, size_t count) {
    T* p = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    CUDA_CHECK(cudaMalloc(&p, bytes));
    if (count) CUDA_CHECK(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

template <typename R> V3<R> hv3(const double a[3]) { return V3<R>{(R)a[0], (R)a[1], (R)a[2]}; }

template <typename R>
void build_tables(const HostScene& hs, std::vector<DevMaterial<R>>& mats, std::vector<DevLight<R>>& lights,
                  DevSensor<R>& sensor, std::vector<double>& cdf, std::vector<float>& epos, std::vector<float>& euv) {
    mats.clear();
    lights.clear();
    cdf.clear();
    epos.clear();
    euv.clear();
    auto add_emitter_mesh = [&](const HostPrimitive& p, int& tri_base, int& cdf_off) {
        tri_base = (int)(epos.size() / 9);
        cdf_off = (int)cdf.size();
        for (double v : p.area_cdf) cdf.push_back(v);
        for (int64_t t = 0; t < p.tri_count; t++) {
            for (int k = 0; k < 9; k++) epos.push_back(hs.tri_pos[9 * (p.tri_first + t) + k]);
            for (int k = 0; k < 6; k++) euv.push_back(hs.tri_uv[6 * (p.tri_first + t) + k]);
        }
    };
    for (size_t i = 0; i < hs.prims.size(); i++) {
        const HostPrimitive& p = hs.prims[i];
        DevMaterial<R> m{};
        m.type = p.type;
        m.bsdf = (p.type & PT_D) ? BSDF_D : (p.type & PT_G) ? BSDF_G : (p.type & PT_S) ? BSDF_S : BSDF_NONE;
        m.s_type = p.s_type;
        m.l_type = p.l_type;
        m.R_ = m.bsdf == BSDF_D ? hv3<R>(p.D_R) : m.bsdf == BSDF_G ? hv3<R>(p.G_R) : hv3<R>(p.S_R);
        m.eta = hv3<R>(p.G_eta);
        m.k = hv3<R>(p.G_k);
        m.roughness = (R)p.G_roughness;
        m.eta1 = (R)p.S_eta1;
        m.eta2 = (R)p.S_eta2;
        m.Le = hv3<R>(p.Le);
        m.We = hv3<R>(p.We);
        m.e_type = p.e_type;
        m.tex = m.bsdf == BSDF_D ? p.D_tex : (m.bsdf == BSDF_G ? p.G_tex : -1);
        m.light_index = -1;
        mats.push_back(m);
    }
    for (size_t li = 0; li < hs.light_prims.size(); li++) {
        const HostPrimitive& p = hs.prims[hs.light_prims[li]];
        mats[hs.light_prims[li]].light_index = (int)li;
        DevLight<R> L{};
        L.type = p.l_type;
        L.prim = hs.light_prims[li];
        L.Le = hv3<R>(p.Le);
        L.inv_area = (R)p.inv_area;
        L.position = hv3<R>(p.l_position);
        L.direction = hv3<R>(p.l_direction);
        L.center = hv3<R>(p.l_center);
        L.radius = (R)p.l_radius;
        if (p.l_type == L_AREA) {
            L.tri_count = (int)p.tri_count;
            add_emitter_mesh(p, L.tri_base, L.cdf_offset);
        }
        lights.push_back(L);
    }
    sensor = DevSensor<R>{};
    sensor.type = -1;
    if (hs.sensor_prim >= 0) {
        const HostPrimitive& p = hs.prims[hs.sensor_prim];
        sensor.type = p.e_type;
        sensor.prim = hs.sensor_prim;
        sensor.eye = hv3<R>(p.eye);
        sensor.Vx = hv3<R>(p.Vx);
        sensor.Vy = hv3<R>(p.Vy);
        sensor.Vz = hv3<R>(p.Vz);
        sensor.tan_fov = (R)std::tan(p.fov * 0.5);
        sensor.aspect = (R)p.aspect;
        sensor.We = hv3<R>(p.We);
        sensor.inv_area = (R)p.inv_area;
        if (p.e_type == E_AREA) {
            sensor.tri_count = (int)p.tri_count;
            add_emitter_mesh(p, sensor.tri_base, sensor.cdf_offset);
        }
    }
    // Next-event estimation at a pinhole sensor connects the eye to a point of the light, and an area
    // light contributes only from the side its normal faces (rt.hpp:917-937). A light all of whose
    // triangles face away from the eye never contributes there, so that estimation stops at the pick
    // (the film is the same: the facing test would reject every sample). The eye must lie behind each
    // triangle's plane by 1e-4 of its distance, far beyond the FP32 rounding of the facing test.
    for (size_t li = 0; li < hs.light_prims.size(); li++) {
        DevLight<R>& L = lights[li];
        L.sensor_facing = 1;
        if (sensor.type != E_PINHOLE || L.type != L_AREA) continue;
        const HostPrimitive& p = hs.prims[hs.light_prims[li]];
        bool away = p.tri_count > 0;
        for (int64_t t = 0; t < p.tri_count && away; t++) {
            const float* P = hs.tri_pos.data() + 9 * (p.tri_first + t);
            const double e1[3] = {(double)P[3] - P[0], (double)P[4] - P[1], (double)P[5] - P[2]};
            const double e2[3] = {(double)P[6] - P[0], (double)P[7] - P[1], (double)P[8] - P[2]};
            const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                 e1[0] * e2[1] - e1[1] * e2[0]};
            const double* eye = hs.prims[hs.sensor_prim].eye;
            const double v[3] = {eye[0] - P[0], eye[1] - P[1], eye[2] - P[2]};
            const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            const double vv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            const double d = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
            away = nn > 0.0 && vv > 0.0 && d < -1e-4 * nn * vv;
        }
        if (away) L.sensor_facing = 0;
    }
}

template <typename R>
SceneView<R> make_view(const DeviceScene& ds) {
    SceneView<R> v{};
    v.nodes = ds.nodes;
    v.tris = ds.tris;
    v.nrm = ds.nrm;
    v.uv = ds.uv;
    v.mats = (const DevMaterial<R>*)(sizeof(R) == 8 ? ds.mats_d : ds.mats_f);
    v.lights = (const DevLight<R>*)(sizeof(R) == 8 ? ds.lights_d : ds.lights_f);
    v.num_lights = ds.num_lights;
    v.num_nodes = ds.num_nodes;
    v.cdf = ds.cdf;
    v.emit_tri_pos = ds.emit_pos;
    v.emit_tri_uv = ds.emit_uv;
    v.texels = ds.texels;
    v.tex_info = ds.tex_info;
    v.num_textures = ds.num_textures;
    std::memcpy(&v.sensor, sizeof(R) == 8 ? ds.sensor_d : ds.sensor_f, sizeof(DevSensor<R>));
    return v;
}

void free_wave(RenderWave* wv) {
    if (!wv) return;
    for (WaveGraphs& g : wv->graphs) {
        if (g.main) cudaGraphExecDestroy(g.main);
        if (g.drain) cudaGraphExecDestroy(g.drain);
    }
    for (void* p : wv->bufs) cudaFree(p);
    if (wv->h_ctr) cudaFreeHost(wv->h_ctr);
    if (wv->ev0) cudaEventDestroy(wv->ev0);
    if (wv->ev1) cudaEventDestroy(wv->ev1);
    delete wv;
}

}  // namespace

void DeviceUpload(HostScene& hs) {
    if (hs.dev) return;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw DeviceError("no CUDA device is visible", NGI_ERR_NO_DEVICE);
    }
    static_assert(sizeof(DevSensor<double>) <= 256, "sensor record too large");
    auto* ds = new DeviceScene();
    hs.dev = ds;
    try {
        CUDA_CHECK(cudaGetDevice(&ds->device));
        CUDA_CHECK(cudaStreamCreateWithFlags(&ds->stream, cudaStreamNonBlocking));
        const int n = (int)hs.NumTriangles();
        ds->num_tris = n;
        float* d_pos = upload<float>(hs.tri_pos.data(), hs.tri_pos.size());
        float* d_nrm = upload<float>(hs.tri_nrm.data(), hs.tri_nrm.size());
        float* d_uv = upload<float>(hs.tri_uv.data(), hs.tri_uv.size());
        int* d_prim = upload<int>(hs.tri_prim.data(), hs.tri_prim.size());
        try {
            BuildBvh(*ds, d_pos, d_nrm, d_uv, d_prim, n, ds->stream);
        } catch (...) {
            cudaFree(d_pos); cudaFree(d_nrm); cudaFree(d_uv); cudaFree(d_prim);
            throw;
        }
        cudaFree(d_pos); cudaFree(d_nrm); cudaFree(d_uv); cudaFree(d_prim);
        if (ds->bvh_depth > kTraversalStack)
            throw DeviceError("BVH depth " + std::to_string(ds->bvh_depth) + " exceeds the traversal stack", NGI_ERR_UNSUPPORTED);

        std::vector<DevMaterial<float>> mf; std::vector<DevLight<float>> lf; DevSensor<float> sf;
        std::vector<DevMaterial<double>> md; std::vector<DevLight<double>> ld; DevSensor<double> sd;
        std::vector<double> cdf; std::vector<float> epos, euv;
        build_tables<float>(hs, mf, lf, sf, cdf, epos, euv);
        build_tables<double>(hs, md, ld, sd, cdf, epos, euv);
        ds->mats_f = upload<DevMaterial<float>>(mf.data(), mf.size());
        ds->mats_d = upload<DevMaterial<double>>(md.data(), md.size());
        ds->lights_f = upload<DevLight<float>>(lf.data(), lf.size());
        ds->lights_d = upload<DevLight<double>>(ld.data(), ld.size());
        ds->cdf = upload<double>(cdf.data(), cdf.size());
        ds->emit_pos = upload<float>(epos.data(), epos.size());
        ds->emit_uv = upload<float>(euv.data(), euv.size());
        if (!hs.textures.empty()) {
            std::vector<int4> info;
            std::vector<float4> texels;
            for (const TextureImage& t : hs.textures) {
                info.push_back(make_int4((int)texels.size(), t.width, t.height, 0));
                for (size_t i = 0; i < (size_t)t.width * t.height; i++)
                    texels.push_back(make_float4(t.rgb[3 * i], t.rgb[3 * i + 1], t.rgb[3 * i + 2], 0.0f));
            }
            ds->tex_info = upload<int4>(info.data(), info.size());
            ds->texels = upload<float4>(texels.data(), texels.size());
            ds->num_textures = (int)info.size();
        }
        ds->num_lights = (int)lf.size();
        std::memcpy(ds->sensor_f, &sf, sizeof(sf));
        std::memcpy(ds->sensor_d, &sd, sizeof(sd));
        CUDA_CHECK(cudaStreamSynchronize(ds->stream));
    } catch (...) {
        DeviceFree(hs);
        throw;
    }
}

void DeviceReleaseBuffers(HostScene& hs) {
    DeviceScene* ds = hs.dev;
    if (!ds) return;
    if (ds->stream) cudaStreamSynchronize(ds->stream);
    free_wave(ds->wave);
    ds->wave = nullptr;
}

void DeviceFree(HostScene& hs) {
    DeviceScene* ds = hs.dev;
    if (!ds) return;
    if (ds->stream) cudaStreamSynchronize(ds->stream);
    free_wave(ds->wave);
    void* ptrs[] = {ds->nodes, ds->tris, ds->nrm, ds->uv, ds->mats_f, ds->mats_d, ds->lights_f,
                    ds->lights_d, ds->cdf, ds->emit_pos, ds->emit_uv, ds->texels, ds->tex_info, ds->film,
                    ds->adj, ds->grads};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (ds->stream) cudaStreamDestroy(ds->stream);
    delete ds;
    hs.dev = nullptr;
}

// The scene's buffers, stream and wave live on the device that was current when it was uploaded.
// Calls that take the caller's device pointers or stream, or that launch on the current device,
// must be made with that device current: mixing two devices' pointers in one launch fails or
// faults.
void RequireSceneDevice(const DeviceScene& ds) {
    int cur = -1;
    CUDA_CHECK(cudaGetDevice(&cur));
    if (cur != ds.device)
        throw DeviceError("the scene lives on device " + std::to_string(ds.device) + " but device " +
                              std::to_string(cur) + " is current: make the scene's device current first",
                          NGI_ERR_INVALID_ARGUMENT);
}

// ---- render driver ------------------------------------------------------------------------------
namespace {

template <typename R>
void alloc_wave_view(RenderWave* wv, WaveView<R>& v, int Q) {
    auto A = [&](size_t bytes) -> void* {
        void* p = nullptr;
        CUDA_CHECK(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
        wv->bufs.push_back(p);
        return p;
    };
    v.Q = Q;
    v.ray_o = (float4*)A(sizeof(float4) * Q);
    v.ray_d = (float4*)A(sizeof(float4) * Q);
    v.hit = (float4*)A(sizeof(float4) * Q);
    v.thr = (Vec4T<R>*)A(sizeof(Vec4T<R>) * Q);
    if (sizeof(R) == 8) {
        v.od_o = (Vec4T<double>*)A(sizeof(Vec4T<double>) * Q);
        v.od_d = (Vec4T<double>*)A(sizeof(Vec4T<double>) * Q);
    } else {
        v.od_o = v.od_d = nullptr;
    }
    v.pixel = (uint32_t*)A(sizeof(uint32_t) * Q);
    v.sample = (unsigned long long*)A(sizeof(unsigned long long) * Q);
    v.nverts = (int*)A(sizeof(int) * Q);
    v.state = (uint8_t*)A(sizeof(uint8_t) * Q);
    v.ext_queue = (int*)A(sizeof(int) * Q);
    v.ext_queue_b = (int*)A(sizeof(int) * Q);
    v.carry_a = (int*)A(sizeof(int) * Q);
    v.carry_b = (int*)A(sizeof(int) * Q);
    v.regen_queue = (int*)A(sizeof(int) * Q);
    v.sh_o = (float4*)A(sizeof(float4) * kShadowPerSlot * (size_t)Q);
    v.sh_d = (float4*)A(sizeof(float4) * kShadowPerSlot * (size_t)Q);
    v.sh_c = (Vec4T<R>*)A(sizeof(Vec4T<R>) * kShadowPerSlot * (size_t)Q);
    v.sh_pix = (uint32_t*)A(sizeof(uint32_t) * kShadowPerSlot * (size_t)Q);
    v.ctr = wv->ctr;
    v.ext_count = &v.ctr->ext_count;
    v.ext_in = v.ext_in_count = v.carry_in = v.carry_in_count = nullptr;  // set per iteration when compacted
    v.carry_out = v.carry_out_count = nullptr;
}

RenderWave* ensure_wave_exact(DeviceScene& ds, int Q, int precision) {
    if (ds.wave && ds.wave->Q == Q && ds.wave->precision == precision) return ds.wave;
    free_wave(ds.wave);
    ds.wave = nullptr;
    auto* wv = new RenderWave();
    try {
        wv->Q = Q;
        wv->precision = precision;
        void* c = nullptr;
        CUDA_CHECK(cudaMalloc(&c, sizeof(WaveCounters)));
        wv->bufs.push_back(c);
        wv->ctr = (WaveCounters*)c;
        CUDA_CHECK(cudaMallocHost(&wv->h_ctr, sizeof(WaveCounters)));
        if (precision == NGI_PRECISION_FP64) alloc_wave_view<double>(wv, wv->vd, Q);
        else alloc_wave_view<float>(wv, wv->vf, Q);
        CUDA_CHECK(cudaEventCreate(&wv->ev0));
        CUDA_CHECK(cudaEventCreate(&wv->ev1));
    } catch (...) {
        free_wave(wv);
        throw;
    }
    ds.wave = wv;
    return wv;
}

// The wave of a render, kept by the scene handle for its next render. When the device cannot hold
// Q slots (other handles keep their own waves), the wave shrinks by halves down to 2^16 slots:
// slower, but the render completes. The caller reads the slot count back from the wave.
RenderWave* ensure_wave(DeviceScene& ds, int Q, int precision) {
    while (true) {
        try {
            return ensure_wave_exact(ds, Q, precision);
        } catch (const DeviceError& e) {
            if (e.code != NGI_ERR_OUT_OF_MEMORY || Q <= (1 << 16)) throw;
            cudaGetLastError();  // clear the allocation error
            Q = std::max(1 << 16, (Q / 2 + 255) / 256 * 256);
        }
    }
}

int grid_for(int items, int block) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int max_blocks = sms * 8;  // persistent-style: 8 x 256 threads resident per SM
    return std::max(1, std::min(max_blocks, (items + block - 1) / block));
}

// Blocks of a persistent kernel that fit on the device at once. Measured and not kept: a preferred
// shared-memory carve-out of 0 (the largest L1) for the traversal (1768 against 1809 Mrays/s on
// the terrain with the CUDA driver's default) or for the path logic (1810: no change).
template <typename K>
int persistent_grid(K kernel, int block) {
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    return std::max(1, sms * std::max(per_sm, 1));
}

constexpr int kTraceBlock = 128;
// Idle lanes that make a traversal warp fetch new rays, with one atomic on the queue cursor for
// them all. Measured and not kept: each warp taking a chunk of 64 queue entries per atomic and
// refilling from it (1871 against 1941 Mrays/s on the terrain, 4206 against 4358 on the Cornell
// box: the launch waits longer on warps that still hold entries at its end).
constexpr int kRefillLanes = 8;

// Grid size of the persistent traversal kernel (queried once per instance, outside any graph capture).
template <typename R, bool STATS, bool ADJ = false, bool BATCH = false>
int trace_grid() {
    static const int g = persistent_grid(k_trace<R, STATS, ADJ, BATCH>, kTraceBlock);
    return g;
}

// Compacted shading applies to ptdirect's camera paths outside batches. Measured and not kept:
// the traversal sending each finished extension ray's slot either to a hit queue for shading or,
// on a miss, straight to the next regeneration queue (43.6% of the terrain's extension rays
// miss), with the appends batched per warp at each refill. Shading visited only hits, but the
// logic kernels' time per iteration stayed at 0.34 ms (a miss costs shading little: one hit
// record read and a queue append), while the traversal launch grew from 0.613 to 0.644 ms:
// 1741 against 1791 Mrays/s on the terrain.
// Batches keep the fused kernel: compacted, with each slot's job choosing its renderer at run time,
// the 256-job batch took 2,000 against 1,245 ms (the split kernels spill 188 B per thread with the
// job lookups, and the batch's shadow rays cannot be staged without their job).
template <bool DIRECT, bool BATCH, int LOGIC>
constexpr bool compact_shading() {
    return !BATCH && (LOGIC == kLogicCameraQ || (DIRECT && LOGIC == kLogicCamera));
}

// Per-iteration counter reset of compacted shading: the queues the iteration fills start empty,
// the ones it reads (filled by the previous iteration) keep their counts.
__global__ void k_iteration_begin(WaveCounters* ctr, int parity) {
    if (threadIdx.x != 0) return;
    ctr->sh_count = 0;
    ctr->active = 0;
    ctr->ext_fetch = 0;
    ctr->sh_fetch = 0;
    ctr->regen_count = ctr->regen_seed;  // the wave's slots in its first iteration, then 0
    ctr->regen_seed = 0;
    if (parity) ctr->ext_count = 0;
    else ctr->ext_count_b = 0;
    ctr->carry_count[1 - parity] = 0;
}

// Every slot of a new wave starts empty, in the regeneration queue of the first iteration: its
// shading launch has no queued slot, and regeneration starts a sample in every slot. (Handing the
// slots through the carry queue instead took the first shading launch 0.28 ms for 2^25 slots.)
// claimed: the samples the first iteration starts without claiming them (a wave that holds every
// sample gives slot i sample i), else 0.
__global__ void k_wave_init_slots(int* regen_queue, int Q, WaveCounters* ctr, unsigned long long claimed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Q) regen_queue[i] = i;
    if (i == 0) {
        ctr->regen_seed = Q;
        ctr->carry_count[0] = 0;
        ctr->next_sample = claimed;
    }
}

template <typename R, bool DIRECT, bool STATS, bool ADJ = false, bool BATCH = false, int LOGIC = 0>
void enqueue_iteration(const SceneView<R>& sv, const WaveView<R>& v, const RenderConsts& rc, WaveCounters* ctr,
                       int g_logic, int g_trace, cudaStream_t stream, cudaEvent_t* ev,
                       const JobView<R>* jobs = nullptr, int num_jobs = 0, int parity = 0, bool regen = true) {
    (void)g_trace;
    constexpr bool compact = compact_shading<DIRECT, BATCH, LOGIC>();
    WaveView<R> vq = v;
    if constexpr (compact) {
        // parity p reads extension queue p and carry queue p, fills extension queue 1-p (traced
        // this iteration) and carry queue 1-p
        int* const cnt_e0 = &ctr->ext_count;
        int* const cnt_e1 = &ctr->ext_count_b;
        vq.ext_in = parity ? v.ext_queue_b : v.ext_queue;
        vq.ext_in_count = parity ? cnt_e1 : cnt_e0;
        vq.ext_queue = parity ? v.ext_queue : v.ext_queue_b;
        vq.ext_count = parity ? cnt_e0 : cnt_e1;
        vq.carry_in = parity ? v.carry_b : v.carry_a;
        vq.carry_in_count = &ctr->carry_count[parity];
        vq.carry_out = parity ? v.carry_a : v.carry_b;
        vq.carry_out_count = &ctr->carry_count[1 - parity];
        k_iteration_begin<<<1, 32, 0, stream>>>(ctr, parity);
    } else {
        const size_t off = offsetof(WaveCounters, ext_count);
        const size_t len = offsetof(WaveCounters, error_flags) - off;
        cudaMemsetAsync((char*)ctr + off, 0, len, stream);
    }
    if (ev) cudaEventRecord(ev[0], stream);
    const size_t adj_bytes = (ADJ && rc.num_prims <= kAdjSmemPrims) ? 6 * sizeof(float) * rc.num_prims : 0;
    if constexpr (LOGIC == kLogicBdpt)
        k_logic_bdpt<R><<<g_logic, kLogicBlock, 0, stream>>>(sv, v, rc);
    else if constexpr (LOGIC == kLogicLight)
        k_logic_lt<R, DIRECT><<<g_logic, kLogicBlock, 0, stream>>>(sv, v, rc);
    else if constexpr (compact) {
        k_logic<R, DIRECT, ADJ, BATCH, kLogicShadeQ><<<g_logic, kLogicBlock, 0, stream>>>(sv, vq, rc, jobs, num_jobs);
        if (regen)
            k_logic<R, DIRECT, ADJ, BATCH, kLogicRegen><<<g_logic, kLogicBlock, 0, stream>>>(sv, vq, rc, jobs, num_jobs);
    } else {
        k_logic<R, DIRECT, ADJ, BATCH><<<g_logic, kLogicBlock, DIRECT ? 0 : adj_bytes, stream>>>(sv, v, rc, jobs, num_jobs);
    }
    if (ev) cudaEventRecord(ev[1], stream);
    const int refill = rc.trace_refill > 0 ? rc.trace_refill : kRefillLanes;
    k_trace<R, STATS, ADJ, BATCH><<<trace_grid<R, STATS, ADJ, BATCH>(), kTraceBlock, adj_bytes, stream>>>(
        sv, vq, refill, rc.num_prims, jobs);
    if (ev) cudaEventRecord(ev[2], stream);
}

template <typename R, bool DIRECT, bool STATS, bool ADJ = false, bool BATCH = false, int LOGIC = 0>
void run_wave(HostScene& hs, RenderWave* wv, WaveView<R> v, RenderConsts rc, int iters_per_graph,
              bool kernel_timing, cudaStream_t stream, const JobView<R>* jobs = nullptr, int num_jobs = 0) {
    DeviceScene& ds = *hs.dev;
    const SceneView<R> sv = make_view<R>(ds);
    const int g_logic = grid_for(v.Q, kLogicBlock);
    const int g_trace = grid_for(2 * v.Q, 256);

    CUDA_CHECK(cudaMemsetAsync(v.state, SLOT_EMPTY, (size_t)v.Q, stream));
    CUDA_CHECK(cudaMemsetAsync(wv->ctr, 0, sizeof(WaveCounters), stream));
    constexpr bool compact = compact_shading<DIRECT, BATCH, LOGIC>();
    // A queued wave that holds every sample starts them all in its first iteration, slot i with
    // sample i (no claims on the sample counter); after it, the regeneration kernel could only mark
    // ended slots done, which nothing reads with queued shading, so the later iterations leave it out
    // (terrain: 0.22 ms per 16-spp render).
    const bool one_pass = compact && (long long)v.Q >= rc.num_samples;
    rc.one_pass = one_pass ? 1 : 0;
    if constexpr (compact) {
        k_wave_init_slots<<<(v.Q + 255) / 256, 256, 0, stream>>>(v.regen_queue, v.Q, wv->ctr,
                                                                  one_pass ? (unsigned long long)v.Q : 0ull);
        CUDA_CHECK(cudaGetLastError());
        iters_per_graph += iters_per_graph & 1;  // queue parity must restart at 0 with every graph launch
    }

    trace_grid<R, STATS, ADJ, BATCH>();
    // the wave's end in one launch (k_finish): pt and ptdirect camera paths, single renders, batches
    // and the adjoint, outside the measurement renders (which time or count the wavefront kernels)
    constexpr bool finish = (LOGIC == kLogicCamera || LOGIC == kLogicCameraQ) && !STATS;
    // Captures n iterations into `exec`: an update of the wave's executable graph when it has one
    // (same launches, this render's arguments), otherwise a new instantiation. first: the graph's
    // first iteration may start samples.
    auto capture = [&](int n, cudaGraphExec_t& exec_slot, bool first) {
        cudaGraph_t graph = nullptr;
        CUDA_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < n; it++)
            enqueue_iteration<R, DIRECT, STATS, ADJ, BATCH, LOGIC>(sv, v, rc, wv->ctr, g_logic, g_trace, stream,
                                                                   nullptr, jobs, num_jobs, it & 1,
                                                                   !one_pass || (first && it == 0));
        const cudaError_t cap = cudaStreamEndCapture(stream, &graph);
        if (cap != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            throw DeviceError(std::string("graph capture failed: ") + cudaGetErrorString(cap));
        }
        if (exec_slot) {
            cudaGraphExecUpdateResultInfo info{};
            if (cudaGraphExecUpdate(exec_slot, graph, &info) == cudaSuccess) {
                cudaGraphDestroy(graph);
                return;
            }
            cudaGetLastError();  // a refused update: instantiate instead
            cudaGraphExecDestroy(exec_slot);
            exec_slot = nullptr;
        }
        const cudaError_t inst = cudaGraphInstantiate(&exec_slot, graph, 0);
        cudaGraphDestroy(graph);
        if (inst != cudaSuccess) {
            exec_slot = nullptr;
            throw DeviceError(std::string("graph instantiate failed: ") + cudaGetErrorString(inst));
        }
    };
    // Once every sample is claimed, the wave drains: the host then reads the counters after every
    // drain graph (two iterations, one outside compacted shading) so that the wave-end launch starts
    // as soon as few paths remain, instead of at the next multiple of iters_per_graph. (One-iteration
    // drain graphs for compacted shading, one per queue parity, were slower: the terrain still reaches
    // the wave-end threshold at iteration 6, and the extra counter reads cost 13.22 -> 13.27 ms per
    // render, Cornell box 6,960 -> 6,857 Mrays/s.)
    const int drain_iters = compact ? 2 : 1;
    cudaGraphExec_t exec = nullptr, exec_drain = nullptr;
    if (!kernel_timing) {
        static const char kind_tag = 0;  // one per instantiation of run_wave
        WaveGraphs* wg = nullptr;
        for (WaveGraphs& g : wv->graphs)
            if (g.kind == &kind_tag && g.iters == iters_per_graph && g.one_pass == one_pass) wg = &g;
        if (!wg) {
            wv->graphs.push_back(WaveGraphs{&kind_tag, iters_per_graph, one_pass, nullptr, nullptr});
            wg = &wv->graphs.back();
        }
        capture(iters_per_graph, wg->main, true);
        if (finish && drain_iters < iters_per_graph) capture(drain_iters, wg->drain, false);
        exec = wg->main;
        exec_drain = (finish && drain_iters < iters_per_graph) ? wg->drain : nullptr;
    }
    cudaEvent_t kev[3] = {nullptr, nullptr, nullptr};
    double kms[2] = {0, 0};
    bool draining = false;
    long long finish_paths = 0;
    long long launches = 0;

    long long iterations = 0;
    // Each path ends within (max vertices) iterations after it starts; the bound below is
    // generous and only guards against a logic error spinning forever.
    const long long per_slot = (long long)((rc.num_samples + v.Q - 1) / v.Q) + 1;
    const long long mv = rc.max_vertices > 0 ? rc.max_vertices : (LOGIC == kLogicBdpt ? kBdptMaxVertices : 4096);
    // bdpt: two subpaths, then its strategies two at a time
    const long long per_path = LOGIC == kLogicBdpt ? 2 * mv + mv * mv + 8 : mv + 2;
    const long long max_iters = per_slot * per_path + 64;
    try {
        if (kernel_timing)
            for (auto& e : kev) CUDA_CHECK(cudaEventCreate(&e));
        CUDA_CHECK(cudaEventRecord(wv->ev0, stream));
        while (true) {
            if (kernel_timing) {
                enqueue_iteration<R, DIRECT, STATS, ADJ, BATCH, LOGIC>(sv, v, rc, wv->ctr, g_logic, g_trace, stream,
                                                                       kev, jobs, num_jobs, (int)(iterations & 1),
                                                                       !one_pass || iterations == 0);
                CUDA_CHECK(cudaGetLastError());
                CUDA_CHECK(cudaEventSynchronize(kev[2]));
                for (int k = 0; k < 2; k++) {
                    float t = 0;
                    CUDA_CHECK(cudaEventElapsedTime(&t, kev[k], kev[k + 1]));
                    kms[k] += t;
                }
                launches++;
                iterations++;
            } else {
                CUDA_CHECK(cudaGraphLaunch(draining ? exec_drain : exec, stream));
                iterations += draining ? drain_iters : iters_per_graph;
            }
            CUDA_CHECK(cudaMemcpyAsync(wv->h_ctr, wv->ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, stream));
            CUDA_CHECK(cudaStreamSynchronize(stream));
            if (wv->h_ctr->error_flags & 1)
                throw DeviceError("traversal stack overflow", NGI_ERR_UNSUPPORTED);
            if (wv->h_ctr->error_flags & 2)
                throw DeviceError("adjoint path longer than 16 surface vertices", NGI_ERR_UNSUPPORTED);
            if (wv->h_ctr->active == 0 && wv->h_ctr->next_sample >= (unsigned long long)rc.num_samples) break;
            if constexpr (finish) {
                // every sample claimed and few paths left: run them to their end in one launch
                const int pending = wv->h_ctr->ext_count;
                const bool claimed = wv->h_ctr->next_sample >= (unsigned long long)rc.num_samples;
                if (claimed && exec_drain) draining = true;
                if (!kernel_timing && claimed && pending <= kFinishMaxPaths) {
                    if (pending > 0) {
                        const size_t finish_smem =
                            (ADJ && rc.num_prims <= kAdjSmemPrims) ? 6 * sizeof(float) * rc.num_prims : 0;
                        k_finish<R, DIRECT, BATCH, ADJ>
                            <<<(pending + kFinishBlock - 1) / kFinishBlock, kFinishBlock, finish_smem, stream>>>(
                                sv, v, rc, jobs);
                        CUDA_CHECK(cudaGetLastError());
                        CUDA_CHECK(cudaMemcpyAsync(wv->h_ctr, wv->ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost,
                                                   stream));
                        CUDA_CHECK(cudaStreamSynchronize(stream));
                        if (wv->h_ctr->error_flags & 1) throw DeviceError("traversal stack overflow", NGI_ERR_UNSUPPORTED);
                        if (wv->h_ctr->error_flags & 2)
                            throw DeviceError("adjoint path longer than 16 surface vertices", NGI_ERR_UNSUPPORTED);
                        if (wv->h_ctr->error_flags & 4)
                            throw DeviceError("a path outran the wave-end vertex cap", NGI_ERR_DEVICE_TIMEOUT);
                        finish_paths = pending;
                    }
                    break;
                }
            }
            if (iterations > max_iters) throw DeviceError("wave did not drain", NGI_ERR_DEVICE_TIMEOUT);
        }
        CUDA_CHECK(cudaEventRecord(wv->ev1, stream));
        CUDA_CHECK(cudaEventSynchronize(wv->ev1));
    } catch (...) {
        cudaStreamSynchronize(stream);  // the wave keeps its graphs
        for (auto& e : kev)
            if (e) cudaEventDestroy(e);
        throw;
    }
    for (auto& e : kev)
        if (e) cudaEventDestroy(e);
    float ms = 0;
    cudaEventElapsedTime(&ms, wv->ev0, wv->ev1);
    const WaveCounters& c = *wv->h_ctr;
    ds.last_stats.logic_ms = kms[0];
    ds.last_stats.logic_launches = ds.last_stats.extend_launches = launches;
    // one traversal launch traces both queues: its time is extend_ms, no shadow launch exists
    ds.last_stats.extend_ms = kms[1];
    ds.last_stats.shadow_ms = 0;
    ds.last_stats.shadow_launches = 0;
    ds.last_stats.extend_nodes = (int64_t)c.ext_nodes;
    ds.last_stats.extend_tris = (int64_t)c.ext_tris;
    ds.last_stats.shadow_nodes = (int64_t)c.sh_nodes;
    ds.last_stats.shadow_tris = (int64_t)c.sh_tris;
    ds.last_stats.camera_rays = (int64_t)c.stat_camera;
    ds.last_stats.extension_rays = (int64_t)c.stat_ext;
    ds.last_stats.shadow_rays = (int64_t)c.stat_shadow;
    ds.last_stats.film_contributions = (int64_t)c.stat_contrib;
    ds.last_stats.nonfinite = (int64_t)c.stat_nonfinite;
    ds.last_stats.iterations = iterations;
    ds.last_stats.render_ms = ms;
    ds.last_stats.finish_paths = finish_paths;
}

}  // namespace

namespace {

// Per-slot subpath vertices and cursors of bdpt, allocated with the wave the first time it runs bdpt.
template <typename R>
void ensure_bdpt_buffers(RenderWave* wv, WaveView<R>& v) {
    if (wv->bdpt_precision >= 0) return;
    void* a = nullptr;
    void* b = nullptr;
    CUDA_CHECK(cudaMalloc(&a, sizeof(BdVert<R>) * 2 * kBdptMaxVertices * (size_t)wv->Q));
    wv->bufs.push_back(a);
    CUDA_CHECK(cudaMalloc(&b, sizeof(int4) * (size_t)wv->Q));
    wv->bufs.push_back(b);
    v.bd_verts = (BdVert<R>*)a;
    v.bd_info = (int4*)b;
    wv->bdpt_precision = wv->precision;
}

// Kernel constants of a render with parameters p on a scene of num_prims primitives.
RenderConsts consts_of(const ngi_render_params& p, int num_prims) {
    RenderConsts rc{};
    rc.renderer = p.renderer;
    rc.max_vertices = p.max_num_vertices;
    rc.num_samples = p.num_samples;
    rc.sample_offset = p.sample_offset;
    rc.seed = p.seed;
    rc.width = p.width;
    rc.height = p.height;
    rc.stratified = p.raster_mode == NGI_RASTER_STRATIFIED ? 1 : 0;
    const long long wh = (long long)p.width * p.height;
    rc.strat_end = ((p.sample_offset + p.num_samples) / wh) * wh;
    rc.trace_refill = p.trace_refill;
    rc.ray_offset = p.ray_offset;
    rc.trace_all = (p.flags & NGI_RENDER_TRACE_ALL_RAYS) ? 1 : 0;
    rc.num_prims = num_prims;
    return rc;
}

}  // namespace

void DeviceRender(HostScene& hs, const ngi_render_params& p, double* d_film, cudaStream_t user_stream) {
    DeviceUpload(hs);
    DeviceScene& ds = *hs.dev;
    RequireSceneDevice(ds);
    if (hs.sensor_prim < 0) throw DeviceError("the scene has no sensor (E) primitive", NGI_ERR_INVALID_ARGUMENT);
    if (p.renderer != NGI_RENDERER_PT && ds.num_lights == 0)
        throw DeviceError("this renderer needs at least one light (the reference indexes an empty light list)",
                          NGI_ERR_UNSUPPORTED);
    cudaStream_t stream = user_stream ? user_stream : ds.stream;
    ds.last_stats = ngi_render_stats{};
    if (p.num_samples == 0) return;
    const bool bdpt = p.renderer == NGI_RENDERER_BDPT;
    // Path slots of the wave (never more than the render's samples). A slot takes about 257 B in
    // FP32 (101 B of path state, three shadow-ray entries) and 400 B in FP64. ptdirect: 2^25
    // (8.6 GB FP32). Each iteration pays a fixed tail (the slowest ray of its traversal launch, the
    // ramp of its logic launches), which a larger wave spreads over more rays, and its shading
    // visits only queued slots. Terrain, with the wave-end launch: 14.75 ms per 16-spp render at
    // 2^23, 14.36 at 2^25 (every sample in flight at once); 65.5 against 54.9 ms per 64-spp render.
    // pt runs the same queued kernels when every sample fits in one such wave (Cornell box bench,
    // 4.2M samples: 6,070 against 4,880 Mrays/s with the fused kernel); longer pt renders keep the
    // fused kernel and 2^23 slots, which wins in a steady state (the Cornell box's 67M-sample
    // convergence renders: 0.218 s to 1% error fused at 2^23, 0.250 s queued at 2^25, 0.466 s queued
    // at 2^23). lt and ltdirect keep 2^23: their logic kernel visits every slot of the wave in each
    // iteration. bdpt keeps 2 x 32 path vertices per slot (3.8 KB FP32, 6.7 KB FP64): 2^18. A smaller
    // default for scenes with a small BVH (2^20 below 32 MB) was measured and not kept: the Cornell box
    // bench ran at 4995 against 4050 Mrays/s, but its convergence study took 0.253 against 0.225 s and
    // the 256-job batch rendered one job at a time 3719 against 4431 Mrays/s.
    const bool pt_queued = p.renderer == NGI_RENDERER_PT &&
                           (p.wave_size > 0 ? (long long)p.wave_size >= p.num_samples : p.num_samples <= (1LL << 25));
    const bool compacted = p.renderer == NGI_RENDERER_PTDIRECT || pt_queued;
    int Q = p.wave_size > 0 ? p.wave_size : (bdpt ? (1 << 18) : (compacted ? (1 << 25) : (1 << 23)));
    const long long need = std::max<long long>(p.num_samples, 256);
    if ((long long)Q > need) Q = (int)need;
    Q = (Q + 255) / 256 * 256;
    RenderWave* wv = ensure_wave(ds, Q, p.precision);
    const RenderConsts rc = consts_of(p, (int)hs.prims.size());
    // Wave iterations between two reads of the counters. A compacted wave that holds every sample
    // runs 6 in its first graph, after which the terrain is below the wave end's threshold without a
    // drain graph and its host round trip: 12.85 against 12.89 ms per 16-spp render, Cornell box bench
    // 7,060 against 6,999 Mrays/s, interior 15.31 against 15.33 ms per 16-spp render. 8 was slower on
    // the terrain (13.07 ms: two more wavefront iterations instead of the wave-end launch). Other
    // waves run 4.
    const bool holds_all = compacted && (long long)wv->Q >= p.num_samples;
    const int ipg = p.iterations_per_graph > 0 ? p.iterations_per_graph : (holds_all ? 6 : 4);
    const bool timing = (p.flags & NGI_RENDER_KERNEL_TIMING) != 0;
    const bool counters = (p.flags & NGI_RENDER_TRAVERSAL_COUNTERS) != 0;
    const bool direct = p.renderer == NGI_RENDERER_PTDIRECT || p.renderer == NGI_RENDERER_LTDIRECT;
    const bool light = p.renderer == NGI_RENDERER_LT || p.renderer == NGI_RENDERER_LTDIRECT;
    if (bdpt) {
        if (p.precision == NGI_PRECISION_FP64) {
            ensure_bdpt_buffers<double>(wv, wv->vd);
            WaveView<double> v = wv->vd;
            v.film = d_film;
            run_wave<double, false, false, false, false, kLogicBdpt>(hs, wv, v, rc, ipg, timing, stream);
        } else {
            ensure_bdpt_buffers<float>(wv, wv->vf);
            WaveView<float> v = wv->vf;
            v.film = d_film;
            run_wave<float, false, false, false, false, kLogicBdpt>(hs, wv, v, rc, ipg, timing, stream);
        }
    } else if (light) {
        if (p.precision == NGI_PRECISION_FP64) {
            WaveView<double> v = wv->vd;
            v.film = d_film;
            if (direct) run_wave<double, true, false, false, false, kLogicLight>(hs, wv, v, rc, ipg, timing, stream);
            else run_wave<double, false, false, false, false, kLogicLight>(hs, wv, v, rc, ipg, timing, stream);
        } else {
            WaveView<float> v = wv->vf;
            v.film = d_film;
            if (direct) run_wave<float, true, false, false, false, kLogicLight>(hs, wv, v, rc, ipg, timing, stream);
            else run_wave<float, false, false, false, false, kLogicLight>(hs, wv, v, rc, ipg, timing, stream);
        }
    } else if (p.precision == NGI_PRECISION_FP64) {
        WaveView<double> v = wv->vd;
        v.film = d_film;
        if (direct) run_wave<double, true, false>(hs, wv, v, rc, ipg, timing, stream);
        else if (pt_queued) run_wave<double, false, false, false, false, kLogicCameraQ>(hs, wv, v, rc, ipg, timing, stream);
        else run_wave<double, false, false>(hs, wv, v, rc, ipg, timing, stream);
    } else {
        WaveView<float> v = wv->vf;
        v.film = d_film;
        if (direct) {
            if (counters) run_wave<float, true, true>(hs, wv, v, rc, ipg, timing, stream);
            else run_wave<float, true, false>(hs, wv, v, rc, ipg, timing, stream);
        } else {
            if (counters) run_wave<float, false, true>(hs, wv, v, rc, ipg, timing, stream);
            else if (pt_queued) run_wave<float, false, false, false, false, kLogicCameraQ>(hs, wv, v, rc, ipg, timing, stream);
            else run_wave<float, false, false>(hs, wv, v, rc, ipg, timing, stream);
        }
    }
}

__global__ void k_scale(double* film, size_t n, double s) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        film[i] *= s;
}

void DeviceRenderToHost(HostScene& hs, const ngi_render_params& p, double* h_film) {
    DeviceUpload(hs);
    DeviceScene& ds = *hs.dev;
    RequireSceneDevice(ds);
    const size_t elems = 3 * (size_t)p.width * (size_t)p.height;
    if (ds.film_elems < elems) {
        if (ds.film) cudaFree(ds.film);
        ds.film = nullptr;
        ds.film_elems = 0;
        CUDA_CHECK(cudaMalloc(&ds.film, elems * sizeof(double)));
        ds.film_elems = elems;
    }
    CUDA_CHECK(cudaMemsetAsync(ds.film, 0, elems * sizeof(double), ds.stream));
    DeviceRender(hs, p, ds.film, ds.stream);
    if (p.num_samples > 0) {
        // RenderProcess gather: film *= W*H / processedSamples (src/nanogi.cpp:434-437)
        const double scale = (double)p.width * (double)p.height / (double)p.num_samples;
        k_scale<<<grid_for((int)std::min<size_t>(elems, 1u << 30), 256), 256, 0, ds.stream>>>(ds.film, elems, scale);
        CUDA_CHECK(cudaGetLastError());
    }
    CUDA_CHECK(cudaMemcpyAsync(h_film, ds.film, elems * sizeof(double), cudaMemcpyDeviceToHost, ds.stream));
    CUDA_CHECK(cudaStreamSynchronize(ds.stream));
}

void DeviceIntersect(HostScene& hs, const float* h_rays, int64_t n, int32_t* prim, float* t, float* uv) {
    DeviceUpload(hs);
    DeviceScene& ds = *hs.dev;
    RequireSceneDevice(ds);
    if (n == 0) return;
    float4* d_rays = nullptr;
    int32_t* d_prim = nullptr;
    float *d_t = nullptr, *d_uv = nullptr;
    int* d_err = nullptr;
    auto cleanup = [&]() { cudaFree(d_rays); cudaFree(d_prim); cudaFree(d_t); cudaFree(d_uv); cudaFree(d_err); };
    try {
        CUDA_CHECK(cudaMalloc(&d_rays, sizeof(float4) * 2 * n));
        CUDA_CHECK(cudaMalloc(&d_prim, sizeof(int32_t) * n));
        CUDA_CHECK(cudaMalloc(&d_t, sizeof(float) * n));
        CUDA_CHECK(cudaMalloc(&d_uv, sizeof(float) * 2 * n));
        CUDA_CHECK(cudaMalloc(&d_err, sizeof(int)));
        CUDA_CHECK(cudaMemsetAsync(d_err, 0, sizeof(int), ds.stream));
        CUDA_CHECK(cudaMemcpyAsync(d_rays, h_rays, sizeof(float) * 8 * n, cudaMemcpyHostToDevice, ds.stream));
        const int block = 256;
        const int grid = (int)std::min<int64_t>((n + block - 1) / block, 152 * 16);
        k_intersect<<<grid, block, 0, ds.stream>>>(ds.nodes, ds.tris, ds.num_nodes, d_rays, n, d_prim, d_t, d_uv, d_err);
        CUDA_CHECK(cudaGetLastError());
        int err = 0;
        CUDA_CHECK(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ds.stream));
        std::vector<int32_t> hp(prim ? 0 : n);
        std::vector<float> ht(t ? 0 : n), huv(uv ? 0 : 2 * n);
        CUDA_CHECK(cudaMemcpyAsync(prim ? prim : hp.data(), d_prim, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ds.stream));
        CUDA_CHECK(cudaMemcpyAsync(t ? t : ht.data(), d_t, sizeof(float) * n, cudaMemcpyDeviceToHost, ds.stream));
        CUDA_CHECK(cudaMemcpyAsync(uv ? uv : huv.data(), d_uv, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, ds.stream));
        CUDA_CHECK(cudaStreamSynchronize(ds.stream));
        if (err) throw DeviceError("traversal stack overflow", NGI_ERR_UNSUPPORTED);
    } catch (...) {
        cudaStreamSynchronize(ds.stream);
        cleanup();
        throw;
    }
    cleanup();
}

void DeviceVisible(HostScene& hs, const double* h_pts, int64_t n, uint8_t* vis) {
    DeviceUpload(hs);
    DeviceScene& ds = *hs.dev;
    RequireSceneDevice(ds);
    if (n == 0) return;
    double* d_pts = nullptr;
    uint8_t* d_vis = nullptr;
    int* d_err = nullptr;
    auto cleanup = [&]() { cudaFree(d_pts); cudaFree(d_vis); cudaFree(d_err); };
    try {
        CUDA_CHECK(cudaMalloc(&d_pts, sizeof(double) * 6 * n));
        CUDA_CHECK(cudaMalloc(&d_vis, n));
        CUDA_CHECK(cudaMalloc(&d_err, sizeof(int)));
        CUDA_CHECK(cudaMemsetAsync(d_err, 0, sizeof(int), ds.stream));
        CUDA_CHECK(cudaMemcpyAsync(d_pts, h_pts, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, ds.stream));
        const int block = 256;
        const int grid = (int)std::min<int64_t>((n + block - 1) / block, 152 * 16);
        k_visible<<<grid, block, 0, ds.stream>>>(ds.nodes, ds.tris, ds.num_nodes, d_pts, n, d_vis, d_err);
        CUDA_CHECK(cudaGetLastError());
        int err = 0;
        CUDA_CHECK(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ds.stream));
        CUDA_CHECK(cudaMemcpyAsync(vis, d_vis, n, cudaMemcpyDeviceToHost, ds.stream));
        CUDA_CHECK(cudaStreamSynchronize(ds.stream));
        if (err) throw DeviceError("traversal stack overflow", NGI_ERR_UNSUPPORTED);
    } catch (...) {
        cudaStreamSynchronize(ds.stream);
        cleanup();
        throw;
    }
    cleanup();
}

void DeviceUpdateTables(HostScene& hs) {
    DeviceScene* ds = hs.dev;
    if (!ds) return;
    std::vector<DevMaterial<float>> mf; std::vector<DevLight<float>> lf; DevSensor<float> sf;
    std::vector<DevMaterial<double>> md; std::vector<DevLight<double>> ld; DevSensor<double> sd;
    std::vector<double> cdf; std::vector<float> epos, euv;
    build_tables<float>(hs, mf, lf, sf, cdf, epos, euv);
    build_tables<double>(hs, md, ld, sd, cdf, epos, euv);
    CUDA_CHECK(cudaStreamSynchronize(ds->stream));
    if (!mf.empty()) {
        CUDA_CHECK(cudaMemcpy(ds->mats_f, mf.data(), mf.size() * sizeof(mf[0]), cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(ds->mats_d, md.data(), md.size() * sizeof(md[0]), cudaMemcpyHostToDevice));
    }
    if (!lf.empty()) {
        CUDA_CHECK(cudaMemcpy(ds->lights_f, lf.data(), lf.size() * sizeof(lf[0]), cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(ds->lights_d, ld.data(), ld.size() * sizeof(ld[0]), cudaMemcpyHostToDevice));
    }
    std::memcpy(ds->sensor_f, &sf, sizeof(sf));
    std::memcpy(ds->sensor_d, &sd, sizeof(sd));
}

namespace {

template <typename R>
void ensure_adjoint_buffers(RenderWave* wv, WaveView<R>& v) {
    if (!wv->adjoint_buffers) {
        auto A = [&](size_t bytes) -> void* {
            void* p = nullptr;
            CUDA_CHECK(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
            wv->bufs.push_back(p);
            return p;
        };
        v.pre = (uint4*)A(sizeof(uint4) * 2 * (size_t)wv->Q);
        v.sh_pre = (uint4*)A(sizeof(uint4) * 2 * kShadowPerSlot * (size_t)wv->Q);
        v.sh_info = (int2*)A(sizeof(int2) * kShadowPerSlot * (size_t)wv->Q);
        wv->adjoint_buffers = true;
    }
}

template <typename R, bool DIRECT>
void run_backward(HostScene& hs, RenderWave* wv, WaveView<R>& v, const RenderConsts& rc, int ipg, cudaStream_t stream) {
    ensure_adjoint_buffers(wv, v);
    run_wave<R, DIRECT, false, true>(hs, wv, v, rc, ipg, false, stream);
}

}  // namespace

void DeviceRenderBackward(HostScene& hs, const ngi_render_params& p, const double* h_dfilm, double* grad_albedo,
                          double* grad_emission) {
    DeviceUpload(hs);
    DeviceScene& ds = *hs.dev;
    RequireSceneDevice(ds);
    if (hs.sensor_prim < 0) throw DeviceError("the scene has no sensor (E) primitive", NGI_ERR_INVALID_ARGUMENT);
    if (p.renderer == NGI_RENDERER_PTDIRECT && ds.num_lights == 0)
        throw DeviceError("ptdirect needs at least one light", NGI_ERR_UNSUPPORTED);
    if (p.max_num_vertices == -1 || p.max_num_vertices > kAdjMaxPrefix + 1)
        throw DeviceError("the adjoint replays paths of at most 17 vertices: set max_num_vertices to 1..17",
                          NGI_ERR_UNSUPPORTED);
    if (hs.prims.size() > 65535) throw DeviceError("the adjoint supports at most 65535 primitives", NGI_ERR_UNSUPPORTED);
    if ((p.flags & ~NGI_RENDER_TRACE_ALL_RAYS) != 0)
        throw DeviceError("measurement flags are not available on the adjoint", NGI_ERR_INVALID_ARGUMENT);
    const size_t np = hs.prims.size();
    const size_t elems = 3 * (size_t)p.width * (size_t)p.height;
    auto ensure = [&](double*& buf, size_t& have, size_t need) {
        if (have < need) {
            if (buf) cudaFree(buf);
            buf = nullptr;
            have = 0;
            CUDA_CHECK(cudaMalloc(&buf, std::max<size_t>(need, 1) * sizeof(double)));
            have = need;
        }
    };
    ensure(ds.film, ds.film_elems, elems);
    ensure(ds.adj, ds.adj_elems, elems);
    ensure(ds.grads, ds.grad_elems, 6 * np);
    cudaStream_t stream = ds.stream;
    CUDA_CHECK(cudaMemsetAsync(ds.grads, 0, 6 * np * sizeof(double), stream));
    ds.last_stats = ngi_render_stats{};
    if (p.num_samples > 0) {
        CUDA_CHECK(cudaMemsetAsync(ds.film, 0, elems * sizeof(double), stream));
        CUDA_CHECK(cudaMemcpyAsync(ds.adj, h_dfilm, elems * sizeof(double), cudaMemcpyHostToDevice, stream));
        // the film is normalised by W*H/N, so d(film)/d(raw contribution) = W*H/N
        const double scale = (double)p.width * (double)p.height / (double)p.num_samples;
        k_scale<<<grid_for((int)std::min<size_t>(elems, 1u << 30), 256), 256, 0, stream>>>(ds.adj, elems, scale);
        CUDA_CHECK(cudaGetLastError());
        // ptdirect: the forward render's 2^25 slots (the inverse box, 512x512 at 64 spp: backward
        // 9.93 ms with every sample in flight against 11.32 ms at 2^22); pt keeps 2^22
        const bool direct = p.renderer == NGI_RENDERER_PTDIRECT;
        int Q = p.wave_size > 0 ? p.wave_size : (direct ? (1 << 25) : (1 << 22));
        const long long need = std::max<long long>(p.num_samples, 256);
        if ((long long)Q > need) Q = (int)need;
        Q = (Q + 255) / 256 * 256;
        RenderWave* wv = ensure_wave(ds, Q, p.precision);
        const RenderConsts rc = consts_of(p, (int)hs.prims.size());
        const int ipg = p.iterations_per_graph > 0 ? p.iterations_per_graph : 4;
        if (p.precision == NGI_PRECISION_FP64) {
            WaveView<double>& v = wv->vd;
            v.film = ds.film;
            v.adj = ds.adj;
            v.grad_albedo = ds.grads;
            v.grad_emission = ds.grads + 3 * np;
            if (direct) run_backward<double, true>(hs, wv, v, rc, ipg, stream);
            else run_backward<double, false>(hs, wv, v, rc, ipg, stream);
        } else {
            WaveView<float>& v = wv->vf;
            v.film = ds.film;
            v.adj = ds.adj;
            v.grad_albedo = ds.grads;
            v.grad_emission = ds.grads + 3 * np;
            if (direct) run_backward<float, true>(hs, wv, v, rc, ipg, stream);
            else run_backward<float, false>(hs, wv, v, rc, ipg, stream);
        }
    }
    std::vector<double> g(6 * np);
    CUDA_CHECK(cudaMemcpyAsync(g.data(), ds.grads, 6 * np * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_CHECK(cudaStreamSynchronize(stream));
    if (grad_albedo) std::memcpy(grad_albedo, g.data(), 3 * np * sizeof(double));
    if (grad_emission) std::memcpy(grad_emission, g.data() + 3 * np, 3 * np * sizeof(double));
}

// ---- batches ----------------------------------------------------------------------------------
namespace {

template <typename R>
void ensure_batch_buffers(RenderWave* wv, WaveView<R>& v) {
    if (!v.job) {
        void* a = nullptr;
        void* b = nullptr;
        CUDA_CHECK(cudaMalloc(&a, sizeof(int) * (size_t)wv->Q));
        wv->bufs.push_back(a);
        CUDA_CHECK(cudaMalloc(&b, sizeof(int) * kShadowPerSlot * (size_t)wv->Q));
        wv->bufs.push_back(b);
        v.job = (int*)a;
        v.sh_job = (int*)b;
    }
}

struct BatchConfig {
    int wave, refill, ipg;
};

// One batch render of `jobs` (job tables already filled but for films / sample bases);
// returns the device milliseconds of the wave.
template <typename R>
double batch_pass(std::vector<HostScene*>& scenes, const std::vector<ngi_render_params>& params,
                  const std::vector<long long>& samples, double* d_films, const std::vector<size_t>& film_off,
                  const BatchConfig& cfg, int precision, cudaStream_t stream, ngi_batch_stats* st) {
    HostScene& hs0 = *scenes[0];
    DeviceScene& ds0 = *hs0.dev;
    const int n = (int)scenes.size();
    std::vector<JobView<R>> jv(n);
    long long total = 0;
    int max_vertices = 1;
    bool unbounded = false;
    for (int j = 0; j < n; j++) {
        jv[j].sv = make_view<R>(*scenes[j]->dev);
        ngi_render_params p = params[j];
        p.num_samples = samples[j];
        jv[j].rc = consts_of(p, (int)scenes[j]->prims.size());
        jv[j].film = d_films + film_off[j];
        jv[j].sample_base = total;
        total += samples[j];
        if (p.max_num_vertices == -1) unbounded = true;
        max_vertices = std::max(max_vertices, p.max_num_vertices);
    }
    JobView<R>* d_jobs = nullptr;
    CUDA_CHECK(cudaMalloc(&d_jobs, sizeof(JobView<R>) * n));
    double ms = 0;
    try {
        CUDA_CHECK(cudaMemcpyAsync(d_jobs, jv.data(), sizeof(JobView<R>) * n, cudaMemcpyHostToDevice, stream));
        long long need = std::max<long long>(total, 256);
        int Q = (int)std::min<long long>(cfg.wave, need);
        Q = (Q + 255) / 256 * 256;
        RenderWave* wv = ensure_wave(ds0, Q, precision);
        WaveView<R>& v = precision == NGI_PRECISION_FP64 ? *(WaveView<R>*)&wv->vd : *(WaveView<R>*)&wv->vf;
        ensure_batch_buffers(wv, v);
        RenderConsts rc0 = consts_of(params[0], 0);
        rc0.num_samples = total;
        rc0.max_vertices = unbounded ? -1 : max_vertices;
        rc0.trace_refill = cfg.refill;
        WaveView<R> vv = v;
        vv.film = d_films;
        if (total > 0) run_wave<R, false, false, false, true>(hs0, wv, vv, rc0, cfg.ipg, false, stream, d_jobs, n);
        ms = ds0.last_stats.render_ms;
        if (st) {
            st->samples = total;
            st->extension_rays = ds0.last_stats.extension_rays;
            st->shadow_rays = ds0.last_stats.shadow_rays;
            st->iterations = ds0.last_stats.iterations;
        }
    } catch (...) {
        cudaStreamSynchronize(stream);
        cudaFree(d_jobs);
        throw;
    }
    CUDA_CHECK(cudaStreamSynchronize(stream));
    cudaFree(d_jobs);
    return ms;
}

template <typename R>
void render_batch(std::vector<HostScene*>& scenes, const std::vector<ngi_render_params>& params, double* const* films,
                  const ngi_batch_options& opt, ngi_batch_stats* stats) {
    const int n = (int)scenes.size();
    const int precision = params[0].precision;
    DeviceScene& ds0 = *scenes[0]->dev;
    cudaStream_t stream = ds0.stream;
    std::vector<size_t> film_off(n + 1, 0);
    for (int j = 0; j < n; j++) film_off[j + 1] = film_off[j] + 3 * (size_t)params[j].width * params[j].height;
    double* d_films = nullptr;
    CUDA_CHECK(cudaMalloc(&d_films, std::max<size_t>(film_off[n], 1) * sizeof(double)));
    try {
        BatchConfig cfg{opt.wave_size > 0 ? opt.wave_size : (1 << 22), opt.trace_refill > 0 ? opt.trace_refill : kRefillLanes,
                        opt.iterations_per_graph > 0 ? opt.iterations_per_graph : 4};
        double tune_ms = 0;
        int trials = 0;
        if (opt.autotune) {
            // Coordinate search over wave size, refill threshold and graph length on a sample of
            // every job (the trials render into the films, which are cleared afterwards).
            const double frac = opt.autotune_fraction > 0 ? opt.autotune_fraction : 0.02;
            std::vector<long long> trial(n);
            long long trial_total = 0;
            for (int j = 0; j < n; j++) {
                const long long wh = (long long)params[j].width * params[j].height;
                trial[j] = std::min<long long>(params[j].num_samples,
                                               std::max<long long>(wh, (long long)(params[j].num_samples * frac)));
                trial_total += trial[j];
            }
            auto measure = [&](const BatchConfig& c) {
                CUDA_CHECK(cudaMemsetAsync(d_films, 0, film_off[n] * sizeof(double), stream));
                const double ms = batch_pass<R>(scenes, params, trial, d_films, film_off, c, precision, stream, nullptr);
                tune_ms += ms;
                trials++;
                return ms;
            };
            measure(cfg);  // warm: kernels, graphs, wave allocation
            double best = measure(cfg);
            const int waves[] = {1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25};
            for (int wv : waves) {
                if (wv == cfg.wave || wv > std::max<long long>(trial_total, 256) * 2) continue;
                BatchConfig c = cfg;
                c.wave = wv;
                const double ms = measure(c);
                if (ms < best) { best = ms; cfg = c; }
            }
            const int refills[] = {4, 8, 12, 16};
            for (int r : refills) {
                if (r == cfg.refill) continue;
                BatchConfig c = cfg;
                c.refill = r;
                const double ms = measure(c);
                if (ms < best) { best = ms; cfg = c; }
            }
            const int ipgs[] = {2, 4, 8};
            for (int g : ipgs) {
                if (g == cfg.ipg) continue;
                BatchConfig c = cfg;
                c.ipg = g;
                const double ms = measure(c);
                if (ms < best) { best = ms; cfg = c; }
            }
        }
        CUDA_CHECK(cudaMemsetAsync(d_films, 0, film_off[n] * sizeof(double), stream));
        std::vector<long long> samples(n);
        for (int j = 0; j < n; j++) samples[j] = params[j].num_samples;
        ngi_batch_stats st{};
        const double ms = batch_pass<R>(scenes, params, samples, d_films, film_off, cfg, precision, stream, &st);
        for (int j = 0; j < n; j++) {
            const size_t elems = film_off[j + 1] - film_off[j];
            if (params[j].num_samples > 0) {
                const double scale = (double)params[j].width * (double)params[j].height / (double)params[j].num_samples;
                k_scale<<<grid_for((int)std::min<size_t>(elems, 1u << 30), 256), 256, 0, stream>>>(d_films + film_off[j],
                                                                                                 elems, scale);
                CUDA_CHECK(cudaGetLastError());
            }
            if (films[j])
                CUDA_CHECK(cudaMemcpyAsync(films[j], d_films + film_off[j], elems * sizeof(double),
                                           cudaMemcpyDeviceToHost, stream));
        }
        CUDA_CHECK(cudaStreamSynchronize(stream));
        if (stats) {
            *stats = st;
            stats->render_ms = ms;
            stats->autotune_ms = tune_ms;
            stats->trials = trials;
            stats->wave_size = cfg.wave;
            stats->trace_refill = cfg.refill;
            stats->iterations_per_graph = cfg.ipg;
        }
    } catch (...) {
        cudaStreamSynchronize(stream);
        cudaFree(d_films);
        throw;
    }
    cudaFree(d_films);
}

}  // namespace

void DeviceRenderBatch(std::vector<HostScene*>& scenes, const std::vector<ngi_render_params>& params,
                       double* const* films, const ngi_batch_options& opt, ngi_batch_stats* stats) {
    if (scenes.empty()) return;
    for (size_t j = 0; j < scenes.size(); j++) {
        DeviceUpload(*scenes[j]);
        const ngi_render_params& p = params[j];
        if (scenes[j]->sensor_prim < 0)
            throw DeviceError("job " + std::to_string(j) + ": the scene has no sensor (E) primitive", NGI_ERR_INVALID_ARGUMENT);
        if (p.renderer == NGI_RENDERER_PTDIRECT && scenes[j]->dev->num_lights == 0)
            throw DeviceError("job " + std::to_string(j) + ": ptdirect needs at least one light", NGI_ERR_UNSUPPORTED);
        if (p.precision != params[0].precision)
            throw DeviceError("every job of a batch must use the same precision", NGI_ERR_INVALID_ARGUMENT);
        if ((p.flags & ~NGI_RENDER_TRACE_ALL_RAYS) != 0)
            throw DeviceError("measurement flags are not available on batches", NGI_ERR_INVALID_ARGUMENT);
        if (scenes[j]->dev->device != scenes[0]->dev->device)
            throw DeviceError("every scene of a batch must live on the same device", NGI_ERR_INVALID_ARGUMENT);
    }
    RequireSceneDevice(*scenes[0]->dev);
    if (params[0].precision == NGI_PRECISION_FP64) render_batch<double>(scenes, params, films, opt, stats);
    else render_batch<float>(scenes, params, films, opt, stats);
}

// ---- allocation-free render --------------------------------------------------------------------
// Some callers cannot allocate device memory at render time: an application whose own
// allocator owns the whole device, a real-time loop that cannot afford the device-wide
// synchronisation a cudaMalloc/cudaFree may cause, or a process working under a fixed
// device-memory budget. For them the render's scratch (the wave of path slots, its queues
// and counters) lives in one file-scope device array instead of per-call allocations.
//
// kNoAllocScratchBytes is the fixed size of that array. CUDA loads this file's device code on a
// device lazily, the first time any of it runs there, and reserves the array at that moment; the
// device keeps it until the process exits. It bounds the wave at kNoAllocMaxWave path slots (the
// number of samples per call is not bounded: samples stream through the wave). All calls share
// the array and it keeps the last call's contents, so each call clears its counters and slot
// states first; two calls that overlap on the GPU (e.g. on two streams) race on it. Each call
// runs a host loop that reads the wave's counters back and synchronises the stream, so it cannot
// be made while that stream is being captured into a graph.
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
constexpr int kNoAllocMaxWave = 1 << 16;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Carves the wave buffers of Q slots out of `base` (when non-null); returns the bytes used.
template <typename R>
size_t carve_wave(unsigned char* base, int Q, WaveView<R>& v) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> void* {
        void* p = base ? (void*)(base + off) : nullptr;
        off = align256(off + std::max<size_t>(bytes, 16));
        return p;
    };
    v.Q = Q;
    v.ctr = (WaveCounters*)take(sizeof(WaveCounters));
    v.ext_count = v.ctr ? &v.ctr->ext_count : nullptr;
    v.ray_o = (float4*)take(sizeof(float4) * Q);
    v.ray_d = (float4*)take(sizeof(float4) * Q);
    v.hit = (float4*)take(sizeof(float4) * Q);
    v.thr = (Vec4T<R>*)take(sizeof(Vec4T<R>) * Q);
    if (sizeof(R) == 8) {
        v.od_o = (Vec4T<double>*)take(sizeof(Vec4T<double>) * Q);
        v.od_d = (Vec4T<double>*)take(sizeof(Vec4T<double>) * Q);
    } else {
        v.od_o = v.od_d = nullptr;
    }
    v.pixel = (uint32_t*)take(sizeof(uint32_t) * Q);
    v.sample = (unsigned long long*)take(sizeof(unsigned long long) * Q);
    v.nverts = (int*)take(sizeof(int) * Q);
    v.state = (uint8_t*)take(sizeof(uint8_t) * Q);
    v.ext_queue = (int*)take(sizeof(int) * Q);
    v.ext_queue_b = (int*)take(sizeof(int) * Q);
    v.carry_a = (int*)take(sizeof(int) * Q);
    v.carry_b = (int*)take(sizeof(int) * Q);
    v.regen_queue = (int*)take(sizeof(int) * Q);
    v.sh_o = (float4*)take(sizeof(float4) * kShadowPerSlot * (size_t)Q);
    v.sh_d = (float4*)take(sizeof(float4) * kShadowPerSlot * (size_t)Q);
    v.sh_c = (Vec4T<R>*)take(sizeof(Vec4T<R>) * kShadowPerSlot * (size_t)Q);
    v.sh_pix = (uint32_t*)take(sizeof(uint32_t) * kShadowPerSlot * (size_t)Q);
    return off;
}

// Device address of the scratch array, looked up once per device with that device current
// (under a lock: host threads may make their first calls at the same time).
unsigned char* noalloc_scratch_address() {
    static unsigned char* addr[64] = {nullptr};
    static std::mutex lock;
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw DeviceError("device ordinal out of range", NGI_ERR_INVALID_ARGUMENT);
    std::lock_guard<std::mutex> guard(lock);
    if (!addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            throw DeviceError(std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
        addr[dev] = (unsigned char*)p;
    }
    return addr[dev];
}

template <typename R, bool DIRECT>
void run_wave_noalloc(HostScene& hs, WaveView<R> v, const RenderConsts& rc, int ipg, cudaStream_t stream) {
    DeviceScene& ds = *hs.dev;
    const SceneView<R> sv = make_view<R>(ds);
    const int g_logic = grid_for(v.Q, kLogicBlock);
    const int g_trace = grid_for(2 * v.Q, 256);
    CUDA_CHECK(cudaMemsetAsync(v.state, SLOT_EMPTY, (size_t)v.Q, stream));
    CUDA_CHECK(cudaMemsetAsync(v.ctr, 0, sizeof(WaveCounters), stream));
    if constexpr (compact_shading<DIRECT, false, kLogicCamera>())
        k_wave_init_slots<<<(v.Q + 255) / 256, 256, 0, stream>>>(v.regen_queue, v.Q, v.ctr, 0ull);
    const long long per_slot = (long long)((rc.num_samples + v.Q - 1) / v.Q) + 1;
    const long long max_iters = per_slot * (long long)(rc.max_vertices > 0 ? rc.max_vertices + 2 : 4096) + 64;
    WaveCounters h{};
    long long iterations = 0;
    while (true) {
        for (int k = 0; k < ipg; k++)
            enqueue_iteration<R, DIRECT, false>(sv, v, rc, v.ctr, g_logic, g_trace, stream, nullptr, nullptr, 0, k & 1);
        iterations += ipg;
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaMemcpyAsync(&h, v.ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, stream));
        CUDA_CHECK(cudaStreamSynchronize(stream));
        if (h.error_flags & 1) throw DeviceError("traversal stack overflow", NGI_ERR_UNSUPPORTED);
        if (h.active == 0 && h.next_sample >= (unsigned long long)rc.num_samples) break;
        if (iterations > max_iters) throw DeviceError("wave did not drain", NGI_ERR_DEVICE_TIMEOUT);
    }
    ds.last_stats = ngi_render_stats{};
    ds.last_stats.camera_rays = (int64_t)h.stat_camera;
    ds.last_stats.extension_rays = (int64_t)h.stat_ext;
    ds.last_stats.shadow_rays = (int64_t)h.stat_shadow;
    ds.last_stats.film_contributions = (int64_t)h.stat_contrib;
    ds.last_stats.nonfinite = (int64_t)h.stat_nonfinite;
    ds.last_stats.iterations = iterations;
}

}  // namespace

void DeviceRenderNoAlloc(HostScene& hs, const ngi_render_params& p, double* d_film, cudaStream_t user_stream) {
    if (!hs.dev)
        throw DeviceError("the scene is not on the device: call ngi_scene_build first (this entry point allocates "
                          "nothing, so it cannot upload the scene)", NGI_ERR_INVALID_ARGUMENT);
    DeviceScene& ds = *hs.dev;
    RequireSceneDevice(ds);
    if (hs.sensor_prim < 0) throw DeviceError("the scene has no sensor (E) primitive", NGI_ERR_INVALID_ARGUMENT);
    if (p.renderer != NGI_RENDERER_PT && ds.num_lights == 0)
        throw DeviceError("this renderer needs at least one light (the reference indexes an empty light list)",
                          NGI_ERR_UNSUPPORTED);
    if ((p.flags & ~NGI_RENDER_TRACE_ALL_RAYS) != 0)
        throw DeviceError("measurement flags are not available on the allocation-free entry point",
                          NGI_ERR_INVALID_ARGUMENT);
    if (p.wave_size > kNoAllocMaxWave)
        throw DeviceError("wave_size " + std::to_string(p.wave_size) + " exceeds the allocation-free maximum of " +
                              std::to_string(kNoAllocMaxWave) + " path slots",
                          NGI_ERR_INVALID_ARGUMENT);
    cudaStream_t stream = user_stream ? user_stream : ds.stream;
    ds.last_stats = ngi_render_stats{};
    // first call on this device: the array's address (and its reservation, when the render code
    // was not loaded on the device yet); a call with no samples does only this
    unsigned char* base = noalloc_scratch_address();
    if (p.num_samples == 0) return;
    int Q = p.wave_size > 0 ? p.wave_size : kNoAllocMaxWave;
    const long long need = std::max<long long>(p.num_samples, 256);
    if ((long long)Q > need) Q = (int)need;
    Q = (Q + 255) / 256 * 256;
    const RenderConsts rc = consts_of(p, (int)hs.prims.size());
    // iterations between host checks of the wave's counters; an even count, so that the queue
    // parity of compacted shading restarts at 0 with every group
    int ipg = p.iterations_per_graph > 0 ? p.iterations_per_graph : 4;
    ipg += ipg & 1;
    const bool direct = p.renderer == NGI_RENDERER_PTDIRECT;
    if (p.precision == NGI_PRECISION_FP64) {
        WaveView<double> v{};
        if (carve_wave<double>(nullptr, Q, v) > kNoAllocScratchBytes)
            throw DeviceError("allocation-free scratch too small for the wave", NGI_ERR_INVALID_ARGUMENT);
        carve_wave<double>(base, Q, v);
        v.film = d_film;
        if (direct) run_wave_noalloc<double, true>(hs, v, rc, ipg, stream);
        else run_wave_noalloc<double, false>(hs, v, rc, ipg, stream);
    } else {
        WaveView<float> v{};
        if (carve_wave<float>(nullptr, Q, v) > kNoAllocScratchBytes)
            throw DeviceError("allocation-free scratch too small for the wave", NGI_ERR_INVALID_ARGUMENT);
        carve_wave<float>(base, Q, v);
        v.film = d_film;
        if (direct) run_wave_noalloc<float, true>(hs, v, rc, ipg, stream);
        else run_wave_noalloc<float, false>(hs, v, rc, ipg, stream);
    }
}

}  // namespace ngi
