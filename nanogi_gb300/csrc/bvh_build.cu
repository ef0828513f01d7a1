// GPU construction of the compressed 8-wide BVH.
//
// Replaces the Embree build of include/nanogi/rt.hpp:2087-2143. Pipeline (all on device):
//   1. per-triangle bounds and centroid bounds
//   2. pre-splitting (Ernst and Greiner 2007; Karras and Aila 2013): a triangle whose box is
//      far larger than the triangle itself (a long thin strip lying diagonally) becomes several
//      references, the triangle clipped to slabs of its box, each with the tight box of its
//      part; every other triangle is one reference
//   3. 63-bit Morton codes of the reference box centroids, radix sort (CUB)
//   4. binary tree: PLOC clustering of the sorted leaves (Meister and Bittner 2018), leaves
//      renumbered depth-first so every subtree is a contiguous range
//   5. top-down, level-synchronous collapse into 8-wide nodes (Ylitie et al. 2017): a
//      bottom-up pass finds the SAH-optimal way to write every subtree as at most 1..8
//      roots, and each node opens its binary descendants as that minimum says; subtrees of
//      <= 3 triangles become leaves, children are assigned to slots by ray octant, and child
//      boxes are quantised to 8 bits per plane relative to the parent.
//   6. triangles, normals and uvs are gathered into leaf order (a split triangle once per leaf
//      holding one of its references; the watertight test always runs on the whole triangle).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "device_scene.hpp"
#include "ngi_device.cuh"

namespace ngi {

namespace {

constexpr int kLeafMax = 3;   // triangles per leaf child (unary count field holds 1..3)
constexpr uint32_t kLeafFlag = 0x80000000u;
const int kNoParent = -1;

#define BVH_CHECK(x)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess)                                                                \
            throw DeviceError(std::string("CUDA error in BVH build: ") + cudaGetErrorString(e_) \
                              + " at " #x);                                                   \
    } while (0)

__device__ __forceinline__ int float_to_ordered(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__host__ __device__ __forceinline__ float ordered_to_float(int i) {
    int b = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

__global__ void k_tri_bounds(const float* __restrict__ pos, int n, float4* __restrict__ lo,
                             float4* __restrict__ hi, int* __restrict__ cbounds) {
    __shared__ int smin[3][32], smax[3][32];
    int cmin[3] = {INT_MAX, INT_MAX, INT_MAX}, cmax[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* p = pos + 9 * (size_t)i;
        float l[3], h[3];
        for (int k = 0; k < 3; k++) {
            l[k] = fminf(fminf(p[k], p[3 + k]), p[6 + k]);
            h[k] = fmaxf(fmaxf(p[k], p[3 + k]), p[6 + k]);
        }
        lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
        hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
        for (int k = 0; k < 3; k++) {
            const int c = float_to_ordered(0.5f * (l[k] + h[k]));
            cmin[k] = min(cmin[k], c);
            cmax[k] = max(cmax[k], c);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            cmin[k] = min(cmin[k], __shfl_xor_sync(0xFFFFFFFFu, cmin[k], o));
            cmax[k] = max(cmax[k], __shfl_xor_sync(0xFFFFFFFFu, cmax[k], o));
        }
        if (lane == 0) { smin[k][warp] = cmin[k]; smax[k][warp] = cmax[k]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        int a = INT_MAX, b = INT_MIN;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a = min(a, smin[k][w]); b = max(b, smax[k][w]); }
        atomicMin(&cbounds[k], a);
        atomicMax(&cbounds[3 + k], b);
    }
}

__device__ __forceinline__ uint64_t expand_bits21(uint64_t x) {
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
                         const int* __restrict__ cbounds, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 l = lo[i], h = hi[i];
    const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
    uint64_t q[3];
    for (int k = 0; k < 3; k++) {
        const float mn = ordered_to_float(cbounds[k]), mx = ordered_to_float(cbounds[3 + k]);
        const float ext = mx - mn;
        float f = ext > 0.0f ? (c[k] - mn) / ext : 0.0f;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        q[k] = (uint64_t)fminf(f * 2097152.0f, 2097151.0f);
    }
    keys[i] = (expand_bits21(q[0]) << 2) | (expand_bits21(q[1]) << 1) | expand_bits21(q[2]);
    vals[i] = (uint32_t)i;
}

// ---- pre-splitting -----------------------------------------------------------------------------
// A triangle is split when the surface area of its box exceeds kSplitRatio times its own area
// (a flat triangle lying in an axis plane has a ratio of 4, a typical mesh triangle 4-10), into
// min(kMaxPieces, ratio / kSplitRatio) references; the extra references of a scene are capped at
// kSplitBudget times its triangle count by scaling every request down. Each reference is the
// triangle clipped to one of equal slabs along the longest axis of its box: for a long thin
// diagonal triangle the k pieces' boxes add up to about 1/k of the whole box's area. Measured on the
// 10M-triangle interior (16-spp bench steps, Mrays/s): budget 0.5: 986, 1: 1,131, 2: 1,226, 3: 1,223,
// 4: 1,326-1,332 (no request scaled down: 8 builds the same BVH, 2.45 GB against 1.10 GB at 1);
// ratio 8: 1,050 and 32: 1,147 at budget 1, 32: 1,283 at budget 4. The budget only bounds the
// references of a pathological scene.
constexpr float kSplitRatio = 16.0f;
constexpr uint32_t kMaxPieces = 64;
constexpr double kSplitBudget = 4.0;

__global__ void k_split_counts(const float* __restrict__ pos, const float4* __restrict__ lo,
                               const float4* __restrict__ hi, int n, uint32_t* __restrict__ pieces,
                               unsigned long long* __restrict__ extra) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t k = 1;
    if (i < n) {
        const float* p = pos + 9 * (size_t)i;
        const double ax = (double)p[3] - p[0], ay = (double)p[4] - p[1], az = (double)p[5] - p[2];
        const double bx = (double)p[6] - p[0], by = (double)p[7] - p[1], bz = (double)p[8] - p[2];
        const double cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
        const double dx = (double)hi[i].x - lo[i].x, dy = (double)hi[i].y - lo[i].y, dz = (double)hi[i].z - lo[i].z;
        const double box = 2.0 * (dx * dy + dy * dz + dz * dx);
        if (area > 0.0 && box > kSplitRatio * area)
            k = (uint32_t)fmin((double)kMaxPieces, floor(box / (kSplitRatio * area)));
        pieces[i] = k;
    }
    // warp sum of the extra references, one atomic per warp
    unsigned long long e = k - 1;
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
    if ((threadIdx.x & 31) == 0 && e) atomicAdd(extra, e);
}

// Scales every triangle's extra references by `scale` (< 1) to keep within the budget.
__global__ void k_split_scale(uint32_t* __restrict__ pieces, int n, double scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pieces[i] = 1u + (uint32_t)floor((double)(pieces[i] - 1u) * scale);
}

// Sutherland-Hodgman clip of a convex polygon (x, y, z per vertex) against coordinate `axis`
// >= v (keep_ge) or <= v; the cut points get the plane coordinate exactly.
__device__ int clip_polygon(const double (*in)[3], int nin, double (*out)[3], int axis, double v, bool keep_ge) {
    int nout = 0;
    for (int a = 0; a < nin; a++) {
        const int b = a + 1 == nin ? 0 : a + 1;
        const double da = keep_ge ? in[a][axis] - v : v - in[a][axis];
        const double db = keep_ge ? in[b][axis] - v : v - in[b][axis];
        if (da >= 0.0) {
            for (int k = 0; k < 3; k++) out[nout][k] = in[a][k];
            nout++;
        }
        if ((da >= 0.0) != (db >= 0.0)) {
            const double t = da / (da - db);
            for (int k = 0; k < 3; k++) out[nout][k] = in[a][k] + t * (in[b][k] - in[a][k]);
            out[nout][axis] = v;
            nout++;
        }
    }
    return nout;
}

// Writes the references of every triangle: its box, or the boxes of its slab pieces, rounded
// outward to float and clamped to the triangle's own box; ref_tri[r] = the triangle of r.
__global__ void k_split_emit(const float* __restrict__ pos, const float4* __restrict__ lo,
                             const float4* __restrict__ hi, int n, const uint32_t* __restrict__ pieces,
                             const uint32_t* __restrict__ first, float4* __restrict__ ref_lo,
                             float4* __restrict__ ref_hi, uint32_t* __restrict__ ref_tri) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = pieces[i], base = first[i];
    const float4 l = lo[i], h = hi[i];
    if (k <= 1) {
        ref_lo[base] = l;
        ref_hi[base] = h;
        ref_tri[base] = (uint32_t)i;
        return;
    }
    const float ext[3] = {h.x - l.x, h.y - l.y, h.z - l.z};
    const int axis = ext[0] >= ext[1] ? (ext[0] >= ext[2] ? 0 : 2) : (ext[1] >= ext[2] ? 1 : 2);
    const double a0 = axis == 0 ? l.x : (axis == 1 ? l.y : l.z);
    const double a1 = axis == 0 ? h.x : (axis == 1 ? h.y : h.z);
    const float* p = pos + 9 * (size_t)i;
    double tri[3][3];
    for (int v = 0; v < 3; v++)
        for (int c = 0; c < 3; c++) tri[v][c] = p[3 * v + c];
    for (uint32_t j = 0; j < k; j++) {
        // adjacent pieces share the same boundary value, so the pieces cover the triangle
        const double s0 = j == 0 ? a0 : a0 + (a1 - a0) * (double)j / (double)k;
        const double s1 = j + 1 == k ? a1 : a0 + (a1 - a0) * (double)(j + 1) / (double)k;
        double q1[5][3], q2[5][3];
        const int n1 = clip_polygon(tri, 3, q1, axis, s0, true);
        const int n2 = clip_polygon(q1, n1, q2, axis, s1, false);
        double bl[3] = {1e300, 1e300, 1e300}, bh[3] = {-1e300, -1e300, -1e300};
        for (int v = 0; v < n2; v++)
            for (int c = 0; c < 3; c++) {
                bl[c] = fmin(bl[c], q2[v][c]);
                bh[c] = fmax(bh[c], q2[v][c]);
            }
        float4 rl = l, rh = h;
        if (n2 > 0) {
            rl = make_float4(fmaxf(__double2float_rd(bl[0]), l.x), fmaxf(__double2float_rd(bl[1]), l.y),
                             fmaxf(__double2float_rd(bl[2]), l.z), 0.0f);
            rh = make_float4(fminf(__double2float_ru(bh[0]), h.x), fminf(__double2float_ru(bh[1]), h.y),
                             fminf(__double2float_ru(bh[2]), h.z), 0.0f);
        }
        ref_lo[base + j] = rl;
        ref_hi[base + j] = rh;
        ref_tri[base + j] = (uint32_t)i;
    }
}

// Bounds of the reference box centroids (the Morton grid).
__global__ void k_centroid_bounds(const float4* __restrict__ lo, const float4* __restrict__ hi, int n,
                                  int* __restrict__ cbounds) {
    __shared__ int smin[3][32], smax[3][32];
    int cmin[3] = {INT_MAX, INT_MAX, INT_MAX}, cmax[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 l = lo[i], h = hi[i];
        const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
        for (int k = 0; k < 3; k++) {
            const int o = float_to_ordered(c[k]);
            cmin[k] = min(cmin[k], o);
            cmax[k] = max(cmax[k], o);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            cmin[k] = min(cmin[k], __shfl_xor_sync(0xFFFFFFFFu, cmin[k], o));
            cmax[k] = max(cmax[k], __shfl_xor_sync(0xFFFFFFFFu, cmax[k], o));
        }
        if (lane == 0) { smin[k][warp] = cmin[k]; smax[k][warp] = cmax[k]; }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        int a = INT_MAX, b = INT_MIN;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a = min(a, smin[k][w]); b = max(b, smax[k][w]); }
        atomicMin(&cbounds[k], a);
        atomicMax(&cbounds[3 + k], b);
    }
}

// ---- PLOC: parallel locally-ordered clustering (Meister and Bittner, TVCG 2018) --------------
// Clusters start as the Morton-sorted leaves. Each round every cluster finds, within R positions
// on either side, the cluster whose merged box has the least surface area; mutual nearest
// neighbours merge into a new internal node at the lower position, and the array is compacted.
// The binary tree this yields has a lower SAH cost than the radix tree of the same keys.
constexpr int kPlocRadius = 16;
constexpr int kPlocBlock = 256;

__device__ __forceinline__ float merged_area(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    const float x = fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x);
    const float y = fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y);
    const float z = fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z);
    return x * y + y * z + z * x;
}

__global__ void k_leaf_gather(int n, const uint32_t* __restrict__ sorted_tri, const float4* __restrict__ tlo,
                              const float4* __restrict__ thi, float4* __restrict__ leaf_lo,
                              float4* __restrict__ leaf_hi, uint32_t* __restrict__ cl_ref) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t t = sorted_tri[j];
    leaf_lo[j] = tlo[t];
    leaf_hi[j] = thi[t];
    cl_ref[j] = kLeafFlag | (uint32_t)j;
}

__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(int count, const float4* __restrict__ lo,
                                                        const float4* __restrict__ hi, int* __restrict__ nn) {
    __shared__ float4 slo[kPlocBlock + 2 * kPlocRadius], shi[kPlocBlock + 2 * kPlocRadius];
    const int base = blockIdx.x * kPlocBlock - kPlocRadius;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += kPlocBlock) {
        const int j = base + k;
        if (j >= 0 && j < count) {
            slo[k] = lo[j];
            shi[k] = hi[j];
        }
    }
    __syncthreads();
    const int i = blockIdx.x * kPlocBlock + threadIdx.x;
    if (i >= count) return;
    const int li = threadIdx.x + kPlocRadius;
    float best = INFINITY;
    int bj = -1;
    for (int d = -kPlocRadius; d <= kPlocRadius; d++) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= count) continue;
        const float a = merged_area(slo[li], shi[li], slo[li + d], shi[li + d]);
        if (a < best || bj < 0) {  // strict: the lower index wins ties
            best = a;
            bj = j;
        }
    }
    nn[i] = bj;
}

// merge[i] = 1 where i starts a new internal node (mutual pair, lower index), keep[i] = 1 where
// position i survives the round (unmerged, or the new node).
__global__ void k_ploc_flags(int count, const int* __restrict__ nn, int* __restrict__ merge, int* __restrict__ keep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > count) return;
    if (i == count) {  // the scans' total entries
        merge[i] = 0;
        keep[i] = 0;
        return;
    }
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    merge[i] = mutual && i < j ? 1 : 0;
    keep[i] = mutual && i > j ? 0 : 1;
}

__global__ void k_ploc_merge(int count, const int* __restrict__ nn, const int* __restrict__ merge_off,
                             const int* __restrict__ keep_off, const uint32_t* __restrict__ ref,
                             const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t node_base,
                             uint32_t* __restrict__ left, uint32_t* __restrict__ right, float4* __restrict__ int_lo,
                             float4* __restrict__ int_hi, int* __restrict__ int_parent, int* __restrict__ leaf_parent,
                             uint32_t* __restrict__ out_ref, float4* __restrict__ out_lo, float4* __restrict__ out_hi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    if (mutual && i > j) return;  // merged into the pair's lower position
    const int dst = keep_off[i];
    if (!mutual) {
        out_ref[dst] = ref[i];
        out_lo[dst] = lo[i];
        out_hi[dst] = hi[i];
        return;
    }
    const uint32_t node = node_base + (uint32_t)merge_off[i];
    const uint32_t a = ref[i], b = ref[j];
    const float4 alo = lo[i], ahi = hi[i], blo = lo[j], bhi = hi[j];
    const float4 mlo = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.0f);
    const float4 mhi = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.0f);
    left[node] = a;
    right[node] = b;
    int_lo[node] = mlo;
    int_hi[node] = mhi;
    if (a & kLeafFlag) leaf_parent[a & ~kLeafFlag] = (int)node; else int_parent[a] = (int)node;
    if (b & kLeafFlag) leaf_parent[b & ~kLeafFlag] = (int)node; else int_parent[b] = (int)node;
    out_ref[dst] = node;
    out_lo[dst] = mlo;
    out_hi[dst] = mhi;
}

// Leaf counts of every internal node, bottom-up (the second child to arrive computes its parent).
__global__ void k_subtree_counts(int n, const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                                 const int* __restrict__ int_parent, const int* __restrict__ leaf_parent,
                                 int* count, int* __restrict__ arrivals, int* __restrict__ error_flag) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int p = leaf_parent[j];
    for (int steps = 0; p >= 0; steps++) {
        if (steps > 4096) { atomicOr(error_flag, 1); return; }
        if (atomicAdd(&arrivals[p], 1) == 0) return;
        __threadfence();
        const uint32_t l = left[p], r = right[p];
        const int cl = (l & kLeafFlag) ? 1 : __ldcg(&count[l]);
        const int cr = (r & kLeafFlag) ? 1 : __ldcg(&count[r]);
        __stcg(&count[p], cl + cr);
        __threadfence();
        p = int_parent[p];
    }
}

// Depth-first position of a subtree: the leaves of the left siblings along its path to the root.
__device__ __forceinline__ int dfs_offset(uint32_t c, int p, const uint32_t* __restrict__ left,
                                          const uint32_t* __restrict__ right, const int* __restrict__ int_parent,
                                          const int* __restrict__ count, int* __restrict__ error_flag) {
    int pos = 0;
    for (int steps = 0; p >= 0; steps++) {
        if (steps > 4096) { atomicOr(error_flag, 1); return 0; }
        if (right[p] == c) {
            const uint32_t l = left[p];
            pos += (l & kLeafFlag) ? 1 : count[l];
        }
        c = (uint32_t)p;
        p = int_parent[p];
    }
    return pos;
}

__global__ void k_dfs_positions(int n, const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                                const int* __restrict__ int_parent, const int* __restrict__ leaf_parent,
                                const int* __restrict__ count, int* __restrict__ leaf_pos, uint8_t* __restrict__ leaf_side,
                                int2* __restrict__ range, int* __restrict__ error_flag) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        const int p = leaf_parent[j];
        leaf_pos[j] = dfs_offset(kLeafFlag | (uint32_t)j, p, left, right, int_parent, count, error_flag);
        leaf_side[j] = (p >= 0 && right[p] == (kLeafFlag | (uint32_t)j)) ? 1 : 0;
    }
    if (j < n) {
        if (leaf_pos[j] < 0 || leaf_pos[j] >= n) atomicOr(error_flag, 1);
    }
    if (j < n - 1) {
        const int first = dfs_offset((uint32_t)j, int_parent[j], left, right, int_parent, count, error_flag);
        range[j] = make_int2(first, first + count[j] - 1);
        if (first < 0 || first + count[j] > n) atomicOr(error_flag, 1);
    }
}

// Leaves renumbered by depth-first position, so every subtree is one contiguous range.
__global__ void k_dfs_remap(int n, const int* __restrict__ leaf_pos, const uint8_t* __restrict__ leaf_side,
                            const int* __restrict__ leaf_parent,
                            const uint32_t* __restrict__ sorted_tri, const float4* __restrict__ leaf_lo,
                            const float4* __restrict__ leaf_hi, uint32_t* __restrict__ left, uint32_t* __restrict__ right,
                            uint32_t* __restrict__ tri_out, float4* __restrict__ lo_out, float4* __restrict__ hi_out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int q = leaf_pos[j];
    if (q < 0 || q >= n) return;  // only a malformed tree (reported by k_dfs_positions) gets here
    tri_out[q] = sorted_tri[j];
    lo_out[q] = leaf_lo[j];
    hi_out[q] = leaf_hi[j];
    const int p = leaf_parent[j];
    if (p < 0) return;
    if (leaf_side[j]) right[p] = kLeafFlag | (uint32_t)q;
    else left[p] = kLeafFlag | (uint32_t)q;
}

struct BinView {
    const uint32_t* left;
    const uint32_t* right;
    const int2* range;
    const float4* leaf_lo;
    const float4* leaf_hi;
    const float4* int_lo;
    const float4* int_hi;
};

__device__ __forceinline__ int ref_count(const BinView& b, uint32_t ref) {
    if (ref & kLeafFlag) return 1;
    const int2 r = b.range[ref];
    return r.y - r.x + 1;
}
__device__ __forceinline__ void ref_bounds(const BinView& b, uint32_t ref, float4& lo, float4& hi) {
    if (ref & kLeafFlag) { lo = b.leaf_lo[ref & ~kLeafFlag]; hi = b.leaf_hi[ref & ~kLeafFlag]; }
    else { lo = b.int_lo[ref]; hi = b.int_hi[ref]; }
}
__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    const float x = hi.x - lo.x, y = hi.y - lo.y, z = hi.z - lo.z;
    return x * y + y * z + z * x;
}
__device__ __forceinline__ int ref_first(const BinView& b, uint32_t ref) {
    return (ref & kLeafFlag) ? (int)(ref & ~kLeafFlag) : b.range[ref].x;
}

struct WorkItem {
    uint32_t ref;   // binary node (or leaf, for a 1-triangle scene) to expand
    uint32_t node;  // output 8-wide node index
};

// ---- SAH-optimal collapse (Ylitie, Karras and Laine, HPG 2017, section 3) -------------------
// C(n, i) is the least SAH cost of the subtree of binary node n written as a forest of at most
// i roots: C(n, 1) = min(leaf cost, internal cost), C(n, i > 1) = min(C(n, 1), the best split
// of the i roots between the two children). A leaf child of p <= 3 triangles costs
// A(n) p kCostTri; an internal child costs A(n) kCostNode plus the best split of 8 roots among
// its children. Computed bottom-up, then read top-down by the collapse, which opens each
// 8-wide node exactly as the minimum says. With kCostNode >= 3 kCostTri a subtree of at most
// 3 triangles is always cheapest as one leaf, so the emit step's rule (internal iff more than
// 3 triangles) matches every choice the minimum makes. Measured on the 1.55M-triangle terrain
// against a greedy collapse (open the child of largest area until 8): 11.96 nodes and 3.99
// triangles per ray instead of 12.51 and 4.66, 1631 Mrays/s against 1563 (kCostTri 0.2: 1628).
constexpr float kCostNode = 1.0f;
constexpr float kCostTri = 0.3f;
static_assert(kCostNode >= kLeafMax * kCostTri, "a leaf of <= kLeafMax triangles must never cost more than a node");

// Per internal node: cost[2p], cost[2p+1] hold C(p, 1..8); split[p] byte i-1 (i >= 2) holds the
// left child's share k of the best split of i roots, with bit 4 set when C(p, 1) is not worse
// (the subtree stays one root).
__device__ __forceinline__ void child_costs(const BinView& b, uint32_t ref, const float4* cost, float c[8]) {
    if (ref & kLeafFlag) {
        const float a = half_area(b.leaf_lo[ref & ~kLeafFlag], b.leaf_hi[ref & ~kLeafFlag]) * kCostTri;
#pragma unroll
        for (int i = 0; i < 8; i++) c[i] = a;
    } else {
        const float4 x = __ldcg(&cost[2 * (size_t)ref]), y = __ldcg(&cost[2 * (size_t)ref + 1]);
        c[0] = x.x; c[1] = x.y; c[2] = x.z; c[3] = x.w;
        c[4] = y.x; c[5] = y.y; c[6] = y.z; c[7] = y.w;
    }
}

__global__ void k_collapse_costs(int n, BinView b, const int* __restrict__ int_parent,
                                 const int* __restrict__ leaf_parent, float4* cost, uint2* split,
                                 int* __restrict__ arrivals, int* __restrict__ error_flag) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int p = leaf_parent[j];
    for (int steps = 0; p >= 0; steps++) {
        if (steps > 4096) { atomicOr(error_flag, 1); return; }
        if (atomicAdd(&arrivals[p], 1) == 0) return;
        __threadfence();
        float cl[8], cr[8];
        child_costs(b, b.left[p], cost, cl);
        child_costs(b, b.right[p], cost, cr);
        const float area = half_area(b.int_lo[p], b.int_hi[p]);
        const int2 rg = b.range[p];
        const int cnt = rg.y - rg.x + 1;
        float dist[9];
        uint32_t k_of[9];
#pragma unroll
        for (int i = 2; i <= 8; i++) {
            float best = INFINITY;
            uint32_t bk = 1;
#pragma unroll
            for (int k = 1; k < i; k++) {
                const float c = cl[k - 1] + cr[i - k - 1];
                if (c < best) { best = c; bk = (uint32_t)k; }
            }
            dist[i] = best;
            k_of[i] = bk;
        }
        const float c_int = dist[8] + area * kCostNode;
        const float c_leaf = cnt <= kLeafMax ? area * (float)cnt * kCostTri : INFINITY;
        const float c1 = fminf(c_leaf, c_int);
        float c[8];
        uint32_t lo = 0, hi = 0;
        c[0] = c1;
#pragma unroll
        for (int i = 2; i <= 8; i++) {
            const bool one = c1 <= dist[i];
            c[i - 1] = one ? c1 : dist[i];
            const uint32_t byte = k_of[i] | (one ? 0x10u : 0u);
            if (i - 1 < 4) lo |= byte << (8 * (i - 1));
            else hi |= byte << (8 * (i - 5));
        }
        __stcg(&cost[2 * (size_t)p], make_float4(c[0], c[1], c[2], c[3]));
        __stcg(&cost[2 * (size_t)p + 1], make_float4(c[4], c[5], c[6], c[7]));
        split[p] = make_uint2(lo, hi);
        __threadfence();
        p = int_parent[p];
    }
}

// The children of the 8-wide node made from binary node `ref`: the roots of the best split of
// 8 (C(ref, 1) as an internal node), expanded as the stored splits say.
__device__ int dp_children(const BinView& b, const uint2* __restrict__ split, uint32_t ref, uint32_t ch[8]) {
    uint32_t st_ref[8];
    int st_budget[8];
    int sp = 0, nc = 0;
    const uint2 s0 = split[ref];
    const uint32_t k0 = (s0.y >> 24) & 0x0Fu;  // byte 7: split of 8 roots
    st_ref[sp] = b.right[ref]; st_budget[sp++] = 8 - (int)k0;
    st_ref[sp] = b.left[ref]; st_budget[sp++] = (int)k0;
    while (sp > 0) {
        const uint32_t r = st_ref[--sp];
        const int budget = st_budget[sp];
        if ((r & kLeafFlag) || budget <= 1 || nc + sp >= 7) {
            ch[nc++] = r;
            continue;
        }
        const uint2 sv = split[r];
        const uint32_t byte = budget - 1 < 4 ? (sv.x >> (8 * (budget - 1))) & 0xFFu : (sv.y >> (8 * (budget - 5))) & 0xFFu;
        const int k = (int)(byte & 0x0Fu);
        if ((byte & 0x10u) || k < 1 || k >= budget) {
            ch[nc++] = r;
            continue;
        }
        st_ref[sp] = b.right[r]; st_budget[sp++] = budget - k;
        st_ref[sp] = b.left[r]; st_budget[sp++] = k;
    }
    return nc;
}

// Plan: choose the (up to) 8 children of each new node, count internal children and leaf triangles.
__global__ void k_collapse_plan(BinView b, const WorkItem* __restrict__ work, int nwork,
                                uint32_t* __restrict__ children, int* __restrict__ n_int, int* __restrict__ n_tri,
                                const uint2* __restrict__ split) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwork) return;
    const uint32_t ref = work[w].ref;
    uint32_t ch[8];
    int nc = 0;
    if (ref & kLeafFlag) ch[nc++] = ref;
    else nc = dp_children(b, split, ref, ch);
    int ni = 0, nt = 0;
    for (int c = 0; c < 8; c++) {
        uint32_t r = c < nc ? ch[c] : 0xFFFFFFFFu;
        children[8 * (size_t)w + c] = r;
        if (c < nc) {
            const int cnt = ref_count(b, r);
            if (!(r & kLeafFlag) && cnt > kLeafMax) ni++;
            else nt += cnt;
        }
    }
    n_int[w] = ni;
    n_tri[w] = nt;
}

// Margin, in quanta, by which every quantised child plane other than the node origin lies outside
// the child's box. The traversal decodes a plane at q quanta as q * (scale / d) + (origin - o) / d;
// when the node origin is far from the ray origin along an axis the two terms nearly cancel and
// the result carries an absolute error of a few float ulps of (origin - o) / d. A plane that fits
// its child exactly (a child boundary on the quantum grid) could then be crossed a little early
// and a box the ray enters be missed (seen on grazing rays off a 60-unit panel inside a
// 1000-unit node). A 1/64-quantum margin exceeds that error while the ray origin lies within
// ~300 node extents of the node origin along the axis; farther out the two terms do not cancel
// and the relative padding of the box test covers the rounding.
constexpr float kQuantMargin = 1.0f / 64.0f;

// Emit: quantise, assign slots, write the node, gather leaf triangles, queue internal children.
__global__ void k_collapse_emit(BinView b, const WorkItem* __restrict__ work, int nwork,
                                const uint32_t* __restrict__ children, const int* __restrict__ int_off,
                                const int* __restrict__ tri_off, uint32_t node_base, uint32_t tri_base_all,
                                const uint32_t* __restrict__ sorted_tri, const uint32_t* __restrict__ ref_tri,
                                const float* __restrict__ pos, CwNode* __restrict__ nodes,
                                float4* __restrict__ tris_out, uint32_t* __restrict__ perm,
                                WorkItem* __restrict__ next_work) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwork) return;
    uint32_t ch[8];
    int nc = 0;
    for (int c = 0; c < 8; c++) {
        const uint32_t r = children[8 * (size_t)w + c];
        if (r != 0xFFFFFFFFu) ch[nc++] = r;
    }
    float4 clo[8], chi[8];
    float4 lo = make_float4(INFINITY, INFINITY, INFINITY, 0), hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0);
    for (int c = 0; c < nc; c++) {
        ref_bounds(b, ch[c], clo[c], chi[c]);
        lo.x = fminf(lo.x, clo[c].x); lo.y = fminf(lo.y, clo[c].y); lo.z = fminf(lo.z, clo[c].z);
        hi.x = fmaxf(hi.x, chi[c].x); hi.y = fmaxf(hi.y, chi[c].y); hi.z = fmaxf(hi.z, chi[c].z);
    }
    CwNode node;
    node.px = lo.x; node.py = lo.y; node.pz = lo.z;
    uint32_t ebits[3];
    float inv_scale[3];
    const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z};
    // Quantum per axis: a power of two at least ext / 254, so that a child's planes fit in 0..255
    // with the margin below.
    for (int k = 0; k < 3; k++) {
        const float ext = __fsub_ru(h3[k], l3[k]);
        const float s = __fdiv_ru(ext, 254.0f);
        uint32_t bits = __float_as_uint(s);
        uint32_t e = (bits >> 23) & 0xFFu;
        if (bits & 0x7FFFFFu) e += 1;
        if (e < 1) e = 1;
        if (e > 253) e = 253;
        ebits[k] = e;
        inv_scale[k] = __uint_as_float((254u - e) << 23);
    }
    node.ex = (uint8_t)ebits[0]; node.ey = (uint8_t)ebits[1]; node.ez = (uint8_t)ebits[2];

    // Octant slot assignment: slot s holds the child a ray of octant s should visit first.
    const float ncx = 0.5f * (lo.x + hi.x), ncy = 0.5f * (lo.y + hi.y), ncz = 0.5f * (lo.z + hi.z);
    float cost[8][8];
    for (int c = 0; c < nc; c++) {
        const float dx = 0.5f * (clo[c].x + chi[c].x) - ncx;
        const float dy = 0.5f * (clo[c].y + chi[c].y) - ncy;
        const float dz = 0.5f * (clo[c].z + chi[c].z) - ncz;
        for (int s = 0; s < 8; s++)
            cost[c][s] = ((s & 1) ? -dx : dx) + ((s & 2) ? -dy : dy) + ((s & 4) ? -dz : dz);
    }
    int slot_of[8];
    uint32_t slot_used = 0, child_done = 0;
    for (int it = 0; it < nc; it++) {
        float best = INFINITY;
        int bc = -1, bs = -1;
        for (int c = 0; c < nc; c++) {
            if (child_done & (1u << c)) continue;
            for (int s = 0; s < 8; s++) {
                if (slot_used & (1u << s)) continue;
                if (cost[c][s] < best || bc < 0) { best = cost[c][s]; bc = c; bs = s; }
            }
        }
        slot_of[bc] = bs;
        child_done |= 1u << bc;
        slot_used |= 1u << bs;
    }
    int child_in_slot[8];
    for (int s = 0; s < 8; s++) child_in_slot[s] = -1;
    for (int c = 0; c < nc; c++) child_in_slot[slot_of[c]] = c;

    const uint32_t child_base = node_base + (uint32_t)int_off[w];
    const uint32_t tri_base = tri_base_all + (uint32_t)tri_off[w];
    node.child_base = child_base;
    node.tri_base = tri_base;
    uint32_t imask = 0;
    int int_rank = 0, tri_rank = 0;
    for (int s = 0; s < 8; s++) {
        const int c = child_in_slot[s];
        if (c < 0) {
            node.meta[s] = 0;
            node.qlo_x[s] = node.qlo_y[s] = node.qlo_z[s] = 0;
            node.qhi_x[s] = node.qhi_y[s] = node.qhi_z[s] = 0;
            continue;
        }
        const float cl[3] = {clo[c].x, clo[c].y, clo[c].z}, chh[3] = {chi[c].x, chi[c].y, chi[c].z};
        uint8_t ql[3], qh[3];
        for (int k = 0; k < 3; k++) {
            // outward by at least kQuantMargin quanta (a plane at q = 0 is the node origin itself)
            const float a = floorf(__fsub_rd(cl[k], l3[k]) * inv_scale[k] - kQuantMargin);
            const float bq = ceilf(__fsub_ru(chh[k], l3[k]) * inv_scale[k] + kQuantMargin);
            ql[k] = (uint8_t)fminf(fmaxf(a, 0.0f), 255.0f);
            qh[k] = (uint8_t)fminf(fmaxf(bq, 0.0f), 255.0f);
        }
        node.qlo_x[s] = ql[0]; node.qlo_y[s] = ql[1]; node.qlo_z[s] = ql[2];
        node.qhi_x[s] = qh[0]; node.qhi_y[s] = qh[1]; node.qhi_z[s] = qh[2];
        const uint32_t r = ch[c];
        const int cnt = ref_count(b, r);
        if (!(r & kLeafFlag) && cnt > kLeafMax) {
            imask |= 1u << s;
            node.meta[s] = (uint8_t)(0x20u | (24u + (uint32_t)s));
            next_work[int_off[w] + int_rank] = WorkItem{r, child_base + (uint32_t)int_rank};
            int_rank++;
        } else {
            const uint32_t unary = cnt == 1 ? 1u : (cnt == 2 ? 3u : 7u);
            node.meta[s] = (uint8_t)((unary << 5) | (uint32_t)tri_rank);
            const int first = ref_first(b, r);
            for (int q = 0; q < cnt; q++) {
                const uint32_t tri = ref_tri[sorted_tri[first + q]];
                const uint32_t dst = tri_base + (uint32_t)tri_rank + (uint32_t)q;
                const float* p = pos + 9 * (size_t)tri;
                tris_out[3 * (size_t)dst + 0] = make_float4(p[0], p[1], p[2], __uint_as_float(tri));
                tris_out[3 * (size_t)dst + 1] = make_float4(p[3], p[4], p[5], 0.0f);
                tris_out[3 * (size_t)dst + 2] = make_float4(p[6], p[7], p[8], 0.0f);
                perm[dst] = tri;
            }
            tri_rank += cnt;
        }
    }
    node.imask = (uint8_t)imask;
    nodes[work[w].node] = node;
}

__global__ void k_gather_shading(int n, const uint32_t* __restrict__ perm, const float* __restrict__ nrm,
                                 const float* __restrict__ uv, const int* __restrict__ tri_prim,
                                 float4* __restrict__ nrm_out, float2* __restrict__ uv_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t t = perm[i];
    const float* q = nrm + 9 * (size_t)t;
    nrm_out[3 * (size_t)i + 0] = make_float4(q[0], q[1], q[2], __int_as_float(tri_prim[t]));
    nrm_out[3 * (size_t)i + 1] = make_float4(q[3], q[4], q[5], 0.0f);
    nrm_out[3 * (size_t)i + 2] = make_float4(q[6], q[7], q[8], 0.0f);
    const float* u = uv + 6 * (size_t)t;
    uv_out[3 * (size_t)i + 0] = make_float2(u[0], u[1]);
    uv_out[3 * (size_t)i + 1] = make_float2(u[2], u[3]);
    uv_out[3 * (size_t)i + 2] = make_float2(u[4], u[5]);
}

template <typename T>
T* dev_alloc(size_t count, std::vector<void*>& temps) {
    void* p = nullptr;
    if (count == 0) count = 1;
    BVH_CHECK(cudaMalloc(&p, count * sizeof(T)));
    temps.push_back(p);
    return (T*)p;
}

}  // namespace

// PLOC binary tree over the Morton-sorted leaves, then depth-first leaf positions so that every
// subtree is a contiguous range (what the 8-wide collapse reads); returns the root's reference.
// Measured against the binary radix tree of the same Morton keys (Karras, HPG 2012) with a
// bottom-up refit: terrain 1322 vs 1305 Mrays/s (12.5 nodes and 4.7 triangles per ray against
// 12.1 and 4.8); the 10M-triangle interior halves its work per ray (30 nodes and 15 triangles
// against 55 and 30). Build: 8 ms for 1.55M triangles, 20 ms for 10M. leaf_tri receives the triangle of
// each depth-first leaf position.
uint32_t BuildPloc(int n, const uint32_t* sorted_tri, const float4* tlo, const float4* thi, uint32_t* left,
                   uint32_t* right, int* int_parent, int* leaf_parent, int2* range, float4* leaf_lo, float4* leaf_hi,
                   float4* int_lo, float4* int_hi, int* arrivals, uint32_t*& leaf_tri, std::vector<void*>& temps,
                   cudaStream_t stream) {
    const int T = 256;
    const int nb = (n + T - 1) / T;
    float4* mlo = dev_alloc<float4>(n, temps);  // leaf boxes in Morton order
    float4* mhi = dev_alloc<float4>(n, temps);
    uint32_t* ref_a = dev_alloc<uint32_t>(n, temps);
    uint32_t* ref_b = dev_alloc<uint32_t>(n, temps);
    float4* lo_a = dev_alloc<float4>(n, temps);
    float4* hi_a = dev_alloc<float4>(n, temps);
    float4* lo_b = dev_alloc<float4>(n, temps);
    float4* hi_b = dev_alloc<float4>(n, temps);
    int* nn = dev_alloc<int>(n, temps);
    int* merge = dev_alloc<int>(n + 1, temps);
    int* keep = dev_alloc<int>(n + 1, temps);
    int* merge_off = dev_alloc<int>(n + 1, temps);
    int* keep_off = dev_alloc<int>(n + 1, temps);
    size_t scan_bytes = 0;
    BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, merge, merge_off, n + 1, stream));
    void* scan_tmp = dev_alloc<uint8_t>(scan_bytes, temps);
    k_leaf_gather<<<nb, T, 0, stream>>>(n, sorted_tri, tlo, thi, mlo, mhi, ref_a);
    BVH_CHECK(cudaMemcpyAsync(lo_a, mlo, sizeof(float4) * n, cudaMemcpyDeviceToDevice, stream));
    BVH_CHECK(cudaMemcpyAsync(hi_a, mhi, sizeof(float4) * n, cudaMemcpyDeviceToDevice, stream));
    int count = n;
    uint32_t node_base = 0;
    for (int round = 0; count > 1; round++) {
        if (round > n) throw DeviceError("PLOC clustering made no progress");
        const int gb = (count + T - 1) / T;
        k_ploc_nn<<<(count + kPlocBlock - 1) / kPlocBlock, kPlocBlock, 0, stream>>>(count, lo_a, hi_a, nn);
        k_ploc_flags<<<(count + 1 + T - 1) / T, T, 0, stream>>>(count, nn, merge, keep);
        BVH_CHECK(cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, merge, merge_off, count + 1, stream));
        BVH_CHECK(cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, keep, keep_off, count + 1, stream));
        k_ploc_merge<<<gb, T, 0, stream>>>(count, nn, merge_off, keep_off, ref_a, lo_a, hi_a, node_base, left, right,
                                          int_lo, int_hi, int_parent, leaf_parent, ref_b, lo_b, hi_b);
        BVH_CHECK(cudaGetLastError());
        int totals[2];
        BVH_CHECK(cudaMemcpyAsync(&totals[0], merge_off + count, sizeof(int), cudaMemcpyDeviceToHost, stream));
        BVH_CHECK(cudaMemcpyAsync(&totals[1], keep_off + count, sizeof(int), cudaMemcpyDeviceToHost, stream));
        BVH_CHECK(cudaStreamSynchronize(stream));
        if (totals[0] <= 0 || totals[1] >= count) throw DeviceError("PLOC clustering made no progress");
        node_base += (uint32_t)totals[0];
        count = totals[1];
        std::swap(ref_a, ref_b);
        std::swap(lo_a, lo_b);
        std::swap(hi_a, hi_b);
    }
    if (node_base != (uint32_t)(n - 1)) throw DeviceError("PLOC produced a malformed tree");
    const uint32_t root = node_base - 1;  // the last merge
    BVH_CHECK(cudaMemcpyAsync(int_parent + root, &kNoParent, sizeof(int), cudaMemcpyHostToDevice, stream));
    // subtree sizes, depth-first positions, contiguous ranges
    const int ni = n - 1;
    int* count_arr = dev_alloc<int>(ni, temps);
    int* leaf_pos = dev_alloc<int>(n, temps);
    uint8_t* leaf_side = dev_alloc<uint8_t>(n, temps);
    BVH_CHECK(cudaMemsetAsync(arrivals, 0, sizeof(int) * (ni + 1), stream));
    k_subtree_counts<<<nb, T, 0, stream>>>(n, left, right, int_parent, leaf_parent, count_arr, arrivals, arrivals + ni);
    k_dfs_positions<<<nb, T, 0, stream>>>(n, left, right, int_parent, leaf_parent, count_arr, leaf_pos, leaf_side, range,
                                          arrivals + ni);
    uint32_t* dfs_tri = dev_alloc<uint32_t>(n, temps);
    k_dfs_remap<<<nb, T, 0, stream>>>(n, leaf_pos, leaf_side, leaf_parent, sorted_tri, mlo, mhi, left, right, dfs_tri,
                                      leaf_lo, leaf_hi);
    BVH_CHECK(cudaGetLastError());
    int err = 0;
    BVH_CHECK(cudaMemcpyAsync(&err, arrivals + ni, sizeof(int), cudaMemcpyDeviceToHost, stream));
    BVH_CHECK(cudaStreamSynchronize(stream));
    if (err) throw DeviceError("PLOC tree deeper than the walk limit");
    leaf_tri = dfs_tri;
    return root;
}

// Builds the BVH of the n triangles in d_pos (9 floats each, original order).
void BuildBvh(DeviceScene& ds, const float* d_pos, const float* d_nrm, const float* d_uv, const int* d_tri_prim,
              int n, cudaStream_t stream) {
    std::vector<void*> temps;
    auto free_temps = [&]() {
        for (void* p : temps) cudaFree(p);
        temps.clear();
    };
    try {
        cudaEvent_t e0, e1;
        BVH_CHECK(cudaEventCreate(&e0));
        BVH_CHECK(cudaEventCreate(&e1));
        BVH_CHECK(cudaEventRecord(e0, stream));
        ds.num_nodes = 0;
        ds.bvh_depth = 0;
        if (n > 0) {
            const int T = 256;
            const int nbt = (n + T - 1) / T;
            float4* tlo = dev_alloc<float4>(n, temps);
            float4* thi = dev_alloc<float4>(n, temps);
            int* cb = dev_alloc<int>(6, temps);
            const int init[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
            BVH_CHECK(cudaMemcpyAsync(cb, init, sizeof(init), cudaMemcpyHostToDevice, stream));
            k_tri_bounds<<<std::min(nbt, 152 * 8), T, 0, stream>>>(d_pos, n, tlo, thi, cb);

            // pre-splitting: m references (m = n when no triangle is split)
            uint32_t* pieces = dev_alloc<uint32_t>(n, temps);
            unsigned long long* extra_d = dev_alloc<unsigned long long>(1, temps);
            BVH_CHECK(cudaMemsetAsync(extra_d, 0, sizeof(unsigned long long), stream));
            k_split_counts<<<nbt, T, 0, stream>>>(d_pos, tlo, thi, n, pieces, extra_d);
            BVH_CHECK(cudaGetLastError());
            unsigned long long extra = 0;
            BVH_CHECK(cudaMemcpyAsync(&extra, extra_d, sizeof(extra), cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaStreamSynchronize(stream));
            const double budget = kSplitBudget * (double)n;
            if ((double)extra > budget) {
                k_split_scale<<<nbt, T, 0, stream>>>(pieces, n, budget / (double)extra);
                BVH_CHECK(cudaGetLastError());
            }
            uint32_t* first = dev_alloc<uint32_t>((size_t)n + 1, temps);
            size_t scan_bytes0 = 0;
            BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes0, pieces, first, n, stream));
            void* scan_tmp0 = dev_alloc<uint8_t>(scan_bytes0, temps);
            BVH_CHECK(cub::DeviceScan::ExclusiveSum(scan_tmp0, scan_bytes0, pieces, first, n, stream));
            uint32_t last_first = 0, last_pieces = 0;
            BVH_CHECK(cudaMemcpyAsync(&last_first, first + (n - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaMemcpyAsync(&last_pieces, pieces + (n - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaStreamSynchronize(stream));
            const int64_t m64 = (int64_t)last_first + last_pieces;
            if (m64 < n || m64 > (int64_t)n + (int64_t)budget + 1 || m64 > (int64_t)INT32_MAX / 2)
                throw DeviceError("BVH pre-splitting produced " + std::to_string(m64) + " references for " +
                                  std::to_string(n) + " triangles");
            const int m = (int)m64;
            float4* rlo = tlo;
            float4* rhi = thi;
            uint32_t* ref_tri = dev_alloc<uint32_t>(m, temps);
            if (m > n) {
                rlo = dev_alloc<float4>(m, temps);
                rhi = dev_alloc<float4>(m, temps);
                BVH_CHECK(cudaMemcpyAsync(cb, init, sizeof(init), cudaMemcpyHostToDevice, stream));
            }
            k_split_emit<<<nbt, T, 0, stream>>>(d_pos, tlo, thi, n, pieces, first, rlo, rhi, ref_tri);
            BVH_CHECK(cudaGetLastError());
            const int nb = (m + T - 1) / T;
            if (m > n) k_centroid_bounds<<<std::min(nb, 152 * 8), T, 0, stream>>>(rlo, rhi, m, cb);

            uint64_t* keys = dev_alloc<uint64_t>(m, temps);
            uint64_t* keys_s = dev_alloc<uint64_t>(m, temps);
            uint32_t* vals = dev_alloc<uint32_t>(m, temps);
            uint32_t* vals_s = dev_alloc<uint32_t>(m, temps);
            k_morton<<<nb, T, 0, stream>>>(rlo, rhi, m, cb, keys, vals);
            size_t tmp_bytes = 0;
            BVH_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys_s, vals, vals_s, m, 0, 63, stream));
            void* tmp = dev_alloc<uint8_t>(tmp_bytes, temps);
            BVH_CHECK(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_s, vals, vals_s, m, 0, 63, stream));
            const int ni = std::max(m - 1, 1);
            uint32_t* left = dev_alloc<uint32_t>(ni, temps);
            uint32_t* right = dev_alloc<uint32_t>(ni, temps);
            int* int_parent = dev_alloc<int>(ni, temps);
            int* leaf_parent = dev_alloc<int>(m, temps);
            int2* range = dev_alloc<int2>(ni, temps);
            float4* leaf_lo = dev_alloc<float4>(m, temps);
            float4* leaf_hi = dev_alloc<float4>(m, temps);
            float4* int_lo = dev_alloc<float4>(ni, temps);
            float4* int_hi = dev_alloc<float4>(ni, temps);
            int* arrivals = dev_alloc<int>(ni + 1, temps);  // last entry: error flag
            BVH_CHECK(cudaMemsetAsync(arrivals, 0, sizeof(int) * (ni + 1), stream));
            uint32_t root_ref = m == 1 ? (kLeafFlag | 0u) : 0u;
            uint32_t* leaf_tri = vals_s;  // reference of each leaf position
            if (m == 1) {
                // a single leaf: its box is the triangle's
                BVH_CHECK(cudaMemsetAsync(leaf_parent, 0xFF, sizeof(int), stream));  // -1
                k_leaf_gather<<<1, 32, 0, stream>>>(1, vals_s, rlo, rhi, leaf_lo, leaf_hi, left);
                BVH_CHECK(cudaGetLastError());
            } else {
                root_ref = BuildPloc(m, vals_s, rlo, rhi, left, right, int_parent, leaf_parent, range, leaf_lo, leaf_hi,
                                     int_lo, int_hi, arrivals, leaf_tri, temps, stream);
            }

            // 8-wide collapse, one level per iteration.
            const size_t max_nodes = (size_t)ni + 1;
            CwNode* nodes = nullptr;
            BVH_CHECK(cudaMalloc(&nodes, max_nodes * sizeof(CwNode)));
            temps.push_back(nodes);
            float4* tris_out = nullptr;
            BVH_CHECK(cudaMalloc(&tris_out, 3 * (size_t)m * sizeof(float4)));
            uint32_t* perm = dev_alloc<uint32_t>(m, temps);
            WorkItem* work_a = dev_alloc<WorkItem>(max_nodes, temps);
            WorkItem* work_b = dev_alloc<WorkItem>(max_nodes, temps);
            uint32_t* children = dev_alloc<uint32_t>(8 * max_nodes, temps);
            int* n_int = dev_alloc<int>(max_nodes + 1, temps);
            int* n_tri = dev_alloc<int>(max_nodes + 1, temps);
            int* int_off = dev_alloc<int>(max_nodes + 1, temps);
            int* tri_off = dev_alloc<int>(max_nodes + 1, temps);
            size_t scan_bytes = 0;
            BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, n_int, int_off, (int)max_nodes + 1, stream));
            void* scan_tmp = dev_alloc<uint8_t>(scan_bytes, temps);

            const WorkItem root{root_ref, 0u};
            BVH_CHECK(cudaMemcpyAsync(work_a, &root, sizeof(root), cudaMemcpyHostToDevice, stream));
            BinView bv{left, right, range, leaf_lo, leaf_hi, int_lo, int_hi};
            uint2* split = nullptr;
            if (m > 1) {
                float4* cost = dev_alloc<float4>(2 * (size_t)ni, temps);
                split = dev_alloc<uint2>(ni, temps);
                BVH_CHECK(cudaMemsetAsync(arrivals, 0, sizeof(int) * (ni + 1), stream));
                k_collapse_costs<<<nb, T, 0, stream>>>(m, bv, int_parent, leaf_parent, cost, split, arrivals,
                                                       arrivals + ni);
                BVH_CHECK(cudaGetLastError());
                int dp_err = 0;
                BVH_CHECK(cudaMemcpyAsync(&dp_err, arrivals + ni, sizeof(int), cudaMemcpyDeviceToHost, stream));
                BVH_CHECK(cudaStreamSynchronize(stream));
                if (dp_err) throw DeviceError("BVH cost pass walked past the maximum tree depth");
            }
            uint32_t node_count = 1, tri_count = 0;
            int nwork = 1, depth = 0;
            while (nwork > 0) {
                depth++;
                const int gb = (nwork + 127) / 128;
                k_collapse_plan<<<gb, 128, 0, stream>>>(bv, work_a, nwork, children, n_int, n_tri, split);
                BVH_CHECK(cudaMemsetAsync(n_int + nwork, 0, sizeof(int), stream));
                BVH_CHECK(cudaMemsetAsync(n_tri + nwork, 0, sizeof(int), stream));
                BVH_CHECK(cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, n_int, int_off, nwork + 1, stream));
                BVH_CHECK(cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, n_tri, tri_off, nwork + 1, stream));
                k_collapse_emit<<<gb, 128, 0, stream>>>(bv, work_a, nwork, children, int_off, tri_off, node_count,
                                                       tri_count, leaf_tri, ref_tri, d_pos, nodes, tris_out, perm, work_b);
                BVH_CHECK(cudaGetLastError());
                int totals[2];
                BVH_CHECK(cudaMemcpyAsync(&totals[0], int_off + nwork, sizeof(int), cudaMemcpyDeviceToHost, stream));
                BVH_CHECK(cudaMemcpyAsync(&totals[1], tri_off + nwork, sizeof(int), cudaMemcpyDeviceToHost, stream));
                BVH_CHECK(cudaStreamSynchronize(stream));
                node_count += (uint32_t)totals[0];
                tri_count += (uint32_t)totals[1];
                nwork = totals[0];
                std::swap(work_a, work_b);
                if (depth > 4096) throw DeviceError("BVH collapse did not terminate");
            }
            if ((int)tri_count != m) {
                cudaFree(tris_out);
                throw DeviceError("BVH collapse lost triangles: " + std::to_string(tri_count) + " of " + std::to_string(m));
            }
            // Shrink the node array to its exact size.
            CwNode* nodes_exact = nullptr;
            BVH_CHECK(cudaMalloc(&nodes_exact, (size_t)node_count * sizeof(CwNode)));
            BVH_CHECK(cudaMemcpyAsync(nodes_exact, nodes, (size_t)node_count * sizeof(CwNode), cudaMemcpyDeviceToDevice, stream));
            float4* nrm_out = nullptr;
            float2* uv_out = nullptr;
            BVH_CHECK(cudaMalloc(&nrm_out, 3 * (size_t)m * sizeof(float4)));
            BVH_CHECK(cudaMalloc(&uv_out, 3 * (size_t)m * sizeof(float2)));
            k_gather_shading<<<nb, T, 0, stream>>>(m, perm, d_nrm, d_uv, d_tri_prim, nrm_out, uv_out);
            BVH_CHECK(cudaGetLastError());
            ds.num_tris = m;
            ds.nodes = nodes_exact;
            ds.tris = tris_out;
            ds.nrm = nrm_out;
            ds.uv = uv_out;
            ds.num_nodes = (int)node_count;
            ds.bvh_depth = depth;
        }
        BVH_CHECK(cudaEventRecord(e1, stream));
        BVH_CHECK(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ds.build_ms = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        free_temps();
    } catch (...) {
        cudaStreamSynchronize(stream);
        free_temps();
        throw;
    }
}

}  // namespace ngi
