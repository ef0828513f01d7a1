// Ray traversal on the GPU: watertight ray/triangle test and compressed 8-wide BVH walk.
//
// Replaces Embree's rtcIntersect (include/nanogi/rt.hpp:2162-2189) and the closest-hit
// visibility query of Scene::Visible (rt.hpp:2251-2261). Everything here is FP32, like
// the reference's float RTCRay (rt.hpp:2166-2173) over float vertices (rt.hpp:2119-2121).
//
// The triangle test is the watertight algorithm of Woop, Benthin and Wald (JCGT 2013)
// written with explicit round-to-nearest intrinsics, so no multiply-add is contracted and
// the result is the same float the CPU oracle computes for the same ray and triangle.
#pragma once

#include "ngi_device.cuh"

namespace ngi {

struct RayPre {
    float ox, oy, oz;
    float Sx, Sy, Sz;
    int kx, ky, kz;
};

NGI_D float comp3(float a, float b, float c, int k) { return k == 0 ? a : (k == 1 ? b : c); }

// Per-ray shear constants (Woop et al. 2013, section 3).
NGI_D RayPre ray_precompute(float ox, float oy, float oz, float dx, float dy, float dz) {
    RayPre r;
    r.ox = ox; r.oy = oy; r.oz = oz;
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    const float dkz = comp3(dx, dy, dz, kz);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = __fdiv_rn(comp3(dx, dy, dz, kx), dkz);
    r.Sy = __fdiv_rn(comp3(dx, dy, dz, ky), dkz);
    r.Sz = __fdiv_rn(1.0f, dkz);
    return r;
}

// Watertight test. On a hit with tmin <= t < tbest returns true with t and the Embree
// barycentrics (u weights p2, v weights p3).
NGI_D bool tri_intersect(const RayPre& r, float4 p0, float4 p1, float4 p2, float tmin, float tbest,
                         float& t_out, float& u_out, float& v_out) {
    const float A0 = __fsub_rn(p0.x, r.ox), A1 = __fsub_rn(p0.y, r.oy), A2 = __fsub_rn(p0.z, r.oz);
    const float B0 = __fsub_rn(p1.x, r.ox), B1 = __fsub_rn(p1.y, r.oy), B2 = __fsub_rn(p1.z, r.oz);
    const float C0 = __fsub_rn(p2.x, r.ox), C1 = __fsub_rn(p2.y, r.oy), C2 = __fsub_rn(p2.z, r.oz);
    const float Akx = comp3(A0, A1, A2, r.kx), Aky = comp3(A0, A1, A2, r.ky), Akz = comp3(A0, A1, A2, r.kz);
    const float Bkx = comp3(B0, B1, B2, r.kx), Bky = comp3(B0, B1, B2, r.ky), Bkz = comp3(B0, B1, B2, r.kz);
    const float Ckx = comp3(C0, C1, C2, r.kx), Cky = comp3(C0, C1, C2, r.ky), Ckz = comp3(C0, C1, C2, r.kz);
    const float Ax = __fsub_rn(Akx, __fmul_rn(r.Sx, Akz));
    const float Ay = __fsub_rn(Aky, __fmul_rn(r.Sy, Akz));
    const float Bx = __fsub_rn(Bkx, __fmul_rn(r.Sx, Bkz));
    const float By = __fsub_rn(Bky, __fmul_rn(r.Sy, Bkz));
    const float Cx = __fsub_rn(Ckx, __fmul_rn(r.Sx, Ckz));
    const float Cy = __fsub_rn(Cky, __fmul_rn(r.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Edge case: the products of two floats are exact in double, so one rounding.
        U = (float)__dsub_rn((double)Cx * (double)By, (double)Cy * (double)Bx);
        V = (float)__dsub_rn((double)Ax * (double)Cy, (double)Ay * (double)Cx);
        W = (float)__dsub_rn((double)Bx * (double)Ay, (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float rcp = __fdiv_rn(1.0f, det);
    const float t = __fmul_rn(T, rcp);
    if (!(t >= tmin && t < tbest)) return false;
    t_out = t;
    u_out = __fmul_rn(V, rcp);
    v_out = __fmul_rn(W, rcp);
    return true;
}

constexpr int kTraversalStack = 64;
// Each lane's stack of node groups (64 entries of 8 bytes) lives in local memory, which L1
// caches. Measured and not kept: the bottom 4, 8 or 16 entries of every lane in shared memory,
// entry-major, the rest local (Ylitie et al. 2017): 1794, 1796 and 1794 Mrays/s on the
// 1.55M-triangle terrain against 1813 all-local, and 3957 against 4027 on the Cornell box. The
// shared-memory carve-out takes L1 capacity from the node fetches, while the local stack's few
// hot lines per lane already hit L1.

// Relative padding of the box interval: keeps the box test conservative against the few
// ulps of rounding in the slab distances (Ize, JCGT 2013). The interval starts at 0 rather
// than at the ray's tmin: the watertight t of a large triangle carries an absolute error of a
// few ulps of its vertex coordinates, so at the reference's absolute tmin = 1e-4 a triangle
// whose plane the ray crosses just below tmin can still test at t >= tmin (a surface point
// reconstructed behind a 550-unit wall, say). The triangle test alone applies tmin, so a hit
// does not depend on which boxes enclose the triangle.
constexpr float kBoxLo = 1.0f - 1.0f / 1048576.0f;
constexpr float kBoxHi = 1.0f + 1.0f / 1048576.0f;
// tn Lo <= tf Hi as one product, tn <= tf (Hi / Lo): the same test for either sign of tn and tf
// (0.7% over two products).
constexpr float kBoxRatio = kBoxHi / kBoxLo;
// The node phase is "while-while" (Aila and Laine 2009): a lane holding triangles waits while
// the other lanes of its warp keep visiting nodes, so the triangle tests of a warp run together.
// Measured on the 1.55M-triangle terrain: 1333 Mrays/s against 1105 with one node per step.
// Measured and not kept: triangle postponing (Ylitie et al. 2017; slower at every threshold), a
// speculative second triangle group (lanes with triangles visiting nodes while others search;
// 1389 vs 1418), a folded quantised-plane form (one subtraction less per plane, boxes two quanta
// wider; 1010 vs 1076), and three-input min.f32 / max.f32 for the slab entry and exit (1631 vs
// 1633: no change).
// Node-phase exit: percentage of a warp's tracing lanes below which the lanes still searching
// for triangles stop, and resume after the triangle tests (0: the node phase runs until no lane
// searches). Without it the lanes holding triangles wait for the warp's longest search. Measured
// on the 1.55M-triangle terrain: 0: 1631, 15: 1760, 30: 1809, 40: 1821, 50: 1818, 60: 1792,
// 75: 1719, 90: 1593 Mrays/s; on the 10M-triangle interior 440 (0) against 512 (60). With the
// triangle-phase exit at 15 and the logic counters in shared memory: 30: 1994, 40: 2036,
// 45: 2059, 50: 2067, 55: 2069, 60: 2061.
constexpr int kNodeExitPct = 50;
// Triangle-phase exit, the same for the triangle tests: lanes with untested triangles keep them
// (in the ray state) and finish them in the next step (0: test until every lane is done).
// Measured with the node-phase exit at 40: terrain 0: 1820, 10: 1888, 15: 1884, 20: 1870,
// 25: 1860, 35: 1812, 50: 1710 Mrays/s; the triangle-heavy 10M-triangle interior (18 triangles
// per ray) loses a little: 512 (0), 493 (10), 497 (15), 499 (20).
constexpr int kTriExitPct = 15;

struct TraceStats {
    uint32_t nodes;
    uint32_t tris;
};

// Packed box test: the near and far plane of an axis are decoded and scaled as one float2
// through the two-wide FADD2 / FFMA2 instructions of sm_100+. Measured on the 1.55M-triangle
// terrain: 1090 Mrays/s against 1060 for the scalar form. (Pairing the watertight triangle
// test's multiplies and subtractions the same way gained nothing and did not reproduce the
// scalar roundings, so that test stays scalar.)
//
// (near, far) plane distances of one axis for child j: (q * s + a) for the two quantised
// bytes, q = byte - 2^23 after the permute builds 2^23 + byte.
NGI_D float2 plane_pair(uint32_t near_word, uint32_t far_word, int j, float2 s2, float2 a2) {
    const float2 q = make_float2(__uint_as_float(__byte_perm(near_word, 0x4B000000u, 0x7440u + (uint32_t)j)),
                                 __uint_as_float(__byte_perm(far_word, 0x4B000000u, 0x7440u + (uint32_t)j)));
    return __ffma2_rn(__fadd2_rn(q, make_float2(-8388608.0f, -8388608.0f)), s2, a2);
}

// Hit-mask bits of four children at once from their meta bytes (SIMD within a register, as
// in Ylitie et al. 2017, section 4): a meta byte is (child bits << 5) | slot, where an
// internal child has slot 24..31 (bits 3 and 4 set) and its bit index is reordered by the
// ray octant; a leaf's slot is its first triangle's offset 0..23. An empty child has meta 0
// and so sets no bit, without a test of its own. Measured on the 1.55M-triangle terrain:
// 1633 Mrays/s against 1559 for the per-child decode.
NGI_D void meta_decode4(uint32_t meta4, uint32_t octinv4, uint32_t& bit_index4, uint32_t& child_bits4) {
    const uint32_t is_inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
    const uint32_t inner_mask4 = (is_inner4 >> 4) * 0xFFu;  // per byte 0x00 or 0xFF (no carries)
    bit_index4 = (meta4 ^ (octinv4 & inner_mask4)) & 0x1F1F1F1Fu;
    child_bits4 = (meta4 >> 5) & 0x07070707u;
}

// Per-ray state of one CWBVH traversal, kept in registers between steps so a warp can
// interleave the rays of its lanes (and refill lanes whose ray has finished).
struct TravState {
    RayPre rp;
    float idx, idy, idz;       // inverse direction (tiny components clamped) for the slab tests
    uint32_t octinv;           // 7 - ray octant: traversal order of the children
    uint32_t dneg;             // bit k set: direction component k is negative (near plane = hi)
    float tmin, tmax;
    float hu, hv;
    int hit;
    uint2 ngroup;              // node group: child base, internal-hit bits [31:24] | imask [7:0]
    uint2 tgroup;              // triangle group left untested by the last step
    int sp;
};

NGI_D void trav_init(TravState& s, float ox, float oy, float oz, float dx, float dy, float dz, float tmin,
                     float tmax) {
    s.rp = ray_precompute(ox, oy, oz, dx, dy, dz);
    const float kTiny = 1e-20f;
    s.idx = __frcp_rn(fabsf(dx) > kTiny ? dx : copysignf(kTiny, dx));
    s.idy = __frcp_rn(fabsf(dy) > kTiny ? dy : copysignf(kTiny, dy));
    s.idz = __frcp_rn(fabsf(dz) > kTiny ? dz : copysignf(kTiny, dz));
    const uint32_t oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
    s.octinv = 7u - oct;
    s.dneg = (s.idx < 0.0f ? 1u : 0u) | (s.idy < 0.0f ? 2u : 0u) | (s.idz < 0.0f ? 4u : 0u);
    s.tmin = tmin;
    s.tmax = tmax;
    s.hu = s.hv = 0.0f;
    s.hit = -1;
    s.ngroup = make_uint2(0u, 0x80000000u);  // the root as the only internal hit, imask 0
    s.tgroup = make_uint2(0u, 0u);
    s.sp = 0;
}

// Intersects the 8 children of a node; returns the CWBVH hit mask
// (bits 24..31: internal children by traversal priority, bits 0..23: leaf triangles).
NGI_D uint32_t intersect_children(const CwNode* nodes, uint32_t idx, const TravState& s, uint32_t& child_base,
                                  uint32_t& tri_base, uint32_t& imask) {
    const float4* np = reinterpret_cast<const float4*>(nodes + idx);
    const float4 n0 = __ldg(np + 0);
    const float4 n1 = __ldg(np + 1);
    const float4 n2 = __ldg(np + 2);
    const float4 n3 = __ldg(np + 3);
    const float4 n4 = __ldg(np + 4);
    const uint32_t e = __float_as_uint(n0.w);
    imask = e >> 24;
    child_base = __float_as_uint(n1.x);
    tri_base = __float_as_uint(n1.y);
    const float sx = __uint_as_float((e & 0xFFu) << 23) * s.idx;
    const float sy = __uint_as_float(((e >> 8) & 0xFFu) << 23) * s.idy;
    const float sz = __uint_as_float(((e >> 16) & 0xFFu) << 23) * s.idz;
    const float ax = (n0.x - s.rp.ox) * s.idx;
    const float ay = (n0.y - s.rp.oy) * s.idy;
    const float az = (n0.z - s.rp.oz) * s.idz;
    const bool nx = s.dneg & 1u, ny = s.dneg & 2u, nz = s.dneg & 4u;
    uint32_t hitmask = 0;
    const uint32_t octinv4 = s.octinv * 0x01010101u;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const uint32_t meta4 = __float_as_uint(half == 0 ? n1.z : n1.w);
        uint32_t bit_index4, child_bits4;
        meta_decode4(meta4, octinv4, bit_index4, child_bits4);
        const uint32_t qlx = __float_as_uint(half == 0 ? n2.x : n2.y);
        const uint32_t qly = __float_as_uint(half == 0 ? n2.z : n2.w);
        const uint32_t qlz = __float_as_uint(half == 0 ? n3.x : n3.y);
        const uint32_t qhx = __float_as_uint(half == 0 ? n3.z : n3.w);
        const uint32_t qhy = __float_as_uint(half == 0 ? n4.x : n4.y);
        const uint32_t qhz = __float_as_uint(half == 0 ? n4.z : n4.w);
        // near / far planes by direction sign: no per-child min/max needed
        const uint32_t nearx = nx ? qhx : qlx, farx = nx ? qlx : qhx;
        const uint32_t neary = ny ? qhy : qly, fary = ny ? qly : qhy;
        const uint32_t nearz = nz ? qhz : qlz, farz = nz ? qlz : qhz;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float2 px = plane_pair(nearx, farx, j, make_float2(sx, sx), make_float2(ax, ax));
            const float2 py = plane_pair(neary, fary, j, make_float2(sy, sy), make_float2(ay, ay));
            const float2 pz = plane_pair(nearz, farz, j, make_float2(sz, sz), make_float2(az, az));
            // the interval starts at 0, not at tmin: tmin belongs to the triangle test alone
            const float tn = fmaxf(fmaxf(px.x, py.x), fmaxf(pz.x, 0.0f));
            const float tf = fminf(fminf(px.y, py.y), fminf(pz.y, s.tmax));
            if (tn <= tf * kBoxRatio) hitmask |= ((child_bits4 >> (8 * j)) & 7u) << ((bit_index4 >> (8 * j)) & 31u);
        }
    }
    return hitmask;
}

// One traversal step (Ylitie, Karras, Laine 2017), while-while. In the node phase every lane
// without triangles visits the highest-priority internal child of its node group until few of
// the warp's lanes still search (kNodeExitPct); in the triangle phase the lanes test their
// triangle groups together until few still have some (kTriExitPct), the rest keeping their
// group in the ray state for the next step. Returns true when the ray is finished (s.hit /
// s.tmax / s.hu / s.hv hold the result). stack_overflow is set, and the ray abandoned, if the
// tree is deeper than the stack. any_hit: stop at the first hit (shadow rays); a run-time flag
// so one kernel can trace both kinds. Every lane of the calling warp that holds a ray calls it.
template <bool STATS>
NGI_D bool trav_step(TravState& s, uint2* stack, const CwNode* __restrict__ nodes, const float4* __restrict__ tris,
                     bool& stack_overflow, TraceStats* stats, bool any_hit) {
    const unsigned act = __activemask();
    uint2 tg = s.tgroup;
    while (true) {
        const bool want = tg.y == 0u && s.ngroup.y > 0x00FFFFFFu;
        // leave the node phase once few lanes still search: the others test their triangles
        // (or take new rays) instead of waiting for the last searching lanes
        const unsigned wm = __ballot_sync(act, want);
        if (wm == 0u || __popc(wm) * 100 < __popc(act) * kNodeExitPct) break;
        if (want) {
            const uint32_t hits = s.ngroup.y;
            const int bit = 31 - __clz(hits);
            s.ngroup.y &= ~(1u << bit);
            if (s.ngroup.y > 0x00FFFFFFu) {
                if (s.sp == kTraversalStack) {
                    stack_overflow = true;
                    s.hit = -1;
                    s.ngroup = make_uint2(0u, 0u);
                    s.sp = 0;
                    continue;
                }
                stack[s.sp++] = s.ngroup;
            }
            const uint32_t slot = (uint32_t)(bit - 24) ^ s.octinv;
            const uint32_t rel = __popc(hits & ~(0xFFFFFFFFu << slot));
            const uint32_t node = s.ngroup.x + rel;
            uint32_t child_base, tri_base, imask;
            const uint32_t hm = intersect_children(nodes, node, s, child_base, tri_base, imask);
            if (STATS) stats->nodes++;
            s.ngroup = make_uint2(child_base, (hm & 0xFF000000u) | imask);
            tg = make_uint2(tri_base, hm & 0x00FFFFFFu);
            if (s.ngroup.y <= 0x00FFFFFFu && tg.y == 0u && s.sp > 0) s.ngroup = stack[--s.sp];
        }
    }
    // every lane of `act` stays in this loop until the warp leaves it (the ballot needs them
    // all): an any-hit ray that is done drops its triangles and returns after the loop
    bool found = false;
    while (true) {
        const unsigned tm = __ballot_sync(act, tg.y != 0u);
        if (tm == 0u || __popc(tm) * 100 < __popc(act) * kTriExitPct) break;
        if (tg.y == 0u) continue;
        const int tb = 31 - __clz(tg.y);
        tg.y &= ~(1u << tb);
        const uint32_t ti = tg.x + (uint32_t)tb;
        const float4* tp = tris + 3 * (size_t)ti;
        const float4 p0 = __ldg(tp + 0), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
        if (STATS) stats->tris++;
        float t, u, v;
        if (tri_intersect(s.rp, p0, p1, p2, s.tmin, s.tmax, t, u, v)) {
            s.tmax = t;
            s.hu = u;
            s.hv = v;
            s.hit = (int)ti;
            if (any_hit) {
                found = true;
                tg.y = 0u;
            }
        }
    }
    s.tgroup = tg;
    if (found) return true;
    if (tg.y != 0u) return false;  // the rest of the group in the next step
    if (s.ngroup.y <= 0x00FFFFFFu) {
        if (s.sp == 0) return true;
        s.ngroup = stack[--s.sp];
    }
    return false;
}

// Whole traversal of one ray (parity hooks and simple callers). Returns the leaf-order
// triangle index of the nearest hit in [tmin, tmax) (ANY_HIT: of any hit) or -1; on a hit
// tmax is lowered to the hit distance.
template <bool ANY_HIT, bool STATS>
NGI_D int trace_ray(const CwNode* __restrict__ nodes, const float4* __restrict__ tris, int num_nodes,
                    float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float& tmax,
                    float& hu, float& hv, bool& stack_overflow, TraceStats* stats) {
    if (num_nodes == 0) return -1;
    TravState s;
    trav_init(s, ox, oy, oz, dx, dy, dz, tmin, tmax);
    uint2 stack[kTraversalStack];
    while (!trav_step<STATS>(s, stack, nodes, tris, stack_overflow, stats, ANY_HIT)) {
    }
    if (s.hit >= 0) {
        tmax = s.tmax;
        hu = s.hu;
        hv = s.hv;
    }
    return s.hit;
}

}  // namespace ngi
