// CPU oracle for nanogi's pt / ptdirect path -- TEST INFRASTRUCTURE ONLY.
//
// A plain FP64 restatement of the reference, written apart from the GPU code:
//   include/nanogi/rt.hpp   : sampling utilities 55-140, Primitive 483-1466,
//                             Scene::Intersect / Visible 2162-2261, emitter choice 2321-2352,
//                             GeometryTerm 2364-2374
//   include/nanogi/basic.hpp: Random 419-434, Distribution1D 440-497
//   src/nanogi.cpp          : ProcessSample_PT 446-607, ProcessSample_PTDirect 609-802,
//                             RenderProcess gather and normalisation 225-440
// Traversal is FP32 (the reference casts rays and vertices to float for Embree,
// rt.hpp:2119-2121, 2166-2173). Embree itself (v2.5.1, not vendored) is not available, so
// the triangle test is the watertight test of Woop, Benthin and Wald (JCGT 2013), evaluated
// with separate float multiplies and adds (build with -ffp-contract=off).
//
// PARITY UNPINNED: no reference outputs exist to pin this against (see ngi_oracle.h).
#include "ngi_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_err;

const double Pi = 3.14159265358979323846;
const double InvPi = 1.0 / Pi;
const float EpsF = 1e-4f;
const float InfF = 3.402823466e+38f;

struct dv3 {
    double x = 0, y = 0, z = 0;
    dv3() {}
    dv3(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
dv3 operator+(dv3 a, dv3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
dv3 operator-(dv3 a, dv3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
dv3 operator-(dv3 a) { return {-a.x, -a.y, -a.z}; }
dv3 operator*(dv3 a, dv3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
dv3 operator*(dv3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
dv3 operator*(double s, dv3 a) { return {a.x * s, a.y * s, a.z * s}; }
dv3 operator/(dv3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
dv3 operator/(dv3 a, dv3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
double dot(dv3 a, dv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
dv3 cross(dv3 a, dv3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double length(dv3 a) { return std::sqrt(dot(a, a)); }
// glm::normalize = v * inversesqrt(dot(v, v))
dv3 normalize(dv3 a) { return a * (1.0 / std::sqrt(dot(a, a))); }
bool is_zero(dv3 a) { return a.x == 0 && a.y == 0 && a.z == 0; }

enum { D = 1, G = 2, S = 4, L = 8, E = 16, BSDF = 7, Emitter = 24 };

// SurfaceGeometry (rt.hpp:282-302)
struct Geom {
    bool degenerated = false;
    dv3 p, sn, gn, dpdu, dpdv;
    double uv[2] = {0, 0};
    float ext = 0.0f;  // largest |coordinate| of the triangle under p (scaled ray offsets only)
    void ComputeTangentSpace() {
        // OrthonormalBasis(sn, dpdu, dpdv) (rt.hpp:55-59)
        const dv3 a = sn;
        dpdv = std::fabs(a.x) > std::fabs(a.y) ? normalize(dv3(a.z, 0, -a.x)) : normalize(dv3(0, a.z, -a.y));
        dpdu = normalize(cross(dpdv, a));
    }
    dv3 ToLocal(dv3 w) const { return {dot(dpdu, w), dot(dpdv, w), dot(sn, w)}; }
    dv3 ToWorld(dv3 l) const { return dpdu * l.x + dpdv * l.y + sn * l.z; }
};

// ---- sampling utilities (rt.hpp:87-140) --------------------------------------------------
void ConcentricDisk(double u0, double u1, double& sx, double& sy) {
    const double vx = 2.0 * u0 - 1.0, vy = 2.0 * u1 - 1.0;
    if (vx == 0 && vy == 0) { sx = sy = 0; return; }
    double r, theta;
    if (vx > -vy) {
        if (vx > vy) { r = vx; theta = (Pi * 0.25) * vy / vx; }
        else { r = vy; theta = (Pi * 0.25) * (2.0 - vx / vy); }
    } else {
        if (vx < vy) { r = -vx; theta = (Pi * 0.25) * (4.0 + vy / vx); }
        else { r = -vy; theta = (Pi * 0.25) * (6.0 - vx / vy); }
    }
    sx = r * std::cos(theta);
    sy = r * std::sin(theta);
}
dv3 CosineSampleHemisphere(double u0, double u1) {
    double sx, sy;
    ConcentricDisk(u0, u1, sx, sy);
    return {sx, sy, std::sqrt(std::max(0.0, 1.0 - sx * sx - sy * sy))};
}
void UniformSampleTriangle(double u0, double u1, double& b0, double& b1) {
    const double s = std::sqrt(std::max(0.0, u0));
    b0 = 1.0 - s;
    b1 = u1 * s;
}
int PixelIndex(double rx, double ry, int w, int h) {
    const int px = std::min(std::max((int)(rx * w), 0), w - 1);
    const int py = std::min(std::max((int)(ry * h), 0), h - 1);
    return py * w + px;
}

// Distribution1D (basic.hpp:440-497)
struct Dist1D {
    std::vector<double> cdf{0.0};
    void Add(double v) { cdf.push_back(cdf.back() + v); }
    void Normalize() {
        const double inv = 1.0 / cdf.back();
        for (auto& v : cdf) v *= inv;
    }
    int SampleReuse(double u, double& u2) const {
        int v = (int)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) - 1;
        int i = std::min(std::max(v, 0), (int)cdf.size() - 2);
        u2 = (u - cdf[i]) / (cdf[i + 1] - cdf[i]);
        return i;
    }
};

struct Prim {
    ora_prim_desc d;
    dv3 Le, lpos, ldir, lcenter;
    double lradius = 0, inv_area = 0;
    Dist1D dist;
    // pinhole
    dv3 eye, Vx, Vy, Vz, We;
    double fov = 0, aspect = 1;
    dv3 DR, GR, Geta, Gk, SR;
    std::vector<float> Dtex, Gtex;  // TexR texels (copies of the descriptor's arrays)
};

void CopyTextures(Prim& p) {
    if (p.d.D_tex) p.Dtex.assign(p.d.D_tex, p.d.D_tex + 3 * (size_t)p.d.D_tex_w * p.d.D_tex_h);
    if (p.d.G_tex) p.Gtex.assign(p.d.G_tex, p.d.G_tex + 3 * (size_t)p.d.G_tex_w * p.d.G_tex_h);
    p.d.D_tex = p.d.G_tex = nullptr;
}

// Texture::Evaluate (rt.hpp:260-266): nearest texel, uv wrapped by fract.
dv3 TexEval(const std::vector<float>& tex, int w, int h, const double uv[2]) {
    const int x = std::min(std::max((int)((uv[0] - std::floor(uv[0])) * w), 0), w - 1);
    const int y = std::min(std::max((int)((uv[1] - std::floor(uv[1])) * h), 0), h - 1);
    const size_t i = (size_t)w * y + x;
    return dv3(tex[3 * i], tex[3 * i + 1], tex[3 * i + 2]);
}

dv3 V(const double a[3]) { return {a[0], a[1], a[2]}; }

// ---- FP32 traversal -------------------------------------------------------------------------
struct Tri {
    float p[3][3];
};

struct RayF {
    float o[3], d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float inv[3];
};

RayF MakeRay(const float o[3], const float d[3]) {
    RayF r;
    for (int k = 0; k < 3; k++) { r.o[k] = o[k]; r.d[k] = d[k]; }
    const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    for (int k = 0; k < 3; k++) {
        const float dd = std::fabs(d[k]) > 1e-20f ? d[k] : std::copysign(1e-20f, d[k]);
        r.inv[k] = 1.0f / dd;
    }
    return r;
}

// Watertight ray/triangle test; hit iff tmin <= t < tbest.
bool TriTest(const RayF& r, const Tri& tr, float tmin, float tbest, float& t, float& u, float& v) {
    float A[3], B[3], C[3];
    for (int k = 0; k < 3; k++) {
        A[k] = tr.p[0][k] - r.o[k];
        B[k] = tr.p[1][k] - r.o[k];
        C[k] = tr.p[2][k] - r.o[k];
    }
    const float Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
    const float Bx = B[r.kx] - r.Sx * B[r.kz], By = B[r.ky] - r.Sy * B[r.kz];
    const float Cx = C[r.kx] - r.Sx * C[r.kz], Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float Vv = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || Vv == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        Vv = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || Vv < 0.0f || W < 0.0f) && (U > 0.0f || Vv > 0.0f || W > 0.0f)) return false;
    const float det = (U + Vv) + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * A[r.kz], Bz = r.Sz * B[r.kz], Cz = r.Sz * C[r.kz];
    const float T = (U * Az + Vv * Bz) + W * Cz;
    const float rcp = 1.0f / det;
    const float tt = T * rcp;
    if (!(tt >= tmin && tt < tbest)) return false;
    t = tt;
    u = Vv * rcp;
    v = W * rcp;
    return true;
}

struct BNode {
    float lo[3], hi[3];
    int left = -1, right = -1;  // internal children; leaf: left = -1
    int first = 0, count = 0;
};

struct Bvh {
    std::vector<BNode> nodes;
    std::vector<int> order;
};

// Box test over [0, tbest]: the ray's tmin is applied by the triangle test alone, so the BVH finds
// every hit the brute force finds (a triangle test can put t above tmin for a triangle whose
// plane the ray crosses just below it: the test's rounding scales with the vertex coordinates).
bool BoxTest(const RayF& r, const BNode& n, float tmin, float tbest) {
    (void)tmin;
    float tn = 0.0f, tf = tbest;
    for (int k = 0; k < 3; k++) {
        float a = (n.lo[k] - r.o[k]) * r.inv[k];
        float b = (n.hi[k] - r.o[k]) * r.inv[k];
        if (a > b) std::swap(a, b);
        tn = std::max(tn, a);
        tf = std::min(tf, b);
    }
    const float kLo = 1.0f - 1.0f / 1048576.0f, kHi = 1.0f + 1.0f / 1048576.0f;
    return tn * kLo <= tf * kHi;
}

void BuildBvh(const std::vector<Tri>& tris, Bvh& bvh) {
    const int n = (int)tris.size();
    bvh.nodes.clear();
    bvh.order.resize(n);
    for (int i = 0; i < n; i++) bvh.order[i] = i;
    if (n == 0) return;
    std::vector<float> cen(3 * (size_t)n), blo(3 * (size_t)n), bhi(3 * (size_t)n);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            const float a = tris[i].p[0][k], b = tris[i].p[1][k], c = tris[i].p[2][k];
            blo[3 * i + k] = std::min(a, std::min(b, c));
            bhi[3 * i + k] = std::max(a, std::max(b, c));
            cen[3 * i + k] = 0.5f * (blo[3 * i + k] + bhi[3 * i + k]);
        }
    struct Item { int node, first, count; };
    bvh.nodes.reserve(2 * (size_t)n);
    bvh.nodes.push_back(BNode());
    std::vector<Item> stack{{0, 0, n}};
    const int kBins = 16;
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        BNode nd;
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = 0; k < 3; k++) { nd.lo[k] = INFINITY; nd.hi[k] = -INFINITY; }
        for (int i = it.first; i < it.first + it.count; i++) {
            const int t = bvh.order[i];
            for (int k = 0; k < 3; k++) {
                nd.lo[k] = std::min(nd.lo[k], blo[3 * t + k]);
                nd.hi[k] = std::max(nd.hi[k], bhi[3 * t + k]);
                clo[k] = std::min(clo[k], cen[3 * t + k]);
                chi[k] = std::max(chi[k], cen[3 * t + k]);
            }
        }
        nd.first = it.first;
        nd.count = it.count;
        int axis = -1, split_bin = -1;
        if (it.count > 4) {
            double best = INFINITY;
            for (int k = 0; k < 3; k++) {
                const float ext = chi[k] - clo[k];
                if (!(ext > 0)) continue;
                int cnt[kBins] = {0};
                float bl[kBins][3], bh[kBins][3];
                for (int b = 0; b < kBins; b++)
                    for (int q = 0; q < 3; q++) { bl[b][q] = INFINITY; bh[b][q] = -INFINITY; }
                for (int i = it.first; i < it.first + it.count; i++) {
                    const int t = bvh.order[i];
                    int b = (int)((cen[3 * t + k] - clo[k]) / ext * kBins);
                    b = std::min(std::max(b, 0), kBins - 1);
                    cnt[b]++;
                    for (int q = 0; q < 3; q++) {
                        bl[b][q] = std::min(bl[b][q], blo[3 * t + q]);
                        bh[b][q] = std::max(bh[b][q], bhi[3 * t + q]);
                    }
                }
                auto area = [](const float* l, const float* h) {
                    if (!(h[0] >= l[0])) return 0.0;
                    const double x = h[0] - l[0], y = h[1] - l[1], z = h[2] - l[2];
                    return x * y + y * z + z * x;
                };
                double rl[kBins], rr[kBins];
                int nl[kBins], nr[kBins];
                float al[3] = {INFINITY, INFINITY, INFINITY}, ah[3] = {-INFINITY, -INFINITY, -INFINITY};
                int c = 0;
                for (int b = 0; b < kBins; b++) {
                    c += cnt[b];
                    for (int q = 0; q < 3; q++) { al[q] = std::min(al[q], bl[b][q]); ah[q] = std::max(ah[q], bh[b][q]); }
                    rl[b] = area(al, ah);
                    nl[b] = c;
                }
                for (int q = 0; q < 3; q++) { al[q] = INFINITY; ah[q] = -INFINITY; }
                c = 0;
                for (int b = kBins - 1; b >= 0; b--) {
                    c += cnt[b];
                    for (int q = 0; q < 3; q++) { al[q] = std::min(al[q], bl[b][q]); ah[q] = std::max(ah[q], bh[b][q]); }
                    rr[b] = area(al, ah);
                    nr[b] = c;
                }
                for (int b = 0; b < kBins - 1; b++) {
                    if (nl[b] == 0 || nr[b + 1] == 0) continue;
                    const double cost = rl[b] * nl[b] + rr[b + 1] * nr[b + 1];
                    if (cost < best) { best = cost; axis = k; split_bin = b; }
                }
            }
        }
        if (axis < 0) {
            if (it.count > 4) {
                // All centroids equal (or no useful split): halve by index.
                axis = 3;
            }
        }
        if (axis < 0) {
            bvh.nodes[it.node] = nd;
            continue;
        }
        int mid;
        if (axis == 3) {
            mid = it.first + it.count / 2;
        } else {
            const float ext = chi[axis] - clo[axis];
            auto pivot = std::partition(bvh.order.begin() + it.first, bvh.order.begin() + it.first + it.count, [&](int t) {
                int b = (int)((cen[3 * t + axis] - clo[axis]) / ext * kBins);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= split_bin;
            });
            mid = (int)(pivot - bvh.order.begin());
            if (mid == it.first || mid == it.first + it.count) mid = it.first + it.count / 2;
        }
        const int l = (int)bvh.nodes.size();
        bvh.nodes.push_back(BNode());
        bvh.nodes.push_back(BNode());
        nd.left = l;
        nd.right = l + 1;
        bvh.nodes[it.node] = nd;
        stack.push_back({l, it.first, mid - it.first});
        stack.push_back({l + 1, mid, it.first + it.count - mid});
    }
}

struct Hit {
    int tri = -1;
    float t = 0, u = 0, v = 0;
};

}  // namespace

struct ora_scene {
    std::vector<Prim> prims;
    std::vector<int> lights;
    int sensor = -1;
    std::vector<Tri> tris;
    std::vector<double> pos;  // 9 per tri (double of the float vertex)
    std::vector<double> nrm;  // 9 per tri
    std::vector<double> uv;   // 6 per tri
    std::vector<int> tri_prim;
    Bvh bvh;
    dv3 bmin, bmax;
};

namespace {

Hit IntersectBrute(const ora_scene& s, const RayF& r, float tmin, float tmax, bool any) {
    Hit h;
    float tb = tmax;
    for (size_t i = 0; i < s.tris.size(); i++) {
        float t, u, v;
        if (TriTest(r, s.tris[i], tmin, tb, t, u, v)) {
            tb = t;
            h.tri = (int)i; h.t = t; h.u = u; h.v = v;
            if (any) return h;
        }
    }
    return h;
}

Hit IntersectBvh(const ora_scene& s, const RayF& r, float tmin, float tmax, bool any) {
    Hit h;
    if (s.bvh.nodes.empty()) return h;
    float tb = tmax;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const BNode& n = s.bvh.nodes[stack[--sp]];
        if (!BoxTest(r, n, tmin, tb)) continue;
        if (n.left < 0) {
            for (int i = n.first; i < n.first + n.count; i++) {
                const int ti = s.bvh.order[i];
                float t, u, v;
                if (TriTest(r, s.tris[ti], tmin, tb, t, u, v)) {
                    tb = t;
                    h.tri = ti; h.t = t; h.u = u; h.v = v;
                    if (any) return h;
                }
            }
        } else {
            if (sp + 2 > 128) { g_err = "oracle BVH stack overflow"; return h; }
            stack[sp++] = n.right;
            stack[sp++] = n.left;
        }
    }
    return h;
}

struct Isect {
    Geom geom;
    int prim = -1;
};

float MaxAbs3(dv3 a, dv3 b, dv3 c) {
    double m = 0.0;
    for (double x : {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z}) m = std::max(m, std::fabs(x));
    return (float)m;
}

// Scene::Intersect (rt.hpp:2162-2244); offset_mode 1 puts the hit point on the triangle
// (barycentric) instead of at o + t d, for the scaled ray offsets.
bool Intersect(const ora_scene& s, bool use_bvh, dv3 o, dv3 d, Isect& is, float minT, float maxT,
               int offset_mode = 0) {
    const float of[3] = {(float)o.x, (float)o.y, (float)o.z};
    const float df[3] = {(float)d.x, (float)d.y, (float)d.z};
    const RayF r = MakeRay(of, df);
    const Hit h = use_bvh ? IntersectBvh(s, r, minT, maxT, false) : IntersectBrute(s, r, minT, maxT, false);
    if (h.tri < 0) return false;
    const int f = h.tri;
    is.prim = s.tri_prim[f];
    const double* P = &s.pos[9 * (size_t)f];
    const dv3 p1(P[0], P[1], P[2]), p2(P[3], P[4], P[5]), p3(P[6], P[7], P[8]);
    is.geom.gn = normalize(cross(p2 - p1, p3 - p1));
    const double* N = &s.nrm[9 * (size_t)f];
    const dv3 n1(N[0], N[1], N[2]), n2(N[3], N[4], N[5]), n3(N[6], N[7], N[8]);
    const float w = 1.0f - h.u - h.v;
    if (offset_mode == 1) {
        is.geom.p = p1 * (double)w + p2 * (double)h.u + p3 * (double)h.v;
        is.geom.ext = MaxAbs3(p1, p2, p3);
    } else {
        is.geom.p = o + d * (double)h.t;
        is.geom.ext = 0.0f;
    }
    is.geom.sn = normalize(n1 * (double)w + n2 * (double)h.u + n3 * (double)h.v);
    if (std::isnan(is.geom.sn.x) || std::isnan(is.geom.sn.y) || std::isnan(is.geom.sn.z)) is.geom.sn = is.geom.gn;
    const double* T = &s.uv[6 * (size_t)f];
    is.geom.uv[0] = T[0] * (double)w + T[2] * (double)h.u + T[4] * (double)h.v;
    is.geom.uv[1] = T[1] * (double)w + T[3] * (double)h.u + T[5] * (double)h.v;
    is.geom.degenerated = false;
    is.geom.ComputeTangentSpace();
    return true;
}

// Scaled ray offsets (not in the reference, which always uses tmin = EpsF, rt.hpp:2248):
// a surface point moves 2^-17 x (largest |coordinate| of its triangle) along the geometric
// normal, to the side the ray leaves by; tmin = 0. Shadow rays move both ends and stop 2^-16
// of their length short of the moved target.
dv3 OffsetPoint(const Geom& g, dv3 toward) {
    if (g.degenerated || !(g.ext > 0.0f)) return g.p;
    const double delta = (double)(g.ext * (1.0f / 131072.0f));
    return g.p + g.gn * (dot(g.gn, toward) >= 0.0 ? delta : -delta);
}

dv3 ToFloat(dv3 v) { return dv3((float)v.x, (float)v.y, (float)v.z); }

// Ray origin (a float point, held in doubles) and tmin for a ray leaving g toward d.
dv3 RayOrigin(const Geom& g, dv3 d, int mode, float& tmin) {
    if (mode != 1) {
        tmin = EpsF;
        return g.p;
    }
    tmin = 0.0f;
    return ToFloat(OffsetPoint(g, d));
}

// Visibility between two moved points (scaled offsets): tmin = 0, tmax short by 2^-16.
bool VisibleBetween(const ora_scene& s, bool use_bvh, dv3 a, dv3 b) {
    const dv3 v = b - a;
    const double len = length(v);
    const dv3 d = v / len;
    const float of[3] = {(float)a.x, (float)a.y, (float)a.z};
    const float df[3] = {(float)d.x, (float)d.y, (float)d.z};
    const RayF r = MakeRay(of, df);
    const float tmax = (float)len * (1.0f - 1.0f / 65536.0f);
    const Hit h = use_bvh ? IntersectBvh(s, r, 0.0f, tmax, true) : IntersectBrute(s, r, 0.0f, tmax, true);
    return h.tri < 0;
}

// Scene::Visible (rt.hpp:2254-2262)
bool Visible(const ora_scene& s, bool use_bvh, dv3 p1, dv3 p2) {
    const dv3 v = p2 - p1;
    const double len = length(v);
    const dv3 d = v / len;
    const float of[3] = {(float)p1.x, (float)p1.y, (float)p1.z};
    const float df[3] = {(float)d.x, (float)d.y, (float)d.z};
    const RayF r = MakeRay(of, df);
    const float tmax = (float)len * (1.0f - EpsF);
    const Hit h = use_bvh ? IntersectBvh(s, r, EpsF, tmax, true) : IntersectBrute(s, r, EpsF, tmax, true);
    return h.tri < 0;
}

// ---- Primitive methods (rt.hpp:483-1466) ------------------------------------------------------
double LocalTan(dv3 v) {
    const double t = 1.0 - v.z * v.z;
    return t <= 0 ? 0 : std::sqrt(t) / v.z;
}
double Beckmann(const Prim& p, dv3 H) {
    if (H.z <= 0) return 0.0;
    const double ex = LocalTan(H) / p.d.G_roughness;
    const double t1 = std::exp(-(ex * ex));
    const double t2 = (Pi * p.d.G_roughness * p.d.G_roughness * std::pow(H.z, 4.0));
    return t1 / t2;
}
double ShadowMasking(dv3 wi, dv3 wo, dv3 H) {
    const double nH = H.z, nwo = wo.z, nwi = wi.z;
    const double woH = std::fabs(dot(wo, H));
    const double wiH = std::fabs(dot(wo, H));  // the reference uses wo here (rt.hpp:1429)
    return std::min(1.0, std::min(2.0 * nH * nwo / woH, 2.0 * nH * nwi / wiH));
}
dv3 FrConductor(const Prim& p, double c) {
    const dv3 eta = p.Geta, k = p.Gk;
    const dv3 tmp = (eta * eta + k * k) * (c * c);
    const dv3 one(1, 1, 1), cc(c * c, c * c, c * c);
    const dv3 rParl2 = (tmp - (eta * (2.0 * c)) + one) / (tmp + (eta * (2.0 * c)) + one);
    const dv3 tmpF = eta * eta + k * k;
    const dv3 rPerp2 = (tmpF - (eta * (2.0 * c)) + cc) / (tmpF + (eta * (2.0 * c)) + cc);
    return (rParl2 + rPerp2) * 0.5;
}
double FresnelTerm(dv3 lwi, double etaI, double etaT) {
    const double wiDotN = lwi.z;
    const double eta = etaI / etaT;
    const double c2t = 1.0 - eta * eta * (1.0 - wiDotN * wiDotN);
    if (c2t <= 0) return 1;
    const double aci = std::fabs(wiDotN), act = std::sqrt(c2t);
    const double rhoS = (etaI * aci - etaT * act) / (etaI * aci + etaT * act);
    const double rhoT = (etaI * act - etaT * aci) / (etaI * act + etaT * aci);
    return (rhoS * rhoS + rhoT * rhoT) * 0.5;
}

bool RasterPosition(const Prim& p, dv3 wo, const Geom& g, double& rx, double& ry) {
    if (p.d.e_type == 1) {
        const dv3 we(dot(p.Vx, wo), dot(p.Vy, wo), dot(p.Vz, wo));
        if (we.z >= 0) return false;
        const double tf = std::tan(p.fov * 0.5);
        rx = (-we.x / we.z / tf / p.aspect + 1.0) * 0.5;
        ry = (-we.y / we.z / tf + 1.0) * 0.5;
        return !(rx < 0 || rx > 1 || ry < 0 || ry > 1);
    }
    rx = g.uv[0];
    ry = g.uv[1];
    return true;
}

void SampleTriangleMesh(const ora_scene& s, const Prim& p, double u0, double u1, Geom& g) {
    double u2;
    const int i = p.dist.SampleReuse(u0, u2);
    double b0, b1;
    UniformSampleTriangle(u2, u1, b0, b1);
    const size_t f = (size_t)(p.d.tri_first + i);
    const double* P = &s.pos[9 * f];
    const dv3 p1(P[0], P[1], P[2]), p2(P[3], P[4], P[5]), p3(P[6], P[7], P[8]);
    g.p = p1 * (1.0 - b0 - b1) + p2 * b0 + p3 * b1;
    const double* T = &s.uv[6 * f];
    g.uv[0] = T[0] * (1.0 - b0 - b1) + T[2] * b0 + T[4] * b1;
    g.uv[1] = T[1] * (1.0 - b0 - b1) + T[3] * b0 + T[5] * b1;
    g.degenerated = false;
    g.ext = MaxAbs3(p1, p2, p3);
    g.gn = normalize(cross(p2 - p1, p3 - p1));
    g.sn = g.gn;
    g.ComputeTangentSpace();
}

// SamplePosition (rt.hpp:483-592)
void SamplePosition(const ora_scene& s, const Prim& p, double u0, double u1, Geom& g) {
    if (p.d.type & L) {
        if (p.d.l_type == 0) { SampleTriangleMesh(s, p, u0, u1, g); return; }
        if (p.d.l_type == 1) { g.degenerated = true; g.p = p.lpos; return; }
        double sx, sy;
        ConcentricDisk(u0, u1, sx, sy);
        sx *= p.lradius;
        sy *= p.lradius;
        g.degenerated = false;
        g.gn = p.ldir;
        g.sn = g.gn;
        g.ComputeTangentSpace();
        g.p = p.lcenter - p.ldir * p.lradius + (g.dpdu * sx + g.dpdv * sy);
        return;
    }
    if (p.d.e_type == 0) { SampleTriangleMesh(s, p, u0, u1, g); return; }
    g.degenerated = true;
    g.p = p.eye;
}

// EvaluatePositionPDF (rt.hpp:643-690) with forceDegenerated = true
double PositionPdf(const Prim& p) {
    if (p.d.type & L) return p.d.l_type == 1 ? 1.0 : p.inv_area;
    return p.d.e_type == 1 ? 1.0 : p.inv_area;
}

// SampleDirection (rt.hpp:692-910); wo stays zero where the reference returns early.
dv3 SampleDirection(const Prim& p, double u0, double u1, double ucomp, int type, const Geom& g, dv3 wi) {
    dv3 wo(0, 0, 0);
    if (type & L) {
        if (p.d.l_type == 0) return g.ToWorld(CosineSampleHemisphere(u0, u1));
        if (p.d.l_type == 1) {
            const double z = 1.0 - 2.0 * u0, r = std::sqrt(std::max(0.0, 1.0 - z * z)), phi = 2.0 * Pi * u1;
            return {r * std::cos(phi), r * std::sin(phi), z};
        }
        return p.ldir;
    }
    if (type & E) {
        if (p.d.e_type == 0) return g.ToWorld(CosineSampleHemisphere(u0, u1));
        const double rx = 2.0 * u0 - 1.0, ry = 2.0 * u1 - 1.0;
        const double tf = std::tan(p.fov * 0.5);
        const dv3 we = normalize(dv3(p.aspect * tf * rx, tf * ry, -1));
        return p.Vx * we.x + p.Vy * we.y + p.Vz * we.z;
    }
    const dv3 lwi = g.ToLocal(wi);
    if (type & D) {
        if (lwi.z <= 0) return wo;
        return g.ToWorld(CosineSampleHemisphere(u0, u1));
    }
    if (type & G) {
        if (lwi.z <= 0) return wo;
        const double r = p.d.G_roughness;
        const double tan2 = -r * r * std::log(1.0 - u0);
        const double ch = 1.0 / std::sqrt(1.0 + tan2);
        const double sh = std::sqrt(std::max(0.0, 1.0 - ch * ch));
        const double phi = 2.0 * Pi * u1;
        const dv3 H(sh * std::cos(phi), sh * std::sin(phi), ch);
        const dv3 lwo = -lwi - 2.0 * dot(-lwi, H) * H;
        if (lwo.z <= 0) return wo;
        return g.ToWorld(lwo);
    }
    if (type & S) {
        if (p.d.s_type == 0) {
            if (lwi.z <= 0) return wo;
            return g.ToWorld(dv3(-lwi.x, -lwi.y, lwi.z));
        }
        double ei = p.d.S_eta1, et = p.d.S_eta2;
        if (lwi.z < 0) std::swap(ei, et);
        const double eta = ei / et;
        bool reflect;
        if (p.d.s_type == 1) reflect = 1.0 - eta * eta * (1.0 - lwi.z * lwi.z) <= 0;
        else reflect = ucomp <= FresnelTerm(lwi, ei, et);
        if (reflect) return g.ToWorld(dv3(-lwi.x, -lwi.y, lwi.z));
        const double c2t = 1.0 - eta * eta * (1.0 - lwi.z * lwi.z);
        const double ct = std::sqrt(c2t) * (lwi.z > 0 ? -1.0 : 1.0);
        return g.ToWorld(dv3(-eta * lwi.x, -eta * lwi.y, ct));
    }
    return wo;
}

// EvaluateDirection (rt.hpp:912-1148), transDir = EL unless le is set
dv3 EvaluateDirection(const Prim& p, const Geom& g, int type, dv3 wi, dv3 wo, bool le, bool force) {
    const dv3 zero(0, 0, 0);
    if (type & Emitter) {
        if (type & L) {
            if (p.d.l_type == 0) return g.ToLocal(wo).z <= 0 ? zero : p.Le;
            if (p.d.l_type == 1) return p.Le;
            return force ? p.Le : zero;
        }
        if (p.d.e_type == 0) return g.ToLocal(wo).z <= 0 ? zero : p.We;
        double rx, ry;
        if (!RasterPosition(p, wo, g, rx, ry)) return zero;
        const double ez = dot(p.Vz, wo);
        const double tf = std::tan(p.fov * 0.5);
        const double cosT = -ez, inv = 1.0 / cosT, A = tf * tf * p.aspect * 4.0;
        const double w = inv * inv * inv / A;
        return {w, w, w};
    }
    const dv3 lwi = g.ToLocal(wi), lwo = g.ToLocal(wo);
    double corr;
    {
        const double wiNg = dot(wi, g.gn), woNg = dot(wo, g.gn);
        if (wiNg * lwi.z <= 0 || woNg * lwo.z <= 0) corr = 0;
        else if (le) corr = lwi.z * woNg / (lwo.z * wiNg);
        else corr = 1;
    }
    if (type & D) {
        if (lwi.z <= 0 || lwo.z <= 0) return zero;
        const dv3 R = p.Dtex.empty() ? p.DR : TexEval(p.Dtex, p.d.D_tex_w, p.d.D_tex_h, g.uv);
        return R * InvPi * corr;
    }
    if (type & G) {
        if (lwi.z <= 0 || lwo.z <= 0) return zero;
        const dv3 H = normalize(lwi + lwo);
        const double Dd = Beckmann(p, H);
        const double Gg = ShadowMasking(lwi, lwo, H);
        const dv3 F = FrConductor(p, dot(lwi, H));
        const dv3 R = p.Gtex.empty() ? p.GR : TexEval(p.Gtex, p.d.G_tex_w, p.d.G_tex_h, g.uv);
        return R * Dd * Gg * F / (4.0 * lwi.z) / lwo.z * corr;
    }
    if (type & S) {
        if (!force) return zero;
        if (p.d.s_type == 0) {
            if (lwi.z <= 0 || lwo.z <= 0) return zero;
            return p.SR * corr;
        }
        double ei = p.d.S_eta1, et = p.d.S_eta2;
        if (lwi.z < 0) std::swap(ei, et);
        const double eta = ei / et;
        const double rc = le ? 1.0 : eta;
        if (p.d.s_type == 1) return p.SR * corr * rc * rc;
        const double Fr = FresnelTerm(lwi, ei, et);
        if (lwi.z * lwo.z >= 0) return p.SR * Fr * corr;
        return p.SR * (1.0 - Fr) * corr * rc * rc;
    }
    return zero;
}

// EvaluateDirectionPDF (rt.hpp:1150-1336), forceDegenerated = true
double EvaluateDirectionPdf(const Prim& p, const Geom& g, int type, dv3 wi, dv3 wo) {
    if (type & L) {
        if (p.d.l_type == 0) return g.ToLocal(wo).z <= 0 ? 0 : InvPi;
        if (p.d.l_type == 1) return InvPi * 0.25;
        return 1;
    }
    if (type & E) {
        if (p.d.e_type == 0) return g.ToLocal(wo).z <= 0 ? 0 : InvPi;
        double rx, ry;
        if (!RasterPosition(p, wo, g, rx, ry)) return 0;
        const double ez = dot(p.Vz, wo);
        const double tf = std::tan(p.fov * 0.5);
        const double inv = 1.0 / -ez, A = tf * tf * p.aspect * 4.0;
        return inv * inv * inv / A;
    }
    const dv3 lwi = g.ToLocal(wi), lwo = g.ToLocal(wo);
    if (type & D) return (lwi.z <= 0 || lwo.z <= 0) ? 0 : InvPi;
    if (type & G) {
        if (lwi.z <= 0 || lwo.z <= 0) return 0;
        const dv3 H = normalize(lwi + lwo);
        return Beckmann(p, H) * H.z / (4.0 * dot(lwo, H)) / lwo.z;
    }
    if (type & S) {
        if (p.d.s_type == 0) return (lwi.z <= 0 || lwo.z <= 0) ? 0 : 1;
        if (p.d.s_type == 1) return 1;
        double ei = p.d.S_eta1, et = p.d.S_eta2;
        if (lwi.z < 0) std::swap(ei, et);
        const double Fr = FresnelTerm(lwi, ei, et);
        return lwi.z * lwo.z >= 0 ? Fr : 1.0 - Fr;
    }
    return 0;
}

double GeometryTerm(const Geom& a, const Geom& b) {
    dv3 d = b.p - a.p;
    const double l2 = dot(d, d), l = std::sqrt(l2);
    d = d / l;
    double t = 1.0;
    if (!a.degenerated) t *= std::fabs(dot(a.sn, d));
    if (!b.degenerated) t *= std::fabs(dot(b.sn, -d));
    return t / l2;
}

// ---- random numbers ----------------------------------------------------------------------------
void Philox(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Random numbers of one sample. Replay mode addresses each number by (vertex, call, lane);
// reference mode returns the next value of the thread's mt19937 stream in the order the
// reference draws them (C++ leaves the order of function-argument evaluation unspecified,
// so Next2D / SampleDirection argument draws are taken left to right here).
struct Sampler {
    bool replay = false;
    // reference mode
    std::mt19937* eng = nullptr;
    std::uniform_real_distribution<double>* dist = nullptr;
    // replay mode
    uint32_t key[2] = {0, 0};
    uint64_t sample = 0;
    uint32_t cache_vertex = 0xFFFFFFFFu, cache_call = 0xFFFFFFFFu;
    uint32_t cache[4] = {0, 0, 0, 0};

    double get(uint32_t vertex, uint32_t call, int lane) {
        if (!replay) return (*dist)(*eng);
        if (vertex != cache_vertex || call != cache_call) {
            const uint32_t ctr[4] = {(uint32_t)sample, (uint32_t)(sample >> 32), vertex, call};
            Philox(ctr, key, cache);
            cache_vertex = vertex;
            cache_call = call;
        }
        return (double)((float)(cache[lane] >> 8) * (1.0f / 16777216.0f));
    }
};

enum : uint32_t { CALL_NEE_RR = 0, CALL_DIR = 1, CALL_SENSOR = 2 };

struct RenderCtx {
    const ora_scene* s;
    const ora_render_params* p;
    std::vector<double>* film;
    int64_t cam = 0, ext = 0, sh = 0, miss = 0;
    long long strat_end = 0;
};

// Pinhole raster sample for the sensor vertex: the reference uses u uniform over the image
// (rt.hpp:735 with u from src/nanogi.cpp:495); replay mode may stratify by pixel.
void CameraRaster(RenderCtx& c, Sampler& smp, double& u0, double& u1) {
    u0 = smp.get(1, CALL_DIR, 0);
    u1 = smp.get(1, CALL_DIR, 1);
    if (smp.replay && c.p->raster_mode == 0 && (long long)smp.sample < c.strat_end) {
        const long long wh = (long long)c.p->width * c.p->height;
        const long long pidx = (long long)(smp.sample % (uint64_t)wh);
        const int px = (int)(pidx % c.p->width), py = (int)(pidx / c.p->width);
        u0 = ((double)px + u0) / (double)c.p->width;
        u1 = ((double)py + u1) / (double)c.p->height;
    }
}

void Accumulate(std::vector<double>& film, int pix, dv3 v) {
    film[3 * (size_t)pix] += v.x;
    film[3 * (size_t)pix + 1] += v.y;
    film[3 * (size_t)pix + 2] += v.z;
}

// ProcessSample_PT / ProcessSample_PTDirect (src/nanogi.cpp:446-802)
void ProcessSample(RenderCtx& c, Sampler& smp) {
    const ora_scene& s = *c.s;
    const ora_render_params& P = *c.p;
    const bool direct = P.renderer == 1;
    const bool bvh = P.use_bvh != 0;
    std::vector<double>& film = *c.film;

    // Sample a sensor: SampleEmitter(E, u) picks the single sensor, pdfE = 1
    smp.get(1, CALL_SENSOR, 2);
    const Prim& Ep = s.prims[s.sensor];
    Geom geomE;
    const double us0 = smp.get(1, CALL_SENSOR, 0), us1 = smp.get(1, CALL_SENSOR, 1);
    SamplePosition(s, Ep, us0, us1, geomE);
    const double pdfPE = PositionPdf(Ep);
    dv3 throughput = dv3(1, 1, 1) / pdfPE / 1.0;
    const Prim* prim = &Ep;
    int type = E;
    Geom geom = geomE;
    dv3 wi(0, 0, 0);
    int pixel = -1;
    int nv = 1;
    c.cam++;
    while (true) {
        if (P.max_vertices != -1 && nv >= P.max_vertices) break;
        if (direct) {
            // Direct light sampling (src/nanogi.cpp:656-707)
            const int n = (int)s.lights.size();
            const double ul = smp.get(nv, CALL_NEE_RR, 0);
            const int li = std::min(std::max((int)(ul * n), 0), n - 1);
            const Prim& Lp = s.prims[s.lights[li]];
            const double pdfL = 1.0 / n;
            Geom geomL;
            const double a0 = smp.get(nv, CALL_NEE_RR, 1), a1 = smp.get(nv, CALL_NEE_RR, 2);
            SamplePosition(s, Lp, a0, a1, geomL);
            const double pdfPL = PositionPdf(Lp);
            const dv3 ppL = normalize(geomL.p - geom.p);
            const dv3 fsE = EvaluateDirection(*prim, geom, type, wi, ppL, false, false);
            const dv3 fsL = EvaluateDirection(Lp, geomL, L, dv3(), -ppL, true, false);
            const double Gt = GeometryTerm(geom, geomL);
            const dv3 Cpre = throughput * fsE * Gt;
            double Vis = 0.0;
            // Only trace the shadow ray when it can matter (same result as always tracing)
            if (!is_zero(Cpre * fsL)) {
                c.sh++;
                if (P.ray_offset == 1) {
                    const dv3 a = ToFloat(OffsetPoint(geom, geomL.p - geom.p));
                    const dv3 b = OffsetPoint(geomL, geom.p - geomL.p);
                    Vis = VisibleBetween(s, bvh, a, b) ? 1.0 : 0.0;
                } else {
                    Vis = Visible(s, bvh, geom.p, geomL.p) ? 1.0 : 0.0;
                }
            }
            const dv3 C = throughput * fsE * Gt * Vis * fsL * 1.0 / pdfL / pdfPL;
            if (!is_zero(C)) {
                int index = pixel;
                if (type == E) {
                    double rx, ry;
                    RasterPosition(*prim, ppL, geom, rx, ry);
                    index = PixelIndex(rx, ry, P.width, P.height);
                }
                Accumulate(film, index, C);
            }
        }
        double u0, u1;
        if (type == E && prim->d.e_type == 1) {
            CameraRaster(c, smp, u0, u1);
        } else {
            u0 = smp.get(nv, CALL_DIR, 0);
            u1 = smp.get(nv, CALL_DIR, 1);
        }
        const double ucomp = smp.get(nv, CALL_DIR, 2);
        const dv3 wo = SampleDirection(*prim, u0, u1, ucomp, type, geom, wi);
        const double pdfD = EvaluateDirectionPdf(*prim, geom, type, wi, wo);
        if (type == E) {
            double rx, ry;
            if (!RasterPosition(*prim, wo, geom, rx, ry)) break;
            pixel = PixelIndex(rx, ry, P.width, P.height);
        }
        const dv3 fs = EvaluateDirection(*prim, geom, type, wi, wo, false, true);
        if (is_zero(fs)) break;
        throughput = throughput * fs / pdfD;
        Isect is;
        c.ext++;
        float tmin;
        const dv3 ro = RayOrigin(geom, wo, P.ray_offset, tmin);
        if (!Intersect(s, bvh, ro, wo, is, tmin, InfF, P.ray_offset)) {
            c.miss++;
            break;
        }
        const Prim& hp = s.prims[is.prim];
        if (!direct && (hp.d.type & L)) {
            const dv3 Le = EvaluateDirection(hp, is.geom, L, dv3(), -wo, false, false);
            const double pos = (hp.d.l_type == 1) ? 0.0 : 1.0;  // EvaluatePosition(.., false)
            Accumulate(film, pixel, throughput * Le * pos);
        }
        const double rr = smp.get(nv, CALL_NEE_RR, 3);
        if (rr > 0.5) break;
        throughput = throughput / 0.5;
        geom = is.geom;
        prim = &hp;
        type = hp.d.type & ~Emitter;
        wi = -wo;
        nv++;
        if ((type & BSDF) == 0) break;  // the reference asserts here (rt.hpp:909)
    }
}

// ProcessSample_LT / ProcessSample_LTDirect (src/nanogi.cpp:804-1131): paths start on a
// light. lt scores only where an extension ray hits an area sensor; ltdirect connects every
// vertex, the light's own included, to a sensor position. Random numbers: light pick and
// position on (vertex 1, CALL_SENSOR); sensor pick and position of the connection on
// (vertex, CALL_NEE_RR) lanes 0-2; direction on (vertex, CALL_DIR); Russian roulette on
// (vertex, CALL_NEE_RR) lane 3 -- the reference's draw order in reference mode.
void ProcessSampleLT(RenderCtx& c, Sampler& smp) {
    const ora_scene& s = *c.s;
    const ora_render_params& P = *c.p;
    const bool direct = P.renderer == 3;
    const bool bvh = P.use_bvh != 0;
    std::vector<double>& film = *c.film;

    // SampleEmitter(L, u), pdfL = 1 / #lights (rt.hpp:2321-2352)
    const int n = (int)s.lights.size();
    const double ul = smp.get(1, CALL_SENSOR, 2);
    const int li = std::min(std::max((int)(ul * n), 0), n - 1);
    const Prim& Lp = s.prims[s.lights[li]];
    const double pdfL = 1.0 / n;
    Geom geomL;
    const double a0 = smp.get(1, CALL_SENSOR, 0), a1 = smp.get(1, CALL_SENSOR, 1);
    SamplePosition(s, Lp, a0, a1, geomL);
    const double pdfPL = PositionPdf(Lp);
    dv3 throughput = dv3(1, 1, 1) / pdfPL / pdfL;  // EvaluatePosition(.., true) = 1
    const Prim* prim = &Lp;
    int type = L;
    Geom geom = geomL;
    dv3 wi(0, 0, 0);
    int nv = 1;
    c.cam++;
    while (true) {
        if (P.max_vertices != -1 && nv >= P.max_vertices) break;
        if (direct) {
            // Direct sensor sampling (src/nanogi.cpp:1001-1051)
            smp.get(nv, CALL_NEE_RR, 0);  // SampleEmitter(E, u): the single sensor, pdfE = 1
            const Prim& Ep = s.prims[s.sensor];
            Geom geomE;
            const double b0 = smp.get(nv, CALL_NEE_RR, 1), b1 = smp.get(nv, CALL_NEE_RR, 2);
            SamplePosition(s, Ep, b0, b1, geomE);
            // The reference divides by the LIGHT's position pdf here (src/nanogi.cpp:1017:
            // L->EvaluatePositionPDF(geomE, true)), not the sensor's; kept for parity.
            const double pdfPE = PositionPdf(Lp);
            const dv3 ppE = normalize(geomE.p - geom.p);
            const dv3 fsL = EvaluateDirection(*prim, geom, type, wi, ppE, true, false);
            const dv3 fsE = EvaluateDirection(Ep, geomE, E, dv3(), -ppE, false, false);
            const double Gt = GeometryTerm(geom, geomE);
            const dv3 Cpre = throughput * fsL * Gt * fsE;
            double Vis = 0.0;
            if (!is_zero(Cpre)) {
                c.sh++;
                if (P.ray_offset == 1) {
                    const dv3 a = ToFloat(OffsetPoint(geom, geomE.p - geom.p));
                    const dv3 b = OffsetPoint(geomE, geom.p - geomE.p);
                    Vis = VisibleBetween(s, bvh, a, b) ? 1.0 : 0.0;
                } else {
                    Vis = Visible(s, bvh, geom.p, geomE.p) ? 1.0 : 0.0;
                }
            }
            const dv3 C = Cpre * Vis * 1.0 / 1.0 / pdfPE;  // x LeP = 1, / pdfE = 1
            if (!is_zero(C)) {
                double rx = 0, ry = 0;
                RasterPosition(Ep, -ppE, geomE, rx, ry);
                Accumulate(film, PixelIndex(rx, ry, P.width, P.height), C);
            }
        }
        const double u0 = smp.get(nv, CALL_DIR, 0), u1 = smp.get(nv, CALL_DIR, 1);
        const double ucomp = smp.get(nv, CALL_DIR, 2);
        const dv3 wo = SampleDirection(*prim, u0, u1, ucomp, type, geom, wi);
        const double pdfD = EvaluateDirectionPdf(*prim, geom, type, wi, wo);
        const dv3 fs = EvaluateDirection(*prim, geom, type, wi, wo, true, true);
        if (is_zero(fs)) break;
        throughput = throughput * fs / pdfD;
        Isect is;
        c.ext++;
        float tmin;
        const dv3 ro = RayOrigin(geom, wo, P.ray_offset, tmin);
        if (!Intersect(s, bvh, ro, wo, is, tmin, InfF, P.ray_offset)) {
            c.miss++;
            break;
        }
        const Prim& hp = s.prims[is.prim];
        if (!direct && (hp.d.type & E)) {
            // Hit with the sensor (src/nanogi.cpp:871-896)
            double rx, ry;
            if (!RasterPosition(hp, -wo, is.geom, rx, ry)) break;
            const dv3 We = EvaluateDirection(hp, is.geom, E, dv3(), -wo, true, false);
            Accumulate(film, PixelIndex(rx, ry, P.width, P.height), throughput * We);  // x EvaluatePosition = 1
        }
        const double rr = smp.get(nv, CALL_NEE_RR, 3);
        if (rr > 0.5) break;
        throughput = throughput / 0.5;
        geom = is.geom;
        prim = &hp;
        type = hp.d.type & ~Emitter;
        wi = -wo;
        nv++;
        if ((type & BSDF) == 0) break;
    }
}

// ---- bdpt: bidirectional path tracing with power-heuristic MIS (include/nanogi/bdpt.hpp) ----------

struct PVert {  // PathVertex (bdpt.hpp:40-45)
    int type = 0;
    Geom geom;
    const Prim* prim = nullptr;
};

dv3 Dir(const PVert& from, const PVert& to) { return normalize(to.geom.p - from.geom.p); }

// Primitive::EvaluatePosition (rt.hpp:594-641)
double EvaluatePosition(const Prim& p, bool force) {
    if (p.d.type & L) return p.d.l_type == 1 ? (force ? 1.0 : 0.0) : 1.0;
    return p.d.e_type == 1 ? (force ? 1.0 : 0.0) : 1.0;
}

// Scene::EvaluateEmitterPDF (rt.hpp:2338-2352)
double EmitterPdf(const ora_scene& s, const Prim& p) {
    if (p.d.type & L) return 1.0 / (double)s.lights.size();
    if (p.d.type & E) return 1.0;
    return 0.0;
}

// Subpaths keep at most 32 vertices (the reference's are unbounded when max_vertices = -1; with
// Russian roulette at 1/2 per bounce a longer one has probability 2^-31).
constexpr int kBdptMaxSubpath = 32;

// Path::SampleSubpath (bdpt.hpp:58-131). Random numbers of step k of a subpath are keyed by
// vertex vbase + k + 1 (light subpath vbase 0, eye subpath 64): emitter pick and position on
// CALL_SENSOR, direction on CALL_DIR, Russian roulette on CALL_NEE_RR lane 3.
void SampleSubpath(RenderCtx& c, Sampler& smp, bool le, uint32_t vbase, std::vector<PVert>& vs) {
    const ora_scene& s = *c.s;
    const ora_render_params& P = *c.p;
    vs.clear();
    for (int step = 0; (P.max_vertices == -1 || step < P.max_vertices) && step < kBdptMaxSubpath; step++) {
        const uint32_t key = vbase + (uint32_t)step + 1;
        if (step == 0) {
            PVert v;
            v.type = le ? L : E;
            const double ue = smp.get(key, CALL_SENSOR, 2);
            if (le) {
                const int n = (int)s.lights.size();
                v.prim = &s.prims[s.lights[std::min(std::max((int)(ue * n), 0), n - 1)]];
            } else {
                v.prim = &s.prims[s.sensor];
            }
            const double a0 = smp.get(key, CALL_SENSOR, 0), a1 = smp.get(key, CALL_SENSOR, 1);
            SamplePosition(s, *v.prim, a0, a1, v.geom);
            vs.push_back(v);
            continue;
        }
        const PVert pv = vs.back();
        const dv3 wi = vs.size() > 1 ? Dir(pv, vs[vs.size() - 2]) : dv3(0, 0, 0);
        const double u0 = smp.get(key, CALL_DIR, 0), u1 = smp.get(key, CALL_DIR, 1);
        const double uc = smp.get(key, CALL_DIR, 2);
        const dv3 wo = SampleDirection(*pv.prim, u0, u1, uc, pv.type, pv.geom, wi);
        const dv3 f = EvaluateDirection(*pv.prim, pv.geom, pv.type, wi, wo, le, true);
        if (is_zero(f)) break;
        Isect is;
        c.ext++;
        float tmin;
        const dv3 ro = RayOrigin(pv.geom, wo, P.ray_offset, tmin);
        if (!Intersect(s, P.use_bvh != 0, ro, wo, is, tmin, InfF, P.ray_offset)) {
            c.miss++;
            break;
        }
        PVert v;
        v.geom = is.geom;
        v.prim = &s.prims[is.prim];
        v.type = v.prim->d.type & ~Emitter;
        const double rr = smp.get(key, CALL_NEE_RR, 3);
        vs.push_back(v);
        if (rr > 0.5) break;
    }
}

// Path::Connect (bdpt.hpp:133-180)
bool Connect(RenderCtx& c, int s, int t, const std::vector<PVert>& sl, const std::vector<PVert>& se,
             std::vector<PVert>& x) {
    x.clear();
    if (s == 0) {
        if ((se[t - 1].prim->d.type & L) == 0) return false;
        for (int i = t - 1; i >= 0; i--) x.push_back(se[i]);
        x.front().type = L;
    } else if (t == 0) {
        if ((sl[s - 1].prim->d.type & E) == 0) return false;
        for (int i = 0; i < s; i++) x.push_back(sl[i]);
        x.back().type = E;
    } else {
        c.sh++;
        const Geom& a = sl[s - 1].geom;
        const Geom& b = se[t - 1].geom;
        bool vis;
        if (c.p->ray_offset == 1) vis = VisibleBetween(*c.s, c.p->use_bvh != 0, ToFloat(OffsetPoint(a, b.p - a.p)), OffsetPoint(b, a.p - b.p));
        else vis = Visible(*c.s, c.p->use_bvh != 0, a.p, b.p);
        if (!vis) return false;
        for (int i = 0; i < s; i++) x.push_back(sl[i]);
        for (int i = t - 1; i >= 0; i--) x.push_back(se[i]);
    }
    return true;
}

// Path::EvaluateCst (bdpt.hpp:213-244)
dv3 EvaluateCst(const std::vector<PVert>& x, int s) {
    const int n = (int)x.size(), t = n - s;
    if (s == 0 && t > 0) {
        const PVert& v = x[0];
        return EvaluateDirection(*v.prim, v.geom, v.type, dv3(0, 0, 0), Dir(v, x[1]), false, false) *
               EvaluatePosition(*v.prim, false);
    }
    if (s > 0 && t == 0) {
        const PVert& v = x[n - 1];
        return EvaluateDirection(*v.prim, v.geom, v.type, dv3(0, 0, 0), Dir(v, x[n - 2]), true, false) *
               EvaluatePosition(*v.prim, false);
    }
    const PVert& vL = x[s - 1];
    const PVert& vE = x[s];
    const dv3 wiL = s - 2 >= 0 ? Dir(vL, x[s - 2]) : dv3(0, 0, 0);
    const dv3 wiE = s + 1 < n ? Dir(vE, x[s + 1]) : dv3(0, 0, 0);
    const dv3 fsL = EvaluateDirection(*vL.prim, vL.geom, vL.type, wiL, Dir(vL, vE), true, false);
    const dv3 fsE = EvaluateDirection(*vE.prim, vE.geom, vE.type, wiE, Dir(vE, vL), false, false);
    return fsL * GeometryTerm(vL.geom, vE.geom) * fsE;
}

// f / p with f = 0 -> 0 (LocalContrb, bdpt.hpp:252-257)
dv3 LocalContrb(dv3 f, double p) { return is_zero(f) ? dv3(0, 0, 0) : f / p; }

// Path::EvaluateUnweightContribution (bdpt.hpp:246-320)
dv3 EvaluateUnweighted(const ora_scene& sc, const std::vector<PVert>& x, int s) {
    const int n = (int)x.size(), t = n - s;
    dv3 aL(1, 1, 1);
    if (s > 0) {
        const PVert& v0 = x[0];
        aL = LocalContrb(dv3(1, 1, 1) * EvaluatePosition(*v0.prim, true), PositionPdf(*v0.prim) * EmitterPdf(sc, *v0.prim));
        for (int i = 0; i < s - 1; i++) {
            const PVert& v = x[i];
            const dv3 wi = i >= 1 ? Dir(v, x[i - 1]) : dv3(0, 0, 0);
            const dv3 wo = Dir(v, x[i + 1]);
            aL = aL * LocalContrb(EvaluateDirection(*v.prim, v.geom, v.type, wi, wo, true, true),
                                  EvaluateDirectionPdf(*v.prim, v.geom, v.type, wi, wo));
        }
    }
    if (is_zero(aL)) return dv3(0, 0, 0);
    dv3 aE(1, 1, 1);
    if (t > 0) {
        const PVert& vn = x[n - 1];
        aE = LocalContrb(dv3(1, 1, 1) * EvaluatePosition(*vn.prim, true), PositionPdf(*vn.prim) * EmitterPdf(sc, *vn.prim));
        for (int i = n - 1; i > s; i--) {
            const PVert& v = x[i];
            const dv3 wi = i < n - 1 ? Dir(v, x[i + 1]) : dv3(0, 0, 0);
            const dv3 wo = Dir(v, x[i - 1]);
            aE = aE * LocalContrb(EvaluateDirection(*v.prim, v.geom, v.type, wi, wo, false, true),
                                  EvaluateDirectionPdf(*v.prim, v.geom, v.type, wi, wo));
        }
    }
    if (is_zero(aE)) return dv3(0, 0, 0);
    const dv3 cst = EvaluateCst(x, s);
    if (is_zero(cst)) return dv3(0, 0, 0);
    return aL * cst * aE;
}

// Path::EvaluatePDF (bdpt.hpp:480-529): area-measure pdf of sampling x with strategy s
double EvaluatePathPdf(const ora_scene& sc, const std::vector<PVert>& x, int s) {
    if (is_zero(EvaluateCst(x, s))) return 0.0;
    const int n = (int)x.size(), t = n - s;
    double pdf = 1.0;
    if (s > 0) {
        pdf *= PositionPdf(*x[0].prim) * EmitterPdf(sc, *x[0].prim);
        for (int i = 0; i < s - 1; i++) {
            const PVert& v = x[i];
            const dv3 wi = i - 1 >= 0 ? Dir(v, x[i - 1]) : dv3(0, 0, 0);
            pdf *= EvaluateDirectionPdf(*v.prim, v.geom, v.type, wi, Dir(v, x[i + 1]));
            pdf *= GeometryTerm(v.geom, x[i + 1].geom);
        }
    }
    if (t > 0) {
        pdf *= PositionPdf(*x[n - 1].prim) * EmitterPdf(sc, *x[n - 1].prim);
        for (int i = n - 1; i >= s + 1; i--) {
            const PVert& v = x[i];
            const dv3 wi = i + 1 < n ? Dir(v, x[i + 1]) : dv3(0, 0, 0);
            pdf *= EvaluateDirectionPdf(*v.prim, v.geom, v.type, wi, Dir(v, x[i - 1]));
            pdf *= GeometryTerm(v.geom, x[i - 1].geom);
        }
    }
    return pdf;
}

// Path::EvaluatePowerHeuristicsMISWeightOpt (bdpt.hpp:366-384)
double MisWeight(const ora_scene& sc, const std::vector<PVert>& x, int s) {
    const int n = (int)x.size();
    const double ps = EvaluatePathPdf(sc, x, s);
    double inv = 0.0;
    for (int i = 0; i <= n; i++) {
        const double pi = EvaluatePathPdf(sc, x, i);
        if (pi > 0) {
            const double r = pi / ps;
            inv += r * r;
        }
    }
    return 1.0 / inv;
}

// Path::SelectionProb (bdpt.hpp:188-202)
double SelectionProb(int n, int s) {
    const int t = n - s;
    double p = 1.0;
    for (int i = 1; i < s - 1; i++) p *= 0.5;
    for (int i = t - 2; i >= 1; i--) p *= 0.5;
    return p;
}

// ProcessSample_BDPT (src/nanogi.cpp:1133-1194)
void ProcessSampleBDPT(RenderCtx& c, Sampler& smp, std::vector<PVert>& sl, std::vector<PVert>& se,
                       std::vector<PVert>& x) {
    const ora_scene& sc = *c.s;
    const ora_render_params& P = *c.p;
    SampleSubpath(c, smp, true, 0, sl);
    SampleSubpath(c, smp, false, 64, se);
    c.cam++;
    const int nL = (int)sl.size(), nE = (int)se.size();
    for (int n = 2; n <= nE + nL; n++) {
        if (P.max_vertices != -1 && n > P.max_vertices) continue;
        for (int s = std::max(0, n - nE); s <= std::min(nL, n); s++) {
            const int t = n - s;
            if (!Connect(c, s, t, sl, se, x)) continue;
            const dv3 Cs = EvaluateUnweighted(sc, x, s);
            if (is_zero(Cs)) continue;
            const dv3 C = Cs * MisWeight(sc, x, s) / SelectionProb(n, s);
            if (is_zero(C)) continue;
            // Path::RasterPosition (bdpt.hpp:204-211)
            const PVert& v = x[x.size() - 1];
            double rx = 0, ry = 0;
            RasterPosition(*v.prim, Dir(v, x[x.size() - 2]), v.geom, rx, ry);
            Accumulate(*c.film, PixelIndex(rx, ry, P.width, P.height), C);
        }
    }
}

ora_scene* Build(const ora_prim_desc* prims, int n_prims, const float* tri_pos, const float* tri_nrm,
                 const float* tri_uv, int64_t n_tris, double aspect) {
    auto s = std::make_unique<ora_scene>();
    s->tris.resize(n_tris);
    s->pos.resize(9 * n_tris);
    s->nrm.resize(9 * n_tris);
    s->uv.assign(6 * n_tris, 0.0);
    s->tri_prim.assign(n_tris, -1);
    double bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < n_tris; i++) {
        for (int v = 0; v < 3; v++)
            for (int k = 0; k < 3; k++) {
                const float x = tri_pos[9 * i + 3 * v + k];
                s->tris[i].p[v][k] = x;
                s->pos[9 * i + 3 * v + k] = x;
                s->nrm[9 * i + 3 * v + k] = tri_nrm[9 * i + 3 * v + k];
                bmin[k] = std::min(bmin[k], (double)x);
                bmax[k] = std::max(bmax[k], (double)x);
            }
        if (tri_uv)
            for (int k = 0; k < 6; k++) s->uv[6 * i + k] = tri_uv[6 * i + k];
    }
    s->bmin = dv3(bmin[0], bmin[1], bmin[2]);
    s->bmax = dv3(bmax[0], bmax[1], bmax[2]);
    for (int i = 0; i < n_prims; i++) {
        Prim p;
        p.d = prims[i];
        if (p.d.has_mesh)
            for (int64_t t = p.d.tri_first; t < p.d.tri_first + p.d.tri_count; t++) s->tri_prim[t] = i;
        p.Le = V(p.d.Le);
        p.lpos = V(p.d.l_position);
        p.ldir = V(p.d.l_direction);
        p.DR = V(p.d.D_R);
        p.GR = V(p.d.G_R);
        CopyTextures(p);
        p.Geta = V(p.d.G_eta);
        p.Gk = V(p.d.G_k);
        p.SR = V(p.d.S_R);
        p.We = V(p.d.We);
        const bool area_mesh = ((p.d.type & L) && p.d.l_type == 0) || ((p.d.type & E) && p.d.e_type == 0);
        if (area_mesh) {
            // CreateTriangleAreaDist (rt.hpp:1747-1765)
            double sum = 0;
            for (int64_t t = p.d.tri_first; t < p.d.tri_first + p.d.tri_count; t++) {
                const double* P = &s->pos[9 * t];
                const dv3 p1(P[0], P[1], P[2]), p2(P[3], P[4], P[5]), p3(P[6], P[7], P[8]);
                const double a = length(cross(p2 - p1, p3 - p1)) * 0.5;
                p.dist.Add(a);
                sum += a;
            }
            p.dist.Normalize();
            p.inv_area = 1.0 / sum;
        }
        if ((p.d.type & E) && p.d.e_type == 1) {
            p.eye = V(p.d.eye);
            const dv3 center = V(p.d.center), up = V(p.d.up);
            p.fov = p.d.fov_deg * Pi / 180.0;
            p.Vz = normalize(p.eye - center);
            p.Vx = normalize(cross(up, p.Vz));
            p.Vy = cross(p.Vz, p.Vx);
            p.aspect = aspect;
        }
        if (p.d.type & E) s->sensor = i;
        if (p.d.type & L) s->lights.push_back(i);
        s->prims.push_back(p);
    }
    for (auto& p : s->prims)
        if ((p.d.type & L) && p.d.l_type == 2) {
            p.lcenter = (s->bmax + s->bmin) * 0.5;
            p.lradius = length(p.lcenter - s->bmax) * 1.01;
            p.inv_area = 1.0 / (2.0 * Pi * p.lradius * p.lradius);
        }
    BuildBvh(s->tris, s->bvh);
    return s.release();
}

}  // namespace

// Runs fn(i) for i in [0, n) on every hardware thread, in contiguous chunks. Each query is
// independent, so the results do not depend on the thread count.
template <typename F>
void ParallelQueries(int64_t n, F fn) {
    const int threads = std::max(1, (int)std::thread::hardware_concurrency());
    const int64_t chunk = 1024;
    std::atomic<int64_t> next{0};
    auto work = [&]() {
        for (int64_t b = next.fetch_add(chunk); b < n; b = next.fetch_add(chunk))
            for (int64_t i = b; i < std::min(n, b + chunk); i++) fn(i);
    };
    if (n <= chunk || threads == 1) {
        work();
        return;
    }
    std::vector<std::thread> pool;
    for (int k = 0; k < threads; k++) pool.emplace_back(work);
    for (auto& th : pool) th.join();
}

extern "C" {

const char* ora_last_error(void) { return g_err.c_str(); }

ora_scene* ora_scene_create(const ora_prim_desc* prims, int32_t n_prims, const float* tri_pos, const float* tri_nrm,
                            const float* tri_uv, int64_t n_tris, double aspect) {
    try {
        return Build(prims, n_prims, tri_pos, tri_nrm, tri_uv, n_tris, aspect);
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

void ora_scene_free(ora_scene* s) { delete s; }

int ora_intersect(ora_scene* s, const float* rays, int64_t n, int32_t use_bvh, int32_t* prim, float* t, float* uv) {
    ParallelQueries(n, [&](int64_t i) {
        const float* r = rays + 8 * i;
        const float o[3] = {r[0], r[1], r[2]}, d[3] = {r[4], r[5], r[6]};
        const RayF ray = MakeRay(o, d);
        const Hit h = use_bvh ? IntersectBvh(*s, ray, r[3], r[7], false) : IntersectBrute(*s, ray, r[3], r[7], false);
        prim[i] = h.tri;
        t[i] = h.tri >= 0 ? h.t : INFINITY;
        uv[2 * i] = h.tri >= 0 ? h.u : 0.0f;
        uv[2 * i + 1] = h.tri >= 0 ? h.v : 0.0f;
    });
    return 0;
}

int ora_visible(ora_scene* s, const double* pts, int64_t n, int32_t use_bvh, uint8_t* vis) {
    ParallelQueries(n, [&](int64_t i) {
        const double* q = pts + 6 * i;
        vis[i] = Visible(*s, use_bvh != 0, dv3(q[0], q[1], q[2]), dv3(q[3], q[4], q[5])) ? 1 : 0;
    });
    return 0;
}

int ora_render(ora_scene* s, const ora_render_params* p, double* film_out, ora_render_stats* stats) {
    if (!s || !p || !film_out) { g_err = "NULL argument"; return 1; }
    if (s->sensor < 0) { g_err = "no sensor"; return 1; }
    if (p->renderer < 0 || p->renderer > 4) { g_err = "unknown renderer"; return 1; }

    if (p->renderer >= 1 && s->lights.empty()) { g_err = "this renderer needs a light"; return 1; }
    const size_t elems = 3 * (size_t)p->width * p->height;
    int threads = p->num_threads > 0 ? p->num_threads : (int)std::thread::hardware_concurrency();
    if (threads < 1) threads = 1;
    const int64_t grain = p->grain_size > 0 ? p->grain_size : 10000;
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::vector<double>> films(threads, std::vector<double>(elems, 0.0));
    std::vector<RenderCtx> ctx(threads);
    std::atomic<int64_t> next(0);
    // Thread seeds drawn from an init generator (src/nanogi.cpp:186-191, 297)
    std::mt19937 init_rng((uint32_t)p->seed);
    std::vector<uint32_t> seeds(threads);
    for (int i = 0; i < threads; i++) seeds[i] = init_rng();
    const long long wh = (long long)p->width * p->height;
    const long long strat_end = ((p->sample_offset + p->num_samples) / wh) * wh;
    auto worker = [&](int tid) {
        RenderCtx& c = ctx[tid];
        c.s = s;
        c.p = p;
        c.film = &films[tid];
        c.strat_end = strat_end;
        std::vector<PVert> sl, se, x;  // bdpt subpaths and full path, reused per sample
        std::mt19937 eng(seeds[tid]);
        std::uniform_real_distribution<double> dist;
        Sampler smp;
        smp.replay = p->rng_mode == 1;
        smp.eng = &eng;
        smp.dist = &dist;
        smp.key[0] = (uint32_t)p->seed;
        smp.key[1] = (uint32_t)(p->seed >> 32);
        while (true) {
            const int64_t b = next.fetch_add(grain);
            if (b >= p->num_samples) break;
            const int64_t e = std::min(b + grain, p->num_samples);
            for (int64_t k = b; k < e; k++) {
                smp.sample = (uint64_t)(p->sample_offset + k);
                smp.cache_vertex = 0xFFFFFFFFu;
                if (p->renderer == 4) ProcessSampleBDPT(c, smp, sl, se, x);
                else if (p->renderer >= 2) ProcessSampleLT(c, smp);
                else ProcessSample(c, smp);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 1; i < threads; i++) pool.emplace_back(worker, i);
    worker(0);
    for (auto& th : pool) th.join();
    std::fill(film_out, film_out + elems, 0.0);
    for (int i = 0; i < threads; i++)
        for (size_t k = 0; k < elems; k++) film_out[k] += films[i][k];
    if (p->num_samples > 0) {
        const double scale = (double)wh / (double)p->num_samples;
        for (size_t k = 0; k < elems; k++) film_out[k] *= scale;
    }
    const auto t1 = std::chrono::steady_clock::now();
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        for (auto& c : ctx) {
            stats->camera_rays += c.cam;
            stats->extension_rays += c.ext;
            stats->shadow_rays += c.sh;
            stats->extension_misses += c.miss;
        }
        stats->seconds = std::chrono::duration<double>(t1 - t0).count();
        stats->threads = threads;
    }
    return 0;
}

void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { Philox(ctr, key, out); }

uint32_t ora_mt19937_nth(uint32_t seed, int64_t n) {
    std::mt19937 e(seed);
    uint32_t v = 0;
    for (int64_t i = 0; i < n; i++) v = e();
    return v;
}

double ora_mt19937_uniform(uint32_t seed, int64_t n) {
    std::mt19937 e(seed);
    std::uniform_real_distribution<double> d;
    double v = 0;
    for (int64_t i = 0; i < n; i++) v = d(e);
    return v;
}

static Prim HookPrim(const ora_prim_desc* d) {
    Prim p;
    p.d = *d;
    p.DR = V(d->D_R);
    p.GR = V(d->G_R);
    p.Geta = V(d->G_eta);
    p.Gk = V(d->G_k);
    p.SR = V(d->S_R);
    CopyTextures(p);
    return p;
}
static Geom HookGeom() {
    Geom g;
    g.sn = dv3(0, 0, 1);
    g.gn = g.sn;
    g.ComputeTangentSpace();
    return g;
}

int ora_bsdf_sample(const ora_prim_desc* d, const double wi_[3], const double u[3], double wo_[3], double* pdf,
                    double fs_[3]) {
    const Prim p = HookPrim(d);
    const Geom g = HookGeom();
    const int type = d->type & BSDF;
    const dv3 wi = V(wi_);
    const dv3 wo = SampleDirection(p, u[0], u[1], u[2], type, g, wi);
    *pdf = EvaluateDirectionPdf(p, g, type, wi, wo);
    const dv3 fs = EvaluateDirection(p, g, type, wi, wo, false, true);
    wo_[0] = wo.x; wo_[1] = wo.y; wo_[2] = wo.z;
    fs_[0] = fs.x; fs_[1] = fs.y; fs_[2] = fs.z;
    return is_zero(wo) ? 0 : 1;
}

int ora_bsdf_eval(const ora_prim_desc* d, const double wi_[3], const double wo_[3], int force, double fs_[3],
                  double* pdf) {
    const Prim p = HookPrim(d);
    const Geom g = HookGeom();
    const int type = d->type & BSDF;
    const dv3 fs = EvaluateDirection(p, g, type, V(wi_), V(wo_), false, force != 0);
    fs_[0] = fs.x; fs_[1] = fs.y; fs_[2] = fs.z;
    *pdf = EvaluateDirectionPdf(p, g, type, V(wi_), V(wo_));
    return 0;
}

}  // extern "C"
