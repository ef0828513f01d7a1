// Surface geometry, BSDFs, emitters and sensors on the device, templated on the shading
// precision R (float: tuned path, double: plain path).
//
// Each function restates one method of the reference's Primitive (include/nanogi/rt.hpp)
// for the EL transport direction the path tracers use; the citation is on each function.
#pragma once

#include "ngi_device.cuh"

namespace ngi {

template <typename R>
struct Geom {
    V3<R> p, sn, gn, du, dv;  // du = dpdu, dv = dpdv: tangent frame (du, dv, sn)
    R uvx, uvy;
    bool degenerated;
    float ext;  // largest |coordinate| of the triangle under p (scale of its rounding error); 0 off surfaces
};

// Largest |coordinate| over three points.
template <typename R>
NGI_D float max_abs3(V3<R> a, V3<R> b, V3<R> c) {
    const R m = fmax_(fmax_(fmax_(fabs_(a.x), fabs_(a.y)), fmax_(fabs_(a.z), fabs_(b.x))),
                      fmax_(fmax_(fabs_(b.y), fabs_(b.z)), fmax_(fmax_(fabs_(c.x), fabs_(c.y)), fabs_(c.z))));
    return (float)m;
}

template <typename R> NGI_D R kPi_() { return R(3.14159265358979323846); }
template <typename R> NGI_D R kInvPi_() { return R(1.0 / 3.14159265358979323846); }

// OrthonormalBasis (rt.hpp:55-59) + ComputeTangentSpace (rt.hpp:295-300)
template <typename R>
NGI_D void tangent_space(Geom<R>& g) {
    const V3<R> a = g.sn;
    g.dv = fabs_(a.x) > fabs_(a.y) ? normalize(v3<R>(a.z, R(0), -a.x)) : normalize(v3<R>(R(0), a.z, -a.y));
    g.du = normalize(cross(g.dv, a));
}
template <typename R> NGI_D V3<R> to_local(const Geom<R>& g, V3<R> w) { return {dot(g.du, w), dot(g.dv, w), dot(g.sn, w)}; }
template <typename R> NGI_D V3<R> to_world(const Geom<R>& g, V3<R> l) { return g.du * l.x + g.dv * l.y + g.sn * l.z; }

// ---- sampling utilities (rt.hpp:87-133) -------------------------------------------------
template <typename R>
NGI_D void concentric_disk(R u0, R u1, R& sx, R& sy) {
    const R vx = R(2) * u0 - R(1), vy = R(2) * u1 - R(1);
    if (vx == R(0) && vy == R(0)) { sx = R(0); sy = R(0); return; }
    R r, q;  // theta = pi * q
    if (vx > -vy) {
        if (vx > vy) { r = vx; q = R(0.25) * (vy / vx); }
        else { r = vy; q = R(0.25) * (R(2) - vx / vy); }
    } else {
        if (vx < vy) { r = -vx; q = R(0.25) * (R(4) + vy / vx); }
        else { r = -vy; q = R(0.25) * (R(6) - vx / vy); }
    }
    R s, c;
    sincospi_(q, &s, &c);
    sx = r * c;
    sy = r * s;
}
template <typename R>
NGI_D V3<R> cosine_hemisphere(R u0, R u1) {
    R sx, sy;
    concentric_disk(u0, u1, sx, sy);
    return v3<R>(sx, sy, sqrt_(fmax_(R(0), R(1) - sx * sx - sy * sy)));
}
template <typename R>
NGI_D void uniform_triangle(R u0, R u1, R& b0, R& b1) {
    const R s = sqrt_(fmax_(R(0), u0));
    b0 = R(1) - s;
    b1 = u1 * s;
}

// PixelIndex (rt.hpp:135-140)
template <typename R>
NGI_D int pixel_index(R rx, R ry, int w, int h) {
    int px = (int)(rx * (R)w), py = (int)(ry * (R)h);
    px = px < 0 ? 0 : (px > w - 1 ? w - 1 : px);
    py = py < 0 ? 0 : (py > h - 1 ? h - 1 : py);
    return py * w + px;
}

// ---- BSDF helpers (rt.hpp:1407-1466) -------------------------------------------------------
template <typename R>
NGI_D R beckmann_d(R rough, V3<R> H) {
    if (H.z <= R(0)) return R(0);
    const R t = R(1) - H.z * H.z;
    const R tan_ = t <= R(0) ? R(0) : sqrt_(t) / H.z;  // LocalTan rt.hpp:71-75
    const R ex = tan_ / rough;
    const R c2 = H.z * H.z;
    return exp_(-(ex * ex)) / (kPi_<R>() * rough * rough * (c2 * c2));
}
// EvalauteShadowMaskingFunc: wi_dot_H is computed from wo in the reference (rt.hpp:1429).
template <typename R>
NGI_D R shadow_masking(V3<R> wi, V3<R> wo, V3<R> H) {
    const R nH = H.z, nwo = wo.z, nwi = wi.z;
    const R woH = fabs_(dot(wo, H));
    const R wiH = fabs_(dot(wo, H));
    return fmin_(R(1), fmin_(R(2) * nH * nwo / woH, R(2) * nH * nwi / wiH));
}
template <typename R>
NGI_D V3<R> fr_conductor(const DevMaterial<R>& m, R c) {
    V3<R> out;
    const R e[3] = {m.eta.x, m.eta.y, m.eta.z}, k[3] = {m.k.x, m.k.y, m.k.z};
    R o[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const R ek = e[i] * e[i] + k[i] * k[i];
        const R tmp = ek * (c * c);
        const R two_ec = e[i] * (R(2) * c);
        const R par = (tmp - two_ec + R(1)) / (tmp + two_ec + R(1));
        const R perp = (ek - two_ec + c * c) / (ek + two_ec + c * c);
        o[i] = (par + perp) * R(0.5);
    }
    out.x = o[0]; out.y = o[1]; out.z = o[2];
    return out;
}
template <typename R>
NGI_D R fresnel_dielectric(R cos_i, R eta_i, R eta_t) {
    const R eta = eta_i / eta_t;
    const R c2t = R(1) - eta * eta * (R(1) - cos_i * cos_i);
    if (c2t <= R(0)) return R(1);
    const R aci = fabs_(cos_i);
    const R act = sqrt_(c2t);
    const R rs = (eta_i * aci - eta_t * act) / (eta_i * aci + eta_t * act);
    const R rt = (eta_i * act - eta_t * aci) / (eta_i * act + eta_t * aci);
    return (rs * rs + rt * rt) * R(0.5);
}

// Shading-normal correction factor (rt.hpp:994-1005): 0 where a direction lies on different
// sides of the geometric and shading normals; otherwise 1 for EL (paths from the sensor) and
// (wi.Ns wo.Ng) / (wo.Ns wi.Ng) for LE (paths from a light).
template <typename R>
NGI_D R shading_correction(const Geom<R>& g, V3<R> wi, V3<R> wo, R lwi_z, R lwo_z, bool le) {
    const R wiNg = dot(wi, g.gn), woNg = dot(wo, g.gn);
    if (wiNg * lwi_z <= R(0) || woNg * lwo_z <= R(0)) return R(0);
    return le ? (lwi_z * woNg) / (lwo_z * wiNg) : R(1);
}

// Albedo R of a D / G material at g: the texel of its TexR under g's uv -- nearest, with
// fract wrap (Texture::Evaluate, rt.hpp:260-266) -- or the constant R.
template <typename R>
NGI_D V3<R> material_albedo(const SceneView<R>& sv, const DevMaterial<R>& m, const Geom<R>& g) {
    if (m.tex < 0) return m.R_;
    const int4 t = sv.tex_info[m.tex];
    const R fu = g.uvx - floor_(g.uvx), fv = g.uvy - floor_(g.uvy);
    int x = (int)(fu * (R)t.y), y = (int)(fv * (R)t.z);
    x = x < 0 ? 0 : (x > t.y - 1 ? t.y - 1 : x);
    y = y < 0 ? 0 : (y > t.z - 1 ? t.z - 1 : y);
    const float4 c = __ldg(sv.texels + t.x + (size_t)y * t.y + x);
    return v3<R>((R)c.x, (R)c.y, (R)c.z);
}

// ---- BSDF evaluation (rt.hpp:988-1140); `le` selects the LE transport direction ----------
// `albedo` is the R of D / G materials at this point (material_albedo); S uses m.R_.
template <typename R>
NGI_D V3<R> bsdf_eval(const DevMaterial<R>& m, V3<R> albedo, const Geom<R>& g, V3<R> wi, V3<R> wo,
                      bool force_degenerated, bool le = false) {
    const V3<R> lwi = to_local(g, wi), lwo = to_local(g, wo);
    const R corr = shading_correction(g, wi, wo, lwi.z, lwo.z, le);
    const V3<R> zero = v3<R>(0, 0, 0);
    if (m.bsdf == BSDF_D) {
        if (lwi.z <= R(0) || lwo.z <= R(0)) return zero;
        return albedo * (kInvPi_<R>() * corr);
    }
    if (m.bsdf == BSDF_G) {
        if (lwi.z <= R(0) || lwo.z <= R(0)) return zero;
        const V3<R> H = normalize(lwi + lwo);
        const R D = beckmann_d(m.roughness, H);
        const R G = shadow_masking(lwi, lwo, H);
        const V3<R> F = fr_conductor(m, dot(lwi, H));
        return albedo * (D * G) * F / (R(4) * lwi.z) / lwo.z * corr;
    }
    if (m.bsdf == BSDF_S) {
        if (!force_degenerated) return zero;
        if (m.s_type == ST_REFLECTION) {
            if (lwi.z <= R(0) || lwo.z <= R(0)) return zero;
            return m.R_ * corr;
        }
        R ei = m.eta1, et = m.eta2;
        if (lwi.z < R(0)) { const R t = ei; ei = et; et = t; }
        const R eta = le ? R(1) : ei / et;  // radiance scaling on refraction, EL only
        if (m.s_type == ST_REFRACTION) return m.R_ * (corr * eta * eta);
        const R Fr = fresnel_dielectric(lwi.z, ei, et);
        if (lwi.z * lwo.z >= R(0)) return m.R_ * (Fr * corr);
        return m.R_ * ((R(1) - Fr) * corr * eta * eta);
    }
    return zero;
}

// EvaluateDirectionPDF with forceDegenerated = true (rt.hpp:1219-1330)
template <typename R>
NGI_D R bsdf_pdf(const DevMaterial<R>& m, const Geom<R>& g, V3<R> wi, V3<R> wo) {
    const V3<R> lwi = to_local(g, wi), lwo = to_local(g, wo);
    if (m.bsdf == BSDF_D) {
        if (lwi.z <= R(0) || lwo.z <= R(0)) return R(0);
        return kInvPi_<R>();
    }
    if (m.bsdf == BSDF_G) {
        if (lwi.z <= R(0) || lwo.z <= R(0)) return R(0);
        const V3<R> H = normalize(lwi + lwo);
        return beckmann_d(m.roughness, H) * H.z / (R(4) * dot(lwo, H)) / lwo.z;
    }
    if (m.bsdf == BSDF_S) {
        if (m.s_type == ST_REFLECTION) return (lwi.z <= R(0) || lwo.z <= R(0)) ? R(0) : R(1);
        if (m.s_type == ST_REFRACTION) return R(1);
        R ei = m.eta1, et = m.eta2;
        if (lwi.z < R(0)) { const R t = ei; ei = et; et = t; }
        const R Fr = fresnel_dielectric(lwi.z, ei, et);
        return lwi.z * lwo.z >= R(0) ? Fr : R(1) - Fr;
    }
    return R(0);
}

// SampleDirection for BSDF vertices (rt.hpp:747-903). Returns false where the reference
// leaves wo at zero (which then yields pdf 0 and fs 0, ending the path).
template <typename R>
NGI_D bool bsdf_sample(const DevMaterial<R>& m, const Geom<R>& g, V3<R> wi, R u0, R u1, R ucomp, V3<R>& wo) {
    const V3<R> lwi = to_local(g, wi);
    if (m.bsdf == BSDF_D) {
        if (lwi.z <= R(0)) return false;
        wo = to_world(g, cosine_hemisphere(u0, u1));
        return true;
    }
    if (m.bsdf == BSDF_G) {
        if (lwi.z <= R(0)) return false;
        const R tan2 = -m.roughness * m.roughness * log_(R(1) - u0);
        const R ch = rsqrt_(R(1) + tan2);
        const R sh = sqrt_(fmax_(R(0), R(1) - ch * ch));
        R sp, cp;
        sincos2pi_(u1, &sp, &cp);
        const V3<R> H = v3<R>(sh * cp, sh * sp, ch);
        const V3<R> lwo = -lwi - H * (R(2) * dot(-lwi, H));
        if (lwo.z <= R(0)) return false;
        wo = to_world(g, lwo);
        return true;
    }
    if (m.bsdf == BSDF_S) {
        if (m.s_type == ST_REFLECTION) {
            if (lwi.z <= R(0)) return false;
            wo = to_world(g, v3<R>(-lwi.x, -lwi.y, lwi.z));
            return true;
        }
        R ei = m.eta1, et = m.eta2;
        if (lwi.z < R(0)) { const R t = ei; ei = et; et = t; }
        const R eta = ei / et;
        bool reflect;
        if (m.s_type == ST_REFRACTION) {
            reflect = R(1) - eta * eta * (R(1) - lwi.z * lwi.z) <= R(0);  // total internal reflection
        } else {
            reflect = ucomp <= fresnel_dielectric(lwi.z, ei, et);
        }
        if (reflect) {
            wo = to_world(g, v3<R>(-lwi.x, -lwi.y, lwi.z));
        } else {
            const R c2t = R(1) - eta * eta * (R(1) - lwi.z * lwi.z);
            const R ct = sqrt_(fmax_(c2t, R(0))) * (lwi.z > R(0) ? R(-1) : R(1));
            wo = to_world(g, v3<R>(-eta * lwi.x, -eta * lwi.y, ct));
        }
        return true;
    }
    return false;
}

// SampleDirection + EvaluateDirection(forceDegenerated) / EvaluateDirectionPDF in one pass:
// the sampled direction and the weight fs/pdf the path throughput is multiplied by
// (src/nanogi.cpp:494-546 / 718-756). False where the reference's fs is zero (path ends).
// The ratio is formed in closed form where the lobe cancels: R*corr for D, and
// R*G*F*(wo.H)/(cos_i cos_H)*corr for G (no Beckmann exp); S keeps the explicit ratio.
template <typename R>
NGI_D bool bsdf_sample_weight(const DevMaterial<R>& m, V3<R> albedo, const Geom<R>& g, V3<R> wi, R u0, R u1, R ucomp,
                              V3<R>& wo, V3<R>& weight, bool le = false) {
    if (!bsdf_sample(m, g, wi, u0, u1, ucomp, wo)) return false;
    if (m.bsdf == BSDF_S) {
        const V3<R> fs = bsdf_eval(m, albedo, g, wi, wo, true, le);
        if (is_zero(fs)) return false;
        weight = fs / bsdf_pdf(m, g, wi, wo);
        return true;
    }
    const V3<R> lwi = to_local(g, wi), lwo = to_local(g, wo);
    if (lwi.z <= R(0) || lwo.z <= R(0)) return false;
    const R corr = shading_correction(g, wi, wo, lwi.z, lwo.z, le);
    if (corr == R(0)) return false;
    if (m.bsdf == BSDF_D) {
        if (is_zero(albedo)) return false;
        weight = le ? albedo * corr : albedo;
        return true;
    }
    // BSDF_G
    const V3<R> H = normalize(lwi + lwo);
    if (H.z <= R(0) || beckmann_d(m.roughness, H) == R(0)) return false;
    const R G = shadow_masking(lwi, lwo, H);
    const V3<R> F = fr_conductor(m, dot(lwi, H));
    weight = albedo * (G * dot(lwo, H) / (lwi.z * H.z) * (le ? corr : R(1))) * F;
    return !is_zero(weight);
}

// ---- pinhole sensor (rt.hpp:733-739, 955-977, 1189-1211, 1348-1378) -----------------------
template <typename R>
NGI_D V3<R> pinhole_direction(const DevSensor<R>& c, R rx, R ry) {
    const R x = R(2) * rx - R(1), y = R(2) * ry - R(1);
    const V3<R> we = normalize(v3<R>(c.aspect * c.tan_fov * x, c.tan_fov * y, R(-1)));
    return c.Vx * we.x + c.Vy * we.y + c.Vz * we.z;
}
template <typename R>
NGI_D bool pinhole_raster(const DevSensor<R>& c, V3<R> wo, R& rx, R& ry) {
    const R ex = dot(c.Vx, wo), ey = dot(c.Vy, wo), ez = dot(c.Vz, wo);
    if (ez >= R(0)) return false;
    rx = (-ex / ez / c.tan_fov / c.aspect + R(1)) * R(0.5);
    ry = (-ey / ez / c.tan_fov + R(1)) * R(0.5);
    return !(rx < R(0) || rx > R(1) || ry < R(0) || ry > R(1));
}
// Pinhole importance W(wo) = 1 / (cos^3 * 4 tan^2 aspect) inside the image, 0 outside.
template <typename R>
NGI_D R pinhole_importance(const DevSensor<R>& c, V3<R> wo) {
    R rx, ry;
    if (!pinhole_raster(c, wo, rx, ry)) return R(0);
    const R cos_t = -dot(c.Vz, wo);
    const R inv = R(1) / cos_t;
    const R A = c.tan_fov * c.tan_fov * c.aspect * R(4);
    return inv * inv * inv / A;
}

// Distribution1D::SampleReuse (basic.hpp:469-475) on an FP64 cdf of n+1 entries.
NGI_D int cdf_sample_reuse(const double* __restrict__ cdf, int n, double u, double& u2) {
    // upper_bound: first index with cdf[i] > u
    int lo = 0, hi = n + 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    int i = lo - 1;
    i = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    u2 = (u - cdf[i]) / (cdf[i + 1] - cdf[i]);
    return i;
}

// The same sample for the FP32 path, on the same FP64 cdf with a fraction of the FP64 arithmetic
// (this GPU issues FP64 at 1/64 of the FP32 rate). The cdf entries and u are non-negative, and
// non-negative IEEE-754 doubles order like their bit patterns read as integers: the search compares
// those, so it returns the index the FP64 comparisons give. The reused variable takes the two
// differences in FP64 and their quotient in FP32 (within an FP32 ulp or so of the FP64 quotient).
NGI_D int cdf_sample_reuse(const double* __restrict__ cdf, int n, float u, float& u2) {
    const double ud = (double)u;
    const long long ub = __double_as_longlong(ud);
    int lo = 0, hi = n + 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__double_as_longlong(cdf[mid]) > ub) hi = mid; else lo = mid + 1;
    }
    int i = lo - 1;
    i = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    const double c0 = cdf[i];
    u2 = (float)(ud - c0) / (float)(cdf[i + 1] - c0);
    return i;
}

// SamplePosition on a triangle mesh emitter (rt.hpp:488-526).
template <typename R>
NGI_D void sample_mesh_position(const SceneView<R>& sv, int tri_base, int tri_count, int cdf_offset, R u0, R u1,
                                Geom<R>& g) {
    R u2;
    const int i = cdf_sample_reuse(sv.cdf + cdf_offset, tri_count, u0, u2);
    R b0, b1;
    uniform_triangle(u2, u1, b0, b1);
    const float* P = sv.emit_tri_pos + 9 * (size_t)(tri_base + i);
    const V3<R> p1 = v3<R>(P[0], P[1], P[2]), p2 = v3<R>(P[3], P[4], P[5]), p3 = v3<R>(P[6], P[7], P[8]);
    g.p = p1 * (R(1) - b0 - b1) + p2 * b0 + p3 * b1;
    const float* T = sv.emit_tri_uv + 6 * (size_t)(tri_base + i);
    g.uvx = (R)T[0] * (R(1) - b0 - b1) + (R)T[2] * b0 + (R)T[4] * b1;
    g.uvy = (R)T[1] * (R(1) - b0 - b1) + (R)T[3] * b0 + (R)T[5] * b1;
    g.degenerated = false;
    g.ext = max_abs3(p1, p2, p3);
    g.gn = normalize(cross(p2 - p1, p3 - p1));
    g.sn = g.gn;
    tangent_space(g);
}

// Primitive::SamplePosition for a light (rt.hpp:483-592): area mesh, point, or the disk of
// the scene's bounding sphere that a directional light shines from.
template <typename R>
NGI_D void sample_light_position(const SceneView<R>& sv, const DevLight<R>& L, R u0, R u1, Geom<R>& g) {
    g.uvx = g.uvy = R(0);
    g.ext = 0.0f;
    if (L.type == LT_AREA) {
        sample_mesh_position(sv, L.tri_base, L.tri_count, L.cdf_offset, u0, u1, g);
        return;
    }
    if (L.type == LT_POINT) {
        g.p = L.position;
        g.degenerated = true;
        g.sn = g.gn = g.du = g.dv = v3<R>(0, 0, 0);
        return;
    }
    R sx, sy;
    concentric_disk(u0, u1, sx, sy);
    g.degenerated = false;
    g.gn = g.sn = L.direction;
    tangent_space(g);
    g.p = L.center - L.direction * L.radius + (g.du * (sx * L.radius) + g.dv * (sy * L.radius));
}

// Primitive::SampleDirection + EvaluateDirection(LE, forceDegenerated) / EvaluateDirectionPDF
// for a light vertex (rt.hpp:697-714, 917-937, 1154-1171): the emitted direction and the
// weight Le / pdf. False where the weight is zero.
template <typename R>
NGI_D bool light_sample_direction(const DevLight<R>& L, const Geom<R>& g, R u0, R u1, V3<R>& wo, V3<R>& weight) {
    if (L.type == LT_AREA) {
        const V3<R> l = cosine_hemisphere(u0, u1);
        wo = to_world(g, l);
        if (!(to_local(g, wo).z > R(0)) || is_zero(L.Le)) return false;
        weight = L.Le / kInvPi_<R>();  // pdf 1/pi per projected solid angle
        return true;
    }
    if (L.type == LT_POINT) {
        const R z = R(1) - R(2) * u0;
        const R r = sqrt_(fmax_(R(0), R(1) - z * z));
        R sp, cp;
        sincos2pi_(u1, &sp, &cp);
        wo = v3<R>(r * cp, r * sp, z);
        weight = L.Le / (kInvPi_<R>() * R(0.25));  // pdf 1/(4 pi) per solid angle
        return !is_zero(L.Le);
    }
    wo = L.direction;
    weight = L.Le;
    return !is_zero(L.Le);
}

// GeometryTerm (rt.hpp:2364-2374)
template <typename R>
NGI_D R geometry_term(const Geom<R>& a, const Geom<R>& b) {
    V3<R> d = b.p - a.p;
    const R l2 = dot(d, d);
    const R l = sqrt_(l2);
    d = d / l;
    R t = R(1);
    if (!a.degenerated) t *= fabs_(dot(a.sn, d));
    if (!b.degenerated) t *= fabs_(dot(b.sn, -d));
    return t / l2;
}

}  // namespace ngi
