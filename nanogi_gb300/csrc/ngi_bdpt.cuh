// Bidirectional path tracing with power-heuristic MIS: the path-space mathematics of the
// reference's Path (include/nanogi/bdpt.hpp:54-532) on vertices kept in HBM.
//
// A sample stores a light subpath and an eye subpath (at most kBdptMaxVertices each). A full
// path of strategy (s, t) is L[0..s-1] followed by E[t-1..0]; as in Path::Connect the first
// vertex becomes a light when s = 0 and the last a sensor when t = 0. Every quantity is
// recomputed from vertex positions, as the reference does, in the precision R.
#pragma once

#include "ngi_shade.cuh"

namespace ngi {

constexpr int kBdptMaxVertices = 32;

template <typename R>
struct BdVert {
    V3<R> p, sn, gn;
    R uvx, uvy;
    float ext;
    int prim;
    int type;         // DT_L, DT_E or the BSDF bits of the primitive
    int degenerated;
};

template <typename R>
NGI_D Geom<R> bd_geom(const BdVert<R>& v) {
    Geom<R> g;
    g.p = v.p;
    g.sn = v.sn;
    g.gn = v.gn;
    g.uvx = v.uvx;
    g.uvy = v.uvy;
    g.ext = v.ext;
    g.degenerated = v.degenerated != 0;
    if (g.degenerated) g.du = g.dv = v3<R>(0, 0, 0);
    else tangent_space(g);
    return g;
}

template <typename R>
NGI_D BdVert<R> bd_vert(const Geom<R>& g, int prim, int type) {
    BdVert<R> v;
    v.p = g.p;
    v.sn = g.sn;
    v.gn = g.gn;
    v.uvx = g.uvx;
    v.uvy = g.uvy;
    v.ext = g.ext;
    v.prim = prim;
    v.type = type;
    v.degenerated = g.degenerated ? 1 : 0;
    return v;
}

// Primitive::EvaluateDirection for any vertex type (rt.hpp:912-1148).
template <typename R>
NGI_D V3<R> bd_eval(const SceneView<R>& sv, const Geom<R>& g, int prim, int type, V3<R> wi, V3<R> wo, bool le,
                    bool force) {
    const DevMaterial<R>& m = sv.mats[prim];
    const V3<R> zero = v3<R>(0, 0, 0);
    if (type & DT_L) {
        if (m.l_type == LT_AREA) return to_local(g, wo).z <= R(0) ? zero : m.Le;
        if (m.l_type == LT_POINT) return m.Le;
        return force ? m.Le : zero;
    }
    if (type & DT_E) {
        if (m.e_type == ET_AREA) return to_local(g, wo).z <= R(0) ? zero : m.We;
        const R w = pinhole_importance(sv.sensor, wo);
        return v3<R>(w, w, w);
    }
    return bsdf_eval(m, material_albedo(sv, m, g), g, wi, wo, force, le);
}

// Primitive::EvaluateDirectionPDF with forceDegenerated = true (rt.hpp:1150-1336).
template <typename R>
NGI_D R bd_pdf(const SceneView<R>& sv, const Geom<R>& g, int prim, int type, V3<R> wi, V3<R> wo) {
    const DevMaterial<R>& m = sv.mats[prim];
    if (type & DT_L) {
        if (m.l_type == LT_AREA) return to_local(g, wo).z <= R(0) ? R(0) : kInvPi_<R>();
        if (m.l_type == LT_POINT) return kInvPi_<R>() * R(0.25);
        return R(1);
    }
    if (type & DT_E) {
        if (m.e_type == ET_AREA) return to_local(g, wo).z <= R(0) ? R(0) : kInvPi_<R>();
        return pinhole_importance(sv.sensor, wo);
    }
    return bsdf_pdf(m, g, wi, wo);
}

// EvaluatePosition (rt.hpp:594-641) and EvaluatePositionPDF(.., true) x EvaluateEmitterPDF
// (rt.hpp:643-690, 2338-2352) of the primitive under a path end.
template <typename R>
NGI_D R bd_position(const SceneView<R>& sv, int prim, bool force) {
    const DevMaterial<R>& m = sv.mats[prim];
    if (m.type & DT_L) return m.l_type == LT_POINT ? (force ? R(1) : R(0)) : R(1);
    return m.e_type == ET_PINHOLE ? (force ? R(1) : R(0)) : R(1);
}
template <typename R>
NGI_D R bd_position_pdf(const SceneView<R>& sv, int prim) {
    const DevMaterial<R>& m = sv.mats[prim];
    if (m.type & DT_L) {
        const R pa = m.l_type == LT_POINT ? R(1) : sv.lights[m.light_index].inv_area;
        return pa * (R(1) / (R)sv.num_lights);
    }
    if (m.type & DT_E) return m.e_type == ET_PINHOLE ? R(1) : sv.sensor.inv_area;
    return R(0);
}

// The full path of strategy s over the stored subpaths (Path::Connect's vertex order).
template <typename R>
struct BdPath {
    const BdVert<R>* L;
    const BdVert<R>* E;
    int s, n;
    NGI_D const BdVert<R>& at(int i) const { return i < s ? L[i] : E[n - 1 - i]; }
    NGI_D int type(int i) const {
        if (s == 0 && i == 0) return DT_L;
        if (s == n && i == n - 1) return DT_E;
        return at(i).type;
    }
    NGI_D Geom<R> geom(int i) const { return bd_geom(at(i)); }
};

template <typename R>
NGI_D V3<R> bd_dir(const BdVert<R>& a, const BdVert<R>& b) { return normalize(b.p - a.p); }

// Path::EvaluateCst (bdpt.hpp:213-244) for strategy i of path x.
template <typename R>
NGI_D V3<R> bd_cst(const SceneView<R>& sv, const BdPath<R>& x, int i) {
    const int n = x.n, t = n - i;
    const V3<R> zero = v3<R>(0, 0, 0);
    if (i == 0 && t > 0) {
        const BdVert<R>& v = x.at(0);
        return bd_eval(sv, x.geom(0), v.prim, x.type(0), zero, bd_dir(v, x.at(1)), false, false) *
               bd_position(sv, v.prim, false);
    }
    if (i > 0 && t == 0) {
        const BdVert<R>& v = x.at(n - 1);
        return bd_eval(sv, x.geom(n - 1), v.prim, x.type(n - 1), zero, bd_dir(v, x.at(n - 2)), true, false) *
               bd_position(sv, v.prim, false);
    }
    const BdVert<R>& vL = x.at(i - 1);
    const BdVert<R>& vE = x.at(i);
    const Geom<R> gL = x.geom(i - 1), gE = x.geom(i);
    const V3<R> wiL = i - 2 >= 0 ? bd_dir(vL, x.at(i - 2)) : zero;
    const V3<R> wiE = i + 1 < n ? bd_dir(vE, x.at(i + 1)) : zero;
    const V3<R> fsL = bd_eval(sv, gL, vL.prim, x.type(i - 1), wiL, bd_dir(vL, vE), true, false);
    if (is_zero(fsL)) return zero;
    const V3<R> fsE = bd_eval(sv, gE, vE.prim, x.type(i), wiE, bd_dir(vE, vL), false, false);
    return fsL * geometry_term(gL, gE) * fsE;
}

// f / p, 0 when f is 0 (bdpt.hpp:252-257)
template <typename R>
NGI_D V3<R> bd_local(V3<R> f, R p) { return is_zero(f) ? v3<R>(0, 0, 0) : f / p; }

// Path::EvaluateUnweightContribution (bdpt.hpp:246-320)
template <typename R>
NGI_D V3<R> bd_unweighted(const SceneView<R>& sv, const BdPath<R>& x) {
    const int n = x.n, s = x.s, t = n - s;
    const V3<R> zero = v3<R>(0, 0, 0), one = v3<R>(1, 1, 1);
    V3<R> aL = one;
    if (s > 0) {
        const int p0 = x.at(0).prim;
        aL = bd_local(one * bd_position(sv, p0, true), bd_position_pdf(sv, p0));
        for (int i = 0; i < s - 1 && !is_zero(aL); i++) {
            const BdVert<R>& v = x.at(i);
            const Geom<R> g = x.geom(i);
            const V3<R> wi = i >= 1 ? bd_dir(v, x.at(i - 1)) : zero;
            const V3<R> wo = bd_dir(v, x.at(i + 1));
            aL = aL * bd_local(bd_eval(sv, g, v.prim, x.type(i), wi, wo, true, true),
                               bd_pdf(sv, g, v.prim, x.type(i), wi, wo));
        }
    }
    if (is_zero(aL)) return zero;
    V3<R> aE = one;
    if (t > 0) {
        const int pn = x.at(n - 1).prim;
        aE = bd_local(one * bd_position(sv, pn, true), bd_position_pdf(sv, pn));
        for (int i = n - 1; i > s && !is_zero(aE); i--) {
            const BdVert<R>& v = x.at(i);
            const Geom<R> g = x.geom(i);
            const V3<R> wi = i < n - 1 ? bd_dir(v, x.at(i + 1)) : zero;
            const V3<R> wo = bd_dir(v, x.at(i - 1));
            aE = aE * bd_local(bd_eval(sv, g, v.prim, x.type(i), wi, wo, false, true),
                               bd_pdf(sv, g, v.prim, x.type(i), wi, wo));
        }
    }
    if (is_zero(aE)) return zero;
    const V3<R> cst = bd_cst(sv, x, s);
    if (is_zero(cst)) return zero;
    return aL * cst * aE;
}

// Path::EvaluatePDF (bdpt.hpp:480-529): area-measure pdf of x under strategy i.
template <typename R>
NGI_D R bd_path_pdf(const SceneView<R>& sv, const BdPath<R>& x, int i) {
    if (is_zero(bd_cst(sv, x, i))) return R(0);
    const int n = x.n, t = n - i;
    const V3<R> zero = v3<R>(0, 0, 0);
    R pdf = R(1);
    if (i > 0) {
        pdf *= bd_position_pdf(sv, x.at(0).prim);
        for (int k = 0; k < i - 1; k++) {
            const BdVert<R>& v = x.at(k);
            const Geom<R> g = x.geom(k);
            const V3<R> wi = k - 1 >= 0 ? bd_dir(v, x.at(k - 1)) : zero;
            pdf *= bd_pdf(sv, g, v.prim, x.type(k), wi, bd_dir(v, x.at(k + 1)));
            pdf *= geometry_term(g, x.geom(k + 1));
        }
    }
    if (t > 0) {
        pdf *= bd_position_pdf(sv, x.at(n - 1).prim);
        for (int k = n - 1; k >= i + 1; k--) {
            const BdVert<R>& v = x.at(k);
            const Geom<R> g = x.geom(k);
            const V3<R> wi = k + 1 < n ? bd_dir(v, x.at(k + 1)) : zero;
            pdf *= bd_pdf(sv, g, v.prim, x.type(k), wi, bd_dir(v, x.at(k - 1)));
            pdf *= geometry_term(g, x.geom(k - 1));
        }
    }
    return pdf;
}

// Path::EvaluatePowerHeuristicsMISWeightOpt (bdpt.hpp:366-384)
template <typename R>
NGI_D R bd_mis_weight(const SceneView<R>& sv, const BdPath<R>& x) {
    const R ps = bd_path_pdf(sv, x, x.s);
    R inv = R(0);
    for (int i = 0; i <= x.n; i++) {
        const R pi = i == x.s ? ps : bd_path_pdf(sv, x, i);
        if (pi > R(0)) {
            const R r = pi / ps;
            inv += r * r;
        }
    }
    return R(1) / inv;
}

// Path::SelectionProb (bdpt.hpp:188-202)
template <typename R>
NGI_D R bd_selection_prob(int n, int s) {
    const int t = n - s;
    R p = R(1);
    for (int i = 1; i < s - 1; i++) p *= R(0.5);
    for (int i = t - 2; i >= 1; i--) p *= R(0.5);
    return p;
}

}  // namespace ngi
