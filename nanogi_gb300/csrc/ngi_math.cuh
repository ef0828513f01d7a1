// Device math for the GB300 path tracer: a 3-vector templated on the shading precision
// (float for the tuned path, double for the plain path) and the counter-based RNG.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define NGI_HD __host__ __device__ __forceinline__
#define NGI_D __device__ __forceinline__

namespace ngi {

template <typename R>
struct V3 {
    R x, y, z;
};

template <typename R> NGI_HD V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> NGI_HD V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R> NGI_HD V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R> NGI_HD V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <typename R> NGI_HD V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename R> NGI_HD V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R> NGI_HD V3<R> operator*(R s, V3<R> a) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R> NGI_HD V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename R> NGI_HD R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> NGI_HD V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename R> NGI_HD bool is_zero(V3<R> a) { return a.x == R(0) && a.y == R(0) && a.z == R(0); }
template <typename R> NGI_HD V3<R> vabs(V3<R> a) { return {a.x < 0 ? -a.x : a.x, a.y < 0 ? -a.y : a.y, a.z < 0 ? -a.z : a.z}; }

template <typename To, typename From> NGI_HD V3<To> vcast(V3<From> a) { return {(To)a.x, (To)a.y, (To)a.z}; }

// ---- precision-specific scalar functions --------------------------------------------
// float: fast paths where the accuracy is far below the Monte-Carlo noise;
// double: the IEEE / libm-grade functions (the reference's glm/std calls).
NGI_D float rsqrt_(float x) { return rsqrtf(x); }
NGI_D double rsqrt_(double x) { return 1.0 / sqrt(x); }
NGI_D float sqrt_(float x) { return sqrtf(x); }
NGI_D double sqrt_(double x) { return sqrt(x); }
NGI_D float log_(float x) { return __logf(x); }
NGI_D double log_(double x) { return log(x); }
NGI_D float exp_(float x) { return __expf(x); }
NGI_D double exp_(double x) { return exp(x); }
NGI_D float rcp_(float x) { return __frcp_rn(x); }
NGI_D double rcp_(double x) { return 1.0 / x; }
NGI_D float fmax_(float a, float b) { return fmaxf(a, b); }
NGI_D double fmax_(double a, double b) { return fmax(a, b); }
NGI_D float fmin_(float a, float b) { return fminf(a, b); }
NGI_D double fmin_(double a, double b) { return fmin(a, b); }
NGI_D float fabs_(float a) { return fabsf(a); }
NGI_D double fabs_(double a) { return fabs(a); }
NGI_D float floor_(float a) { return floorf(a); }
NGI_D double floor_(double a) { return floor(a); }
// sin / cos of 2*pi*u for u in [0,1)
NGI_D void sincos2pi_(float u, float* s, float* c) { sincospif(2.0f * u, s, c); }
NGI_D void sincos2pi_(double u, double* s, double* c) { sincospi(2.0 * u, s, c); }
NGI_D void sincospi_(float x, float* s, float* c) { sincospif(x, s, c); }
NGI_D void sincospi_(double x, double* s, double* c) { sincospi(x, s, c); }
NGI_D void sincos_(float a, float* s, float* c) { sincosf(a, s, c); }
NGI_D void sincos_(double a, double* s, double* c) { sincos(a, s, c); }
NGI_D bool isnan_(float a) { return isnan(a); }
NGI_D bool isnan_(double a) { return isnan(a); }

// glm::normalize(v) = v * inversesqrt(dot(v, v))
template <typename R> NGI_D V3<R> normalize(V3<R> a) { return a * rsqrt_(dot(a, a)); }

// ---- Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ------------------------------
// Counter-based: the 4 outputs are a pure function of (counter, key), so every random
// number of a path is addressed by (seed, sample index, vertex, call) and any path can be
// replayed in isolation.
NGI_HD uint4 philox4x32_10(uint4 c, uint2 k) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r > 0) {
            k.x += W0;
            k.y += W1;
        }
#ifdef __CUDA_ARCH__
        const uint32_t hi0 = __umulhi(M0, c.x), hi1 = __umulhi(M1, c.z);
#else
        const uint32_t hi0 = (uint32_t)(((uint64_t)M0 * c.x) >> 32), hi1 = (uint32_t)(((uint64_t)M1 * c.z) >> 32);
#endif
        const uint32_t lo0 = M0 * c.x, lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

// 24-bit uniform in [0,1), exactly representable in float and double alike.
NGI_HD float u24(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// The 4 uniforms of call `call` at path vertex `vertex` of global sample `sample`.
struct RngKey {
    uint2 key;
    uint32_t s_lo, s_hi;
};
NGI_HD RngKey make_rng(uint64_t seed, uint64_t sample) {
    return RngKey{make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)), (uint32_t)sample, (uint32_t)(sample >> 32)};
}
NGI_HD float4 rng4(const RngKey& r, uint32_t vertex, uint32_t call) {
    uint4 o = philox4x32_10(make_uint4(r.s_lo, r.s_hi, vertex, call), r.key);
    return make_float4(u24(o.x), u24(o.y), u24(o.z), u24(o.w));
}

// Dimension layout per vertex v (v = 1 is the sensor vertex):
//   call 0: x = light pick, y,z = light position, w = Russian roulette after this vertex's ray
//   call 1: x,y = direction (raster position at the sensor), z = component choice
//   call 2: x,y = sensor position (area sensor)
enum : uint32_t { RNG_NEE_RR = 0, RNG_DIR = 1, RNG_SENSOR = 2 };

}  // namespace ngi
