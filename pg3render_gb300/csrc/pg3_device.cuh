// Device building blocks of the path-tracing hot path (sm_103a).
//
// Each function restates one piece of the reference renderer's arithmetic
// (file:line given per function, paths relative to the reference project) in
// a form suited to a GPU thread: float3 registers instead of Vec3f objects,
// a counter-based random stream instead of a per-renderer mt19937_64, and no
// virtual dispatch (materials are a switch over a 64-byte record).
#pragma once

// The triangle test's plane distance by the fast division (__fdividef, within 2 ulp of the
// IEEE quotient for the denominators that occur, |n . dir| <= 1) instead of the IEEE one (+1.9% on
// the environment-map benchmark). Every query (list, binary and 4-wide BVH, batch) uses the same
// test, so they still agree bit for bit.
#ifndef PG3_FAST_HIT_DIV
#define PG3_FAST_HIT_DIV 1
#endif
// The sphere test's divisions likewise (|dir|^2 = 1 to float rounding).
#ifndef PG3_FAST_SPHERE_DIV
#define PG3_FAST_SPHERE_DIV 1
#endif

#include <cstdint>
#include <cuda_runtime.h>

#include "pg3_scene_view.h"

namespace pg3 {

#define PG3_DI __device__ __forceinline__

// ------------------------------------------------------------------------------------------
// float3 helpers
// ------------------------------------------------------------------------------------------
PG3_DI float3 f3(float a) { return make_float3(a, a, a); }
PG3_DI float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
PG3_DI float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
PG3_DI float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
PG3_DI float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
PG3_DI float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
PG3_DI float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
PG3_DI float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
PG3_DI void operator+=(float3 &a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
PG3_DI float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PG3_DI float3 cross(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
PG3_DI float length(float3 a) { return sqrtf(dot(a, a)); }
PG3_DI float3 normalize(float3 a) { return a / length(a); }
PG3_DI float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
PG3_DI bool isZero(float3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
PG3_DI float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
// sRGB luminance (src/spectrum.hxx:74-80)
PG3_DI float luminance(float3 a) { return 0.212671f * a.x + 0.715160f * a.y + 0.072169f * a.z; }

constexpr float kPiF = 3.14159265358979f;             // src/math.hxx:12
constexpr float kPiInvF = 1.f / kPiF;
constexpr float kTinyF = 9.5367431640625E-7f;         // src/math.hxx:46
constexpr float kEpsRay = 1e-3f;                      // src/geom.hxx:16
constexpr float kEpsDist = 1e-6f;                     // src/geom.hxx:27
constexpr float kFloatMax = 3.402823466e+38f;
constexpr uint32_t kMaxPathLengthHard = 1200;         // src/path_tracer.hxx:461-462

PG3_DI bool isTiny(float x) { return fabsf(x) < kTinyF; }
PG3_DI float sqr(float x) { return x * x; }
PG3_DI float safeSqrt(float x) { return sqrtf(fmaxf(0.f, x)); }
PG3_DI float clampf(float v, float a, float b) { return fminf(fmaxf(v, a), b); }
PG3_DI float infF() { return __int_as_float(0x7f800000); }

// ------------------------------------------------------------------------------------------
// Counter-based random numbers: Philox4x32-10 (Salmon et al., SC'11). The counter is
// (pixel, sample, vertex, group) and the key the 64-bit seed, so any path vertex can be
// regenerated independently (wavefront stages, path replay).
// ------------------------------------------------------------------------------------------
struct Rand4 { float a, b, c, d; };

PG3_DI float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

PG3_DI Rand4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    Rand4 r;
    r.a = u01(c0); r.b = u01(c1); r.c = u01(c2); r.d = u01(c3);
    return r;
}
PG3_DI Rand4 draw(const SceneView &S, uint32_t pixel, uint32_t sample, uint32_t vertex, uint32_t group)
{
    return philox(pixel, sample, vertex, group, S.seedLo, S.seedHi);
}

// ------------------------------------------------------------------------------------------
// Frames and directions (src/math.hxx:981-999, src/geom.hxx)
// ------------------------------------------------------------------------------------------
struct Frame { float3 x, y, z; };
PG3_DI Frame frameFromZ(float3 z)
{
    Frame f;
    f.z = z;
    const float3 tmpX = (fabsf(z.x) > 0.99f) ? make_float3(0, 1, 0) : make_float3(1, 0, 0);
    f.y = normalize(cross(z, tmpX));
    f.x = cross(f.y, z);
    return f;
}
PG3_DI float3 toWorld(const Frame &f, float3 a) { return f.x * a.x + f.y * a.y + f.z * a.z; }
PG3_DI float3 toLocal(const Frame &f, float3 a) { return make_float3(dot(a, f.x), dot(a, f.y), dot(a, f.z)); }

PG3_DI float epsRayCos(float c) { return (1.f + 2.f * (1.f - c)) * kEpsRay; }   // src/geom.hxx:22-25

// src/geom.hxx:65-73
PG3_DI float3 latLong2Dir(float u, float v)
{
    const float phi = -(u - 0.5f) * 2.f * kPiF;
    const float theta = v * kPiF;
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    return make_float3(st * cp, st * sp, ct);
}
// src/geom.hxx:77-95
PG3_DI void dir2LatLong(float3 d, float &u, float &v)
{
    const float phi = -atan2f(d.y, d.x);
    const float theta = acosf(d.z);
    u = clampf(0.5f + phi * 0.5f * kPiInvF, 0.f, 1.f);
    v = clampf(theta * kPiInvF, 0.f, 1.f);
}
// src/geom.hxx:97-107
PG3_DI float tanThetaSqr(float3 d)
{
    const float c2 = d.z * d.z;
    const float s2 = 1.f - c2;
    return (s2 <= 0.0f) ? 0.0f : s2 / c2;
}
// src/geom.hxx:116-133
PG3_DI float3 reflect(bool &above, float3 in, float3 n)
{
    const float d = dot(in, n);
    above = d > 0.0f;
    return (2.0f * d) * n - in;
}
// src/geom.hxx:145-179
PG3_DI float3 refract(bool &inAbove, float3 in, float3 n, float eta)
{
    const float cosI = dot(in, n);
    inAbove = cosI > 0.0f;
    if (inAbove) eta = 1.0f / eta;
    const float cosT2 = 1.f - (1.f - cosI * cosI) * (eta * eta);
    if (cosT2 < 0.0f) { bool d; return reflect(d, in, n); }
    float cosT = sqrtf(cosT2);
    cosT = (cosI > 0.0f) ? -cosT : cosT;
    return n * (cosI * eta + cosT) - in * eta;
}

// ------------------------------------------------------------------------------------------
// Hemisphere sampling (src/sampling.hxx:289-361)
// ------------------------------------------------------------------------------------------
PG3_DI float3 sampleCosHemisphere(float u0, float u1, float &pdf)
{
    float s, c;
    sincosf(2.f * kPiF * u0, &s, &c);
    const float t2 = sqrtf(1.f - u1);
    const float3 r = make_float3(c * t2, s * t2, sqrtf(u1));
    pdf = r.z * kPiInvF;
    return r;
}
PG3_DI float cosHemispherePdf(float z) { return fmaxf(0.f, z) * kPiInvF; }
// SamplePowerCosHemisphereW / PowerCosHemispherePdfW (src/sampling.hxx:250-285): density
// (n + 1) cos^n / (2 pi) around +z
PG3_DI float3 samplePowerCosHemisphere(float u0, float u1, float power)
{
    const float t2 = powf(u1, 1.f / (power + 1.f));
    const float t3 = sqrtf(1.f - t2 * t2);
    float s, c;
    sincosf(2.f * kPiF * u0, &s, &c);
    return make_float3(c * t3, s * t3, t2);
}
PG3_DI float powerCosHemispherePdf(float z, float power)
{
    return (power + 1.f) * powf(fmaxf(0.f, z), power) * (kPiInvF * 0.5f);
}
// ReflectLocal (src/geom.hxx:110-113): mirror direction about the local normal
PG3_DI float3 reflectLocal(float3 v) { return make_float3(-v.x, -v.y, v.z); }
// upper hemisphere only: every material on this path samples lights from the front side
// (kBsdfFrontSideLightSampling, src/materials.hxx:253-266, 788-806, 992-1021)
PG3_DI float cosSpherePdfFront(float3 local) { return (local.z < 0.f) ? 0.f : cosHemispherePdf(fabsf(local.z)); }

// ------------------------------------------------------------------------------------------
// Fresnel (src/physics.hxx:5-148, Mitsuba conductor variant per src/hard_config.hxx:15)
// ------------------------------------------------------------------------------------------
PG3_DI float fresnelDielectric(float cosI, float etaAbs)
{
    if (etaAbs < 0.f) return 1.f;
    float eta;
    if (cosI < 0.f) { cosI = -cosI; eta = etaAbs; }
    else eta = 1.f / etaAbs;
    const float sinT2 = sqr(eta) * (1.f - sqr(cosI));
    const float cosT = safeSqrt(1.f - sinT2);
    if (sinT2 > 1.0f) return 1.0f;
    const float t2 = eta * cosI;
    const float rs = sqr((t2 - cosT) / (t2 + cosT));
    const float t1 = eta * cosT;
    const float rp = sqr((cosI - t1) / (cosI + t1));
    return 0.5f * (rp + rs);
}
PG3_DI float fresnelConductor(float cosI, float eta, float k)
{
    if (cosI < -0.00001f) return 0.0f;
    cosI = clampf(cosI, 0.0f, 1.0f);
    const float c2 = cosI * cosI, s2 = 1.f - c2, s4 = s2 * s2;
    const float eta2 = eta * eta, k2 = k * k;
    const float temp1 = eta2 - k2 - s2;
    const float a2pb2 = safeSqrt(temp1 * temp1 + 4.f * k2 * eta2);
    const float a = safeSqrt(0.5f * (a2pb2 + temp1));
    const float term1 = a2pb2 + c2, term2 = 2.f * a * cosI;
    const float Rs2 = (term1 - term2) / (term1 + term2);
    const float term3 = a2pb2 * c2 + s4, term4 = term2 * s2;
    const float Rp2 = Rs2 * (term3 - term4) / (term3 + term4);
    return 0.5f * (Rp2 + Rs2);
}

// ------------------------------------------------------------------------------------------
// GGX microfacet model (src/microfacet.hxx)
// ------------------------------------------------------------------------------------------
PG3_DI float reflectionJacobian(float3 wo, float3 m)          // :16-31
{
    return 1.0f / (4.0f * fmaxf(dot(m, wo), 0.000001f));
}
PG3_DI float refractionJacobian(float3 wi, float3 wo, float3 m, float etaOutIn)   // :34-56
{
    const float cOM = dot(m, wo), cIM = dot(m, wi);
    return fabsf(cOM) / fmaxf(sqr(etaOutIn * cIM + cOM), 0.000001f);
}
PG3_DI float3 halfwayReflection(float3 wi, float3 wo)         // :60-84
{
    float3 h = wi + wo;
    const float l = length(h);
    h = isTiny(l) ? make_float3(0.f, 0.f, 1.f) : h / l;
    return h * ((h.z >= 0.0f) ? 1.0f : -1.0f);
}
PG3_DI float3 halfwayRefraction(float3 wi, float3 wo, float etaInOut)   // :88-123
{
    float3 h = wi + wo * etaInOut;
    const float l = length(h);
    h = isTiny(l) ? wi : h / l;
    return h * ((h.z >= 0.0f) ? 1.0f : -1.0f);
}
PG3_DI float ggxD(float3 m, float a)                           // :505-527
{
    if (m.z <= 0.f) return 0.0f;
    const float a2 = a * a, c2 = m.z * m.z;
    const float t = c2 * (a2 + tanThetaSqr(m));
    return a2 / (kPiF * t * t);
}
PG3_DI float smithG1(float3 v, float3 m, float a)              // :529-554
{
    if (m.z <= 0.f) return 0.0f;
    if (v.z * dot(v, m) < 0.0f) return 0.0f;
    return 2.0f / (1.0f + sqrtf(1.0f + a * a * tanThetaSqr(v)));
}
// Visible-normal slope sampling for unit roughness, src/microfacet.hxx:610-673
// (Heitz & d'Eon 2014 with the reference's rational fit of the conditional CDF^-1).
PG3_DI void sampleGgxP11(float &sx, float &sy, float thetaI, float u0, float u1)
{
    if (thetaI < 0.0001f) {
        const float ux = fminf(u0, 0.9999f);
        const float r = safeSqrt(ux / (1.f - ux));
        float s, c;
        sincosf(2.f * kPiF * u1, &s, &c);
        sx = r * c;
        sy = r * s;
        return;
    }
    const float tanI = tanf(thetaI);
    const float tanIInv = 1.0f / tanI;
    const float G1 = 2.0f / (1.0f + safeSqrt(1.0f + 1.0f / (tanIInv * tanIInv)));
    float A = 2.0f * u0 / G1 - 1.0f;
    if (fabsf(A) == 1.0f) A -= (signbit(A) ? -1.f : 1.f) * 1e-4f;
    const float B = tanI;
    const float tmp = 1.0f / (A * A - 1.0f);
    const float D = safeSqrt(B * B * tmp * tmp - (A * A - B * B) * tmp);
    const float x1 = B * tmp - D, x2 = B * tmp + D;
    sx = (A < 0.0f || x2 > (1.0f / tanI)) ? x1 : x2;
    float sign, ys;
    if (u1 > 0.5f) { sign = 1.0f; ys = 2.0f * (u1 - 0.5f); }
    else { sign = -1.0f; ys = 2.0f * (0.5f - u1); }
    const float z = (ys * (ys * (ys * -0.365728915865723f + 0.790235037209296f) - 0.424965825137544f) +
                     0.000152998850436920f) /
                    (ys * (ys * (ys * (ys * 0.169507819808272f - 0.397203533833404f) - 0.232500544458471f) + 1.0f) -
                     0.539825872510702f);
    sy = sign * z * sqrtf(1.0f + sx * sx);
}
PG3_DI float3 sampleGgxVisibleNormals(float3 wo, float a, float u0, float u1)   // :678-729
{
    const float3 ws = normalize(make_float3(wo.x * a, wo.y * a, fmaxf(wo.z, 0.0f)));
    float theta = 0.0f, phi = 0.0f;
    if (ws.z < 0.999f) {
        theta = acosf(ws.z);
        phi = atan2f(ws.y, ws.x);
    }
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float sx, sy;
    sampleGgxP11(sx, sy, theta, u0, u1);
    const float x = (sx * cp - sy * sp) * a;
    const float y = (sx * sp + sy * cp) * a;
    const float inv = 1.0f / sqrtf(x * x + y * y + 1.0f);
    return make_float3(-x * inv, -y * inv, inv);
}
// Exact visible-normal sampling (Heitz, "Sampling the GGX Distribution of Visible Normals",
// JCGT 7(4), 2018): the same density D_wo(m) as the routine above, without its rational fit
// of the slope CDF (whose tails over-produce sideways-tilted normals by up to 2x).
PG3_DI float3 sampleGgxVndfExact(float3 wo, float a, float u0, float u1)
{
    const float3 vh = normalize(make_float3(a * wo.x, a * wo.y, fmaxf(wo.z, 0.0f)));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const float3 t1 = lensq > 0.f ? make_float3(-vh.y, vh.x, 0.f) * rsqrtf(lensq) : make_float3(1.f, 0.f, 0.f);
    const float3 t2 = cross(vh, t1);
    const float r = sqrtf(u0);
    float sp, cp;
    sincosf(2.f * kPiF * u1, &sp, &cp);
    const float p1 = r * cp;
    const float s = 0.5f * (1.f + vh.z);
    const float p2 = (1.f - s) * sqrtf(fmaxf(0.f, 1.f - p1 * p1)) + s * (r * sp);
    const float3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(0.f, 1.f - p1 * p1 - p2 * p2));
    return normalize(make_float3(a * nh.x, a * nh.y, fmaxf(1e-6f, nh.z)));
}
PG3_DI float3 sampleGgxVndf(float3 wo, float a, float u0, float u1, bool exact)
{
    return exact ? sampleGgxVndfExact(wo, a, u0, u1) : sampleGgxVisibleNormals(wo, a, u0, u1);
}

PG3_DI float ggxPdfVisibleNormals(float3 wo, float3 h, float D, float a)          // :732-756
{
    if (h.z <= 0.f) return 0.0f;
    return (smithG1(wo, h, a) * fabsf(dot(h, wo)) * D) / fmaxf(wo.z, 0.00001f);
}

// ------------------------------------------------------------------------------------------
// Materials (src/materials.hxx). A record holds what the estimator reads after an
// EvalBsdf (with kOptSamplingProbs) or a SampleBsdf call.
// ------------------------------------------------------------------------------------------
struct BsdfRec {
    float3 wil;
    float3 att;
    float pdfW;
    float compProb;
    float dAtt;   // with derivatives requested: Lambert d att_c / d albedo_c, GGX d ln att / d alpha
};
PG3_DI bool isBlocker(const BsdfRec &r) { return maxc(r.att) * fabsf(r.wil.z) <= 1e-5f; }   // :63-67

PG3_DI DevMaterial loadMat(const SceneView &S, int id) { return S.mats[id]; }

// GGX conductor: src/materials.hxx:878-989
PG3_DI float3 condEval(const DevMaterial &m, float3 wil, float3 wol, float3 h, float F, float D)
{
    if (wil.z <= 0.f || wol.z <= 0.f || isTiny(4.0f * wil.z * wol.z)) return f3(0.f);
    const float G = smithG1(wil, h, m.alpha) * smithG1(wol, h, m.alpha);
    return f3((F * G * D) / (4.0f * wil.z * wol.z));
}
// pdfs and sampling use the sampling roughness alphaS (equal to alpha unless derivatives are
// checked with the sampling held fixed); Dp is D evaluated with alphaS
PG3_DI float condPdf(const DevMaterial &m, float3 wol, float3 h, float Dp)
{
    if (wol.z < 0.f) return 0.0f;
    return ggxPdfVisibleNormals(wol, h, Dp, m.alphaS) * reflectionJacobian(wol, h);
}
// d ln(D(m) G1(wi, m) G1(wo, m)) / d alpha, from ggxD and smithG1 above:
// d ln D / da = 2/a - 4a / (a^2 + tan^2 m),  d ln G1(v) / da = -a tan^2 v / (s (1 + s)), s = sqrt(1 + a^2 tan^2 v)
PG3_DI float ggxDlnDGda(float3 wi, float3 wo, float3 m, float a)
{
    const float a2 = a * a;
    const float ti = tanThetaSqr(wi), to = tanThetaSqr(wo);
    const float si = sqrtf(1.f + a2 * ti), so = sqrtf(1.f + a2 * to);
    return 2.f / a - 4.f * a / (a2 + tanThetaSqr(m)) - a * ti / (si * (1.f + si)) - a * to / (so * (1.f + so));
}
PG3_DI float ggxDp(const DevMaterial &m, float3 h, float D) { return (m.alphaS == m.alpha) ? D : ggxD(h, m.alphaS); }

// GGX dielectric: src/materials.hxx:1123-1266 (directions already switched to the wo side)
struct DielCtx { float3 wo, wi, m; bool refl; float etaS, etaInvS, F, D, Dp; };
PG3_DI float3 dielEval(const DevMaterial &mt, const DielCtx &c)
{
    const float ci = fabsf(c.wi.z), co = fabsf(c.wo.z);
    if ((!c.refl && isTiny(ci * co)) || (c.refl && isTiny(4.0f * ci * co))) return f3(0.f);
    const float G = smithG1(c.wi, c.m, mt.alpha) * smithG1(c.wo, c.m, mt.alpha);
    float v;
    if (c.refl) {
        v = (c.F * G * c.D) / (4.0f * ci * co);
    } else {
        const float cMI = dot(c.m, c.wi), cMO = dot(c.m, c.wo);
        v = ((fabsf(cMI) * fabsf(cMO)) / (ci * co)) *
            ((sqr(c.etaInvS) * (1.0f - c.F) * G * c.D) / sqr(cMI + c.etaInvS * cMO));
        v *= sqr(c.etaS);
    }
    return f3(v);
}
PG3_DI float dielPdf(const DevMaterial &mt, const DielCtx &c)
{
    if (c.wo.z < 0.f) return 0.0f;
    const float vn = ggxPdfVisibleNormals(c.wo, c.m, c.Dp, mt.alphaS);
    const float J = c.refl ? reflectionJacobian(c.wi, c.m) : refractionJacobian(c.wo, c.wi, c.m, c.etaInvS);
    return vn * J * (c.refl ? c.F : (1.f - c.F));
}

// Phong: src/materials.hxx:353-602. Diffuse plus a power-cosine lobe around the mirror direction;
// sampling picks the component by the luminance estimates below (the glossy one attenuated to
// half at grazing angles) and the pdf is the whole mixture.
PG3_DI float3 phongGlossy(const DevMaterial &m) { return make_float3(m.gr, m.gg, m.gb); }
PG3_DI float phongDiffuseEst(const DevMaterial &m) { return luminance(make_float3(m.r, m.g, m.b)); }
PG3_DI float phongGlossyEst(const DevMaterial &m, float3 wol)
{
    return luminance(phongGlossy(m)) * (0.5f + 0.5f * fmaxf(wol.z, 0.f));
}
PG3_DI float3 phongEval(const DevMaterial &m, float3 wil, float3 wol)      // :404-414
{
    if (wil.z <= 0.f || wol.z <= 0.f) return f3(0.f);
    const float cc = (m.exponent + 2.0f) / (2.0f * kPiF);
    const float c = fmaxf(dot(reflectLocal(wil), wol), 0.f);
    return make_float3(m.r, m.g, m.b) * kPiInvF + phongGlossy(m) * (cc * powf(c, m.exponent));
}
PG3_DI float phongPdf(const DevMaterial &m, float3 wol, float3 wil, float dEst, float gEst)   // :497-531
{
    const float tot = dEst + gEst;
    if (tot < 1e-5f) return cosHemispherePdf(wil.z);   // diffuse fallback of blockers
    // the lobe frame's z axis is the mirror direction: the canonical cosine is dot(wil, wrl)
    const float cz = dot(wil, reflectLocal(wol));
    return (dEst / tot) * cosHemispherePdf(wil.z) + (gEst / tot) * powerCosHemispherePdf(cz, m.exponent);
}
PG3_DI float smoothDielectricFresnel(const DevMaterial &m, float3 wol) { return fresnelDielectric(wol.z, m.eta); }

// SRA layered material (SraLayeredMaterial, src/materials.hxx:1304-1566): a GGX dielectric outer
// layer taken for reflection only, an inner Lambert or GGX conductor seen through the refracted
// directions, and a Beer-Lambert medium between them. The inner layer's record fields: r,g,b
// (Lambert), innerAlpha / innerEta / absorb (conductor); the medium: gr,gg,gb and exponent.
PG3_DI float3 sraMediumTrans(const DevMaterial &m, float len)   // Physics::BeerLambert
{
    return make_float3(expf(-(m.gr * len)), expf(-(m.gg * len)), expf(-(m.gb * len)));
}
// the inner layer's value, pdf and reflectance estimate (LambertMaterial :262-345; GGX conductor
// :878-989, its estimate the microfacet Fresnel reflectance :978-982)
PG3_DI void sraInnerEval(const DevMaterial &m, float3 wi, float3 wo, float3 &att, float &pdf, float &refl)
{
    if (m.innerKind == kMatLambert) {
        const float3 R = make_float3(m.r, m.g, m.b);
        att = (wi.z <= 0.f || wo.z <= 0.f) ? f3(0.f) : R * kPiInvF;
        pdf = cosHemispherePdf(wi.z);
        refl = luminance(R);
        return;
    }
    const float a = m.innerAlpha;
    const float3 h = halfwayReflection(wi, wo);
    const float D = ggxD(h, a);
    const float F = fresnelConductor(dot(h, wo), m.innerEta, m.absorb);
    if (wi.z <= 0.f || wo.z <= 0.f || isTiny(4.0f * wi.z * wo.z)) att = f3(0.f);
    else att = f3((F * smithG1(wi, h, a) * smithG1(wo, h, a) * D) / (4.0f * wi.z * wo.z));
    pdf = (wo.z < 0.f) ? 0.f : ggxPdfVisibleNormals(wo, h, D, a) * reflectionJacobian(wo, h);
    refl = F;
}
// EvalBsdf with kOptSamplingProbs (:1328-1451)
PG3_DI void sraEval(const DevMaterial &m, float3 wil, float3 wol, BsdfRec &r)
{
    r.wil = wil;
    r.compProb = 1.f;
    if (wil.z <= 0.f || wol.z <= 0.f) {   // no transmission below the horizon
        r.att = f3(0.f);
        r.pdfW = 0.f;
        return;
    }
    // outer layer, reflection only: the dielectric's reflection lobe, component probability 1
    DielCtx c;
    c.refl = true;
    c.wo = wol;
    c.wi = wil;
    c.etaS = m.eta;
    c.etaInvS = m.etaInv;
    c.m = halfwayReflection(wil, wol);
    c.D = ggxD(c.m, m.alpha);
    c.Dp = c.D;
    c.F = fresnelDielectric(dot(c.m, c.wo), c.etaS);
    const float3 attO = dielEval(m, c);
    const float pdfO = ggxPdfVisibleNormals(wol, c.m, c.D, m.alpha) * reflectionJacobian(wil, c.m);
    // inner layer through the refracted directions
    bool ab;
    const float3 n = make_float3(0.f, 0.f, 1.f);
    const float3 wiR = refract(ab, wil, n, m.eta), woR = refract(ab, wol, n, m.eta);
    const float Ti = 1.f - fresnelDielectric(wil.z, m.eta), Fo = fresnelDielectric(wol.z, m.eta);
    const float To = 1.f - Fo;
    const float cO = fmaxf(wol.z, 0.0001f), cI = fmaxf(wil.z, 0.0001f);
    const float3 mt = sraMediumTrans(m, m.exponent * (1.f / cO + 1.f / cI));
    float3 attI;
    float pdfI, reflI;
    sraInnerEval(m, -wiR, -woR, attI, pdfI, reflI);
    const float invEta2 = sqr(1.f / m.eta);
    r.att = attO + attI * (Ti * To) * invEta2 * mt;
    // mixture pdf with the component weights of the sampling routine
    const float3 mtEst = sraMediumTrans(m, m.exponent * (1.f / cO * 2.f));
    const float outerC = Fo, innerC = reflI * To * luminance(mtEst);
    const float tot = outerC + innerC;
    const float compr = invEta2 * (wil.z / -wiR.z);
    r.pdfW = pdfO * (outerC / tot) + (pdfI * compr) * (innerC / tot);
}
// SampleBsdf (:1457-1537): u2 picks the layer, (u0, u1) the direction
PG3_DI void sraSample(const DevMaterial &m, float3 wol, float u0, float u1, float u2, BsdfRec &r)
{
    const float Fo = fresnelDielectric(wol.z, m.eta), To = 1.f - Fo;
    float reflI;
    if (m.innerKind == kMatLambert) {
        reflI = luminance(make_float3(m.r, m.g, m.b));
    } else {
        // the inner record is queried before a direction exists (incoming direction zero): the
        // estimate is the Fresnel reflectance at the outgoing direction's own half vector
        const float3 h = halfwayReflection(f3(0.f), wol);
        reflI = fresnelConductor(dot(h, wol), m.innerEta, m.absorb);
    }
    const float cO = fmaxf(wol.z, 0.0001f);
    const float3 mtEst = sraMediumTrans(m, m.exponent * (1.f / cO * 2.f));
    const float outerC = Fo, innerC = reflI * To * luminance(mtEst);
    const float tot = outerC + innerC;
    float3 wil;
    bool ab;
    const float3 n = make_float3(0.f, 0.f, 1.f);
    if (u2 * tot < outerC) {
        // the outer dielectric sampled for reflection only (:1045-1079 with kReflectionOnly)
        const bool below = wol.z < 0.f;
        const float s = below ? -1.0f : 1.0f;
        const float3 wo = wol * s;
        const float3 mf = sampleGgxVndf(wo, m.alpha, u0, u1, m.vndfExact != 0);
        wil = reflect(ab, wo, mf) * s;
    } else {
        const float3 woR = refract(ab, wol, n, m.eta);
        const float3 wo = -woR;
        float3 wi;
        if (m.innerKind == kMatLambert) {
            float pdf;
            wi = sampleCosHemisphere(u0, u1, pdf);
        } else {
            const float3 h = sampleGgxVndf(wo, m.innerAlpha, u0, u1, m.vndfExact != 0);
            wi = reflect(ab, wo, h);
        }
        wil = refract(ab, -wi, n, m.eta);   // total internal reflection can send it below
    }
    sraEval(m, wil, wol, r);
}

// EvalBsdf + GetOptData(kOptSamplingProbs) per material kind: :277-283 (Lambert),
// :809-817 (conductor), :1023-1031 with InitEvalContext :1123-1160 (dielectric)
// DA: also compute BsdfRec::dAtt
template <int K, bool DA = false>
PG3_DI void evalBsdfK(const DevMaterial &m, float3 wil, float3 wol, BsdfRec &r)
{
    r.wil = wil;
    r.compProb = 1.f;
    if (K == kMatLambert) {
        const bool valid = !(wil.z <= 0.f || wol.z <= 0.f);
        r.att = valid ? make_float3(m.r, m.g, m.b) * kPiInvF : f3(0.f);
        r.pdfW = cosHemispherePdf(wil.z);
        if (DA) r.dAtt = valid ? kPiInvF : 0.f;
    } else if (K == kMatGgxConductor) {
        const float3 h = halfwayReflection(wil, wol);
        const float D = ggxD(h, m.alpha);
        const float F = fresnelConductor(dot(h, wol), m.eta, m.absorb);
        r.att = condEval(m, wil, wol, h, F, D);
        r.pdfW = condPdf(m, wol, h, ggxDp(m, h, D));
        if (DA) r.dAtt = ggxDlnDGda(wil, wol, h, m.alpha);
    } else if (K == kMatGgxDielectric) {
        DielCtx c;
        const bool below = wol.z < 0.f;
        c.refl = (wil.z > 0.f) == (wol.z > 0.f);
        const float s = below ? -1.0f : 1.0f;
        c.wo = wol * s;
        c.wi = wil * s;
        c.etaS = below ? m.etaInv : m.eta;
        c.etaInvS = below ? m.eta : m.etaInv;
        c.m = c.refl ? halfwayReflection(c.wi, c.wo) : halfwayRefraction(c.wi, c.wo, c.etaInvS);
        c.D = ggxD(c.m, m.alpha);
        c.Dp = ggxDp(m, c.m, c.D);
        c.F = fresnelDielectric(dot(c.m, c.wo), c.etaS);
        r.att = dielEval(m, c);
        r.pdfW = dielPdf(m, c);
        if (DA) r.dAtt = ggxDlnDGda(c.wi, c.wo, c.m, m.alpha);
    } else if (K == kMatPhong) {
        r.att = phongEval(m, wil, wol);
        r.pdfW = phongPdf(m, wol, wil, phongDiffuseEst(m), phongGlossyEst(m, wol));
        if (DA) r.dAtt = 0.f;
    } else if (K == kMatSra) {
        sraEval(m, wil, wol, r);
        if (DA) r.dAtt = 0.f;
    } else {
        // smooth conductor / dielectric (:611-655): Dirac lobes only, no finite component
        r.att = f3(0.f);
        r.pdfW = 0.f;
        r.compProb = 0.f;
        if (DA) r.dAtt = 0.f;
    }
}
PG3_DI void evalBsdf(const DevMaterial &m, float3 wil, float3 wol, BsdfRec &r)
{
    switch (m.kind) {
    case kMatLambert: evalBsdfK<kMatLambert>(m, wil, wol, r); break;
    case kMatGgxConductor: evalBsdfK<kMatGgxConductor>(m, wil, wol, r); break;
    case kMatGgxDielectric: evalBsdfK<kMatGgxDielectric>(m, wil, wol, r); break;
    case kMatPhong: evalBsdfK<kMatPhong>(m, wil, wol, r); break;
    case kMatSra: evalBsdfK<kMatSra>(m, wil, wol, r); break;
    default: evalBsdfK<kMatSmoothConductor>(m, wil, wol, r); break;
    }
}

// SampleBsdf per material kind: :285-292 (Lambert), :819-851 (conductor), :1033-1100 (dielectric)
template <int K, bool DA = false>
PG3_DI void sampleBsdfK(const DevMaterial &m, float3 wol, float u0, float u1, float u2, BsdfRec &r)
{
    r.compProb = 1.f;
    if (K == kMatLambert) {
        r.wil = sampleCosHemisphere(u0, u1, r.pdfW);
        const bool valid = !(r.wil.z <= 0.f || wol.z <= 0.f);
        r.att = valid ? make_float3(m.r, m.g, m.b) * kPiInvF : f3(0.f);
        if (DA) r.dAtt = valid ? kPiInvF : 0.f;
    } else if (K == kMatGgxConductor) {
        // The value and pdf of the drawn direction come from the evaluation routine, so that
        // sampled and evaluated pdfs agree to the bit (the reference evaluates them from the
        // drawn microfacet normal, which equals the recomputed half vector up to rounding).
        const float3 h = sampleGgxVndf(wol, m.alphaS, u0, u1, m.vndfExact != 0);
        bool above;
        const float3 wil = reflect(above, wol, h);
        evalBsdfK<K, DA>(m, wil, wol, r);
        if (!above || wil.z < 0.0f) r.att = f3(0.f);
    } else if (K == kMatGgxDielectric) {
        DielCtx c;
        const bool below = wol.z < 0.f;
        const float s = below ? -1.0f : 1.0f;
        c.wo = wol * s;
        c.etaS = below ? m.etaInv : m.eta;
        c.etaInvS = below ? m.eta : m.etaInv;
        c.m = sampleGgxVndf(c.wo, m.alphaS, u0, u1, m.vndfExact != 0);
        c.F = fresnelDielectric(dot(c.m, c.wo), c.etaS);
        bool above;
        float cosAbs;
        if (u2 <= c.F) {
            c.wi = reflect(above, c.wo, c.m);
            cosAbs = c.wi.z;
        } else {
            c.wi = refract(above, c.wo, c.m, c.etaS);
            cosAbs = -c.wi.z;
        }
        // value and pdf (with the Fresnel component probability) from the evaluation routine
        const float3 wil = c.wi * s;
        evalBsdfK<K, DA>(m, wil, wol, r);
        if (!above || cosAbs < 0.0f) r.att = f3(0.f);
    } else if (K == kMatPhong) {
        // :437-495; u2 picks the component, (u0, u1) the direction
        if (DA) r.dAtt = 0.f;
        const float dEst = phongDiffuseEst(m), gEst = phongGlossyEst(m, wol);
        const float tot = dEst + gEst;
        if (tot < 1e-5f) {   // diffuse fallback of blockers
            r.att = f3(0.f);
            r.wil = sampleCosHemisphere(u0, u1, r.pdfW);
            return;
        }
        float pdfDummy;
        if (u2 * tot < dEst) {
            r.wil = sampleCosHemisphere(u0, u1, pdfDummy);
        } else {
            const float3 cs = samplePowerCosHemisphere(u0, u1, m.exponent);
            r.wil = toWorld(frameFromZ(reflectLocal(wol)), cs);
        }
        r.pdfW = phongPdf(m, wol, r.wil, dEst, gEst);
        r.att = (r.wil.z > 0.f) ? phongEval(m, r.wil, wol) : f3(0.f);
    } else if (K == kMatSra) {
        if (DA) r.dAtt = 0.f;
        sraSample(m, wol, u0, u1, u2, r);
    } else if (K == kMatSmoothConductor) {
        // :670-689: mirror direction, grey conductor Fresnel
        if (DA) r.dAtt = 0.f;
        r.wil = reflectLocal(wol);
        r.pdfW = infF();
        r.att = f3(fresnelConductor(r.wil.z, m.eta, m.absorb));
    } else {
        // :725-767: reflection with probability F (total internal reflection included), else
        // refraction with the radiance scaled by eta^2 or 1/eta^2
        if (DA) r.dAtt = 0.f;
        const float F = smoothDielectricFresnel(m, wol);
        float a;
        if (u2 <= F) {
            r.wil = reflectLocal(wol);
            a = F;
            r.compProb = F;
        } else {
            bool above;
            r.wil = refract(above, wol, make_float3(0.f, 0.f, 1.f), m.eta);
            a = (1.0f - F) * (above ? sqr(m.eta) : sqr(m.etaInv));
            r.compProb = 1.0f - F;
        }
        r.att = f3(a);
        r.pdfW = infF();
    }
}
PG3_DI void sampleBsdf(const DevMaterial &m, float3 wol, float u0, float u1, float u2, BsdfRec &r)
{
    switch (m.kind) {
    case kMatLambert: sampleBsdfK<kMatLambert>(m, wol, u0, u1, u2, r); break;
    case kMatGgxConductor: sampleBsdfK<kMatGgxConductor>(m, wol, u0, u1, u2, r); break;
    case kMatGgxDielectric: sampleBsdfK<kMatGgxDielectric>(m, wol, u0, u1, u2, r); break;
    case kMatPhong: sampleBsdfK<kMatPhong>(m, wol, u0, u1, u2, r); break;
    case kMatSmoothConductor: sampleBsdfK<kMatSmoothConductor>(m, wol, u0, u1, u2, r); break;
    case kMatSra: sampleBsdfK<kMatSra>(m, wol, u0, u1, u2, r); break;
    default: sampleBsdfK<kMatSmoothDielectric>(m, wol, u0, u1, u2, r); break;
    }
}
// The two Dirac materials share one wavefront bucket (kind read at run time).
template <bool DA = false>
PG3_DI void sampleBsdfSmooth(const DevMaterial &m, float3 wol, float u2, BsdfRec &r)
{
    if (m.kind == kMatSmoothConductor) sampleBsdfK<kMatSmoothConductor, DA>(m, wol, 0.f, 0.f, u2, r);
    else sampleBsdfK<kMatSmoothDielectric, DA>(m, wol, 0.f, 0.f, u2, r);
}

// Does the material take light samples? Every kind but the Dirac ones samples lights from its
// front side (kBsdfFrontSideLightSampling); smooth materials have no finite component
// (kBsdfNone, src/materials.hxx:604-609), so their light samples are always zero.
PG3_DI bool takesLightSamples(const DevMaterial &m)
{
    return m.kind != kMatSmoothConductor && m.kind != kMatSmoothDielectric;
}

// GetRRContinuationProb (src/materials.hxx:301-322, 542-570, 691-700, 770-775, 853-869, 1093-1098)
// clamped to [0, 0.997] (src/path_tracer.hxx:281-283). Phong and the smooth conductor depend on
// the outgoing direction; the others are constants of the record. KS: the kinds the caller can
// see (-1 any, 0-3 that kind, 4 the smooth pair).
template <int KS = -1>
PG3_DI float rrContinuation(const DevMaterial &m, float3 wol)
{
    if ((KS < 0 || KS == kMatPhong) && m.kind == kMatPhong) {
        const float3 gl = phongGlossy(m);
        const float g = (0.15f * luminance(gl) + 0.85f * maxc(gl)) * (0.5f + 0.5f * fmaxf(wol.z, 0.f));
        return fminf(clampf(m.rrProb + g, 0.f, 1.f), 0.997f);
    }
    if ((KS < 0 || KS == kMatSmoothConductor) && m.kind == kMatSmoothConductor)
        return clampf(fresnelConductor(wol.z, m.eta, m.absorb), 0.f, 0.997f);
    return m.rrProb;
}

// ------------------------------------------------------------------------------------------
// Geometry (src/scene_graph.hxx, src/scene.hxx:42-74)
// ------------------------------------------------------------------------------------------
struct Hit {
    float t;
    int prim;      // triangles [0, ntri), spheres ntri + i
};

// Signed-volume triangle test with plane distance, src/scene_graph.hxx:103-134.
PG3_DI bool hitTriangle(float4 a, float4 b, float4 c, float3 org, float3 dir, float tmin, float &tmax)
{
    const float3 ao = xyz(a) - org, bo = xyz(b) - org, co = xyz(c) - org;
    const float3 v0 = cross(co, bo), v1 = cross(bo, ao), v2 = cross(ao, co);
    const float d0 = dot(v0, dir), d1 = dot(v1, dir), d2 = dot(v2, dir);
    if ((d0 < 0.f && d1 < 0.f && d2 < 0.f) || (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f)) {
        const float3 n = make_float3(a.w, b.w, c.w);
#if PG3_FAST_HIT_DIV
        const float dist = __fdividef(dot(n, ao), dot(n, dir));
#else
        const float dist = dot(n, ao) / dot(n, dir);
#endif
        if ((dist > tmin) & (dist < tmax)) { tmax = dist; return true; }
    }
    return false;
}

// Sphere: the reference solves the quadratic with a double-precision discriminant and
// Muller's second root (src/scene_graph.hxx:176-245). Here in fp32, with the discriminant
// in the cancellation-free form r^2 - |o - (o.d)d|^2 (Haines et al., "Precision
// Improvements for Ray/Sphere Intersection", Ray Tracing Gems 2019) and the same root
// selection.
PG3_DI bool hitSphere(float4 s, float3 org, float3 dir, float tmin, float &tmax)
{
    const float3 o = org - xyz(s);
    const float A = dot(dir, dir);
#if PG3_FAST_SPHERE_DIV
    const float invA = __fdividef(1.f, A);
    const float b = dot(dir, o) * invA;               // half of B / A
#else
    const float invA = 1.f / A;
    const float b = dot(dir, o) / A;                  // half of B / A
#endif
    const float3 l = o - dir * b;
    const float disc = s.w * s.w - dot(l, l);
    if (disc < 0.f) return false;
    const float C = dot(o, o) - s.w * s.w;
    const float q = (b >= 0.f) ? (-b - sqrtf(disc * invA)) : (-b + sqrtf(disc * invA));
    float t0 = q;
#if PG3_FAST_SPHERE_DIV
    float t1 = (fabsf(q) > 0.1f) ? __fdividef(C, A * q) : t0;
#else
    float t1 = (fabsf(q) > 0.1f) ? (C / (A * q)) : t0;
#endif
    if (t0 > t1) { const float t = t0; t0 = t1; t1 = t; }
    if (t0 > tmin && t0 < tmax) { tmax = t0; return true; }
    if (t1 > tmin && t1 < tmax) { tmax = t1; return true; }
    return false;
}

// Closest hit over the primitive list in list order (src/scene_graph.hxx:47-57).
PG3_DI bool intersectList(const SceneView &S, float3 org, float3 dir, float tmin, Hit &h)
{
    float tmax = 1e36f;
    int prim = -1;
    for (uint32_t i = 0; i < S.ntri; ++i) {
        const float4 a = __ldg(&S.tri[3 * i]), b = __ldg(&S.tri[3 * i + 1]), c = __ldg(&S.tri[3 * i + 2]);
        if (hitTriangle(a, b, c, org, dir, tmin, tmax)) prim = (int)i;
    }
    for (uint32_t i = 0; i < S.nsph; ++i)
        if (hitSphere(__ldg(&S.sph[i]), org, dir, tmin, tmax)) prim = (int)(S.ntri + i);
    h.t = tmax;
    h.prim = prim;
    return prim >= 0;
}

// Any hit (src/scene.hxx:61-74): origin pushed by kEpsRay, tmax = dist - 2 kEpsRay.
PG3_DI bool occludedList(const SceneView &S, float3 pt, float3 dir, float dist)
{
    const float3 org = pt + dir * kEpsRay;
    float tmax = dist - 2.f * kEpsRay;
    for (uint32_t i = 0; i < S.ntri; ++i) {
        const float4 a = __ldg(&S.tri[3 * i]), b = __ldg(&S.tri[3 * i + 1]), c = __ldg(&S.tri[3 * i + 2]);
        if (hitTriangle(a, b, c, org, dir, 0.f, tmax)) return true;
    }
    for (uint32_t i = 0; i < S.nsph; ++i)
        if (hitSphere(__ldg(&S.sph[i]), org, dir, 0.f, tmax)) return true;
    return false;
}

// Hit attributes: geometric normal (triangle) or outward normal (sphere), material.
// After the 3 float4 per triangle: per triangle (normal, material as int bits), one load per hit.
PG3_DI const float4 *triShade(const SceneView &S) { return S.tri + 3 * (size_t)S.ntri; }

PG3_DI void hitAttributes(const SceneView &S, const Hit &h, float3 org, float3 dir, float3 &pt, float3 &n, int &mat)
{
    pt = org + dir * h.t;
    if ((uint32_t)h.prim < S.ntri) {
        const float4 r = __ldg(&triShade(S)[h.prim]);
        n = xyz(r);
        mat = __float_as_int(r.w);
    } else {
        const uint32_t i = (uint32_t)h.prim - S.ntri;
        const float4 s = __ldg(&S.sph[i]);
        n = normalize((org - xyz(s)) + f3(h.t) * dir);
        mat = __ldg(&S.sphMat[i]);
    }
}

// ------------------------------------------------------------------------------------------
// Area lights (src/lights.hxx:55-229)
// ------------------------------------------------------------------------------------------
PG3_DI float3 lightRadiance(const DevAreaLight &L) { return make_float3(L.e1_r.w, L.e2_g.w, L.n_b.w); }

// ComputeSample (:171-219) for a front-side-sampling material
PG3_DI void areaComputeSample(const DevAreaLight &L, float3 pt, float3 sp, float3 sn, float3 &wig, float &dist,
                              float3 &smp, float &pdfW)
{
    wig = sp - pt;
    const float d2 = dot(wig, wig);
    dist = sqrtf(d2);
    wig = wig / dist;
    const float cosOut = -dot(xyz(L.n_b), wig);
    const float cosIn = fmaxf(dot(sn, wig), 0.0f);
    smp = (cosOut > 0.f) ? lightRadiance(L) * cosIn : f3(0.f);
    pdfW = fmaxf(L.p0_invArea.w * (d2 / fabsf(cosOut)), kEpsDist);
}
// EstimateContribution (:133-167)
PG3_DI float areaEstimate(const DevAreaLight &L, float3 pt, float3 sn)
{
    const float3 p0 = xyz(L.p0_invArea), e1 = xyz(L.e1_r), e2 = xyz(L.e2_g);
    const float3 pts[4] = {p0, p0 + e1, p0 + e2, p0 + 0.33f * e1 + 0.33f * e2};
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float3 w, s; float d, p;
        areaComputeSample(L, pt, pts[i], sn, w, d, s, p);
        acc += luminance(s) / p;
    }
    return acc / 4.f;
}
// SampleIllumination (:114-130): uniform point via the square-root barycentric map
// (src/sampling.hxx:66-75, src/geom.hxx:675-705, 820-833)
PG3_DI void areaSample(const DevAreaLight &L, float3 pt, float3 sn, float u0, float u1, float3 &wig, float &dist,
                       float3 &smp, float &pdfW)
{
    const float3 p0 = xyz(L.p0_invArea), e1 = xyz(L.e1_r), e2 = xyz(L.e2_g);
    const float xs = sqrtf(u0);
    const float bx = 1.f - xs, by = u1 * xs, bz = 1.0f - bx - by;
    const float3 sp = bx * p0 + by * (p0 + e1) + bz * (p0 + e2);
    areaComputeSample(L, pt, sp, sn, wig, dist, smp, pdfW);
}
// GetEmmision with pdf (:78-101)
PG3_DI float3 areaEmission(const DevAreaLight &L, float3 lightPt, float wolZ, float3 surfPt, float &pdf)
{
    float3 w = lightPt - surfPt;
    const float d2 = dot(w, w);
    w = w / sqrtf(d2);
    pdf = fmaxf(L.p0_invArea.w * (d2 / fabsf(dot(xyz(L.n_b), w))), kEpsDist);
    return (wolZ <= 0.f) ? f3(0.f) : lightRadiance(L);
}

// ------------------------------------------------------------------------------------------
// Point lights (src/lights.hxx:232-343): entries of the light table marked by a negative 1/area
// ------------------------------------------------------------------------------------------
PG3_DI bool isPointLight(const DevAreaLight &L) { return L.p0_invArea.w < 0.f; }
// ComputeIllumination (:300-337) for a front-side-sampling material: I cos / d^2, pdf infinite
PG3_DI void pointSample(const DevAreaLight &L, float3 pt, float3 sn, float3 &wig, float &dist, float3 &smp,
                        float &pdfW)
{
    wig = xyz(L.p0_invArea) - pt;
    const float d2 = dot(wig, wig);
    dist = sqrtf(d2);
    wig = wig / dist;
    const float cosIn = fmaxf(dot(sn, wig), 0.0f);
    smp = (cosIn > 0.f) ? lightRadiance(L) * cosIn / d2 : f3(0.f);
    pdfW = infF();
}
// A light-table entry: sample (area: :114-131) and contribution estimate (area: :133-167,
// point: the luminance of its only sample, :279-291)
PG3_DI void tableSample(const DevAreaLight &L, float3 pt, float3 sn, float u0, float u1, float3 &wig, float &dist,
                        float3 &smp, float &pdfW)
{
    if (isPointLight(L)) pointSample(L, pt, sn, wig, dist, smp, pdfW);
    else areaSample(L, pt, sn, u0, u1, wig, dist, smp, pdfW);
}
PG3_DI float tableEstimate(const DevAreaLight &L, float3 pt, float3 sn)
{
    if (isPointLight(L)) {
        float3 w, s;
        float d, p;
        pointSample(L, pt, sn, w, d, s, p);
        return luminance(s);
    }
    return areaEstimate(L, pt, sn);
}

// ------------------------------------------------------------------------------------------
// Environment map (src/em_image.hxx, src/filter.hxx, src/distribution.hxx,
// src/em_simple_spherical_sampler.hxx, src/em_cosine_sampler.hxx)
// ------------------------------------------------------------------------------------------
// NormalizeImgCoords (src/em_image.hxx:269-302)
PG3_DI void emWrap(const SceneView &S, int x, int y, uint32_t &ox, uint32_t &oy)
{
    const int W = (int)S.emW, H = (int)S.emH;
    int rx = x, ry = y;
    if (y >= H) { rx = x + W / 2; ry = H - 1; }
    else if (y < 0) { rx = x + W / 2; ry = 0; }
    int m = rx % W;
    if (m < 0) m += W;
    ox = (uint32_t)m;
    oy = (uint32_t)ry;
}
// Bilinear (tent) lookup, src/em_image.hxx:95-143 + src/filter.hxx:22-31
PG3_DI float3 emEvaluate(const SceneView &S, float u, float v)
{
    const float xf = u * (float)S.emW, yf = v * (float)S.emH;
    const int cx = (int)(xf + 0.5f), cy = (int)(yf + 0.5f);
    const int x0 = cx - 1, y0 = cy - 1;
    const float xl = xf - ((float)x0 + 0.5f), yl = yf - ((float)y0 + 0.5f);
    uint32_t ax, ay, bx, by;
    emWrap(S, x0, y0, ax, ay);
    emWrap(S, cx, cy, bx, by);
    const float3 a = xyz(__ldg(&S.em[ay * S.emW + ax])), b = xyz(__ldg(&S.em[ay * S.emW + bx]));
    const float3 c = xyz(__ldg(&S.em[by * S.emW + ax])), d = xyz(__ldg(&S.em[by * S.emW + bx]));
    const float3 top = (1.f - xl) * a + xl * b;
    const float3 bot = (1.f - xl) * c + xl * d;
    return (1.f - yl) * top + yl * bot;
}
PG3_DI float3 emEvaluateDir(const SceneView &S, float3 d)
{
    float u, v;
    dir2LatLong(d, u, v);
    return emEvaluate(S, u, v);
}
PG3_DI float sinMidTheta(const SceneView &S, uint32_t row) { return sinf(kPiF * (row + 0.5f) / S.emH); }

// upper_bound over cdf[0..n]: first index with cdf[i] > t (n+1 entries)
PG3_DI uint32_t upperBound(const float *cdf, uint32_t n1, float t)
{
    uint32_t lo = 0, len = n1;
    while (len > 0) {
        const uint32_t half = len >> 1;
        const uint32_t mid = lo + half;
        if (!(t < __ldg(&cdf[mid]))) { lo = mid + 1; len = len - half - 1; }
        else len = half;
    }
    return lo;
}
// Distribution1D::SampleContinuous, src/distribution.hxx:404-461 (the hierarchical search
// finds the same segment as upper_bound over the full CDF)
PG3_DI void cdfSample(const float *cdf, uint32_t n, float u, float &x, uint32_t &segm, float &pdf)
{
    const float t = u * 0.999999f;
    int s = (int)upperBound(cdf, n + 1, t) - 1;
    s = min(max(s, 0), (int)n - 1);
    segm = (uint32_t)s;
    const float c0 = __ldg(&cdf[segm]), c1 = __ldg(&cdf[segm + 1]);
    const float p = c1 - c0;
    const float off = (t - c0) / p;
    pdf = p * n;
    x = (segm + off) / n;
}
// EnvironmentMapSimpleSphericalSampler::PdfW, src/em_simple_spherical_sampler.hxx:85-97
PG3_DI float emCdfPdf(const SceneView &S, float3 dir)
{
    float u, v;
    dir2LatLong(dir, u, v);
    const uint32_t iu = min((uint32_t)(u * S.emW), S.emW - 1u);
    const uint32_t iv = min((uint32_t)(v * S.emH), S.emH - 1u);
    const float *row = S.emCond + (size_t)iv * (S.emW + 1);
    const float pc = (__ldg(&row[iu + 1]) - __ldg(&row[iu])) * S.emW;
    const float pm = (__ldg(&S.emMarg[iv + 1]) - __ldg(&S.emMarg[iv])) * S.emH;
    return pc * pm * (1.0f / (2.0f * kPiF * kPiF)) / sinMidTheta(S, iv);
}
// SampleImpl, src/em_simple_spherical_sampler.hxx:27-82
PG3_DI void emCdfSample(const SceneView &S, float3 sn, float u0, float u1, float3 &wig, float &pdfW, float3 &radCos)
{
    float v, u, mp, cp;
    uint32_t sy, sx;
    cdfSample(S.emMarg, S.emH, u0, v, sy, mp);
    cdfSample(S.emCond + (size_t)sy * (S.emW + 1), S.emW, u1, u, sx, cp);
    wig = latLong2Dir(u, v);
    pdfW = mp * cp * (1.0f / (2.0f * kPiF * kPiF)) / sinMidTheta(S, sy);
    const float3 L = emEvaluate(S, u, v);
    const float c = dot(wig, sn);
    radCos = (c > 0.0f) ? L * fabsf(c) : f3(0.f);
}

}  // namespace pg3
