// CPU oracle for the path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain scalar C++, the
// algorithm of the reference renderer's NEE+MIS path tracer so that tests can
// check the CUDA kernels against it. Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load it; the product library never does.
//
// Every function cites the reference file:line it follows (paths relative to
// the reference project). Differences from the reference, all deliberate:
//   * random numbers come from Philox4x32-10 (Salmon et al., SC'11) keyed by
//     (seed) and counted by (pixel, sample, vertex, group) instead of one
//     mt19937_64 stream per renderer (src/rng.hxx:16-61). The CUDA path draws
//     the same numbers, so the two can be compared path by path; against the
//     reference itself the comparison is statistical.
//   * the splitting budget is 1, the light/BSDF sample ratio 1 and indirect
//     clipping off (the reference's unbiased setting "-sb 1 -iic 0").
//   * optional Russian roulette from a given path length on while a maximum
//     path length is also set (rr_min_path_length > 0); with 0 the reference's
//     rule applies (roulette only when max_path_length == 0,
//     src/path_tracer.hxx:267-286).
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -shared -fPIC
//        pt_oracle.cpp -o _build/libpg3oracle.so   (done by oracle/build.py)

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace pg3o {

// --------------------------------------------------------------------------------------------
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw 2011), checked against the
// published known-answer vectors by tests/test_oracle.py.
// --------------------------------------------------------------------------------------------
static inline void Philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0; c[1] = (uint32_t)p1; c[2] = n2; c[3] = (uint32_t)p0;
    }
}

static inline float U01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Four uniforms for one (pixel, sample, vertex, group) counter.
struct Rand4 { float v[4]; };
static inline Rand4 Draw(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t vertex, uint32_t group)
{
    uint32_t c[4] = {pixel, sample, vertex, group};
    Philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    Rand4 r;
    for (int i = 0; i < 4; ++i) r.v[i] = U01(c[i]);
    return r;
}

// --------------------------------------------------------------------------------------------
// Vectors, spectra, frames (src/math.hxx, src/spectrum.hxx)
// --------------------------------------------------------------------------------------------
struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit V3(float a) : x(a), y(a), z(a) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
static inline V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
static inline float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 Cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline float Len(V3 a) { return std::sqrt(Dot(a, a)); }
static inline V3 Normalize(V3 a) { return a / Len(a); }
static inline float MaxC(V3 a) { return std::max(a.x, std::max(a.y, a.z)); }
static inline bool IsZero(V3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
// sRGB luminance (src/spectrum.hxx:74-80)
static inline float Luminance(V3 a) { return 0.212671f * a.x + 0.715160f * a.y + 0.072169f * a.z; }

const float kPiF = 3.14159265358979f;                 // src/math.hxx:12
const float kPiInvF = 1.f / kPiF;
const float kTinyF = 9.5367431640625E-7f;             // src/math.hxx:46
const float kEpsRay = 1e-3f;                          // src/geom.hxx:16
const float kEpsDist = 1e-6f;                         // src/geom.hxx:27
const float kInf = std::numeric_limits<float>::infinity();
static inline bool IsTiny(float x) { return std::fabs(x) < kTinyF; }
static inline float Sqr(float x) { return x * x; }
static inline float SafeSqrt(float x) { return std::sqrt(std::max(0.f, x)); }
static inline float Clampf(float v, float a, float b) { return std::min(std::max(v, a), b); }

// src/math.hxx:955-1013
struct Frame {
    V3 mX{1, 0, 0}, mY{0, 1, 0}, mZ{0, 0, 1};
    void SetFromZ(V3 z)
    {
        mZ = z;
        V3 tmpX = (std::fabs(mZ.x) > 0.99f) ? V3(0, 1, 0) : V3(1, 0, 0);
        mY = Normalize(Cross(mZ, tmpX));
        mX = Cross(mY, mZ);
    }
    V3 ToWorld(V3 a) const { return mX * a.x + mY * a.y + mZ * a.z; }
    V3 ToLocal(V3 a) const { return V3(Dot(a, mX), Dot(a, mY), Dot(a, mZ)); }
    V3 Normal() const { return mZ; }
};

// src/geom.hxx:22-25
static inline float EpsRayCos(float c) { return (1.f + 2.f * (1.f - c)) * kEpsRay; }

// src/geom.hxx:29-48
static inline V3 CreateDirection(float sinT, float cosT, float sinP, float cosP)
{
    return V3(sinT * cosP, sinT * sinP, cosT);
}

// src/geom.hxx:65-73
static inline V3 LatLong2Dir(float u, float v)
{
    const float phi = -(u - 0.5f) * 2 * kPiF;
    const float theta = v * kPiF;
    return CreateDirection(std::sin(theta), std::cos(theta), std::sin(phi), std::cos(phi));
}

// src/geom.hxx:77-95
static inline void Dir2LatLong(V3 d, float &u, float &v)
{
    const float phi = -std::atan2(d.y, d.x);
    const float theta = std::acos(d.z);
    u = Clampf(0.5f + phi * 0.5f * kPiInvF, 0.f, 1.f);
    v = Clampf(theta * kPiInvF, 0.f, 1.f);
}

// src/geom.hxx:97-107
static inline float TanThetaSqr(V3 d)
{
    const float c2 = d.z * d.z;
    const float s2 = 1.f - c2;
    if (s2 <= 0.0f) return 0.0f;
    return s2 / c2;
}

// src/geom.hxx:116-133
static inline V3 Reflect(bool &above, V3 in, V3 n)
{
    const float dot = Dot(in, n);
    above = dot > 0.0f;
    return (2.0f * dot) * n - in;
}

// src/geom.hxx:145-179
static inline V3 Refract(bool &inAbove, V3 in, V3 n, float eta)
{
    const float cosI = Dot(in, n);
    inAbove = cosI > 0.0f;
    if (inAbove) eta = 1.0f / eta;
    const float cosT2 = 1 - (1 - cosI * cosI) * (eta * eta);
    if (cosT2 < 0.0f) {
        bool dummy;
        return Reflect(dummy, in, n);
    }
    float cosT = std::sqrt(cosT2);
    cosT = (cosI > 0.0f) ? -cosT : cosT;
    return n * (cosI * eta + cosT) - in * eta;
}

// --------------------------------------------------------------------------------------------
// Sampling (src/sampling.hxx)
// --------------------------------------------------------------------------------------------
// src/sampling.hxx:289-306
static inline V3 SampleCosHemisphereW(float u0, float u1, float *pdf)
{
    const float t1 = 2.f * kPiF * u0;
    const float t2 = std::sqrt(1.f - u1);
    V3 r(std::cos(t1) * t2, std::sin(t1) * t2, std::sqrt(u1));
    if (pdf) *pdf = r.z * kPiInvF;
    return r;
}
// src/sampling.hxx:308-311
static inline float CosHemispherePdfW(float z) { return std::max(0.f, z) * kPiInvF; }
// src/sampling.hxx:250-285
static inline V3 SamplePowerCosHemisphereW(float u0, float u1, float power)
{
    const float term1 = 2.f * kPiF * u0;
    const float term2 = std::pow(u1, 1.f / (power + 1.f));
    const float term3 = std::sqrt(1.f - term2 * term2);
    return V3(std::cos(term1) * term3, std::sin(term1) * term3, term2);
}
static inline float PowerCosHemispherePdfW(V3 local, float power)
{
    const float cosTheta = std::max(0.f, local.z);
    return (power + 1.f) * std::pow(cosTheta, power) * (kPiInvF * 0.5f);
}
// src/geom.hxx:110-113
static inline V3 ReflectLocal(V3 v) { return V3(-v.x, -v.y, v.z); }

// src/sampling.hxx:326-343
static inline V3 SampleCosSphereParamPdfW(float u0, float u1, float u2, bool upper, bool lower, float &pdf)
{
    V3 w = SampleCosHemisphereW(u0, u1, &pdf);
    if (upper && lower) {
        if (u2 < 0.5f) w = w * -1.0f;
        pdf *= 0.5f;
    } else if (lower) {
        w = w * -1.0f;
    }
    return w;
}
// src/sampling.hxx:345-361
static inline float CosSpherePdfW(bool upper, bool lower, V3 local)
{
    if ((!upper && local.z > 0.f) || (!lower && local.z < 0.f)) return 0.f;
    float pdf = CosHemispherePdfW(std::fabs(local.z));
    if (upper && lower) pdf *= 0.5f;
    return pdf;
}

// Uniform triangle point: src/sampling.hxx:66-75, src/geom.hxx:675-705, 820-833
static inline V3 SampleUniformTriangle(V3 p0, V3 p1, V3 p2, float u0, float u1)
{
    const float xs = std::sqrt(u0);
    const float bx = 1.f - xs, by = u1 * xs;
    const float bz = 1.0f - bx - by;
    return bx * p0 + by * p1 + bz * p2;
}

// --------------------------------------------------------------------------------------------
// Fresnel (src/physics.hxx)
// --------------------------------------------------------------------------------------------
// src/physics.hxx:5-47
static float FresnelDielectric(float cosI, float etaAbs)
{
    if (etaAbs < 0) return 1.f;
    float eta;
    if (cosI < 0.f) { cosI = -cosI; eta = etaAbs; }
    else eta = 1.f / etaAbs;
    const float sinT2 = Sqr(eta) * (1.f - Sqr(cosI));
    const float cosT = SafeSqrt(1.f - sinT2);
    if (sinT2 > 1.0f) return 1.0f;
    const float t2 = eta * cosI;
    const float rs = Sqr((t2 - cosT) / (t2 + cosT));
    const float t1 = eta * cosT;
    const float rp = Sqr((cosI - t1) / (cosI + t1));
    return 0.5f * (rp + rs);
}

// Mitsuba variant selected by src/hard_config.hxx:15; src/physics.hxx:50-148
static float FresnelConductor(float cosI, float eta, float k)
{
    if (cosI < -0.00001f) return 0.0f;
    cosI = Clampf(cosI, 0.0f, 1.0f);
    const float c2 = cosI * cosI;
    const float s2 = 1 - c2;
    const float s4 = s2 * s2;
    const float eta2 = eta * eta, k2 = k * k;
    const float temp1 = eta2 - k2 - s2;
    const float a2pb2 = SafeSqrt(temp1 * temp1 + 4 * k2 * eta2);
    const float a = SafeSqrt(0.5f * (a2pb2 + temp1));
    const float term1 = a2pb2 + c2;
    const float term2 = 2 * a * cosI;
    const float Rs2 = (term1 - term2) / (term1 + term2);
    const float term3 = a2pb2 * c2 + s4;
    const float term4 = term2 * s2;
    const float Rp2 = Rs2 * (term3 - term4) / (term3 + term4);
    return 0.5f * (Rp2 + Rs2);
}

// --------------------------------------------------------------------------------------------
// Microfacet GGX (src/microfacet.hxx)
// --------------------------------------------------------------------------------------------
// src/microfacet.hxx:16-31
static inline float ReflectionJacobian(V3 wo, V3 m)
{
    const float c = std::max(Dot(m, wo), 0.000001f);
    return 1.0f / (4.0f * c);
}
// src/microfacet.hxx:34-56
static inline float RefractionJacobian(V3 wi, V3 wo, V3 m, float etaOutIn)
{
    const float cOM = Dot(m, wo), cIM = Dot(m, wi);
    const float den = Sqr(etaOutIn * cIM + cOM);
    return std::fabs(cOM) / std::max(den, 0.000001f);
}
// src/microfacet.hxx:60-84
static inline V3 HalfwayReflection(V3 wi, V3 wo)
{
    V3 h = wi + wo;
    const float l = Len(h);
    if (IsTiny(l)) h = V3(0, 0, 1);
    else h = h / l;
    return h * ((h.z >= 0.0f) ? 1.0f : -1.0f);
}
// src/microfacet.hxx:88-123
static inline V3 HalfwayRefraction(V3 wi, V3 wo, float etaInOut)
{
    V3 h = wi + wo * etaInOut;
    const float l = Len(h);
    if (IsTiny(l)) h = wi;
    else h = h / l;
    return h * ((h.z >= 0.0f) ? 1.0f : -1.0f);
}
// src/microfacet.hxx:505-527
static inline float DistributionGgx(V3 m, float a)
{
    if (m.z <= 0.f) return 0.0f;
    const float a2 = a * a;
    const float c2 = m.z * m.z;
    const float t2 = TanThetaSqr(m);
    const float temp2 = c2 * (a2 + t2);
    return a2 / (kPiF * temp2 * temp2);
}
// src/microfacet.hxx:529-554
static inline float SmithG1(V3 v, V3 m, float a)
{
    if (m.z <= 0) return 0.0f;
    const float cVM = Dot(v, m);
    if ((v.z * cVM) < 0.0f) return 0.0f;
    const float root = std::sqrt(1.0f + a * a * TanThetaSqr(v));
    return 2.0f / (1.0f + root);
}
// src/microfacet.hxx:610-673
static void SampleGgxP11(float &sx, float &sy, float thetaI, float u0, float u1)
{
    if (thetaI < 0.0001f) {
        const float ux = std::min(u0, 0.9999f);
        const float r = SafeSqrt(ux / (1 - ux));
        const float phi = 2 * kPiF * u1;
        sx = r * std::cos(phi);
        sy = r * std::sin(phi);
        return;
    }
    const float tanI = std::tan(thetaI);
    const float tanIInv = 1.0f / tanI;
    const float G1 = 2.0f / (1.0f + SafeSqrt(1.0f + 1.0f / (tanIInv * tanIInv)));
    float A = 2.0f * u0 / G1 - 1.0f;
    if (std::fabs(A) == 1.0f) A -= (std::signbit(A) ? -1.f : 1.f) * 1e-4f;
    const float B = tanI;
    const float tmp = 1.0f / (A * A - 1.0f);
    const float D = SafeSqrt(B * B * tmp * tmp - (A * A - B * B) * tmp);
    const float x1 = B * tmp - D, x2 = B * tmp + D;
    sx = (A < 0.0f || x2 > (1.0f / tanI)) ? x1 : x2;
    float sign, ys;
    if (u1 > 0.5f) { sign = 1.0f; ys = 2.0f * (u1 - 0.5f); }
    else { sign = -1.0f; ys = 2.0f * (0.5f - u1); }
    const float z = (ys * (ys * (ys * -(float)0.365728915865723 + (float)0.790235037209296) -
                           (float)0.424965825137544) + (float)0.000152998850436920) /
                    (ys * (ys * (ys * (ys * (float)0.169507819808272 - (float)0.397203533833404) -
                                 (float)0.232500544458471) + (float)1) - (float)0.539825872510702);
    sy = sign * z * std::sqrt(1.0f + sx * sx);
}
// src/microfacet.hxx:678-729
static V3 SampleGgxVisibleNormals(V3 wo, float a, float u0, float u1)
{
    const V3 ws = Normalize(V3(wo.x * a, wo.y * a, std::max(wo.z, 0.0f)));
    float theta = 0.0f, phi = 0.0f;
    if (ws.z < 0.999f) {
        theta = std::acos(ws.z);
        phi = std::atan2(ws.y, ws.x);
    }
    const float sp = std::sin(phi), cp = std::cos(phi);
    float sx, sy;
    SampleGgxP11(sx, sy, theta, u0, u1);
    const float rx = sx * cp - sy * sp;
    const float ry = sx * sp + sy * cp;
    const float x = rx * a, y = ry * a;
    const float inv = 1.0f / Len(V3(x, y, 1.0f));
    return V3(-x * inv, -y * inv, inv);
}
// Exact visible-normal sampling, Heitz, "Sampling the GGX Distribution of Visible Normals"
// (JCGT 2018): same density as SampleGgxVisibleNormals above, without its rational fit.
static V3 SampleGgxVndfExact(V3 wo, float a, float u0, float u1)
{
    const V3 vh = Normalize(V3(a * wo.x, a * wo.y, std::max(wo.z, 0.0f)));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const V3 t1 = lensq > 0.f ? V3(-vh.y, vh.x, 0.f) / std::sqrt(lensq) : V3(1.f, 0.f, 0.f);
    const V3 t2 = Cross(vh, t1);
    const float r = std::sqrt(u0);
    const float phi = 2.f * kPiF * u1;
    const float p1 = r * std::cos(phi);
    const float s = 0.5f * (1.f + vh.z);
    const float p2 = (1.f - s) * std::sqrt(std::max(0.f, 1.f - p1 * p1)) + s * (r * std::sin(phi));
    const V3 nh = t1 * p1 + t2 * p2 + vh * std::sqrt(std::max(0.f, 1.f - p1 * p1 - p2 * p2));
    return Normalize(V3(a * nh.x, a * nh.y, std::max(1e-6f, nh.z)));
}
static bool g_vndfExact = true;   // false: the reference's fitted routine
static V3 SampleVndf(V3 wo, float a, float u0, float u1)
{
    return g_vndfExact ? SampleGgxVndfExact(wo, a, u0, u1) : SampleGgxVisibleNormals(wo, a, u0, u1);
}

// src/microfacet.hxx:732-756
static inline float GgxPdfVisibleNormals(V3 wo, V3 h, float D, float a)
{
    if (h.z <= 0.f) return 0.0f;
    const float G1 = SmithG1(wo, h, a);
    const float cOM = Dot(h, wo);
    const float cO = std::max(wo.z, 0.00001f);
    return (G1 * std::fabs(cOM) * D) / cO;
}

// --------------------------------------------------------------------------------------------
// Materials (src/materials.hxx)
// --------------------------------------------------------------------------------------------
enum { kLambert = 0, kGgxConductor = 1, kGgxDielectric = 2, kPhong = 3, kSmoothConductor = 4, kSmoothDielectric = 5,
       kSra = 6 };

struct MatRecord {   // src/materials.hxx:48-207 (the fields the path tracer reads)
    V3 wol, wil, attenuation;
    float pdfW = 0.f, compProb = 0.f;
    bool IsBlocker() const { return MaxC(attenuation) * std::fabs(wil.z) <= 1e-5; }   // :63-67
    float CosAbs() const { return std::fabs(wil.z); }
    bool IsFinite() const { return pdfW != kInf; }
};

struct Material {
    int kind = kLambert;
    V3 reflectance;            // Lambert reflectance; Phong diffuse reflectance (mDiffuseReflectance)
    V3 glossy;                 // Phong mPhongReflectance
    float exponent = 1.f;      // Phong mPhongExponent
    // SRA layered (:1304-1324): this record is the outer GGX dielectric (alpha, eta, etaInv); the
    // inner Lambert (reflectance) or GGX conductor (innerAlpha, innerEta, absorb); the medium
    int innerKind = kLambert;
    float innerAlpha = 0.1f, innerEta = 1.f;
    V3 mediumAtt;
    float mediumThickness = 0.f;
    float alpha = 0.1f, eta = 1.f, etaInv = 1.f, absorb = 0.f;
    // Sampling overrides (not in the reference): the GGX roughness that sampling and pdfs use and
    // the roulette continuation probability, for finite differences that hold sampling fixed
    // while the BSDF value changes. Negative: follow alpha / the reflectance.
    float alphaSample = -1.f, rrOverride = -1.f;
    float AlphaS() const { return alphaSample >= 0.f ? alphaSample : alpha; }

    // src/materials.hxx:262-266, 791-806, 996-1021
    static Material Lambert(V3 r) { Material m; m.kind = kLambert; m.reflectance = r; return m; }
    static Material Conductor(float a, float n, float no, float k)
    {
        Material m; m.kind = kGgxConductor;
        m.eta = IsTiny(no) ? 1.0f : n / no;
        m.absorb = k;
        m.alpha = Clampf(a, 0.001f, 1.0f);
        return m;
    }
    static Material Dielectric(float a, float n, float no)
    {
        Material m; m.kind = kGgxDielectric;
        if (!IsTiny(no)) { m.eta = n / no; m.etaInv = no / n; }
        m.alpha = Clampf(a, 0.001f, 1.0f);
        return m;
    }

    // PhongMaterial (:366-381), with the diffuse part as the material holds it
    static Material Phong(V3 d, V3 g, float e)
    {
        Material m; m.kind = kPhong; m.reflectance = d; m.glossy = g; m.exponent = e;
        return m;
    }
    static Material SmoothConductor(float n, float no, float k)   // :658-668
    {
        Material m; m.kind = kSmoothConductor;
        m.eta = IsTiny(no) ? 1.0f : n / no;
        m.absorb = k;
        return m;
    }
    static Material Sra(const Material &outer, const Material &inner, V3 att, float thickness)
    {
        Material m = outer;
        m.kind = kSra;
        m.innerKind = inner.kind;
        m.reflectance = inner.reflectance;
        m.innerAlpha = inner.alpha;
        m.innerEta = inner.eta;
        m.absorb = inner.absorb;
        m.mediumAtt = att;
        m.mediumThickness = thickness;
        return m;
    }
    static Material SmoothDielectric(float n, float no)   // :713-727
    {
        Material m; m.kind = kSmoothDielectric;
        m.eta = IsTiny(no) ? 1.0f : n / no;
        m.etaInv = IsTiny(n) ? 1.0f : no / n;
        return m;
    }

    // Light-sampling sides (:36-45): front side for all but the smooth materials, whose Dirac
    // lobes take no light samples (kBsdfNone, :604-609) -- their light samples are all zero.
    bool SamplesLights() const { return kind != kSmoothConductor && kind != kSmoothDielectric; }

    bool IsReflectanceZero() const   // :321-324, 572-575, 702-705, 777-780, 873-876, 1110-1113
    {
        if (kind == kLambert) return IsZero(reflectance);
        if (kind == kPhong) return IsZero(reflectance) && IsZero(glossy);
        return false;
    }

    // :300-319, 542-570, 691-700, 770-775, 853-858, 1102-1108
    float RRContinuationProb(V3 wol) const
    {
        if (rrOverride >= 0.f) return rrOverride;
        if (kind == kLambert) {
            const float p = 0.15f * Luminance(reflectance) + 0.85f * MaxC(reflectance);
            return Clampf(p, 0.f, 1.f);
        }
        if (kind == kPhong) {
            const float d = 0.15f * Luminance(reflectance) + 0.85f * MaxC(reflectance);
            const float g = (0.15f * Luminance(glossy) + 0.85f * MaxC(glossy)) * (0.5f + 0.5f * std::max(wol.z, 0.f));
            return Clampf(d + g, 0.f, 1.f);
        }
        if (kind == kSmoothConductor) return FresnelConductor(wol.z, eta, absorb);
        return 1.0f;
    }

    // ---- SRA layered material (:1304-1566)
    V3 BeerLambert(float len) const   // Physics::BeerLambert
    {
        return V3(std::exp(-(mediumAtt.x * len)), std::exp(-(mediumAtt.y * len)), std::exp(-(mediumAtt.z * len)));
    }
    // the inner layer: EvalBsdf with kOptSamplingProbs and kOptReflectance
    void SraInner(V3 wi, V3 wo, V3 &att, float &pdf, float &refl) const
    {
        if (innerKind == kLambert) {
            att = (wi.z <= 0.f || wo.z <= 0.f) ? V3(0.f) : reflectance / kPiF;
            pdf = CosHemispherePdfW(wi.z);
            refl = Luminance(reflectance);
            return;
        }
        const V3 h = HalfwayReflection(wi, wo);
        const float D = DistributionGgx(h, innerAlpha);
        const float F = FresnelConductor(Dot(h, wo), innerEta, absorb);
        if (wi.z <= 0.f || wo.z <= 0.f || IsTiny(4.0f * wi.z * wo.z)) att = V3(0.f);
        else att = V3((F * SmithG1(wi, h, innerAlpha) * SmithG1(wo, h, innerAlpha) * D) / (4.0f * wi.z * wo.z));
        pdf = (wo.z < 0.f) ? 0.0f : GgxPdfVisibleNormals(wo, h, D, innerAlpha) * ReflectionJacobian(wo, h);
        refl = F;   // GetReflectanceEst: the microfacet Fresnel reflectance (:978-982)
    }
    void SraEval(MatRecord &r) const   // :1328-1451
    {
        const V3 wil = r.wil, wol = r.wol;
        r.compProb = 1.f;
        if (wil.z <= 0.f || wol.z <= 0.f) { r.attenuation = V3(0.f); r.pdfW = 0.f; return; }
        // outer layer, reflection only
        DielCtx c = DielInit(wil, wol);
        const V3 outerAtt = DielEval(c);
        const float outerPdf = (c.wo.z < 0.f) ? 0.f
                               : GgxPdfVisibleNormals(c.wo, c.m, c.Dp, AlphaS()) * ReflectionJacobian(c.wi, c.m);
        V3 wilRefract, wolRefract;
        bool dummy;
        wilRefract = Refract(dummy, wil, V3(0.f, 0.f, 1.f), eta);
        wolRefract = Refract(dummy, wol, V3(0.f, 0.f, 1.f), eta);
        const float wilFresnelTrans = 1.f - FresnelDielectric(wil.z, eta);
        const float wolFresnelRefl = FresnelDielectric(wol.z, eta);
        const float wolFresnelTrans = 1.f - wolFresnelRefl;
        const float cO = std::max(wol.z, 0.0001f), cI = std::max(wil.z, 0.0001f);
        const V3 mediumTrans = BeerLambert(mediumThickness * (1.f / cO + 1.f / cI));
        V3 innerAtt;
        float innerPdf, innerRefl;
        SraInner(-wilRefract, -wolRefract, innerAtt, innerPdf, innerRefl);
        const float innerSolAngCompr = Sqr(1.f / eta);
        r.attenuation = outerAtt + innerAtt * (wilFresnelTrans * wolFresnelTrans) * innerSolAngCompr * mediumTrans;
        const V3 mediumTransEst = BeerLambert(mediumThickness * (1.f / cO * 2.f));
        const float outerC = wolFresnelRefl, innerC = innerRefl * wolFresnelTrans * Luminance(mediumTransEst);
        const float tot = outerC + innerC;
        const float innerPdfSolAngCompr = Sqr(1.f / eta) * (wil.z / -wilRefract.z);
        r.pdfW = outerPdf * (outerC / tot) + (innerPdf * innerPdfSolAngCompr) * (innerC / tot);
    }
    void SraSample(const float u[3], MatRecord &r) const   // :1457-1537; u[2] picks the layer
    {
        const V3 wol = r.wol;
        const float wolFresnelRefl = FresnelDielectric(wol.z, eta);
        const float wolFresnelTrans = 1.f - wolFresnelRefl;
        float innerRefl;
        if (innerKind == kLambert) innerRefl = Luminance(reflectance);
        else innerRefl = FresnelConductor(Dot(HalfwayReflection(V3(0.f), wol), wol), innerEta, absorb);
        const float cO = std::max(wol.z, 0.0001f);
        const V3 mediumTransEst = BeerLambert(mediumThickness * (1.f / cO * 2.f));
        const float outerC = wolFresnelRefl, innerC = innerRefl * wolFresnelTrans * Luminance(mediumTransEst);
        const float tot = outerC + innerC;
        bool dummy;
        if (u[2] * tot < outerC) {
            const bool below = wol.z < 0.f;
            const float s = below ? -1.0f : 1.0f;
            const V3 wo = wol * s;
            const V3 m = SampleVndf(wo, AlphaS(), u[0], u[1]);
            r.wil = Reflect(dummy, wo, m) * s;
        } else {
            const V3 wolRefract = Refract(dummy, wol, V3(0.f, 0.f, 1.f), eta);
            const V3 wo = -wolRefract;
            V3 wi;
            if (innerKind == kLambert) wi = SampleCosHemisphereW(u[0], u[1], nullptr);
            else wi = Reflect(dummy, wo, SampleVndf(wo, innerAlpha, u[0], u[1]));
            r.wil = Refract(dummy, -wi, V3(0.f, 0.f, 1.f), eta);
        }
        SraEval(r);
    }

    // ---- Phong helpers (:383-531)
    float PhongDiffuseEst() const { return Luminance(reflectance); }
    float PhongGlossyEst(V3 wol) const { return Luminance(glossy) * (0.5f + 0.5f * std::max(wol.z, 0.f)); }
    V3 PhongEval(V3 wil, V3 wol) const
    {
        if (wil.z <= 0.f || wol.z <= 0.f) return V3(0.f);
        const float constComponent = (exponent + 2.0f) / (2.0f * kPiF);
        const V3 wrl = ReflectLocal(wil);
        const float thetaRCos = std::max(Dot(wrl, wol), 0.f);
        return reflectance / kPiF + glossy * (constComponent * std::pow(thetaRCos, exponent));
    }
    float PhongPdf(V3 wol, V3 wil, float dEst, float gEst) const
    {
        const float tot = dEst + gEst;
        if (tot < 1e-5f) return CosHemispherePdfW(wil.z);
        Frame lobe;
        lobe.SetFromZ(ReflectLocal(wol));
        const V3 wc = lobe.ToLocal(wil);
        return (dEst / tot) * CosHemispherePdfW(wil.z) + (gEst / tot) * PowerCosHemispherePdfW(wc, exponent);
    }

    // ---- GGX conductor helpers (src/materials.hxx:878-989)
    struct CondCtx { V3 wol, wil, m; float F, D, Dp; };   // Dp: D of the sampling roughness
    V3 CondEval(const CondCtx &c) const
    {
        if (c.wil.z <= 0.f || c.wol.z <= 0.f || IsTiny(4.0f * c.wil.z * c.wol.z)) return V3(0.f);
        const float G = SmithG1(c.wil, c.m, alpha) * SmithG1(c.wol, c.m, alpha);
        const float v = (c.F * G * c.D) / (4.0f * c.wil.z * c.wol.z);
        return V3(v);
    }
    float CondPdf(const CondCtx &c) const
    {
        if (c.wol.z < 0.f) return 0.0f;
        return GgxPdfVisibleNormals(c.wol, c.m, c.Dp, AlphaS()) * ReflectionJacobian(c.wol, c.m);
    }

    // ---- GGX dielectric helpers (src/materials.hxx:1123-1266)
    struct DielCtx { V3 wo, wi, m; bool below, refl; float etaS, etaInvS, F, D, Dp; };
    V3 DielEval(const DielCtx &c) const
    {
        const float ci = std::fabs(c.wi.z), co = std::fabs(c.wo.z);
        if ((!c.refl && IsTiny(ci * co)) || (c.refl && IsTiny(4.0f * ci * co))) return V3(0.f);
        const float G = SmithG1(c.wi, c.m, alpha) * SmithG1(c.wo, c.m, alpha);
        float v;
        if (c.refl) {
            v = (c.F * G * c.D) / (4.0f * ci * co);
        } else {
            const float cMI = Dot(c.m, c.wi), cMO = Dot(c.m, c.wo);
            v = ((std::fabs(cMI) * std::fabs(cMO)) / (ci * co)) *
                ((Sqr(c.etaInvS) * (1.0f - c.F) * G * c.D) / Sqr(cMI + c.etaInvS * cMO));
            v *= Sqr(c.etaS);
        }
        return V3(v);
    }
    float DielPdf(const DielCtx &c) const
    {
        if (c.wo.z < 0.f) return 0.0f;
        const float vn = GgxPdfVisibleNormals(c.wo, c.m, c.Dp, AlphaS());
        const float J = c.refl ? ReflectionJacobian(c.wi, c.m)
                               : RefractionJacobian(c.wo, c.wi, c.m, c.etaInvS);
        const float comp = c.refl ? c.F : (1.f - c.F);
        return vn * J * comp;
    }
    DielCtx DielInit(V3 wil, V3 wol) const   // :1123-1160
    {
        DielCtx c;
        c.below = wol.z < 0.f;
        c.refl = (wil.z > 0.f) == (wol.z > 0.f);
        const float s = c.below ? -1.0f : 1.0f;
        c.wo = wol * s;
        c.wi = wil * s;
        c.etaS = c.below ? etaInv : eta;
        c.etaInvS = c.below ? eta : etaInv;
        c.m = c.refl ? HalfwayReflection(c.wi, c.wo) : HalfwayRefraction(c.wi, c.wo, c.etaInvS);
        c.D = DistributionGgx(c.m, alpha);
        c.Dp = DistributionGgx(c.m, AlphaS());
        c.F = FresnelDielectric(Dot(c.m, c.wo), c.etaS);
        return c;
    }

    // EvalBsdf with kOptSamplingProbs requested (:277-283, :809-817, :1023-1031)
    void Eval(MatRecord &r) const
    {
        if (kind == kLambert) {
            r.attenuation = (r.wil.z <= 0.f || r.wol.z <= 0.f) ? V3(0.f) : reflectance / kPiF;
            r.pdfW = CosHemispherePdfW(r.wil.z);
            r.compProb = 1.f;
        } else if (kind == kGgxConductor) {
            CondCtx c;
            c.wol = r.wol; c.wil = r.wil;
            c.m = HalfwayReflection(c.wil, c.wol);
            c.D = DistributionGgx(c.m, alpha);
            c.Dp = DistributionGgx(c.m, AlphaS());
            c.F = FresnelConductor(Dot(c.m, c.wol), eta, absorb);
            r.attenuation = CondEval(c);
            r.compProb = 1.0f;
            r.pdfW = CondPdf(c);
        } else if (kind == kGgxDielectric) {
            DielCtx c = DielInit(r.wil, r.wol);
            r.attenuation = DielEval(c);
            r.compProb = 1.0f;
            r.pdfW = DielPdf(c);
        } else if (kind == kSra) {
            SraEval(r);
        } else if (kind == kPhong) {   // :416-431, 577-593
            r.attenuation = PhongEval(r.wil, r.wol);
            r.pdfW = PhongPdf(r.wol, r.wil, PhongDiffuseEst(), PhongGlossyEst(r.wol));
            r.compProb = 1.0f;
        } else {   // smooth materials (:611-655): no finite component
            r.attenuation = V3(0.f);
            r.pdfW = 0.f;
            r.compProb = 0.f;
        }
    }

    // SampleBsdf (:285-292, :819-851, :1033-1100); u[0..1] direction, u[2] lobe choice
    void Sample(const float u[3], MatRecord &r) const
    {
        if (kind == kLambert) {
            r.wil = SampleCosHemisphereW(u[0], u[1], &r.pdfW);
            r.attenuation = (r.wil.z <= 0.f || r.wol.z <= 0.f) ? V3(0.f) : reflectance / kPiF;
            r.compProb = 1.f;
        } else if (kind == kGgxConductor) {
            CondCtx c;
            c.wol = r.wol;
            c.m = SampleVndf(c.wol, AlphaS(), u[0], u[1]);
            c.D = DistributionGgx(c.m, alpha);
            c.Dp = DistributionGgx(c.m, AlphaS());
            bool above;
            c.wil = Reflect(above, c.wol, c.m);
            r.wil = c.wil;
            c.F = FresnelConductor(Dot(c.m, c.wol), eta, absorb);
            r.compProb = 1.0f;
            r.pdfW = CondPdf(c);
            if (!above || c.wil.z < 0.0f) r.attenuation = V3(0.f);
            else r.attenuation = CondEval(c);
        } else if (kind == kGgxDielectric) {
            DielCtx c;
            c.below = r.wol.z < 0.f;
            const float s = c.below ? -1.0f : 1.0f;
            c.wo = r.wol * s;
            c.etaS = c.below ? etaInv : eta;
            c.etaInvS = c.below ? eta : etaInv;
            c.m = SampleVndf(c.wo, AlphaS(), u[0], u[1]);
            c.D = DistributionGgx(c.m, alpha);
            c.Dp = DistributionGgx(c.m, AlphaS());
            c.F = FresnelDielectric(Dot(c.m, c.wo), c.etaS);
            bool above;
            float cosAbs;
            if (u[2] <= c.F) {
                c.wi = Reflect(above, c.wo, c.m);
                cosAbs = c.wi.z;
                c.refl = true;
            } else {
                c.wi = Refract(above, c.wo, c.m, c.etaS);
                cosAbs = -c.wi.z;
                c.refl = false;
            }
            r.wil = c.wi * s;
            r.compProb = 1.0f;
            r.pdfW = DielPdf(c);
            if (!above || cosAbs < 0.0f) r.attenuation = V3(0.f);
            else r.attenuation = DielEval(c);
        } else if (kind == kSra) {
            SraSample(u, r);
        } else if (kind == kPhong) {   // :437-495; u[2] picks the component
            const float dEst = PhongDiffuseEst(), gEst = PhongGlossyEst(r.wol);
            const float tot = dEst + gEst;
            if (tot < 1e-5f) {
                r.attenuation = V3(0.f);
                r.wil = SampleCosHemisphereW(u[0], u[1], &r.pdfW);
                r.compProb = 1.f;
                return;
            }
            if (u[2] * tot < dEst) {
                r.wil = SampleCosHemisphereW(u[0], u[1], nullptr);
            } else {
                const V3 cs = SamplePowerCosHemisphereW(u[0], u[1], exponent);
                Frame lobe;
                lobe.SetFromZ(ReflectLocal(r.wol));
                r.wil = lobe.ToWorld(cs);
            }
            r.compProb = 1.f;
            r.pdfW = PhongPdf(r.wol, r.wil, dEst, gEst);
            r.attenuation = (r.wil.z > 0.0f) ? PhongEval(r.wil, r.wol) : V3(0.f);
        } else if (kind == kSmoothConductor) {   // :670-689
            r.wil = ReflectLocal(r.wol);
            r.pdfW = kInf;
            r.compProb = 1.f;
            r.attenuation = V3(FresnelConductor(r.wil.z, eta, absorb));
        } else {   // smooth dielectric, :730-767
            const float F = FresnelDielectric(r.wol.z, eta);
            float a;
            if (u[2] <= F) {
                r.wil = ReflectLocal(r.wol);
                a = F;
                r.compProb = F;
            } else {
                bool above;
                r.wil = Refract(above, r.wol, V3(0.f, 0.f, 1.f), eta);
                a = 1.0f - F;
                a *= above ? Sqr(eta) : Sqr(etaInv);
                r.compProb = 1.0f - F;
            }
            r.attenuation = V3(a);
            r.pdfW = kInf;
        }
    }
};

// --------------------------------------------------------------------------------------------
// Environment map (src/em_image.hxx, src/filter.hxx, src/distribution.hxx,
// src/em_simple_spherical_sampler.hxx, src/em_cosine_sampler.hxx)
// --------------------------------------------------------------------------------------------
enum { kEmCdf = 0, kEmCosine = 1 };

// src/distribution.hxx:45-74 (leading zero; f/n accumulation; normalisation)
static void ComputeCdf(std::vector<float> &cdf, float &integral, const float *f, size_t n)
{
    cdf.assign(n + 1, 0.f);
    for (size_t i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / n;
    integral = cdf[n];
    if (integral == 0.f)
        for (size_t i = 1; i < n + 1; ++i) cdf[i] = (float)i / n;
    else
        for (size_t i = 1; i < n + 1; ++i) cdf[i] /= integral;
}

struct Dist1D {
    std::vector<float> cdf;
    float integral = 0.f;
    size_t n = 0;
    void Build(const float *f, size_t count) { n = count; ComputeCdf(cdf, integral, f, count); }
    // src/distribution.hxx:404-461 (hierarchical search == upper_bound over the full CDF)
    void Sample(float u, float &x, size_t &segm, float &pdf) const
    {
        const float t = u * 0.999999f;
        const float *it = std::upper_bound(cdf.data(), cdf.data() + n + 1, t);
        long s = (long)(it - cdf.data()) - 1;
        s = std::min(std::max(s, 0L), (long)n - 1);
        segm = (size_t)s;
        const float p = cdf[segm + 1] - cdf[segm];
        const float off = (t - cdf[segm]) / p;
        pdf = p * n;
        x = (segm + off) / n;
    }
    float Pdf(size_t s) const { return (cdf[s + 1] - cdf[s]) * n; }   // :463-472
};

struct EnvMap {
    uint32_t W = 0, H = 0;
    std::vector<V3> px;
    int sampler = kEmCdf;
    std::vector<Dist1D> cond;
    Dist1D marg;
    float plan2Ang = 1.0f / (2.0f * kPiF * kPiF);   // src/em_simple_spherical_sampler.hxx:13-14

    const V3 &At(uint32_t x, uint32_t y) const { return px[(size_t)W * y + x]; }

    // src/em_image.hxx:269-302
    void Norm(int x, int y, uint32_t &ox, uint32_t &oy) const
    {
        int rx, ry;
        if (y >= (int)H) { rx = x + (int)W / 2; ry = (int)H - 1; }
        else if (y < 0) { rx = x + (int)W / 2; ry = 0; }
        else { rx = x; ry = y; }
        int m = rx % (int)W;
        if (m < 0) m += (int)W;
        ox = (uint32_t)m; oy = (uint32_t)ry;
    }

    // Bilinear (tent) evaluation, src/em_image.hxx:95-143 with src/filter.hxx:22-31
    V3 Evaluate(float u, float v) const
    {
        const float xf = u * (float)W, yf = v * (float)H;
        const int cx = (int)(xf + 0.5f), cy = (int)(yf + 0.5f);
        const int x0 = cx - 1, y0 = cy - 1;
        const float xl = xf - ((float)x0 + 0.5f), yl = yf - ((float)y0 + 0.5f);
        uint32_t ax, ay, bx, by;
        Norm(x0, y0, ax, ay);
        Norm(cx, cy, bx, by);
        const V3 a = At(ax, ay), b = At(bx, ay), c = At(ax, by), d = At(bx, by);
        const V3 top = (1.f - xl) * a + xl * b;
        const V3 bot = (1.f - xl) * c + xl * d;
        return (1.f - yl) * top + yl * bot;
    }
    V3 Evaluate(V3 dir) const { float u, v; Dir2LatLong(dir, u, v); return Evaluate(u, v); }

    // src/em_image.hxx:152-183, src/filter.hxx:37-60
    float AvgLum(uint32_t x, uint32_t y) const
    {
        uint32_t x0, y0, x2, y2;
        Norm((int)x - 1, (int)y - 1, x0, y0);
        Norm((int)x + 1, (int)y + 1, x2, y2);
        const float w0 = 1 / 24.f, w1 = 2 / 3.f;
        const float l00 = Luminance(At(x0, y0)), l01 = Luminance(At(x0, y)), l02 = Luminance(At(x0, y2));
        const float l10 = Luminance(At(x, y0)), l11 = Luminance(At(x, y)), l12 = Luminance(At(x, y2));
        const float l20 = Luminance(At(x2, y0)), l21 = Luminance(At(x2, y)), l22 = Luminance(At(x2, y2));
        return l00 * w0 + l01 * w0 + l02 * w0 + l10 * w0 + l11 * w1 + l12 * w0 + l20 * w0 + l21 * w0 + l22 * w0;
    }
    float SinMid(uint32_t row) const { return std::sin(kPiF * (row + 0.5f) / H); }   // :186-199

    // src/em_simple_spherical_sampler.hxx:117-152, src/distribution.hxx:488-501
    void BuildCdf()
    {
        std::vector<float> f((size_t)W * H);
        for (uint32_t r = 0; r < H; ++r) {
            const float s = SinMid(r);
            for (uint32_t c = 0; c < W; ++c) f[(size_t)r * W + c] = s * AvgLum(c, r);
        }
        cond.resize(H);
        std::vector<float> mf(H);
        for (uint32_t r = 0; r < H; ++r) { cond[r].Build(&f[(size_t)r * W], W); mf[r] = cond[r].integral; }
        marg.Build(mf.data(), H);
    }

    // src/em_simple_spherical_sampler.hxx:27-82 (CDF) / src/em_cosine_sampler.hxx:13-37 (cosine)
    void Sample(const Frame &frame, bool front, bool back, const float u[3], V3 &wig, float &pdfW, V3 &radCos) const
    {
        if (sampler == kEmCosine) {
            const V3 wil = SampleCosSphereParamPdfW(u[0], u[1], u[2], front, back, pdfW);
            wig = frame.ToWorld(wil);
            radCos = Evaluate(wig) * std::fabs(wil.z);
            return;
        }
        float v, uu, mp, cp;
        size_t sy, sx;
        marg.Sample(u[0], v, sy, mp);
        cond[sy].Sample(u[1], uu, sx, cp);
        const float dp = mp * cp;
        wig = LatLong2Dir(uu, v);
        pdfW = dp * plan2Ang / SinMid((uint32_t)sy);
        const V3 L = Evaluate(uu, v);
        const float c = Dot(wig, frame.Normal());
        radCos = ((front && c > 0.0f) || (back && c < 0.0f)) ? L * std::fabs(c) : V3(0.f);
    }
    // :85-97 / :40-48
    float Pdf(V3 dir, const Frame &frame, bool front, bool back) const
    {
        if (sampler == kEmCosine) return CosSpherePdfW(front, back, frame.ToLocal(dir));
        float u, v;
        Dir2LatLong(dir, u, v);
        const size_t iu = std::min((size_t)(u * W), (size_t)W - 1);
        const size_t iv = std::min((size_t)(v * H), (size_t)H - 1);
        const float pdf = cond[iv].Pdf(iu) * marg.Pdf(iv);
        return pdf * plan2Ang / SinMid((uint32_t)std::min((uint32_t)(v * H), H - 1u));
    }
};

// --------------------------------------------------------------------------------------------
// Geometry and scene (src/scene_graph.hxx, src/scene.hxx)
// --------------------------------------------------------------------------------------------
struct Tri { V3 p[3]; V3 n; int mat; };
struct Sph { V3 c; float r; int mat; };
struct Hit { float dist; int mat; int light; V3 normal; };

// src/scene_graph.hxx:103-134
static bool IntersectTri(const Tri &t, V3 org, V3 dir, float tmin, Hit &h)
{
    const V3 ao = t.p[0] - org, bo = t.p[1] - org, co = t.p[2] - org;
    const V3 v0 = Cross(co, bo), v1 = Cross(bo, ao), v2 = Cross(ao, co);
    const float d0 = Dot(v0, dir), d1 = Dot(v1, dir), d2 = Dot(v2, dir);
    if ((d0 < 0.f && d1 < 0.f && d2 < 0.f) || (d0 >= 0.f && d1 >= 0.f && d2 >= 0.f)) {
        const float dist = Dot(t.n, ao) / Dot(t.n, dir);
        if ((dist > tmin) & (dist < h.dist)) {
            h.normal = t.n; h.mat = t.mat; h.dist = dist;
            return true;
        }
    }
    return false;
}

// src/scene_graph.hxx:176-245 (double discriminant, Muller's second root)
static bool IntersectSph(const Sph &s, V3 org, V3 dir, float tmin, Hit &h)
{
    const V3 o = org - s.c;
    const float A = Dot(dir, dir);
    const float B = 2 * Dot(dir, o);
    const float C = Dot(o, o) - s.r * s.r;
    const double disc = (double)B * B - 4 * (double)A * C;
    if (disc < 0) return false;
    const double ds = std::sqrt(disc);
    const double q = (B >= 0) ? ((-B - ds) / 2.f) : ((-B + ds) / 2.f);
    double t0 = q / A;
    double t1 = (std::fabs(q) > 0.1) ? (C / q) : t0;
    if (t0 > t1) std::swap(t0, t1);
    float rt;
    if (t0 > tmin && t0 < h.dist) rt = (float)t0;
    else if (t1 > tmin && t1 < h.dist) rt = (float)t1;
    else return false;
    h.dist = rt; h.mat = s.mat;
    h.normal = Normalize(o + V3(rt) * dir);
    return true;
}

struct AreaLight {   // src/lights.hxx:55-229
    V3 p0, e1, e2;
    Frame frame;
    V3 radiance;
    float invArea = 0.f;
    void Init(V3 a, V3 b, V3 c, V3 L)
    {
        p0 = a; e1 = b - a; e2 = c - a;
        const V3 n = Cross(e1, e2);
        const float len = Len(n);
        invArea = 2.f / len;
        frame.SetFromZ(n / len);
        radiance = L;
    }
    // ComputeSample (:171-219); front-side light sampling for every material in scope
    void ComputeSample(V3 pt, V3 sp, const Frame &sf, V3 &wig, float &dist, V3 &sample, float &pdfW) const
    {
        wig = sp - pt;
        const float d2 = Dot(wig, wig);
        dist = std::sqrt(d2);
        wig = wig / dist;
        const float cosOut = -Dot(frame.Normal(), wig);
        const float cosIn = std::max(Dot(sf.Normal(), wig), 0.0f);
        sample = (cosOut > 0.f) ? radiance * cosIn : V3(0.f);
        pdfW = std::max(invArea * (d2 / std::fabs(cosOut)), kEpsDist);
    }
    // :133-167
    float Estimate(V3 pt, const Frame &sf) const
    {
        const V3 P1 = p0 + e1, P2 = p0 + e2, P3 = p0 + 0.33f * e1 + 0.33f * e2;
        const V3 pts[4] = {p0, P1, P2, P3};
        float acc = 0.f;
        V3 w, s; float d, p;
        for (int i = 0; i < 4; ++i) { ComputeSample(pt, pts[i], sf, w, d, s, p); acc += Luminance(s) / p; }
        return acc / 4.f;
    }
    // :78-101
    V3 Emission(V3 lightPt, V3 wol, V3 surfPt, float *pdf) const
    {
        if (pdf) {
            V3 w = lightPt - surfPt;
            const float d2 = Dot(w, w);
            w = w / std::sqrt(d2);
            const float c = std::fabs(Dot(frame.Normal(), w));
            *pdf = std::max(invArea * (d2 / c), kEpsDist);
        }
        return (wol.z <= 0.) ? V3(0.f) : radiance;
    }
};

struct PointLight {   // src/lights.hxx:232-343
    V3 position, intensity;
    void SetPower(V3 power) { intensity = power / (4 * kPiF); }   // :244-247
    // ComputeIllumination (:300-337) for a front-side-sampling material; the pdf is infinite
    void Sample(V3 pt, const Frame &sf, V3 &wig, float &dist, V3 &sample, float &pdfW) const
    {
        wig = position - pt;
        const float distSqr = Dot(wig, wig);
        dist = std::sqrt(distSqr);
        wig = wig / dist;
        const float cosThetaIn = std::max(Dot(sf.Normal(), wig), 0.0f);
        sample = (cosThetaIn > 0.f) ? intensity * cosThetaIn / distSqr : V3(0.f);
        pdfW = kInf;
    }
    float Estimate(V3 pt, const Frame &sf) const   // :279-291
    {
        V3 w, s;
        float d, p;
        Sample(pt, sf, w, d, s, p);
        return Luminance(s);
    }
};

struct Scene {
    float camPos[3]{}, camFwd[3]{}, camUp[3]{};
    uint32_t W = 0, H = 0;
    float hfov = 45.f;
    V3 cPos, cFwd, cRight, cUpV;     // derived pinhole basis
    float tanX = 0.f, tanY = 0.f;
    std::vector<Material> mats;
    std::vector<Tri> tris;
    std::vector<Sph> sphs;
    std::vector<AreaLight> lights;        // area lights, ids 0..n-1
    std::vector<PointLight> points;       // point lights, ids n..n+m-1 (src/scene.hxx:817-825)
    std::vector<int> mat2light;
    bool hasBg = false, bgIsEm = false;
    V3 bgConst;
    EnvMap em;
    int bgLightId = -1;
    int algorithm = 7;    // kPathTracing (src/config.hxx:23-34)
    uint32_t minPL = 1, maxPL = 8, rrMinPL = 0;
    // splitting budget, level, light-to-BSDF sample ratio, indirect clipping (src/config.hxx:1129-1133)
    uint32_t splitBudget = 1;
    float splitLevel = 1.f, lightRatio = 1.f, clipping = 0.f;

    size_t LightCount() const { return lights.size() + points.size() + (hasBg ? 1 : 0); }
    float shL[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};   // SH coefficients of the map's luminance
    // (texel luminance x basis x texel solid angle, the steerable sampler's basis)
    void ComputeShL()
    {
        double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        const double pi = 3.14159265358979323846;
        for (uint32_t r = 0; r < em.H; ++r) {
            const double theta = pi * (r + 0.5) / em.H;
            const double dOmega = (2.0 * pi / em.W) * (pi / em.H) * std::sin(theta);
            for (uint32_t c = 0; c < em.W; ++c) {
                const double phi = -((c + 0.5) / em.W - 0.5) * 2.0 * pi;
                const double x = std::sin(theta) * std::cos(phi), y = std::sin(theta) * std::sin(phi), z = std::cos(theta);
                const V3 &p = em.At(c, r);
                const double L = (0.212671 * p.x + 0.715160 * p.y + 0.072169 * p.z) * dOmega;
                acc[0] += L * 0.282095;
                acc[1] += L * 0.488603 * y;
                acc[2] += L * 0.488603 * z;
                acc[3] += L * 0.488603 * x;
                acc[4] += L * 1.092548 * x * y;
                acc[5] += L * 1.092548 * y * z;
                acc[6] += L * 0.315392 * (3.0 * z * z - 1.0);
                acc[7] += L * 1.092548 * x * z;
                acc[8] += L * 0.546274 * (x * x - y * y);
            }
        }
        for (int k = 0; k < 9; ++k) shL[k] = (float)acc[k];
    }

    // src/scene.hxx:42-59, src/scene_graph.hxx:47-57
    bool Intersect(V3 org, V3 dir, float tmin, Hit &h) const
    {
        bool any = false;
        for (const auto &t : tris) any |= IntersectTri(t, org, dir, tmin, h);
        for (const auto &s : sphs) any |= IntersectSph(s, org, dir, tmin, h);
        if (any) h.light = (h.mat >= 0 && h.mat < (int)mat2light.size()) ? mat2light[h.mat] : -1;
        return any;
    }
    // src/scene.hxx:61-74, src/scene_graph.hxx:59-70
    bool Occluded(V3 pt, V3 dir, float tmax) const
    {
        const V3 org = pt + dir * kEpsRay;
        Hit h;
        h.dist = tmax - 2 * kEpsRay;
        for (const auto &t : tris) if (IntersectTri(t, org, dir, 0.f, h)) return true;
        for (const auto &s : sphs) if (IntersectSph(s, org, dir, 0.f, h)) return true;
        return false;
    }

    // Pinhole camera equivalent to src/camera.hxx:13-59, 91-100: the raster-to-world matrix
    // maps raster (x, y) to the direction forward + right * ndc_x * tan(hfov/2)
    //  - up * ndc_y * tan(vfov/2), with tan(vfov/2) = tan(hfov/2) * H / W.
    void SetupCamera()
    {
        const V3 aPos(camPos[0], camPos[1], camPos[2]);
        const V3 fwd = Normalize(V3(camFwd[0], camFwd[1], camFwd[2]));
        const V3 aUp(camUp[0], camUp[1], camUp[2]);
        cRight = Normalize(Cross(aUp, -fwd));   // the reference calls this vector "up"
        cUpV = Cross(-fwd, cRight);             // ... and this one "left"
        cFwd = fwd;
        cPos = aPos;
        tanX = std::tan(0.5f * hfov * (2.f * kPiF / 360.f));
        tanY = tanX * (float)H / (float)W;
    }
    V3 CameraDir(float rx, float ry) const
    {
        const float nx = rx * (2.f / W) - 1.f;
        const float ny = ry * (2.f / H) - 1.f;
        return Normalize(cFwd + cRight * (nx * tanX) - cUpV * (ny * tanY));
    }

    // Background emission incl. MIS pdf (src/lights.hxx:379-407, src/em.hxx:87-121)
    V3 BgEmission(V3 dir, float *pdf, const Frame *f) const
    {
        if (bgIsEm) {
            const V3 L = em.Evaluate(dir);
            if (pdf && f) *pdf = em.Pdf(dir, *f, true, false);
            return L;
        }
        if (pdf && f) *pdf = CosSpherePdfW(true, false, f->ToLocal(dir));
        return bgConst;
    }
    // Background light sample (src/lights.hxx:424-445)
    void BgSample(const Frame &f, const float u[3], V3 &wig, float &pdfW, V3 &radCos) const
    {
        if (bgIsEm) { em.Sample(f, true, false, u, wig, pdfW, radCos); return; }
        const V3 wil = SampleCosSphereParamPdfW(u[0], u[1], u[2], true, false, pdfW);
        wig = f.ToWorld(wil);
        radCos = bgConst * std::fabs(wil.z);
    }
};

// --------------------------------------------------------------------------------------------
// The estimator
// --------------------------------------------------------------------------------------------
struct PathKey { uint64_t seed; uint32_t pixel, sample; };

class Tracer {
public:
    explicit Tracer(const Scene &s) : S(s) {}

    // Light contribution estimates of the current vertex for every light, in light-id order
    // (src/path_tracer_base.hxx:22-32, 216-232). The background's (src/lights.hxx:447-470): pi x
    // luminance when constant; for a map the clamped-cosine SH estimate of the irradiance, 9 SH
    // coefficients of the map's luminance (the steerable sampler's estimate,
    // src/em_steerable_sampler.hxx:2300-2355; the reference's other samplers draw a random MIS
    // estimate instead, src/em.hxx:130-169 -- either keeps the picking unbiased).
    void Estimates(V3 pt, const Frame &f, std::vector<float> &est) const
    {
        est.resize(S.LightCount());
        for (size_t i = 0; i < S.lights.size(); ++i) est[i] = S.lights[i].Estimate(pt, f);
        for (size_t i = 0; i < S.points.size(); ++i) est[S.lights.size() + i] = S.points[i].Estimate(pt, f);
        if (S.hasBg) {
            if (!S.bgIsEm) {
                est[S.bgLightId] = Luminance(S.bgConst) * kPiF;
            } else {
                const V3 n = f.Normal();
                const float c1 = .429043f, c2 = .511644f, c3 = .743125f, c4 = .886227f, c5 = .247708f;
                const float c[9] = {c4 + 0.15f, 2.f * c2 * n.y, 2.f * c2 * n.z, 2.f * c2 * n.x, 2.f * c1 * n.x * n.y,
                                    2.f * c1 * n.y * n.z, c3 * n.z * n.z - c5, 2.f * c1 * n.x * n.z,
                                    c1 * (n.x * n.x - n.y * n.y)};
                float e = 0.f;
                for (int k = 0; k < 9; ++k) e += S.shL[k] * c[k];
                est[S.bgLightId] = std::max(e, 0.f);
            }
        }
    }

    // PickSingleLight (src/path_tracer_base.hxx:191-257)
    void Pick(const std::vector<float> &est, float u, int &id, float &prob) const
    {
        const size_t n = S.LightCount();
        if (n == 0) { id = -1; return; }
        if (n == 1) { id = 0; prob = 1.f; return; }
        std::vector<float> cdf(n + 1);
        float sum = 0.f;
        cdf[0] = 0.f;
        for (size_t i = 0; i < n; ++i) { sum += est[i]; cdf[i + 1] = sum; }
        if (sum > 0.f) {
            const float r = u * sum;
            uint32_t l = 0;
            for (; (l < n) && (r > cdf[l + 1]); l++);
            if (l >= n) l = (uint32_t)n - 1;
            id = (int)l;
            prob = (cdf[l + 1] - cdf[l]) / sum;
        } else {
            id = std::min((int)(u * n), (int)n - 1);
            prob = 1.f / n;
        }
    }
    // LightPickingProbability (src/path_tracer_base.hxx:260-313)
    float PickProb(const std::vector<float> &est, int id) const
    {
        const size_t n = S.LightCount();
        if (n == 0) return 0.f;
        if (n == 1) return 1.f;
        float sum = 0.f, mine = 0.f;
        for (size_t i = 0; i < n; ++i) { sum += est[i]; if ((int)i == id) mine = est[i]; }
        return (sum > 0.f) ? mine / sum : 1.f / n;
    }

    // MISWeight2Power (src/path_tracer_base.hxx:522-541), both counts 1
    static float MIS(float a, float b) { const float a2 = a * a, b2 = b * b; return a2 / (a2 + b2) / 1; }

    // MISWeight2Power with sample counts (src/path_tracer_base.hxx:522-541)
    static float MISn(float p1, uint32_t n1, float p2, uint32_t n2)
    {
        const float s1 = n1 * p1, s2 = n2 * p2;
        const float q1 = s1 * s1, q2 = s2 * s2;
        return q1 / (q1 + q2) / n1;
    }

    // ComputeSplittingCounts (src/path_tracer.hxx:432-454)
    void SplittingCounts(float budget, uint32_t &nBsdf, uint32_t &nLight, float &nextBudget) const
    {
        nBsdf = (uint32_t)std::lroundf((1.f - S.splitLevel) * 1.f + S.splitLevel * budget);
        nLight = (uint32_t)std::lroundf(std::max(S.lightRatio * nBsdf, 1.f));
        nextBudget = 1 + ((budget - nBsdf) / (float)nBsdf);
    }

    // EstimateIncomingRadiancePT (src/path_tracer.hxx:167-430), with splitting (:240-248,
    // 432-454) and indirect clipping (:400-402). Random numbers are keyed by the vertex's
    // preorder index in the path tree (1 for the camera ray's hit; a chain without splitting
    // gives index = path length): light sample j draws group 2j, BSDF sample i group 2i+1.
    void EstimatePT(const PathKey &key, V3 org, V3 dir, float tmin, uint32_t pathLength, bool computeRefl,
                    float budget, uint32_t &vid, V3 &emitted, V3 &reflected, const Frame *shFrame, bool havePdf,
                    float *emPdf, int *emLight) const
    {
        emitted = V3(0.f);
        reflected = V3(0.f);
        Hit h;
        h.dist = 1e36f;
        if (!S.Intersect(org, dir, tmin, h)) {
            if (pathLength >= S.minPL && S.hasBg) {
                emitted += S.BgEmission(dir, havePdf ? emPdf : nullptr, shFrame);
                if (emLight) *emLight = S.bgLightId;
            }
            return;
        }
        const V3 pt = org + dir * h.dist;
        Frame frame;
        frame.SetFromZ(h.normal);
        const V3 wol = frame.ToLocal(-dir);
        const Material &mat = S.mats[h.mat];
        if (h.light >= 0 && pathLength >= S.minPL) {
            emitted += S.lights[h.light].Emission(pt, wol, org, havePdf ? emPdf : nullptr);
            if (emLight) *emLight = h.light;
        }
        if (!computeRefl) return;
        if (mat.IsReflectanceZero()) return;
        if (S.maxPL > 0 && pathLength >= S.maxPL) return;
        if (pathLength >= 1200) return;   // kMaxPathLengthHard (src/path_tracer.hxx:461-462)
        const uint32_t me = ++vid;

        uint32_t nBsdf, nLight;
        float nextBudget;
        SplittingCounts(budget, nBsdf, nLight, nextBudget);

        std::vector<float> est;
        if (S.LightCount() > 1 && mat.SamplesLights()) Estimates(pt, frame, est);

        // Light samples + MIS (src/path_tracer.hxx:250-265, src/path_tracer_base.hxx:156-188, 350-423)
        if (pathLength + 1 >= S.minPL && mat.SamplesLights()) {
            for (uint32_t j = 0; j < nLight; ++j) {
                const Rand4 ra = Draw(key.seed, key.pixel, key.sample, me, 2 * j);
                int lid = -1;
                float lprob = 0.f;
                Pick(est, ra.v[0], lid, lprob);
                if (lid < 0) continue;
                V3 wig, smp;
                float dist, pdfW;
                const float lu[3] = {ra.v[1], ra.v[2], ra.v[3]};
                SampleLight(lid, pt, frame, lu, wig, dist, smp, pdfW);
                if (MaxC(smp) > 0. && !S.Occluded(pt, wig, dist)) {
                    MatRecord mr;
                    mr.wil = frame.ToLocal(wig);
                    mr.wol = wol;
                    mat.Eval(mr);
                    if (pdfW == kInf) {   // point light: exact contribution, only the picking is estimated
                        reflected += (smp * mr.attenuation) / (lprob * nLight);
                    } else {
                        const float bsdfPdf = mr.pdfW * mr.compProb;
                        const float lightPdf = pdfW * lprob;
                        reflected += (smp * mr.attenuation * MISn(lightPdf, nLight, bsdfPdf, nBsdf)) / lightPdf;
                    }
                }
            }
        }

        // Russian roulette (src/path_tracer.hxx:267-303)
        const bool rrActive = (S.maxPL == 0) || (S.rrMinPL > 0 && pathLength >= S.rrMinPL);
        const float rrProb = rrActive ? Clampf(mat.RRContinuationProb(wol), 0.0f, 0.997f) : 1.0f;

        // BSDF samples (src/path_tracer.hxx:305-405)
        for (uint32_t i = 0; i < nBsdf; ++i) {
            const Rand4 rb = Draw(key.seed, key.pixel, key.sample, me, 2 * i + 1);
            const bool cut = rrActive && rb.v[0] > rrProb;
            MatRecord mr;
            mr.wol = wol;
            const float bu[3] = {rb.v[1], rb.v[2], rb.v[3]};
            mat.Sample(bu, mr);
            if (mr.IsBlocker()) continue;
            const V3 wig = frame.ToWorld(mr.wil);
            const float rayMin = EpsRayCos(mr.CosAbs());
            V3 bEm, bRefl;
            float bPdf = 0.f;
            int bLight = -1;
            EstimatePT(key, pt, wig, rayMin, pathLength + 1, !cut, nextBudget, vid, bEm, bRefl, &frame, true, &bPdf,
                       &bLight);
            // Direct light hit by the BSDF sample (:327-369)
            if (!IsZero(bEm) && bLight >= 0) {
                if (mr.IsFinite()) {
                    const float lightPdf = bPdf * PickProb(est, bLight);
                    const float bsdfPdf = mr.pdfW * mr.compProb;
                    reflected += (mr.attenuation * mr.CosAbs() * bEm * MISn(bsdfPdf, nBsdf, lightPdf, nLight)) / bsdfPdf;
                } else {
                    reflected += (mr.attenuation * bEm) / ((float)nBsdf * mr.compProb);
                }
            }
            // Indirect light (:372-405), clipped proportionally (src/math.hxx:538-549)
            if (!cut && !IsZero(bRefl)) {
                V3 ind = mr.IsFinite()
                             ? (mr.attenuation * mr.CosAbs() * bRefl) / (mr.pdfW * nBsdf * rrProb * mr.compProb)
                             : (mr.attenuation * bRefl) / (nBsdf * rrProb * mr.compProb);
                if (S.clipping > 0.f) {
                    const float mx = MaxC(ind);
                    if (mx > S.clipping) ind = ind * (S.clipping / mx);
                }
                reflected += ind;
            }
        }
    }

    // EstimateIncomingRadiancePTNaive (src/path_tracer.hxx:45-165)
    V3 EstimatePTN(const PathKey &key, V3 org, V3 dir) const
    {
        V3 L(0.f), T(1.f);
        float tmin = 0.f;
        for (uint32_t pl = 1;;) {
            Hit h;
            h.dist = 1e36f;
            if (!S.Intersect(org, dir, tmin, h)) {
                if (pl >= S.minPL && S.hasBg) L += S.BgEmission(dir, nullptr, nullptr) * T;
                return L;
            }
            const V3 pt = org + dir * h.dist;
            Frame frame;
            frame.SetFromZ(h.normal);
            const V3 wol = frame.ToLocal(-dir);
            const Material &mat = S.mats[h.mat];
            if (h.light >= 0 && pl >= S.minPL) L += S.lights[h.light].Emission(pt, wol, V3(0.f), nullptr) * T;
            if (mat.IsReflectanceZero()) return L;
            if (S.maxPL > 0 && pl >= S.maxPL) return L;
            if (pl >= 1200) return L;
            const Rand4 rb = Draw(key.seed, key.pixel, key.sample, pl, 1);
            const bool rrActive = (S.maxPL == 0) || (S.rrMinPL > 0 && pl >= S.rrMinPL);
            float rr = 1.0f;
            if (rrActive) {
                rr = Clampf(mat.RRContinuationProb(wol), 0.0f, 0.997f);
                if (rb.v[0] > rr) return L;
            }
            MatRecord mr;
            mr.wol = wol;
            const float bu[3] = {rb.v[1], rb.v[2], rb.v[3]};
            mat.Sample(bu, mr);
            if (mr.IsBlocker()) return L;
            org = pt;
            dir = frame.ToWorld(mr.wil);
            tmin = EpsRayCos(mr.CosAbs());
            const V3 seg = mr.IsFinite() ? (mr.attenuation * mr.CosAbs()) / (mr.pdfW * rr * mr.compProb)
                                         : mr.attenuation / (rr * mr.compProb);
            T = T * seg;
            pl++;
        }
    }

    // Light sample of light `lid` from the shading point (area: src/lights.hxx:114-131; point:
    // :255-266; background: :424-445); u holds three uniforms.
    void SampleLight(int lid, V3 pt, const Frame &frame, const float u[3], V3 &wig, float &dist, V3 &smp,
                     float &pdfW) const
    {
        if (lid == S.bgLightId) {
            S.BgSample(frame, u, wig, pdfW, smp);
            dist = std::numeric_limits<float>::max();
        } else if (lid >= (int)S.lights.size()) {
            S.points[lid - S.lights.size()].Sample(pt, frame, wig, dist, smp, pdfW);
        } else {
            const AreaLight &L = S.lights[lid];
            const V3 sp = SampleUniformTriangle(L.p0, L.p0 + L.e1, L.p0 + L.e2, u[0], u[1]);
            L.ComputeSample(pt, sp, frame, wig, dist, smp, pdfW);
        }
    }

    // GetDirectRadianceFromDirection (src/path_tracer_base.hxx:92-154): radiance arriving
    // along the BSDF-sampled local direction wil, its light-sampling pdf and picking probability.
    V3 DirectFromDirection(V3 pt, const Frame &frame, V3 wil, const std::vector<float> &est, float *pdfW,
                           float *pickProb) const
    {
        const V3 wig = frame.ToWorld(wil);
        Hit h;
        h.dist = 1e36f;
        int lightId = -1;
        V3 L(0.f);
        if (S.Intersect(pt, wig, EpsRayCos(wil.z), h)) {
            if (h.light >= 0) {
                const V3 lightPt = pt + wig * h.dist;
                Frame lf;
                lf.SetFromZ(h.normal);
                L = S.lights[h.light].Emission(lightPt, lf.ToLocal(-wig), pt, pdfW);
                lightId = h.light;
            }
        } else if (S.hasBg) {
            L = S.BgEmission(wig, pdfW, &frame);
            lightId = S.bgLightId;
        }
        // (no estimates at a vertex without light samples: its Dirac BSDF samples take no MIS)
        if (pickProb && lightId >= 0) *pickProb = (S.LightCount() > 1 && est.empty()) ? 0.f : PickProb(est, lightId);
        return L;
    }

    // Direct illumination (src/direct_illumination.hxx:15-156), eye light
    // (src/eye_light.hxx:21-60) and normal visualiser (src/normal_visualiser.hxx:21-62).
    // Random numbers: camera jitter (vertex 0, group 0), light pick + sample (vertex 1, group 0),
    // BSDF sample (vertex 1, group 1), light i of the all-lights estimator (vertex 1, group 2 + i).
    V3 EstimateDirect(const PathKey &key, V3 dir) const
    {
        const int alg = S.algorithm;
        Hit h;
        h.dist = 1e36f;
        if (!S.Intersect(S.cPos, dir, 0.f, h)) {
            if (alg <= 1 || !S.hasBg) return V3(0.f);
            return S.BgEmission(dir, nullptr, nullptr);
        }
        if (alg == 0) {
            const float dotLN = Dot(h.normal, -dir);
            return dotLN > 0.f ? V3(dotLN) : V3(-dotLN, 0.f, 0.f);
        }
        if (alg == 1)
            return V3(Clampf(h.normal.x / 2.f + 0.5f, 0.f, 1.f), Clampf(h.normal.y / 2.f + 0.5f, 0.f, 1.f),
                      Clampf(h.normal.z / 2.f + 0.5f, 0.f, 1.f));
        const V3 pt = S.cPos + dir * h.dist;
        Frame frame;
        frame.SetFromZ(h.normal);
        const V3 wol = frame.ToLocal(-dir);
        const Material &mat = S.mats[h.mat];
        std::vector<float> est;
        const bool lights = mat.SamplesLights();
        if (S.LightCount() > 1 && lights) Estimates(pt, frame, est);
        const Rand4 ra = Draw(key.seed, key.pixel, key.sample, 1, 0);
        const Rand4 rb = Draw(key.seed, key.pixel, key.sample, 1, 1);
        V3 Lo(0.f);
        // AddSingleLightSampleContribution (src/path_tracer_base.hxx:315-348)
        auto single = [&](int lid, float prob, const float u[3]) {
            V3 wig, smp;
            float dist, pdfW;
            SampleLight(lid, pt, frame, u, wig, dist, smp, pdfW);
            if (!(MaxC(smp) > 0.) || S.Occluded(pt, wig, dist)) return;
            MatRecord mr;
            mr.wil = frame.ToLocal(wig);
            mr.wol = wol;
            mat.Eval(mr);
            if (pdfW == kInf) Lo += smp * mr.attenuation / prob;   // point light (:333-348)
            else Lo += smp * mr.attenuation / (pdfW * prob);
        };
        if (alg == 3 && lights) {
            for (size_t i = 0; i < S.LightCount(); ++i) {
                const Rand4 rl = Draw(key.seed, key.pixel, key.sample, 1, 2 + (uint32_t)i);
                const float lu[3] = {rl.v[1], rl.v[2], rl.v[3]};
                single((int)i, 1.f, lu);
            }
        } else if (alg == 4 && lights) {
            int lid = -1;
            float lprob = 0.f;
            Pick(est, ra.v[0], lid, lprob);
            const float lu[3] = {ra.v[1], ra.v[2], ra.v[3]};
            if (lid >= 0) single(lid, lprob, lu);
        } else if (alg == 2) {
            MatRecord mr;
            mr.wol = wol;
            const float bu[3] = {rb.v[1], rb.v[2], rb.v[3]};
            mat.Sample(bu, mr);
            if (!mr.IsBlocker()) {
                const V3 Li = DirectFromDirection(pt, frame, mr.wil, est, nullptr, nullptr);
                Lo = mr.IsFinite() ? (mr.attenuation * mr.CosAbs() * Li) / (mr.pdfW * mr.compProb)
                                   : (mr.attenuation * Li) / mr.compProb;
            }
        } else if (alg == 5) {
            // kDirectIllumMis: one light sample and one BSDF sample (:99-114), power heuristic
            int lid = -1;
            float lprob = 0.f;
            if (lights) Pick(est, ra.v[0], lid, lprob);
            if (lid >= 0) {
                V3 wig, smp;
                float dist, pdfW;
                const float lu[3] = {ra.v[1], ra.v[2], ra.v[3]};
                SampleLight(lid, pt, frame, lu, wig, dist, smp, pdfW);
                if (MaxC(smp) > 0. && !S.Occluded(pt, wig, dist)) {   // :350-411
                    MatRecord mr;
                    mr.wil = frame.ToLocal(wig);
                    mr.wol = wol;
                    mat.Eval(mr);
                    if (pdfW == kInf) {
                        Lo += (smp * mr.attenuation) / lprob;
                    } else {
                        const float lightPdf = pdfW * lprob;
                        Lo += (smp * mr.attenuation * MIS(lightPdf, mr.pdfW * mr.compProb)) / lightPdf;
                    }
                }
            }
            MatRecord mr;   // AddDirectIllumMISBrdfSampleContribution (:427-486)
            mr.wol = wol;
            const float bu[3] = {rb.v[1], rb.v[2], rb.v[3]};
            mat.Sample(bu, mr);
            if (!mr.IsBlocker()) {
                float lightPdfW = 0.f, pick = 0.f;
                const V3 Li = DirectFromDirection(pt, frame, mr.wil, est, &lightPdfW, &pick);
                if (MaxC(Li) > 0.f) {
                    if (mr.IsFinite()) {
                        const float bsdfPdf = mr.pdfW * mr.compProb;
                        Lo += (mr.attenuation * mr.CosAbs() * Li * MIS(bsdfPdf, lightPdfW * pick)) / bsdfPdf;
                    } else {
                        Lo += (mr.attenuation * Li) / mr.compProb;
                    }
                }
            }
        }
        V3 Le(0.f);
        if (h.light >= 0) Le = S.lights[h.light].Emission(pt, wol, V3(0.f), nullptr);
        return Le + Lo;
    }

    // One sample of one pixel (src/path_tracer_base.hxx:66-87; the visualisers take the pixel
    // centre for sample 0, src/eye_light.hxx:35-37)
    V3 Radiance(uint64_t seed, uint32_t pixel, uint32_t sample) const
    {
        const PathKey key{seed, pixel, sample};
        const uint32_t x = pixel % S.W, y = pixel / S.W;
        const Rand4 rc = Draw(seed, pixel, sample, 0, 0);
        const bool centre = S.algorithm <= 1 && sample == 0;
        const V3 dir = S.CameraDir((float)x + (centre ? 0.5f : rc.v[0]), (float)y + (centre ? 0.5f : rc.v[1]));
        if (S.algorithm <= 5) return EstimateDirect(key, dir);
        if (S.algorithm == 6) return EstimatePTN(key, S.cPos, dir);
        V3 e, r;
        uint32_t vid = 0;
        EstimatePT(key, S.cPos, dir, 0.f, 1, true, (float)S.splitBudget, vid, e, r, nullptr, false, nullptr, nullptr);
        return e + r;
    }

private:
    const Scene &S;
};

// --------------------------------------------------------------------------------------------
// Scene file (same text format as oracle/ref_harness.cpp)
// --------------------------------------------------------------------------------------------
static bool LoadEnv(const std::string &path, EnvMap &em)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[4];
    uint32_t hdr[3];
    bool ok = std::fread(magic, 1, 4, f) == 4 && std::memcmp(magic, "PG3F", 4) == 0 &&
              std::fread(hdr, 4, 3, f) == 3 && hdr[2] == 3;
    if (ok) {
        em.W = hdr[0]; em.H = hdr[1];
        std::vector<float> buf((size_t)em.W * em.H * 3);
        ok = std::fread(buf.data(), 4, buf.size(), f) == buf.size();
        em.px.resize((size_t)em.W * em.H);
        for (size_t i = 0; i < em.px.size(); ++i) em.px[i] = V3(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]);
    }
    std::fclose(f);
    return ok;
}

static bool ParseScene(const char *text, Scene &s, std::string &err)
{
    std::istringstream in(text);
    std::string line;
    std::vector<std::pair<int, V3>> pendingLights;   // (mat, radiance) for area_light records
    EnvMap samplingEm;
    bool hasSamplingEm = false;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string k;
        if (!(ls >> k) || k[0] == '#') continue;
        if (k == "camera") {
            ls >> s.camPos[0] >> s.camPos[1] >> s.camPos[2] >> s.camFwd[0] >> s.camFwd[1] >> s.camFwd[2] >>
                s.camUp[0] >> s.camUp[1] >> s.camUp[2] >> s.W >> s.H >> s.hfov;
        } else if (k == "lambert") {
            float r, g, b; ls >> r >> g >> b;
            s.mats.push_back(Material::Lambert(V3(r, g, b)));
        } else if (k == "ggx_conductor") {
            float a, n, no, kk; ls >> a >> n >> no >> kk;
            s.mats.push_back(Material::Conductor(a, n, no, kk));
        } else if (k == "ggx_dielectric") {
            float a, n, no; ls >> a >> n >> no;
            s.mats.push_back(Material::Dielectric(a, n, no));
        } else if (k == "phong") {
            float d[3], g[3], e;
            ls >> d[0] >> d[1] >> d[2] >> g[0] >> g[1] >> g[2] >> e;
            s.mats.push_back(Material::Phong(V3(d[0], d[1], d[2]), V3(g[0], g[1], g[2]), e));
        } else if (k == "smooth_conductor") {
            float n, no, kk; ls >> n >> no >> kk;
            s.mats.push_back(Material::SmoothConductor(n, no, kk));
        } else if (k == "smooth_dielectric") {
            float n, no; ls >> n >> no;
            s.mats.push_back(Material::SmoothDielectric(n, no));
        } else if (k == "sra") {
            // sra outer_alpha outer_n outer_no (lambert r g b | ggx_conductor a n no k) att_r att_g att_b thickness
            float a, n, no;
            std::string ik;
            ls >> a >> n >> no >> ik;
            Material inner;
            if (ik == "lambert") {
                float r, g, b; ls >> r >> g >> b;
                inner = Material::Lambert(V3(r, g, b));
            } else if (ik == "ggx_conductor") {
                float ia, in, ino, kk; ls >> ia >> in >> ino >> kk;
                inner = Material::Conductor(ia, in, ino, kk);
            } else { err = "sra: unknown inner layer " + ik; return false; }
            float att[3], th;
            ls >> att[0] >> att[1] >> att[2] >> th;
            s.mats.push_back(Material::Sra(Material::Dielectric(a, n, no), inner, V3(att[0], att[1], att[2]), th));
        } else if (k == "point_light") {
            float p[3], w[3];
            ls >> p[0] >> p[1] >> p[2] >> w[0] >> w[1] >> w[2];
            PointLight pl;
            pl.position = V3(p[0], p[1], p[2]);
            pl.SetPower(V3(w[0], w[1], w[2]));
            s.points.push_back(pl);
        } else if (k == "triangle" || k == "area_light") {
            float v[9]; int mat;
            for (float &x : v) ls >> x;
            ls >> mat;
            Tri t;
            t.p[0] = V3(v[0], v[1], v[2]); t.p[1] = V3(v[3], v[4], v[5]); t.p[2] = V3(v[6], v[7], v[8]);
            t.mat = mat;
            t.n = Normalize(Cross(t.p[1] - t.p[0], t.p[2] - t.p[0]));   // src/scene_graph.hxx:88-101
            s.tris.push_back(t);
            if (k == "area_light") {
                float L[3]; ls >> L[0] >> L[1] >> L[2];
                AreaLight al;
                al.Init(t.p[0], t.p[1], t.p[2], V3(L[0], L[1], L[2]));
                s.lights.push_back(al);
                if ((int)s.mat2light.size() <= mat) s.mat2light.resize(mat + 1, -1);
                s.mat2light[mat] = (int)s.lights.size() - 1;
            }
        } else if (k == "sphere") {
            Sph sp; ls >> sp.c.x >> sp.c.y >> sp.c.z >> sp.r >> sp.mat;
            s.sphs.push_back(sp);
        } else if (k == "background_const") {
            s.hasBg = true; s.bgIsEm = false;
            ls >> s.bgConst.x >> s.bgConst.y >> s.bgConst.z;
        } else if (k == "background_em") {
            std::string p; ls >> p;
            s.hasBg = true; s.bgIsEm = true;
            if (!LoadEnv(p, s.em)) { err = "cannot read environment map " + p; return false; }
        } else if (k == "options") {
            // algorithm names of the reference's command line (src/config.hxx:23-34, 292-318)
            std::string alg; ls >> alg >> s.minPL >> s.maxPL;
            const char *names[8] = {"el", "nv", "dbs", "dlsa", "dlss", "dmis", "ptn", "pt"};
            s.algorithm = -1;
            for (int a = 0; a < 8; ++a) if (alg == names[a]) s.algorithm = a;
            if (s.algorithm < 0) { err = "unknown algorithm " + alg; return false; }
            // optional: splitting budget, splitting level, light-to-BSDF ratio, indirect clipping
            uint32_t sb;
            float lvl, ratio, clip;
            if (ls >> sb >> lvl >> ratio >> clip) {
                if (sb < 1) { err = "splitting budget must be >= 1"; return false; }
                s.splitBudget = sb; s.splitLevel = lvl; s.lightRatio = ratio; s.clipping = clip;
            }
        } else if (k == "sampling_material") {
            // sampling overrides of one material: GGX sampling roughness, roulette probability
            // (negative: unchanged); finite differences with the sampling held fixed
            int mat; float aS, rr; ls >> mat >> aS >> rr;
            if (mat < 0 || mat >= (int)s.mats.size()) { err = "sampling_material: material out of range"; return false; }
            if (aS >= 0.f) s.mats[mat].alphaSample = Clampf(aS, 0.001f, 1.0f);
            if (rr >= 0.f) s.mats[mat].rrOverride = rr;
        } else if (k == "background_em_sampling") {
            // the environment-map sampler's tables come from this map instead of the lit one
            std::string p; ls >> p;
            if (!LoadEnv(p, samplingEm)) { err = "cannot read environment map " + p; return false; }
            hasSamplingEm = true;
        } else {
            err = "unknown record " + k;
            return false;
        }
    }
    s.mat2light.resize(std::max(s.mat2light.size(), s.mats.size()), -1);
    if (s.hasBg) s.bgLightId = (int)(s.lights.size() + s.points.size());   // pushed last (src/scene.hxx:948-953)
    if (s.bgIsEm) {
        s.em.BuildCdf();
        if (hasSamplingEm) {
            if (samplingEm.W != s.em.W || samplingEm.H != s.em.H) { err = "sampling map size differs"; return false; }
            samplingEm.BuildCdf();
            s.em.cond = samplingEm.cond;
            s.em.marg = samplingEm.marg;
        }
    }
    s.SetupCamera();
    if (s.bgIsEm) s.ComputeShL();
    return true;
}

}  // namespace pg3o

// ============================================================================================
// C API (ctypes)
// ============================================================================================
extern "C" {

// Renders samples [sample0, sample0 + spp) of every pixel and writes
//   sum_rgb[pixel*3+c]  += radiance         (double)
//   sumsq_rgb[...]      += radiance^2       (double, may be null)
//   per_sample          [((s - sample0) * npix + pixel)*3 + c] (float, may be null)
// em_sampler: 0 CDF, 1 cosine. rr_min_path_length as in the header comment.
// Returns 0 on success, nonzero on a scene error (message in err, up to errlen bytes).
int pg3o_render(const char *scene_text, uint64_t seed, uint32_t sample0, uint32_t spp, int em_sampler,
                uint32_t rr_min_path_length, int threads, double *sum_rgb, double *sumsq_rgb, float *per_sample,
                char *err, int errlen)
{
    using namespace pg3o;
    Scene s;
    std::string e;
    if (!ParseScene(scene_text, s, e)) {
        if (err && errlen > 0) { std::strncpy(err, e.c_str(), errlen - 1); err[errlen - 1] = 0; }
        return 1;
    }
    s.em.sampler = em_sampler;
    s.rrMinPL = rr_min_path_length;
    if (s.algorithm >= 6)
        for (const Material &m : s.mats)
            if (m.kind == kSra) {
                // the reference's path tracers stop with a fatal error on this material
                // (IsReflectanceZero / GetRRContinuationProb not implemented, src/materials.hxx:1544-1557)
                const char *msg = "the path tracers cannot render the SRA layered material";
                if (err && errlen > 0) { std::strncpy(err, msg, errlen - 1); err[errlen - 1] = 0; }
                return 1;
            }
    const Tracer tr(s);
    const uint32_t npix = s.W * s.H;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (long p = 0; p < (long)npix; ++p) {
        for (uint32_t k = 0; k < spp; ++k) {
            const V3 L = tr.Radiance(seed, (uint32_t)p, sample0 + k);
            for (int c = 0; c < 3; ++c) {
                if (sum_rgb) sum_rgb[(size_t)p * 3 + c] += L[c];
                if (sumsq_rgb) sumsq_rgb[(size_t)p * 3 + c] += (double)L[c] * L[c];
                if (per_sample) per_sample[((size_t)k * npix + p) * 3 + c] = L[c];
            }
        }
    }
    return 0;
}

// Philox4x32-10 block for the known-answer test.
// GGX visible-normal sampling for all later calls: 1 exact (default), 0 the reference's fit.
void pg3o_set_ggx_exact(int exact) { pg3o::g_vndfExact = exact != 0; }

void pg3o_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    pg3o::Philox4x32_10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}

// Camera ray directions for raster points (x, y) (n points), for the camera check.
int pg3o_camera_dirs(const char *scene_text, const float *raster_xy, int n, float *dirs)
{
    pg3o::Scene s;
    std::string e;
    if (!pg3o::ParseScene(scene_text, s, e)) return 1;
    for (int i = 0; i < n; ++i) {
        const pg3o::V3 d = s.CameraDir(raster_xy[2 * i], raster_xy[2 * i + 1]);
        dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    }
    return 0;
}

// Environment-map CDF sampler tables (marginal H+1, conditional H*(W+1)) for the table check.
int pg3o_em_cdf(const char *em_path, float *marg, float *cond)
{
    pg3o::EnvMap em;
    if (!pg3o::LoadEnv(em_path, em)) return 1;
    em.BuildCdf();
    std::memcpy(marg, em.marg.cdf.data(), sizeof(float) * (em.H + 1));
    for (uint32_t r = 0; r < em.H; ++r) std::memcpy(cond + (size_t)r * (em.W + 1), em.cond[r].cdf.data(), sizeof(float) * (em.W + 1));
    return 0;
}

}  // extern "C"

extern "C" {
// BSDF sampler probe: material (kind 0/1/2 with alpha, eta=n/n_out, k), n samples for one wol;
// u[3n] uniforms; outputs wil[3n], pdf_sampled[n], pdf_eval[n], att_sampled[n] (grey), att_eval[n].
void pg3o_probe_bsdf(int kind, float alpha, float n_in, float n_out, float k, const float *wol, int n,
                     const float *u, float *wil, float *pdfS, float *pdfE, float *attS, float *attE)
{
    using namespace pg3o;
    Material m = kind == kLambert ? Material::Lambert(V3(0.5f))
               : kind == kGgxConductor ? Material::Conductor(alpha, n_in, n_out, k)
                                       : Material::Dielectric(alpha, n_in, n_out);
    const V3 wo(wol[0], wol[1], wol[2]);
    for (int i = 0; i < n; ++i) {
        MatRecord s;
        s.wol = wo;
        m.Sample(u + 3 * i, s);
        MatRecord e;
        e.wil = s.wil;
        e.wol = wo;
        m.Eval(e);
        wil[3 * i] = s.wil.x; wil[3 * i + 1] = s.wil.y; wil[3 * i + 2] = s.wil.z;
        pdfS[i] = s.pdfW * s.compProb;
        pdfE[i] = e.pdfW * e.compProb;
        attS[i] = s.attenuation.x;
        attE[i] = e.attenuation.x;
    }
}
void pg3o_bsdf_pdf(int kind, float alpha, float n_in, float n_out, float k, const float *wol, int n,
                   const float *wil, float *pdf, float *att)
{
    using namespace pg3o;
    Material m = kind == kLambert ? Material::Lambert(V3(0.5f))
               : kind == kGgxConductor ? Material::Conductor(alpha, n_in, n_out, k)
                                       : Material::Dielectric(alpha, n_in, n_out);
    for (int i = 0; i < n; ++i) {
        MatRecord e;
        e.wil = V3(wil[3 * i], wil[3 * i + 1], wil[3 * i + 2]);
        e.wol = V3(wol[0], wol[1], wol[2]);
        m.Eval(e);
        pdf[i] = e.pdfW * e.compProb;
        if (att) att[i] = e.attenuation.x;
    }
}
}

extern "C" void pg3o_probe_vndf(const float *wol, float alpha, int n, const float *u, float *m)
{
    using namespace pg3o;
    const V3 wo(wol[0], wol[1], wol[2]);
    for (int i = 0; i < n; ++i) {
        const V3 h = SampleGgxVisibleNormals(wo, alpha, u[2 * i], u[2 * i + 1]);
        m[3 * i] = h.x; m[3 * i + 1] = h.y; m[3 * i + 2] = h.z;
    }
}
