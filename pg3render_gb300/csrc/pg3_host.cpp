// Host-side scene preparation for the device layout (see pg3_host.h).
#include "pg3_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace pg3 {

namespace {

struct V { float x, y, z; };
V sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V crossv(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float dotv(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float lenv(V a) { return std::sqrt(dotv(a, a)); }
V scale(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
V divv(V a, float s) { return {a.x / s, a.y / s, a.z / s}; }
V normv(V a) { return divv(a, lenv(a)); }
V ld(const float *p) { return {p[0], p[1], p[2]}; }
float3 f3(V a) { return make_float3(a.x, a.y, a.z); }
bool finite3(const float *p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

const float kPi = 3.14159265358979f;
const float kTiny = 9.5367431640625E-7f;
float lum(float r, float g, float b) { return 0.212671f * r + 0.715160f * g + 0.072169f * b; }

// ComputeCdf (src/distribution.hxx:45-74): running sum of f/n, then divide by the total.
void computeCdf(const float *f, uint32_t n, float *cdf, float &integral)
{
    cdf[0] = 0.f;
    for (uint32_t i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / n;
    integral = cdf[n];
    if (integral == 0.f)
        for (uint32_t i = 1; i < n + 1; ++i) cdf[i] = (float)i / n;
    else
        for (uint32_t i = 1; i < n + 1; ++i) cdf[i] /= integral;
}

}  // namespace

void buildEmCdf(const float *rgb, uint32_t W, uint32_t H, std::vector<float> &marg, std::vector<float> &cond)
{
    // texel luminances once; the filter below reads them through the wrap rule at the border
    std::vector<float> lumImg((size_t)W * H);
    for (size_t i = 0; i < lumImg.size(); ++i) lumImg[i] = lum(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    auto L = [&](int x, int y) {
        if (x >= 0 && x < (int)W && y >= 0 && y < (int)H) return lumImg[(size_t)y * W + (size_t)x];
        // NormalizeImgCoords (src/em_image.hxx:269-302)
        int rx = x, ry = y;
        if (y >= (int)H) { rx = x + (int)W / 2; ry = (int)H - 1; }
        else if (y < 0) { rx = x + (int)W / 2; ry = 0; }
        int m = rx % (int)W;
        if (m < 0) m += (int)W;
        return lumImg[(size_t)ry * W + (size_t)m];
    };
    std::vector<float> f((size_t)W);
    cond.assign((size_t)H * (W + 1), 0.f);
    std::vector<float> rowInt(H);
    const float w0 = 1 / 24.f, w1 = 2 / 3.f;
    for (uint32_t r = 0; r < H; ++r) {
        const float s = std::sin(kPi * (r + 0.5f) / H);   // SinMidTheta (src/em_simple_spherical_sampler.hxx:186-199)
        for (uint32_t c = 0; c < W; ++c) {
            // tent-filter pixel integral (src/em_image.hxx:152-183, src/filter.hxx:37-60)
            const int x = (int)c, y = (int)r;
            const float l00 = L(x - 1, y - 1), l01 = L(x - 1, y), l02 = L(x - 1, y + 1);
            const float l10 = L(x, y - 1), l11 = L(x, y), l12 = L(x, y + 1);
            const float l20 = L(x + 1, y - 1), l21 = L(x + 1, y), l22 = L(x + 1, y + 1);
            const float avg = l00 * w0 + l01 * w0 + l02 * w0 + l10 * w0 + l11 * w1 + l12 * w0 + l20 * w0 +
                              l21 * w0 + l22 * w0;
            f[c] = s * avg;
        }
        computeCdf(f.data(), W, &cond[(size_t)r * (W + 1)], rowInt[r]);
    }
    marg.assign(H + 1, 0.f);
    float total;
    computeCdf(rowInt.data(), H, marg.data(), total);
}

void emShCoefficients(const float *rgb, uint32_t W, uint32_t H, std::vector<float> &out)
{
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double pi = 3.14159265358979323846;
    std::vector<double> cosPhi(W), sinPhi(W);
    for (uint32_t c = 0; c < W; ++c) {
        const double phi = -((c + 0.5) / W - 0.5) * 2.0 * pi;   // latLong2Dir
        cosPhi[c] = std::cos(phi);
        sinPhi[c] = std::sin(phi);
    }
    for (uint32_t r = 0; r < H; ++r) {
        const double theta = pi * (r + 0.5) / H;
        const double sinT = std::sin(theta), z = std::cos(theta);
        const double dOmega = (2.0 * pi / W) * (pi / H) * sinT;
        for (uint32_t c = 0; c < W; ++c) {
            const double x = sinT * cosPhi[c], y = sinT * sinPhi[c];
            const float *p = rgb + ((size_t)r * W + c) * 3;
            const double L = (0.212671 * p[0] + 0.715160 * p[1] + 0.072169 * p[2]) * dOmega;
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
    out.assign(9, 0.f);
    for (int k = 0; k < 9; ++k) out[k] = (float)acc[k];
}

int prepareScene(const pg3gpu_scene &sc, const pg3gpu_options &o, HostScene &out, std::string &err)
{
    char buf[256];
    auto bad = [&](int st, const char *msg) { err = msg; return st; };
    const pg3gpu_camera &c = sc.camera;
    if (c.width == 0 || c.height == 0 || (uint64_t)c.width * c.height > (1ull << 28))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "camera resolution must be positive and at most 2^28 pixels");
    if (!finite3(c.position) || !finite3(c.forward) || !finite3(c.up) || !(c.hfov_deg > 0.f && c.hfov_deg < 180.f))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "camera parameters must be finite, 0 < hfov < 180");
    if (o.algorithm < PG3GPU_ALG_EYE_LIGHT || o.algorithm > PG3GPU_ALG_PATH_TRACING)
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "unknown algorithm (the reference's ids 0-7, src/config.hxx:23-34)");
    if (o.min_path_length < 1) return bad(PG3GPU_ERR_INVALID_ARGUMENT, "min_path_length must be >= 1");
    // the reference rejects these combinations (src/config.hxx:1063-1077)
    if (o.max_path_length == 0 && o.min_path_length != 1)
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "min path length != 1 with Russian roulette ending paths");
    if (o.max_path_length != 0 && o.min_path_length > o.max_path_length)
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "min path length larger than max path length");
    if (!(o.indirect_clipping >= 0.f) || !std::isfinite(o.indirect_clipping))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "indirect clipping must be finite and >= 0");
    if (o.splitting_budget < 1 || o.splitting_budget > 64)
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "splitting budget must be in 1..64");
    if (!(o.splitting_level >= 0.f && o.splitting_level <= 1.f))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "splitting level must be in [0, 1]");
    if (!(o.light_to_bsdf_ratio > 0.f && o.light_to_bsdf_ratio <= 16.f))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "light-to-BSDF sample ratio must be in (0, 16]");
    if (o.em_sampler != PG3GPU_EM_CDF && o.em_sampler != PG3GPU_EM_COSINE && o.em_sampler != PG3GPU_EM_STEERABLE)
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "unknown environment-map sampler");
    if (o.steer_weights != PG3GPU_STEER_WEIGHTS_POINT && o.steer_weights != PG3GPU_STEER_WEIGHTS_PROJECTED)
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "unknown steerable vertex weights");
    const bool adaptive = o.steer_max_subdiv_level > o.steer_subdiv_level;
    if (adaptive && (o.steer_max_subdiv_level > kSteerMaxAdaptiveLevel || !(o.steer_max_approx_error > 0.f) ||
                     !std::isfinite(o.steer_max_approx_error)))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT,
                   "adaptive steerable triangulation: maximum subdivision level must be <= 12 and the maximum "
                   "approximation error finite and > 0");
    if (sc.num_materials == 0 || !sc.materials) return bad(PG3GPU_ERR_INVALID_ARGUMENT, "scene has no materials");
    if ((sc.num_triangles && !sc.triangles) || (sc.num_spheres && !sc.spheres) ||
        (sc.num_area_lights && !sc.area_lights) || (sc.num_point_lights && !sc.point_lights))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "NULL array with a nonzero count");
    if (sc.num_triangles + (uint64_t)sc.num_spheres > (1u << 30))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "too many primitives");

    SceneView &v = out.view;
    // camera: the reference's raster-to-world matrix (src/camera.hxx:13-59) sends raster
    // (x, y) along forward + right * ndc_x * tan(hfov/2) - up * ndc_y * tan(vfov/2)
    {
        const V fwd = normv(ld(c.forward));
        const V up = ld(c.up);
        const V mfwd = scale(fwd, -1.f);
        const V right = normv(crossv(up, mfwd));
        const V upv = crossv(mfwd, right);
        v.camPos = f3(ld(c.position));
        v.camFwd = f3(fwd);
        v.camRight = f3(right);
        v.camUp = f3(upv);
        v.tanX = std::tan(0.5f * c.hfov_deg * (2.f * kPi / 360.f));
        v.tanY = v.tanX * (float)c.height / (float)c.width;
        v.width = c.width;
        v.height = c.height;
    }

    // materials (src/materials.hxx:262-266, 366-381, 658-668, 713-727, 791-806, 996-1021)
    v.nmat = sc.num_materials;
    out.mats.resize(sc.num_materials);
    for (uint32_t i = 0; i < sc.num_materials; ++i) {
        const pg3gpu_material &m = sc.materials[i];
        DevMaterial d{};
        d.kind = m.kind;
        d.r = m.albedo[0]; d.g = m.albedo[1]; d.b = m.albedo[2];
        d.alpha = std::min(std::max(m.alpha, 0.001f), 1.0f);
        d.alphaS = d.alpha;
        d.eta = 1.f; d.etaInv = 1.f;
        if (m.kind == PG3GPU_MAT_LAMBERT) {
            if (!finite3(m.albedo) || m.albedo[0] < 0.f || m.albedo[1] < 0.f || m.albedo[2] < 0.f)
                return bad(PG3GPU_ERR_INVALID_ARGUMENT, "Lambert albedo must be finite and non-negative");
            const float mx = std::max(d.r, std::max(d.g, d.b));
            const float p = std::min(std::max(0.15f * lum(d.r, d.g, d.b) + 0.85f * mx, 0.f), 1.f);
            d.rrProb = std::min(std::max(p, 0.0f), 0.997f);
            d.zeroRefl = (d.r == 0.f && d.g == 0.f && d.b == 0.f) ? 1 : 0;
        } else if (m.kind == PG3GPU_MAT_GGX_CONDUCTOR) {
            d.eta = (std::fabs(m.ior_outer) < kTiny) ? 1.0f : m.ior / m.ior_outer;
            d.absorb = m.absorb;
            d.rrProb = 0.997f;
        } else if (m.kind == PG3GPU_MAT_GGX_DIELECTRIC) {
            if (std::fabs(m.ior_outer) >= kTiny) { d.eta = m.ior / m.ior_outer; d.etaInv = m.ior_outer / m.ior; }
            d.rrProb = 0.997f;
        } else if (m.kind == PG3GPU_MAT_PHONG) {
            if (!finite3(m.albedo) || !finite3(m.glossy) || m.albedo[0] < 0.f || m.albedo[1] < 0.f ||
                m.albedo[2] < 0.f || m.glossy[0] < 0.f || m.glossy[1] < 0.f || m.glossy[2] < 0.f)
                return bad(PG3GPU_ERR_INVALID_ARGUMENT, "Phong reflectances must be finite and non-negative");
            if (!(m.phong_exponent >= 0.f) || !std::isfinite(m.phong_exponent))
                return bad(PG3GPU_ERR_INVALID_ARGUMENT, "Phong exponent must be finite and >= 0");
            d.gr = m.glossy[0]; d.gg = m.glossy[1]; d.gb = m.glossy[2];
            d.exponent = m.phong_exponent;
            // the diffuse part of GetRRContinuationProb (:542-570); the glossy part depends on wo
            d.rrProb = 0.15f * lum(d.r, d.g, d.b) + 0.85f * std::max(d.r, std::max(d.g, d.b));
            d.zeroRefl = (d.r == 0.f && d.g == 0.f && d.b == 0.f && d.gr == 0.f && d.gg == 0.f && d.gb == 0.f) ? 1 : 0;
        } else if (m.kind == PG3GPU_MAT_SMOOTH_CONDUCTOR) {
            d.eta = (std::fabs(m.ior_outer) < kTiny) ? 1.0f : m.ior / m.ior_outer;
            d.absorb = m.absorb;
            d.rrProb = 0.997f;   // unused: the roulette probability is the Fresnel reflectance of wo
        } else if (m.kind == PG3GPU_MAT_SMOOTH_DIELECTRIC) {
            d.eta = (std::fabs(m.ior_outer) < kTiny) ? 1.0f : m.ior / m.ior_outer;
            d.etaInv = (std::fabs(m.ior) < kTiny) ? 1.0f : m.ior_outer / m.ior;
            d.rrProb = 0.997f;
        } else if (m.kind == PG3GPU_MAT_SRA_LAYERED) {
            // outer GGX dielectric as MicrofacetGGXDielectricMaterial (:996-1021); inner Lambert
            // or GGX conductor (:262-266, 791-806); the medium between them (:1307-1324)
            if (std::fabs(m.ior_outer) >= kTiny) { d.eta = m.ior / m.ior_outer; d.etaInv = m.ior_outer / m.ior; }
            if (!(d.eta > 0.f) || !std::isfinite(d.eta))
                return bad(PG3GPU_ERR_INVALID_ARGUMENT, "SRA outer layer needs positive indices of refraction");
            d.innerKind = m.inner_kind;
            if (m.inner_kind == PG3GPU_MAT_LAMBERT) {
                if (!finite3(m.albedo) || m.albedo[0] < 0.f || m.albedo[1] < 0.f || m.albedo[2] < 0.f)
                    return bad(PG3GPU_ERR_INVALID_ARGUMENT, "SRA inner Lambert reflectance must be finite and >= 0");
            } else if (m.inner_kind == PG3GPU_MAT_GGX_CONDUCTOR) {
                if (!(m.inner_alpha >= 0.f) || !std::isfinite(m.inner_ior) || !std::isfinite(m.inner_ior_outer))
                    return bad(PG3GPU_ERR_INVALID_ARGUMENT, "SRA inner conductor needs alpha >= 0 and finite IORs");
                d.innerAlpha = std::min(std::max(m.inner_alpha, 0.001f), 1.0f);
                d.innerEta = (std::fabs(m.inner_ior_outer) < kTiny) ? 1.0f : m.inner_ior / m.inner_ior_outer;
                d.absorb = m.absorb;
            } else {
                return bad(PG3GPU_ERR_INVALID_ARGUMENT, "SRA inner layer must be Lambert or GGX conductor");
            }
            if (!finite3(m.medium_attenuation) || m.medium_attenuation[0] < 0.f || m.medium_attenuation[1] < 0.f ||
                m.medium_attenuation[2] < 0.f || !(m.medium_thickness >= 0.f) || !std::isfinite(m.medium_thickness))
                return bad(PG3GPU_ERR_INVALID_ARGUMENT, "SRA medium attenuation and thickness must be finite and >= 0");
            d.gr = m.medium_attenuation[0]; d.gg = m.medium_attenuation[1]; d.gb = m.medium_attenuation[2];
            d.exponent = m.medium_thickness;
            d.rrProb = 1.f;   // (not used: the path tracers refuse the material)
        } else {
            std::snprintf(buf, sizeof buf, "material %u: unknown kind %d", i, m.kind);
            err = buf;
            return PG3GPU_ERR_INVALID_ARGUMENT;
        }
        if (!(m.alpha >= 0.f) && (m.kind == PG3GPU_MAT_GGX_CONDUCTOR || m.kind == PG3GPU_MAT_GGX_DIELECTRIC ||
                                  m.kind == PG3GPU_MAT_SRA_LAYERED))
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "GGX roughness must be >= 0");
        if ((m.kind == PG3GPU_MAT_GGX_CONDUCTOR || m.kind == PG3GPU_MAT_GGX_DIELECTRIC ||
             m.kind == PG3GPU_MAT_SMOOTH_CONDUCTOR || m.kind == PG3GPU_MAT_SMOOTH_DIELECTRIC) &&
            !(std::isfinite(m.ior) && std::isfinite(m.ior_outer) && std::isfinite(m.absorb)))
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "indices of refraction and absorbance must be finite");
        d.vndfExact = (o.ggx_sampler == PG3GPU_GGX_VNDF_REFERENCE_FIT) ? 0 : 1;
        out.mats[i] = d;
        out.kindMask |= 1u << m.kind;
    }

    // geometry
    out.tri.resize((size_t)sc.num_triangles * 3);
    out.triMat.resize(sc.num_triangles);
    for (uint32_t i = 0; i < sc.num_triangles; ++i) {
        const pg3gpu_triangle &t = sc.triangles[i];
        if (t.material < 0 || (uint32_t)t.material >= sc.num_materials)
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "triangle material id out of range");
        const V p0 = ld(t.p), p1 = ld(t.p + 3), p2 = ld(t.p + 6);
        const V nrm = normv(crossv(sub(p1, p0), sub(p2, p0)));   // src/scene_graph.hxx:88-101
        if (!(std::isfinite(nrm.x) && std::isfinite(nrm.y) && std::isfinite(nrm.z)))
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "degenerate or non-finite triangle");
        out.tri[3 * i] = make_float4(p0.x, p0.y, p0.z, nrm.x);
        out.tri[3 * i + 1] = make_float4(p1.x, p1.y, p1.z, nrm.y);
        out.tri[3 * i + 2] = make_float4(p2.x, p2.y, p2.z, nrm.z);
        out.triMat[i] = t.material;
    }
    // after the vertices, per triangle its normal and material (int bits): what a hit reads
    for (uint32_t i = 0; i < sc.num_triangles; ++i) {
        float m;
        std::memcpy(&m, &out.triMat[i], sizeof m);
        out.tri.push_back(make_float4(out.tri[3 * i].w, out.tri[3 * i + 1].w, out.tri[3 * i + 2].w, m));
    }
    out.sph.resize(sc.num_spheres);
    out.sphMat.resize(sc.num_spheres);
    for (uint32_t i = 0; i < sc.num_spheres; ++i) {
        const pg3gpu_sphere &s = sc.spheres[i];
        if (s.material < 0 || (uint32_t)s.material >= sc.num_materials)
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "sphere material id out of range");
        if (!finite3(s.center) || !(s.radius > 0.f) || !std::isfinite(s.radius))
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "sphere needs a finite centre and a positive radius");
        out.sph[i] = make_float4(s.center[0], s.center[1], s.center[2], s.radius);
        out.sphMat[i] = s.material;
    }
    v.ntri = sc.num_triangles;
    v.nsph = sc.num_spheres;

    // lights: area lights keep their order, point lights follow, the background comes last
    // (src/scene.hxx:767-825, 948-953)
    if (sc.num_area_lights + (uint64_t)sc.num_point_lights > (1u << 20))
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "too many lights");
    out.mat2light.assign(sc.num_materials, -1);
    out.lights.resize(sc.num_area_lights + sc.num_point_lights);
    for (uint32_t i = 0; i < sc.num_area_lights; ++i) {
        const pg3gpu_area_light &a = sc.area_lights[i];
        if (a.triangle >= sc.num_triangles) return bad(PG3GPU_ERR_INVALID_ARGUMENT, "area light triangle out of range");
        if (!finite3(a.radiance)) return bad(PG3GPU_ERR_INVALID_ARGUMENT, "area light radiance must be finite");
        const pg3gpu_triangle &t = sc.triangles[a.triangle];
        const V p0 = ld(t.p), e1 = sub(ld(t.p + 3), p0), e2 = sub(ld(t.p + 6), p0);
        const V n = crossv(e1, e2);
        const float len = lenv(n);
        const V nz = divv(n, len);   // src/lights.hxx:59-75
        DevAreaLight L;
        L.p0_invArea = make_float4(p0.x, p0.y, p0.z, 2.f / len);
        L.e1_r = make_float4(e1.x, e1.y, e1.z, a.radiance[0]);
        L.e2_g = make_float4(e2.x, e2.y, e2.z, a.radiance[1]);
        L.n_b = make_float4(nz.x, nz.y, nz.z, a.radiance[2]);
        out.lights[i] = L;
        if (out.mat2light[t.material] >= 0)
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "two area lights share one emitting material");
        out.mat2light[t.material] = (int)i;
    }
    for (uint32_t i = 0; i < sc.num_point_lights; ++i) {
        const pg3gpu_point_light &p = sc.point_lights[i];
        if (!finite3(p.position) || !finite3(p.power))
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "point light position and power must be finite");
        // PointLight::SetPower (src/lights.hxx:244-247): intensity = power / (4 pi)
        DevAreaLight L;
        L.p0_invArea = make_float4(p.position[0], p.position[1], p.position[2], -1.f);
        L.e1_r = make_float4(0.f, 0.f, 0.f, p.power[0] / (4 * kPi));
        L.e2_g = make_float4(0.f, 0.f, 0.f, p.power[1] / (4 * kPi));
        L.n_b = make_float4(0.f, 0.f, 0.f, p.power[2] / (4 * kPi));
        out.lights[sc.num_area_lights + i] = L;
    }
    out.numPointLights = sc.num_point_lights;
    v.nArea = sc.num_area_lights + sc.num_point_lights;
    v.bgKind = sc.background;
    v.lightCount = v.nArea + (sc.background != PG3GPU_BG_NONE ? 1 : 0);
    v.bgLightId = (sc.background != PG3GPU_BG_NONE) ? (int)v.nArea : -1;
    v.bgConst = make_float3(sc.background_radiance[0], sc.background_radiance[1], sc.background_radiance[2]);
    if (sc.background == PG3GPU_BG_ENVMAP) {
        if (!sc.env_map || sc.env_width < 2 || sc.env_height < 2 || (uint64_t)sc.env_width * sc.env_height > (1ull << 26))
            return bad(PG3GPU_ERR_INVALID_ARGUMENT, "environment map needs data and 2 <= size <= 2^26 pixels");
        const size_t np = (size_t)sc.env_width * sc.env_height;
        // every component finite and non-negative, tested on the bit patterns (a vectorised pass):
        // finite non-negative floats are 0x00000000-0x7F7FFFFF, and -0 (0x80000000) counts as 0
        uint32_t invalid = 0;
        for (size_t i = 0; i < 3 * np; ++i) {
            uint32_t u;
            std::memcpy(&u, sc.env_map + i, sizeof u);
            invalid |= (uint32_t)(u > 0x7F7FFFFFu) & (uint32_t)(u != 0x80000000u);
        }
        if (invalid) return bad(PG3GPU_ERR_INVALID_ARGUMENT, "environment map texels must be finite and non-negative");
        out.emRgb = sc.env_map;   // uploaded as RGB and widened to float4 on the device
        out.emTexels = np;
        // the CDF tables serve the CDF sampler only (the device rebuilds them on map updates)
        if (o.em_sampler == PG3GPU_EM_CDF) buildEmCdf(sc.env_map, sc.env_width, sc.env_height, out.emMarg, out.emCond);
        v.emW = sc.env_width;
        v.emH = sc.env_height;
        if (o.em_sampler == PG3GPU_EM_STEERABLE) {
            if (adaptive) {
                // the map-dependent triangulation of this context
                out.steer = steerAdaptiveGeometry(sc.env_map, sc.env_width, sc.env_height, o.steer_subdiv_level,
                                                  o.steer_max_subdiv_level, o.steer_max_approx_error, err);
            } else {
                // the shared geometry of the level (process lifetime; not owned here)
                const SteerGeom *g = steerGeometry(o.steer_subdiv_level, err);
                if (g) out.steer = std::shared_ptr<const SteerGeom>(std::shared_ptr<const SteerGeom>(), g);
            }
            if (!out.steer) return PG3GPU_ERR_INVALID_ARGUMENT;
            out.hasSteer = true;   // the picking estimate is the sampler's own whole integral (device)
        } else {
            emShCoefficients(sc.env_map, sc.env_width, sc.env_height, out.bgShL);
        }
    } else if (sc.background != PG3GPU_BG_NONE && sc.background != PG3GPU_BG_CONSTANT) {
        return bad(PG3GPU_ERR_INVALID_ARGUMENT, "unknown background kind");
    }
    v.emSampler = (o.em_sampler == PG3GPU_EM_STEERABLE && out.steer && out.steer->adaptive) ? kEmSteerableAdaptive
                                                                                             : o.em_sampler;
    v.algorithm = o.algorithm;
    v.splitBudget = (float)o.splitting_budget;
    v.splitLevel = o.splitting_level;
    v.lightRatio = o.light_to_bsdf_ratio;
    v.clipping = o.indirect_clipping;
    // the recursive estimator is needed when a vertex takes more than one BSDF or light sample,
    // or when indirect estimates are clipped (src/path_tracer.hxx:240-265, 400-402, 432-454)
    {
        const float b = (1.f - o.splitting_level) + o.splitting_level * (float)o.splitting_budget;
        const long nB = std::lround(b);
        const long nL = std::lround(std::max(o.light_to_bsdf_ratio * (float)nB, 1.f));
        v.treeMode = (o.splitting_budget > 1 || o.indirect_clipping > 0.f || nB != 1 || nL != 1) ? 1 : 0;
    }
    v.minPL = o.min_path_length;
    v.maxPL = o.max_path_length;
    v.rrMinPL = o.rr_min_path_length;
    v.seedLo = (uint32_t)o.seed;
    v.seedHi = (uint32_t)(o.seed >> 32);
    return PG3GPU_OK;
}

}  // namespace pg3
