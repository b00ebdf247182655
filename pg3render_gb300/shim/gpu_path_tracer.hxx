// gpu_path_tracer.hxx -- the reference-side renderer class that drops this library into
// PG3Render.
//
// A PG3Render maintainer adds this header to the reference's src/ directory and one case to
// its renderer factory (CreateRenderer, src/pg3render.cxx:24-50):
//
//     #include "gpu_path_tracer.hxx"
//     ...
//     if (aConfig.mUseGpu) return new GpuPathTracer(aConfig, aSeed);   // any algorithm id
//
// GpuPathTracer derives from the reference's AbstractRenderer (src/renderer.hxx:232-278) and
// keeps its contract: the constructor takes the Config (and the scene it points to), every
// RunIteration(algorithm, iteration) adds one sample per pixel of that iteration, and
// GetFramebuffer returns the accumulated image divided by the iteration count. The scene is
// translated once, in the constructor, from the reference's own objects (Scene::mGeometry /
// mMaterials / mLights / mMaterial2Light / mBackgroundLight / mCamera, src/scene.hxx:1276-1289)
// into the library's C description (include/pg3gpu.h) and copied to the device.
//
// Two things differ from the CPU renderers, both because the image lives on the GPU:
//  * GetFramebuffer is not virtual in the reference, so the device image is copied into the
//    renderer's Framebuffer by Sync(); Render() (src/pg3render.cxx:136-162) calls it before
//    GetFramebuffer. RunIteration never waits for the GPU.
//  * one GPU context per process: run with -j 1 (Render then calls RunIteration serially).
//
// Errors the library reports (a scene or option combination it does not support, a CUDA
// failure) end the program through PG3_FATAL_ERROR, the reference's own convention
// (src/debugging.hxx:44-66).
//
// Reading the reference's objects: the material parameters are protected members and the
// environment map's image is a private member of EnvironmentMap (src/em.hxx:191-200). The
// Peek helpers below read them without changing the reference's headers (a pointer to a
// protected member formed through a derived class; for the private image, the explicit
// template instantiation rule, which does not check access). A maintainer who can edit the
// reference would add public getters instead.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "config.hxx"
#include "lights.hxx"
#include "materials.hxx"
#include "renderer.hxx"
#include "scene.hxx"
#include "scene_graph.hxx"

#include "pg3gpu.h"

namespace gpu_shim {

// ---- access to protected material parameters (pointer to member through a derived class)
struct LambertPeek : LambertMaterial {
    static const SpectrumF &Reflectance(const LambertMaterial &m) { return m.*(&LambertPeek::mReflectance); }
};
struct PhongPeek : PhongMaterial {
    static const SpectrumF &Diffuse(const PhongMaterial &m) { return m.*(&PhongPeek::mDiffuseReflectance); }
    static const SpectrumF &Glossy(const PhongMaterial &m) { return m.*(&PhongPeek::mPhongReflectance); }
    static float Exponent(const PhongMaterial &m) { return m.*(&PhongPeek::mPhongExponent); }
};
struct GgxConductorPeek : MicrofacetGGXConductorMaterial {
    static float Eta(const MicrofacetGGXConductorMaterial &m) { return m.*(&GgxConductorPeek::mEta); }
    static float Absorbance(const MicrofacetGGXConductorMaterial &m) { return m.*(&GgxConductorPeek::mAbsorbance); }
    static float Alpha(const MicrofacetGGXConductorMaterial &m) { return m.*(&GgxConductorPeek::mRoughnessAlpha); }
};
struct GgxDielectricPeek : MicrofacetGGXDielectricMaterial {
    static float Eta(const MicrofacetGGXDielectricMaterial &m) { return m.*(&GgxDielectricPeek::mEta); }
    static float Alpha(const MicrofacetGGXDielectricMaterial &m) { return m.*(&GgxDielectricPeek::mRoughnessAlpha); }
};
struct SmoothConductorPeek : SmoothConductorMaterial {
    static float Eta(const SmoothConductorMaterial &m) { return m.*(&SmoothConductorPeek::mEta); }
    static float Absorbance(const SmoothConductorMaterial &m) { return m.*(&SmoothConductorPeek::mAbsorbance); }
};
struct SmoothDielectricPeek : SmoothDielectricMaterial {
    static float Eta(const SmoothDielectricMaterial &m) { return m.*(&SmoothDielectricPeek::mEta); }
};
struct SraPeek : SraLayeredMaterial {
    static const AbstractMaterial *Outer(const SraLayeredMaterial &m) { return (m.*(&SraPeek::mOuterLayerMaterial)).get(); }
    static const AbstractMaterial *Inner(const SraLayeredMaterial &m) { return (m.*(&SraPeek::mInnerLayerMaterial)).get(); }
    static const SpectrumF &Attenuation(const SraLayeredMaterial &m) { return m.*(&SraPeek::mMediumAttCoeff); }
    static float Thickness(const SraLayeredMaterial &m) { return m.*(&SraPeek::mMediumThickness); }
};

// ---- the environment map's image (private member of EnvironmentMap)
template <typename Tag, typename Tag::type Member>
struct PrivateMember {
    friend typename Tag::type Get(Tag) { return Member; }
};
struct EmImageTag {
    typedef std::shared_ptr<EnvironmentMapImage> EnvironmentMap::*type;
    friend type Get(EmImageTag);
};
template struct PrivateMember<EmImageTag, &EnvironmentMap::mEmImage>;

inline const EnvironmentMapImage *EmImage(const EnvironmentMap &em) { return (em.*Get(EmImageTag())).get(); }

inline void Copy3(float *dst, const SpectrumF &s)
{
    for (int c = 0; c < 3; ++c) dst[c] = s.Get(c);
}
inline void Copy3(float *dst, const Vec3f &v)
{
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
}

// The library's description of one reference material (src/materials.hxx:253-1566).
inline pg3gpu_material TranslateMaterial(const AbstractMaterial *am)
{
    pg3gpu_material m;
    std::memset(&m, 0, sizeof m);
    m.ior_outer = 1.f;   // the reference keeps only the ratio inner / outer
    if (auto *p = dynamic_cast<const LambertMaterial *>(am)) {
        m.kind = PG3GPU_MAT_LAMBERT;
        Copy3(m.albedo, LambertPeek::Reflectance(*p));
    } else if (auto *p = dynamic_cast<const PhongMaterial *>(am)) {
        m.kind = PG3GPU_MAT_PHONG;
        Copy3(m.albedo, PhongPeek::Diffuse(*p));   // as held: already halved with a glossy lobe
        Copy3(m.glossy, PhongPeek::Glossy(*p));
        m.phong_exponent = PhongPeek::Exponent(*p);
    } else if (auto *p = dynamic_cast<const MicrofacetGGXConductorMaterial *>(am)) {
        m.kind = PG3GPU_MAT_GGX_CONDUCTOR;
        m.alpha = GgxConductorPeek::Alpha(*p);
        m.ior = GgxConductorPeek::Eta(*p);
        m.absorb = GgxConductorPeek::Absorbance(*p);
    } else if (auto *p = dynamic_cast<const MicrofacetGGXDielectricMaterial *>(am)) {
        m.kind = PG3GPU_MAT_GGX_DIELECTRIC;
        m.alpha = GgxDielectricPeek::Alpha(*p);
        m.ior = GgxDielectricPeek::Eta(*p);
    } else if (auto *p = dynamic_cast<const SmoothConductorMaterial *>(am)) {
        m.kind = PG3GPU_MAT_SMOOTH_CONDUCTOR;
        m.ior = SmoothConductorPeek::Eta(*p);
        m.absorb = SmoothConductorPeek::Absorbance(*p);
    } else if (auto *p = dynamic_cast<const SmoothDielectricMaterial *>(am)) {
        m.kind = PG3GPU_MAT_SMOOTH_DIELECTRIC;
        m.ior = SmoothDielectricPeek::Eta(*p);
    } else if (auto *p = dynamic_cast<const SraLayeredMaterial *>(am)) {
        m.kind = PG3GPU_MAT_SRA_LAYERED;
        auto *outer = dynamic_cast<const MicrofacetGGXDielectricMaterial *>(SraPeek::Outer(*p));
        if (!outer) PG3_FATAL_ERROR("GPU renderer: SRA layered material without a GGX dielectric outer layer");
        m.alpha = GgxDielectricPeek::Alpha(*outer);
        m.ior = GgxDielectricPeek::Eta(*outer);
        const AbstractMaterial *in = SraPeek::Inner(*p);
        if (auto *l = dynamic_cast<const LambertMaterial *>(in)) {
            m.inner_kind = PG3GPU_MAT_LAMBERT;
            Copy3(m.albedo, LambertPeek::Reflectance(*l));
        } else if (auto *c = dynamic_cast<const MicrofacetGGXConductorMaterial *>(in)) {
            m.inner_kind = PG3GPU_MAT_GGX_CONDUCTOR;
            m.inner_alpha = GgxConductorPeek::Alpha(*c);
            m.inner_ior = GgxConductorPeek::Eta(*c);
            m.inner_ior_outer = 1.f;
            m.absorb = GgxConductorPeek::Absorbance(*c);
        } else
            PG3_FATAL_ERROR("GPU renderer: SRA layered material with an unsupported inner layer");
        Copy3(m.medium_attenuation, SraPeek::Attenuation(*p));
        m.medium_thickness = SraPeek::Thickness(*p);
    } else
        PG3_FATAL_ERROR("GPU renderer: unsupported material type");
    return m;
}

// The owned arrays behind a pg3gpu_scene (the library copies them in pg3gpu_create).
struct SceneDesc {
    std::vector<pg3gpu_material> materials;
    std::vector<pg3gpu_triangle> triangles;
    std::vector<pg3gpu_sphere> spheres;
    std::vector<pg3gpu_area_light> areaLights;
    std::vector<pg3gpu_point_light> pointLights;
    std::vector<float> envMap;
    pg3gpu_scene desc;
};

// Camera::Setup (src/camera.hxx:13-59) keeps the position, the normalised forward direction,
// the resolution and the raster <-> world matrices. The up direction it was given (its part
// orthogonal to forward, all Setup uses) points from the bottom to the top image row, and
// the horizontal field of view follows from the pixel area 4 tan^2(fov/2) / width^2.
inline pg3gpu_camera TranslateCamera(const Camera &cam)
{
    pg3gpu_camera c;
    std::memset(&c, 0, sizeof c);
    Copy3(c.position, cam.mPosition);
    Copy3(c.forward, cam.mForward);
    const float w = cam.mResolution.x, h = cam.mResolution.y;
    const Vec3f top = cam.RasterToWorld(Vec2f(0.5f * w, 0.f));
    const Vec3f bottom = cam.RasterToWorld(Vec2f(0.5f * w, h));
    Copy3(c.up, Normalize(top - bottom));
    c.width = (uint32_t)w;
    c.height = (uint32_t)h;
    const double tanHalf = std::sqrt((double)cam.mPixelArea) * 0.5 * (double)w;
    c.hfov_deg = (float)(2.0 * std::atan(tanHalf) * 180.0 / 3.14159265358979323846);
    return c;
}

inline void TranslateScene(const Scene &s, SceneDesc &d)
{
    std::memset(&d.desc, 0, sizeof d.desc);
    d.desc.camera = TranslateCamera(s.mCamera);
    for (const AbstractMaterial *am : s.mMaterials) d.materials.push_back(TranslateMaterial(am));

    auto *list = dynamic_cast<const GeometryList *>(s.mGeometry);
    if (!list) PG3_FATAL_ERROR("GPU renderer: the scene geometry is not a GeometryList");
    // triangles whose material maps to an area light become its emitter (src/scene.hxx:42-59)
    std::map<const AbstractLight *, uint32_t> areaOf;
    for (const AbstractGeometry *g : list->mGeometry) {
        if (auto *t = dynamic_cast<const Triangle *>(g)) {
            pg3gpu_triangle tr;
            for (int k = 0; k < 3; ++k) Copy3(tr.p + 3 * k, t->p[k]);
            tr.material = t->mMatId;
            const uint32_t idx = (uint32_t)d.triangles.size();
            d.triangles.push_back(tr);
            auto it = s.mMaterial2Light.find(t->mMatId);
            if (it != s.mMaterial2Light.end()) {
                const AbstractLight *l = s.mLights[it->second].get();
                if (auto *al = dynamic_cast<const AreaLight *>(l)) {
                    if (areaOf.count(l)) PG3_FATAL_ERROR("GPU renderer: an area light with two triangles");
                    areaOf[l] = idx;
                    pg3gpu_area_light a;
                    a.triangle = idx;
                    Copy3(a.radiance, al->mRadiance);
                    d.areaLights.push_back(a);
                }
            }
        } else if (auto *sp = dynamic_cast<const Sphere *>(g)) {
            pg3gpu_sphere q;
            Copy3(q.center, sp->mCenter);
            q.radius = sp->mRadius;
            q.material = sp->mMatId;
            d.spheres.push_back(q);
        } else
            PG3_FATAL_ERROR("GPU renderer: unsupported geometry (nested lists are not translated)");
    }
    d.desc.background = PG3GPU_BG_NONE;
    for (const Scene::TLightSharedPtr &lp : s.mLights) {
        const AbstractLight *l = lp.get();
        if (dynamic_cast<const AreaLight *>(l)) {
            if (!areaOf.count(l)) PG3_FATAL_ERROR("GPU renderer: an area light without a scene triangle");
        } else if (auto *pl = dynamic_cast<const PointLight *>(l)) {
            pg3gpu_point_light p;
            Copy3(p.position, pl->mPosition);
            // SetPower stores intensity = power / (4 pi) (src/lights.hxx:242-245)
            for (int c = 0; c < 3; ++c) p.power[c] = pl->mIntensity.Get(c) * (4.f * Math::kPiF);
            d.pointLights.push_back(p);
        } else if (auto *bl = dynamic_cast<const BackgroundLight *>(l)) {
            if (l != s.mBackgroundLight.get()) PG3_FATAL_ERROR("GPU renderer: a second background light");
            if (bl->mEnvMap) {
                const EnvironmentMapImage *img = EmImage(*bl->mEnvMap);
                if (!img) PG3_FATAL_ERROR("GPU renderer: environment map without an image");
                const uint32_t W = img->Width(), H = img->Height();
                d.envMap.resize((size_t)W * H * 3);
                for (uint32_t y = 0; y < H; ++y)
                    for (uint32_t x = 0; x < W; ++x) Copy3(&d.envMap[((size_t)y * W + x) * 3], img->ElementAt(x, y));
                d.desc.background = PG3GPU_BG_ENVMAP;
                d.desc.env_map = d.envMap.data();
                d.desc.env_width = W;
                d.desc.env_height = H;
            } else {
                d.desc.background = PG3GPU_BG_CONSTANT;
                Copy3(d.desc.background_radiance, bl->mConstantRadiance);
            }
        } else
            PG3_FATAL_ERROR("GPU renderer: unsupported light type");
    }
    d.desc.materials = d.materials.data();
    d.desc.num_materials = (uint32_t)d.materials.size();
    d.desc.triangles = d.triangles.data();
    d.desc.num_triangles = (uint32_t)d.triangles.size();
    d.desc.spheres = d.spheres.data();
    d.desc.num_spheres = (uint32_t)d.spheres.size();
    d.desc.area_lights = d.areaLights.data();
    d.desc.num_area_lights = (uint32_t)d.areaLights.size();
    d.desc.point_lights = d.pointLights.data();
    d.desc.num_point_lights = (uint32_t)d.pointLights.size();
}

// The environment-map sampler this reference build was compiled with (src/hard_config.hxx:17-18)
// and, for the steerable sampler, its subdivision level from the aux parameters (src/em.hxx:56-62;
// minimum = maximum level, the uniform triangulation).
inline void SamplerOptions(const Config &cfg, pg3gpu_options &o)
{
#if defined PG3_USE_ENVMAP_STEERABLE_SAMPLER
    o.em_sampler = PG3GPU_EM_STEERABLE;
    if (cfg.mAuxDbgParams.float2 != cfg.mAuxDbgParams.float3)
        PG3_FATAL_ERROR("GPU renderer: the steerable sampler needs minimum = maximum subdivision level");
    if (cfg.mAuxDbgParams.float2 >= 0.f) o.steer_subdiv_level = (uint32_t)cfg.mAuxDbgParams.float2;
    o.steer_weights = PG3GPU_STEER_WEIGHTS_POINT;   // the reference's vertex weights
#elif defined PG3_USE_ENVMAP_COSINE_SAMPLER
    (void)cfg;
    o.em_sampler = PG3GPU_EM_COSINE;
#else
    (void)cfg;
    o.em_sampler = PG3GPU_EM_CDF;
#endif
}

}  // namespace gpu_shim

class GpuPathTracer : public AbstractRenderer
{
public:
    GpuPathTracer(const Config &aConfig, int32_t aSeed = 1234, int aDevice = 0) : AbstractRenderer(aConfig)
    {
        gpu_shim::SceneDesc scene;
        gpu_shim::TranslateScene(*aConfig.mScene, scene);
        pg3gpu_options o;
        pg3gpu_default_options(&o);
        o.algorithm = (int32_t)aConfig.mAlgorithm;
        o.min_path_length = aConfig.mMinPathLength;
        o.max_path_length = aConfig.mMaxPathLength;
        o.indirect_clipping = aConfig.mIndirectIllumClipping;
        o.splitting_budget = aConfig.mSplittingBudget;
        o.splitting_level = aConfig.mDbgSplittingLevel;
        o.light_to_bsdf_ratio = aConfig.mDbgSplittingLightToBrdfSmplRatio;
        o.seed = (uint64_t)(uint32_t)aSeed;
        gpu_shim::SamplerOptions(aConfig, o);
        if (pg3gpu_create(&scene.desc, &o, aDevice, &mCtx) != PG3GPU_OK)
            PG3_FATAL_ERROR("GPU renderer: %s", pg3gpu_last_error(nullptr));
        mWidth = scene.desc.camera.width;
        mHeight = scene.desc.camera.height;
    }

    ~GpuPathTracer() override
    {
        if (mCtx) pg3gpu_destroy(mCtx);
    }

    GpuPathTracer(const GpuPathTracer &) = delete;

    // One sample per pixel of iteration aIteration (PathTracerBase::RunIteration,
    // src/path_tracer_base.hxx:57-90), queued on the GPU; returns without waiting.
    void RunIteration(const Algorithm aAlgorithm, uint32_t aIteration) override
    {
        RunIterations(aAlgorithm, aIteration, 1);
    }

    // aCount iterations aFirst .. aFirst+aCount-1 in one call: the same image as aCount
    // RunIteration calls, with the launches of all of them batched.
    void RunIterations(const Algorithm aAlgorithm, uint32_t aFirst, uint32_t aCount)
    {
        if (pg3gpu_run_iteration(mCtx, (int32_t)aAlgorithm, aFirst, aCount) != PG3GPU_OK)
            PG3_FATAL_ERROR("GPU renderer: %s", pg3gpu_last_error(mCtx));
        mIterations += aCount;   // GetFramebuffer's 1/iterations scaling and WasUsed()
    }

    // Copies the GPU's accumulated sum into mFramebuffer so that the reference's
    // GetFramebuffer (not virtual) returns sum / iterations. Each double is added as three
    // floats (its leading 24 bits, the next 24, the rest) through the public AddRadiance, whose
    // double accumulator restores it to double precision.
    void Sync()
    {
        const size_t n = (size_t)mWidth * mHeight;
        std::vector<double> mean(3 * n);
        uint64_t iters = 0;
        if (pg3gpu_read_framebuffer(mCtx, mean.data(), mVariance.empty() ? nullptr : mVariance.data(), &iters) !=
            PG3GPU_OK)
            PG3_FATAL_ERROR("GPU renderer: %s", pg3gpu_last_error(mCtx));
        if (iters != mIterations) PG3_FATAL_ERROR("GPU renderer: iteration count mismatch");
        mFramebuffer.Clear();
        for (size_t i = 0; i < n; ++i) {
            float part[3][3];
            for (int c = 0; c < 3; ++c) {
                double v = mean[3 * i + c] * (double)mIterations;
                for (int k = 0; k < 3; ++k) {
                    part[k][c] = (float)v;
                    v -= (double)part[k][c];
                }
            }
            for (int k = 0; k < 3; ++k) {
                SpectrumF s;
                s.SetSRGBLight(part[k][0], part[k][1], part[k][2]);
                mFramebuffer.AddRadiance((uint32_t)(i % mWidth), (uint32_t)(i / mWidth), s);
            }
        }
    }

    // Per-pixel sample variance of the radiance estimates (width*height*3 doubles, filled by the
    // next Sync after EnableVariance); not part of the reference's interface.
    void EnableVariance() { mVariance.assign((size_t)mWidth * mHeight * 3, 0.0); }
    const std::vector<double> &Variance() const { return mVariance; }

    pg3gpu_ctx *Context() const { return mCtx; }

private:
    pg3gpu_ctx *mCtx = nullptr;
    uint32_t mWidth = 0, mHeight = 0;
    std::vector<double> mVariance;
};
