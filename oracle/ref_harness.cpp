// Test-infrastructure harness around the reference renderer (oracle only).
//
// Compiled by oracle/build_ref.py against a patched copy of the reference
// headers. It builds a scene from the repository's plain-text scene file
// directly through the reference's public Scene members
// (src/scene.hxx:1276-1289), runs K independent reference renderers of the
// requested algorithm (PathTracer, src/path_tracer.hxx:5-14; DirectIllumination,
// src/direct_illumination.hxx:5-13; EyeLight; NormalVisualiser) with seeds base+i exactly like
// Render() does (src/pg3render.cxx:65-70, 112-128), and writes
//   * the mean image over all K*N iterations (double RGB), and
//   * the per-pixel variance of the K per-renderer means (for z-tests).
// With --time it only renders and reports wall-clock Msamples/s. --preset ID W H EM replaces
// the file's scene by the reference's own built-in scene number ID (Scene::LoadCornellBox with
// g_SceneConfigs[ID], src/scene.hxx:176-1000, src/config.hxx:45-115) at W x H with environment
// map type EM; the file then only supplies the options record. --save-image P writes the
// first renderer's framebuffer through the reference's own SaveBMP (gamma 2.2) or SaveHDR
// (by P's extension, as src/pg3render.cxx:266-273) and its pixels to P.fb (double RGB).
//
// Scene file format (one record per line, '#' comments):
//   camera px py pz  fx fy fz  ux uy uz  width height hfov_deg
//   lambert r g b
//   ggx_conductor alpha n_inner n_outer k
//   ggx_dielectric alpha n_inner n_outer
//   phong dr dg db gr gg gb exponent         (diffuse part as the material holds it)
//   smooth_conductor n_inner n_outer k
//   smooth_dielectric n_inner n_outer
//   sra outer_alpha outer_n outer_no (lambert r g b | ggx_conductor alpha n no k) att_r att_g att_b thickness
//   triangle x0 y0 z0 x1 y1 z1 x2 y2 z2 material
//   sphere cx cy cz radius material
//   area_light x0 y0 z0 x1 y1 z1 x2 y2 z2 material Lr Lg Lb
//   point_light x y z power_r power_g power_b
//   background_const r g b
//   background_em path
//   options algorithm(el|nv|dbs|dlsa|dlss|dmis|ptn|pt) min_path_length max_path_length
//           [splitting_budget splitting_level light_to_bsdf_ratio indirect_clipping]
#include "config.hxx"
#include "direct_illumination.hxx"
#include "eye_light.hxx"
#include "normal_visualiser.hxx"
#include "path_tracer.hxx"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct SceneFile {
    Scene *scene = nullptr;
    Algorithm algorithm = kPathTracing;
    uint32_t minPathLength = 1;
    uint32_t maxPathLength = 0;
    uint32_t splittingBudget = 1;
    float splittingLevel = 1.f, lightToBrdfRatio = 1.f, clipping = 0.f;
};

void Fail(const std::string &msg)
{
    std::fprintf(stderr, "ref_harness: %s\n", msg.c_str());
    std::exit(2);
}

SceneFile LoadScene(const char *path, const AuxDbgParams &aux)
{
    std::ifstream in(path);
    if (!in) Fail(std::string("cannot open scene ") + path);
    SceneFile sf;
    Scene *s = new Scene;
    GeometryList *geom = new GeometryList;
    s->mGeometry = geom;
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string kind;
        if (!(ls >> kind) || kind[0] == '#') continue;
        if (kind == "camera") {
            float p[3], f[3], u[3], w, h, fov;
            ls >> p[0] >> p[1] >> p[2] >> f[0] >> f[1] >> f[2] >> u[0] >> u[1] >> u[2] >> w >> h >> fov;
            s->mCamera.Setup(Vec3f(p[0], p[1], p[2]), Vec3f(f[0], f[1], f[2]), Vec3f(u[0], u[1], u[2]),
                             Vec2f(w, h), fov);
        } else if (kind == "lambert") {
            float r, g, b;
            ls >> r >> g >> b;
            SpectrumF refl;
            refl.SetSRGBAttenuation(r, g, b);
            s->mMaterials.push_back(new LambertMaterial(refl));
        } else if (kind == "ggx_conductor") {
            float a, n, no, k;
            ls >> a >> n >> no >> k;
            s->mMaterials.push_back(new MicrofacetGGXConductorMaterial(a, n, no, k));
        } else if (kind == "ggx_dielectric") {
            float a, n, no;
            ls >> a >> n >> no;
            s->mMaterials.push_back(new MicrofacetGGXDielectricMaterial(a, n, no));
        } else if (kind == "phong") {
            // PhongMaterial halves the diffuse part when the glossy lobe is on: hand it twice
            // the held value (exact in binary floating point)
            float d[3], g[3], e;
            ls >> d[0] >> d[1] >> d[2] >> g[0] >> g[1] >> g[2] >> e;
            const bool glossy = g[0] != 0.f || g[1] != 0.f || g[2] != 0.f;
            const float k = glossy ? 2.f : 1.f;
            SpectrumF dr, gr;
            dr.SetSRGBAttenuation(k * d[0], k * d[1], k * d[2]);
            gr.SetSRGBAttenuation(g[0], g[1], g[2]);
            s->mMaterials.push_back(new PhongMaterial(dr, gr, e, 1u, glossy ? 1u : 0u));
        } else if (kind == "smooth_conductor") {
            float n, no, k;
            ls >> n >> no >> k;
            s->mMaterials.push_back(new SmoothConductorMaterial(n, no, k));
        } else if (kind == "smooth_dielectric") {
            float n, no;
            ls >> n >> no;
            s->mMaterials.push_back(new SmoothDielectricMaterial(n, no));
        } else if (kind == "sra") {
            float a, n, no;
            std::string ik;
            ls >> a >> n >> no >> ik;
            AbstractMaterial *inner = nullptr;
            if (ik == "lambert") {
                float r, g, b;
                ls >> r >> g >> b;
                SpectrumF refl;
                refl.SetSRGBAttenuation(r, g, b);
                inner = new LambertMaterial(refl);
            } else if (ik == "ggx_conductor") {
                float ia, in, ino, k;
                ls >> ia >> in >> ino >> k;
                inner = new MicrofacetGGXConductorMaterial(ia, in, ino, k);
            } else {
                Fail("sra: unknown inner layer " + ik);
            }
            float att[3], th;
            ls >> att[0] >> att[1] >> att[2] >> th;
            SpectrumF medium;
            medium.SetSRGBAttenuation(att[0], att[1], att[2]);
            s->mMaterials.push_back(
                new SraLayeredMaterial(new MicrofacetGGXDielectricMaterial(a, n, no), inner, medium, th, aux));
        } else if (kind == "point_light") {
            float p[3], w[3];
            ls >> p[0] >> p[1] >> p[2] >> w[0] >> w[1] >> w[2];
            PointLight *light = new PointLight(Vec3f(p[0], p[1], p[2]));
            SpectrumF power;
            power.SetSRGBLight(w[0], w[1], w[2]);
            light->SetPower(power);
            s->mLights.push_back(Scene::TLightSharedPtr(light));
        } else if (kind == "triangle" || kind == "area_light") {
            float v[9];
            int mat;
            for (float &x : v) ls >> x;
            ls >> mat;
            Vec3f p0(v[0], v[1], v[2]), p1(v[3], v[4], v[5]), p2(v[6], v[7], v[8]);
            geom->mGeometry.push_back(new Triangle(p0, p1, p2, mat));
            if (kind == "area_light") {
                float L[3];
                ls >> L[0] >> L[1] >> L[2];
                AreaLight *light = new AreaLight(p0, p1, p2);
                light->mRadiance.SetSRGBLight(L[0], L[1], L[2]);
                s->mLights.push_back(Scene::TLightSharedPtr(light));
                s->mMaterial2Light.insert(std::make_pair(mat, (int32_t)s->mLights.size() - 1));
            }
        } else if (kind == "sphere") {
            float c[3], r;
            int mat;
            ls >> c[0] >> c[1] >> c[2] >> r >> mat;
            geom->mGeometry.push_back(new Sphere(Vec3f(c[0], c[1], c[2]), r, mat));
        } else if (kind == "background_const" || kind == "background_em") {
            BackgroundLight *light = new BackgroundLight();
            if (kind == "background_const") {
                float r, g, b;
                ls >> r >> g >> b;
                SpectrumF L;
                L.SetSRGBLight(r, g, b);
                light->SetConstantRadiance(L);
            } else {
                std::string em;
                ls >> em;
                light->LoadEnvironmentMap(em, 0.0f, 1.0f, true, aux);
            }
            s->mBackgroundLight = Scene::TLightSharedPtr(light);
            s->mLights.push_back(s->mBackgroundLight);
            s->mBackgroundLightId = (int32_t)(s->mLights.size() - 1);
        } else if (kind == "options") {
            std::string alg;
            ls >> alg >> sf.minPathLength >> sf.maxPathLength;
            bool known = false;
            for (int a = 0; a < (int)kAlgorithmCount; ++a)
                if (alg == Config::GetAcronym((Algorithm)a)) { sf.algorithm = (Algorithm)a; known = true; }
            if (!known) Fail("unknown algorithm " + alg);
            uint32_t sb;
            float lvl, ratio, clip;
            if (ls >> sb >> lvl >> ratio >> clip) {
                sf.splittingBudget = sb;
                sf.splittingLevel = lvl;
                sf.lightToBrdfRatio = ratio;
                sf.clipping = clip;
            }
        } else {
            Fail("unknown scene record " + kind);
        }
    }
    sf.scene = s;
    return sf;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr,
                     "usage: %s scene.txt out.bin [--renderers K] [--iters N] [--threads T] [--seed S]"
                     " [--time] [--em-params maxErr minLevel maxLevel]\n", argv[0]);
        return 2;
    }
    const char *scenePath = argv[1];
    const char *outPath = argv[2];
    int K = 8, N = 1, T = 0, seed = 1234;
    bool timeOnly = false;
    std::string saveImage;
    int presetId = -1, presetW = 0, presetH = 0, presetEm = 0;
    AuxDbgParams aux;
    for (int i = 3; i < argc; ++i) {
        std::string a(argv[i]);
        if (a == "--renderers") K = std::atoi(argv[++i]);
        else if (a == "--iters") N = std::atoi(argv[++i]);
        else if (a == "--threads") T = std::atoi(argv[++i]);
        else if (a == "--seed") seed = std::atoi(argv[++i]);
        else if (a == "--time") timeOnly = true;
        else if (a == "--save-image") saveImage = argv[++i];
        else if (a == "--preset") {
            presetId = std::atoi(argv[++i]);
            presetW = std::atoi(argv[++i]);
            presetH = std::atoi(argv[++i]);
            presetEm = std::atoi(argv[++i]);
        }
        else if (a == "--em-params") {
            aux.float1 = (float)std::atof(argv[++i]);
            aux.float2 = (float)std::atof(argv[++i]);
            aux.float3 = (float)std::atof(argv[++i]);
        } else Fail("unknown option " + a);
    }
    if (T <= 0) T = omp_get_num_procs();

    SceneFile sf = LoadScene(scenePath, aux);
    if (presetId >= 0) {
        if (presetId >= (int)(sizeof(g_SceneConfigs) / sizeof(g_SceneConfigs[0]))) Fail("preset id out of range");
        delete sf.scene;
        sf.scene = new Scene;
        sf.scene->LoadCornellBox(Vec2i(presetW, presetH), aux, g_SceneConfigs[presetId],
                                 Scene::EnvironmentMapType(presetEm));
    }

    // Options as the reference's Config carries them (src/config.hxx:1100-1137); -sb 1 -iic 0
    // unless the scene file's options record gives them.
    Config config;
    config.mScene = sf.scene;
    config.mAlgorithm = sf.algorithm;
    config.mMinPathLength = sf.minPathLength;
    config.mMaxPathLength = sf.maxPathLength;
    config.mIndirectIllumClipping = sf.clipping;
    config.mSplittingBudget = sf.splittingBudget;
    config.mDbgSplittingLevel = sf.splittingLevel;
    config.mDbgSplittingLightToBrdfSmplRatio = sf.lightToBrdfRatio;
    config.mIterations = N;
    config.mNumThreads = T;
    config.mQuietMode = true;
    config.mBaseSeed = seed;

    const uint32_t W = (uint32_t)sf.scene->mCamera.mResolution.x;
    const uint32_t H = (uint32_t)sf.scene->mCamera.mResolution.y;
    const size_t npx = (size_t)W * H;

    // the renderer CreateRenderer picks for the algorithm (src/pg3render.cxx:24-50)
    std::vector<AbstractRenderer *> renderers(K);
    for (int i = 0; i < K; ++i) {
        switch (sf.algorithm) {
        case kEyeLight: renderers[i] = new EyeLight(config, seed + i); break;
        case kNormalVisualiser: renderers[i] = new NormalVisualiser(config, seed + i); break;
        case kDirectIllumBsdfSampling:
        case kDirectIllumLightSamplingAll:
        case kDirectIllumLightSamplingSingle:
        case kDirectIllumMis: renderers[i] = new DirectIllumination(config, seed + i); break;
        default: renderers[i] = new PathTracer(config, seed + i); break;
        }
    }

    omp_set_num_threads(T);
    const auto t0 = std::chrono::steady_clock::now();
    // Each renderer is used by one thread at a time, as in Render() (src/pg3render.cxx:84-128).
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < K; ++i)
        for (int it = 0; it < N; ++it)
            renderers[i]->RunIteration(sf.algorithm, (uint32_t)it);
    const auto t1 = std::chrono::steady_clock::now();
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    const double samples = (double)npx * K * N;
    std::printf("{\"seconds\": %.6f, \"samples\": %.0f, \"msamples_per_s\": %.6f, \"threads\": %d}\n",
                secs, samples, samples / secs / 1e6, T);

    if (!saveImage.empty()) {
        Framebuffer fb;
        renderers[0]->GetFramebuffer(fb);
        const std::string ext = saveImage.substr(saveImage.size() - 3, 3);
        if (ext == "bmp") fb.SaveBMP(saveImage.c_str(), 2.2f);
        else if (ext == "hdr") fb.SaveHDR(saveImage.c_str());
        else Fail("--save-image wants a .bmp or .hdr path");
        const std::vector<FramebufferSpectrum> *rad = reinterpret_cast<const std::vector<FramebufferSpectrum> *>(&fb);
        FILE *f = std::fopen((saveImage + ".fb").c_str(), "wb");
        if (!f) Fail("cannot write the framebuffer dump");
        for (size_t p = 0; p < npx; ++p)
            for (int c = 0; c < 3; ++c) {
                const double v = (*rad)[p].Get(c);
                std::fwrite(&v, 8, 1, f);
            }
        std::fclose(f);
    }

    if (!timeOnly) {
        std::vector<double> mean(npx * 3, 0.0), m2(npx * 3, 0.0);
        for (int i = 0; i < K; ++i) {
            Framebuffer fb;
            renderers[i]->GetFramebuffer(fb);  // already divided by N (src/renderer.hxx:255-262)
            // Framebuffer's only storage is a private std::vector of spectra declared as
            // its first member (src/frame_buffer.hxx:202-207); it is a standard-layout
            // class, so that vector sits at offset 0.
            static_assert(std::is_standard_layout<Framebuffer>::value, "layout");
            const std::vector<FramebufferSpectrum> *rad =
                reinterpret_cast<const std::vector<FramebufferSpectrum> *>(&fb);
            for (size_t p = 0; p < npx; ++p)
                for (int c = 0; c < 3; ++c) {
                    const double v = (*rad)[p].Get(c);
                    const double d = v - mean[p * 3 + c];
                    mean[p * 3 + c] += d / (i + 1);
                    m2[p * 3 + c] += d * (v - mean[p * 3 + c]);
                }
        }
        FILE *f = std::fopen(outPath, "wb");
        if (!f) Fail("cannot write output");
        const uint32_t hdr[4] = {W, H, (uint32_t)K, (uint32_t)N};
        std::fwrite(hdr, 4, 4, f);
        std::fwrite(mean.data(), 8, mean.size(), f);
        for (auto &v : m2) v = (K > 1) ? v / (K - 1) : 0.0;  // variance of one renderer's mean
        std::fwrite(m2.data(), 8, m2.size(), f);
        std::fclose(f);
    }
    for (auto *r : renderers) delete r;
    delete sf.scene;
    return 0;
}
