// pg3render_gpu -- PG3Render's own command line and render loop with the GPU renderer.
//
// This is what the reference's main program does (src/pg3render.cxx:54-174, 205-285) once its
// renderer factory returns GpuPathTracer (gpu_path_tracer.hxx): the reference's Config parses
// the reference's command line (src/config.hxx:553-1098) and builds the scene with the
// reference's own Scene::LoadCornellBox (src/scene.hxx:176-1000); one renderer (one GPU
// context, the -j 1 case) runs RunIteration(algorithm, iteration) once per iteration, as the
// iteration loop of Render() does, and the framebuffer comes back through the reference's
// AbstractRenderer::GetFramebuffer. It is built against the reference's headers (which this
// repository does not contain) by oracle/build_ref.py.
//
// Options of this program on top of the reference's:
//   --res W H        render the -s scene at W x H (the reference's command line fixes 512 x 512)
//   --out PATH       write uint32 W, H, iterations, then the mean image and the per-pixel sample
//                    variance (W*H*3 doubles each, row 0 at the top)
//   --batch N        N iterations per RunIterations call instead of one RunIteration each
//   --device D       CUDA device
//   --dump-scene P   write the scene as GpuPathTracer translates it (JSON) and exit without
//                    rendering (needs no GPU)
// It prints one JSON line: seconds of the render loop (first call to the synchronised
// framebuffer), samples and Msamples/s.
#include "config.hxx"
#include "gpu_path_tracer.hxx"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

void Fail(const std::string &msg)
{
    std::fprintf(stderr, "pg3render_gpu: %s\n", msg.c_str());
    std::exit(2);
}

void PutFloats(FILE *f, const float *v, int n)
{
    std::fputc('[', f);
    for (int i = 0; i < n; ++i) std::fprintf(f, "%s%.9g", i ? ", " : "", v[i]);
    std::fputc(']', f);
}

// The translated scene description as JSON (field names of include/pg3gpu.h).
void DumpScene(const gpu_shim::SceneDesc &d, const char *path)
{
    FILE *f = std::fopen(path, "w");
    if (!f) Fail(std::string("cannot write ") + path);
    const pg3gpu_camera &c = d.desc.camera;
    std::fprintf(f, "{\"camera\": {\"position\": ");
    PutFloats(f, c.position, 3);
    std::fprintf(f, ", \"forward\": ");
    PutFloats(f, c.forward, 3);
    std::fprintf(f, ", \"up\": ");
    PutFloats(f, c.up, 3);
    std::fprintf(f, ", \"width\": %u, \"height\": %u, \"hfov_deg\": %.9g},\n", c.width, c.height, c.hfov_deg);
    std::fprintf(f, "\"materials\": [");
    for (size_t i = 0; i < d.materials.size(); ++i) {
        const pg3gpu_material &m = d.materials[i];
        std::fprintf(f, "%s\n {\"kind\": %d, \"albedo\": ", i ? "," : "", m.kind);
        PutFloats(f, m.albedo, 3);
        std::fprintf(f, ", \"alpha\": %.9g, \"ior\": %.9g, \"ior_outer\": %.9g, \"absorb\": %.9g, \"glossy\": ",
                     m.alpha, m.ior, m.ior_outer, m.absorb);
        PutFloats(f, m.glossy, 3);
        std::fprintf(f, ", \"phong_exponent\": %.9g, \"inner_kind\": %d, \"inner_alpha\": %.9g, \"inner_ior\": %.9g, "
                     "\"medium_attenuation\": ", m.phong_exponent, m.inner_kind, m.inner_alpha, m.inner_ior);
        PutFloats(f, m.medium_attenuation, 3);
        std::fprintf(f, ", \"medium_thickness\": %.9g}", m.medium_thickness);
    }
    std::fprintf(f, "],\n\"triangles\": [");
    for (size_t i = 0; i < d.triangles.size(); ++i) {
        std::fprintf(f, "%s\n {\"p\": ", i ? "," : "");
        PutFloats(f, d.triangles[i].p, 9);
        std::fprintf(f, ", \"material\": %d}", d.triangles[i].material);
    }
    std::fprintf(f, "],\n\"spheres\": [");
    for (size_t i = 0; i < d.spheres.size(); ++i) {
        std::fprintf(f, "%s\n {\"center\": ", i ? "," : "");
        PutFloats(f, d.spheres[i].center, 3);
        std::fprintf(f, ", \"radius\": %.9g, \"material\": %d}", d.spheres[i].radius, d.spheres[i].material);
    }
    std::fprintf(f, "],\n\"area_lights\": [");
    for (size_t i = 0; i < d.areaLights.size(); ++i) {
        std::fprintf(f, "%s\n {\"triangle\": %u, \"radiance\": ", i ? "," : "", d.areaLights[i].triangle);
        PutFloats(f, d.areaLights[i].radiance, 3);
        std::fputc('}', f);
    }
    std::fprintf(f, "],\n\"point_lights\": [");
    for (size_t i = 0; i < d.pointLights.size(); ++i) {
        std::fprintf(f, "%s\n {\"position\": ", i ? "," : "");
        PutFloats(f, d.pointLights[i].position, 3);
        std::fprintf(f, ", \"power\": ");
        PutFloats(f, d.pointLights[i].power, 3);
        std::fputc('}', f);
    }
    std::fprintf(f, "],\n\"background\": %d, \"background_radiance\": ", d.desc.background);
    PutFloats(f, d.desc.background_radiance, 3);
    std::fprintf(f, ", \"env_width\": %u, \"env_height\": %u}\n", d.desc.env_width, d.desc.env_height);
    std::fclose(f);
}

}  // namespace

int main(int argc, char **argv)
{
    int resW = 0, resH = 0, batch = 1, device = 0;
    std::string outPath, dumpPath;
    int sceneId = 0, emId = Scene::kEMDefault;
    std::vector<const char *> refArgs{argv[0]};
    for (int i = 1; i < argc; ++i) {
        const std::string a(argv[i]);
        auto need = [&](int k) {
            if (i + k >= argc) Fail("missing value after " + a);
        };
        if (a == "--res") {
            need(2);
            resW = std::atoi(argv[++i]);
            resH = std::atoi(argv[++i]);
        } else if (a == "--out") {
            need(1);
            outPath = argv[++i];
        } else if (a == "--batch") {
            need(1);
            batch = std::atoi(argv[++i]);
        } else if (a == "--device") {
            need(1);
            device = std::atoi(argv[++i]);
        } else if (a == "--dump-scene") {
            need(1);
            dumpPath = argv[++i];
        } else {
            if (a == "-s" && i + 1 < argc) sceneId = std::atoi(argv[i + 1]);
            if (a == "-em" && i + 1 < argc) emId = std::atoi(argv[i + 1]);
            refArgs.push_back(argv[i]);
        }
    }
    if (batch < 1) Fail("--batch must be >= 1");

    Config config;
    if (!config.ProcessCommandline((int32_t)refArgs.size(), refArgs.data())) return 1;
    if (resW > 0 && resH > 0) {
        // the same scene as -s / -em, built by the reference at the requested resolution
        delete config.mScene;
        Scene *scene = new Scene;
        scene->LoadCornellBox(Vec2i(resW, resH), config.mAuxDbgParams, g_SceneConfigs[sceneId],
                              Scene::EnvironmentMapType(emId));
        config.mScene = scene;
    }
    if (!dumpPath.empty()) {
        gpu_shim::SceneDesc d;
        gpu_shim::TranslateScene(*config.mScene, d);
        DumpScene(d, dumpPath.c_str());
        delete config.mScene;
        return 0;
    }
    Framebuffer fb;
    config.mFramebuffer = &fb;

    GpuPathTracer renderer(config, config.mBaseSeed, device);
    if (!outPath.empty()) renderer.EnableVariance();

    const auto t0 = std::chrono::steady_clock::now();
    const uint32_t iterations = (uint32_t)config.mIterations;
    for (uint32_t it = 0; it < iterations;) {
        if (batch == 1) {
            renderer.RunIteration(config.mAlgorithm, it);   // Render()'s iteration loop
            ++it;
        } else {
            const uint32_t n = std::min<uint32_t>((uint32_t)batch, iterations - it);
            renderer.RunIterations(config.mAlgorithm, it, n);
            it += n;
        }
    }
    renderer.Sync();   // waits for the GPU
    const auto t1 = std::chrono::steady_clock::now();

    // the merge of Render() (src/pg3render.cxx:136-162) with one used renderer
    if (!renderer.WasUsed()) Fail("no iteration ran");
    renderer.GetFramebuffer(*config.mFramebuffer);
    config.mFramebuffer->Scale(FramebufferFloat(1.));

    const uint32_t W = (uint32_t)config.mScene->mCamera.mResolution.x;
    const uint32_t H = (uint32_t)config.mScene->mCamera.mResolution.y;
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    const double samples = (double)W * H * iterations;
    std::printf("{\"seconds\": %.6f, \"samples\": %.0f, \"msamples_per_s\": %.6f, \"iterations\": %u, "
                "\"batch\": %d, \"scene\": \"%s\"}\n",
                secs, samples, samples / secs / 1e6, iterations, batch, config.mScene->mSceneAcronym.c_str());

    if (!outPath.empty()) {
        // Framebuffer's only storage is a private std::vector of spectra declared as its first
        // member (src/frame_buffer.hxx:202-207); it is a standard-layout class, so that vector
        // sits at offset 0.
        static_assert(std::is_standard_layout<Framebuffer>::value, "layout");
        const std::vector<FramebufferSpectrum> *rad = reinterpret_cast<const std::vector<FramebufferSpectrum> *>(&fb);
        if (rad->size() != (size_t)W * H) Fail("framebuffer size");
        FILE *f = std::fopen(outPath.c_str(), "wb");
        if (!f) Fail("cannot write " + outPath);
        const uint32_t hdr[3] = {W, H, iterations};
        std::fwrite(hdr, 4, 3, f);
        for (size_t p = 0; p < (size_t)W * H; ++p)
            for (int c = 0; c < 3; ++c) {
                const double v = (*rad)[p].Get(c);
                std::fwrite(&v, 8, 1, f);
            }
        std::fwrite(renderer.Variance().data(), 8, renderer.Variance().size(), f);
        std::fclose(f);
    }
    delete config.mScene;
    return 0;
}
