// Host-side scene preparation: validation, camera basis, material records,
// light table and the environment-map sampling tables, in device layout.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pg3gpu.h"
#include "pg3_scene_view.h"
#include "pg3_steerable.h"

namespace pg3 {

struct HostScene {
    SceneView view{};                    // counts, camera, options (device pointers filled later)
    std::vector<float4> tri;
    std::vector<int> triMat;
    std::vector<float4> sph;
    std::vector<int> sphMat;
    std::vector<DevMaterial> mats;
    std::vector<int> mat2light;
    std::vector<DevAreaLight> lights;
    const float *emRgb = nullptr;        // the caller's map (RGB, validated); widened to float4 on the device
    size_t emTexels = 0;
    std::vector<float> emMarg, emCond;
    std::vector<float> bgShL;            // 9 SH coefficients of the map's luminance (picking estimate)
    std::shared_ptr<const SteerGeom> steer;   // steerable sampler geometry (uniform levels: the shared,
                                              // process-lifetime build; adaptive: this scene's); its
                                              // weights are built on the device
    bool hasSteer = false;
    uint32_t kindMask = 0;               // material kinds present (bit per PG3GPU_MAT_* kind)
    uint32_t numPointLights = 0;
};

// pg3_image.cpp: writes a mean image as BMP or Radiance HDR by the path's extension.
int writeImage(const double *rgb, uint32_t width, uint32_t height, const char *path, float gamma, std::string &err);

// Returns PG3GPU_OK or an error status with a message in err.
int prepareScene(const pg3gpu_scene &scene, const pg3gpu_options &opts, HostScene &out, std::string &err);

// Environment-map CDF tables of the reference's spherical sampler
// (src/em_simple_spherical_sampler.hxx:117-152, src/distribution.hxx:45-74, 484-501):
// marg has H+1 entries, cond H rows of W+1 entries.
void buildEmCdf(const float *rgb, uint32_t W, uint32_t H, std::vector<float> &marg, std::vector<float> &cond);

// 9 SH coefficients of the map's texel luminance (basis of the steerable sampler), integrated
// over the texels' solid angles: with the clamped-cosine coefficients of a normal n, their dot
// product estimates the irradiance at n (the background's light-picking estimate).
void emShCoefficients(const float *rgb, uint32_t W, uint32_t H, std::vector<float> &out);

}  // namespace pg3
