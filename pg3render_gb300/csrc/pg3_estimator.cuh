// Path estimators of the hot path as per-thread device functions.
//
// The reference evaluates EstimateIncomingRadiancePT recursively, one call per
// path vertex (src/path_tracer.hxx:167-430). With one BSDF and one light
// sample per vertex (splitting budget 1) the recursion is a chain, so it is
// unrolled here into a loop that carries, from each vertex to the next:
//   beta   - the throughput of everything the child vertex reflects
//            (indirect factor att*cos/(pdf*rr*compProb), :372-405),
//   ew     - the weight of the child's emission, i.e. the parent's
//            throughput times att*cos/(pdf*compProb) without the roulette
//            factor (direct term, :327-369),
//   the parent's BSDF pdf, Dirac flag, position, normal and light-estimate
//   sum, which the MIS weight of an emitter hit needs (:338-356).
// Random numbers are drawn per (pixel, sample, vertex, group) so the loop
// order does not change which numbers a decision uses.
#pragma once

#include "pg3_device.cuh"
#include "pg3_steer.cuh"
#include "pg3_traverse.cuh"

namespace pg3 {

struct PathCounters {
    uint32_t ext = 0, shadow = 0, rr = 0, bg = 0, blocker = 0, maxl = 0, safety = 0;
};

// MISWeight2Power with both sample counts 1 (src/path_tracer_base.hxx:522-541)
PG3_DI float misPower(float a, float b)
{
    const float a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}

// Sum of the area lights' contribution estimates at a vertex (src/path_tracer_base.hxx:216-232).
PG3_DI float estimateSum(const SceneView &S, float3 pt, float3 n)
{
    float sum = 0.f;
    for (uint32_t i = 0; i < S.nArea; ++i) sum += areaEstimate(S.lights[i], pt, n);
    return sum;
}

// PickSingleLight (src/path_tracer_base.hxx:191-257); est sum computed by the caller.
PG3_DI void pickLight(const SceneView &S, float3 pt, float3 n, float sum, float u, int &id, float &prob)
{
    const uint32_t cnt = S.lightCount;
    if (cnt == 0) { id = -1; return; }
    if (cnt == 1) { id = 0; prob = 1.f; return; }
    if (sum > 0.f) {
        const float r = u * sum;
        float cum = 0.f, e = 0.f;
        uint32_t l = 0;
        for (; l < S.nArea; ++l) {
            e = areaEstimate(S.lights[l], pt, n);
            cum += e;
            if (!(r > cum)) break;
        }
        if (l >= S.nArea) { l = S.nArea - 1; }
        id = (int)l;
        prob = e / sum;
    } else {
        id = min((int)(u * cnt), (int)cnt - 1);
        prob = 1.f / cnt;
    }
}
// LightPickingProbability (src/path_tracer_base.hxx:260-313)
PG3_DI float pickProb(const SceneView &S, float3 pt, float3 n, float sum, int id)
{
    const uint32_t cnt = S.lightCount;
    if (cnt <= 1) return cnt == 1 ? 1.f : 0.f;
    if (!(sum > 0.f)) return 1.f / cnt;
    return areaEstimate(S.lights[id], pt, n) / sum;
}

// Background emission and its light-sampling pdf for MIS (src/lights.hxx:379-407,
// src/em.hxx:87-121).
// EMK selects the environment-map sampler at compile time (-1: read it from the scene), so a
// specialised kernel carries only the sampler it uses.
template <int EMK = -1>
PG3_DI float3 bgEmission(const SceneView &S, float3 dir, bool wantPdf, const Frame &pf, float &pdf)
{
    const int em = (EMK >= 0) ? EMK : S.emSampler;
    if (S.bgKind == kBgEnvMap) {
        const float3 L = emEvaluateDir(S, dir);
        if (wantPdf)
            pdf = (em == kEmCdf) ? emCdfPdf(S, dir)
                  : (em == kEmSteerable) ? steerPdf(S.steer, dir, pf.z) : cosSpherePdfFront(toLocal(pf, dir));
        return L;
    }
    if (wantPdf) pdf = cosSpherePdfFront(toLocal(pf, dir));
    return S.bgConst;
}
// BackgroundLight::SampleIllumination (src/lights.hxx:424-445)
template <int EMK = -1>
PG3_DI void bgSample(const SceneView &S, const Frame &f, float u0, float u1, float u2, float3 &wig, float &pdfW,
                     float3 &radCos)
{
    const int em = (EMK >= 0) ? EMK : S.emSampler;
    if (S.bgKind == kBgEnvMap && em == kEmCdf) {
        emCdfSample(S, f.z, u0, u1, wig, pdfW, radCos);
        return;
    }
    if (S.bgKind == kBgEnvMap && em == kEmSteerable) {
        steerSample(S, f.z, u0, u1, u2, wig, pdfW, radCos);
        return;
    }
    const float3 wil = sampleCosHemisphere(u0, u1, pdfW);   // cosine sampler, front side only
    wig = toWorld(f, wil);
    const float3 L = (S.bgKind == kBgEnvMap) ? emEvaluateDir(S, wig) : S.bgConst;
    radCos = L * fabsf(wil.z);
}

// One camera path of the NEE + MIS path tracer (algorithm kPathTracing).
PG3_DI float3 tracePath(const SceneView &S, uint32_t pixel, uint32_t sample, PathCounters &pc)
{
    const uint32_t px = pixel % S.width, py = pixel / S.width;
    const Rand4 rc = draw(S, pixel, sample, 0, 0);
    const float nx = ((float)px + rc.a) * (2.f / S.width) - 1.f;
    const float ny = ((float)py + rc.b) * (2.f / S.height) - 1.f;
    float3 dir = normalize(S.camFwd + S.camRight * (nx * S.tanX) - S.camUp * (ny * S.tanY));
    float3 org = S.camPos;
    float tmin = 0.f;

    float3 L = f3(0.f);
    float3 beta = f3(1.f);       // throughput of the current vertex's reflected radiance
    float3 ew = f3(0.f);         // weight of emission found at the current vertex (from the parent)
    float prevBsdfPdf = 0.f;     // parent's pdfW * compProb
    bool prevFinite = true;
    float3 prevPt = org, prevN = make_float3(0.f, 0.f, 1.f);
    float prevSum = 0.f;
    bool computeRefl = true;

    for (uint32_t pl = 1;; ++pl) {
        ++pc.ext;
        Hit h;
        if (!intersectClosest(S, org, dir, tmin, h)) {
            // background (src/path_tracer.hxx:408-429)
            if (pl >= S.minPL && S.bgKind != kBgNone) {
                float pdf = 0.f;
                const Frame pf = frameFromZ(prevN);
                const float3 Le = bgEmission(S, dir, pl > 1 && prevFinite, pf, pdf);
                if (pl == 1) {
                    L += Le;
                } else if (prevFinite) {
                    const float lp = pdf * pickProb(S, prevPt, prevN, prevSum, S.bgLightId);
                    L += ew * Le * misPower(prevBsdfPdf, lp);
                } else {
                    L += ew * Le;
                }
            }
            if (computeRefl) ++pc.bg;
            break;
        }
        float3 pt, n;
        int matId;
        hitAttributes(S, h, org, dir, pt, n, matId);
        const Frame frame = frameFromZ(n);
        const float3 wol = toLocal(frame, -dir);
        const int lightId = __ldg(&S.mat2light[matId]);

        // emitter hit (src/path_tracer.hxx:198-210, 327-369)
        if (lightId >= 0 && pl >= S.minPL) {
            float pdfA = 0.f;
            const float3 Le = areaEmission(S.lights[lightId], pt, wol.z, org, pdfA);
            if (pl == 1) {
                L += Le;
            } else if (!isZero(Le)) {
                if (prevFinite) {
                    const float lp = pdfA * pickProb(S, prevPt, prevN, prevSum, lightId);
                    L += ew * Le * misPower(prevBsdfPdf, lp);
                } else {
                    L += ew * Le;
                }
            }
        }
        if (!computeRefl) break;
        const DevMaterial mat = loadMat(S, matId);
        if (mat.zeroRefl) { ++pc.blocker; break; }
        if (S.maxPL > 0 && pl >= S.maxPL) { ++pc.maxl; break; }
        if (pl >= kMaxPathLengthHard) { ++pc.safety; break; }

        const Rand4 ra = draw(S, pixel, sample, pl, 0);
        const Rand4 rb = draw(S, pixel, sample, pl, 1);
        const float sum = (S.lightCount > 1) ? estimateSum(S, pt, n) : 0.f;

        // light sample with MIS (src/path_tracer.hxx:250-265, src/path_tracer_base.hxx:350-411)
        if (pl + 1 >= S.minPL) {
            int lid;
            float lprob = 0.f;
            pickLight(S, pt, n, sum, ra.a, lid, lprob);
            if (lid >= 0) {
                float3 wig, smp;
                float dist, pdfW;
                if (lid == S.bgLightId) {
                    bgSample(S, frame, ra.b, ra.c, ra.d, wig, pdfW, smp);
                    dist = kFloatMax;
                } else {
                    areaSample(S.lights[lid], pt, n, ra.b, ra.c, wig, dist, smp, pdfW);
                }
                if (maxc(smp) > 0.f) {
                    ++pc.shadow;
                    if (!occludedAny(S, pt, wig, dist)) {
                        BsdfRec br;
                        evalBsdf(mat, toLocal(frame, wig), wol, br);
                        const float lightPdf = pdfW * lprob;
                        L += beta * (smp * br.att) * (misPower(lightPdf, br.pdfW * br.compProb) / lightPdf);
                    }
                }
            }
        }

        // Russian roulette (src/path_tracer.hxx:267-303)
        float rrProb = 1.0f;
        bool cut = false;
        if (S.maxPL == 0 || (S.rrMinPL > 0 && pl >= S.rrMinPL)) {
            rrProb = mat.rrProb;
            cut = rb.a > rrProb;
        }

        // BSDF sample (src/path_tracer.hxx:305-322)
        BsdfRec br;
        sampleBsdf(mat, wol, rb.b, rb.c, rb.d, br);
        if (isBlocker(br)) { ++pc.blocker; break; }
        const bool finite = br.pdfW != infF();
        const float cosAbs = fabsf(br.wil.z);
        const float3 f = finite ? br.att * (cosAbs / (br.pdfW * br.compProb)) : br.att / br.compProb;
        ew = beta * f;
        beta = ew / rrProb;
        prevBsdfPdf = br.pdfW * br.compProb;
        prevFinite = finite;
        prevPt = pt;
        prevN = n;
        prevSum = sum;
        computeRefl = !cut;
        if (cut) ++pc.rr;
        org = pt;
        dir = toWorld(frame, br.wil);
        tmin = epsRayCos(cosAbs);
    }
    return L;
}

// Light sample of light `lid` (area: src/lights.hxx:114-131; background: :424-445).
PG3_DI void sampleLightAt(const SceneView &S, int lid, float3 pt, const Frame &frame, float3 n, float u0, float u1,
                          float u2, float3 &wig, float &dist, float3 &smp, float &pdfW)
{
    if (lid == S.bgLightId) {
        bgSample(S, frame, u0, u1, u2, wig, pdfW, smp);
        dist = kFloatMax;
    } else {
        areaSample(S.lights[lid], pt, n, u0, u1, wig, dist, smp, pdfW);
    }
}

// GetDirectRadianceFromDirection (src/path_tracer_base.hxx:92-154): radiance arriving along
// the local direction wil, its light-sampling pdf and the light's id (-1: none).
PG3_DI float3 directFromDirection(const SceneView &S, float3 pt, const Frame &frame, float3 wil, float &pdfW,
                                  int &lightId)
{
    const float3 wig = toWorld(frame, wil);
    Hit h;
    lightId = -1;
    pdfW = 0.f;
    if (intersectClosest(S, pt, wig, epsRayCos(wil.z), h)) {
        float3 lp, ln;
        int mat;
        hitAttributes(S, h, pt, wig, lp, ln, mat);
        const int lid = __ldg(&S.mat2light[mat]);
        if (lid < 0) return f3(0.f);
        lightId = lid;
        return areaEmission(S.lights[lid], lp, toLocal(frameFromZ(ln), -wig).z, pt, pdfW);
    }
    if (S.bgKind == kBgNone) return f3(0.f);
    lightId = S.bgLightId;
    return bgEmission(S, wig, true, frame, pdfW);
}

// Direct illumination (algorithms 2-5, src/direct_illumination.hxx:15-156), eye light (0,
// src/eye_light.hxx:21-60) and normal visualiser (1, src/normal_visualiser.hxx:21-62): one hit.
// Random numbers: camera jitter (vertex 0, group 0; the visualisers take the pixel centre on
// sample 0), light pick + sample (vertex 1, group 0), BSDF sample (vertex 1, group 1), light i
// of the all-lights estimator (vertex 1, group 2 + i).
PG3_DI float3 traceDirect(const SceneView &S, int alg, uint32_t pixel, uint32_t sample, PathCounters &pc)
{
    const uint32_t px = pixel % S.width, py = pixel / S.width;
    const Rand4 rc = draw(S, pixel, sample, 0, 0);
    const bool centre = alg <= 1 && sample == 0;
    const float nx = ((float)px + (centre ? 0.5f : rc.a)) * (2.f / S.width) - 1.f;
    const float ny = ((float)py + (centre ? 0.5f : rc.b)) * (2.f / S.height) - 1.f;
    const float3 dir = normalize(S.camFwd + S.camRight * (nx * S.tanX) - S.camUp * (ny * S.tanY));
    ++pc.ext;
    Hit h;
    if (!intersectClosest(S, S.camPos, dir, 0.f, h)) {
        ++pc.bg;
        if (alg <= 1 || S.bgKind == kBgNone) return f3(0.f);
        float pdf;
        return bgEmission(S, dir, false, frameFromZ(make_float3(0.f, 0.f, 1.f)), pdf);
    }
    float3 pt, n;
    int matId;
    hitAttributes(S, h, S.camPos, dir, pt, n, matId);
    if (alg == 0) {
        const float dotLN = dot(n, -dir);
        return dotLN > 0.f ? f3(dotLN) : make_float3(-dotLN, 0.f, 0.f);
    }
    if (alg == 1)
        return make_float3(clampf(n.x / 2.f + 0.5f, 0.f, 1.f), clampf(n.y / 2.f + 0.5f, 0.f, 1.f),
                           clampf(n.z / 2.f + 0.5f, 0.f, 1.f));
    const Frame frame = frameFromZ(n);
    const float3 wol = toLocal(frame, -dir);
    const DevMaterial mat = loadMat(S, matId);
    const float sum = (S.lightCount > 1) ? estimateSum(S, pt, n) : 0.f;
    const Rand4 ra = draw(S, pixel, sample, 1, 0);
    const Rand4 rb = draw(S, pixel, sample, 1, 1);
    float3 Lo = f3(0.f);
    if (alg == 3 || alg == 4) {
        // AddSingleLightSampleContribution (src/path_tracer_base.hxx:315-348)
        const uint32_t count = (alg == 3) ? S.lightCount : 1u;
        for (uint32_t k = 0; k < count; ++k) {
            int lid;
            float prob;
            Rand4 rl = ra;
            if (alg == 3) {
                lid = (int)k;
                prob = 1.f;
                rl = draw(S, pixel, sample, 1, 2 + k);
            } else {
                pickLight(S, pt, n, sum, ra.a, lid, prob);
                if (lid < 0) break;
            }
            float3 wig, smp;
            float dist, pdfW;
            sampleLightAt(S, lid, pt, frame, n, rl.b, rl.c, rl.d, wig, dist, smp, pdfW);
            ++pc.shadow;
            if (!(maxc(smp) > 0.f) || occludedAny(S, pt, wig, dist)) continue;
            BsdfRec br;
            evalBsdf(mat, toLocal(frame, wig), wol, br);
            Lo += smp * br.att / (pdfW * prob);
        }
    } else if (alg == 2) {
        BsdfRec br;
        sampleBsdf(mat, wol, rb.b, rb.c, rb.d, br);
        if (!isBlocker(br)) {
            float pdfL;
            int lid;
            ++pc.ext;
            const float3 Li = directFromDirection(S, pt, frame, br.wil, pdfL, lid);
            Lo = (br.pdfW != infF()) ? (br.att * fabsf(br.wil.z) * Li) / (br.pdfW * br.compProb)
                                     : (br.att * Li) / br.compProb;
        }
    } else {
        // kDirectIllumMis: one light sample and one BSDF sample (:99-114)
        int lid;
        float lprob = 0.f;
        pickLight(S, pt, n, sum, ra.a, lid, lprob);
        if (lid >= 0) {
            float3 wig, smp;
            float dist, pdfW;
            sampleLightAt(S, lid, pt, frame, n, ra.b, ra.c, ra.d, wig, dist, smp, pdfW);
            ++pc.shadow;
            if (maxc(smp) > 0.f && !occludedAny(S, pt, wig, dist)) {   // src/path_tracer_base.hxx:350-411
                BsdfRec br;
                evalBsdf(mat, toLocal(frame, wig), wol, br);
                const float lightPdf = pdfW * lprob;
                Lo += (smp * br.att) * (misPower(lightPdf, br.pdfW * br.compProb) / lightPdf);
            }
        }
        BsdfRec br;   // AddDirectIllumMISBrdfSampleContribution (:427-486)
        sampleBsdf(mat, wol, rb.b, rb.c, rb.d, br);
        if (!isBlocker(br)) {
            float pdfL;
            int hitLight;
            ++pc.ext;
            const float3 Li = directFromDirection(S, pt, frame, br.wil, pdfL, hitLight);
            if (maxc(Li) > 0.f) {
                if (br.pdfW != infF()) {
                    const float bsdfPdf = br.pdfW * br.compProb;
                    const float pick = pickProb(S, pt, n, sum, hitLight);
                    Lo += (br.att * fabsf(br.wil.z) * Li) * (misPower(bsdfPdf, pdfL * pick) / bsdfPdf);
                } else {
                    Lo += (br.att * Li) / br.compProb;
                }
            }
        }
    }
    const int lightId = __ldg(&S.mat2light[matId]);
    float3 Le = f3(0.f);
    if (lightId >= 0) {
        float pdfA;
        Le = areaEmission(S.lights[lightId], pt, wol.z, make_float3(0.f, 0.f, 0.f), pdfA);
    }
    return Le + Lo;
}

// One camera path of the BSDF-sampling-only tracer (algorithm kPathTracingNaive,
// src/path_tracer.hxx:45-165).
PG3_DI float3 tracePathNaive(const SceneView &S, uint32_t pixel, uint32_t sample, PathCounters &pc)
{
    const uint32_t px = pixel % S.width, py = pixel / S.width;
    const Rand4 rc = draw(S, pixel, sample, 0, 0);
    const float nx = ((float)px + rc.a) * (2.f / S.width) - 1.f;
    const float ny = ((float)py + rc.b) * (2.f / S.height) - 1.f;
    float3 dir = normalize(S.camFwd + S.camRight * (nx * S.tanX) - S.camUp * (ny * S.tanY));
    float3 org = S.camPos;
    float tmin = 0.f;
    float3 L = f3(0.f), T = f3(1.f);
    for (uint32_t pl = 1;; ++pl) {
        ++pc.ext;
        Hit h;
        if (!intersectClosest(S, org, dir, tmin, h)) {
            if (pl >= S.minPL && S.bgKind != kBgNone) {
                float pdf;
                const Frame pf = frameFromZ(make_float3(0.f, 0.f, 1.f));
                L += bgEmission(S, dir, false, pf, pdf) * T;
            }
            ++pc.bg;
            break;
        }
        float3 pt, n;
        int matId;
        hitAttributes(S, h, org, dir, pt, n, matId);
        const Frame frame = frameFromZ(n);
        const float3 wol = toLocal(frame, -dir);
        const int lightId = __ldg(&S.mat2light[matId]);
        if (lightId >= 0 && pl >= S.minPL) {
            float pdfA;
            L += areaEmission(S.lights[lightId], pt, wol.z, org, pdfA) * T;
        }
        const DevMaterial mat = loadMat(S, matId);
        if (mat.zeroRefl) { ++pc.blocker; break; }
        if (S.maxPL > 0 && pl >= S.maxPL) { ++pc.maxl; break; }
        if (pl >= kMaxPathLengthHard) { ++pc.safety; break; }
        const Rand4 rb = draw(S, pixel, sample, pl, 1);
        float rr = 1.0f;
        if (S.maxPL == 0 || (S.rrMinPL > 0 && pl >= S.rrMinPL)) {
            rr = mat.rrProb;
            if (rb.a > rr) { ++pc.rr; break; }
        }
        BsdfRec br;
        sampleBsdf(mat, wol, rb.b, rb.c, rb.d, br);
        if (isBlocker(br)) { ++pc.blocker; break; }
        const float cosAbs = fabsf(br.wil.z);
        const float3 seg = (br.pdfW != infF()) ? br.att * (cosAbs / (br.pdfW * rr * br.compProb))
                                               : br.att / (rr * br.compProb);
        T = T * seg;
        org = pt;
        dir = toWorld(frame, br.wil);
        tmin = epsRayCos(cosAbs);
    }
    return L;
}

}  // namespace pg3
