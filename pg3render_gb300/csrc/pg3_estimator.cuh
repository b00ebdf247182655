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

// MISWeight2Power with sample counts (src/path_tracer_base.hxx:522-541)
PG3_DI float misPowerN(float p1, uint32_t n1, float p2, uint32_t n2)
{
    const float s1 = n1 * p1, s2 = n2 * p2;
    const float q1 = s1 * s1, q2 = s2 * s2;
    return q1 / (q1 + q2) / n1;
}

// Contribution estimate of the background light (BackgroundLight::EstimateContribution,
// src/lights.hxx:447-470): a constant background integrates to pi * luminance; for a map the
// clamped-cosine SH estimate of the irradiance (the steerable sampler's own estimate,
// src/em_steerable_sampler.hxx:2300-2355; the reference's other samplers estimate it by random
// MIS samples, em.hxx:130-169 -- any positive estimate keeps the picking unbiased).
PG3_DI float bgEstimate(const SceneView &S, float3 n)
{
    if (S.bgKind == kBgConstant) return luminance(S.bgConst) * kPiF;
    if (S.bgKind != kBgEnvMap) return 0.f;
    float c[9];
    steerCoeffs(n, c);
    return fmaxf(dot9(S.bgShL, c), 0.f);
}
// Estimate of light l (area lights first, then point lights, the background last;
// src/scene.hxx:767-825, 948-953).
PG3_DI float lightEstimate(const SceneView &S, uint32_t l, float3 pt, float3 n)
{
    return (l < S.nArea) ? tableEstimate(S.lights[l], pt, n) : bgEstimate(S, n);
}

// Weight of one of nL light samples against nB BSDF samples (AddMISLightSampleContribution,
// src/path_tracer_base.hxx:350-423): area and background samples are MIS-weighted with the
// BSDF's pdf of the same direction; a point light's sample is its exact contribution, left to
// the estimate of the sum over lights (divided by the picking probability and the count).
PG3_DI float lightSampleWeight(float pdfW, float lprob, uint32_t nL, float bsdfPdf, uint32_t nB)
{
    if (pdfW == infF()) return 1.f / (lprob * (float)nL);
    const float lightPdf = pdfW * lprob;
    return misPowerN(lightPdf, nL, bsdfPdf, nB) / lightPdf;
}

// Sum of the lights' contribution estimates at a vertex (src/path_tracer_base.hxx:216-232).
PG3_DI float estimateSum(const SceneView &S, float3 pt, float3 n)
{
    float sum = 0.f;
    for (uint32_t i = 0; i < S.lightCount; ++i) sum += lightEstimate(S, i, pt, n);
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
        for (; l < cnt; ++l) {
            e = lightEstimate(S, l, pt, n);
            cum += e;
            if (!(r > cum)) break;
        }
        if (l >= cnt) { l = cnt - 1; e = lightEstimate(S, l, pt, n); }
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
    return lightEstimate(S, (uint32_t)id, pt, n) / sum;
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
            pdf = (em == kEmCdf)                 ? emCdfPdf(S, dir)
                  : (em == kEmSteerable)         ? steerPdf<false>(S.steer, dir, pf.z)
                  : (em == kEmSteerableAdaptive) ? steerPdf<true>(S.steer, dir, pf.z)
                                                 : cosSpherePdfFront(toLocal(pf, dir));
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
        steerSample<false>(S, f.z, u0, u1, u2, wig, pdfW, radCos);
        return;
    }
    if (S.bgKind == kBgEnvMap && em == kEmSteerableAdaptive) {
        steerSample<true>(S, f.z, u0, u1, u2, wig, pdfW, radCos);
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
        const bool lights = takesLightSamples(mat);
        const float sum = (S.lightCount > 1 && lights) ? estimateSum(S, pt, n) : 0.f;

        // light sample with MIS (src/path_tracer.hxx:250-265, src/path_tracer_base.hxx:350-411)
        if (pl + 1 >= S.minPL && lights) {
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
                    tableSample(S.lights[lid], pt, n, ra.b, ra.c, wig, dist, smp, pdfW);
                }
                if (maxc(smp) > 0.f) {
                    ++pc.shadow;
                    if (!occludedAny(S, pt, wig, dist)) {
                        BsdfRec br;
                        evalBsdf(mat, toLocal(frame, wig), wol, br);
                        L += beta * (smp * br.att) * lightSampleWeight(pdfW, lprob, 1u, br.pdfW * br.compProb, 1u);
                    }
                }
            }
        }

        // Russian roulette (src/path_tracer.hxx:267-303)
        float rrProb = 1.0f;
        bool cut = false;
        if (S.maxPL == 0 || (S.rrMinPL > 0 && pl >= S.rrMinPL)) {
            rrProb = rrContinuation(mat, wol);
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

// Light sample of light `lid` (area: src/lights.hxx:114-131; point: :255-266; background: :424-445).
PG3_DI void sampleLightAt(const SceneView &S, int lid, float3 pt, const Frame &frame, float3 n, float u0, float u1,
                          float u2, float3 &wig, float &dist, float3 &smp, float &pdfW)
{
    if (lid == S.bgLightId) {
        bgSample(S, frame, u0, u1, u2, wig, pdfW, smp);
        dist = kFloatMax;
    } else {
        tableSample(S.lights[lid], pt, n, u0, u1, wig, dist, smp, pdfW);
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
    const bool lights = takesLightSamples(mat);
    const float sum = (S.lightCount > 1 && lights) ? estimateSum(S, pt, n) : 0.f;
    const Rand4 ra = draw(S, pixel, sample, 1, 0);
    const Rand4 rb = draw(S, pixel, sample, 1, 1);
    float3 Lo = f3(0.f);
    if ((alg == 3 || alg == 4) && lights) {
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
            // a point light's sample is exact: only the picking is estimated (:333-348)
            Lo += smp * br.att / ((pdfW == infF()) ? prob : pdfW * prob);
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
    } else if (alg == 5) {
        // kDirectIllumMis: one light sample and one BSDF sample (:99-114)
        int lid = -1;
        float lprob = 0.f;
        if (lights) pickLight(S, pt, n, sum, ra.a, lid, lprob);
        if (lid >= 0) {
            float3 wig, smp;
            float dist, pdfW;
            sampleLightAt(S, lid, pt, frame, n, ra.b, ra.c, ra.d, wig, dist, smp, pdfW);
            ++pc.shadow;
            if (maxc(smp) > 0.f && !occludedAny(S, pt, wig, dist)) {   // src/path_tracer_base.hxx:350-411
                BsdfRec br;
                evalBsdf(mat, toLocal(frame, wig), wol, br);
                Lo += (smp * br.att) * lightSampleWeight(pdfW, lprob, 1u, br.pdfW * br.compProb, 1u);
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

// ------------------------------------------------------------------------------------------
// The recursive estimator with splitting, the light-to-BSDF sample ratio and indirect clipping
// (src/path_tracer.hxx:167-454). A vertex takes nLight light samples and nBsdf BSDF samples
// (ComputeSplittingCounts, :432-454); each BSDF sample starts a sub-path whose reflected
// estimate is clipped proportionally before it is added (:400-402), so the estimator is a tree
// walked depth first with an explicit stack of vertex frames in device memory. Random numbers
// are keyed by the vertex's preorder index in the tree (1 for the camera ray's hit; a chain
// without splitting gives index == path length, the streams of tracePath): light sample j
// draws group 2j, BSDF sample i group 2i+1.
// ------------------------------------------------------------------------------------------


PG3_DI void splittingCounts(const SceneView &S, float budget, uint32_t &nB, uint32_t &nL, float &next)
{
    nB = (uint32_t)max(lroundf((1.f - S.splitLevel) * 1.f + S.splitLevel * budget), 1l);
    nL = (uint32_t)lroundf(fmaxf(S.lightRatio * nB, 1.f));
    next = 1.f + ((budget - nB) / (float)nB);
}

// A new vertex on the stack: counts, roulette probability, and its light samples
// (src/path_tracer.hxx:240-265, src/path_tracer_base.hxx:156-188, 350-411).
PG3_DI void treeVertex(const SceneView &S, TreeFrame *F, float3 pt, float3 n, float3 wol, int mat, uint32_t pl,
                       float budget, uint32_t vid, uint32_t pixel, uint32_t sample, PathCounters &pc)
{
    uint32_t nB, nL;
    float next;
    splittingCounts(S, budget, nB, nL, next);
    const DevMaterial m = loadMat(S, mat);
    const bool rrActive = S.maxPL == 0 || (S.rrMinPL > 0 && pl >= S.rrMinPL);
    const bool lights = takesLightSamples(m);
    const float sum = (S.lightCount > 1 && lights) ? estimateSum(S, pt, n) : 0.f;
    const Frame frame = frameFromZ(n);
    float3 R = f3(0.f);
    if (pl + 1 >= S.minPL && lights) {
        for (uint32_t j = 0; j < nL; ++j) {
            const Rand4 ra = draw(S, pixel, sample, vid, 2 * j);
            int lid;
            float lprob = 0.f;
            pickLight(S, pt, n, sum, ra.a, lid, lprob);
            if (lid < 0) continue;
            float3 wig, smp;
            float dist, pdfW;
            sampleLightAt(S, lid, pt, frame, n, ra.b, ra.c, ra.d, wig, dist, smp, pdfW);
            if (!(maxc(smp) > 0.f)) continue;
            ++pc.shadow;
            if (occludedAny(S, pt, wig, dist)) continue;
            BsdfRec br;
            evalBsdf(m, toLocal(frame, wig), wol, br);
            R += (smp * br.att) * lightSampleWeight(pdfW, lprob, nL, br.pdfW * br.compProb, nB);
        }
    }
    F->pt = pt;
    F->budget = next;
    F->n = n;
    F->rr = rrActive ? rrContinuation(m, wol) : 1.0f;
    F->wol = wol;
    F->sum = sum;
    F->R = R;
    F->vid = vid;
    F->mat = mat;
    F->pl = pl;
    F->i = 0;
    F->nBsdf = nB;
    F->nLight = nL;
    F->flags = rrActive ? 4u : 0u;   // 4: roulette active at this vertex
}

// Can the vertex reached at path length pl start its own samples? (src/path_tracer.hxx:212-238)
PG3_DI bool treeReflects(const SceneView &S, const DevMaterial &m, uint32_t pl, PathCounters &pc)
{
    if (m.zeroRefl) { ++pc.blocker; return false; }
    if (S.maxPL > 0 && pl >= S.maxPL) { ++pc.maxl; return false; }
    if (pl >= kMaxPathLengthHard) { ++pc.safety; return false; }
    return true;
}

PG3_DI float3 traceTree(const SceneView &S, uint32_t pixel, uint32_t sample, PathCounters &pc, TreeFrame *stack,
                        uint32_t maxDepth)
{
    const uint32_t px = pixel % S.width, py = pixel / S.width;
    const Rand4 rc = draw(S, pixel, sample, 0, 0);
    const float nx = ((float)px + rc.a) * (2.f / S.width) - 1.f;
    const float ny = ((float)py + rc.b) * (2.f / S.height) - 1.f;
    const float3 dir = normalize(S.camFwd + S.camRight * (nx * S.tanX) - S.camUp * (ny * S.tanY));
    ++pc.ext;
    Hit h;
    float3 L = f3(0.f);
    if (!intersectClosest(S, S.camPos, dir, 0.f, h)) {
        ++pc.bg;
        if (S.minPL <= 1 && S.bgKind != kBgNone) {
            float pdf;
            L = bgEmission(S, dir, false, frameFromZ(make_float3(0.f, 0.f, 1.f)), pdf);
        }
        return L;
    }
    float3 pt, n;
    int matId;
    hitAttributes(S, h, S.camPos, dir, pt, n, matId);
    const float3 wol0 = toLocal(frameFromZ(n), -dir);
    const int light0 = __ldg(&S.mat2light[matId]);
    if (light0 >= 0 && S.minPL <= 1) {
        float pdfA;
        L = areaEmission(S.lights[light0], pt, wol0.z, S.camPos, pdfA);
    }
    if (!treeReflects(S, loadMat(S, matId), 1, pc)) return L;
    uint32_t vid = 1;
    treeVertex(S, &stack[0], pt, n, wol0, matId, 1, S.splitBudget, vid, pixel, sample, pc);
    int d = 0;
    for (uint32_t guard = 0; guard < (1u << 26); ++guard) {
        TreeFrame *F = &stack[d];
        if (F->i < F->nBsdf) {
            const uint32_t i = F->i;
            const Rand4 rb = draw(S, pixel, sample, F->vid, 2 * i + 1);
            const bool cut = (F->flags & 4u) && rb.a > F->rr;
            if (cut) ++pc.rr;
            const DevMaterial m = loadMat(S, F->mat);
            BsdfRec br;
            sampleBsdf(m, F->wol, rb.b, rb.c, rb.d, br);
            if (isBlocker(br)) {
                ++pc.blocker;
                F->i = i + 1;
                continue;
            }
            const bool finite = br.pdfW != infF();
            const float cosAbs = fabsf(br.wil.z);
            const Frame pf = frameFromZ(F->n);
            const float3 wig = toWorld(pf, br.wil);
            const uint32_t pl = F->pl + 1;
            // the sample's ray: emission found at its end (src/path_tracer.hxx:198-210, 408-429)
            ++pc.ext;
            Hit ch;
            float3 Le = f3(0.f), cpt, cn, cwol;
            float lpdf = 0.f;
            int lid = -1, cmat = 0;
            bool childRefl = false;
            if (!intersectClosest(S, F->pt, wig, epsRayCos(cosAbs), ch)) {
                if (pl >= S.minPL && S.bgKind != kBgNone) {
                    Le = bgEmission(S, wig, finite, pf, lpdf);
                    lid = S.bgLightId;
                }
                if (!cut) ++pc.bg;
            } else {
                hitAttributes(S, ch, F->pt, wig, cpt, cn, cmat);
                cwol = toLocal(frameFromZ(cn), -wig);
                const int l = __ldg(&S.mat2light[cmat]);
                if (l >= 0 && pl >= S.minPL) {
                    Le = areaEmission(S.lights[l], cpt, cwol.z, F->pt, lpdf);
                    lid = l;
                }
                childRefl = !cut && treeReflects(S, loadMat(S, cmat), pl, pc);
            }
            // direct light hit by the sample (:324-369)
            float3 R = F->R;
            if (!isZero(Le) && lid >= 0) {
                if (finite) {
                    const float bsdfPdf = br.pdfW * br.compProb;
                    const float lightPdf = lpdf * pickProb(S, F->pt, F->n, F->sum, lid);
                    R += (br.att * cosAbs * Le) * (misPowerN(bsdfPdf, F->nBsdf, lightPdf, F->nLight) / bsdfPdf);
                } else {
                    R += (br.att * Le) / ((float)F->nBsdf * br.compProb);
                }
            }
            F->R = R;
            if (childRefl && (uint32_t)d + 1 < maxDepth) {
                F->att = br.att;
                F->cosAbs = cosAbs;
                F->pdfW = br.pdfW;
                F->compProb = br.compProb;
                F->flags = (F->flags & 4u) | (finite ? 1u : 0u);
                ++vid;
                treeVertex(S, &stack[d + 1], cpt, cn, cwol, cmat, pl, F->budget, vid, pixel, sample, pc);
                ++d;
            } else {
                if (childRefl) atomicOr(S.errorFlag, kErrTreeStack);
                F->i = i + 1;
            }
            continue;
        }
        // this vertex's estimate is complete: hand it to the parent's indirect term (:372-405)
        const float3 Rv = F->R;
        if (d == 0) return L + Rv;
        --d;
        TreeFrame *P = &stack[d];
        if (!isZero(Rv)) {
            const float denom = ((P->flags & 1u) ? P->pdfW : 1.f) * P->nBsdf * P->rr * P->compProb;
            float3 ind = (P->flags & 1u) ? (P->att * P->cosAbs * Rv) / denom : (P->att * Rv) / denom;
            if (S.clipping > 0.f) {
                const float mx = maxc(ind);
                if (mx > S.clipping) ind = ind * (S.clipping / mx);
            }
            P->R = P->R + ind;
        }
        P->i = P->i + 1;
    }
    atomicOr(S.errorFlag, kErrTreeStack);
    return L;
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
            rr = rrContinuation(mat, wol);
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
